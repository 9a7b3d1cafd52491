"""Generate the golden fixtures for the energy/force/stress path.

Reads, from the upstream CALYPSO-GAP checkout, the example model
``gappy/example/ASE-GAPPY/gap_parameters`` and the MD trajectory
``gappy/example/ASE-GAPPY/ase.traj`` (ASE "Ulm" format, written by
``gappy/example/ASE-GAPPY/run_md.py:10-21`` with ``GAP(rcut=6.0)``), and writes

* ``tests/golden/gap_parameters_c_diamond`` - the model file, byte for byte;
* ``tests/golden/ase_traj_frames.npz`` - for each of the 11 frames: numbers,
  cell (rows = lattice vectors), positions, and the reference calculator's
  energy (eV), forces (eV/A) and stress (GPa, order XX YY ZZ XY YZ ZX).

The Ulm container is parsed here without ASE: every frame is a JSON header
whose ``"ndarray": [shape, dtype, offset]`` entries point at raw
little-endian payloads at absolute file offsets.

Usage: python tests/golden/make_golden.py [path/to/CALYPSO-GAP]
"""
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _frame_headers(data):
    """Yield the decoded JSON header of every frame in an Ulm file.

    Layout: 8-byte magic ``- of Ulm``, 16-byte tag, then little-endian int64
    ``version, nitems, offsets_pos``; at ``offsets_pos`` sit ``nitems`` int64
    item offsets, and each item is an int64 byte length followed by JSON.
    """
    version, nitems, offsets_pos = np.frombuffer(data[24:48], "<i8")
    offsets = np.frombuffer(data, "<i8", count=int(nitems), offset=int(offsets_pos))
    dec = json.JSONDecoder()
    for off in offsets:
        start = int(off) + 8
        obj, _ = dec.raw_decode(data[start:].decode("latin-1"))
        yield obj


def _ndarray(data, spec):
    shape, dtype, offset = spec["ndarray"]
    count = int(np.prod(shape))
    arr = np.frombuffer(data, dtype=np.dtype(dtype).newbyteorder("<"),
                        count=count, offset=offset)
    return arr.reshape(shape).copy()


def read_ulm_frames(path):
    """Frames of an ASE trajectory; later frames inherit ``numbers`` from frame 0."""
    data = open(path, "rb").read()
    frames = []
    numbers = None
    for h in _frame_headers(data):
        if "numbers." in h:
            numbers = _ndarray(data, h["numbers."]).astype(np.int64)
        calc = h["calculator."]
        frames.append(dict(
            numbers=numbers.copy(),
            positions=_ndarray(data, h["positions."]).astype(np.float64),
            cell=np.asarray(h["cell"], dtype=np.float64),
            energy=float(calc["energy"]),
            forces=_ndarray(data, calc["forces."]).astype(np.float64),
            stress=np.asarray(calc["stress"], dtype=np.float64),
        ))
    return frames


def main(ref_root):
    ex = os.path.join(ref_root, "gappy", "example", "ASE-GAPPY")
    frames = read_ulm_frames(os.path.join(ex, "ase.traj"))
    assert len(frames) == 11, len(frames)
    np.savez_compressed(
        os.path.join(HERE, "ase_traj_frames.npz"),
        numbers=np.stack([f["numbers"] for f in frames]),
        cell=np.stack([f["cell"] for f in frames]),
        positions=np.stack([f["positions"] for f in frames]),
        energy=np.array([f["energy"] for f in frames]),
        forces=np.stack([f["forces"] for f in frames]),
        stress=np.stack([f["stress"] for f in frames]),
        rcut=np.float64(6.0),
    )
    shutil.copyfile(os.path.join(ex, "gap_parameters"),
                    os.path.join(HERE, "gap_parameters_c_diamond"))
    print("wrote", len(frames), "frames; E0 =", frames[0]["energy"])


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <path of the CALYPSO-GAP source tree>")
    main(sys.argv[1])
