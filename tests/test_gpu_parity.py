"""Parity of the CUDA path (through the C ABI) with the oracle.

Bars: neighbour lists bit-identical; FP64 path within 1e-9 relative energy,
1e-7 eV/A forces, 1e-7 GPa stress (the plain-path tolerance); FP32 path
within 1 meV/atom energy and 20 meV/A forces (the reduced-precision bar).
"""
import ctypes
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN_MODEL
from helpers import synth_model_file

pytestmark = pytest.mark.gpu

E_REL, F_ABS, S_ABS = 1e-9, 1e-7, 1e-7


@pytest.fixture(scope="module")
def golden_model(gapgb_mod):
    m = gapgb_mod.GapModel.load(GOLDEN_MODEL)
    yield m
    m.close()


@pytest.fixture(scope="module")
def synth_si(oracle_mod, gapgb_mod, tmp_path_factory):
    """Si model (zeta extension on) + its oracle twin, read from one file."""
    import gapgb.synth as S
    path = str(tmp_path_factory.mktemp("si") / "gap_parameters")
    synth_model_file(path, oracle_mod, [S.si64(seed=s) for s in range(3)], M=300,
                     theta_scale=1.0, coeff_std=1.0, seed=1)
    g = gapgb_mod.GapModel.load(path)
    yield g, oracle_mod.Model(path)
    g.close()


@pytest.fixture(scope="module")
def synth_pop(oracle_mod, gapgb_mod, tmp_path_factory):
    """4-species model over small triclinic population members."""
    import gapgb.synth as S
    rng = np.random.default_rng(7)
    structs = [S.random_structure(rng, n, species_pool=(3, 8, 14, 26)) for n in (12, 20, 31, 9)]
    # make every species appear in the sparse set
    structs.append(S.random_structure(np.random.default_rng(8), 16, species_pool=(3, 8, 14, 26)))
    path = str(tmp_path_factory.mktemp("pop") / "gap_parameters")
    lat, pos, z = structs[0]
    z = np.array([3, 8, 14, 26] * 3, np.int32)
    structs[0] = (lat, pos, z)
    synth_model_file(path, oracle_mod, structs, M=150, theta_scale=2.0, coeff_std=0.5, seed=3,
                     zeta=False)
    g = gapgb_mod.GapModel.load(path)
    yield g, oracle_mod.Model(path), structs
    g.close()


def _assert_nbr_equal(gcnt, gnb, ocnt, onb):
    assert np.array_equal(gcnt, ocnt)
    for i in range(len(gcnt)):
        a = gnb[i, : gcnt[i]]
        b = onb[i, : ocnt[i]]
        # bit-identical image positions, distances, weights and partner indices
        assert np.array_equal(a.view(np.int64), b.view(np.int64)), i


# ---------------------------------------------------------------- neighbours

@pytest.mark.parametrize("f", [0, 5, 10])
def test_neighbours_bit_exact_golden(golden_model, oracle_mod, golden_oracle_model, frames, f):
    z, lat, pos = frames["numbers"][f], frames["cell"][f], frames["positions"][f]
    gcnt, gnb = golden_model.neighbors(z, lat, pos, cap=1000)
    ocnt, onb = oracle_mod.neighbors(lat, pos, golden_oracle_model.weights(z), 6.0, 1000)
    _assert_nbr_equal(gcnt, gnb, ocnt, onb)


def test_neighbours_bit_exact_triclinic(synth_pop, oracle_mod):
    g, o, structs = synth_pop
    for lat, pos, z in structs:
        gcnt, gnb = g.neighbors(z, lat, pos, cap=600)
        ocnt, onb = oracle_mod.neighbors(lat, pos, o.weights(z), 6.0, 600)
        _assert_nbr_equal(gcnt, gnb, ocnt, onb)


def test_neighbours_bit_exact_alloy512(gapgb_mod, oracle_mod, synth_pop):
    import gapgb.synth as S
    lat, pos, z = S.alloy512(seed=3)
    zt, wt = S.species_table(z)
    m = gapgb_mod.GapModel.create(zt, wt, [1], [0.5], [6.0], np.ones(2), np.zeros((1, 2)),
                                  np.zeros(1))
    gcnt, gnb = m.neighbors(z, lat, pos, cap=128)
    w = dict(zip(zt.tolist(), wt.tolist()))
    ocnt, onb = oracle_mod.neighbors(lat, pos, np.array([w[v] for v in z]), 6.0, 128)
    _assert_nbr_equal(gcnt, gnb, ocnt, onb)
    m.close()


def test_neighbours_bit_exact_binned_cell(gapgb_mod, oracle_mod):
    """A cell of >= 2048 atoms takes the binned build (27 bins around each
    atom, hits sorted into the reference's order); its list must equal the
    oracle's O(N^2) scan bit for bit, including atoms jittered out of the cell."""
    import gapgb.synth as S
    lat, pos, z = S.sige(seed=2, reps=8, jitter=0.3)
    pos = pos.copy()
    pos[:5] -= lat[0] * 0.02  # a few atoms outside the cell
    zt, wt = S.species_table(z)
    m = gapgb_mod.GapModel.create(zt, wt, [1], [0.5], [6.0], np.ones(2), np.zeros((1, 2)),
                                  np.zeros(1))
    gcnt, gnb = m.neighbors(z, lat, pos, cap=128)
    w = dict(zip(zt.tolist(), wt.tolist()))
    ocnt, onb = oracle_mod.neighbors(lat, pos, np.array([w[v] for v in z]), 6.0, 128)
    _assert_nbr_equal(gcnt, gnb, ocnt, onb)
    m.close()


# ---------------------------------------------------------------- descriptors

def test_descriptors_match_oracle(synth_si, oracle_mod):
    import gapgb.synth as S
    g, o = synth_si
    lat, pos, z = S.si64(seed=11)
    xx = g.descriptors([0, len(pos)], z, lat[None], pos)
    cnt, nb = oracle_mod.neighbors(lat, pos, o.weights(z), 6.0, 400)
    ox, _, _ = oracle_mod.car2acsf(o, pos, cnt, nb)
    scale = np.abs(ox).max(0) + 1e-300
    assert np.max(np.abs(xx - ox) / scale) < 1e-12


def test_descriptors_golden_model(golden_model, oracle_mod, golden_oracle_model, frames):
    z, lat, pos = frames["numbers"][2], frames["cell"][2], frames["positions"][2]
    xx = golden_model.descriptors([0, len(pos)], z, lat[None], pos)
    *_, ex = oracle_mod.gap_calc(golden_oracle_model, z, lat, pos, 6.0, False, extras=True)
    scale = np.abs(ex["xx"]).max(0) + 1e-300
    assert np.max(np.abs(xx - ex["xx"]) / scale) < 1e-12


# ---------------------------------------------------------------- full path FP64

@pytest.mark.parametrize("f", range(11))
def test_fp64_golden_frames(golden_model, frames, f):
    golden_model.set_precision("fp64")
    E, F, S, var = golden_model.eval(frames["numbers"][f], frames["cell"][f],
                                     frames["positions"][f])
    assert abs(E - frames["energy"][f]) <= E_REL * abs(frames["energy"][f])
    assert np.abs(F - frames["forces"][f]).max() <= F_ABS
    assert np.abs(S - frames["stress"][f]).max() <= S_ABS
    assert var == 0.0


def test_fp64_vs_oracle_si_zeta(synth_si, oracle_mod):
    import gapgb.synth as S
    g, o = synth_si
    g.set_precision("fp64")
    for seed in (21, 22):
        lat, pos, z = S.si64(seed=seed)
        E, F, St, _ = g.eval(z, lat, pos)
        oE, oF, oS, _ = oracle_mod.gap_calc(o, z, lat, pos, 6.0, True)
        assert abs(E - oE) <= E_REL * max(1.0, abs(oE))
        assert np.abs(F - oF).max() <= F_ABS
        assert np.abs(St - oS).max() <= S_ABS


def test_fp64_vs_oracle_population_batch(synth_pop, oracle_mod):
    import gapgb.synth as S
    g, o, structs = synth_pop
    g.set_precision("fp64")
    rng = np.random.default_rng(99)
    batch = [S.random_structure(rng, n, species_pool=(3, 8, 14, 26)) for n in (8, 17, 40, 23, 64)]
    off, sp, lat, pos = S.pack(batch)
    E, F, St, ae = g.eval_batch(off, sp, lat, pos, atom_energy=True)
    for s, (l, p, z) in enumerate(batch):
        oE, oF, oS, _, ex = oracle_mod.gap_calc(o, z, l, p, 6.0, True, extras=True)
        assert abs(E[s] - oE) <= E_REL * max(1.0, abs(oE))
        assert np.abs(F[off[s]:off[s + 1]] - oF).max() <= F_ABS
        assert np.abs(St[s] - oS).max() <= S_ABS
        assert np.abs(ae[off[s]:off[s + 1]] - ex["e"]).max() <= 1e-9 * max(1.0, np.abs(ex["e"]).max())


def _edge_structures():
    """Atoms with no neighbour at all (15 A apart in a 30 A cell), one atom
    whose only neighbours are its own images (2.7 A cubic cell), and a dimer
    whose atoms have exactly one neighbour each (no angular pair)."""
    iso = (np.eye(3) * 30.0, np.array([[1.0, 1.0, 1.0], [16.0, 16.0, 16.0]]),
           np.array([14, 8], np.int32))
    lone = (np.eye(3) * 2.7 + np.array([[0.0, 0.0, 0.0], [0.3, 0.0, 0.0], [0.0, 0.2, 0.0]]),
            np.array([[0.4, 0.5, 0.6]]), np.array([14], np.int32))
    dimer = (np.eye(3) * 25.0, np.array([[5.0, 5.0, 5.0], [6.2, 5.9, 5.8]]),
             np.array([8, 14], np.int32))
    return [iso, lone, dimer]


@pytest.mark.parametrize("prec", ["fp64", "fp32", "tc"])
def test_edge_structures_match_oracle(synth_pop, oracle_mod, prec):
    """No neighbours, only self-images, one neighbour: alone and as one
    ragged batch, against the oracle (FP64 bar for fp64, the
    reduced-precision bar otherwise)."""
    import gapgb.synth as S
    g, o, _ = synth_pop
    g.set_precision(prec)
    e_tol, f_tol, s_tol = (E_REL, F_ABS, S_ABS) if prec == "fp64" else (1e-3, 20e-3, 1e-2)
    edge = _edge_structures()
    ref = [oracle_mod.gap_calc(o, z, l, p, 6.0, True) for l, p, z in edge]
    for k, (l, p, z) in enumerate(edge):
        E, F, St, _ = g.eval(z, l, p)
        oE, oF, oS, _ = ref[k]
        assert abs(E - oE) <= (e_tol * max(1.0, abs(oE)) if prec == "fp64" else e_tol * len(z)), k
        assert np.abs(F - oF).max() <= f_tol, k
        assert np.abs(St - oS).max() <= s_tol, k
    # the isolated atoms feel nothing
    E0, F0, S0, _ = g.eval(edge[0][2], edge[0][0], edge[0][1])
    assert np.abs(F0).max() == 0.0 and np.abs(S0).max() == 0.0
    off, sp, lat, pos = S.pack(edge)
    E, F, St = g.eval_batch(off, sp, lat, pos)
    for k in range(len(edge)):
        oE, oF, oS, _ = ref[k]
        n = off[k + 1] - off[k]
        assert abs(E[k] - oE) <= (e_tol * max(1.0, abs(oE)) if prec == "fp64" else e_tol * n), k
        assert np.abs(F[off[k]:off[k + 1]] - oF).max() <= f_tol, k
        assert np.abs(St[k] - oS).max() <= s_tol, k
    g.set_precision("fp64")


def test_batch_equals_single(synth_si):
    import gapgb.synth as S
    g, _ = synth_si
    g.set_precision("fp64")
    structs = [S.si64(seed=s) for s in (31, 32, 33)]
    off, sp, lat, pos = S.pack(structs)
    E, F, St = g.eval_batch(off, sp, lat, pos)
    for s, (l, p, z) in enumerate(structs):
        e1, f1, s1, _ = g.eval(z, l, p)
        assert abs(E[s] - e1) <= 1e-12 * max(1.0, abs(e1))
        assert np.abs(F[off[s]:off[s + 1]] - f1).max() <= 1e-10
        assert np.abs(St[s] - s1).max() <= 1e-10


def _wide_si(seed, outside=0):
    """216-atom Si cell (16.3 A, wider than twice the 6 A cutoff on every
    axis); `outside` atoms moved past the cell's faces."""
    import gapgb.synth as S
    rng = np.random.default_rng(seed)
    lat, pos = S._supercell(S._diamond_basis(), 5.43, (3, 3, 3))
    pos = pos + rng.normal(0.0, 0.05, pos.shape)
    pos[:outside] += lat[0] * 1.04 - lat[2] * 0.03
    return lat, pos, np.full(len(pos), 14, np.int32)


@pytest.mark.parametrize("prec", ["fp64", "tc"])
def test_mixed_wide_and_narrow_batch(synth_si, oracle_mod, prec):
    """Cells wider than twice the cutoff and narrower ones in one batch: the
    two neighbour-build kernels each take their own cells' atoms and skip the
    others', so every structure's results equal its evaluation alone, and
    the wide cell with atoms outside the cell has the oracle's list and
    results."""
    import gapgb.synth as S
    g, o = synth_si
    g.set_precision(prec)
    structs = [_wide_si(1), S.si64(seed=41), _wide_si(2, outside=7), S.si64(seed=42)]
    off, sp, lat, pos = S.pack(structs)
    E, F, St = g.eval_batch(off, sp, lat, pos)
    for s, (l, p, z) in enumerate(structs):
        e1, f1, s1, _ = g.eval(z, l, p)
        assert abs(E[s] - e1) <= 1e-12 * max(1.0, abs(e1)), s
        assert np.abs(F[off[s]:off[s + 1]] - f1).max() <= 1e-10, s
        assert np.abs(St[s] - s1).max() <= 1e-10, s
    l, p, z = structs[2]
    gcnt, gnb = g.neighbors(z, l, p, cap=400)
    ocnt, onb = oracle_mod.neighbors(l, p, o.weights(z), 6.0, 400)
    _assert_nbr_equal(gcnt, gnb, ocnt, onb)
    oE, oF, oS, _ = oracle_mod.gap_calc(o, z, l, p, 6.0, True)
    # this stiff model's cell carries stresses near 280 GPa: the reduced-
    # precision bar is 1e-2 GPa or 1e-4 of the largest component
    e_tol, f_tol, s_tol = ((E_REL, F_ABS, S_ABS) if prec == "fp64"
                           else (1e-3, 20e-3, max(1e-2, 1e-4 * np.abs(oS).max())))
    assert abs(E[2] - oE) <= (e_tol * max(1.0, abs(oE)) if prec == "fp64" else e_tol * len(z))
    assert np.abs(F[off[2]:off[3]] - oF).max() <= f_tol
    assert np.abs(St[2] - oS).max() <= s_tol
    g.set_precision("fp64")


def test_lgrad_false(golden_model, frames):
    golden_model.set_precision("fp64")
    E, F, S, _ = golden_model.eval(frames["numbers"][0], frames["cell"][0], frames["positions"][0],
                                   lgrad=False)
    assert abs(E - frames["energy"][0]) <= E_REL * abs(frames["energy"][0])
    assert not F.any() and not S.any()


def test_repeatable_bitwise(golden_model, frames):
    golden_model.set_precision("fp64")
    a = golden_model.eval(frames["numbers"][4], frames["cell"][4], frames["positions"][4])
    b = golden_model.eval(frames["numbers"][4], frames["cell"][4], frames["positions"][4])
    assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


# ---------------------------------------------------------------- FP32 path

def test_mixed_golden_frames(golden_model, frames):
    """The trained model's coefficients cancel ~2.4e4-fold: FP32 kernel values
    miss 1 meV/atom there, FP32 descriptors with the FP64 GPR do not."""
    golden_model.set_precision("mixed")
    try:
        for f in range(11):
            E, F, S, _ = golden_model.eval(frames["numbers"][f], frames["cell"][f],
                                           frames["positions"][f])
            n = len(F)
            assert abs(E - frames["energy"][f]) / n <= 1e-3
            assert np.abs(F - frames["forces"][f]).max() <= 20e-3
    finally:
        golden_model.set_precision("fp64")


def test_fp32_population(synth_pop, oracle_mod):
    import gapgb.synth as S
    g, o, _ = synth_pop
    g.set_precision("fp32")
    try:
        rng = np.random.default_rng(5)
        batch = [S.random_structure(rng, n, species_pool=(3, 8, 14, 26)) for n in (30, 50)]
        off, sp, lat, pos = S.pack(batch)
        E, F, St = g.eval_batch(off, sp, lat, pos)
        for s, (l, p, z) in enumerate(batch):
            oE, oF, oS, _ = oracle_mod.gap_calc(o, z, l, p, 6.0, True)
            assert abs(E[s] - oE) / len(p) <= 1e-3
            assert np.abs(F[off[s]:off[s + 1]] - oF).max() <= 20e-3
    finally:
        g.set_precision("fp64")


# ---------------------------------------------------------------- large-size properties

def test_supercell_consistency_sige():
    """E, F, stress of a 2x2x2 replica (32768 atoms, the MD cell) equal 8x E,
    tiled F and the same stress of the 4096-atom cell."""
    import gapgb
    import gapgb.synth as S
    lat, pos, z = S.sige(seed=4, reps=8)
    zt, wt = S.species_table(z)
    ty, al, rc, ze = S.sf_table()
    rng = np.random.default_rng(0)
    D = 64
    mm = rng.normal(1.0, 0.3, (64, D)) * 5
    m = gapgb.GapModel.create(zt, wt, ty, al, rc, np.full(D, 40.0), mm, rng.normal(0, 1, 64),
                              sf_zeta=ze)
    m.set_precision("fp64")
    E1, F1, S1, _ = m.eval(z, lat, pos)
    shifts = np.array([[i, j, k] for i in range(2) for j in range(2) for k in range(2)])
    big = np.concatenate([pos + s @ lat for s in shifts])
    E8, F8, S8, _ = m.eval(np.tile(z, 8), lat * 2, big)
    assert abs(E8 - 8 * E1) <= 1e-9 * abs(E8)
    assert np.abs(F8 - np.tile(F1, (8, 1))).max() <= 1e-7
    assert np.abs(S8 - S1).max() <= 1e-7
    assert np.abs(F8.sum(0)).max() <= 1e-8
    m.close()


# ---------------------------------------------------------------- drop-in APIs

def test_libgap_calculator_and_ase(gapgb_mod, frames, tmp_path, monkeypatch):
    shutil.copy(GOLDEN_MODEL, tmp_path / "gap_parameters")
    monkeypatch.chdir(tmp_path)
    from libgap.GAP import Calculator
    c = Calculator(rcut=6.0)
    c.gap_read()
    species = ["C"] * 64
    e, f, s, v = c.gap_calc(species, frames["cell"][1], frames["positions"][1], True)
    assert abs(e - frames["energy"][1]) <= E_REL * abs(frames["energy"][1])
    assert np.abs(f - frames["forces"][1]).max() <= F_ABS
    assert np.abs(s - frames["stress"][1]).max() <= S_ABS and v == 0.0

    from ase_gap.gap_calc import GAP

    class Atoms:
        def __init__(self, z, cell, pos):
            self.numbers, self.cell, self.positions = z, cell, pos

        def get_atomic_numbers(self):
            return self.numbers

        def copy(self):
            return Atoms(self.numbers.copy(), self.cell.copy(), self.positions.copy())

    calc = GAP(rcut=6.0)
    at = Atoms(frames["numbers"][2], frames["cell"][2], frames["positions"][2])
    calc.calculate(at, ["energy", "forces", "stress"])
    assert abs(calc.results["energy"] - frames["energy"][2]) <= E_REL * abs(frames["energy"][2])
    assert calc.results["free_energy"] == calc.results["energy"]
    assert np.abs(calc.results["forces"] - frames["forces"][2]).max() <= F_ABS
    assert np.abs(calc.results["stress"] - frames["stress"][2]).max() <= S_ABS


def test_fortran_abi_shim(gapgb_mod, frames, tmp_path, monkeypatch):
    """fgap_read_/fgap_calc_/fget_bond_ with gfortran conventions (by reference,
    column-major) - what calypso-side callers link against."""
    shutil.copy(GOLDEN_MODEL, tmp_path / "gap_parameters")
    monkeypatch.chdir(tmp_path)
    L = ctypes.CDLL(gapgb_mod.lib_path())
    I, Dp = ctypes.c_int, ctypes.POINTER(ctypes.c_double)
    nsp, dl = I(), I()
    theta = np.zeros(100)
    MM = np.zeros((4000, 100), order="F")
    inv = np.zeros((4000, 4000), order="F")
    coeff = np.zeros(4000)
    L.fgap_read_(ctypes.byref(nsp), ctypes.byref(dl), theta.ctypes.data_as(Dp),
                 MM.ctypes.data_as(Dp), inv.ctypes.data_as(Dp), coeff.ctypes.data_as(Dp))
    assert (nsp.value, dl.value) == (129, 66)
    M, D = nsp.value, dl.value
    mm_f = np.asfortranarray(MM[:M, :D])
    f = 3
    na = I(64)
    species = np.asfortranarray(frames["numbers"][f].astype(np.int32))
    lat_f = np.asfortranarray(frames["cell"][f])
    pos_f = np.asfortranarray(frames["positions"][f])
    ene, var = ctypes.c_double(), ctypes.c_double()
    force = np.zeros((64, 3), order="F")
    stress = np.zeros(6)
    rc = ctypes.c_double(6.0)
    lg = I(1)
    qmm = np.zeros((M, M), order="F")
    th = np.ascontiguousarray(theta[:D])
    co = np.ascontiguousarray(coeff[:M])
    L.fgap_calc_(ctypes.byref(na), species.ctypes.data_as(ctypes.POINTER(I)),
                 lat_f.ctypes.data_as(Dp), pos_f.ctypes.data_as(Dp), ctypes.byref(ene),
                 force.ctypes.data_as(Dp), stress.ctypes.data_as(Dp), ctypes.byref(var),
                 ctypes.byref(nsp), ctypes.byref(dl), th.ctypes.data_as(Dp),
                 mm_f.ctypes.data_as(Dp), qmm.ctypes.data_as(Dp), co.ctypes.data_as(Dp),
                 ctypes.byref(rc), ctypes.byref(lg))
    assert abs(ene.value - frames["energy"][f]) <= E_REL * abs(frames["energy"][f])
    assert np.abs(force - frames["forces"][f]).max() <= F_ABS
    assert np.abs(stress - frames["stress"][f]).max() <= S_ABS
    mb = ctypes.c_double()
    L.fget_bond_(ctypes.byref(na), lat_f.ctypes.data_as(Dp), species.ctypes.data_as(ctypes.POINTER(I)),
                 pos_f.ctypes.data_as(Dp), ctypes.byref(rc), ctypes.byref(mb))
    from oracle import oracle
    assert mb.value == oracle.min_bond(frames["cell"][f], frames["positions"][f], 6.0)


def test_bond_and_wacsf_modules(gapgb_mod, oracle_mod, golden_oracle_model, frames, tmp_path,
                                monkeypatch):
    shutil.copy(GOLDEN_MODEL, tmp_path / "gap_parameters")
    monkeypatch.chdir(tmp_path)
    from libgap.BOND import Bond
    from libgap.WACSF import Wacsf
    lat, pos = frames["cell"][7], frames["positions"][7]
    assert Bond(rcut=6.0).get_min_bond(lat, ["C"] * 64, pos) == oracle_mod.min_bond(lat, pos, 6.0)
    xx = Wacsf(rcut=6.0).car2wacsf(lat, ["C"] * 64, pos)
    *_, ex = oracle_mod.gap_calc(golden_oracle_model, frames["numbers"][7], lat, pos, 6.0, False,
                                 extras=True)
    assert np.max(np.abs(xx - ex["xx"]) / (np.abs(ex["xx"]).max(0) + 1e-300)) < 1e-12


# ---------------------------------------------------------------- errors

def test_unknown_species_is_an_error(golden_model, frames, gapgb_mod):
    z = frames["numbers"][0].copy()
    z[5] = 14
    with pytest.raises(gapgb_mod.GapError) as ei:
        golden_model.eval(z, frames["cell"][0], frames["positions"][0])
    assert ei.value.status == 4


def test_image_limit_is_an_error(golden_model, gapgb_mod):
    """A 0.02 A lattice vector needs ~300 images along it, beyond the 127 the
    shift encoding holds: CAP_EXCEEDED, reported before any capacity growth
    (the clamped range overflows every capacity)."""
    lat = np.diag([10.0, 10.0, 0.02])
    pos = np.array([[1.0, 2.0, 0.01]])
    with pytest.raises(gapgb_mod.GapError) as ei:
        golden_model.eval(np.array([6], np.int32), lat, pos)
    assert ei.value.status == 3
    # the model stays usable
    golden_model.set_precision("fp64")
    lat2 = np.eye(3) * 8.0
    E, F, S, _ = golden_model.eval(np.array([6, 6], np.int32), lat2,
                                   np.array([[0.0, 0.0, 0.0], [1.5, 0.2, 0.1]]))
    assert np.isfinite(E)


def test_neighbour_capacity_grows(gapgb_mod, frames):
    m = gapgb_mod.GapModel.load(GOLDEN_MODEL)
    m.set_neighbour_cap(16)
    E, F, S, _ = m.eval(frames["numbers"][0], frames["cell"][0], frames["positions"][0])
    assert abs(E - frames["energy"][0]) <= E_REL * abs(frames["energy"][0])
    assert m.get_option(gapgb_mod.OPT_NEIGHBOUR_CAP) >= 158
    m.close()


def test_device_path_reports_overflow(gapgb_mod, frames):
    import torch
    m = gapgb_mod.GapModel.load(GOLDEN_MODEL)
    m.set_neighbour_cap(32)
    dev = torch.device("cuda:0")
    off = torch.tensor([0, 64], dtype=torch.int32, device=dev)
    sp = torch.tensor(frames["numbers"][0], dtype=torch.int32, device=dev)
    lat = torch.tensor(frames["cell"][0], dtype=torch.float64, device=dev)
    pos = torch.tensor(frames["positions"][0], dtype=torch.float64, device=dev)
    e = torch.zeros(1, dtype=torch.float64, device=dev)
    f = torch.zeros(64, 3, dtype=torch.float64, device=dev)
    s = torch.zeros(6, dtype=torch.float64, device=dev)
    m.eval_batch_ptrs(1, 64, 64, off.data_ptr(), sp.data_ptr(), lat.data_ptr(), pos.data_ptr(), 1,
                      e.data_ptr(), f.data_ptr(), s.data_ptr())
    with pytest.raises(gapgb_mod.GapError) as ei:
        m.check_device_status()
    assert ei.value.status == 5
    # with enough capacity the device path matches the reference frame
    m.set_neighbour_cap(192)
    m.eval_batch_ptrs(1, 64, 64, off.data_ptr(), sp.data_ptr(), lat.data_ptr(), pos.data_ptr(), 1,
                      e.data_ptr(), f.data_ptr(), s.data_ptr())
    m.check_device_status()
    assert abs(e.item() - frames["energy"][0]) <= E_REL * abs(frames["energy"][0])
    assert np.abs(f.cpu().numpy() - frames["forces"][0]).max() <= F_ABS
    m.close()


def test_min_bond_matches_oracle(gapgb_mod, oracle_mod, synth_pop):
    _, _, structs = synth_pop
    for lat, pos, _ in structs:
        assert gapgb_mod.min_bond(lat, pos, 6.0) == oracle_mod.min_bond(lat, pos, 6.0)


# ---------------------------------------------------------------- tensor-core GPR

def test_tc_si_vs_oracle(synth_si, oracle_mod):
    """Split-BF16 tcgen05 GPR (FP32 descriptors) within the reduced-precision bar."""
    import gapgb.synth as S
    g, o = synth_si
    g.set_precision("tc")
    try:
        structs = [S.si64(seed=s) for s in (41, 42, 43)]
        off, sp, lat, pos = S.pack(structs)
        E, F, St = g.eval_batch(off, sp, lat, pos)
        for s, (l, p, z) in enumerate(structs):
            oE, oF, oS, _ = oracle_mod.gap_calc(o, z, l, p, 6.0, True)
            assert abs(E[s] - oE) / len(p) <= 1e-3
            assert np.abs(F[off[s]:off[s + 1]] - oF).max() <= 20e-3
    finally:
        g.set_precision("fp64")


def test_tc_matches_fp32_path_alloy(gapgb_mod, oracle_mod, tmp_path):
    """TC and FP32 forms on the alloy workload (M = 600, many atom tiles)."""
    import gapgb.synth as S
    path = str(tmp_path / "gp")
    synth_model_file(path, oracle_mod, [S.alloy512(seed=s) for s in range(2)], M=600,
                     theta_scale=0.8, coeff_std=1e-2, seed=2)
    m = gapgb_mod.GapModel.load(path)
    structs = [S.alloy512(seed=s) for s in (50, 51)]
    off, sp, lat, pos = S.pack(structs)
    m.set_precision("fp32")
    E32, F32, S32 = m.eval_batch(off, sp, lat, pos)
    m.set_precision("tc")
    Etc, Ftc, Stc = m.eval_batch(off, sp, lat, pos)
    assert np.abs(Etc - E32).max() / 512 <= 1e-4
    assert np.abs(Ftc - F32).max() <= 2e-3
    o = oracle_mod.Model(path)
    l, p, z = structs[1]
    oE, oF, _, _ = oracle_mod.gap_calc(o, z, l, p, 6.0, True)
    assert abs(Etc[1] - oE) / 512 <= 1e-3
    assert np.abs(Ftc[512:] - oF).max() <= 20e-3
    m.close()


def test_tf32_alloy_and_si_vs_oracle(gapgb_mod, oracle_mod, synth_si, tmp_path):
    """Single-term TF32 tensor-core GPR (kind::tf32, FP32 accumulation) within the
    reduced-precision bar, on the alloy model (M = 600) and the Si model."""
    import gapgb.synth as S
    path = str(tmp_path / "gp")
    synth_model_file(path, oracle_mod, [S.alloy512(seed=s) for s in range(2)], M=600,
                     theta_scale=0.8, coeff_std=1e-2, seed=2)
    m = gapgb_mod.GapModel.load(path)
    structs = [S.alloy512(seed=s) for s in (52, 53)]
    off, sp, lat, pos = S.pack(structs)
    m.set_precision("tc")
    Etc, Ftc, Stc = m.eval_batch(off, sp, lat, pos)
    m.set_precision("tf32")
    E, F, St = m.eval_batch(off, sp, lat, pos)
    o = oracle_mod.Model(path)
    for s_, (l, p, z) in enumerate(structs):
        oE, oF, oS, _ = oracle_mod.gap_calc(o, z, l, p, 6.0, True)
        print("tf32 alloy: dE/atom %.3g eV, dF %.3g eV/A; tc: %.3g, %.3g" % (
            abs(E[s_] - oE) / 512, np.abs(F[512 * s_:512 * (s_ + 1)] - oF).max(),
            abs(Etc[s_] - oE) / 512, np.abs(Ftc[512 * s_:512 * (s_ + 1)] - oF).max()))
        assert abs(E[s_] - oE) / 512 <= 1e-3
        assert np.abs(F[512 * s_:512 * (s_ + 1)] - oF).max() <= 20e-3
    m.close()
    # The Si test model is stiff (coefficients ~ N(0, 1): forces ~ 100 eV/A).
    # Single TF32 products keep 11 significant bits, so the form's error is
    # relative (~1e-3 of the force scale): inside the absolute bar for the
    # alloy above, not for forces this large - which the split-BF16x3 form
    # (~2^-22 relative) handles.  Checked here as a relative bound.
    g, og = synth_si
    g.set_precision("tf32")
    try:
        si = [S.si64(seed=s) for s in (71, 72)]
        off, sp, lat, pos = S.pack(si)
        E, F, St = g.eval_batch(off, sp, lat, pos)
        for s_, (l, p, z) in enumerate(si):
            oE, oF, _, _ = oracle_mod.gap_calc(og, z, l, p, 6.0, True)
            assert abs(E[s_] - oE) / len(p) <= 1e-3
            assert np.abs(F[off[s_]:off[s_ + 1]] - oF).max() <= 5e-3 * np.abs(oF).max()
    finally:
        g.set_precision("fp64")


def test_tc_rejects_long_descriptors(golden_model, gapgb_mod):
    for prec in ("tc", "tf32"):
        with pytest.raises(gapgb_mod.GapError) as ei:
            golden_model.set_precision(prec)
        assert ei.value.status == 3


def test_fp32_fast_and_generic_kernels_agree(synth_si, oracle_mod):
    """The register/queue fast path and the generic FP32 descriptor kernels."""
    import gapgb
    import gapgb.synth as S
    g, o = synth_si
    structs = [S.si64(seed=s) for s in (61, 62)]
    off, sp, lat, pos = S.pack(structs)
    g.set_precision("fp32")
    try:
        load = gapgb.load()
        load.gapgb_set_option(g.handle, 3, 1)
        Eg, Fg, Sg = g.eval_batch(off, sp, lat, pos)
        load.gapgb_set_option(g.handle, 3, 0)
        Ef, Ff, Sf = g.eval_batch(off, sp, lat, pos)
        assert np.abs(Ef - Eg).max() <= 1e-5 * np.abs(Eg).max()
        assert np.abs(Ff - Fg).max() <= 1e-4 * max(1.0, np.abs(Fg).max())
        assert np.abs(Sf - Sg).max() <= 1e-4 * max(1.0, np.abs(Sg).max())
        oE, oF, _, _ = oracle_mod.gap_calc(o, structs[0][2], structs[0][0], structs[0][1], 6.0, True)
        assert abs(Ef[0] - oE) / 64 <= 1e-3 and np.abs(Ff[:64] - oF).max() <= 20e-3
    finally:
        g.set_precision("fp64")


# ---------------------------------------------------------------- graphs and tuning

def _dev_batch(batch):
    import torch
    import gapgb.synth as S
    off, sp, lat, pos = S.pack(batch)
    dev = torch.device("cuda:0")
    t = dict(off=torch.from_numpy(off).to(dev), sp=torch.from_numpy(sp).to(dev),
             lat=torch.from_numpy(lat).to(dev), pos=torch.from_numpy(pos).to(dev))
    S_, N = len(batch), int(off[-1])
    t["E"] = torch.zeros(S_, dtype=torch.float64, device=dev)
    t["F"] = torch.zeros(N, 3, dtype=torch.float64, device=dev)
    t["S"] = torch.zeros(S_, 6, dtype=torch.float64, device=dev)
    return (off, sp, lat, pos), t


def test_graph_replay_matches_direct(synth_pop):
    """A captured graph replays the evaluation bit for bit and follows new
    positions written into its bound buffers."""
    import torch
    import gapgb.synth as S
    g, _, _ = synth_pop
    g.set_precision("fp64")
    rng = np.random.default_rng(12)
    batch = [S.random_structure(rng, n, species_pool=(3, 8, 14, 26)) for n in (9, 30, 21)]
    (off, sp, lat, pos), t = _dev_batch(batch)
    nmax = int(np.diff(off).max())
    gr = g.graph(len(batch), int(off[-1]), nmax, t["off"].data_ptr(), t["sp"].data_ptr(),
                 t["lat"].data_ptr(), t["pos"].data_ptr(), 1, t["E"].data_ptr(),
                 t["F"].data_ptr(), t["S"].data_ptr())
    stream = torch.cuda.current_stream().cuda_stream
    gr.launch(stream)
    torch.cuda.synchronize()
    g.check_device_status()
    E0, F0, S0 = g.eval_batch(off, sp, lat, pos)
    assert np.array_equal(t["E"].cpu().numpy(), E0)
    assert np.array_equal(t["F"].cpu().numpy(), F0)
    pos2 = pos + rng.normal(0, 0.02, pos.shape)
    t["pos"].copy_(torch.from_numpy(pos2))
    gr.launch(stream)
    torch.cuda.synchronize()
    g.check_device_status()
    E2, F2, _ = g.eval_batch(off, sp, lat, pos2)
    assert np.array_equal(t["E"].cpu().numpy(), E2)
    assert np.array_equal(t["F"].cpu().numpy(), F2)
    gr.close()


def test_graph_follows_new_coefficients_and_pins_its_buffers(gapgb_mod, oracle_mod, tmp_path):
    """A graph captured on the tensor-core form replays with coefficients set
    after the capture (the operand image is rewritten in place), and while it
    is alive the model refuses what would move the buffers it captured: a
    precision change, or a batch larger than the workspace."""
    import torch
    import gapgb.synth as S
    path = str(tmp_path / "gp")
    synth_model_file(path, oracle_mod, [S.si64(seed=s) for s in range(2)], M=200, seed=3)
    m = gapgb_mod.GapModel.load(path)
    m.set_precision("tc")
    batch = [S.si64(seed=40 + s, jitter=0.1) for s in range(3)]
    (off, sp, lat, pos), t = _dev_batch(batch)
    gr = m.graph(len(batch), int(off[-1]), int(np.diff(off).max()), t["off"].data_ptr(),
                 t["sp"].data_ptr(), t["lat"].data_ptr(), t["pos"].data_ptr(), 1,
                 t["E"].data_ptr(), t["F"].data_ptr(), t["S"].data_ptr())
    stream = torch.cuda.current_stream().cuda_stream
    gr.launch(stream)
    torch.cuda.synchronize()
    m.check_device_status()
    E1, F1 = t["E"].cpu().numpy().copy(), t["F"].cpu().numpy().copy()
    m.set_coeff(2.0 * m.arrays()[2])
    gr.launch(stream)
    torch.cuda.synchronize()
    m.check_device_status()
    E2, F2 = t["E"].cpu().numpy(), t["F"].cpu().numpy()
    # the energy is linear in c; forces too, to the resolution of the
    # gradient kernel's fixed-point slot sums (each term rounded to 2^-29
    # eV/A, a few hundred terms per force); a stale image would be off by
    # |F1|, here about 0.07 eV/A
    assert np.allclose(E2, 2.0 * E1, rtol=1e-12, atol=0.0)
    assert np.abs(F2 - 2.0 * F1).max() <= 1e-6
    # the host-buffer path (same sizes: the workspace stays) agrees; a stale
    # image would be off by a factor of two
    Eh, Fh, _ = m.eval_batch(off, sp, lat, pos)
    assert np.allclose(E2, Eh, rtol=1e-6, atol=0.0)
    assert np.abs(F2 - Fh).max() <= 1e-5 * np.abs(F2).max()
    with pytest.raises(gapgb_mod.GapError):
        m.set_precision("fp64")
    o2, s2, l2, p2 = S.pack(batch * 4)
    with pytest.raises(gapgb_mod.GapError):
        m.eval_batch(o2, s2, l2, p2)
    gr.close()
    m.set_precision("fp64")
    E3, _, _ = m.eval_batch(o2, s2, l2, p2)
    assert np.allclose(E3[:3], E3[3:6], rtol=0.0, atol=1e-9 * np.abs(E3).max())
    m.close()


def test_autotune_choice_within_tolerance(synth_si):
    import gapgb.synth as S
    from gapgb import tune
    g, _ = synth_si
    batch = [S.si64(seed=s) for s in (71, 72, 73, 74)]
    off, sp, lat, pos = S.pack(batch)
    best = tune.autotune(g, off, sp, lat, pos, reps=2)
    # any form the tuner can return is acceptable, as long as its measured
    # errors against the FP64 form pass the gates
    assert best["precision"] in tune.FORMS
    assert best["dE_per_atom"] <= 1e-3 and best["dF"] <= 20e-3
    E, F, _ = g.eval_batch(off, sp, lat, pos)
    g.set_precision("fp64")
    E64, F64, _ = g.eval_batch(off, sp, lat, pos)
    assert np.max(np.abs(E - E64)) / 64 <= 1e-3 and np.abs(F - F64).max() <= 20e-3
    g.set_neighbour_cap(256)
    gapgb_load = __import__("gapgb").load()
    gapgb_load.gapgb_set_option(g.handle, 3, 0)
