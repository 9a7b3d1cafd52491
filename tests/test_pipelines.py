"""Two pipelines (GAPGB_OPT_PIPELINES = 2): a large tensor-core batch runs as
two halves of the atom range on two streams.  The halves split at a multiple
of the 128-atom GPR tile, here inside a structure (41 alloy512 cells, split
at atom 10 496 of cell 20), so the force scatter of one half adds onto atoms
of the other.  The results must equal the one-stream evaluation: energies
and stresses bit for bit (per-atom sums in a fixed order), forces to FP64
rounding (the scatter's atomics add in another order), directly and through a
captured CUDA graph; and one straddling cell must match the oracle.
"""
import numpy as np
import pytest

from helpers import write_model_file

pytestmark = pytest.mark.gpu

NCELLS = 41  # 20 992 atoms: above the 20 480-atom threshold, split inside cell 20


@pytest.fixture(scope="module")
def alloy(gapgb_mod):
    import gapgb.synth as S
    arrays = S.alloy_model(M=600, theta_scale=0.8, coeff_std=1e-3, seed=2, ncells=4)
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    m = gapgb_mod.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
    m.set_neighbour_cap(96)
    structs = [S.alloy512(seed=300 + s) for s in range(NCELLS)]
    yield m, arrays, structs
    m.close()


@pytest.mark.parametrize("prec", ["tc", "tf32"])
def test_two_pipelines_match_one(alloy, prec):
    import gapgb.synth as S
    m, _, structs = alloy
    off, sp, lat, pos = S.pack(structs)
    m.set_precision(prec)
    m.set_pipelines(1)
    E1, F1, S1 = m.eval_batch(off, sp, lat, pos)
    m.set_pipelines(2)
    E2, F2, S2 = m.eval_batch(off, sp, lat, pos)
    assert np.array_equal(E1, E2)
    assert np.array_equal(S1, S2)
    np.testing.assert_allclose(F2, F1, rtol=0, atol=1e-12)
    assert np.abs(F1).max() > 1e-3  # forces of this smooth model are a few 10 meV/A


def test_two_pipelines_in_a_graph(alloy):
    import torch
    import gapgb.synth as S
    m, _, structs = alloy
    off, sp, lat, pos = S.pack(structs)
    m.set_precision("tc")
    m.set_pipelines(2)
    E0, F0, S0 = m.eval_batch(off, sp, lat, pos)
    dev = torch.device("cuda:0")
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
         for k, v in (("off", off), ("sp", sp), ("lat", lat), ("pos", pos))}
    N = int(off[-1])
    E = torch.zeros(len(structs), dtype=torch.float64, device=dev)
    F = torch.zeros(N, 3, dtype=torch.float64, device=dev)
    St = torch.zeros(len(structs), 6, dtype=torch.float64, device=dev)
    gr = m.graph(len(structs), N, 512, t["off"].data_ptr(), t["sp"].data_ptr(),
                 t["lat"].data_ptr(), t["pos"].data_ptr(), 1, E.data_ptr(), F.data_ptr(),
                 St.data_ptr())
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        gr.launch(stream)
    torch.cuda.synchronize()
    m.check_device_status()
    gr.close()
    assert np.array_equal(E.cpu().numpy(), E0)
    assert np.array_equal(St.cpu().numpy(), S0)
    np.testing.assert_allclose(F.cpu().numpy(), F0, rtol=0, atol=1e-12)


def test_straddling_cell_matches_oracle(alloy, oracle_mod, tmp_path):
    import gapgb.synth as S
    m, arrays, structs = alloy
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    off, sp, lat, pos = S.pack(structs)
    h = (int(off[-1]) // 2) // 128 * 128
    s = int(np.searchsorted(off, h, side="right")) - 1
    assert off[s] < h < off[s + 1]  # the split falls inside cell s
    m.set_precision("tc")
    m.set_pipelines(2)
    E, F, St = m.eval_batch(off, sp, lat, pos)
    o = oracle_mod.Model(write_model_file(str(tmp_path / "gp"), zt, wt, ty, al, rc, theta, mm,
                                          coeff, ze))
    l, p, z = structs[s]
    oE, oF, oS, _ = oracle_mod.gap_calc(o, z, l, p, 6.0, True)
    assert abs(E[s] - oE) / len(p) <= 1e-3
    assert np.abs(F[off[s]:off[s + 1]] - oF).max() <= 20e-3
    assert np.abs(St[s] - oS).max() <= 1e-2


def test_slot_sums_repeat(alloy):
    """The grouped gradient kernel sums slot gradients in fixed point, so the
    per-atom virials, hence the stresses, are the same bit for bit in every
    run; only the forces' FP64 scatter atomics may add in another order."""
    import gapgb.synth as S
    m, _, structs = alloy
    off, sp, lat, pos = S.pack(structs[:8])
    m.set_precision("tc")
    m.set_pipelines(1)
    runs = [m.eval_batch(off, sp, lat, pos) for _ in range(3)]
    for E, F, St in runs[1:]:
        assert np.array_equal(E, runs[0][0])
        assert np.array_equal(St, runs[0][2])
        np.testing.assert_allclose(F, runs[0][1], rtol=0, atol=1e-12)
