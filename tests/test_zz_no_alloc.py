"""gapgb_gpr_noalloc through the C ABI, checked against the library's regular
path.

The entry point computes the sparse-GPR energies and dE/dG without any
device allocation (its working memory is a fixed array in device memory).
It is for callers that cannot allocate at that point: hosts that keep all
device memory in their own pool, where a cudaMalloc behind their back fails
or eats into the pool, and loops that cannot take the synchronisation of a
cudaMalloc / cudaFree.  This file is collected last so that a run stopping
at the first failure has already run every other test; it builds everything
it needs itself, so it also passes alone in a fresh process.
"""
import numpy as np
import pytest

from helpers import synth_model_file

pytestmark = pytest.mark.gpu

E_REL = 1e-9  # the FP64 tolerance of the parity tests
SCRATCH_DOUBLES = 1 << 20  # the entry point's fixed scratch


def _model(gapgb_mod, oracle_mod, tmp_path):
    import gapgb.synth as S
    path = synth_model_file(str(tmp_path / "gap_parameters"), oracle_mod,
                            [S.si64(seed=s) for s in range(2)], M=200, theta_scale=1.0,
                            coeff_std=1.0, seed=4)
    m = gapgb_mod.GapModel.load(path)
    m.set_precision("fp64")
    return path, m


def _gpr_fp64_torch(G, mm, theta, coeff):
    """Plain torch FP64 statement of GET_COV, the energy and dE/dG
    (gap_calc.f90:143-166): e_i = sum_k c_k K_ik,
    dedg_id = -sum_k (x_id - m_kd) / theta_d^2 K_ik c_k."""
    import torch
    e, dedg = [], []
    for a in range(0, G.shape[0], 2048):
        x = G[a:a + 2048]
        diff = (x[:, None, :] - mm[None, :, :]) / theta
        w = torch.exp(-0.5 * (diff * diff).sum(-1)) * coeff
        e.append(w.sum(1))
        dedg.append(-(diff * w[:, :, None]).sum(1) / theta)
    return torch.cat(e), torch.cat(dedg)


def test_noalloc_gpr_matches_regular_path(gapgb_mod, oracle_mod, tmp_path):
    import torch
    import gapgb.synth as S
    path, m = _model(gapgb_mod, oracle_mod, tmp_path)
    o = oracle_mod.Model(path)
    L = gapgb_mod.load()
    dev = torch.device("cuda:0")
    # two calls in a row, on batches of different sizes
    for seeds in ((81, 82, 83), (84,)):
        structs = [S.si64(seed=s) for s in seeds]
        off, sp, lat, pos = S.pack(structs)
        # the regular path (it also makes the model resident on the device)
        _, _, _, ae = m.eval_batch(off, sp, lat, pos, atom_energy=True)
        xx = m.descriptors(off, sp, lat, pos)
        N, D = xx.shape
        d_G = torch.from_numpy(xx).to(dev)
        d_e = torch.full((N,), np.nan, dtype=torch.float64, device=dev)
        d_dedg = torch.full((N, D), np.nan, dtype=torch.float64, device=dev)
        st = L.gapgb_gpr_noalloc(m.handle, N, d_G.data_ptr(), d_e.data_ptr(), d_dedg.data_ptr(),
                                 None)
        assert st == 0, gapgb_mod.last_error()
        torch.cuda.synchronize()
        e = d_e.cpu().numpy()
        dedg = d_dedg.cpu().numpy()
        assert np.abs(e - ae).max() <= E_REL * max(1.0, np.abs(ae).max())
        for s, (l, p, z) in enumerate(structs):
            *_, ex = oracle_mod.gap_calc(o, z, l, p, 6.0, True, extras=True)
            ref = ex["dedg"]
            assert np.abs(dedg[off[s]:off[s + 1]] - ref).max() <= E_REL * max(1.0, np.abs(ref).max())
    # sizes beyond the fixed scratch are refused, not allocated for
    st = L.gapgb_gpr_noalloc(m.handle, 1 << 20, d_G.data_ptr(), d_e.data_ptr(),
                             d_dedg.data_ptr(), None)
    assert st == 3
    assert "exceeds the fixed scratch" in gapgb_mod.last_error()
    m.close()


def test_noalloc_gpr_at_the_size_limit_allocates_nothing(gapgb_mod, oracle_mod, tmp_path):
    """250 Si cells (16000 atoms, natoms * (D + 1) just under the scratch
    size): energies against the regular path, dE/dG against a plain torch
    FP64 statement, two calls in a row, and free device memory unchanged
    across the calls (read after a warm call, with nothing else running)."""
    import torch
    import gapgb.synth as S
    _, m = _model(gapgb_mod, oracle_mod, tmp_path)
    L = gapgb_mod.load()
    dev = torch.device("cuda:0")
    structs = [S.si64(seed=1000 + s) for s in range(250)]
    off, sp, lat, pos = S.pack(structs)
    _, _, _, ae = m.eval_batch(off, sp, lat, pos, atom_energy=True)
    xx = m.descriptors(off, sp, lat, pos)
    N, D = xx.shape
    assert N * (D + 1) <= SCRATCH_DOUBLES < (N + 250) * (D + 1)
    theta, mm, coeff = m.arrays()
    d_G = torch.from_numpy(xx).to(dev)
    ref_e, ref_d = _gpr_fp64_torch(d_G, torch.from_numpy(mm).to(dev),
                                   torch.from_numpy(theta).to(dev),
                                   torch.from_numpy(coeff).to(dev))
    ref_e, ref_d = ref_e.cpu().numpy(), ref_d.cpu().numpy()
    d_e = torch.empty((N,), dtype=torch.float64, device=dev)
    d_dedg = torch.empty((N, D), dtype=torch.float64, device=dev)

    def call():
        st = L.gapgb_gpr_noalloc(m.handle, N, d_G.data_ptr(), d_e.data_ptr(),
                                 d_dedg.data_ptr(), None)
        assert st == 0, gapgb_mod.last_error()

    call()  # warm: the one-time set-up on this device
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(dev)
    for _ in range(2):
        d_e.fill_(np.nan)
        d_dedg.fill_(np.nan)
        call()
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info(dev)
        assert free1 == free0
        e = d_e.cpu().numpy()
        dedg = d_dedg.cpu().numpy()
        assert np.abs(e - ae).max() <= E_REL * max(1.0, np.abs(ae).max())
        assert np.abs(e - ref_e).max() <= E_REL * max(1.0, np.abs(ref_e).max())
        assert np.abs(dedg - ref_d).max() <= E_REL * max(1.0, np.abs(ref_d).max())
    # one atom more than the scratch holds is refused
    nmax = SCRATCH_DOUBLES // (D + 1)
    st = L.gapgb_gpr_noalloc(m.handle, nmax + 1, d_G.data_ptr(), d_e.data_ptr(),
                             d_dedg.data_ptr(), None)
    assert st == 3
    m.close()
