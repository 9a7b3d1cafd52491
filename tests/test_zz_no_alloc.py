"""gapgb_gpr_noalloc through the C ABI, checked against the library's regular
path.

The entry point computes the sparse-GPR energies and dE/dG without any
device allocation (its working memory is a fixed array in device memory),
for callers that cannot allocate at that point: inside a stream capture, in
hosts that pool all device memory themselves, or in loops that cannot take
an allocation's synchronisation.  This file is collected last so that a run
stopping at the first failure has already run every other test; it builds
everything it needs itself, so it also passes alone in a fresh process.
"""
import numpy as np
import pytest

from helpers import synth_model_file

pytestmark = pytest.mark.gpu

E_REL = 1e-9  # the FP64 tolerance of the parity tests


def test_noalloc_gpr_matches_regular_path(gapgb_mod, oracle_mod, tmp_path):
    import torch
    import gapgb.synth as S
    path = synth_model_file(str(tmp_path / "gap_parameters"), oracle_mod,
                            [S.si64(seed=s) for s in range(2)], M=200, theta_scale=1.0,
                            coeff_std=1.0, seed=4)
    m = gapgb_mod.GapModel.load(path)
    o = oracle_mod.Model(path)
    m.set_precision("fp64")
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
