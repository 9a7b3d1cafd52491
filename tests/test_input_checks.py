"""Invalid geometry through the host-buffer call: the checks run on the host
(while the inputs are being copied) and end the call before any kernel is
launched; the model stays usable."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_MODEL

pytestmark = pytest.mark.gpu

ERR_ARG = 8  # GAPGB_ERR_ARG (include/gapgb.h)


def test_non_finite_and_singular_inputs_are_refused(gapgb_mod):
    fr = np.load(os.path.join(GOLDEN, "ase_traj_frames.npz"))
    z, lat, pos = fr["numbers"][0], fr["cell"][0], fr["positions"][0]
    m = gapgb_mod.GapModel.load(GOLDEN_MODEL)
    try:
        E0, F0, S0, _ = m.eval(z, lat, pos)
        bad = pos.copy()
        bad[5, 1] = np.nan
        with pytest.raises(gapgb_mod.GapError) as e:
            m.eval(z, lat, bad)
        assert e.value.status == ERR_ARG
        bad[5, 1] = np.inf
        with pytest.raises(gapgb_mod.GapError):
            m.eval(z, lat, bad)
        flat = lat.copy()
        flat[2] = flat[0] + flat[1]  # linearly dependent rows: det = 0
        with pytest.raises(gapgb_mod.GapError) as e:
            m.eval(z, flat, pos)
        assert e.value.status == ERR_ARG
        E1, F1, S1, _ = m.eval(z, lat, pos)  # the model is unaffected
        assert E1 == E0 and np.array_equal(F1, F0) and np.array_equal(S1, S0)
    finally:
        m.close()


ERR_CAP = 3  # GAPGB_ERR_CAP_EXCEEDED


def test_fp32_gradient_range_is_reported(gapgb_mod):
    """The FP32 forms sum slot gradients in fixed point, for terms up to 2047
    eV/A.  A model whose terms exceed that (coefficients scaled by 1e8) is
    refused with GAPGB_ERR_CAP_EXCEEDED in an FP32 form; the FP64 form
    evaluates it, and once the coefficients are restored the FP32 form gives
    its earlier results again."""
    import gapgb.synth as S
    zt, wt, ty, al, rc, ze, theta, mm, coeff = S.alloy_model(M=200, seed=2, ncells=2)
    m = gapgb_mod.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
    try:
        m.set_neighbour_cap(96)
        off, sp, lat, pos = S.pack([S.alloy512(seed=7)])
        m.set_precision("fp32")
        E0, F0, S0 = m.eval_batch(off, sp, lat, pos)
        m.set_coeff(coeff * 1e8)
        with pytest.raises(gapgb_mod.GapError) as e:
            m.eval_batch(off, sp, lat, pos)
        assert e.value.status == ERR_CAP
        m.set_precision("fp64")
        _, F64, _ = m.eval_batch(off, sp, lat, pos)
        assert np.abs(F64).max() > 2047.0
        m.set_precision("fp32")
        m.set_coeff(coeff)
        E1, F1, S1 = m.eval_batch(off, sp, lat, pos)
        assert np.array_equal(E1, E0) and np.array_equal(S1, S0)
        np.testing.assert_allclose(F1, F0, rtol=0, atol=1e-12)  # FP64 scatter order
    finally:
        m.close()
