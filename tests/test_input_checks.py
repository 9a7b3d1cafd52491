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
