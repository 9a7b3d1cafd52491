"""GPR predictive variance (gapgb_model_set_qmm / gapgb_variance).

The reference carries the variance block of FGAP_CALC commented out
(gap_calc.f90:206-210: covf(i) = delta - ckm(i,:).matmul(qmm, ckm(i,:)),
VARIANCE = mean covf) and zero-fills qmm, so it has no outputs to compare
with.  The oracle's restatement (oracle.variance) is pinned against an
independent numpy statement of the same formula on the reference's example
model (CPU), and the CUDA forms are compared with the oracle (GPU).
"""
import numpy as np
import pytest

from conftest import GOLDEN_MODEL
from helpers import synth_model_file


def _kmat(xx, mm, theta):
    return np.exp(-0.5 * (((xx[:, None, :] - mm[None, :, :]) / theta) ** 2).sum(-1))


def _qmm(mm, theta, lam):
    """(K_MM + lam I)^-1: the inverse covariance of a sparse set with jitter."""
    return np.linalg.inv(_kmat(mm, mm, theta) + lam * np.eye(len(mm)))


def test_oracle_variance_matches_numpy(oracle_mod, golden_oracle_model, frames):
    o = golden_oracle_model
    z, lat, pos = frames["numbers"][0], frames["cell"][0], frames["positions"][0]
    *_, ex = oracle_mod.gap_calc(o, z, lat, pos, 6.0, False, extras=True)
    xx = ex["xx"]
    K = _kmat(xx, o.mm, o.theta)
    Q = _qmm(o.mm, o.theta, 1e-2)
    covf, var = oracle_mod.variance(o, xx, Q)
    ref = 1.0 - np.einsum("im,mn,in->i", K, Q, K)
    assert np.abs(covf - ref).max() <= 1e-11
    assert var == pytest.approx(ref.mean(), abs=1e-12)
    # the qmm FGAP_READ leaves (zeros): covf = delta
    c0, v0 = oracle_mod.variance(o, xx, np.zeros_like(Q))
    assert np.all(c0 == 1.0) and v0 == pytest.approx(1.0, abs=1e-14)
    # a non-symmetric qmm enters as written, matmul(qmm, k)
    A = np.random.default_rng(0).normal(size=Q.shape) * 1e-3
    ca, _ = oracle_mod.variance(o, xx, A)
    assert np.abs(ca - (1.0 - np.einsum("im,mn,in->i", K, A, K))).max() <= 1e-12


def test_set_qmm_checks_the_size(gapgb_mod):
    import ctypes
    m = gapgb_mod.GapModel.load(GOLDEN_MODEL)
    q = np.zeros((m.nsparse, m.nsparse))
    assert gapgb_mod.load().gapgb_model_set_qmm(m.handle, q.ctypes.data, m.nsparse - 1) == 8
    m.set_qmm(q)
    m.set_qmm(None)
    m.close()


def _oracle_covf(oracle_mod, o, structs, Q):
    out = []
    for lat, pos, z in structs:
        *_, ex = oracle_mod.gap_calc(o, z, lat, pos, 6.0, False, extras=True)
        out.append(oracle_mod.variance(o, ex["xx"], Q))
    return np.concatenate([c for c, _ in out]), np.array([v for _, v in out])


def _tol(scale):
    """Bound of the tensor-core contraction against the FP64 one on the same
    descriptors: split-BF16 products and FP32 accumulation err by ~1e-5 of
    the terms that cancel; the floor covers atoms whose K row underflows FP32
    (their covf is delta to far below it)."""
    return 5e-5 * scale + 1e-7


def _scale(oracle_mod, o, structs, Q):
    """sum_mn |K_im| |Q_mn| |K_in| per atom: the size of the terms that cancel."""
    out = []
    for lat, pos, z in structs:
        *_, ex = oracle_mod.gap_calc(o, z, lat, pos, 6.0, False, extras=True)
        K = _kmat(ex["xx"], o.mm, o.theta)
        out.append(np.einsum("im,mn,in->i", K, np.abs(Q), K))
    return np.concatenate(out)


@pytest.fixture(scope="module")
def si_var(oracle_mod, tmp_path_factory):
    import gapgb.synth as S
    path = str(tmp_path_factory.mktemp("var") / "gap_parameters")
    synth_model_file(path, oracle_mod, [S.si64(seed=s) for s in range(3)], M=300,
                     theta_scale=1.0, coeff_std=1.0, seed=1)
    o = oracle_mod.Model(path)
    Q = _qmm(o.mm, o.theta, 1e-2)
    structs = [S.si64(seed=30 + s, jitter=0.08) for s in range(3)]
    covf, var = _oracle_covf(oracle_mod, o, structs, Q)
    return path, Q, structs, covf, var, _scale(oracle_mod, o, structs, Q)


@pytest.mark.gpu
def test_variance_fp64_matches_oracle(gapgb_mod, si_var):
    import gapgb.synth as S
    path, Q, structs, rc, rv, _ = si_var
    m = gapgb_mod.GapModel.load(path)
    m.set_precision("fp64")
    with pytest.raises(gapgb_mod.GapError) as ei:
        m.variance(*S.pack(structs))
    assert ei.value.status == 8  # no qmm attached
    m.set_qmm(Q)
    covf, var = m.variance(*S.pack(structs))
    print("fp64 variance vs oracle: max |dcovf| %.3g (covf %.4g..%.4g)"
          % (np.abs(covf - rc).max(), rc.min(), rc.max()))
    assert np.abs(covf - rc).max() <= 1e-9
    assert np.abs(var - rv).max() <= 1e-9
    # gapgb_eval reports the mean covf while a qmm is attached, 0 otherwise
    lat, pos, z = structs[1]
    v = m.eval(z, lat, pos)[3]
    assert abs(v - rv[1]) <= 1e-9
    m.set_qmm(None)
    assert m.eval(z, lat, pos)[3] == 0.0
    m.close()


@pytest.mark.gpu
def test_variance_reduced_forms(gapgb_mod, si_var):
    """The error sources one at a time.  mixed (FP32 descriptors, FP64 K and
    contraction) against the oracle: the descriptors' FP32 rounding, an
    absolute bar on covf.  tc and fp32 (FP32 K, tcgen05 split-BF16 products,
    FP32 accumulation) against mixed on the same descriptors: the
    contraction, bounded relative to sum |K||Q||K|, the size of the terms
    that cancel in k^T Q k (a numpy emulation of the split-BF16 arithmetic
    errs by 5e-6 of it)."""
    import gapgb.synth as S
    path, Q, structs, rc, rv, scale = si_var
    m = gapgb_mod.GapModel.load(path)
    m.set_qmm(Q)
    out = {}
    for prec in ("mixed", "tc", "fp32"):
        m.set_precision(prec)
        out[prec] = m.variance(*S.pack(structs))
    dm = np.abs(out["mixed"][0] - rc)
    print("mixed vs oracle: max |dcovf| %.3g" % dm.max())
    assert dm.max() <= 1e-4 and np.abs(out["mixed"][1] - rv).max() <= 1e-4
    for prec in ("tc", "fp32"):
        d = np.abs(out[prec][0] - out["mixed"][0])
        do = np.abs(out[prec][0] - rc)
        print("%s vs mixed: max |dcovf| %.3g, max / tol %.3g; vs oracle %.3g (scale %.3g..%.3g)"
              % (prec, d.max(), (d / _tol(scale)).max(), do.max(), scale.min(), scale.max()))
        assert np.all(d <= _tol(scale))
        assert do.max() <= 2e-3
    assert np.array_equal(out["tc"][0], out["fp32"][0])
    m.close()


@pytest.mark.gpu
def test_variance_tc_alloy_many_tiles(gapgb_mod, oracle_mod, tmp_path):
    """M = 600 (three 256-wide column tiles, padded) and 1024 atoms (eight
    128-atom tiles): tensor-core form against the FP64 form and the oracle."""
    import gapgb.synth as S
    path = str(tmp_path / "gp")
    synth_model_file(path, oracle_mod, [S.alloy512(seed=s) for s in range(2)], M=600,
                     theta_scale=0.8, coeff_std=1e-2, seed=2)
    o = oracle_mod.Model(path)
    Q = _qmm(o.mm, o.theta, 3e-2)
    structs = [S.alloy512(seed=s) for s in (60, 61)]
    off, sp, lat, pos = S.pack(structs)
    m = gapgb_mod.GapModel.load(path)
    m.set_qmm(Q)
    m.set_precision("fp64")
    c64, v64 = m.variance(off, sp, lat, pos)
    m.set_precision("mixed")
    cmx, _ = m.variance(off, sp, lat, pos)
    m.set_precision("tc")
    ctc, vtc = m.variance(off, sp, lat, pos)
    rc, rv = _oracle_covf(oracle_mod, o, structs[1:], Q)
    scale = _scale(oracle_mod, o, structs[1:], Q)
    d = np.abs(ctc[512:] - cmx[512:])
    print("alloy variance: fp64 vs oracle %.3g; tc vs mixed %.3g (max / tol %.3g); tc vs oracle "
          "%.3g; covf %.4g..%.4g" % (np.abs(c64[512:] - rc).max(), d.max(),
                                    (d / _tol(scale)).max(), np.abs(ctc[512:] - rc).max(),
                                    rc.min(), rc.max()))
    assert np.abs(c64[512:] - rc).max() <= 1e-9
    assert np.all(d <= _tol(scale))
    assert np.abs(ctc[512:] - rc).max() <= 2e-3
    assert np.abs(vtc - v64).max() <= 1e-3
    m.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec,ncells", [("fp64", 136), ("tc", 1026)])
def test_variance_chunks_are_row_independent(gapgb_mod, si_var, prec, ncells):
    """Batches longer than one chunk of atoms (FP64 form: 8192, tensor-core
    form: 65536): a cell after the chunk boundary gets bit for bit the covf
    it gets alone, since every row of K qmm^T is its own."""
    import gapgb.synth as S
    path, Q, *_ = si_var
    m = gapgb_mod.GapModel.load(path)
    m.set_precision(prec)
    m.set_qmm(Q)
    cells = [S.si64(seed=700 + s % 7, jitter=0.08) for s in range(ncells - 1)]
    cells.append(S.si64(seed=999, jitter=0.08))
    off, sp, lat, pos = S.pack(cells)
    covf, var = m.variance(off, sp, lat, pos)
    last = S.pack(cells[-1:])
    c1, v1 = m.variance(*last)
    assert off[-1] > (8192 if prec == "fp64" else 65536)
    assert np.array_equal(covf[int(off[-2]):], c1)
    assert var[-1] == v1[0]
    # the first cells repeat with period 7: their rows agree across the batch
    n7 = int(off[7])
    assert np.array_equal(covf[:n7], covf[n7:2 * n7])
    m.close()
