"""Sparse-GPR fitting from structure energies and forces (gapgb_fit,
gapgb_fit_energies).

The reference only evaluates fitted models (its fitting codes, calypso.x and
ngap.x, are not in the repository), so the oracle here is the same normal
equations written out in numpy on the CPU oracle's FP64 descriptors:
  Phi_sk = sum_{i in s} K(x_i, m_k),  A = K_MM + jitter I + Phi^T W Phi,
  b = Phi^T W E,  W = diag(1 / (sigma_e^2 n_s)),  c = A^-1 b,
plus, with forces and stresses, PhiF^T PhiF / sigma_f^2, PhiF^T F / sigma_f^2
and the same for stress, where column k of PhiF (PhiS) is the oracle's force
field (stress) with coefficients e_k.
"""
import numpy as np
import pytest

from helpers import synth_model_file

pytestmark = pytest.mark.gpu


def _kmat(xx, mm, theta):
    return np.exp(-0.5 * (((xx[:, None, :] - mm[None, :, :]) / theta) ** 2).sum(-1))


def _phi(oracle_mod, o, structs):
    rows = []
    for lat, pos, z in structs:
        *_, ex = oracle_mod.gap_calc(o, z, lat, pos, 6.0, False, extras=True)
        rows.append(_kmat(ex["xx"], o.mm, o.theta).sum(0))
    return np.array(rows)


def _normal(o, phi, E, n, sigma_e, jitter):
    w = 1.0 / (sigma_e ** 2 * n)
    A = _kmat(o.mm, o.mm, o.theta) + jitter * np.eye(len(o.mm)) + (phi * w[:, None]).T @ phi
    b = phi.T @ (w * E)
    return A, b


@pytest.mark.parametrize("kind", ["si", "alloy"])
def test_fit_energies_matches_normal_equations(gapgb_mod, oracle_mod, tmp_path, kind):
    import gapgb.synth as S
    path = str(tmp_path / "gp")
    if kind == "si":
        # M = 300: five 64-wide Cholesky panels, the last one padded
        synth_model_file(path, oracle_mod, [S.si64(seed=s) for s in range(3)], M=300,
                         theta_scale=1.0, coeff_std=0.05, seed=1)
        train = [S.si64(seed=100 + s, jitter=0.1) for s in range(48)]
        test = [S.si64(seed=500 + s, jitter=0.1) for s in range(6)]
    else:
        # M = 600: ten panels; 512-atom structures span many passes of the design-row kernel
        synth_model_file(path, oracle_mod, [S.alloy512(seed=s) for s in range(2)], M=600,
                         theta_scale=0.8, coeff_std=1e-3, seed=2)
        train = [S.alloy512(seed=100 + s) for s in range(12)]
        test = [S.alloy512(seed=500 + s) for s in range(2)]
    o = oracle_mod.Model(path)
    m = gapgb_mod.GapModel.load(path)
    m.set_precision("fp64")
    off, sp, lat, pos = S.pack(train)
    E_teacher, _, _ = m.eval_batch(off, sp, lat, pos, lgrad=False)
    n = np.diff(off).astype(float)
    rng = np.random.default_rng(3)
    E = E_teacher + rng.normal(0, 1e-3, len(n)) * np.sqrt(n)
    sigma_e, jitter = 1e-3, 1e-6
    c = m.fit_energies(off, sp, lat, pos, E, sigma_e=sigma_e, jitter=jitter)
    phi = _phi(oracle_mod, o, train)
    A, b = _normal(o, phi, E, n, sigma_e, jitter)
    c_ref = np.linalg.solve(A, b)
    res = np.linalg.norm(A @ c - b) / (np.linalg.norm(A, 2) * np.linalg.norm(c))
    pred, pred_ref = phi @ c, phi @ c_ref
    phi_t = _phi(oracle_mod, o, test)
    dt = np.abs(phi_t @ c - phi_t @ c_ref).max()
    print("%s fit: backward error %.3g, |c| %.3g, train dE %.3g eV, held-out dE %.3g eV, "
          "train rmse vs labels %.3g eV/atom" % (kind, res, np.abs(c).max(),
                                                np.abs(pred - pred_ref).max(), dt,
                                                np.sqrt(np.mean(((pred - E) / n) ** 2))))
    # Cholesky is backward stable: the device solution solves A to rounding
    assert res <= 1e-12
    # and predicts what the numpy solution predicts (energies of 1e2-1e4 eV)
    assert np.abs(pred - pred_ref).max() <= 1e-6 * np.abs(pred_ref).max()
    assert dt <= 1e-6 * np.abs(phi_t @ c_ref).max()
    # the model now carries the fitted coefficients in every form
    assert np.array_equal(m.arrays()[2], c)
    E_fit, _, _ = m.eval_batch(off, sp, lat, pos, lgrad=False)
    assert np.abs(E_fit - pred_ref).max() <= 1e-6 * np.abs(pred_ref).max()
    m.set_precision("tc")
    E_tc, _, _ = m.eval_batch(off, sp, lat, pos, lgrad=False)
    assert np.abs(E_tc - E_fit).max() / n.min() <= 1e-3
    m.close()


def test_fit_rejects_bad_arguments(gapgb_mod, tmp_path, oracle_mod):
    import gapgb.synth as S
    path = str(tmp_path / "gp")
    synth_model_file(path, oracle_mod, [S.si64(seed=0)], M=50, seed=1)
    m = gapgb_mod.GapModel.load(path)
    off, sp, lat, pos = S.pack([S.si64(seed=1)])
    with pytest.raises(gapgb_mod.GapError) as ei:
        m.fit_energies(off, sp, lat, pos, [0.0], sigma_e=0.0)
    assert ei.value.status == 8
    with pytest.raises(gapgb_mod.GapError):
        m.set_coeff(np.full(m.nsparse, np.nan))
    m.close()


def test_fit_with_forces_and_stress_matches_normal_equations(gapgb_mod, oracle_mod, tmp_path):
    """Energy, force and stress rows.  The oracle's force and stress design
    columns k are the oracle's forces and stress with the coefficients set
    to the unit vector e_k."""
    import gapgb.synth as S
    path = str(tmp_path / "gp")
    synth_model_file(path, oracle_mod, [S.si64(seed=s) for s in range(3)], M=60,
                     theta_scale=1.0, coeff_std=0.05, seed=5)
    o = oracle_mod.Model(path)
    m = gapgb_mod.GapModel.load(path)
    m.set_precision("fp64")
    train = [S.si64(seed=300 + s, jitter=0.1) for s in range(4)]
    off, sp, lat, pos = S.pack(train)
    E, F, St = m.eval_batch(off, sp, lat, pos)  # teacher: the model itself
    n = np.diff(off).astype(float)
    sigma_e, sigma_f, sigma_s, jitter = 1e-3, 1e-2, 1e-2, 1e-8
    c = m.fit(off, sp, lat, pos, E, forces=F, stress=St, sigma_e=sigma_e, sigma_f=sigma_f,
              sigma_s=sigma_s, jitter=jitter)
    # oracle design matrices
    phi = _phi(oracle_mod, o, train)
    cview = np.ctypeslib.as_array(o._m.coeff, (o.M,))
    saved = cview.copy()
    phif = np.zeros((3 * len(sp), o.M))
    phis = np.zeros((6 * len(train), o.M))
    for k in range(o.M):
        cview[:] = 0.0
        cview[k] = 1.0
        outs = [oracle_mod.gap_calc(o, z, l, p, 6.0, True) for l, p, z in train]
        phif[:, k] = np.concatenate([x[1].ravel() for x in outs])
        phis[:, k] = np.concatenate([x[2] for x in outs])
    cview[:] = saved
    A, b = _normal(o, phi, E, n, sigma_e, jitter)
    A = A + phif.T @ phif / sigma_f ** 2 + phis.T @ phis / sigma_s ** 2
    b = b + phif.T @ F.ravel() / sigma_f ** 2 + phis.T @ St.ravel() / sigma_s ** 2
    c_ref = np.linalg.solve(A, b)
    res = np.linalg.norm(A @ c - b) / (np.linalg.norm(A, 2) * np.linalg.norm(c))
    df = np.abs(phif @ c - phif @ c_ref).max()
    ds = np.abs(phis @ c - phis @ c_ref).max()
    print("fit with forces and stress: backward error %.3g, dF %.3g eV/A, dS %.3g GPa "
          "(device vs numpy solution); |F - F_teacher| max %.3g eV/A"
          % (res, df, ds, np.abs(phif @ c - F.ravel()).max()))
    assert res <= 1e-12
    assert df <= 1e-6 * np.abs(F).max()
    assert ds <= 1e-6 * np.abs(St).max()
    # the fitted model evaluates to the solution's forces and stress
    _, F2, S2 = m.eval_batch(off, sp, lat, pos)
    assert np.abs(F2.ravel() - phif @ c).max() <= 1e-9 * np.abs(F).max()
    assert np.abs(S2.ravel() - phis @ c).max() <= 1e-9 * np.abs(St).max()
    m.close()
