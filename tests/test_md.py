"""Velocity-Verlet MD on the device (gapgb_md_*) against a host integrator
driven by the CPU oracle's forces, the Verlet-list refresh against fresh
evaluations, NVE energy conservation and the skin check.

The host integrator here is the oracle for the MD driver: the same
velocity-Verlet update in numpy, with forces from oracle.gap_calc (which
builds its own exact-cutoff neighbour list at every step, as the reference
does on every FGAP_CALC call).
"""
import numpy as np
import pytest

from helpers import synth_model_file

KB = 8.617333262e-5


def _mic(d, lat):
    """Minimum-image version of displacement rows d for cell rows lat."""
    f = d @ np.linalg.inv(lat)
    f -= np.round(f)
    return f @ lat


def oracle_vv(oracle_mod, model, z, lat, pos, vel, masses, dt, nsteps):
    """Host velocity Verlet with oracle forces: positions, velocities and
    (Epot, Ekin) per step."""
    from gapgb.md import EV_PER_AMU_A2_FS2, kinetic
    acc = 1.0 / (masses * EV_PER_AMU_A2_FS2)
    x, v = pos.copy(), vel.copy()
    e, f, _, _ = oracle_mod.gap_calc(model, z, lat, x, 6.0, True)
    hist = []
    for _ in range(nsteps):
        v += 0.5 * dt * f * acc[:, None]
        x += dt * v
        e, f, _, _ = oracle_mod.gap_calc(model, z, lat, x, 6.0, True)
        v += 0.5 * dt * f * acc[:, None]
        hist.append((e, kinetic(masses, v)))
    return x, v, np.array(hist)


def test_maxwell_boltzmann_velocities():
    from gapgb.md import maxwell_boltzmann, kinetic, masses_of
    z = np.array([14] * 2000 + [32] * 2000)
    m = masses_of(z)
    off = np.array([0, 1000, 4000])
    v = maxwell_boltzmann(off, m, 600.0, seed=3)
    for a, b in ((0, 1000), (1000, 4000)):
        assert np.allclose((m[a:b, None] * v[a:b]).sum(0), 0.0, atol=1e-12)
    T = 2 * kinetic(m, v) / (3 * len(m) * KB)
    assert abs(T - 600.0) < 30.0
    assert np.array_equal(v, maxwell_boltzmann(off, m, 600.0, seed=3))


@pytest.fixture(scope="module")
def si_model(oracle_mod, tmp_path_factory):
    import gapgb.synth as S
    path = str(tmp_path_factory.mktemp("md") / "gap_parameters")
    synth_model_file(path, oracle_mod, [S.si64(seed=s) for s in range(3)], M=300,
                     theta_scale=1.0, coeff_std=0.05, seed=2)
    return path


@pytest.mark.gpu
def test_md_matches_host_integrator_with_oracle_forces(gapgb_mod, oracle_mod, si_model):
    import gapgb.synth as S
    from gapgb.md import MD, masses_of, maxwell_boltzmann
    lat, pos, z = S.si64(seed=11, jitter=0.08)
    m = masses_of(z)
    vel = maxwell_boltzmann([0, len(z)], m, 900.0, seed=5)
    model = gapgb_mod.GapModel.load(si_model)
    model.set_precision("fp64")
    md = MD(model, [0, len(z)], z, lat[None], pos, vel, m, dt=1.0, skin=0.6, rebuild_every=5)
    ep, ek = md.run(20)
    om = oracle_mod.Model(si_model)
    x_ref, v_ref, hist = oracle_vv(oracle_mod, om, z, lat, pos, vel, m, 1.0, 20)
    dx = np.abs(_mic(md.positions() - x_ref, lat)).max()
    dv = np.abs(md.velocities() - v_ref).max()
    de = np.abs(ep[:, 0] - hist[:, 0]).max()
    dk = np.abs(ek[:, 0] - hist[:, 1]).max()
    print("20 steps vs host VV + oracle: dx %.2g A, dv %.2g A/fs, dEpot %.2g eV, dEkin %.2g eV"
          % (dx, dv, de, dk))
    # FP64 forces agree with the oracle's to summation order (~1e-10 eV/A
    # here); 20 steps of the trajectory amplify that to ~1e-9 A
    assert dx <= 1e-8 and dv <= 1e-9
    assert de <= 1e-9 * len(z) and dk <= 1e-9 * len(z)
    md.close()
    model.close()


@pytest.mark.gpu
def test_md_refreshed_steps_equal_fresh_evaluation(gapgb_mod, si_model):
    import gapgb.synth as S
    from gapgb.md import MD, masses_of, maxwell_boltzmann
    structs = [S.si64(seed=20 + s, jitter=0.08) for s in range(3)]
    off, sp, lat, pos = S.pack(structs)
    m = masses_of(sp)
    vel = maxwell_boltzmann(off, m, 1200.0, seed=1)
    for prec in ("fp64", "tc"):
        model = gapgb_mod.GapModel.load(si_model)
        model.set_precision(prec)
        md = MD(model, off, sp, lat, pos, vel, m, dt=1.0, skin=0.8, rebuild_every=10)
        md.run(7)  # steps 1..7 are refreshes of the list built at t = 0
        E, F, Sg, _ = md.outputs()
        fresh = gapgb_mod.GapModel.load(si_model)
        fresh.set_precision(prec)
        E0, F0, S0 = fresh.eval_batch(off, sp, lat, md.positions())
        if prec == "fp64":
            e_tol, f_tol, s_tol = 1e-11 * len(sp), 1e-10, 1e-9
        else:
            # the refreshed list holds extra (skin) slots, so the FP32
            # descriptor sums round differently, and a last-bit change can
            # flip a BF16 hi/lo split: the two tensor-core evaluations agree
            # to the form's own error against FP64, measured here
            fresh.set_precision("fp64")
            E64, F64, S64 = fresh.eval_batch(off, sp, lat, md.positions())
            e_tol = max(1e-6 * len(sp), 3 * np.abs(E0 - E64).max())
            f_tol = max(1e-4, 3 * np.abs(F0 - F64).max())
            s_tol = max(1e-3, 3 * np.abs(S0 - S64).max())
        print("%s refresh vs fresh: dE %.3g eV, dF %.3g eV/A (bound %.3g), dS %.3g GPa"
              % (prec, np.abs(E - E0).max(), np.abs(F - F0).max(), f_tol, np.abs(Sg - S0).max()))
        assert np.abs(E - E0).max() <= e_tol
        assert np.abs(F - F0).max() <= f_tol
        assert np.abs(Sg - S0).max() <= s_tol
        md.close()
        model.close()
        fresh.close()


@pytest.mark.gpu
def test_md_nve_error_scales_as_dt_squared_and_tc_tracks_fp64(gapgb_mod, si_model):
    """Velocity Verlet's energy error is O(dt^2): halving dt over the same
    100 fs cuts the largest |E_tot(t) - E_tot(0)| about fourfold (an energy
    inconsistent with the forces would not scale).  The tensor-core form's
    error must follow the FP64 path's."""
    import gapgb.synth as S
    from gapgb.md import MD, masses_of, maxwell_boltzmann
    structs = [S.si64(seed=40 + s, jitter=0.05) for s in range(4)]
    off, sp, lat, pos = S.pack(structs)
    m = masses_of(sp)
    vel = maxwell_boltzmann(off, m, 600.0, seed=2)
    err = {}
    for prec, dt in (("fp64", 1.0), ("fp64", 0.5), ("tc", 1.0)):
        model = gapgb_mod.GapModel.load(si_model)
        model.set_precision(prec)
        md = MD(model, off, sp, lat, pos, vel, m, dt=dt, skin=0.5, rebuild_every=10)
        E0, _, _, K0 = md.outputs()
        ep, ek = md.run(int(round(100 / dt)))
        et = (ep + ek).sum(1)
        err[(prec, dt)] = np.abs(et - (E0.sum() + K0.sum())).max() / len(sp)
        md.close()
        model.close()
    print("NVE max |dE_tot| per atom over 100 fs: fp64 dt=1 %.3g, dt=0.5 %.3g, tc dt=1 %.3g eV"
          % (err[("fp64", 1.0)], err[("fp64", 0.5)], err[("tc", 1.0)]))
    ratio = err[("fp64", 1.0)] / err[("fp64", 0.5)]
    assert 2.5 < ratio < 6.0
    assert abs(err[("tc", 1.0)] - err[("fp64", 1.0)]) <= 0.05 * err[("fp64", 1.0)] + 1e-6


@pytest.mark.gpu
def test_md_reports_skin_exceeded(gapgb_mod, si_model):
    import gapgb.synth as S
    from gapgb.md import MD, masses_of, maxwell_boltzmann
    lat, pos, z = S.si64(seed=3)
    m = masses_of(z)
    vel = maxwell_boltzmann([0, len(z)], m, 3000.0, seed=9)
    model = gapgb_mod.GapModel.load(si_model)
    md = MD(model, [0, len(z)], z, lat[None], pos, vel, m, dt=1.0, skin=0.001, rebuild_every=10)
    with pytest.raises(gapgb_mod.GapError) as ei:
        md.run(3)
    assert ei.value.status == 3
    assert "skin" in gapgb_mod.last_error()
    md.close()
    model.close()
