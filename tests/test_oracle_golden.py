"""The oracle against the reference's own outputs (CPU).

The 11 frames of gappy/example/ASE-GAPPY/ase.traj hold energy, forces and
stress computed by the reference (libgap through its ASE calculator,
gappy/example/ASE-GAPPY/run_md.py:10-21) for a 64-atom carbon cell with the
example model; tests/golden/make_golden.py extracted them.
"""
import numpy as np
import pytest

from conftest import GOLDEN_MODEL


def test_model_file_parsed(golden_oracle_model):
    m = golden_oracle_model
    assert (m.M, m.D) == (129, 66)
    assert list(m.species_z) == [5, 6] and list(m.species_w) == [-1.0, 4.0]
    assert len(m.sf_type) == 33 and sorted(set(m.sf_type)) == [1, 2, 3, 4]
    assert np.all(m.sf_zeta == 1.0)
    assert m.theta[0] == pytest.approx(2.1695365180)


@pytest.mark.parametrize("f", range(11))
def test_golden_frame(oracle_mod, golden_oracle_model, frames, f):
    E, F, S, var = oracle_mod.gap_calc(golden_oracle_model, frames["numbers"][f],
                                       frames["cell"][f], frames["positions"][f], 6.0, True)
    assert abs(E - frames["energy"][f]) <= 1e-9 * abs(frames["energy"][f])
    assert np.abs(F - frames["forces"][f]).max() <= 1e-7
    assert np.abs(S - frames["stress"][f]).max() <= 1e-7
    assert var == 0.0


def test_forces_are_minus_energy_gradient(oracle_mod, golden_oracle_model, frames):
    """Central differences of E reproduce F (pins the derivative loops)."""
    z, lat, pos = frames["numbers"][0], frames["cell"][0], frames["positions"][0].copy()
    _, F, _, _ = oracle_mod.gap_calc(golden_oracle_model, z, lat, pos, 6.0, True)
    h = 1e-5
    for atom, c in [(0, 0), (7, 1), (33, 2)]:
        p1, p2 = pos.copy(), pos.copy()
        p1[atom, c] += h
        p2[atom, c] -= h
        e1 = oracle_mod.gap_calc(golden_oracle_model, z, lat, p1, 6.0, False)[0]
        e2 = oracle_mod.gap_calc(golden_oracle_model, z, lat, p2, 6.0, False)[0]
        assert abs(-(e1 - e2) / (2 * h) - F[atom, c]) < 2e-5


def test_stress_is_strain_derivative(oracle_mod, golden_oracle_model, frames):
    """stress = -(1/V) dE/d(strain) in GPa, order XX YY ZZ XY YZ ZX."""
    z, lat, pos = frames["numbers"][0], frames["cell"][0], frames["positions"][0]
    _, _, S, _ = oracle_mod.gap_calc(golden_oracle_model, z, lat, pos, 6.0, True)
    V = abs(np.linalg.det(lat))
    h = 1e-6
    for q, (a, b) in enumerate([(0, 0), (1, 1), (2, 2), (0, 1), (1, 2), (0, 2)]):
        es = []
        for sgn in (1, -1):
            eps = np.eye(3)
            eps[a, b] += sgn * h / (1 if a == b else 2)
            eps[b, a] += 0 if a == b else sgn * h / 2
            es.append(oracle_mod.gap_calc(golden_oracle_model, z, lat @ eps, pos @ eps, 6.0, False)[0])
        dEde = (es[0] - es[1]) / (2 * h)
        assert abs(-dEde / V / 6.24219e-3 - S[q]) < 1e-3


def test_total_force_vanishes(oracle_mod, golden_oracle_model, frames):
    _, F, _, _ = oracle_mod.gap_calc(golden_oracle_model, frames["numbers"][3], frames["cell"][3],
                                     frames["positions"][3], 6.0, True)
    assert np.abs(F.sum(0)).max() < 1e-10


def test_neighbour_order_and_count(oracle_mod, golden_oracle_model, frames):
    """Reference order: j ascending, then n1, n2, n3 ascending (gap_calc.f90:92-120)."""
    z, lat, pos = frames["numbers"][0], frames["cell"][0], frames["positions"][0]
    cnt, nb = oracle_mod.neighbors(lat, pos, golden_oracle_model.weights(z), 6.0)
    assert cnt.min() > 100 and cnt.max() < 200
    for i in (0, 17):
        js = nb[i, : cnt[i], 5]
        assert np.all(np.diff(js) >= 0)
        assert np.all(nb[i, : cnt[i], 3] <= 6.0)


def test_min_bond(oracle_mod, frames):
    lat, pos = frames["cell"][0], frames["positions"][0]
    mb = oracle_mod.min_bond(lat, pos, 6.0)
    d = pos[:, None, :] - pos[None, :, :]
    inv = np.linalg.inv(lat)
    f = d @ inv
    f -= np.round(f)
    r = np.sqrt(((f @ lat) ** 2).sum(-1))
    r[np.arange(len(pos)), np.arange(len(pos))] = np.inf
    assert mb == pytest.approx(r.min(), abs=1e-12)


def test_zeta_extension_matches_finite_difference(oracle_mod, tmp_path):
    """zeta > 1 (extension): forces still equal -dE/dr."""
    import gapgb.synth as S
    from helpers import synth_model_file
    structs = [S.si64(seed=s) for s in range(2)]
    path = synth_model_file(str(tmp_path / "gp"), oracle_mod, structs, M=40, theta_scale=1.0,
                            coeff_std=1.0)
    m = oracle_mod.Model(path)
    assert set(m.sf_zeta.tolist()) == {1.0, 2.0, 4.0}
    lat, pos, z = S.si64(seed=5)
    _, F, _, _ = oracle_mod.gap_calc(m, z, lat, pos, 6.0, True)
    h = 1e-5
    for atom, c in [(3, 0), (40, 2)]:
        p1, p2 = pos.copy(), pos.copy()
        p1[atom, c] += h
        p2[atom, c] -= h
        e1 = oracle_mod.gap_calc(m, z, lat, p1, 6.0, False)[0]
        e2 = oracle_mod.gap_calc(m, z, lat, p2, 6.0, False)[0]
        assert abs(-(e1 - e2) / (2 * h) - F[atom, c]) < 1e-5 * max(1.0, abs(F[atom, c]))


def test_three_species_weighting_matches_finite_difference(oracle_mod, tmp_path):
    """Species-weighted copies (wacsf.f90:86-87, 326-328) with three species:
    the oracle's forces equal -dE/dr and its stress -(1/V) dE/d(strain), on a
    jittered 3-species fcc cell (no reference fixture covers mixed weights)."""
    from helpers import synth_model_file, three_species_cell as _three_species_cell
    path = synth_model_file(str(tmp_path / "gp"), oracle_mod,
                            [_three_species_cell(s) for s in range(4)], M=60, theta_scale=1.0,
                            coeff_std=0.1, seed=9)
    m = oracle_mod.Model(path)
    assert sorted(m.species_z.tolist()) == [13, 28, 40]
    lat, pos, z = _three_species_cell(11)
    _, F, S, _ = oracle_mod.gap_calc(m, z, lat, pos, 6.0, True)
    h = 1e-5
    for atom, c in [(0, 0), (5, 1), (17, 2), (30, 0)]:
        p1, p2 = pos.copy(), pos.copy()
        p1[atom, c] += h
        p2[atom, c] -= h
        e1 = oracle_mod.gap_calc(m, z, lat, p1, 6.0, False)[0]
        e2 = oracle_mod.gap_calc(m, z, lat, p2, 6.0, False)[0]
        assert abs(-(e1 - e2) / (2 * h) - F[atom, c]) < 1e-5 * max(1.0, abs(F[atom, c]))
    V = abs(np.linalg.det(lat))
    hs = 1e-6
    for q, (a, b) in enumerate([(0, 0), (1, 1), (2, 2), (0, 1), (1, 2), (0, 2)]):
        es = []
        for sgn in (1, -1):
            eps = np.eye(3)
            eps[a, b] += sgn * hs / (1 if a == b else 2)
            eps[b, a] += 0 if a == b else sgn * hs / 2
            es.append(oracle_mod.gap_calc(m, z, lat @ eps, pos @ eps, 6.0, False)[0])
        dEde = (es[0] - es[1]) / (2 * hs)
        assert abs(-dEde / V / 6.24219e-3 - S[q]) < 1e-4 * max(1.0, abs(S[q]))
