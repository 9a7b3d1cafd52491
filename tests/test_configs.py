"""Parity on the benchmark configurations themselves, in every precision
form, against the oracle.

- Si64 (2x2x2 diamond, a = 5.43 A, jitter 0.05 A), M = 500 sparse points
  drawn from 20 seeded jittered cells, theta = 1.0 x std, coefficients
  N(0, 1e-3), the 20 radial + 12 angular SF set with zeta in {1, 2, 4}; and
  the zeta = 1 variant (lambda +-1 x eta {0.003, 0.03} x cutoffs
  {6.0, 4.5, 3.5} A) that the reference itself supports.
- The ternary alloy (512-atom fcc, Z 13/28/40) at M = 4000, theta = 0.8 x std,
  on two cells.
- A 256-atom, 4-species population member at M = 4000.
- Central finite differences of the FP64 path's energy on a 3-species cell
  (forces and stress), which pin the species-weighted copies of every SF
  (wacsf.f90:86-87, 326-328) independently of the oracle.

Bars: the plain FP64 path within 1e-9 relative energy, 1e-7 eV/A and 1e-7
GPa; the reduced-precision forms within 1 meV/atom and 20 meV/A (stress
within 1e-2 GPa).
"""
import numpy as np
import pytest

from helpers import synth_model_file, three_species_cell as _three_species_cell

pytestmark = pytest.mark.gpu

E_REL, F_ABS, S_ABS = 1e-9, 1e-7, 1e-7
E_FAST, F_FAST, S_FAST = 1e-3, 20e-3, 1e-2
FORMS = ["fp64", "fp32", "mixed", "tc", "tf32"]


def _check_forms(m, o, oracle_mod, structs, forms=FORMS):
    import gapgb.synth as S
    off, sp, lat, pos = S.pack(structs)
    ref = [oracle_mod.gap_calc(o, z, l, p, 6.0, True) for l, p, z in structs]
    report = {}
    for prec in forms:
        m.set_precision(prec)
        E, F, St = m.eval_batch(off, sp, lat, pos)
        worst = [0.0, 0.0, 0.0]
        for s, (l, p, z) in enumerate(structs):
            oE, oF, oS, _ = ref[s]
            n = len(p)
            dE, dF = abs(E[s] - oE), np.abs(F[off[s]:off[s + 1]] - oF).max()
            dS = np.abs(St[s] - oS).max()
            worst = [max(worst[0], dE / n), max(worst[1], dF), max(worst[2], dS)]
            if prec == "fp64":
                assert dE <= E_REL * max(1.0, abs(oE)), (prec, s, dE)
                assert dF <= F_ABS and dS <= S_ABS, (prec, s, dF, dS)
            else:
                assert dE / n <= E_FAST, (prec, s, dE / n)
                assert dF <= F_FAST and dS <= S_FAST, (prec, s, dF, dS)
        report[prec] = worst
    m.set_precision("fp64")
    print({k: ["%.2e" % v for v in w] for k, w in report.items()})
    return report


def _si_zeta1_sf():
    """The zeta = 1 SF set: 20 radial (eta 0.003..2.0, rc 6) and 12 angular,
    lambda +-1 x eta {0.003, 0.03} x cutoffs {6.0, 4.5, 3.5}."""
    ty, al, rc = [], [], []
    for a in np.geomspace(0.003, 2.0, 20):
        ty.append(1), al.append(float(a)), rc.append(6.0)
    for cut in (6.0, 4.5, 3.5):
        for t in (2, 4):
            for a in (0.003, 0.03):
                ty.append(t), al.append(a), rc.append(cut)
    return np.array(ty, np.int32), np.array(al), np.array(rc), np.ones(len(ty))


@pytest.mark.parametrize("sf_set", ["zeta124", "zeta1_three_cutoffs"])
def test_si64_m500_every_form(gapgb_mod, oracle_mod, tmp_path, sf_set):
    import gapgb.synth as S
    sf = None if sf_set == "zeta124" else _si_zeta1_sf()
    path = synth_model_file(str(tmp_path / "gap_parameters"), oracle_mod,
                            [S.si64(seed=s) for s in range(1, 21)], M=500, theta_scale=1.0,
                            coeff_std=1e-3, seed=11, sf=sf)
    m = gapgb_mod.GapModel.load(path)
    o = oracle_mod.Model(path)
    assert (m.nsparse, m.des_len) == (500, 64)
    try:
        _check_forms(m, o, oracle_mod, [S.si64(seed=s) for s in (101, 102)])
    finally:
        m.close()


def test_alloy512_m4000_every_form(gapgb_mod, oracle_mod, tmp_path):
    import gapgb.synth as S
    path = synth_model_file(str(tmp_path / "gap_parameters"), oracle_mod,
                            [S.alloy512(seed=s) for s in range(8)], M=4000, theta_scale=0.8,
                            coeff_std=1e-3, seed=0)
    m = gapgb_mod.GapModel.load(path)
    o = oracle_mod.Model(path)
    assert (m.nsparse, m.des_len) == (4000, 64)
    try:
        _check_forms(m, o, oracle_mod, [S.alloy512(seed=s) for s in (200, 201)])
    finally:
        m.close()


def _four_species(rng, n):
    import gapgb.synth as S
    lat, pos, _ = S.random_structure(rng, n, species_pool=(3, 8, 14, 26))
    z = np.array([3, 8, 14, 26], np.int32)[rng.permutation(np.arange(n) % 4)]
    return lat, pos, z


def test_population_member_256_atoms_4_species_m4000(gapgb_mod, oracle_mod, tmp_path):
    rng = np.random.default_rng(2024)
    cells = [_four_species(rng, 256) for _ in range(16)]
    path = synth_model_file(str(tmp_path / "gap_parameters"), oracle_mod, cells, M=4000,
                            theta_scale=0.8, coeff_std=1e-3, seed=5)
    m = gapgb_mod.GapModel.load(path)
    o = oracle_mod.Model(path)
    try:
        member = _four_species(np.random.default_rng(77), 256)
        assert len(set(member[2].tolist())) == 4
        _check_forms(m, o, oracle_mod, [member])
    finally:
        m.close()


def test_three_species_finite_differences_fp64(gapgb_mod, oracle_mod, tmp_path):
    """F = -dE/dr and sigma = -(1/V) dE/d(strain) (GPa, XX YY ZZ XY YZ ZX) by
    central differences of the FP64 path's own energy on a 3-species cell."""
    path = synth_model_file(str(tmp_path / "gap_parameters"), oracle_mod,
                            [_three_species_cell(s) for s in range(4)], M=60, theta_scale=1.0,
                            coeff_std=0.1, seed=9)
    m = gapgb_mod.GapModel.load(path)
    m.set_precision("fp64")
    lat, pos, z = _three_species_cell(11)
    try:
        E, F, St, _ = m.eval(z, lat, pos)
        h = 1e-5
        for atom, c in [(0, 0), (5, 1), (17, 2), (30, 0)]:
            p1, p2 = pos.copy(), pos.copy()
            p1[atom, c] += h
            p2[atom, c] -= h
            e1 = m.eval(z, lat, p1, lgrad=False)[0]
            e2 = m.eval(z, lat, p2, lgrad=False)[0]
            assert abs(-(e1 - e2) / (2 * h) - F[atom, c]) <= 1e-5 * max(1.0, abs(F[atom, c]))
        V = abs(np.linalg.det(lat))
        hs = 1e-6
        for q, (a, b) in enumerate([(0, 0), (1, 1), (2, 2), (0, 1), (1, 2), (0, 2)]):
            es = []
            for sgn in (1, -1):
                eps = np.eye(3)
                eps[a, b] += sgn * hs / (1 if a == b else 2)
                eps[b, a] += 0 if a == b else sgn * hs / 2
                es.append(m.eval(z, lat @ eps, pos @ eps, lgrad=False)[0])
            dEde = (es[0] - es[1]) / (2 * hs)
            assert abs(-dEde / V / 6.24219e-3 - St[q]) <= 1e-4 * max(1.0, abs(St[q]))
        # and the oracle agrees with the FP64 path on this cell
        o = oracle_mod.Model(path)
        oE, oF, oS, _ = oracle_mod.gap_calc(o, z, lat, pos, 6.0, True)
        assert abs(E - oE) <= E_REL * max(1.0, abs(oE))
        assert np.abs(F - oF).max() <= F_ABS and np.abs(St - oS).max() <= S_ABS
    finally:
        m.close()
