"""C-ABI library on the CPU: it loads, exports every symbol include/gapgb.h
declares (and the Fortran-ABI symbols of the reference's subroutines), and
its host-side model reader agrees with the oracle's.  No compute calls."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN_MODEL, ROOT


def _declared_symbols():
    txt = open(os.path.join(ROOT, "include", "gapgb.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gapgb_[a-z_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(gapgb_mod):
    L = ctypes.CDLL(gapgb_mod.lib_path())
    declared = _declared_symbols()
    assert len(declared) >= 18
    for name in declared:
        assert hasattr(L, name), name
    bound = {n for n, _, _ in gapgb_mod.SYMBOLS}
    assert set(declared) == bound
    for name in gapgb_mod.FORTRAN_SYMBOLS:
        assert hasattr(L, name), name


def test_status_strings(gapgb_mod):
    L = gapgb_mod.load()
    assert L.gapgb_status_string(0) == b"ok"
    assert L.gapgb_status_string(5) == b"neighbour capacity exceeded"
    assert b"sm_103a" in L.gapgb_version()


def test_model_reader_matches_oracle(gapgb_mod, golden_oracle_model):
    m = gapgb_mod.GapModel.load(GOLDEN_MODEL)
    try:
        assert (m.nsparse, m.des_len, m.nsf, m.nspecies, m.rcut) == (129, 66, 33, 2, 6.0)
        th, mm, co = m.arrays()
        o = golden_oracle_model
        assert np.array_equal(th, o.theta)
        assert np.array_equal(mm, o.mm)
        assert np.array_equal(co, o.coeff)
        z, w, ty, al, cu, ze = m.tables()
        assert np.array_equal(z, o.species_z) and np.array_equal(w, o.species_w)
        assert np.array_equal(ty, o.sf_type) and np.array_equal(al, o.sf_alpha)
        assert np.array_equal(cu, o.sf_cutoff) and np.array_equal(ze, o.sf_zeta)
    finally:
        m.close()


def test_missing_file_is_a_status(gapgb_mod, tmp_path):
    with pytest.raises(gapgb_mod.GapError) as ei:
        gapgb_mod.GapModel.load(str(tmp_path / "nope"))
    assert ei.value.status == 1


@pytest.mark.parametrize("mutate,status", [
    (lambda L: L[:40], 2),                                    # truncated
    (lambda L: L[:4] + ["1 0.5 six\n"] + L[5:], 2),             # bad token on an SF line
    (lambda L: L[:37] + ["129 10\n"] + L[38:], 2),             # D < 2*nsf
])
def test_malformed_files(gapgb_mod, tmp_path, mutate, status):
    lines = open(GOLDEN_MODEL).readlines()
    p = tmp_path / "gp"
    p.write_text("".join(mutate(lines)))
    with pytest.raises(gapgb_mod.GapError) as ei:
        gapgb_mod.GapModel.load(str(p))
    assert ei.value.status == status


def test_zeta_column_and_fortran_exponent(gapgb_mod, tmp_path):
    lines = open(GOLDEN_MODEL).readlines()
    lines[12] = lines[12].rstrip("\n") + "   2.0\n"    # an angular SF (type 2) gets zeta 2
    lines[42] = lines[42].replace("E", "D")
    p = tmp_path / "gp"
    p.write_text("".join(lines))
    m = gapgb_mod.GapModel.load(str(p))
    z, w, ty, al, cu, ze = m.tables()
    assert ze[8] == 2.0 and ty[8] == 2 and np.all(np.delete(ze, 8) == 1.0)
    m.close()


def test_list_directed_reads(gapgb_mod, golden_oracle_model, tmp_path):
    """theta may span records and use r*v repeats (Fortran list-directed input)."""
    lines = open(GOLDEN_MODEL).readlines()
    vals = lines[41].split()
    lines[41] = " ".join(vals[:30]) + "\n" + ", ".join(vals[30:]) + "\n"
    p = tmp_path / "gp"
    p.write_text("".join(lines))
    m = gapgb_mod.GapModel.load(str(p))
    th, mm, co = m.arrays()
    assert np.array_equal(th, golden_oracle_model.theta)
    assert np.array_equal(mm, golden_oracle_model.mm)
    m.close()


def test_libgap_fgap_read_shapes(gapgb_mod, tmp_path, monkeypatch):
    """fgap_read returns the reference's fixed-size arrays (gap_calc.f90:309-314)."""
    import shutil
    shutil.copy(GOLDEN_MODEL, tmp_path / "gap_parameters")
    monkeypatch.chdir(tmp_path)
    from libgap.libgap import fgap_read
    M, D, theta, mm, invcmm, coeff = fgap_read()
    assert (M, D) == (129, 66)
    assert theta.shape == (100,) and mm.shape == (4000, 100)
    assert invcmm.shape == (4000, 4000) and coeff.shape == (4000,)
    assert not invcmm.any()
    from libgap.GAP import Calculator
    c = Calculator(rcut=6.0)
    assert c.nsparseX == 129 and c.des_len == 66
    assert c.get_elenum(["B", "C"]) == [5, 6]


def _same_model(a, b):
    for x, y in zip(a.arrays(), b.arrays()):
        assert np.array_equal(x, y)
    for x, y in zip(a.tables(), b.tables()):
        assert np.array_equal(x, y)
    assert (a.nsparse, a.des_len, a.nsf, a.nspecies) == (b.nsparse, b.des_len, b.nsf, b.nspecies)


def test_model_writer_round_trip(gapgb_mod, oracle_mod, tmp_path):
    """gapgb_model_write: the written file reads back (library and oracle) to
    the same doubles, and the reference's example model round-trips."""
    m = gapgb_mod.GapModel.load(GOLDEN_MODEL)
    p = m.save(str(tmp_path / "gp"))
    m2 = gapgb_mod.GapModel.load(p)
    _same_model(m, m2)
    o = oracle_mod.Model(p)
    th, mm, co = m.arrays()
    assert np.array_equal(o.theta, th) and np.array_equal(o.mm, mm)
    assert np.array_equal(o.coeff, co)
    # the reference's own SF types have zeta 1: no fourth column is written
    lines = open(p).read().split("\n")
    assert all(len(ln.split()) == 3 for ln in lines[4:4 + m.nsf])
    m.close()
    m2.close()


def test_write_parameters_matches_test_writer(gapgb_mod, tmp_path):
    """The package's writer and the test suite's independent writer give the
    same bytes, zeta column included."""
    from helpers import write_model_file
    rng = np.random.default_rng(4)
    ty = np.array([1, 1, 3, 2, 4, 2], np.int32)
    al = rng.uniform(0.01, 2.0, 6)
    cu = np.full(6, 6.0)
    ze = np.array([1, 1, 1, 2, 4, 1.0])
    th = rng.uniform(0.5, 3.0, 12)
    mm = rng.normal(size=(7, 12)) * 1e3
    co = rng.normal(size=7) * 1e-3
    a = gapgb_mod.write_parameters(str(tmp_path / "a"), [14, 32], [1.0, -2.5], ty, al, cu, th, mm,
                                   co, sf_zeta=ze)
    b = write_model_file(str(tmp_path / "b"), [14, 32], [1.0, -2.5], ty, al, cu, th, mm, co, ze)
    assert open(a).read() == open(b).read()
    m = gapgb_mod.GapModel.load(a)
    assert np.array_equal(m.arrays()[1], mm) and np.array_equal(m.tables()[5], ze)
    m.close()


def test_fit_and_variance_argument_checks(gapgb_mod):
    """Argument errors come back as statuses before any device work."""
    import gapgb.synth as S
    m = gapgb_mod.GapModel.load(GOLDEN_MODEL)
    L = gapgb_mod.load()
    off, sp, lat, pos = S.pack([S.si64(seed=1)])
    off, sp = np.ascontiguousarray(off, np.int32), np.ascontiguousarray(sp, np.int32)
    lat, pos = np.ascontiguousarray(lat), np.ascontiguousarray(pos)
    e = np.zeros(1)
    args = (m.handle, 1, off.ctypes.data, sp.ctypes.data, lat.ctypes.data, pos.ctypes.data,
            e.ctypes.data)
    # sigma_e must be positive; a force fit needs a positive sigma_f
    assert L.gapgb_fit(*args, None, None, 0.0, 1.0, 1.0, 1e-8, None) == 8
    f = np.zeros((64, 3))
    assert L.gapgb_fit(*args, f.ctypes.data, None, 1e-3, 0.0, 1.0, 1e-8, None) == 8
    assert L.gapgb_fit(*args, None, None, 1e-3, 1.0, 1.0, -1.0, None) == 8
    # the variance needs an attached qmm
    covf, var = np.zeros(64), np.zeros(1)
    assert L.gapgb_variance(m.handle, 1, off.ctypes.data, sp.ctypes.data, lat.ctypes.data,
                            pos.ctypes.data, covf.ctypes.data, var.ctypes.data) == 8
    m.close()
