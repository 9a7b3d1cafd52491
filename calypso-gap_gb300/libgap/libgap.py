"""The f2py surface of the reference's ``libgap.libgap`` extension.

Same names, argument order and return values as the Fortran subroutines
exposed by f2py (gappy/setup.py:38-47):

  fgap_read()                      FGAP_READ   gappy/libgap/gap_calc.f90:303-364
      -> (nsparsex, des_len, theta(100), mm(4000,100), invcmm(4000,4000), coeff(4000))
  fgap_calc(species, lat, pos, theta, mm, qmm, coeff, rcut, lgrad)
                                   FGAP_CALC   gappy/libgap/gap_calc.f90:1-301
      -> (ene, force(N,3), stress(6), variance)
  fget_bond(lat, elements, pos, rcut)
                                   FGET_BOND   gappy/libgap/get_bond.f90:4-116
      -> min_bond

As in the reference, the species weights and the symmetry-function table
come from ``./gap_parameters`` in the current directory, and theta/mm/coeff
from the arguments.  The evaluation runs on the GPU (gapgb); a model is
cached on the device and reused while the file and the arrays are unchanged.
Differences: errors raise ``gapgb.GapError`` instead of stopping the process,
and models beyond the reference's fixed arrays (M > 4000, D > 100) are
returned in arrays large enough to hold them.
"""
import os

import numpy as np

import gapgb

_NSF_MAX = 100       # gap_calc.f90:306
_NSPARSE_MAX = 4000  # gap_calc.f90:307
_MODEL_FILE = "gap_parameters"

_cache = {"key": None, "model": None, "arrays": None}
# fgap_read's parse of the file, reused while the file is unchanged (same
# path, size and modification time); every call still returns fresh arrays
_read_cache = {"key": None, "arrays": None}


def _file_key():
    path = os.path.abspath(_MODEL_FILE)
    try:
        st = os.stat(path)
    except FileNotFoundError:
        raise gapgb.GapError(1, "gap_parameters file does not exist!")
    return (path, st.st_mtime_ns, st.st_size)


def fgap_read():
    key = _file_key()
    if _read_cache["key"] == key:
        th, mm, co = _read_cache["arrays"]
    else:
        m = gapgb.GapModel.load(key[0])
        try:
            th, mm, co = m.arrays()
        finally:
            m.close()
        _read_cache.update(key=key, arrays=(th, mm, co))
    M, D = mm.shape
    nsf = max(_NSF_MAX, D)
    nsp = max(_NSPARSE_MAX, M)
    theta = np.zeros(nsf)
    theta[:D] = th
    MM = np.zeros((nsp, nsf), order="F")
    MM[:M, :D] = mm
    invcmm = np.zeros((nsp, nsp), order="F")  # zero-filled, gap_calc.f90:361
    coeff = np.zeros(nsp)
    coeff[:M] = co
    return M, D, theta, MM, invcmm, coeff


def _model_for(theta, mm, coeff, rcut):
    theta = np.ascontiguousarray(theta, np.float64)
    mm = np.ascontiguousarray(mm, np.float64)
    coeff = np.ascontiguousarray(coeff, np.float64)
    key = _file_key() + (float(rcut), mm.shape)
    c = _cache
    if c["key"] == key and c["arrays"] is not None:
        t0, m0, c0 = c["arrays"]
        if np.array_equal(t0, theta) and np.array_equal(m0, mm) and np.array_equal(c0, coeff):
            return c["model"]
    base = gapgb.GapModel.load(key[0], rcut=rcut)
    th_f, mm_f, co_f = base.arrays()
    if th_f.shape == theta.shape and mm_f.shape == mm.shape and np.array_equal(th_f, theta) \
            and np.array_equal(mm_f, mm) and np.array_equal(co_f, coeff):
        model = base
    else:
        z, w, ty, al, cu, ze = base.tables()
        base.close()
        model = gapgb.GapModel.create(z, w, ty, al, cu, theta, mm, coeff, sf_zeta=ze, rcut=rcut)
    if c["model"] is not None and c["model"] is not model:
        c["model"].close()
    c.update(key=key, model=model, arrays=(theta.copy(), mm.copy(), coeff.copy()))
    return model


def fgap_calc(species, lat, pos, theta, mm, qmm, coeff, rcut, lgrad):
    del qmm  # never read by the reference (variance is 0, gap_calc.f90:206-210)
    model = _model_for(theta, mm, coeff, rcut)
    return model.eval(np.asarray(species), np.asarray(lat), np.asarray(pos), bool(lgrad))


def fget_bond(lat, elements, pos, rcut):
    del elements  # unused by the reference (get_bond.f90:11)
    return gapgb.min_bond(np.asarray(lat), np.asarray(pos), float(rcut))
