"""ctypes wrapper around liboracle.so (gap_oracle.c).

TEST INFRASTRUCTURE ONLY - the oracle and the CPU baseline.  The product
path never imports this module.

Each function names the reference routine it restates:
  read_model        FGAP_READ       gappy/libgap/gap_calc.f90:303-364
  neighbors         FGAP_CALC       gappy/libgap/gap_calc.f90:85-120
  car2acsf          CAR2ACSF        gappy/libgap/wacsf.f90:2-796
  gap_calc          FGAP_CALC       gappy/libgap/gap_calc.f90:1-301
  min_bond          FGET_BOND       gappy/libgap/get_bond.f90:4-116
  variance          FGAP_CALC       gappy/libgap/gap_calc.f90:206-210 (commented out there)
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class OrcModel(C.Structure):
    _fields_ = [
        ("nspecies", C.c_int),
        ("species_z", C.c_int * 128),
        ("species_w", C.c_double * 128),
        ("nsf", C.c_int),
        ("sf_type", C.c_int * 256),
        ("sf_alpha", C.c_double * 256),
        ("sf_cutoff", C.c_double * 256),
        ("sf_zeta", C.c_double * 256),
        ("nsparse", C.c_int),
        ("des_len", C.c_int),
        ("theta", C.POINTER(C.c_double)),
        ("mm", C.POINTER(C.c_double)),
        ("coeff", C.POINTER(C.c_double)),
    ]


def build(force=False):
    """Compile liboracle.so with the committed Makefile."""
    src = os.path.join(HERE, "gap_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-B", "liboracle.so"], cwd=HERE)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_model_read.argtypes = [C.c_char_p, C.POINTER(OrcModel)]
        L.orc_model_free.argtypes = [C.POINTER(OrcModel)]
        L.orc_nabc.argtypes = [_dp, C.c_double, _ip]
        L.orc_neighbors.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double, C.c_int, _ip, _dp]
        L.orc_car2acsf.argtypes = [C.POINTER(OrcModel), C.c_int, C.c_int, _dp, _dp, _ip,
                                   _dp, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_gap_calc.argtypes = [C.POINTER(OrcModel), C.c_int, _ip, _dp, _dp, C.c_double,
                                   C.c_int, C.POINTER(C.c_double), _dp, _dp,
                                   C.POINTER(C.c_double), C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_gap_calc_batch.argtypes = [C.POINTER(OrcModel), C.c_int, _ip, _ip, _dp, _dp,
                                         C.c_double, C.c_int, _dp, _dp, _dp]
        L.orc_variance.argtypes = [C.POINTER(OrcModel), C.c_int, _dp, _dp, _dp,
                                   C.POINTER(C.c_double)]
        L.orc_min_bond.argtypes = [C.c_int, _dp, _dp, C.c_double]
        L.orc_min_bond.restype = C.c_double
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


class Model:
    """A parsed gap_parameters file (FGAP_READ + species and SF tables)."""

    def __init__(self, path):
        self._m = OrcModel()
        st = lib().orc_model_read(os.fsencode(path), C.byref(self._m))
        if st:
            raise OracleError(f"orc_model_read({path}) failed with status {st}")
        m = self._m
        self.M, self.D = m.nsparse, m.des_len
        self.species_z = np.array(m.species_z[: m.nspecies], dtype=np.int32)
        self.species_w = np.array(m.species_w[: m.nspecies])
        self.sf_type = np.array(m.sf_type[: m.nsf], dtype=np.int32)
        self.sf_alpha = np.array(m.sf_alpha[: m.nsf])
        self.sf_cutoff = np.array(m.sf_cutoff[: m.nsf])
        self.sf_zeta = np.array(m.sf_zeta[: m.nsf])
        self.theta = np.ctypeslib.as_array(m.theta, (self.D,)).copy()
        self.mm = np.ctypeslib.as_array(m.mm, (self.M * self.D,)).reshape(self.M, self.D).copy()
        self.coeff = np.ctypeslib.as_array(m.coeff, (self.M,)).copy()

    def __del__(self):
        try:
            lib().orc_model_free(C.byref(self._m))
        except Exception:
            pass

    def weights(self, species):
        table = dict(zip(self.species_z.tolist(), self.species_w.tolist()))
        return np.array([table[int(z)] for z in species], dtype=np.float64)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def nabc(lat, rcut):
    out = np.zeros(3, np.int32)
    lib().orc_nabc(_f64(lat, (3, 3)), rcut, out)
    return out


def neighbors(lat, pos, weights, rcut, max_nb=1000):
    """(count[N], nb[N, max_nb, 6]) with nb = (x, y, z, r, w_j, j+1)."""
    pos = _f64(pos)
    na = pos.shape[0]
    count = np.zeros(na, np.int32)
    nb = np.zeros((na, max_nb, 6))
    st = lib().orc_neighbors(na, _f64(lat, (3, 3)), pos, _f64(weights), rcut, max_nb, count, nb)
    if st:
        raise OracleError(f"orc_neighbors status {st}")
    return count, nb


def car2acsf(model, pos, count, nb, lgrad=False):
    pos = _f64(pos)
    na = pos.shape[0]
    max_nb = nb.shape[1]
    xx = np.zeros((na, model.D))
    if lgrad:
        dxdy = np.zeros((3, na, na, model.D))
        strs = np.zeros((na, model.D, 3, 3))
        pd, ps = dxdy.ctypes.data, strs.ctypes.data
    else:
        dxdy = strs = None
        pd = ps = None
    st = lib().orc_car2acsf(C.byref(model._m), na, max_nb, pos, _f64(nb), np.ascontiguousarray(count, np.int32),
                            xx, pd, ps, int(lgrad))
    if st:
        raise OracleError(f"orc_car2acsf status {st}")
    return xx, dxdy, strs


def gap_calc(model, species, lat, pos, rcut=6.0, lgrad=True, extras=False):
    """FGAP_CALC: (energy, force[N,3], stress[6] GPa XX YY ZZ XY YZ ZX, variance).

    With extras=True also returns dict(xx, dedg, e) of the intermediates."""
    pos = _f64(pos)
    na = pos.shape[0]
    sp = np.ascontiguousarray(species, dtype=np.int32)
    ene = C.c_double()
    var = C.c_double()
    force = np.zeros((na, 3))
    stress = np.zeros(6)
    xx = np.zeros((na, model.D))
    dedg = np.zeros((na, model.D))
    e = np.zeros(na)
    st = lib().orc_gap_calc(C.byref(model._m), na, sp, _f64(lat, (3, 3)), pos, rcut, int(lgrad),
                            C.byref(ene), force, stress, C.byref(var),
                            xx.ctypes.data, dedg.ctypes.data, e.ctypes.data)
    if st:
        raise OracleError(f"orc_gap_calc status {st}")
    out = (ene.value, force, stress, var.value)
    if extras:
        return out + (dict(xx=xx, dedg=dedg, e=e),)
    return out


def gap_calc_batch(model, atom_off, species, lat, pos, rcut=6.0, nthreads=0):
    """Many structures on nthreads host threads (0 = OpenMP default)."""
    atom_off = np.ascontiguousarray(atom_off, np.int32)
    ns = atom_off.shape[0] - 1
    ene = np.zeros(ns)
    force = np.zeros((int(atom_off[-1]), 3))
    stress = np.zeros((ns, 6))
    st = lib().orc_gap_calc_batch(C.byref(model._m), ns, atom_off, np.ascontiguousarray(species, np.int32),
                                  _f64(lat), _f64(pos), rcut, nthreads, ene, force, stress)
    if st:
        raise OracleError(f"orc_gap_calc_batch status {st}")
    return ene, force, stress


def variance(model, xx, qmm):
    """FGAP_CALC's commented-out variance block (gap_calc.f90:206-210) for
    descriptors xx[na, D] and qmm[M, M]: (covf[na], VARIANCE = mean)."""
    xx = _f64(xx)
    qmm = _f64(qmm)
    na = xx.shape[0]
    covf = np.zeros(na)
    var = C.c_double()
    st = lib().orc_variance(C.byref(model._m), na, xx, qmm, covf, C.byref(var))
    if st:
        raise OracleError(f"orc_variance status {st}")
    return covf, var.value


def min_bond(lat, pos, rcut=6.0):
    pos = _f64(pos)
    return lib().orc_min_bond(pos.shape[0], _f64(lat, (3, 3)), pos, rcut)
