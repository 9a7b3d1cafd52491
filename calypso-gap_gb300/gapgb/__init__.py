"""gapgb - GB300 (sm_103a) CALYPSO-GAP energy / force / stress evaluator.

Python binding of the C ABI in include/gapgb.h (libgapgb.so, built by
gapgb.build).  The product path is the CUDA library: nothing here computes
on the CPU, and every call fails loudly if the library cannot be loaded.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

PREC_FP64, PREC_FP32, PREC_TC, PREC_MIXED, PREC_SURROGATE, PREC_TF32 = 0, 1, 2, 3, 4, 5
OPT_PRECISION, OPT_NEIGHBOUR_CAP, OPT_DEVICE, OPT_GENERIC_KERNELS, OPT_PIPELINES = 0, 1, 2, 3, 4
PRECISIONS = {"fp64": PREC_FP64, "fp32": PREC_FP32, "tc": PREC_TC, "mixed": PREC_MIXED,
              "surrogate": PREC_SURROGATE, "tf32": PREC_TF32}

STATUS = {
    0: "OK", 1: "ERR_FILE", 2: "ERR_PARSE", 3: "ERR_CAP_EXCEEDED", 4: "ERR_UNKNOWN_SPECIES",
    5: "ERR_NEIGHBOUR_OVERFLOW", 6: "ERR_CUDA", 7: "ERR_TIMEOUT", 8: "ERR_ARG", 9: "ERR_ALLOC",
    10: "ERR_NO_DEVICE",
}

# (name, restype, argtypes) of every symbol declared in include/gapgb.h
_P = C.c_void_p
_I = C.c_int
_D = C.c_double
SYMBOLS = [
    ("gapgb_status_string", C.c_char_p, [_I]),
    ("gapgb_last_error", C.c_char_p, []),
    ("gapgb_version", C.c_char_p, []),
    ("gapgb_model_load", _I, [C.c_char_p, _D, C.POINTER(_P)]),
    ("gapgb_model_create", _I, [_I, _P, _P, _I, _P, _P, _P, _P, _I, _I, _P, _P, _P, _D, C.POINTER(_P)]),
    ("gapgb_model_write", _I, [_P, C.c_char_p]),
    ("gapgb_model_set_qmm", _I, [_P, _P, _I]),
    ("gapgb_model_set_coeff", _I, [_P, _P]),
    ("gapgb_fit_energies", _I, [_P, _I, _P, _P, _P, _P, _P, _D, _D, _P]),
    ("gapgb_fit", _I, [_P, _I, _P, _P, _P, _P, _P, _P, _P, _D, _D, _D, _D, _P]),
    ("gapgb_variance", _I, [_P, _I, _P, _P, _P, _P, _P, _P]),
    ("gapgb_variance_time", _I, [_P, C.POINTER(C.c_float)]),
    ("gapgb_model_free", None, [_P]),
    ("gapgb_model_info", _I, [_P, _P, _P, _P, _P, _P]),
    ("gapgb_model_arrays", _I, [_P, _P, _P, _P]),
    ("gapgb_model_tables", _I, [_P, _P, _P, _P, _P, _P, _P]),
    ("gapgb_set_option", _I, [_P, _I, C.c_int64]),
    ("gapgb_get_option", _I, [_P, _I, _P]),
    ("gapgb_eval", _I, [_P, _I, _P, _P, _P, _I, _P, _P, _P, _P]),
    ("gapgb_eval_batch", _I, [_P, _I, _P, _P, _P, _P, _I, _P, _P, _P, _P]),
    ("gapgb_eval_batch_device", _I, [_P, _I, _I, _I, _P, _P, _P, _P, _I, _P, _P, _P, _P, _P]),
    ("gapgb_check_device_status", _I, [_P]),
    ("gapgb_graph_create", _I, [_P, _I, _I, _I, _P, _P, _P, _P, _I, _P, _P, _P, _P, C.POINTER(_P)]),
    ("gapgb_graph_launch", _I, [_P, _P]),
    ("gapgb_graph_free", None, [_P]),
    ("gapgb_gpr_noalloc", _I, [_P, _I, _P, _P, _P, _P]),
    ("gapgb_stage_times", _I, [_P, _P]),
    ("gapgb_measure_peaks", _I, [_P]),
    ("gapgb_surrogate_create", _I, [_I, _P, _I, _I, _I, C.c_ulonglong, C.POINTER(_P)]),
    ("gapgb_surrogate_free", None, [_P]),
    ("gapgb_surrogate_info", _I, [_P, _P, _P, _P, _P, _P]),
    ("gapgb_surrogate_set_norm", _I, [_P, _P, _P, _P, _D]),
    ("gapgb_surrogate_params", _I, [_P, _P, _P]),
    ("gapgb_surrogate_train_step", _I, [_P, _I, _P, _P, _P, _P, C.c_float, C.c_float, _I, _P, _P]),
    ("gapgb_surrogate_predict", _I, [_P, _I, _P, _P, _P, _P, _P, _P, _P]),
    ("gapgb_model_set_surrogate", _I, [_P, _P, _D]),
    ("gapgb_model_set_fallback_triggers", _I, [_P, _D, _D]),
    ("gapgb_surrogate_fallback_count", _I, [_P, _P]),
    ("gapgb_gpr_labels", _I, [_P, _I, _P, _P, _P, _P, _P, _P, _P]),
    ("gapgb_md_create", _I, [_P, _I, _I, _P, _P, _P, _P, _P, _P, _D, _D, _I, C.POINTER(_P)]),
    ("gapgb_md_run", _I, [_P, _I, _P, _P, _P]),
    ("gapgb_md_outputs", _I, [_P, _P, _P, _P, _P]),
    ("gapgb_md_check", _I, [_P]),
    ("gapgb_md_free", None, [_P]),
    ("gapgb_descriptors", _I, [_P, _I, _P, _P, _P, _P, _P]),
    ("gapgb_neighbors", _I, [_P, _I, _P, _P, _P, _I, _P, _P]),
    ("gapgb_min_bond", _I, [_I, _P, _P, _D, _P]),
]
FORTRAN_SYMBOLS = ["fgap_read_", "fgap_calc_", "fget_bond_"]

_lib = None


class GapError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        msg = "%s: %s (%s)" % (where, STATUS.get(status, status), last_error())
        super().__init__(msg)


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libgapgb.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError("libgapgb.so not built: run gapgb.build.build()")
        _build.build()
    L = C.CDLL(path)
    for name, res, args in SYMBOLS:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def last_error():
    if _lib is None:
        return ""
    return _lib.gapgb_last_error().decode(errors="replace")


def _check(st, where):
    if st != 0:
        raise GapError(st, where)


def _ptr(a):
    return a.ctypes.data if a is not None else None


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def measure_peaks():
    """Measured FP32 / FP64 FMA rates (TFLOP/s) and MUFU ex2 rate (1e12/s)
    of the current device."""
    out = (C.c_double * 3)()
    _check(load().gapgb_measure_peaks(out), "gapgb_measure_peaks")
    return {"fp32_tflops": out[0], "fp64_tflops": out[1], "ex2_per_s_1e12": out[2]}


class GapModel:
    """A GAP model resident on one GPU (gapgb_model)."""

    def __init__(self, handle):
        self._h = handle
        L = load()
        M, D, nsf, nsp, rc = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_double()
        _check(L.gapgb_model_info(self._h, C.byref(M), C.byref(D), C.byref(nsf), C.byref(nsp),
                                  C.byref(rc)), "gapgb_model_info")
        self.nsparse, self.des_len, self.nsf, self.nspecies, self.rcut = (
            M.value, D.value, nsf.value, nsp.value, rc.value)

    @classmethod
    def load(cls, path, rcut=6.0):
        h = C.c_void_p()
        _check(load().gapgb_model_load(os.fsencode(path), float(rcut), C.byref(h)),
               "gapgb_model_load")
        return cls(h)

    @classmethod
    def create(cls, species_z, species_w, sf_type, sf_alpha, sf_cutoff, theta, mm, coeff,
               sf_zeta=None, rcut=6.0):
        z = _i32(species_z)
        w = _f64(species_w)
        ty = _i32(sf_type)
        al = _f64(sf_alpha)
        cu = _f64(sf_cutoff)
        ze = _f64(sf_zeta) if sf_zeta is not None else None
        th = _f64(theta)
        mm = _f64(mm)
        co = _f64(coeff)
        h = C.c_void_p()
        _check(load().gapgb_model_create(len(z), _ptr(z), _ptr(w), len(ty), _ptr(ty), _ptr(al),
                                         _ptr(cu), _ptr(ze), mm.shape[0], mm.shape[1], _ptr(th),
                                         _ptr(mm), _ptr(co), float(rcut), C.byref(h)),
               "gapgb_model_create")
        return cls(h)

    def save(self, path):
        """Write the model as a gap_parameters file (gapgb_model_write)."""
        _check(load().gapgb_model_write(self._h, os.fsencode(path)), "gapgb_model_write")
        return path

    def close(self):
        if getattr(self, "_h", None):
            load().gapgb_model_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def arrays(self):
        th = np.zeros(self.des_len)
        mm = np.zeros((self.nsparse, self.des_len))
        co = np.zeros(self.nsparse)
        _check(load().gapgb_model_arrays(self._h, _ptr(th), _ptr(mm), _ptr(co)), "gapgb_model_arrays")
        return th, mm, co

    def tables(self):
        """(species_z, species_w, sf_type, sf_alpha, sf_cutoff, sf_zeta)."""
        z = np.zeros(self.nspecies, np.int32)
        w = np.zeros(self.nspecies)
        ty = np.zeros(self.nsf, np.int32)
        al = np.zeros(self.nsf)
        cu = np.zeros(self.nsf)
        ze = np.zeros(self.nsf)
        _check(load().gapgb_model_tables(self._h, _ptr(z), _ptr(w), _ptr(ty), _ptr(al), _ptr(cu),
                                         _ptr(ze)), "gapgb_model_tables")
        return z, w, ty, al, cu, ze

    def set_coeff(self, coeff):
        c = _f64(coeff, (self.nsparse,))
        _check(load().gapgb_model_set_coeff(self._h, _ptr(c)), "gapgb_model_set_coeff")

    def fit_energies(self, atom_off, species, lat, pos, energy, sigma_e=1e-3, jitter=1e-8):
        """Fit the coefficients to structure energies (eV) on the device and
        set them on the model; returns them."""
        off = _i32(atom_off)
        S = off.shape[0] - 1
        N = int(off[-1])
        c = np.zeros(self.nsparse)
        _check(load().gapgb_fit_energies(self._h, S, _ptr(off), _ptr(_i32(species)),
                                         _ptr(_f64(lat, (S, 3, 3))), _ptr(_f64(pos, (N, 3))),
                                         _ptr(_f64(energy, (S,))), float(sigma_e), float(jitter),
                                         _ptr(c)), "gapgb_fit_energies")
        return c

    def fit(self, atom_off, species, lat, pos, energy, forces=None, stress=None, sigma_e=1e-3,
            sigma_f=0.1, sigma_s=0.1, jitter=1e-8):
        """Fit the coefficients to structure energies (eV) and, when given,
        forces [N, 3] (eV/A) and stresses [S, 6] (GPa, XX YY ZZ XY YZ ZX) on
        the device; sets and returns them."""
        off = _i32(atom_off)
        S = off.shape[0] - 1
        N = int(off[-1])
        c = np.zeros(self.nsparse)
        fv = _f64(forces, (N, 3)) if forces is not None else None
        sv = _f64(stress, (S, 6)) if stress is not None else None
        _check(load().gapgb_fit(self._h, S, _ptr(off), _ptr(_i32(species)),
                                _ptr(_f64(lat, (S, 3, 3))), _ptr(_f64(pos, (N, 3))),
                                _ptr(_f64(energy, (S,))), _ptr(fv), _ptr(sv), float(sigma_e),
                                float(sigma_f), float(sigma_s), float(jitter), _ptr(c)),
               "gapgb_fit")
        return c

    def set_qmm(self, qmm):
        """Attach qmm [M, M] for the predictive variance (None detaches)."""
        if qmm is None:
            _check(load().gapgb_model_set_qmm(self._h, None, 0), "gapgb_model_set_qmm")
            return
        q = _f64(qmm, (self.nsparse, self.nsparse))
        _check(load().gapgb_model_set_qmm(self._h, _ptr(q), self.nsparse), "gapgb_model_set_qmm")

    def variance(self, atom_off, species, lat, pos):
        """Packed batch: (covf[N], variance[S]) of the GPR variance block."""
        off = _i32(atom_off)
        S = off.shape[0] - 1
        N = int(off[-1])
        sp = _i32(species)
        covf = np.zeros(N)
        var = np.zeros(S)
        _check(load().gapgb_variance(self._h, S, _ptr(off), _ptr(sp), _ptr(_f64(lat, (S, 3, 3))),
                                     _ptr(_f64(pos, (N, 3))), _ptr(covf), _ptr(var)),
               "gapgb_variance")
        return covf, var

    def set_precision(self, prec):
        prec = PRECISIONS.get(prec, prec)
        _check(load().gapgb_set_option(self._h, OPT_PRECISION, int(prec)), "gapgb_set_option")

    def set_neighbour_cap(self, cap):
        _check(load().gapgb_set_option(self._h, OPT_NEIGHBOUR_CAP, int(cap)), "gapgb_set_option")

    def set_pipelines(self, n):
        """1: one stream; 2 (default): large TC / TF32 batches run as two
        halves on two streams (GAPGB_OPT_PIPELINES)."""
        _check(load().gapgb_set_option(self._h, OPT_PIPELINES, int(n)), "gapgb_set_option")

    def get_option(self, opt):
        v = C.c_int64()
        _check(load().gapgb_get_option(self._h, opt, C.byref(v)), "gapgb_get_option")
        return v.value

    def eval(self, species, lat, pos, lgrad=True):
        """One structure: (energy, force[N,3], stress[6] GPa XX YY ZZ XY YZ ZX, variance)."""
        sp = _i32(species)
        pos = _f64(pos, (-1, 3))
        n = pos.shape[0]
        e = C.c_double()
        var = C.c_double()
        f = np.zeros((n, 3))
        s = np.zeros(6)
        _check(load().gapgb_eval(self._h, n, _ptr(sp), _ptr(_f64(lat, (3, 3))), _ptr(pos),
                                 int(bool(lgrad)), C.byref(e), _ptr(f), _ptr(s), C.byref(var)),
               "gapgb_eval")
        return e.value, f, s, var.value

    def eval_batch(self, atom_off, species, lat, pos, lgrad=True, atom_energy=False):
        """Packed batch: (energy[S], force[N,3], stress[S,6] [, atom_energy[N]])."""
        off = _i32(atom_off)
        S = off.shape[0] - 1
        N = int(off[-1])
        sp = _i32(species)
        lat = _f64(lat, (S, 3, 3))
        pos = _f64(pos, (N, 3))
        e = np.zeros(S)
        f = np.zeros((N, 3))
        s = np.zeros((S, 6))
        ae = np.zeros(N) if atom_energy else None
        _check(load().gapgb_eval_batch(self._h, S, _ptr(off), _ptr(sp), _ptr(lat), _ptr(pos),
                                       int(bool(lgrad)), _ptr(e), _ptr(f), _ptr(s), _ptr(ae)),
               "gapgb_eval_batch")
        return (e, f, s, ae) if atom_energy else (e, f, s)

    def eval_batch_ptrs(self, nstruct, natoms, max_atoms, atom_off, species, lat, pos, lgrad,
                        energy, force, stress, atom_energy=0, stream=0):
        """Device-buffer call with raw pointers (ints), enqueued on `stream`."""
        _check(load().gapgb_eval_batch_device(self._h, nstruct, natoms, max_atoms, atom_off,
                                              species, lat, pos, int(lgrad), energy, force,
                                              stress, atom_energy or None, stream or None),
               "gapgb_eval_batch_device")

    def eval_batch_host_ptrs(self, nstruct, atom_off, species, lat, pos, lgrad, energy, force,
                             stress):
        """Host-buffer call with raw pointers (ints) - e.g. pinned buffers."""
        _check(load().gapgb_eval_batch(self._h, nstruct, atom_off, species, lat, pos, int(lgrad),
                                       energy, force, stress, None), "gapgb_eval_batch")

    def graph(self, nstruct, natoms, max_atoms, atom_off, species, lat, pos, lgrad, energy, force,
              stress, atom_energy=0):
        """Capture the device-buffer evaluation on these device pointers into a
        CUDA graph (see gapgb_graph_create); returns a Graph."""
        h = C.c_void_p()
        _check(load().gapgb_graph_create(self._h, nstruct, natoms, max_atoms, atom_off, species, lat,
                                         pos, int(lgrad), energy, force, stress,
                                         atom_energy or None, C.byref(h)), "gapgb_graph_create")
        return Graph(h, self)

    def attach_surrogate(self, sur, threshold=0.005, contact=0.0, grad_spread=0.0):
        """Use a trained gapgb.surrogate.Surrogate at precision "surrogate";
        atoms whose committee std exceeds `threshold` (eV), whose members'
        dE/dG spread exceeds `grad_spread` (eV per descriptor unit, 0 = off),
        or with a neighbour closer than `contact` (Angstrom, 0 = off), take
        the GPR."""
        _check(load().gapgb_model_set_surrogate(self._h, sur.handle if sur is not None else None,
                                                float(threshold)), "gapgb_model_set_surrogate")
        self._surrogate = sur  # keeps it alive while attached
        _check(load().gapgb_model_set_fallback_triggers(self._h, float(grad_spread),
                                                        float(contact)),
               "gapgb_model_set_fallback_triggers")

    def fallback_count(self):
        """Atoms sent to the GPR by the last surrogate evaluation."""
        n = C.c_int()
        _check(load().gapgb_surrogate_fallback_count(self._h, C.byref(n)),
               "gapgb_surrogate_fallback_count")
        return n.value

    def check_device_status(self):
        _check(load().gapgb_check_device_status(self._h), "gapgb_check_device_status")

    def variance_time(self):
        """Device ms of the last gapgb_variance call's variance kernels
        (GAPGB_PROFILE_STAGES set before the model's first GPU call)."""
        t = C.c_float()
        _check(load().gapgb_variance_time(self._h, C.byref(t)), "gapgb_variance_time")
        return t.value

    def stage_times(self):
        t = (C.c_float * 4)()
        _check(load().gapgb_stage_times(self._h, t), "gapgb_stage_times")
        return list(t)

    def descriptors(self, atom_off, species, lat, pos):
        off = _i32(atom_off)
        S = off.shape[0] - 1
        N = int(off[-1])
        xx = np.zeros((N, self.des_len))
        _check(load().gapgb_descriptors(self._h, S, _ptr(off), _ptr(_i32(species)),
                                        _ptr(_f64(lat, (S, 3, 3))), _ptr(_f64(pos, (N, 3))),
                                        _ptr(xx)), "gapgb_descriptors")
        return xx

    def neighbors(self, species, lat, pos, cap=1000):
        pos = _f64(pos, (-1, 3))
        n = pos.shape[0]
        cnt = np.zeros(n, np.int32)
        nb = np.zeros((n, cap, 6))
        _check(load().gapgb_neighbors(self._h, n, _ptr(_i32(species)), _ptr(_f64(lat, (3, 3))),
                                      _ptr(pos), cap, _ptr(cnt), _ptr(nb)), "gapgb_neighbors")
        return cnt, nb


class Graph:
    """A captured evaluation (gapgb_graph); launch() replays it on a stream."""

    def __init__(self, handle, model):
        self._h = handle
        self.model = model  # keeps the model alive

    def launch(self, stream=0):
        _check(load().gapgb_graph_launch(self._h, stream or None), "gapgb_graph_launch")

    def close(self):
        if getattr(self, "_h", None):
            load().gapgb_graph_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def min_bond(lat, pos, rcut=6.0):
    pos = _f64(pos, (-1, 3))
    out = C.c_double()
    _check(load().gapgb_min_bond(pos.shape[0], _ptr(_f64(lat, (3, 3))), _ptr(pos), float(rcut),
                                 C.byref(out)), "gapgb_min_bond")
    return out.value


def write_parameters(path, species_z, species_w, sf_type, sf_alpha, sf_cutoff, theta, mm, coeff,
                     sf_zeta=None):
    """Write a gap_parameters file from arrays: the species table (Z, weight),
    the SF table (type, alpha, cutoff[, zeta]), theta[D], mm[M, D] and
    coeff[M] - the file FGAP_READ / CAR2ACSF read (gap_calc.f90:303-364,
    wacsf.f90:45-56).  Returns path."""
    m = GapModel.create(species_z, species_w, sf_type, sf_alpha, sf_cutoff, theta, mm, coeff,
                        sf_zeta=sf_zeta)
    try:
        return m.save(path)
    finally:
        m.close()
