"""NVE velocity-Verlet molecular dynamics on the GPU (the gapgb_md_* C ABI).

Every step (kick + drift, neighbour rebuild or refresh, evaluation, kick,
kinetic energy) is one CUDA-graph launch inside libgapgb; PyTorch only holds
the device buffers.  Units: Angstrom, fs, amu, eV.
"""
import ctypes as C

import numpy as np

from . import _check, _f64, _i32, load

# standard atomic masses (amu)
MASSES = {3: 6.94, 6: 12.011, 8: 15.999, 13: 26.9815385, 14: 28.0855, 26: 55.845,
          28: 58.6934, 32: 72.630, 40: 91.224}
KB = 8.617333262e-5          # eV / K
EV_PER_AMU_A2_FS2 = 103.642697


def masses_of(species):
    return np.array([MASSES[int(z)] for z in species], np.float64)


def maxwell_boltzmann(atom_off, masses, T, seed=0):
    """Seeded Maxwell-Boltzmann velocities (A/fs) at temperature T with the
    centre-of-mass momentum of every structure removed."""
    rng = np.random.default_rng(seed)
    m = np.asarray(masses, np.float64)
    sig = np.sqrt(KB * T / (m * EV_PER_AMU_A2_FS2))
    v = rng.normal(0.0, 1.0, (len(m), 3)) * sig[:, None]
    off = np.asarray(atom_off)
    for s in range(len(off) - 1):
        a, b = off[s], off[s + 1]
        v[a:b] -= (m[a:b, None] * v[a:b]).sum(0) / m[a:b].sum()
    return v


def kinetic(masses, vel):
    return 0.5 * EV_PER_AMU_A2_FS2 * float((np.asarray(masses)[:, None] * np.asarray(vel) ** 2).sum())


class MD:
    """gapgb_md bound to device copies of a packed batch (the model is
    dedicated to this object while it lives)."""

    def __init__(self, model, atom_off, species, lat, pos, vel, masses, dt=1.0, skin=0.5,
                 rebuild_every=10):
        import torch
        self.model = model
        off = _i32(atom_off)
        self.S, self.N = len(off) - 1, int(off[-1])
        dev = torch.device("cuda", torch.cuda.current_device())
        self.t = {
            "off": torch.from_numpy(off).to(dev),
            "sp": torch.from_numpy(_i32(species)).to(dev),
            "lat": torch.from_numpy(_f64(lat, (self.S, 3, 3)).copy()).to(dev),
            "pos": torch.from_numpy(_f64(pos, (self.N, 3)).copy()).to(dev),
            "vel": torch.from_numpy(_f64(vel, (self.N, 3)).copy()).to(dev),
            "mass": torch.from_numpy(_f64(masses).copy()).to(dev),
        }
        torch.cuda.synchronize(dev)
        h = C.c_void_p()
        t = self.t
        _check(load().gapgb_md_create(model.handle, self.S, self.N, t["off"].data_ptr(),
                                      t["sp"].data_ptr(), t["lat"].data_ptr(), t["pos"].data_ptr(),
                                      t["vel"].data_ptr(), t["mass"].data_ptr(), float(dt),
                                      float(skin), int(rebuild_every), C.byref(h)),
               "gapgb_md_create")
        self._h = h
        self.dev = dev

    @property
    def handle(self):
        return self._h

    def run(self, nsteps, record=True):
        """Advance nsteps; returns (epot[nsteps, S], ekin[nsteps, S]) as numpy
        arrays when record, else None."""
        import torch
        ep = ek = None
        if record:
            ep = torch.zeros((nsteps, self.S), dtype=torch.float64, device=self.dev)
            ek = torch.zeros((nsteps, self.S), dtype=torch.float64, device=self.dev)
        torch.cuda.synchronize(self.dev)
        _check(load().gapgb_md_run(self._h, int(nsteps), ep.data_ptr() if record else None,
                                   ek.data_ptr() if record else None, None), "gapgb_md_run")
        self.check()
        if record:
            return ep.cpu().numpy(), ek.cpu().numpy()
        return None

    def run_async(self, nsteps, stream):
        _check(load().gapgb_md_run(self._h, int(nsteps), None, None, stream or None), "gapgb_md_run")

    def check(self):
        _check(load().gapgb_md_check(self._h), "gapgb_md_check")

    def outputs(self):
        """(energy[S], force[N, 3], stress[S, 6], ekin[S]) of the latest step."""
        ptrs = [C.c_void_p() for _ in range(4)]
        _check(load().gapgb_md_outputs(self._h, *[C.byref(p) for p in ptrs]), "gapgb_md_outputs")
        self.check()
        out = [device_copy(p.value, n)
               for p, n in zip(ptrs, (self.S, 3 * self.N, 6 * self.S, self.S))]
        return out[0], out[1].reshape(self.N, 3), out[2].reshape(self.S, 6), out[3]

    def positions(self):
        import torch
        torch.cuda.synchronize(self.dev)
        return self.t["pos"].cpu().numpy().copy()

    def velocities(self):
        import torch
        torch.cuda.synchronize(self.dev)
        return self.t["vel"].cpu().numpy().copy()

    def close(self):
        if getattr(self, "_h", None):
            load().gapgb_md_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def device_copy(dptr, n):
    """Host copy of n doubles at device pointer dptr."""
    import torch
    return torch.as_tensor(_DevicePtr(dptr, n), device="cuda").cpu().numpy().copy()


class _DevicePtr:
    """Minimal __cuda_array_interface__ view of a device double array."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False),
                                         "version": 3}
