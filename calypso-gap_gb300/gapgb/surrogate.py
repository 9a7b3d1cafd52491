"""Learned surrogate with GPR fallback (the gapgb_surrogate_* C ABI).

A committee of per-species MLPs over the wACSF descriptors, trained on the
GPU by the library's own forward / backward / Adam kernels on the atomic
energies and dE/dG that the GAP itself produces, then attached to a GapModel
so that an evaluation at precision "surrogate" uses the committee mean and
sends every atom whose committee standard deviation exceeds the threshold to
the exact GPR.  PyTorch only holds the device buffers here (labels, index
lists); every computation on them is a libgapgb kernel.
"""
import ctypes as C

import numpy as np

from . import GapError, _check, _f64, _i32, _ptr, load


class Surrogate:
    """gapgb_surrogate: `members` x `nspecies` networks D -> H -> H -> 1."""

    def __init__(self, species_z, des_len, hidden=128, members=4, seed=0):
        z = _i32(species_z)
        h = C.c_void_p()
        _check(load().gapgb_surrogate_create(len(z), _ptr(z), int(des_len), int(hidden),
                                             int(members), C.c_ulonglong(seed), C.byref(h)),
               "gapgb_surrogate_create")
        self._h = h
        self.species_z = z.copy()
        nsp, D, H, Q, P = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_size_t()
        _check(load().gapgb_surrogate_info(self._h, C.byref(nsp), C.byref(D), C.byref(H),
                                           C.byref(Q), C.byref(P)), "gapgb_surrogate_info")
        self.nspecies, self.des_len, self.hidden, self.members, self.params_per_block = (
            nsp.value, D.value, H.value, Q.value, P.value)
        self.norm = None

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            load().gapgb_surrogate_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_norm(self, g_mean, g_std, e_shift, e_scale):
        g_mean, g_std, e_shift = _f64(g_mean), _f64(g_std), _f64(e_shift)
        _check(load().gapgb_surrogate_set_norm(self._h, _ptr(g_mean), _ptr(g_std), _ptr(e_shift),
                                               float(e_scale)), "gapgb_surrogate_set_norm")
        self.norm = (g_mean.copy(), g_std.copy(), e_shift.copy(), float(e_scale))

    def params(self):
        """FP32 master weights, shape (members, nspecies, params_per_block)."""
        w = np.zeros((self.members, self.nspecies, self.params_per_block), np.float32)
        _check(load().gapgb_surrogate_params(self._h, _ptr(w), None), "gapgb_surrogate_params")
        return w

    def set_params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32).reshape(
            self.members, self.nspecies, self.params_per_block)
        _check(load().gapgb_surrogate_params(self._h, None, _ptr(w)), "gapgb_surrogate_params")

    def train_step_ptrs(self, rows_per_species, d_rows, d_G, d_e, d_dedg, lam, lr, update=True,
                        want_loss=False, d_grad=0):
        loss = np.zeros(self.members * self.nspecies) if want_loss else None
        _check(load().gapgb_surrogate_train_step(self._h, int(rows_per_species), d_rows, d_G, d_e,
                                                 d_dedg, C.c_float(lam), C.c_float(lr),
                                                 int(bool(update)), _ptr(loss), d_grad or None),
               "gapgb_surrogate_train_step")
        return loss

    def predict_ptrs(self, natoms, d_species, d_G, d_e, d_std, d_dedg, stream=0, d_gstd=0):
        _check(load().gapgb_surrogate_predict(self._h, int(natoms), d_species, d_G, d_e, d_std,
                                              d_dedg, d_gstd or None, stream or None),
               "gapgb_surrogate_predict")

    def predict(self, species, G):
        """Host convenience: (e[N], std[N], dedg[N, D]) for FP32 descriptors G."""
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        Z = torch.from_numpy(_i32(species)).to(dev)
        Gd = torch.from_numpy(np.ascontiguousarray(G, np.float32)).to(dev)
        n = Gd.shape[0]
        e = torch.empty(n, dtype=torch.float64, device=dev)
        sd = torch.empty(n, dtype=torch.float32, device=dev)
        dg = torch.empty((n, self.des_len), dtype=torch.float32, device=dev)
        self.predict_ptrs(n, Z.data_ptr(), Gd.data_ptr(), e.data_ptr(), sd.data_ptr(), dg.data_ptr(),
                          torch.cuda.current_stream().cuda_stream)
        return e.cpu().numpy(), sd.cpu().numpy(), dg.cpu().numpy()


def grad_spread(sur, G, Z, chunk=1 << 18):
    """The committee members' dE/dG spread of every row of the CUDA tensors
    G [N, D] float32 and Z [N] int32 (eV per descriptor unit), as the
    force-sensitive fallback trigger reads it: e.g. a high quantile of it
    over training atoms calibrates that trigger."""
    import torch
    n = G.shape[0]
    out = torch.empty(n, dtype=torch.float32, device=G.device)
    e = torch.empty(min(n, chunk), dtype=torch.float64, device=G.device)
    sd = torch.empty(min(n, chunk), dtype=torch.float32, device=G.device)
    dg = torch.empty((min(n, chunk), sur.des_len), dtype=torch.float32, device=G.device)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        Gc = G[a:b].contiguous()
        Zc = Z[a:b].contiguous()
        sur.predict_ptrs(b - a, Zc.data_ptr(), Gc.data_ptr(), e.data_ptr(), sd.data_ptr(),
                         dg.data_ptr(), torch.cuda.current_stream().cuda_stream,
                         d_gstd=out[a:b].data_ptr())
    return out


def gpr_labels(model, atom_off, species, lat, pos, chunk_atoms=1 << 17):
    """(G float32 [N, D], e float64 [N], dE/dG float32 [N, D]) as CUDA tensors,
    from the model's GPR at its current precision, in chunks of whole
    structures of about chunk_atoms atoms."""
    import torch
    off = _i32(atom_off)
    S = off.shape[0] - 1
    N = int(off[-1])
    D = model.des_len
    sp = _i32(species)
    lat = _f64(lat, (S, 3, 3))
    pos = _f64(pos, (N, 3))
    dev = torch.device("cuda", torch.cuda.current_device())
    G = torch.empty((N, D), dtype=torch.float32, device=dev)
    e = torch.empty(N, dtype=torch.float64, device=dev)
    t = torch.empty((N, D), dtype=torch.float32, device=dev)
    s0 = 0
    while s0 < S:
        s1 = s0 + 1
        while s1 < S and off[s1 + 1] - off[s0] <= chunk_atoms:
            s1 += 1
        a0, a1 = int(off[s0]), int(off[s1])
        o = np.ascontiguousarray(off[s0:s1 + 1] - a0, np.int32)
        _check(load().gapgb_gpr_labels(model.handle, s1 - s0, _ptr(o), _ptr(sp[a0:a1]),
                                       _ptr(lat[s0:s1]), _ptr(pos[a0:a1]),
                                       G[a0:a1].data_ptr(), e[a0:a1].data_ptr(),
                                       t[a0:a1].data_ptr()), "gapgb_gpr_labels")
        s0 = s1
    return G, e, t


def fit_norm(sur, G, e, Z):
    """Standardisation from the training labels: descriptor mean / std, per
    species energy mean (shift) and the pooled energy std (scale)."""
    import torch
    g_mean = G.double().mean(0).cpu().numpy()
    g_std = G.double().std(0).cpu().numpy()
    shift = np.zeros(sur.nspecies)
    resid = []
    for k, z in enumerate(sur.species_z):
        sel = Z == int(z)
        if bool(sel.any()):
            shift[k] = float(e[sel].mean())
            resid.append(e[sel] - shift[k])
    scale = float(torch.cat(resid).std()) if resid else 1.0
    sur.set_norm(g_mean, g_std, shift, scale if scale > 0 else 1.0)


def train(sur, G, e, t, Z, epochs=10, rows_per_species=1024, lam=1.0, lr=2e-3, lr_final=2e-5,
          seed=0, log=None):
    """Adam training of every committee member on the labels (CUDA tensors
    G [N, D] float32, e [N] float64, t [N, D] float32, Z [N] int32 atomic
    numbers).  An epoch is enough steps for every member to see every atom of
    the most frequent species once, each member in its own order; rows of the
    rarer species wrap around.  Cosine learning-rate decay from lr to
    lr_final.  Returns the per-epoch mean block loss."""
    import torch
    R = int(rows_per_species)
    dev = G.device
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    pools = []
    for z in sur.species_z:
        idx = torch.nonzero(Z == int(z)).flatten().to(torch.int32)
        if idx.numel() == 0:
            raise GapError(4, "surrogate train: no training atoms of Z=%d" % int(z))
        pools.append(idx)
    steps = max(1, -(-max(int(p.numel()) for p in pools) // R))
    total = steps * epochs
    hist = []
    k = 0
    for ep in range(epochs):
        # [steps, members, nspecies, R] rows, an independent order per member
        rows = torch.empty((steps, sur.members, sur.nspecies, R), dtype=torch.int32, device=dev)
        for q in range(sur.members):
            for s, pool in enumerate(pools):
                n = pool.numel()
                need = steps * R
                order = torch.cat([torch.randperm(n, generator=gen, device=dev)
                                   for _ in range(-(-need // n))])[:need]
                rows[:, q, s, :] = pool[order].view(steps, R)
        # the steps run on the surrogate's own stream: the index lists (made
        # on torch's stream) must be complete first
        torch.cuda.synchronize(dev)
        acc = 0.0
        for st in range(steps):
            lr_k = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * k / max(1, total - 1)))
            want = st == steps - 1
            loss = sur.train_step_ptrs(R, rows[st].data_ptr(), G.data_ptr(), e.data_ptr(),
                                       t.data_ptr(), lam, lr_k, True, want)
            if want:
                acc = float(np.mean(loss))
            k += 1
        hist.append(acc)
        if log:
            log("epoch %d loss %.4g" % (ep, acc))
    return hist
