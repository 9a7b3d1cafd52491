"""The learned surrogate: its CPU oracle, the CUDA training / prediction
kernels against that oracle, and the surrogate-with-GPR-fallback evaluation
against the exact GPR.

The CPU tests check oracle/mlp_ref.py (the float64 statement of the network,
its input gradient and the double-backpropagation weight gradient) against
finite differences.  The GPU tests call the C ABI: one training step's weight
gradient, the committee prediction and the Adam update are compared with the
oracle evaluated with the same BF16 rounding points; then a committee is
trained on GAP labels and evaluated through GapModel at precision
"surrogate", which must stay within 1 meV/atom and 20 meV/A of the exact GPR
on held-out structures, fall back exactly, and be faster than the plain FP64
path - the gain the trained network brings over the GPR alone.
"""
import time

import numpy as np
import pytest

import oracle.mlp_ref as MR

# tolerances of the GPU-vs-oracle checks (BF16 operands on both sides; the
# remaining differences are FP32 accumulation order, __expf, and BF16 ties
# that FP32-vs-FP64 rounding pushes to the other side)
GRAD_REL = 3e-3   # relative Frobenius norm of each block's weight gradient
LOSS_REL = 1e-4
PRED_ABS = 1e-4   # normalised units (y), i.e. 1e-4 * e_scale eV
E_TOL = 1e-3      # eV / atom, surrogate vs exact GPR (RMS over held-out atoms)
F_TOL = 0.020     # eV / A, RMS over held-out force components


# ---- CPU: the oracle itself ----------------------------------------------

def test_mlp_ref_weight_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    D, H = 6, 5
    p = rng.normal(0, 0.6, MR.layout(D, H)["P"])
    x = rng.normal(0, 1, (11, D))
    y = rng.normal(0, 1, 11)
    t = rng.normal(0, 1, (11, D))
    _, g = MR.loss_and_grad(p, x, y, t, 0.7, D, H)
    ng = MR.numeric_grad(p, x, y, t, 0.7, D, H)
    assert np.abs(g - ng).max() <= 1e-7 * np.abs(ng).max()


def test_mlp_ref_input_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    D, H = 5, 7
    p = rng.normal(0, 0.6, MR.layout(D, H)["P"])
    x = rng.normal(0, 1, (4, D))
    g = MR.forward(p, x, D, H)["g"]
    h = 1e-6
    for d in range(D):
        xp, xm = x.copy(), x.copy()
        xp[:, d] += h
        xm[:, d] -= h
        fd = (MR.forward(p, xp, D, H)["y"] - MR.forward(p, xm, D, H)["y"]) / (2 * h)
        assert np.allclose(fd, g[:, d], atol=1e-8)


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2.0**-8, 1.0 + 3 * 2.0**-9, -2.0 - 2.0**-7 - 2.0**-9, 0.0])
    assert list(MR.bf16(v)) == [1.0, 1.0, 1.0 + 2.0**-7, -2.0 - 2.0**-6, 0.0]


# ---- GPU -------------------------------------------------------------------

def _norm_inputs(rng, N, D, species):
    G = (rng.normal(0, 1, (N, D)) * rng.uniform(0.5, 3, D) + rng.uniform(-2, 2, D)).astype(np.float32)
    Z = rng.choice(species, N).astype(np.int32)
    e = rng.normal(0, 0.02, N) + np.where(Z == species[0], -1.0, -2.0)
    t = rng.normal(0, 0.05, (N, D)).astype(np.float32)
    mean, std = G.astype(np.float64).mean(0), G.astype(np.float64).std(0)
    shift = np.array([e[Z == z].mean() for z in species])
    scale = float(np.concatenate([e[Z == z] - shift[k] for k, z in enumerate(species)]).std())
    return G, Z, e, t, mean, std, shift, scale


def _std_x(G, mean, std):
    # the kernel's arithmetic: (G - mu) * (1 / sd) in FP32
    mu = mean.astype(np.float32)
    isig = (1.0 / std).astype(np.float32)
    return ((G - mu) * isig).astype(np.float64)


@pytest.mark.gpu
def test_train_step_gradient_matches_cpu_oracle(gapgb_mod):
    import torch
    import gapgb.surrogate as SU
    D, H, Q, R = 64, 128, 2, 128
    species = [13, 28]
    rng = np.random.default_rng(5)
    G, Z, e, t, mean, std, shift, scale = _norm_inputs(rng, 1500, D, species)
    sur = SU.Surrogate(species, D, H, Q, seed=11)
    sur.set_norm(mean, std, shift, scale)
    P = sur.params_per_block
    rows = np.zeros((Q, len(species), R), np.int32)
    for q in range(Q):
        for k, z in enumerate(species):
            rows[q, k] = rng.choice(np.nonzero(Z == z)[0], R, replace=False)
    dev = torch.device("cuda:0")
    dG, de, dt = (torch.from_numpy(a).to(dev) for a in (G, e, t))
    drows = torch.from_numpy(rows).to(dev)
    grad = torch.zeros(Q * len(species) * P, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()  # the step runs on the surrogate's own stream
    lam = 0.5
    w0 = sur.params()
    loss = sur.train_step_ptrs(R, drows.data_ptr(), dG.data_ptr(), de.data_ptr(), dt.data_ptr(),
                               lam, 1e-3, update=False, want_loss=True, d_grad=grad.data_ptr())
    torch.cuda.synchronize()
    g_gpu = grad.cpu().numpy().reshape(Q, len(species), P)
    assert np.array_equal(sur.params(), w0)  # update=False leaves the weights
    # the kernel's label normalisation, in its FP32 constants
    inv_es = np.float32(1.0) / np.float32(scale)
    sd32 = std.astype(np.float32)
    for q in range(Q):
        for k in range(len(species)):
            r = rows[q, k]
            x = _std_x(G[r], mean, std)
            y_lab = (e[r] - float(np.float32(shift[k]))) * float(inv_es)
            t_lab = (t[r] * sd32 * inv_es).astype(np.float64)
            l_ref, g_ref = MR.loss_and_grad(w0[q, k].astype(np.float64), x, y_lab, t_lab, lam, D, H,
                                            emulate_bf16=True)
            rel = np.linalg.norm(g_gpu[q, k] - g_ref) / np.linalg.norm(g_ref)
            assert rel <= GRAD_REL, (q, k, rel)
            assert abs(loss[q * len(species) + k] - l_ref) <= LOSS_REL * l_ref
            # each parameter tensor on its own
            L = MR.layout(D, H)
            for a, b in (("W1", "b1"), ("b1", "W2"), ("W2", "b2"), ("b2", "w3"), ("w3", "b3")):
                s = slice(L[a], L[b])
                assert np.linalg.norm(g_gpu[q, k][s] - g_ref[s]) <= 1e-2 * np.linalg.norm(g_ref[s]) + 1e-9


@pytest.mark.gpu
def test_adam_update_matches_formula(gapgb_mod):
    import torch
    import gapgb.surrogate as SU
    D, H, Q, R = 64, 128, 1, 64
    species = [14]
    rng = np.random.default_rng(2)
    G, Z, e, t, mean, std, shift, scale = _norm_inputs(rng, 300, D, species)
    sur = SU.Surrogate(species, D, H, Q, seed=1)
    sur.set_norm(mean, std, shift, scale)
    dev = torch.device("cuda:0")
    dG, de, dt = (torch.from_numpy(a).to(dev) for a in (G, e, t))
    drows = torch.from_numpy(rng.choice(300, R, replace=False).astype(np.int32)).to(dev)
    grad = torch.zeros(sur.params_per_block, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()  # the step runs on the surrogate's own stream
    w0 = sur.params().ravel().astype(np.float64)
    lr = 1e-3
    sur.train_step_ptrs(R, drows.data_ptr(), dG.data_ptr(), de.data_ptr(), dt.data_ptr(), 1.0, lr,
                        update=True, want_loss=True, d_grad=grad.data_ptr())
    torch.cuda.synchronize()
    g = grad.cpu().numpy().astype(np.float64)
    # first Adam step: m_hat = g, v_hat = g^2
    w1 = w0 - lr * g / (np.abs(g) + 1e-8)
    assert np.allclose(sur.params().ravel(), w1, rtol=1e-5, atol=1e-7)


@pytest.mark.gpu
def test_predict_matches_cpu_oracle(gapgb_mod):
    import gapgb.surrogate as SU
    D, H, Q = 64, 128, 4
    species = [13, 28, 40]
    rng = np.random.default_rng(9)
    G, Z, e, t, mean, std, shift, scale = _norm_inputs(rng, 777, D, species)
    sur = SU.Surrogate(species, D, H, Q, seed=4)
    sur.set_norm(mean, std, shift, scale)
    e_g, s_g, g_g = sur.predict(Z, G)
    w = sur.params().astype(np.float64)
    isig32 = (1.0 / std).astype(np.float32)
    for k, z in enumerate(species):
        sel = np.nonzero(Z == z)[0]
        x = _std_x(G[sel], mean, std)
        # D <= 64 and H = 128: prediction runs on the tensor cores
        e_r, s_r, g_r = MR.committee([w[q, k] for q in range(Q)], x, D, H, scale, shift[k],
                                     1.0 / isig32.astype(np.float64), emulate_bf16=True, tc=True)
        assert np.abs(e_g[sel] - e_r).max() <= PRED_ABS * scale
        assert np.abs(s_g[sel] - s_r).max() <= PRED_ABS * scale
        # gradients compared in normalised units (dy/dx)
        gn = lambda a: a / isig32 / scale
        assert np.abs(gn(g_g[sel]) - gn(g_r)).max() <= PRED_ABS
    # an atomic number outside the surrogate's species is an error, not a guess
    Zbad = Z.copy()
    Zbad[3] = 99
    with pytest.raises(gapgb_mod.GapError) as ei:
        sur.predict(Zbad, G)
    assert ei.value.status == 4


@pytest.fixture(scope="module")
def trained(gapgb_mod):
    """A committee trained on the smooth alloy GAP's labels (small budget)."""
    import torch
    import gapgb.synth as S
    import gapgb.surrogate as SU
    arrays = S.alloy_model(M=1000, theta_scale=4.0, coeff_std=1e-3, seed=0, ncells=4)
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    label_model = gapgb_mod.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
    label_model.set_precision("mixed")
    train_structs = [S.alloy512(seed=5000 + s) for s in range(96)]
    off, sp, lat, pos = S.pack(train_structs)
    G, e, t = SU.gpr_labels(label_model, off, sp, lat, pos)
    Zd = torch.from_numpy(sp).to(G.device)
    sur = SU.Surrogate(zt, G.shape[1], 128, 4, seed=0)
    SU.fit_norm(sur, G, e, Zd)
    untrained = SU.Surrogate(zt, G.shape[1], 128, 4, seed=0)
    untrained.set_norm(*sur.norm)
    hist = SU.train(sur, G, e, t, Zd, epochs=30, rows_per_species=256, lam=1.0, lr=2e-3,
                    lr_final=2e-5, seed=0)
    label_model.close()
    return arrays, sur, untrained, hist


def _eval(model, structs, prec):
    import gapgb.synth as S
    off, sp, lat, pos = S.pack(structs)
    model.set_precision(prec)
    E, F, SIG, ae = model.eval_batch(off, sp, lat, pos, atom_energy=True)
    return E, F, SIG, ae


@pytest.mark.gpu
def test_surrogate_with_fallback_against_exact_gpr(gapgb_mod, trained):
    import gapgb.synth as S
    arrays, sur, untrained, hist = trained
    assert hist[-1] < 0.25 * hist[0]
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    m = gapgb_mod.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
    held = [S.alloy512(seed=90000 + s) for s in range(6)]
    N = 512 * len(held)
    E0, F0, S0, ae0 = _eval(m, held, "fp64")
    # untrained committee, no fallback: the error the training removes
    m.attach_surrogate(untrained, threshold=np.inf)
    Eu, Fu, _, aeu = _eval(m, held, "surrogate")
    # trained committee, fallback above 5 meV committee std
    m.attach_surrogate(sur, threshold=0.005)
    E1, F1, S1, ae1 = _eval(m, held, "surrogate")
    nfb = m.fallback_count()
    e_rms = np.sqrt(np.mean((ae1 - ae0) ** 2))
    f_rms = np.sqrt(np.mean((F1 - F0) ** 2))
    eu_rms = np.sqrt(np.mean((aeu - ae0) ** 2))
    fu_rms = np.sqrt(np.mean((Fu - F0) ** 2))
    print("surrogate e_rms %.3g eV f_rms %.3g eV/A fallback %d/%d; untrained %.3g %.3g"
          % (e_rms, f_rms, nfb, N, eu_rms, fu_rms))
    assert e_rms <= E_TOL and f_rms <= F_TOL
    assert np.abs(E1 - E0).max() / 512 <= E_TOL
    assert eu_rms > 5 * e_rms and fu_rms > 3 * f_rms
    assert 0 <= nfb < N // 2
    # threshold 0: every atom takes the GPR, which is the mixed form exactly
    m.attach_surrogate(sur, threshold=0.0)
    E2, F2, S2, ae2 = _eval(m, held, "surrogate")
    assert m.fallback_count() == N
    Em, Fm, Sm, aem = _eval(m, held, "mixed")
    assert np.abs(ae2 - aem).max() <= 1e-12 * max(1.0, np.abs(aem).max())
    assert np.abs(F2 - Fm).max() <= 1e-6 * max(1.0, np.abs(Fm).max())
    # infinite threshold: nothing falls back
    m.attach_surrogate(sur, threshold=np.inf)
    _eval(m, held, "surrogate")
    assert m.fallback_count() == 0
    # detaching drops the precision back to a GPR form
    m.attach_surrogate(None)
    assert m.get_option(0) == gapgb_mod.PREC_MIXED
    with pytest.raises(gapgb_mod.GapError):
        m.set_precision("surrogate")
    m.close()


@pytest.mark.gpu
def test_surrogate_gain_over_plain_gpu_path(gapgb_mod, trained):
    """Throughput of the surrogate-with-fallback path against the plain FP64
    path on the same device-resident batch (CUDA events, after warm-up)."""
    import torch
    import gapgb.synth as S
    arrays, sur, _, _ = trained
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    structs = [S.alloy512(seed=70000 + s) for s in range(16)]
    off, sp, lat, pos = S.pack(structs)
    dev = torch.device("cuda:0")
    Sn, N = len(structs), int(off[-1])
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
         for k, v in (("off", off), ("sp", sp), ("lat", lat), ("pos", pos))}
    eo = torch.zeros(Sn, dtype=torch.float64, device=dev)
    fo = torch.zeros((N, 3), dtype=torch.float64, device=dev)
    so = torch.zeros((Sn, 6), dtype=torch.float64, device=dev)
    times = {}
    for prec in ("fp64", "surrogate"):
        m = gapgb_mod.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
        if prec == "surrogate":
            m.attach_surrogate(sur, threshold=0.005)
        m.set_precision(prec)
        m.set_neighbour_cap(128)
        stream = torch.cuda.current_stream().cuda_stream

        def step():
            m.eval_batch_ptrs(Sn, N, 512, d["off"].data_ptr(), d["sp"].data_ptr(),
                              d["lat"].data_ptr(), d["pos"].data_ptr(), 1, eo.data_ptr(),
                              fo.data_ptr(), so.data_ptr(), 0, stream)
        for _ in range(3):
            step()
        torch.cuda.synchronize()
        m.check_device_status()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(5):
            step()
        b.record()
        torch.cuda.synchronize()
        times[prec] = a.elapsed_time(b) / 5
        m.check_device_status()
        m.close()
    gain = times["fp64"] / times["surrogate"]
    print("plain fp64 %.3f ms, surrogate %.3f ms per %d atoms: %.1fx" %
          (times["fp64"], times["surrogate"], N, gain))
    assert gain > 2.0


def _with_contacts(seed, ncell=6, per_cell=4, r=2.3):
    """Held-out alloy cells in which `per_cell` atoms are moved towards their
    nearest neighbour until the pair is r apart (a short contact the training
    cells do not contain)."""
    import gapgb.synth as S
    rng = np.random.default_rng(seed)
    out = []
    for c in range(ncell):
        lat, pos, z = S.alloy512(seed=seed + c)
        pos = pos.copy()
        inv = np.linalg.inv(lat)
        for a in rng.choice(len(pos), per_cell, replace=False):
            d = (pos - pos[a]) @ inv
            d -= np.round(d)
            v = d @ lat
            r2 = (v ** 2).sum(1)
            r2[a] = np.inf
            b = int(np.argmin(r2))
            u = -v[b] / np.sqrt(r2[b])   # from b towards a
            pos[a] = pos[a] + v[b] + u * r  # a at distance r from b's image
        out.append((lat, pos, z))
    return out


@pytest.mark.gpu
def test_contact_trigger_sends_short_contacts_to_the_gpr(gapgb_mod, trained):
    """The force-sensitive trigger: with planted 2.3 A contacts, the atoms of
    every contact take the exact GPR, the fallback count rises, and the
    largest force error against the exact GPR falls within the bar."""
    arrays, sur, _, _ = trained
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    m = gapgb_mod.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
    held = _with_contacts(91000)
    E0, F0, _, ae0 = _eval(m, held, "fp64")
    m.attach_surrogate(sur, threshold=0.005, contact=0.0)
    _, F1, _, _ = _eval(m, held, "surrogate")
    n1 = m.fallback_count()
    m.attach_surrogate(sur, threshold=0.005, contact=2.45)
    E2, F2, _, ae2 = _eval(m, held, "surrogate")
    n2 = m.fallback_count()
    d1, d2 = np.abs(F1 - F0).max(), np.abs(F2 - F0).max()
    print("contacts: committee only F_max %.3g eV/A (%d fallbacks); with the contact "
          "trigger F_max %.3g eV/A (%d fallbacks of %d atoms)" % (d1, n1, d2, n2, len(F0)))
    assert n2 >= 2 * 6 * 4 and n2 > n1  # both atoms of every planted contact
    assert d2 <= 0.020
    assert d2 < d1
    assert np.abs(E2 - E0).max() / 512 <= E_TOL
    # r_contact and the gradient spread must be >= 0
    with pytest.raises(gapgb_mod.GapError):
        m.attach_surrogate(sur, threshold=0.005, contact=-1.0)
    with pytest.raises(gapgb_mod.GapError):
        m.attach_surrogate(sur, threshold=0.005, grad_spread=-1.0)
    m.close()


@pytest.mark.gpu
def test_gradient_spread_trigger(gapgb_mod, trained):
    """The members' dE/dG spread (gapgb_surrogate_predict's d_gstd) equals its
    definition on the committee's own members, and the trigger built on it
    sends exactly the atoms above the threshold to the GPR."""
    import torch
    import gapgb.synth as S
    import gapgb.surrogate as SU
    arrays, sur, _, _ = trained
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    m = gapgb_mod.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
    held = [S.alloy512(seed=93000 + s) for s in range(4)]
    off, sp, lat, pos = S.pack(held)
    m.set_precision("fp32")
    G = m.descriptors(off, sp, lat, pos).astype(np.float32)
    dev = torch.device("cuda:0")
    Gd = torch.from_numpy(G).to(dev)
    Zd = torch.from_numpy(sp.astype(np.int32)).to(dev)
    gs = SU.grad_spread(sur, Gd, Zd).cpu().numpy()
    assert np.all(np.isfinite(gs)) and gs.max() > 0
    # the definition: |std over members of dE/dG_q| with one member at a time
    w = sur.params()
    per = []
    for q in range(sur.members):
        one = SU.Surrogate(zt, sur.des_len, sur.hidden, 1, seed=0)
        one.set_norm(*sur.norm)
        one.set_params(w[q:q + 1])
        per.append(one.predict(sp, G)[2].astype(np.float64))
        one.close()
    per = np.stack(per)
    ref = np.sqrt(per.var(0, ddof=1).sum(1))
    assert np.allclose(gs, ref, rtol=2e-3, atol=1e-6 * ref.max())
    # a threshold near the 95 % quantile, in the middle of the widest gap
    # between neighbouring values there: the library's own descriptors come
    # from the FP32-form neighbour list, so its spreads may differ from gs in
    # the last bits, and no atom may sit that close to the threshold
    srt = np.sort(gs)
    lo, hi = int(0.93 * len(srt)), int(0.97 * len(srt))
    k = lo + int(np.argmax(np.diff(srt[lo:hi + 1])))
    thr = float(0.5 * (srt[k] + srt[k + 1]))
    m.attach_surrogate(sur, threshold=np.inf, grad_spread=thr)
    _eval(m, held, "surrogate")
    assert m.fallback_count() == int((gs > thr).sum())
    m.close()
