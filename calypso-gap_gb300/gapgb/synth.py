"""Seeded synthetic structures and GAP models for the benchmark workloads.

No public dataset is used: every structure and model here is generated from
numpy ``default_rng(seed)`` with the shapes and distributions of the five
workloads the evaluator is measured on:

  si64      periodic Si diamond 2x2x2 conventional (64 atoms), a = 5.43 A,
            jitter N(0, 0.05 A); 20 radial + 12 angular SFs (D = 64); M = 500
  alloy512  fcc 4x4x8 conventional (512 atoms), a = 3.9 A, Z = 13/28/40 at
            0.5/0.3/0.2 shuffled, jitter 0.08 A; D = 64; M = 4000, theta 0.8
  population  structures of 8-256 atoms, 1-4 species from {3, 8, 14, 26},
            12-20 A^3/atom, triclinic angles 60-120 deg, min distance 1.6 A
  sige      Si/Ge 50/50 diamond 16x16x16 (32768 atoms), a = 5.54 A, jitter 0.1
  surrogate the alloy512 generator with a smooth alloy GAP (theta = 4 std):
            the narrow theta = 0.8 std GAP is a sum of 4000 sharp bumps that a
            64-128-128-1 network cannot represent, so the learned surrogate is
            trained and evaluated on the smooth one

SF set (used by all synthetic models): 20 type-1 radial functions with alpha
log-spaced 0.003..2.0 A^-2, cutoff 6 A; 12 angular functions = zeta {1,2,4}
x lambda {+1 (type 2), -1 (type 4)} x alpha {0.003, 0.03}, cutoff 6 A.  The
reference writes every SF twice (unweighted, then weighted by the atomic
number), so D = 2 * 32 = 64.  theta_d = scale * std_d(MM): the length scales
track the descriptor spread, as trained models' do.
"""
import numpy as np

RCUT = 6.0


def sf_table():
    """(type, alpha, cutoff, zeta) arrays of the 32-function SF set."""
    ty, al, rc, ze = [], [], [], []
    for a in np.geomspace(0.003, 2.0, 20):
        ty.append(1), al.append(float(a)), rc.append(RCUT), ze.append(1.0)
    for zeta in (1.0, 2.0, 4.0):
        for t in (2, 4):
            for a in (0.003, 0.03):
                ty.append(t), al.append(a), rc.append(RCUT), ze.append(zeta)
    return (np.array(ty, np.int32), np.array(al), np.array(rc), np.array(ze))


def _diamond_basis():
    fcc = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
    return np.concatenate([fcc, fcc + 0.25])


def _fcc_basis():
    return np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])


def _supercell(basis, a, reps):
    n1, n2, n3 = reps
    g = np.stack(np.meshgrid(np.arange(n1), np.arange(n2), np.arange(n3), indexing="ij"), -1)
    frac = (g.reshape(-1, 1, 3) + basis[None]).reshape(-1, 3)
    lat = np.diag([a * n1, a * n2, a * n3]).astype(np.float64)
    return lat, frac / np.array(reps) @ lat


def si64(seed=0, jitter=0.05):
    rng = np.random.default_rng(seed)
    lat, pos = _supercell(_diamond_basis(), 5.43, (2, 2, 2))
    pos = pos + rng.normal(0.0, jitter, pos.shape)
    return lat, pos, np.full(len(pos), 14, np.int32)


def alloy512(seed=0, jitter=0.08):
    rng = np.random.default_rng(seed)
    lat, pos = _supercell(_fcc_basis(), 3.9, (4, 4, 8))
    n = len(pos)
    counts = [int(round(0.5 * n)), int(round(0.3 * n))]
    counts.append(n - sum(counts))
    z = np.repeat(np.array([13, 28, 40], np.int32), counts)
    rng.shuffle(z)
    pos = pos + rng.normal(0.0, jitter, pos.shape)
    return lat, pos, z


def sige(seed=0, reps=16, jitter=0.1):
    rng = np.random.default_rng(seed)
    lat, pos = _supercell(_diamond_basis(), 5.54, (reps, reps, reps))
    n = len(pos)
    z = np.repeat(np.array([14, 32], np.int32), [n // 2, n - n // 2])
    rng.shuffle(z)
    pos = pos + rng.normal(0.0, jitter, pos.shape)
    return lat, pos, z


def _triclinic(rng, volume):
    """Random cell with angles in 60..120 deg and a valid metric."""
    while True:
        al, be, ga = np.radians(rng.uniform(60, 120, 3))
        ca, cb, cg = np.cos([al, be, ga])
        m = 1 - ca * ca - cb * cb - cg * cg + 2 * ca * cb * cg
        if m <= 0.05:
            continue
        ratios = rng.uniform(0.8, 1.25, 3)
        a, b, c = ratios
        v1 = np.array([a, 0, 0])
        v2 = np.array([b * cg, b * np.sin(ga), 0])
        cx = c * cb
        cy = c * (ca - cb * cg) / np.sin(ga)
        cz = np.sqrt(max(c * c - cx * cx - cy * cy, 1e-12))
        lat = np.array([v1, v2, [cx, cy, cz]])
        s = (volume / abs(np.linalg.det(lat))) ** (1 / 3)
        return lat * s


def _min_image_dist(lat, frac_new, frac_old):
    d = frac_old - frac_new
    d -= np.round(d)
    shifts = np.stack(np.meshgrid([-1, 0, 1], [-1, 0, 1], [-1, 0, 1], indexing="ij"), -1).reshape(-1, 3)
    cart = (d[:, None, :] + shifts[None]) @ lat
    return np.sqrt((cart ** 2).sum(-1)).min() if len(d) else np.inf


def random_structure(rng, n=None, species_pool=(3, 8, 14, 26), dmin=1.6, max_tries=200):
    """One population member (random sequential addition with rejection)."""
    if n is None:
        n = int(rng.integers(8, 257))
    nsp = int(rng.integers(1, 5))
    elems = rng.choice(np.array(species_pool, np.int32), nsp, replace=False)
    while True:
        lat = _triclinic(rng, n * rng.uniform(12, 20))
        # the shortest lattice translation must also respect dmin (self images)
        shifts = np.stack(np.meshgrid([-1, 0, 1], [-1, 0, 1], [-1, 0, 1], indexing="ij"),
                          -1).reshape(-1, 3)
        shifts = shifts[np.abs(shifts).sum(1) > 0]
        if np.sqrt(((shifts @ lat) ** 2).sum(1)).min() < dmin:
            continue
        frac = np.zeros((0, 3))
        ok = True
        for _ in range(n):
            for _t in range(max_tries):
                f = rng.random(3)
                if _min_image_dist(lat, f, frac) >= dmin:
                    frac = np.vstack([frac, f])
                    break
            else:
                ok = False
                break
        if ok:
            z = elems[rng.integers(0, nsp, n)].astype(np.int32)
            return lat, frac @ lat, z


def population(count, seed=0, nmin=8, nmax=256):
    """(atom_off, species, lat[S,3,3], pos[N,3]) of a packed population."""
    rng = np.random.default_rng(seed)
    lats, poss, zs, off = [], [], [], [0]
    for _ in range(count):
        lat, pos, z = random_structure(rng, int(rng.integers(nmin, nmax + 1)))
        lats.append(lat), poss.append(pos), zs.append(z)
        off.append(off[-1] + len(pos))
    return (np.array(off, np.int32), np.concatenate(zs), np.stack(lats), np.concatenate(poss))


def pack(structs):
    """Pack [(lat, pos, z), ...] into (atom_off, species, lat[S,3,3], pos[N,3])."""
    off = np.cumsum([0] + [len(p) for _, p, _ in structs]).astype(np.int32)
    return (off, np.concatenate([z for _, _, z in structs]).astype(np.int32),
            np.stack([l for l, _, _ in structs]), np.concatenate([p for _, p, _ in structs]))


def model_arrays(descriptors, M, theta_scale=1.0, coeff_std=1e-3, seed=0):
    """theta, MM, coeff of a synthetic sparse GPR.

    descriptors: (n, D) array of atomic descriptors to draw M sparse points
    from (without replacement); theta_d = theta_scale * std_d(MM) (1 where the
    spread is zero); coeff ~ N(0, coeff_std^2)."""
    rng = np.random.default_rng(seed)
    X = np.asarray(descriptors, np.float64)
    idx = rng.choice(len(X), size=M, replace=len(X) < M)
    mm = X[idx].copy()
    sd = mm.std(axis=0)
    theta = np.where(sd > 0, theta_scale * sd, 1.0)
    coeff = rng.normal(0.0, coeff_std, M)
    return theta, mm, coeff


def species_table(zs):
    """Atomic-number weights (the wACSF weights of the synthetic models)."""
    z = np.array(sorted(set(int(v) for v in zs)), np.int32)
    return z, z.astype(np.float64)


def alloy_model(M=4000, theta_scale=0.8, coeff_std=1e-3, seed=0, ncells=8):
    """Arrays (species_z, species_w, sf_type, sf_alpha, sf_cutoff, sf_zeta,
    theta, mm, coeff) of the synthetic ternary-alloy GAP: its sparse points
    are descriptors of `ncells` seeded alloy512 cells computed by the library
    itself (needs the GPU)."""
    from . import GapModel
    ty, al, rc, ze = sf_table()
    zt = np.array([13, 28, 40], np.int32)
    wt = zt.astype(np.float64)
    D = 2 * len(ty)
    probe = GapModel.create(zt, wt, ty, al, rc, np.ones(D), np.zeros((1, D)), np.zeros(1),
                            sf_zeta=ze)
    off, sp, lat, pos = pack([alloy512(seed=s) for s in range(ncells)])
    X = probe.descriptors(off, sp, lat, pos)
    probe.close()
    theta, mm, coeff = model_arrays(X, M, theta_scale=theta_scale, coeff_std=coeff_std, seed=seed)
    return zt, wt, ty, al, rc, ze, theta, mm, coeff


def model_from_cells(cells, species_z, M, theta_scale=1.0, coeff_std=1e-3, seed=0):
    """Arrays of a synthetic GAP (atomic-number weights, the standard SF set)
    whose M sparse points are library descriptors of `cells` (needs the GPU)."""
    from . import GapModel
    ty, al, rc, ze = sf_table()
    zt = np.asarray(species_z, np.int32)
    wt = zt.astype(np.float64)
    D = 2 * len(ty)
    probe = GapModel.create(zt, wt, ty, al, rc, np.ones(D), np.zeros((1, D)), np.zeros(1),
                            sf_zeta=ze)
    off, sp, lat, pos = pack(cells)
    X = probe.descriptors(off, sp, lat, pos)
    probe.close()
    theta, mm, coeff = model_arrays(X, M, theta_scale=theta_scale, coeff_std=coeff_std, seed=seed)
    return zt, wt, ty, al, rc, ze, theta, mm, coeff
