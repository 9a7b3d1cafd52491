"""Shared helpers of the test suite: synthetic models written as
gap_parameters files so that the oracle and the CUDA library read the same
bytes."""
import os

import numpy as np


def write_model_file(path, species_z, species_w, sf_type, sf_alpha, sf_cutoff, theta, mm,
                     coeff, sf_zeta=None):
    """Write a gap_parameters file (the grammar of FGAP_READ, gap_calc.f90:303-364)."""
    with open(path, "w") as f:
        f.write("%d\n" % len(species_z))
        for z, w in zip(species_z, species_w):
            f.write("%6d %.17g\n" % (z, w))
        f.write("%d\n" % len(sf_type))
        for q, (t, a, c) in enumerate(zip(sf_type, sf_alpha, sf_cutoff)):
            if sf_zeta is not None and sf_zeta[q] != 1.0:
                f.write("%d %.17g %.17g %.17g\n" % (t, a, c, sf_zeta[q]))
            else:
                f.write("%d %.17g %.17g\n" % (t, a, c))
        M, D = mm.shape
        f.write("%d %d\n\n\n\n" % (M, D))
        f.write(" ".join("%.17g" % v for v in theta) + "\n")
        for row in mm:
            f.write(" ".join("%.17g" % v for v in row) + "\n")
        f.write(" ".join("%.17g" % v for v in coeff) + "\n")
    return path


def synth_model_file(path, oracle, structs, M, theta_scale=1.0, coeff_std=1e-3, seed=0,
                     sf=None, zeta=True):
    """A synthetic model whose sparse points are oracle descriptors of `structs`."""
    import gapgb.synth as S
    ty, al, rc, ze = sf if sf is not None else S.sf_table()
    if not zeta:
        ze = np.ones_like(ze)
    zs = np.concatenate([z for _, _, z in structs])
    sz, sw = S.species_table(zs)
    D = 2 * len(ty)
    # descriptors with a placeholder GPR (theta = 1, one sparse point)
    tmp = path + ".tmp"
    write_model_file(tmp, sz, sw, ty, al, rc, np.ones(D), np.zeros((1, D)), np.zeros(1), ze)
    om = oracle.Model(tmp)
    X = []
    for lat, pos, z in structs:
        cnt, nb = oracle.neighbors(lat, pos, om.weights(z), 6.0, max_nb=400)
        xx, _, _ = oracle.car2acsf(om, pos, cnt, nb)
        X.append(xx)
    os.remove(tmp)
    theta, mm, coeff = S.model_arrays(np.concatenate(X), M, theta_scale, coeff_std, seed)
    return write_model_file(path, sz, sw, ty, al, rc, theta, mm, coeff, ze)


def three_species_cell(seed):
    """2x2x2 fcc cell (a = 3.9 A) of Z 13/28/40, jittered."""
    rng = np.random.default_rng(seed)
    basis = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
    g = np.stack(np.meshgrid(np.arange(2), np.arange(2), np.arange(2), indexing="ij"), -1)
    frac = (g.reshape(-1, 1, 3) + basis[None]).reshape(-1, 3)
    lat = np.diag([7.8, 7.8, 7.8]) + rng.normal(0.0, 0.05, (3, 3))
    pos = (frac / 2.0) @ lat + rng.normal(0.0, 0.08, (len(frac), 3))
    z = np.array([13, 28, 40], np.int32)[rng.permutation(np.arange(len(frac)) % 3)]
    return lat, pos, z
