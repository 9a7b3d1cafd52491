"""Descriptor export: a working ``Wacsf`` (gappy/libgap/WACSF.py:14-52).

The reference's ``car2wacsf`` calls ``fcar2wacsf``, which its extension never
defines (WACSF.py:7, :51), so it raises NameError.  Here it returns the wACSF
descriptors of every atom, shape (N, D), computed on the GPU with the model
in ./gap_parameters (the layout of CAR2ACSF's XX transposed, as the
reference's ``xx.T``).
"""
import numpy as np

import gapgb
from .GAP import _atomic_num


class Wacsf(object):
    def __init__(self, nf=None, rcut=6.0, lgrad=True):
        self.nf = nf
        self.rcut = rcut
        self.lgrad = lgrad

    def get_elenum(self, x):
        return [_atomic_num[element] for element in x]

    def car2wacsf(self, lat, elements, pos):
        try:
            Elements = self.get_elenum(elements)
        except (KeyError, TypeError):
            Elements = elements
        pos = np.asarray(pos, np.float64).reshape(-1, 3)
        m = gapgb.GapModel.load("gap_parameters", rcut=self.rcut)
        try:
            xx = m.descriptors([0, pos.shape[0]], Elements, np.asarray(lat), pos)
        finally:
            m.close()
        if self.nf is not None:
            xx = xx[:, :self.nf]
        return xx
