"""Minimum-bond utility: drop-in for gappy/libgap/BOND.py:14-52 (FGET_BOND)."""
try:
    from libgap.libgap import fget_bond
except ImportError:
    from .libgap import fget_bond
from .GAP import _atomic_num


class Bond(object):
    def __init__(self, nf=None, rcut=6.0, lgrad=True):
        self.nf = nf
        self.rcut = rcut
        self.lgrad = lgrad

    def get_elenum(self, x):
        return [_atomic_num[element] for element in x]

    def get_min_bond(self, lat, elements, pos):
        try:
            Elements = self.get_elenum(elements)
        except (KeyError, TypeError):
            Elements = elements
        return fget_bond(lat, Elements, pos, self.rcut)
