"""GAP calculator: drop-in for gappy/libgap/GAP.py:14-61.

``Calculator(rcut=6.0)`` reads the model (``gap_read``) and ``gap_calc``
returns ``(ene, force, stress, variance)`` with energy in eV, forces (N, 3)
in eV/A, stress (6,) in GPa ordered XX YY ZZ XY YZ ZX, and variance 0.
"""
import numpy as np

try:
    from libgap.libgap import fgap_read, fgap_calc
except ImportError:  # package imported under another name
    from .libgap import fgap_read, fgap_calc

ChemicalSymbols = ['X', 'H', 'He', 'Li', 'Be', 'B', 'C', 'N', 'O', 'F',
                   'Ne', 'Na', 'Mg', 'Al', 'Si', 'P', 'S', 'Cl', 'Ar', 'K',
                   'Ca', 'Sc', 'Ti', 'V', 'Cr', 'Mn', 'Fe', 'Co', 'Ni', 'Cu',
                   'Zn', 'Ga', 'Ge', 'As', 'Se', 'Br', 'Kr', 'Rb', 'Sr', 'Y',
                   'Zr', 'Nb', 'Mo', 'Tc', 'Ru', 'Rh', 'Pd', 'Ag', 'Cd', 'In',
                   'Sn', 'Sb', 'Te', 'I', 'Xe', 'Cs', 'Ba', 'La', 'Ce', 'Pr',
                   'Nd', 'Pm', 'Sm', 'Eu', 'Gd', 'Tb', 'Dy', 'Ho', 'Er', 'Tm',
                   'Yb', 'Lu', 'Hf', 'Ta', 'W', 'Re', 'Os', 'Ir', 'Pt', 'Au',
                   'Hg', 'Tl', 'Pb', 'Bi', 'Po', 'At', 'Rn', 'Fr', 'Ra', 'Ac',
                   'Th', 'Pa', 'U', 'Np', 'Pu', 'Am', 'Cm', 'Bk', 'Cf', 'Es',
                   'Fm', 'Md', 'No', 'Lr']
_atomic_num = {s: i for i, s in enumerate(ChemicalSymbols)}


class Calculator(object):
    def __init__(self, rcut=6.0):
        self.gap_read()
        self.rcut = rcut

    def get_elenum(self, x):
        return [_atomic_num[element] for element in x]

    def gap_read(self):
        (self.nsparseX, self.des_len, self.theta, self.mm, self.invcmm,
         self.coeff) = fgap_read()

    def gap_calc(self, species, lat, pos, lgrad):
        try:
            Species = self.get_elenum(species)
        except (KeyError, TypeError):
            Species = species
        return fgap_calc(Species, lat, pos,
                         self.theta[0:self.des_len],
                         self.mm[0:self.nsparseX, 0:self.des_len],
                         self.invcmm[0:self.nsparseX, 0:self.nsparseX],
                         self.coeff[0:self.nsparseX],
                         self.rcut, lgrad)
