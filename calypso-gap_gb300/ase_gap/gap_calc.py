"""
ASE calculator ``GAP``: drop-in for gappy/ASE/gap_calc.py:19-52.

Like the reference it builds a ``libgap.GAP.Calculator`` on every
``calculate`` (the device model is cached by libgap.libgap, so the GPU upload
happens once), always asks for gradients, and stores energy, free_energy,
forces (eV/A), stress (GPa, order XX YY ZZ XY YZ ZX - the reference's units
and order, which gappy/ASE/logger.py relies on) and variance.

Copy this file into ``ase/calculators/`` as the reference's README says, or
import it from here.  When ASE is not installed a minimal stand-in base
class keeps the same ``calculate``/``results`` protocol.
"""
from __future__ import division

import numpy as np

try:
    from ase.calculators.calculator import Calculator, all_changes
except ImportError:  # ASE absent: same protocol, no ASE machinery
    all_changes = ["positions", "numbers", "cell", "pbc"]

    class Calculator(object):
        implemented_properties = []

        def __init__(self, **kwargs):
            self.atoms = None
            self.results = {}
            self.parameters = dict(kwargs)

        def calculate(self, atoms=None, properties=["energy"], system_changes=all_changes):
            if atoms is not None:
                self.atoms = atoms.copy() if hasattr(atoms, "copy") else atoms

        def get_property(self, name, atoms=None):
            self.calculate(atoms, [name])
            return self.results[name]

        def get_potential_energy(self, atoms=None, force_consistent=False):
            return self.get_property("energy", atoms)

        def get_forces(self, atoms=None):
            return self.get_property("forces", atoms)

        def get_stress(self, atoms=None):
            return self.get_property("stress", atoms)

import libgap.GAP as my_gap


class GAP(Calculator):
    implemented_properties = ['energy', 'forces', 'stress']

    nolabel = True

    def __init__(self, rcut=6.0):
        Calculator.__init__(self)
        self.rcut = rcut

    def calculate(self, atoms=None, properties=['energy'], system_changes=all_changes):
        Calculator.calculate(self, atoms, properties, system_changes)

        gap_calc = my_gap.Calculator(rcut=self.rcut)
        species = self.atoms.get_atomic_numbers()
        lat = np.asarray(self.atoms.cell)
        pos = self.atoms.positions
        lgrad = True
        energy, forces, stress, variance = gap_calc.gap_calc(species, lat, pos, lgrad)

        self.results['energy'] = energy
        self.results['free_energy'] = energy
        self.results['forces'] = forces
        self.results['stress'] = stress
        self.results['variance'] = variance
