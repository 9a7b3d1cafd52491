"""
GAP calculator module (GB300 build)
===================================
Drop-in for gappy's ``libgap`` package (gappy/libgap/__init__.py): the same
modules and entry points, evaluated on one GPU by libgapgb.so.
Provides
  1. fgap_read / fgap_calc / fget_bond   (libgap.libgap, the f2py surface)
  2. GAP.Calculator                       (gap_read, gap_calc)
  3. BOND.Bond, WACSF.Wacsf
"""
from __future__ import absolute_import

__version__ = "0.1.0"
