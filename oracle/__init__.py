"""CPU FP64 oracle for the CALYPSO-GAP energy/force/stress path.

Test infrastructure: imported only by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference leg of bench.py, as the reference for parity.  The product
library never imports it.
"""
