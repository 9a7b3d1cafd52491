"""ASE calculator for the GB300 GAP evaluator (drop-in for gappy/ASE)."""
