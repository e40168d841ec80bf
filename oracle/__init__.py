"""CPU oracle of the FluidSim hot path — test infrastructure only.

Nothing in the product imports this package; tests, smoke() and bench.py's
CPU-baseline leg use it as the checker.
"""
