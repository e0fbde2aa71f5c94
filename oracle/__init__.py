"""CPU oracle of the Langevin hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package; the product library never does.
"""
