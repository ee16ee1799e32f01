"""CPU oracle for the SAGESim per-tick agent step (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package; the engine never does.
"""
