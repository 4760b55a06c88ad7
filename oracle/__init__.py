"""CPU oracle for the NaiveDynamics.jl hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
