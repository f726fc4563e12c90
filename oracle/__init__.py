"""CPU oracle for the texture-synthesis hot loop (test infrastructure only).

Only tests/, __graft_entry__.smoke() (as the checker) and bench.py's CPU
baseline import this package; the product never does.
"""
