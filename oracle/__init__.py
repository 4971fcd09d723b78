"""Test infrastructure: the CPU oracle for gap-affine BiWFA (see biwfa_oracle.h).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this package.
"""
