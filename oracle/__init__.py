"""CPU oracle of the reference's coupled LBM-MPM timestep (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this package, and only as the checker or the timed CPU baseline.
"""
