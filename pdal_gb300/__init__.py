"""GB300-native restarted reflected-Halpern primal-dual LP/QP solver.

The compute path is hand-written CUDA for sm_103a in pdal_gb300/csrc, exported
as C entry points that keep the CP_AL / FA_CP interfaces (include/*.h).  The
Python modules here are thin ctypes front ends; there is no CPU fallback.
"""
__all__ = ["lp", "instances", "build"]
