"""FA_CP convex QP interface (the reference's `fa_cp` package:
QP/FA_CP/python/fa_cp/__init__.py) over the CUDA library libfa_cp_gb300.so.

    from pdal_gb300.fa_cp import Model
"""
from . import FA_CP
from .model import Model

__all__ = ["Model", "FA_CP"]
