"""GB300-native FastS structured solve step.

Python layer mirroring FastS / FastC (fasts.py, fastc.py, pytree.py) over the
C ABI of libfastgb300.so (include/fast_gb300.h), whose hand-written sm_103a
kernels do all the numerical work.
"""
from . import fastc, fasts, pytree  # noqa: F401

__all__ = ["fastc", "fasts", "pytree"]
