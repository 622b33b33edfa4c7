"""cppimpact_gb300: GB300-native explicit tet4/tet10 impact step behind the cppimpact interface.

The compute path is ``libcppimpact_gb300.so`` (hand-written sm_103a CUDA, C ABI in
``include/cppimpact_gb300.h``); this package holds its build script, the ctypes mirror
of the reference classes (``api``) and the synthetic mesh generator (``meshgen``).
"""
from . import meshgen  # noqa: F401

__all__ = ["meshgen", "api", "build"]
