"""qpms_gb300: GB300-native implementation of the QPMS mode-problem hot path.

The compute path is the CUDA library libqpms_gb300.so (C-ABI, include/qpms_gb300.h);
this package is a thin Python mirror of the reference's Cython interface over it.
"""
from ._lib import QpmsGpuError, lib, last_error  # noqa: F401
from .translations import trans_calculator  # noqa: F401
from .scatsystem import ScatteringSystem  # noqa: F401,E402
