"""muxi_spmv_gb300 -- SpMV for one GB300 (sm_103a) behind the muxi_spmv API.

The compute lives in libmuxispmv.so (hand-written CUDA for sm_103a, C ABI in
include/muxi_spmv.h).  This package holds its build recipe, a ctypes binding,
a Python mirror of the reference interface (api.py) and the named synthetic
workloads (workloads.py).
"""
from ._lib import SpmvError, lib, last_error  # noqa: F401
from .api import *  # noqa: F401,F403
from . import workloads  # noqa: F401
