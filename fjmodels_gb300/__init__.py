"""fjmodels_gb300: the fJmodels density / moment evaluation path on GB300 (sm_103a).

The compute lives in libfjgpu.so (hand-written CUDA behind the C ABI of
include/fjgpu.h); this package holds its ctypes bindings and a host-side mirror
of the reference's calls.  There is no CPU fallback.
"""
from . import _abi
from .api import (OUT_TABLES, XPT11, XW11, Anderson, Context, DFParams, FJError, Rule, Surrogate, composeName, gauleg,
                  guess_rhl, log_grid, readOut, readParam, tabulate_delta, tanh_sinh01, tanh_sinh_rule, writeOut)

__all__ = ["Context", "DFParams", "Rule", "Surrogate", "Anderson", "FJError", "XPT11", "XW11", "log_grid", "gauleg", "guess_rhl",
           "tabulate_delta", "writeOut", "readOut", "OUT_TABLES", "composeName", "readParam", "tanh_sinh_rule", "tanh_sinh01",
           "load_library"]


def load_library():
    return _abi.load()
