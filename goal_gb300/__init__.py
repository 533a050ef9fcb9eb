"""GB300-native implementation of goal's element hot path and its primal/adjoint
solves. The compute path is libgoal_gb300.so (hand-written sm_103a CUDA behind
the C ABI of include/goal_gb300.h); this package loads it with ctypes and
mirrors goal's host classes on top of it (see goal_gb300.api).

There is no CPU fallback: importing the bindings raises if the library has not
been built (``python -c "import __graft_entry__ as g; g.build()"``).
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgoal_gb300.so")

_lib = None


def lib() -> ctypes.CDLL:
    """The loaded CUDA library; raises RuntimeError when it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA library first (goal_gb300.build.build())")
        from . import _abi
        _lib = _abi.bind(ctypes.CDLL(LIB_PATH))
    return _lib
