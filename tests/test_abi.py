"""CPU checks of the C ABI: the library loads and exports every declared symbol,
and the host side of the expression evaluator reproduces the reference's
known-answer test (no GPU work is done here)."""
import ctypes
import math
import os

import pytest

from goal_gb300 import _abi

LIB = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "goal_gb300", "libgoal_gb300.so")


def _lib():
    if not os.path.exists(LIB):
        pytest.skip("libgoal_gb300.so not built")
    import goal_gb300
    return goal_gb300.lib()


def test_header_parses():
    decls = _abi.parse_header()
    assert "goal_assemble" in decls and "goal_disc_create" in decls
    assert len(decls) >= 30


def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(LIB) if os.path.exists(LIB) else None
    if L is None:
        pytest.skip("libgoal_gb300.so not built")
    missing = [name for name in _abi.parse_header() if not hasattr(L, name)]
    assert not missing, f"not exported: {missing}"


def test_every_prototype_binds():
    """ctypes prototypes for every declared function (no GPU work)."""
    L = _lib()
    for name in _abi.parse_header():
        assert getattr(L, name).argtypes is not None


def test_expression_kat_host():
    """test/control.cpp:12-15: sin(x)*cos(y) + 2*exp(t) - z at (1,2,3,4) within 1e-15."""
    L = _lib()
    out = ctypes.c_double()
    assert L.goal_eval(b"sin(x)*cos(y) + 2*exp(t) - z", 1.0, 2.0, 3.0, 4.0, ctypes.byref(out)) == 0
    v2 = math.sin(1.0) * math.cos(2.0) + 2.0 * math.exp(4.0) - 3.0
    assert abs(out.value - v2) < 1e-15


@pytest.mark.parametrize("expr,val", [("0.01*t", 0.03), ("-(2^3)+x", -7.0), ("pow(2,10)/y", 512.0),
                                      ("1.0e-3*sin(pi*x)", 1.0e-3 * math.sin(math.pi)), ("0.0", 0.0)])
def test_expressions(expr, val):
    L = _lib()
    out = ctypes.c_double()
    assert L.goal_eval(expr.encode(), 1.0, 2.0, 3.0, 3.0, ctypes.byref(out)) == 0
    assert abs(out.value - val) < 1e-15


def test_expression_errors_are_reported():
    L = _lib()
    out = ctypes.c_double()
    rc = L.goal_eval(b"sin(x", 0.0, 0.0, 0.0, 0.0, ctypes.byref(out))
    assert rc == 1
    assert b"missing" in L.goal_last_error()
    assert L.goal_eval(b"foo(x)", 0.0, 0.0, 0.0, 0.0, ctypes.byref(out)) == 1
