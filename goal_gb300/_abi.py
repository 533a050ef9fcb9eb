"""ctypes prototypes generated from include/goal_gb300.h (the header is the single
source of truth for the C ABI)."""
import ctypes
import os
import re

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "goal_gb300.h")


class Chain(ctypes.Structure):
    """goal_chain"""
    _fields_ = [("mode", ctypes.c_int), ("jacobian", ctypes.c_int), ("save_states", ctypes.c_int),
                ("qoi", ctypes.c_int), ("rho", ctypes.c_double), ("error_chain", ctypes.c_int),
                ("overwrite", ctypes.c_int), ("colored", ctypes.c_int)]


class SolveParams(ctypes.Structure):
    """goal_solve_params"""
    _fields_ = [("krylov_size", ctypes.c_int), ("max_iters", ctypes.c_int), ("tolerance", ctypes.c_double),
                ("precision", ctypes.c_int), ("inner_iters", ctypes.c_int), ("precond", ctypes.c_int),
                ("learned_cap", ctypes.c_int)]


class SolveStats(ctypes.Structure):
    """goal_solve_stats"""
    _fields_ = [("iters", ctypes.c_int), ("inner_iters", ctypes.c_int), ("converged", ctypes.c_int),
                ("fell_back", ctypes.c_int), ("rel_res", ctypes.c_double), ("seconds", ctypes.c_double),
                ("spmv64", ctypes.c_longlong), ("spmv32", ctypes.c_longlong)]


class NewtonStats(ctypes.Structure):
    """goal_newton_stats"""
    _fields_ = [("iters", ctypes.c_int), ("converged", ctypes.c_int), ("linear_iters", ctypes.c_int),
                ("inner_iters", ctypes.c_int), ("norms", ctypes.c_double * 32),
                ("seconds_assembly", ctypes.c_double), ("seconds_solve", ctypes.c_double),
                ("backtracks", ctypes.c_int)]


class DwrResult(ctypes.Structure):
    """goal_dwr_result"""
    _fields_ = [("eta", ctypes.c_double), ("bound", ctypes.c_double), ("qoi", ctypes.c_double),
                ("solve", SolveStats), ("seconds_adjoint", ctypes.c_double), ("seconds_solve", ctypes.c_double),
                ("seconds_localize", ctypes.c_double)]


def parse_header(path: str = HEADER):
    """Returns {name: (return type, [argument types])} for every function declared."""
    with open(path) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"#[^\n]*", "", text)
    text = re.sub(r"typedef struct \{.*?\}\s*\w+;", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(goal_\w+)\s*\(([^)]*)\)\s*;", text):
        ret, name, args = m.group(1).strip(), m.group(2), m.group(3).strip()
        arglist = [] if args in ("", "void") else [a.strip() for a in args.split(",")]
        out[name] = (ret, arglist)
    return out


def _ctype(decl: str):
    decl = decl.strip()
    if "char" in decl and "*" in decl:
        return ctypes.c_char_p
    if "*" in decl:
        return ctypes.c_void_p
    base = decl.rsplit(" ", 1)[0] if " " in decl else decl
    base = base.replace("const", "").strip()
    if base == "int":
        return ctypes.c_int
    if base == "long long":
        return ctypes.c_longlong
    if base == "double":
        return ctypes.c_double
    if base == "float":
        return ctypes.c_float
    if base.startswith("goal_"):
        return ctypes.c_void_p  # opaque handle
    if base == "void":
        return None
    raise ValueError(f"unmapped C type: {decl}")


def bind(L: ctypes.CDLL) -> ctypes.CDLL:
    for name, (ret, args) in parse_header().items():
        fn = getattr(L, name)
        fn.restype = _ctype(ret + " x") if ret != "void" else None
        fn.argtypes = [_ctype(a) for a in args]
    return L
