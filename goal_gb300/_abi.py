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
                ("overwrite", ctypes.c_int)]


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
