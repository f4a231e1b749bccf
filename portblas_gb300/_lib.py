"""ctypes binding of libgbblas.so, generated from the C header.

The argument types of every entry point are read from ``include/gbblas.h``
so the Python mirror can never drift from the C ABI.  Loading fails loudly
when the library has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HEADER = os.path.join(ROOT, "include", "gbblas.h")
LIB_PATH = os.path.join(HERE, "lib", "libgbblas.so")

_TYPES = {
    "gbblas_handle_t": C.c_void_p,
    "gbblas_grouped_plan_t": C.c_void_p,
    "int64_t": C.c_int64,
    "int32_t": C.c_int32,
    "int": C.c_int,
    "char": C.c_char,
    "float": C.c_float,
    "double": C.c_double,
    "void": None,
    "uint64_t": C.c_uint64,
    "size_t": C.c_size_t,
    "gbblas_status_t": C.c_int,
    "const char*": C.c_char_p,
}


def _ctype(decl: str):
    decl = decl.strip()
    if decl in ("void", ""):
        return None
    # strip the parameter name
    m = re.match(r"^(.*?)([A-Za-z_][A-Za-z_0-9]*)$", decl)
    typ = m.group(1).strip() if m and m.group(1).strip() else decl
    if "*" in typ:
        return C.c_void_p
    typ = typ.replace("const ", "").strip()
    return _TYPES[typ]


def parse_header(path: str = HEADER) -> dict[str, tuple]:
    """Returns {name: (restype, [argtypes])} for every function in the header."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for m in re.finditer(r"([A-Za-z_][A-Za-z_0-9 \*]*?)\s*\b(gbblas_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        ret, name, args = m.group(1).strip(), m.group(2), m.group(3)
        if ret.startswith("typedef"):
            continue
        rt = C.c_char_p if ret.replace(" ", "") == "constchar*" else _TYPES.get(ret, C.c_int)
        argl = [] if args.strip() in ("", "void") else [_ctype(a) for a in args.split(",")]
        out[name] = (rt, argl)
    return out


_lib = None


def load(path: str = LIB_PATH):
    """Loads libgbblas.so and sets restype/argtypes from the header."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libgbblas.so is not built ({path}); run "
                           "`python -c 'import __graft_entry__ as g; g.build()'` first")
    L = C.CDLL(path)
    for name, (rt, args) in parse_header().items():
        fn = getattr(L, name)  # AttributeError = header/library mismatch
        fn.restype = rt
        fn.argtypes = args
    _lib = L
    return L
