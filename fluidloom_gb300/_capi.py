"""ctypes binding of the C ABI declared in include/fluidloom_gb300.h.

The header is the single source of truth: its declarations are parsed here and
every entry point gets its argtypes/restype from it.  The library must be
built (fluidloom_gb300.build); there is no fallback implementation.
"""
import ctypes
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
HEADER = os.path.join(ROOT, "include", "fluidloom_gb300.h")
LIB_PATH = os.path.join(PKG, "_lib", "libfluidloom_gb300.so")

_SCALARS = {
    "int": ctypes.c_int, "int32_t": ctypes.c_int32, "uint32_t": ctypes.c_uint32,
    "int64_t": ctypes.c_int64, "uint64_t": ctypes.c_uint64, "uint8_t": ctypes.c_uint8,
    "uint16_t": ctypes.c_uint16, "size_t": ctypes.c_size_t, "float": ctypes.c_float,
    "double": ctypes.c_double, "void": None,
}


def _ctype(t):
    t = t.replace("const", " ").strip()
    t = re.sub(r"\s+", " ", t)
    stars = t.count("*")
    base = t.replace("*", "").strip()
    if stars == 0:
        return _SCALARS[base]
    if base == "char" and stars == 1:
        return ctypes.c_char_p
    return ctypes.c_void_p


def parse_header(path=HEADER):
    """Return {name: (restype, [argtypes])} for every function declared."""
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    src = re.sub(r"//[^\n]*", " ", src)
    src = re.sub(r"#[^\n]*", " ", src)
    src = re.sub(r"typedef struct[^;]*?\{.*?\}\s*\w+\s*;", " ", src, flags=re.S)
    src = re.sub(r"typedef[^;]*;", " ", src)
    decls = {}
    for m in re.finditer(r"([\w\s\*]+?)\b(fl_\w+)\s*\(([^)]*)\)\s*;", src):
        ret, name, args = m.group(1).strip(), m.group(2), m.group(3).strip()
        argtypes = []
        if args and args != "void":
            for a in args.split(","):
                a = a.strip()
                mm = re.match(r"(.*?)(\w+)$", a)
                argtypes.append(_ctype(mm.group(1)))
        decls[name] = (_ctype(ret), argtypes)
    return decls


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("fluidloom_gb300 CUDA library is not built (%s); run "
                               "fluidloom_gb300.build.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in parse_header().items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib
