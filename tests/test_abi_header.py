"""The ctypes signatures of the Python binding against the prototypes of include/edgpu.h
(parsed here, no compiler and no GPU): every declared entry point has a signature with the
same number of arguments, the same scalar types in the same positions and a pointer wherever
the header has one; so argument-order drift between the header and the binding fails here."""

import ctypes as C
import os
import re

import pytest

from impuritymodel_gb300 import _lib as L

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "edgpu.h")

SCALARS = {
    "int": C.c_int,
    "int64_t": C.c_int64,
    "size_t": C.c_size_t,
    "double": C.c_double,
    "uint32_t": C.c_uint32,
    "uint64_t": C.c_uint64,
    "float": C.c_float,
    "long long": C.c_longlong,
}


def _prototypes():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    out = {}
    for m in re.finditer(r"^([A-Za-z_][\w \t\*]*?)\b(edgpu_\w+)\s*\(([^;{]*?)\)\s*;", text, flags=re.M):
        ret, name, args = m.group(1).strip(), m.group(2), m.group(3).strip()
        if ret.startswith("typedef") or "(" in args:
            continue
        params = [] if args in ("", "void") else [a.strip() for a in args.split(",")]
        out[name] = (ret, params)
    return out


def _kind(decl):
    """('ptr', None) for a pointer parameter, ('scalar', ctype) otherwise."""
    d = re.sub(r"\b(const|volatile)\b", " ", decl)
    if "*" in d or "[" in d:
        return "ptr", None
    toks = d.split()
    base = toks[0] if len(toks) == 1 else " ".join(toks[:-1])
    return "scalar", SCALARS[base]


def _is_pointer_ctype(t):
    return t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer))


def _floating(t):
    return t in (C.c_float, C.c_double)


PROTOS = _prototypes()


def test_header_parses_every_exported_signature():
    assert len(PROTOS) >= 40
    assert set(PROTOS) == set(L.SIGNATURES), (set(PROTOS) ^ set(L.SIGNATURES))


@pytest.mark.parametrize("name", sorted(PROTOS))
def test_binding_matches_prototype(name):
    ret, params = PROTOS[name]
    res, args = L.SIGNATURES[name]
    assert len(args) == len(params), (name, len(args), len(params))
    for i, (decl, t) in enumerate(zip(params, args)):
        kind, ctype = _kind(decl)
        if kind == "ptr":
            assert _is_pointer_ctype(t), (name, i, decl, t)
        else:
            assert C.sizeof(t) == C.sizeof(ctype) and _floating(t) == _floating(ctype), (name, i, decl, t)
    rk, rt = _kind(ret + " r") if ret != "void" else ("void", None)
    if rk == "ptr":
        assert _is_pointer_ctype(res), (name, ret, res)
    elif rk == "scalar":
        assert C.sizeof(res) == C.sizeof(rt) and _floating(res) == _floating(rt), (name, ret, res)
