"""The ctypes argument and result types that dips_gb300/_lib.py gives every entry point agree
with the prototypes of include/dips.h: the same number of arguments, and at each position the
same kind (pointer, or an integer / floating type of the same size and signedness).  ctypes does
not check a call against the C prototype, so a missing or shifted argument would pass garbage
across the boundary without an error.  No GPU and no compiler needed: the header is parsed."""

import ctypes
import os
import re

import pytest

from dips_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_SCALARS = {
    "int": ("int", 4, True), "int32_t": ("int", 4, True), "uint32_t": ("int", 4, False),
    "int64_t": ("int", 8, True), "uint64_t": ("int", 8, False), "size_t": ("int", 8, False),
    "float": ("float", 4, True), "double": ("float", 8, True),
}


def _header_text():
    text = open(os.path.join(ROOT, "include", "dips.h")).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    return "\n".join(line for line in text.splitlines() if not line.lstrip().startswith("#"))


def _split_top(args):
    out, depth, cur = [], 0, ""
    for ch in args:
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
            continue
        depth += ch == "("
        depth -= ch == ")"
        cur += ch
    if cur.strip():
        out.append(cur)
    return [a.strip() for a in out]


def _c_kind(decl, pointer_typedefs):
    """Kind of one C parameter (or result) declaration."""
    if "*" in decl or "[" in decl or "(" in decl:
        return ("ptr",)
    words = [w for w in re.findall(r"\w+", decl) if w not in ("const", "struct", "unsigned", "signed")]
    if not words:
        return None
    if words[0] == "void" and len(words) == 1:
        return None
    if words[0] in pointer_typedefs or words[0] == "cudaStream_t":
        return ("ptr",)
    if words[0] in _SCALARS:
        return _SCALARS[words[0]]
    raise AssertionError(f"unclassified C type in {decl!r}")


def _ct_kind(t):
    """Kind of one ctypes type."""
    if t is None:
        return None
    if t in (ctypes.c_void_p, ctypes.c_char_p) or issubclass(t, (ctypes._Pointer, ctypes._CFuncPtr)):
        return ("ptr",)
    if t in (ctypes.c_float, ctypes.c_double):
        return ("float", ctypes.sizeof(t), True)
    return ("int", ctypes.sizeof(t), t(-1).value < 0)


def header_prototypes():
    text = _header_text()
    pointer_typedefs = set(re.findall(r"typedef[^;]*?\(\s*\*\s*(\w+)\s*\)", text))
    protos = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(dips_\w+)\s*\((.*?)\)\s*;", text, flags=re.S):
        ret, name, args = m.group(1), m.group(2), m.group(3)
        if "typedef" in ret:
            continue
        params = [] if args.strip() in ("", "void") else _split_top(args)
        protos[name] = (_c_kind(ret.strip(), pointer_typedefs), [_c_kind(p, pointer_typedefs) for p in params])
    return protos


PROTOS = header_prototypes()


def test_every_declared_entry_point_has_a_ctypes_signature():
    assert len(PROTOS) >= 40, sorted(PROTOS)
    missing = sorted(set(PROTOS) - set(_lib._SIGS))
    extra = sorted(set(_lib._SIGS) - set(PROTOS))
    assert not missing, f"declared in dips.h without a ctypes signature: {missing}"
    assert not extra, f"ctypes signatures for names dips.h does not declare: {extra}"


@pytest.mark.parametrize("name", sorted(PROTOS))
def test_ctypes_signature_matches_the_prototype(name):
    c_ret, c_args = PROTOS[name]
    res, args = _lib._SIGS[name]
    assert len(args) == len(c_args), f"{name}: {len(args)} ctypes arguments, {len(c_args)} in dips.h"
    for i, (ct, ck) in enumerate(zip(args, c_args)):
        assert _ct_kind(ct) == ck, f"{name} argument {i}: ctypes {ct} vs C {ck}"
    # an int status may be declared as c_int32 or c_int; const char* results as c_char_p
    assert _ct_kind(res) == c_ret, f"{name} result: ctypes {res} vs C {c_ret}"


def test_the_parser_sees_a_function_pointer_parameter_and_array_parameters():
    assert PROTOS["dips_xla_set_status_fn"] == (None, [("ptr",)])
    ret, args = PROTOS["dips_geometry_assemble_scratch_bytes"]
    assert ret == ("int", 8, False) and args == [("int", 8, True)]
    # const float h[3] is a pointer
    assert ("ptr",) in PROTOS["dips_geometry_classify"][1]
