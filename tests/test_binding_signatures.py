"""CPU checks that both host bindings agree with the C header, argument by argument.

The header (include/tenet_gb300.h) is the one source of truth for the boundary.  The
Python ctypes table (tenetgb/_lib.py) and the Julia binding
(tenet.jl_gb300/julia/TenetGB300.jl, which cannot run here: no Julia toolchain) each
restate every signature they use; a wrong arity or a 32/64-bit mix-up there corrupts
the call without any error.  These tests parse the header and both bindings and compare
return types, arities and every argument's type class."""

import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tenet_gb300.h")
JULIA = os.path.join(ROOT, "tenet.jl_gb300", "julia", "TenetGB300.jl")

# C scalar types by class
INT32 = {"int32_t", "int", "tn_dtype_t", "tn_precision_t", "tn_status_t"}
INT64 = {"int64_t"}
UINT64 = {"uint64_t", "size_t"}
DOUBLE = {"double"}
FLOAT = {"float"}
CHAR = {"char"}


def parse_c_param(p):
    """'const void* const* h_sites' -> ('void', 2); 'int device' -> ('int', 0)."""
    p = p.replace("*", " * ")
    toks = [t for t in p.split() if t not in ("const", "struct")]
    stars = toks.count("*")
    words = [t for t in toks if t != "*"]
    assert words, p
    base = words[0]
    if base == "unsigned":  # 'unsigned long long' and friends are not used by the header
        raise AssertionError("unexpected unsigned type in " + p)
    return base, stars


def header_decls():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    txt = "\n".join(line for line in txt.splitlines() if not line.lstrip().startswith("#"))
    decls = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(tn_\w+)\s*\(([^;{}]*?)\)\s*;", txt, flags=re.S):
        ret, name, params = " ".join(m.group(1).split()), m.group(2), " ".join(m.group(3).split())
        if ret.startswith("typedef"):
            continue
        plist = [] if params in ("", "void") else [parse_c_param(p) for p in params.split(",")]
        decls[name] = (parse_c_param(ret + " x")[0] + "*" * ret.count("*"), plist)
    return decls


@pytest.fixture(scope="module")
def decls():
    d = header_decls()
    assert len(d) > 60
    return d


# ---------------------------------------------------------------------------------- Python

def ctypes_ok(ct, base, stars):
    from tenetgb import _lib

    if stars == 0:
        if base in INT32:
            return ct in (C.c_int32, C.c_int)
        if base in INT64:
            return ct is C.c_int64
        if base in UINT64:
            return ct in (C.c_uint64, C.c_size_t)
        if base in DOUBLE:
            return ct is C.c_double
        if base in FLOAT:
            return ct is C.c_float
        if base in CHAR:
            return ct is C.c_char
        return False
    if ct is C.c_void_p:
        return True
    if stars == 1 and base in CHAR:
        return ct is C.c_char_p
    if stars == 1:
        target = getattr(ct, "_type_", None)
        if target is None:
            return False
        if base == "tn_tensor":
            return target is _lib.tn_tensor
        if base == "tn_query":
            return target is _lib.tn_query
        return ctypes_ok(target, base, 0)
    if stars == 2:
        return getattr(ct, "_type_", None) is C.c_void_p
    return False


def test_python_table_matches_header(decls):
    from tenetgb import _lib

    bad = []
    for name, (ret, args) in _lib.SIGNATURES.items():
        assert name in decls, name
        cret, cparams = decls[name]
        if len(args) != len(cparams):
            bad.append(f"{name}: {len(args)} ctypes args, header has {len(cparams)}")
            continue
        if cret == "tn_status_t" and ret not in (C.c_int32, C.c_int):
            bad.append(f"{name}: status return as {ret}")
        if cret in ("char*",) and ret is not C.c_char_p:
            bad.append(f"{name}: string return as {ret}")
        for i, (ct, (base, stars)) in enumerate(zip(args, cparams)):
            if not ctypes_ok(ct, base, stars):
                bad.append(f"{name} arg {i}: {ct} for {base}{'*' * stars}")
    assert not bad, "\n".join(bad)


# ----------------------------------------------------------------------------------- Julia

def split_top(s):
    """Split on commas outside (), {} and []."""
    out, depth, cur = [], 0, []
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    if "".join(cur).strip():
        out.append("".join(cur).strip())
    return out


def julia_ccalls():
    src = open(JULIA).read()
    src = "\n".join(re.sub(r"#.*$", "", line) for line in src.splitlines())
    calls = []
    for m in re.finditer(r"\bccall\(", src):
        i, depth = m.end(), 1
        while depth:
            depth += {"(": 1, ")": -1}.get(src[i], 0)
            i += 1
        parts = split_top(src[m.end(): i - 1])
        fn = re.match(r"\(:(tn_\w+),\s*libtenetgb\)", parts[0])
        assert fn, parts[0]
        assert parts[2].startswith("(") and parts[2].endswith(")"), parts[2]
        types = split_top(parts[2][1:-1])
        calls.append((fn.group(1), parts[1], types, parts[3:]))
    return calls


JL_SCALAR = {
    "int32": {"Int32", "Cint"},
    "int64": {"Int64", "Clonglong"},
    "uint64": {"UInt64", "Csize_t", "Culonglong"},
    "double": {"Float64", "Cdouble"},
    "float": {"Float32", "Cfloat"},
}
JL_ELEM = {"int32": "Int32", "int64": "Int64", "double": "Float64", "float": "Float32"}


def scalar_class(base):
    for cls, names in (("int32", INT32), ("int64", INT64), ("uint64", UINT64), ("double", DOUBLE),
                       ("float", FLOAT)):
        if base in names:
            return cls
    return None


def julia_ok(jt, base, stars):
    jt = jt.replace(" ", "")
    if stars == 0:
        cls = scalar_class(base)
        return cls is not None and jt in JL_SCALAR[cls]
    if stars == 1:
        if base in CHAR:
            return jt in ("Cstring", "Ptr{UInt8}", "Ptr{Cchar}")
        if jt == "Ptr{Cvoid}":
            return True
        if base == "tn_tensor":
            return jt in ("Ref{TnTensor}", "Ptr{TnTensor}")
        if base == "void":  # host data of any element type
            return re.fullmatch(r"Ptr\{\w+\}", jt) is not None
        cls = scalar_class(base)
        return cls in JL_ELEM and jt in (f"Ptr{{{JL_ELEM[cls]}}}", f"Ref{{{JL_ELEM[cls]}}}")
    if stars == 2:
        return re.fullmatch(r"(Ref|Ptr)\{Ptr\{\w+\}\}", jt) is not None
    return False


def test_julia_ccalls_match_header(decls):
    calls = julia_ccalls()
    assert len(calls) >= 30
    bad = []
    for name, ret, types, args in calls:
        if name not in decls:
            bad.append(f"{name}: not declared in the header")
            continue
        cret, cparams = decls[name]
        if len(types) != len(cparams):
            bad.append(f"{name}: {len(types)} Julia argument types, header has {len(cparams)}")
        if len(args) != len(types):
            bad.append(f"{name}: {len(args)} arguments for {len(types)} types")
        want_ret = {"tn_status_t": "Int32", "char*": "Cstring", "void*": "Ptr{Cvoid}"}.get(cret)
        if ret.strip() != want_ret:
            bad.append(f"{name}: returns {ret}, header {cret}")
        for i, (jt, (base, stars)) in enumerate(zip(types, cparams)):
            if not julia_ok(jt, base, stars):
                bad.append(f"{name} arg {i}: {jt} for {base}{'*' * stars}")
    assert not bad, "\n".join(bad)


def test_julia_binding_calls_only_declared_entry_points(decls):
    names = {c[0] for c in julia_ccalls()}
    for must in ("tn_contract", "tn_tensor_qr_thin", "tn_tensor_svd_thin", "tn_simple_update_absorb",
                 "tn_hadamard", "tn_permute", "tn_mps_evolve_mpo", "tn_mps_sample", "tn_mps_dmrg"):
        assert must in names, must
    assert names <= set(decls)


def test_parser_sees_a_known_declaration(decls):
    ret, params = decls["tn_mps_dmrg"]
    assert ret == "tn_status_t"
    assert params[1] == ("void", 2) and params[6] == ("int64_t", 0) and params[10] == ("double", 1)
