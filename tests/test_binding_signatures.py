"""CPU checks that both host bindings call the C ABI with its declared prototypes.

The Julia binding (``julia/QrochetGPU.jl``) cannot run in this image (no Julia), so its ``ccall``
sites are parsed as text: every symbol it calls must be declared in ``include/qrochet_gpu.h``, the
return type and every argument type must match the prototype (by ABI class: int, double, long,
uint64, string, pointer to each of those, opaque handle, pointer to a handle), and each call must
pass exactly as many arguments as its type tuple lists.  The Python ctypes table
(``qrochet/_lib.py``) is checked against the same prototypes, and the status, precision, direction
and method constants of both bindings against the header's ``#define``s.  The gate matrices the
Julia binding builds are checked for the C ABI's row-major memory order by a NumPy restatement of
its column-major steps, and every call site for passing them on unchanged.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
JULIA = os.path.join(ROOT, "qrochet.jl_gb300", "julia", "QrochetGPU.jl")

_SCALAR = {"int": "int", "double": "double", "long": "long", "uint64_t": "u64", "unsigned": "u32"}
_OPAQUE = {"void", "qr_chain", "qr_mpo", "qr_server", "qr_batch"}


def _strip_c_comments(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def _c_class(param):
    """ABI class of one C parameter declaration (name optional)."""
    p = param.replace("const", " ").strip()
    stars = p.count("*")
    words = p.replace("*", " ").split()
    base = words[0]
    if stars == 0:
        assert base in _SCALAR, param
        return _SCALAR[base]
    if stars == 2:
        assert base in _OPAQUE, param
        return "handle*"
    if base == "char":
        return "str"
    if base in _OPAQUE:
        return "handle"
    assert base in _SCALAR, param
    return _SCALAR[base] + "*"


def header_prototypes():
    """{name: (return class, [argument classes])} from every header under include/."""
    text = ""
    for f in sorted(os.listdir(INCLUDE)):
        if f.endswith(".h"):
            text += _strip_c_comments(open(os.path.join(INCLUDE, f)).read())
    protos = {}
    for ret, name, args in re.findall(r"(int|const\s+char\s*\*)\s*(qr_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text):
        args = args.strip()
        classes = [] if args in ("", "void") else [_c_class(a) for a in args.split(",")]
        protos[name] = ("str" if "char" in ret else "int", classes)
    return protos


def header_defines():
    text = "".join(open(os.path.join(INCLUDE, f)).read() for f in sorted(os.listdir(INCLUDE)) if f.endswith(".h"))
    return {k: int(v) for k, v in re.findall(r"#define\s+(QR_[A-Z0-9_]+)\s+(\d+)", text)}


def _compatible(binding, c):
    """A binding's generic pointer (c_void_p, Ptr{Cvoid}) passes any single-level C pointer."""
    if binding == c:
        return True
    return binding == "ptr" and (c == "handle" or c == "str" or c.endswith("*") and c != "handle*")


# ---- Python ctypes ------------------------------------------------------------------------------
def _ctypes_class(t):
    scalars = {C.c_int: "int", C.c_double: "double", C.c_long: "long", C.c_uint64: "u64", C.c_uint32: "u32",
               C.c_char_p: "str", C.c_void_p: "ptr"}
    for k, v in scalars.items():
        if t is k:
            return v
    inner = getattr(t, "_type_", None)
    if inner is C.c_void_p:
        return "handle*"
    for k, v in scalars.items():
        if inner is k and v not in ("str", "ptr"):
            return v + "*"
    raise AssertionError(f"unclassified ctypes type {t}")


def test_python_signatures_match_header():
    from qrochet import _lib

    protos = header_prototypes()
    assert len(protos) >= 60
    for name, argtypes in _lib.SIGNATURES.items():
        assert name in protos, f"{name} is bound in Python but not declared"
        ret, cargs = protos[name]
        assert ret == "int", name
        got = [_ctypes_class(t) for t in argtypes]
        assert len(got) == len(cargs), f"{name}: {len(got)} ctypes arguments, {len(cargs)} declared"
        for i, (b, c) in enumerate(zip(got, cargs)):
            assert _compatible(b, c), f"{name} argument {i}: ctypes {b}, header {c}"


def test_python_constants_match_header():
    from qrochet import _lib

    for k, v in header_defines().items():
        if hasattr(_lib, k):
            assert getattr(_lib, k) == v, k
    for k in ("QR_OK", "QR_EINVAL", "QR_EASSERT", "QR_ENO_SCHMIDT", "QR_EDIM", "QR_ENOCONV", "QR_FP64",
              "QR_MIXED", "QR_DIR_LEFT", "QR_DIR_RIGHT", "QR_METHOD_QR", "QR_METHOD_SVD"):
        assert hasattr(_lib, k), k


# ---- Julia ccall sites ----------------------------------------------------------------------------
_JL = {
    "Cint": "int", "Int32": "int", "Cdouble": "double", "Float64": "double", "Clong": "long", "UInt64": "u64",
    "Culonglong": "u64", "Cstring": "str", "Ptr{Cvoid}": "ptr", "Ref{Ptr{Cvoid}}": "handle*",
    "Ptr{Ptr{Cvoid}}": "handle*", "Ptr{Cint}": "int*", "Ref{Cint}": "int*", "Ptr{Float64}": "double*",
    "Ref{Float64}": "double*", "Ptr{Cdouble}": "double*", "Ref{Cdouble}": "double*",
    # complex arrays cross as interleaved (re, im) doubles
    "Ptr{ComplexF64}": "double*", "Ref{ComplexF64}": "double*", "Ptr{UInt64}": "u64*", "Ref{UInt64}": "u64*",
}


def _split_top(s):
    """Split at commas outside (), [], {} and string literals."""
    out, depth, cur, instr = [], 0, "", False
    for ch in s:
        if instr:
            cur += ch
            instr = ch != '"'
            continue
        if ch == '"':
            instr = True
        elif ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        elif ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
            continue
        cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _balanced(text, start):
    """Contents of the parenthesis opening at text[start]."""
    assert text[start] == "("
    depth, instr = 0, False
    for i in range(start, len(text)):
        ch = text[i]
        if instr:
            instr = ch != '"'
        elif ch == '"':
            instr = True
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
            if depth == 0:
                return text[start + 1:i]
    raise AssertionError("unbalanced ccall")


def julia_ccalls():
    """[(symbol, return type, [argument types], number of argument expressions)]."""
    text = "\n".join(line.split("#", 1)[0] if not line.lstrip().startswith('"') else line
                     for line in open(JULIA).read().splitlines())
    calls = []
    for m in re.finditer(r"\bccall\(", text):
        body = _balanced(text, m.end() - 1)
        parts = _split_top(body)
        sym = re.fullmatch(r"\(:(qr_[a-z0-9_]+),\s*libqrochet\)", parts[0])
        assert sym, parts[0]
        tup = parts[2].strip()
        assert tup.startswith("(") and tup.endswith(")"), tup
        types = _split_top(tup[1:-1])
        calls.append((sym.group(1), parts[1], types, len(parts) - 3))
    return calls


def test_julia_ccalls_match_header():
    protos = header_prototypes()
    calls = julia_ccalls()
    assert len(calls) >= 30
    for sym, ret, types, nargs in calls:
        assert sym in protos, f"Julia calls {sym}, which the header does not declare"
        cret, cargs = protos[sym]
        assert {"Cint": "int", "Cstring": "str"}[ret] == cret, f"{sym}: return {ret}"
        assert len(types) == len(cargs), f"{sym}: {len(types)} ccall types, {len(cargs)} declared"
        assert nargs == len(types), f"{sym}: {nargs} arguments passed for {len(types)} types"
        for i, (t, c) in enumerate(zip(types, cargs)):
            assert t in _JL, f"{sym} argument {i}: unmapped Julia type {t}"
            assert _compatible(_JL[t], c), f"{sym} argument {i}: Julia {t}, header {c}"


def test_julia_binds_the_reference_methods():
    """The Julia shim reaches every entry point that replaces a reference method."""
    called = {c[0] for c in julia_ccalls()}
    for sym in ("qr_chain_create", "qr_chain_create_periodic", "qr_chain_upload_site", "qr_chain_download_site",
                "qr_chain_copy", "qr_canonize_site", "qr_canonize", "qr_mixed_canonize", "qr_normalize",
                "qr_truncate", "qr_evolve_1site", "qr_evolve_2site", "qr_evolve_layer", "qr_expect",
                "qr_overlap", "qr_norm", "qr_chain_random", "qr_chain_save", "qr_chain_load",
                "qr_chain_has_lambda", "qr_chain_get_lambda", "qr_chain_set_precision", "qr_canonicality_error",
                "qr_contract_between", "qr_mpo_create", "qr_mpo_upload_site", "qr_mpo_expect", "qr_mpo_free"):
        assert sym in called, sym


def test_julia_constants_match_header():
    text = open(JULIA).read()
    defs = header_defines()
    seen = 0
    for lhs, rhs in re.findall(r"^const\s+(QR_[A-Z0-9_, ]+?)\s*=\s*([0-9, ]+)$", text, flags=re.M):
        names = [x.strip() for x in lhs.split(",")]
        vals = [int(x) for x in rhs.split(",")]
        assert len(names) == len(vals), lhs
        for k, v in zip(names, vals):
            assert defs[k] == v, k
            seen += 1
    assert seen >= 11


@pytest.mark.parametrize("name", ["qr_evolve_2site", "qr_expect", "qr_truncate"])
def test_prototype_parser_sees_known_shapes(name):
    protos = header_prototypes()
    shapes = {
        "qr_evolve_2site": ["handle", "int", "double*", "double", "int", "int", "int"],
        "qr_expect": ["handle", "int", "int*", "int*", "double*", "double*"],
        "qr_truncate": ["handle", "int", "int", "double", "int"],
    }
    assert protos[name] == ("int", shapes[name])


# ---- gate memory order across the Julia binding --------------------------------------------------
def _julia_gatematrix_memory(array, sites, lanes):
    """NumPy restatement of QrochetGPU.gatematrix step by step with Julia's column-major rules
    (permutedims = axis transpose, reshape in column-major order, collect(transpose(M))), returning
    the memory a ccall passes: the result's column-major flattening."""
    k = len(lanes)
    perm = [sites.index((l, False)) for l in lanes] + [sites.index((l, True)) for l in lanes]
    t = np.transpose(array, perm)
    t = np.transpose(t, list(reversed(range(k))) + list(reversed(range(k, 2 * k))))
    d = t.shape[0]
    M = np.reshape(t, (d ** k, d ** k), order="F")
    R = M.T.copy()
    return R.flatten(order="F"), M


def test_julia_gate_memory_is_row_major_like_python():
    """For a non-symmetric two-site gate given with its sites in a scrambled order, the memory the
    Julia binding passes equals the Python mirror's row-major matrix (the C ABI's convention), and
    the transposed form would not."""
    import qrochet as Q

    g = np.random.default_rng(7)
    arr = g.standard_normal((2, 2, 2, 2)) + 1j * g.standard_normal((2, 2, 2, 2))
    order = [(5, True), (4, False), (5, False), (4, True)]
    mem, M = _julia_gatematrix_memory(arr, order, [4, 5])
    dense = Q.Dense(Q.Operator(), arr, [Q.Site(i, dual) for i, dual in order])
    row_major = np.ascontiguousarray(dense.matrix([4, 5])).ravel()
    np.testing.assert_array_equal(mem, row_major)
    assert not np.array_equal(M.flatten(order="F"), row_major), "the transposed memory differs"


def test_julia_gate_call_sites_pass_gatematrix_unchanged():
    """Every gate that crosses the C ABI from Julia is gatematrix's result as it is (no further
    transpose), so evolve!, evolve_layer! and expect agree on the memory order."""
    text = open(JULIA).read()
    uses = [m.start() for m in re.finditer(r"gatematrix\(", text)]
    calls = [i for i in uses if not text[max(0, i - 9):i].endswith("function ")]
    assert len(calls) >= 3
    for i in calls:
        assert text[i - 12:i] == "ComplexF64.(", text[i - 40:i + 30]
    assert "permutedims(gatematrix" not in text and "transpose(gatematrix" not in text
