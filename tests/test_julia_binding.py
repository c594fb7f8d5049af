"""The Julia binding sources (justpic.jl_gb300/julia/*.jl) against the C ABI
in include/justpic_gb300.h, read as text (there is no Julia here): every
``ccall`` names a declared entry point, passes as many arguments as the
prototype takes, and declares each argument with a Julia type of the same
C shape. An array of pointers (``const double* const coords[3]``, ``double*
const* F``) is a pointer to pointers on the C side, so the ccall must declare
``Ptr{Ptr{...}}`` (a tuple declared by value would be passed as an aggregate)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "justpic_gb300.h")
JULIA = os.path.join(ROOT, "justpic.jl_gb300", "julia")


def _split_top(s, sep=","):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == sep and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def prototypes():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    protos = {}
    for m in re.finditer(r"\b[\w\s\*]*?\b(jp_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        params = [p for p in _split_top(" ".join(m.group(2).split())) if p and p != "void"]
        protos[m.group(1)] = params
    return protos


def c_shape(param):
    """'pp' pointer to pointers, 'p' pointer, or the scalar type."""
    p = param.strip()
    if re.search(r"\[\s*\d*\s*\]\s*$", p):
        base = re.sub(r"\w+\s*\[\s*\d*\s*\]\s*$", "", p)
        return "pp" if "*" in base else "p"
    if p.count("*") >= 2:
        return "pp"
    if "*" in p:
        return "p"
    scalar = p.rsplit(" ", 1)[0].replace("const ", "").strip()
    return {"double": "f64", "float": "f32", "int32_t": "i32", "int": "i32", "int64_t": "i64",
            "uint64_t": "u64", "uint32_t": "u32", "size_t": "u64", "uint8_t": "u8"}.get(scalar, scalar)


def julia_shape(t):
    t = t.strip()
    if re.fullmatch(r"(Ptr|Ref)\{(Ptr|Ref)\{.*\}\}", t):
        return "pp"
    if t.startswith(("Ptr{", "Ref{")) or t in ("Cstring", "Ptr"):
        return "p"
    return {"Float64": "f64", "Cdouble": "f64", "Float32": "f32", "Cfloat": "f32", "Int32": "i32",
            "Cint": "i32", "Int64": "i64", "UInt64": "u64", "Csize_t": "u64", "UInt32": "u32",
            "UInt8": "u8"}.get(t, t)


def _types_after(text, start):
    i, depth = start, 1
    while depth:
        depth += {"(": 1, ")": -1}.get(text[i], 0)
        i += 1
    return _split_top(" ".join(text[start:i - 1].split()))


def ccalls():
    """(file, line, entry point, argument types) of every ccall: the literal ones,
    and those an `@eval` loop generates (`for (f, sym) in ((:f, :jp_x), ...)`
    around `ccall(($(QuoteNode(sym)), lib), ...)`), once per symbol."""
    out = []
    for fn in sorted(os.listdir(JULIA)):
        if not fn.endswith(".jl"):
            continue
        text = open(os.path.join(JULIA, fn)).read()
        for m in re.finditer(r"ccall\(\(:(jp_[a-z0-9_]+),\s*lib\),\s*\w+,\s*\(", text):
            line = text.count("\n", 0, m.start()) + 1
            out.append((fn, line, m.group(1), _types_after(text, m.end())))
        for loop in re.finditer(r"for \(f, sym\) in \(((?:[^()]|\([^()]*\))*)\)", text):
            syms = re.findall(r":(jp_[a-z0-9_]+)", loop.group(1))
            m = re.compile(r"ccall\(\(\$\(QuoteNode\(sym\)\),\s*lib\),\s*\w+,\s*\(").search(text, loop.end())
            assert m and syms, f"{fn}: a generated ccall loop the test cannot read"
            line = text.count("\n", 0, m.start()) + 1
            for sym in syms:
                out.append((fn, line, sym, _types_after(text, m.end())))
    return out


# entry points the Julia sources leave to other callers, with the reason
NOT_BOUND = {
    "jp_particles_info": "the extension keeps the sizes in its Particles object",
    "jp_selftest_weight": "a test of the library's weight arithmetic (tests/test_gpu_weight.py)",
    "jp_advection_vjp_f32": "the FP32-offset adjoint is driven from Python (adjoint.py)",
    "jp_inject_vjp_i32": "the FP32-offset adjoint is driven from Python (adjoint.py)",
    "jp_particle2grid_f32_with_weights": "the FP32-offset adjoint is driven from Python (adjoint.py)",
    "jp_particle2grid_vjp_f32": "the FP32-offset adjoint is driven from Python (adjoint.py)",
    "jp_slot_ids_i32": "the FP32-offset adjoint is driven from Python (adjoint.py)",
}


def test_every_entry_point_is_bound_or_accounted_for():
    bound = {name for _, _, name, _ in ccalls()}
    missing = sorted(set(prototypes()) - bound - set(NOT_BOUND))
    assert not missing, f"header entry points with no ccall in the Julia sources: {missing}"
    assert not (bound & set(NOT_BOUND)), "an entry point listed as not bound has a ccall"


def test_julia_sources_have_ccalls():
    assert len(ccalls()) > 30


@pytest.mark.parametrize("fn,line,name,types", ccalls(), ids=lambda v: v if isinstance(v, str) else None)
def test_ccall_matches_the_header(fn, line, name, types):
    protos = prototypes()
    assert name in protos, f"{fn}:{line}: {name} is not declared in the header"
    params = protos[name]
    assert len(types) == len(params), f"{fn}:{line}: {name} takes {len(params)} arguments, ccall declares {len(types)}"
    for k, (p, t) in enumerate(zip(params, types)):
        assert c_shape(p) == julia_shape(t), f"{fn}:{line}: {name} argument {k + 1}: C '{p}' vs Julia '{t}'"
