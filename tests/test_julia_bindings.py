"""The Julia bindings (severo.jl_gb300/julia/SeveroGPU.jl and the ccall stubs
given for the reference side) against the C declarations they call.

Julia is installed on neither machine, so the glue cannot run here; this reads
every `ccall((:name, lib), Ret, (types...), ...)` and checks it against
include/severo_gpu.h: the symbol is declared, the return type and the number of
arguments agree, every scalar has the C type's Julia counterpart, and every
pointer is passed as a pointer whose element type, where both sides name one,
is the same.
"""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "severo_gpu.h"
SOURCES = [ROOT / "severo.jl_gb300" / "julia" / "SeveroGPU.jl", ROOT / "INTEGRATION.md"]

SCALARS = {
    "int": {"Cint", "Int32"}, "int32_t": {"Cint", "Int32"}, "int64_t": {"Int64", "Clonglong"},
    "long long": {"Clonglong", "Int64"}, "uint64_t": {"UInt64", "Culonglong"},
    "size_t": {"Csize_t", "UInt64"}, "double": {"Cdouble", "Float64"}, "float": {"Cfloat", "Float32"},
    "char": {"Cchar", "UInt8"},
}
ELEMENTS = {   # C pointee -> Julia element types that have its layout
    "int64_t": {"Int64"}, "int32_t": {"Int32", "Cint"}, "int": {"Cint", "Int32"},
    "double": {"Float64", "Cdouble"}, "float": {"Float32", "Cfloat"}, "uint8_t": {"UInt8"},
    "char": {"UInt8", "Cchar"},
}
RETURNS = {"int": {"Cint", "Int32"}, "int64_t": {"Int64"}}


def header_decls():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    decls = {}
    for m in re.finditer(r"^\s*(int64_t|int|void)\s+\**\s*([A-Za-z_]\w*)\s*\(([^;]*?)\)\s*;", text,
                         flags=re.M | re.S):
        ret, name, params = m.groups()
        params = " ".join(params.split())
        plist = [] if params in ("", "void") else [p.strip() for p in params.split(",")]
        decls[name] = (ret, plist)
    return decls


def julia_ccalls():
    out = []
    for src in SOURCES:
        text = src.read_text()
        for m in re.finditer(r"ccall\(\(:(\w+),\s*\w+\),\s*(\w+),\s*\(([^()]*)\)", text):
            name, ret, types = m.groups()
            line = text.count("\n", 0, m.start()) + 1
            out.append((f"{src.name}:{line}", name, ret, [t.strip() for t in types.split(",") if t.strip()]))
    return out


def _c_param(p):
    """'const int64_t* colptr' -> ('int64_t', 1); 'double scale' -> ('double', 0)."""
    p = p.replace("const ", "").strip()
    stars = p.count("*")
    base = p.replace("*", " ").split()
    base = " ".join(base[:-1]) if len(base) > 1 else base[0]
    return base, stars


def _julia_elem(t):
    m = re.fullmatch(r"(Ptr|Ref)\{(.+)\}", t)
    return m.group(2) if m else None


def test_bindings_cover_the_entry_points():
    calls = julia_ccalls()
    names = {c[1] for c in calls}
    assert len(calls) >= 40
    for must in ("sv_normalize_cells", "sv_scale_features", "sv_pca", "sv_knn_embed", "sv_snn_knn",
                 "sv_filter_counts", "sv_find_variable_features_vst_surface", "sv_counts_read_mtx"):
        assert must in names, must


@pytest.mark.parametrize("where,name,ret,jtypes", julia_ccalls(), ids=lambda v: v if isinstance(v, str) else None)
def test_ccall_matches_declaration(where, name, ret, jtypes):
    decls = header_decls()
    if name not in decls:
        # the reference-named drop-ins are declared too; anything else is a typo
        pytest.fail(f"{where}: {name} is not declared in include/severo_gpu.h")
    cret, cparams = decls[name]
    assert ret in RETURNS[cret], f"{where}: {name} returns {cret}, ccall says {ret}"
    assert len(jtypes) == len(cparams), f"{where}: {name} takes {len(cparams)} arguments, ccall passes {len(jtypes)}"
    for jt, cp in zip(jtypes, cparams):
        base, stars = _c_param(cp)
        if base.endswith("_fn"):                  # callback typedefs: a C function pointer
            assert jt == "Ptr{Cvoid}", f"{where}: {name}: {cp} needs Ptr{{Cvoid}}, got {jt}"
            continue
        if stars == 0:
            assert jt in SCALARS[base], f"{where}: {name}: {cp} is {base}, ccall passes {jt}"
            continue
        if base == "char" and stars == 1:
            assert jt in ("Cstring", "Ptr{UInt8}"), f"{where}: {name}: {cp} needs a string, got {jt}"
            continue
        elem = _julia_elem(jt)
        assert elem is not None, f"{where}: {name}: {cp} is a pointer, ccall passes {jt}"
        if stars == 2:                             # an out-handle: sv_x** -> Ref{Ptr{Cvoid}}
            assert elem == "Ptr{Cvoid}", f"{where}: {name}: {cp} needs Ref{{Ptr{{Cvoid}}}}, got {jt}"
            continue
        if base in ELEMENTS and elem not in ("Cvoid", "T") and not elem.startswith(("Node", "Edge")):
            assert elem in ELEMENTS[base], f"{where}: {name}: {cp} points to {base}, ccall says {jt}"
