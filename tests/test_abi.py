"""The C-ABI libraries load and export every symbol their headers declare.

No compute call is made here: these run on machines without a GPU.
"""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import PKG, ROOT

INCLUDE = os.path.join(ROOT, "include")


def declared(header: str) -> list[str]:
    src = open(os.path.join(INCLUDE, header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(lvgg?_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def exported(lib: str) -> set[str]:
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_graphgen_exports_everything(lvg):
    names = declared("louvain_gb300_graphgen.h")
    assert len(names) >= 7
    missing = [n for n in names if n not in exported(lvg.gen_path())]
    assert not missing, missing


def test_cuda_library_builds_loads_and_exports_everything(lvg):
    import lvg_build

    lvg_build.build_cuda()
    names = declared("louvain_gb300.h")
    assert {"lvg_static", "lvg_naive_dynamic", "lvg_delta_screening", "lvg_frontier", "lvg_result_free"} <= set(names)
    ex = exported(lvg.lib_path())
    missing = [n for n in names if n not in ex]
    assert not missing, missing
    lib = ctypes.CDLL(lvg.lib_path())  # loads without a GPU; no compute call
    for n in names:
        assert hasattr(lib, n)


def test_cuda_objects_are_sm_103a_only():
    """Every device object is compiled for sm_103a (checked from the build flags)."""
    import lvg_build

    assert lvg_build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_options_defaults_match_reference(lvg):
    o = lvg.LouvainOptions()
    # LouvainOptions(int repeat=1, double resolution=1, double tolerance=1e-2,
    #   double aggregationTolerance=1.0, double toleranceDrop=10, int maxIterations=20, int maxPasses=10)
    assert (o.repeat, o.resolution, o.tolerance, o.aggregationTolerance, o.toleranceDrop, o.maxIterations,
            o.maxPasses) == (1, 1.0, 1e-2, 1.0, 10.0, 20, 10)
    assert not o.deterministic
    assert o.effective_colors() == 8 and lvg.LouvainOptions(deterministic=True).effective_colors() == 16


def test_missing_library_fails_loudly(lvg, monkeypatch, tmp_path):
    monkeypatch.setattr(lvg, "LIBDIR", str(tmp_path))
    monkeypatch.setattr(lvg, "_lib", None)
    with pytest.raises(lvg.LvgError):
        lvg.load_library()


def _struct_fields(header: str, name: str) -> list[tuple[str, int]]:
    """(field, array length) of `typedef struct name {...} name;` in a header."""
    src = open(os.path.join(INCLUDE, header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", src, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        # "type a, *b, c[12]" -> every declarator
        head = re.match(r"((?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**)\s*(.*)", decl, flags=re.S)
        for d in head.group(2).split(","):
            m = re.match(r"\s*\**\s*([A-Za-z_][A-Za-z0-9_]*)\s*(?:\[(\d+)\])?\s*$", d)
            fields.append((m.group(1), int(m.group(2) or 0)))
    return fields


@pytest.mark.parametrize("header,cname,pyname", [
    ("louvain_gb300.h", "lvg_tuning", "_Tuning"), ("louvain_gb300.h", "lvg_stats", "_Stats"),
    ("louvain_gb300.h", "lvg_options", "_Options"), ("louvain_gb300.h", "lvg_result", "_Result"),
    ("louvain_gb300.h", "lvg_batch", "_Batch"), ("louvain_gb300.h", "lvg_batch_buf", "_BatchBuf"),
    ("louvain_gb300.h", "lvg_server_options", "_ServerOptions"),
    ("louvain_gb300.h", "lvg_request_info", "_RequestInfo"),
    ("louvain_gb300.h", "lvg_server_stats_t", "_ServerStats"),
    ("louvain_gb300_graphgen.h", "lvgg_csr", "_Csr"), ("louvain_gb300_graphgen.h", "lvgg_batch", "_GBatch"),
    ("louvain_gb300_graphgen.h", "lvgg_edges", "_Edges")])
def test_python_mirrors_follow_the_header(lvg, header, cname, pyname):
    """The ctypes mirrors in lvg.py list the C structs' fields in the header's
    order, with the same array lengths (a mismatch would shift every later
    field across the boundary)."""
    c_fields = _struct_fields(header, cname)
    py = getattr(lvg, pyname)
    py_fields = [(n, getattr(t, "_length_", 0)) for n, t in py._fields_]
    assert py_fields == c_fields, (cname, c_fields, py_fields)


def _prototypes(header: str) -> dict[str, int]:
    """Each function the header declares, with its parameter count."""
    src = open(os.path.join(INCLUDE, header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    out = {}
    for m in re.finditer(r"\b(lvgg?_[a-z0-9_]+)\s*\(([^;{()]*)\)\s*;", src):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else len(params.split(","))
    return out


@pytest.mark.parametrize("header,loader", [("louvain_gb300.h", "load_library"),
                                           ("louvain_gb300_graphgen.h", "load_graphgen")])
def test_python_binding_declares_every_argument(lvg, header, loader):
    """Every entry point lvg.py calls with arguments has ctypes argtypes of the
    header's arity (without them ctypes passes Python ints as C int, which
    truncates pointers and sizes)."""
    import lvg_build

    if loader == "load_library":
        lvg_build.build_cuda()
    protos = _prototypes(header)
    assert len(protos) == len(declared(header))
    src = open(os.path.join(PKG, "lvg.py")).read()
    # called directly, or by name through getattr
    used = (set(re.findall(r"\b(lvgg?_[a-z0-9_]+)\(", src)) | set(re.findall(r'"(lvgg?_[a-z0-9_]+)"', src))) & set(protos)
    assert used
    L = getattr(lvg, loader)()
    bad = [(n, protos[n], getattr(L, n).argtypes) for n in sorted(used)
           if protos[n] and len(getattr(L, n).argtypes or ()) != protos[n]]
    assert not bad, bad


def _return_types(header: str) -> dict[str, str]:
    src = open(os.path.join(INCLUDE, header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    pat = r"(?:^|[;}\n])\s*((?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**)\s*\b(lvgg?_[a-z0-9_]+)\s*\(([^;{()]*)\)\s*;"
    return {m.group(2): " ".join(m.group(1).split()) for m in re.finditer(pat, src)}


@pytest.mark.parametrize("header,loader", [("louvain_gb300.h", "load_library"),
                                           ("louvain_gb300_graphgen.h", "load_graphgen")])
def test_python_binding_declares_wide_returns(lvg, header, loader):
    """Entry points that return a size or a pointer have a ctypes restype that
    holds it (the default, C int, would cut it to 32 bits)."""
    import lvg_build

    if loader == "load_library":
        lvg_build.build_cuda()
    rts = _return_types(header)
    assert set(rts) == set(_prototypes(header))
    src = open(os.path.join(PKG, "lvg.py")).read()
    used = set(re.findall(r"\b(lvgg?_[a-z0-9_]+)\(", src)) & set(rts)
    L = getattr(lvg, loader)()
    wide = {"size_t": (ctypes.c_size_t, ctypes.c_uint64, ctypes.c_ulonglong),
            "pointer": (ctypes.c_void_p, ctypes.c_char_p)}
    bad = []
    for n in sorted(used):
        rt = rts[n]
        kind = "pointer" if rt.endswith("*") else "size_t" if rt == "size_t" else None
        if kind and getattr(L, n).restype not in wide[kind]:
            bad.append((n, rt, getattr(L, n).restype))
    assert not bad, bad


def _params(header: str) -> dict[str, list[str]]:
    src = open(os.path.join(INCLUDE, header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    out = {}
    for m in re.finditer(r"\b(lvgg?_[a-z0-9_]+)\s*\(([^;{()]*)\)\s*;", src):
        p = m.group(2).strip()
        out[m.group(1)] = [] if p in ("", "void") else [x.strip() for x in p.split(",")]
    return out


def _null_cases():
    out = []
    for header in ("louvain_gb300.h", "louvain_gb300_graphgen.h"):
        rts = _return_types(header)
        for n, ps in sorted(_params(header).items()):
            if any("*" in p for p in ps) and (rts[n] == "int" or n.endswith(("_free", "_close"))):
                out.append((header, n))
    return out


@pytest.mark.parametrize("header,name", _null_cases())
def test_null_arguments_are_rejected_not_dereferenced(lvg, header, name):
    """Every status-returning entry point with pointer arguments, called with
    every pointer NULL (and every number 0), returns LVG_EINVAL with a message
    before touching the device; the destructors (and the graph generators'
    free/close calls) accept NULL as free() does. Runs without a GPU."""
    import lvg_build

    if header == "louvain_gb300.h":
        lvg_build.build_cuda()
        L = ctypes.CDLL(lvg.lib_path())  # its own function objects: no argtypes of lvg.py's
        err = L.lvg_last_error
    else:
        L = ctypes.CDLL(lvg.gen_path())
        err = L.lvgg_last_error
    err.restype = ctypes.c_char_p
    args = []
    for p in _params(header)[name]:
        t = p.split()[0] if not p.startswith("const ") else p.split()[1]
        if "*" in p:
            args.append(ctypes.c_void_p(None))
        elif t in ("double", "float"):
            args.append(ctypes.c_double(0.0) if t == "double" else ctypes.c_float(0.0))
        elif t in ("size_t", "uint64_t"):
            args.append(ctypes.c_uint64(0))
        else:
            args.append(ctypes.c_int(0))
    f = getattr(L, name)
    if _return_types(header)[name] == "void":
        f.restype = None
        f(*args)
        return
    rc = f(*args)
    if name.endswith("_destroy"):
        assert rc == lvg.LVG_OK
    else:
        assert rc == lvg.LVG_EINVAL, (name, rc)
        assert err(), name
