"""C-ABI surface checks that need no GPU: every declared entry point is
exported by the CUDA library and mirrored by the oracle, and the library
fails loudly (WF_ERR_CUDA) when no device is present."""
import ctypes
import os
import re

import pytest

import __graft_entry__ as ge
import weldform_gb300 as wf

HEADER = os.path.join(ge.ROOT, "include", "weldform_gb300.h")


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(wf_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def cuda_lib_path():
    p = wf.LIB_PATH
    if not os.path.exists(p):
        ge.build_cuda()
    return p


def test_header_declares_every_bound_entry_point():
    names = declared()
    for e in wf.EXPORTS:
        assert "wf_" + e in names, e


def test_library_exports_every_declared_symbol(cuda_lib_path):
    lib = ctypes.CDLL(cuda_lib_path)
    for name in declared():
        assert hasattr(lib, name), name
    wf.bind(lib, "wf_")


def test_oracle_mirrors_the_abi():
    from tests._support import oracle_lib
    lib = oracle_lib()
    for name in declared():
        if name == "wf_neighbour_list_static":  # product-only helper, no reference counterpart
            continue
        assert hasattr(lib, "wfo_" + name[3:]), name


def test_no_device_is_a_loud_error(cuda_lib_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = wf.bind(ctypes.CDLL(cuda_lib_path), "wf_")
    h = ctypes.c_void_p()
    rc = lib.wf_domain_create(3, ctypes.byref(h))
    assert rc == 2  # WF_ERR_CUDA
    assert b"device" in lib.wf_last_error()
    with pytest.raises(wf.WFError):
        wf.Domain()


def test_header_documents_every_domain_field():
    """Every field name the library's domain setters and getters accept is
    documented in the header (the C ABI's only description for a caller)."""
    src = open(os.path.join(ge.ROOT, "weldform_gb300", "csrc", "wf_domain.cu")).read()
    hdr = open(HEADER).read()
    names = set(re.findall(r'n == "([A-Za-z_.|0-9]+)"', src))
    assert len(names) > 50
    missing = sorted(n for n in names if '"' + n + '"' not in hdr)
    assert not missing, missing


def test_header_documents_every_particle_array():
    """Every per-particle f64 array in the library's column table (the names
    wf_get/set_particle_array_f64 accept) is named in the header."""
    src = open(os.path.join(ge.ROOT, "weldform_gb300", "csrc", "wf_domain.cu")).read()
    hdr = open(HEADER).read()
    names = set(re.findall(r'\{"([A-Za-z_0-9]+)", C_[A-Z0-9]+, \d\}', src))
    assert len(names) > 40
    missing = sorted(n for n in names if '"' + n + '"' not in hdr)
    assert not missing, missing


def _ctype(param):
    """ctypes type of one C parameter declaration of the header."""
    stars = param.count("*") + param.count("[")
    words = re.sub(r"\[.*?\]", "", re.sub(r"\bconst\b", "", param)).replace("*", " ").split()
    base = words[0] if words else ""
    if base == "char" and stars == 1:
        return ctypes.c_char_p
    if base in ("wf_domain", "void"):
        return ctypes.c_void_p if stars == 1 else ctypes.POINTER(ctypes.c_void_p)
    scalar = {"double": ctypes.c_double, "int": ctypes.c_int, "int64_t": ctypes.c_int64,
              "int32_t": ctypes.c_int32, "float": ctypes.c_float}[base]
    return ctypes.POINTER(scalar) if stars == 1 else scalar


def _header_signatures():
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    out = {}
    for name, args in re.findall(r"\b(?:int|const char\s*\*|double|void)\s+(wf_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", txt):
        params = [a for a in args.split(",") if a.strip() and a.strip() != "void"]
        out[name] = [_ctype(a) for a in params]
    return out


def test_ctypes_signatures_match_the_header():
    """Every entry point the Python mirror binds has the header's arity and
    argument types (a width mismatch, int against int64_t, would truncate
    silently through ctypes)."""
    assert _ctype("const double V[3]") is ctypes.POINTER(ctypes.c_double)
    assert _ctype("wf_domain** out") is ctypes.POINTER(ctypes.c_void_p)
    assert _ctype("int64_t n") is ctypes.c_int64 and _ctype("const char* field") is ctypes.c_char_p
    sigs = _header_signatures()
    assert set(declared()) == set(sigs)
    for key, argtypes in wf._SIGS.items():
        assert sigs["wf_" + key] == list(argtypes), key


def test_oracle_definitions_match_the_header():
    """The oracle's wfo_* definitions take the header's argument types, so the
    same ctypes table drives both libraries."""
    src = open(os.path.join(ge.ROOT, "oracle", "wf_oracle.cpp")).read()
    src = re.sub(r"//[^\n]*", "", re.sub(r"/\*.*?\*/", "", src, flags=re.S))
    defs = dict(re.findall(r"\b(?:int|const char\s*\*|double)\s+wfo_([a-z0-9_]+)\s*\(([^)]*)\)\s*\{", src))
    for name, sig in _header_signatures().items():
        if name == "wf_neighbour_list_static":  # product-only helper
            continue
        params = [a for a in defs[name[3:]].split(",") if a.strip() and a.strip() != "void"]
        assert [_ctype(a.replace("wfo_domain", "wf_domain")) for a in params] == sig, name
