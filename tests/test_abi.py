"""The C-ABI library builds, loads and exports every symbol include/severo_gpu.h
declares; host-side argument handling.  No GPU compute (CPU only)."""
import ctypes as C
import subprocess

import numpy as np
import pytest

import __graft_entry__ as ge


@pytest.fixture(scope="module")
def lib():
    ge._build_module().build()
    pkg = ge.load_package()
    return pkg._lib


def test_exports_every_declared_symbol(lib):
    declared = lib.header_symbols()
    assert len(declared) >= 50
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    # nothing else leaks out of the library besides the declared C ABI
    extra = sorted(s for s in exported if not s.startswith("_") and s not in declared)
    assert not extra, extra


def test_ctypes_table_matches_header(lib):
    assert sorted(lib.SIGNATURES) == lib.header_symbols()


def test_load_and_version(lib):
    L = lib.load()
    assert L.sv_version() == 100


def test_errors_without_device(lib):
    """On a host without a GPU, creating a context fails with a status code, not a crash."""
    L = lib.load()
    h = C.c_void_p()
    st = L.sv_context_create(0, C.byref(h))
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        assert st == 0
        L.sv_context_destroy(h)
    else:
        assert st < 0
        assert len(lib.last_error()) > 0


def test_null_arguments_are_rejected(lib):
    L = lib.load()
    assert L.sv_counts_info(None, None, None, None) == lib.SV_ERR_ARG
    assert "null" in lib.last_error()
    assert L.sv_context_create(0, None) == lib.SV_ERR_ARG


def test_python_api_validates_method(lib):
    pkg = ge.load_package()
    with pytest.raises(ValueError, match="unknown normalization method"):
        pkg.normalize_cells(None, method="bogus")


def test_missing_library_fails_loudly(lib, monkeypatch, tmp_path):
    """Without the built library there is no fallback: loading raises."""
    monkeypatch.setattr(lib, "_lib", None)
    with pytest.raises(lib.SeveroGPUError, match="is missing"):
        lib.load(tmp_path / "libseverogpu.so")
