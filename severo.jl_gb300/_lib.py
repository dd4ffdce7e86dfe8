"""ctypes binding of libseverogpu.so (the C ABI declared in include/severo_gpu.h).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libseverogpu.so"
HEADER = PKG.parent / "include" / "severo_gpu.h"

SV_OK = 0
SV_ERR_ARG = -1
SV_ERR_OOM = -2
SV_ERR_CUDA = -3
SV_ERR_NOCONV = -4
SV_ERR_UNSUPPORTED = -5
SV_ERR_STATE = -6
SV_ERR_DEVICE = -7

SV_I32, SV_I64, SV_F32, SV_F64, SV_BF16 = 1, 2, 3, 4, 5
SV_LOGNORMALIZE, SV_RELATIVECOUNTS = 0, 1
SV_EUCLIDEAN, SV_COSINE = 0, 1
SV_KNN_FP32, SV_KNN_BF16 = 0, 1

_ERRNAMES = {
    SV_ERR_ARG: "invalid argument", SV_ERR_OOM: "out of memory", SV_ERR_CUDA: "CUDA error",
    SV_ERR_NOCONV: "convergence failed", SV_ERR_UNSUPPORTED: "unsupported",
    SV_ERR_STATE: "bad state", SV_ERR_DEVICE: "device-side check failed",
}


class SeveroGPUError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


class ConvergenceError(SeveroGPUError):
    pass


vp = C.c_void_p
i64 = C.c_int64
i32 = C.c_int
dbl = C.c_double
P = C.POINTER
RANDV = C.CFUNCTYPE(None, P(C.c_double), C.c_int, C.c_void_p)
MATMUL = C.CFUNCTYPE(None, P(C.c_double), C.c_char, P(C.c_double), P(C.c_double), C.c_void_p)

# name -> (restype, argtypes)
SIGNATURES = {
    "sv_version": (i32, []),
    "sv_last_error": (i32, [C.c_char_p, C.c_size_t]),
    "sv_context_create": (i32, [i32, P(vp)]),
    "sv_context_destroy": (i32, [vp]),
    "sv_synchronize": (i32, [vp]),
    "sv_host_register": (i32, [vp, C.c_size_t]),
    "sv_host_unregister": (i32, [vp]),
    "sv_host_alloc": (i32, [P(vp), C.c_size_t]),
    "sv_host_free": (i32, [vp]),
    "sv_mark": (i32, [vp, i32]),
    "sv_elapsed_ms": (i32, [vp, i32, i32, P(dbl)]),
    "sv_launch_count": (i32, [vp, P(i64)]),
    "sv_profile_enable": (i32, [vp, i32]),
    "sv_profile_reset": (i32, [vp]),
    "sv_profile_query": (i32, [vp, C.c_char_p, P(dbl), P(i64)]),
    "sv_profile_report": (i32, [vp, C.c_char_p, C.c_size_t]),
    "sv_device_memory": (i32, [vp, P(C.c_size_t), P(C.c_size_t)]),
    "sv_counts_upload_csc": (i32, [vp, i64, i64, i64, vp, i32, vp, i32, vp, i32, i32, P(vp)]),
    "sv_counts_upload_csr": (i32, [vp, i64, i64, i64, vp, i32, vp, i32, vp, i32, i32, P(vp)]),
    "sv_counts_read_mtx": (i32, [vp, C.c_char_p, i32, P(vp)]),
    "sv_counts_parse_mtx": (i32, [vp, C.c_char_p, i64, i32, P(vp)]),
    "sv_counts_generate": (i32, [vp, i64, i64, vp, vp, vp, vp, C.c_int32, dbl, dbl, C.c_uint64, P(vp)]),
    "sv_counts_info": (i32, [vp, P(i64), P(i64), P(i64)]),
    "sv_counts_download_csc": (i32, [vp, vp, vp, vp, vp]),
    "sv_counts_download_csr": (i32, [vp, vp, vp, vp, vp]),
    "sv_counts_free": (i32, [vp]),
    "sv_filter_counts": (i32, [vp, vp, i64, i64, i64, i64, vp, vp, P(vp)]),
    "sv_counts_select_cells": (i32, [vp, vp, i64, i64, P(vp)]),
    "sv_find_variable_features_vst": (i32, [vp, vp, i64, C.c_double, vp, vp]),
    "sv_find_variable_features_vst_surface": (i32, [vp, vp, i64, C.c_double, i32, vp, vp]),
    "sv_loess_vertices": (i64, [vp, i64, C.c_double, vp, i64]),
    "sv_normalize_cells": (i32, [vp, vp, i32, dbl, i32, P(vp)]),
    "sv_selftest_wait_timeout": (i32, [vp, C.c_longlong]),
    "sv_centered_gram": (i32, [vp, vp, vp, dbl, dbl, vp]),
    "sv_sparse_mul_spvec": (i32, [vp, i64, i64, vp, vp, vp, i64, vp, vp, i32, dbl, dbl, vp]),
    "sv_sparse_mul_sparse": (i32, [vp, i64, i64, i64, vp, vp, vp, i32, vp, vp, vp, i32, dbl, dbl, vp]),
    "sv_normalize_csc_noalloc": (i32, [vp, vp, vp, i64, i64, i64, i32, dbl, vp, vp]),
    "sv_data_download_csc": (i32, [vp, vp, vp]),
    "sv_data_download_csr": (i32, [vp, vp, vp]),
    "sv_data_cell_totals": (i32, [vp, vp, vp]),
    "sv_data_free": (i32, [vp]),
    "sv_scale_features": (i32, [vp, vp, vp, i64, dbl, P(vp)]),
    "sv_centered_create": (i32, [vp, i64, i64, i64, vp, vp, vp, vp, i32, P(vp)]),
    "sv_gene_moments": (i32, [vp, vp, vp, vp]),
    "sv_centered_info": (i32, [vp, P(i64), P(i64), P(i64)]),
    "sv_centered_stats": (i32, [vp, vp, vp, vp, vp]),
    "sv_centered_mul": (i32, [vp, vp, C.c_char, i64, dbl, vp, i64, dbl, vp, i64]),
    "sv_centered_free": (i32, [vp]),
    "sv_irlba": (i32, [vp, vp, i64, i64, i64, dbl, vp, C.c_uint64, vp, vp, vp, P(i64), P(i64)]),
    "sv_pca": (i32, [vp, vp, i64, i64, dbl, vp, C.c_uint64, P(vp), vp, vp, vp, P(i64), P(i64)]),
    "sv_embed_info": (i32, [vp, P(i64), P(i64)]),
    "sv_embed_free": (i32, [vp]),
    "irlba": (i32, [i64, i64, i64, i64, i64, i64, dbl, vp, vp, vp, vp, RANDV, MATMUL, vp]),
    "sv_knn_host": (i32, [vp, vp, i32, i64, i64, i64, i64, i32, i32, i32, vp, vp, P(vp)]),
    "sv_knn_embed": (i32, [vp, vp, i64, i64, i32, i32, i32, vp, vp, P(vp)]),
    "sv_knn_info": (i32, [vp, P(i64), P(i64)]),
    "sv_knn_free": (i32, [vp]),
    "FindNeighboursEuclidean32": (None, [vp, i32, i32, i32, i32, i32, i32, i32, vp, vp]),
    "FindNeighboursEuclidean64": (None, [vp, i32, i32, i32, i32, i32, i32, i32, vp, vp]),
    "FindNeighboursCosine32": (None, [vp, i32, i32, i32, i32, i32, i32, i32, vp, vp]),
    "FindNeighboursCosine64": (None, [vp, i32, i32, i32, i32, i32, i32, i32, vp, vp]),
    "sv_snn_host": (i32, [vp, vp, i64, i64, i64, dbl, i32, P(vp)]),
    "sv_snn_knn": (i32, [vp, vp, i64, dbl, i32, P(vp)]),
    "sv_graph_info": (i32, [vp, P(i64), P(i64)]),
    "sv_graph_download": (i32, [vp, vp, vp, vp, vp]),
    "sv_graph_network": (i32, [vp, vp, P(i64), vp, vp, vp]),
    "sv_graph_free": (i32, [vp]),
    "sv_batch_create": (i32, [vp, vp, vp, i64, vp, i64, C.c_double, P(vp)]),
    "sv_batch_info": (i32, [vp, P(i64), P(i64), P(i64)]),
    "sv_batch_stats": (i32, [vp, vp, vp, vp, vp]),
    "sv_batch_pca": (i32, [vp, vp, i64, i64, C.c_double, vp, C.c_uint64, P(vp), vp, vp, vp, P(i64)]),
    "sv_batch_knn": (i32, [vp, vp, vp, i64, i64, i32, i32, i32, vp, vp, P(vp)]),
    "sv_batch_tuning": (i32, [vp, P(i64)]),
    "sv_batch_free": (i32, [vp]),
}

_lib = None


def header_symbols():
    """Function names declared in include/severo_gpu.h."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:int64_t|int|void)\s+\**\s*([A-Za-z_]\w*)\s*\(", text, flags=re.M)
    return sorted(set(names))


def load(path: os.PathLike | None = None):
    """Loads the library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise SeveroGPUError(SV_ERR_STATE, f"{p} is missing: build it with "
                             "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    lib = load()
    buf = C.create_string_buffer(2048)
    lib.sv_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int):
    if status != SV_OK:
        msg = last_error()
        if status == SV_ERR_NOCONV:
            raise ConvergenceError(status, msg)
        raise SeveroGPUError(status, msg)
