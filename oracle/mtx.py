"""ctypes wrapper of the MatrixMarket oracle (mtx_oracle.c) -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__`` (to build it) and the CPU-baseline leg of
``bench.py`` use this module.  ``build()`` compiles mtx_oracle.c with gcc into
``oracle/_build/``; ``parse()`` returns the cells x genes CSC the reference's
reader would hold, or raises ``MtxOracleError`` with the failing stage.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import scipy.sparse as sp

HERE = Path(__file__).resolve().parent
SRC = HERE / "mtx_oracle.c"
LIB = HERE / "_build" / "libmtx_oracle.so"

STAGES = {1: "header", 2: "entry", 3: "range", 4: "value"}


class MtxOracleError(ValueError):
    def __init__(self, code, msg):
        super().__init__(f"{STAGES.get(code, code)}: {msg}")
        self.stage = STAGES.get(code, str(code))


class _Result(C.Structure):
    _fields_ = [("n_cells", C.c_int64), ("n_genes", C.c_int64), ("nnz", C.c_int64),
                ("colptr", C.POINTER(C.c_int64)), ("rowidx", C.POINTER(C.c_int32)),
                ("val", C.POINTER(C.c_int32)), ("err", C.c_char * 256)]


_lib = None


def build() -> Path:
    LIB.parent.mkdir(exist_ok=True)
    if not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        tmp = LIB.with_suffix(".tmp")
        subprocess.run(["gcc", "-O2", "-shared", "-fPIC", str(SRC), "-o", str(tmp)], check=True)
        tmp.replace(LIB)
    return LIB


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        lib.mtx_oracle_parse.argtypes = [C.c_char_p, C.c_int64, C.c_int, C.POINTER(_Result)]
        lib.mtx_oracle_parse.restype = C.c_int
        lib.mtx_oracle_free.argtypes = [C.POINTER(_Result)]
        _lib = lib
    return _lib


def parse(text: bytes, rows_are_features: bool = True) -> sp.csc_matrix:
    lib = _load()
    r = _Result()
    rc = lib.mtx_oracle_parse(text, len(text), int(rows_are_features), C.byref(r))
    if rc != 0:
        raise MtxOracleError(rc, r.err.decode())
    try:
        ng, nnz = r.n_genes, r.nnz
        colptr = np.ctypeslib.as_array(r.colptr, (ng + 1,)).copy()
        rowidx = np.ctypeslib.as_array(r.rowidx, (max(nnz, 1),))[:nnz].copy()
        val = np.ctypeslib.as_array(r.val, (max(nnz, 1),))[:nnz].copy()
        return sp.csc_matrix((val, rowidx, colptr), shape=(r.n_cells, ng))
    finally:
        lib.mtx_oracle_free(C.byref(r))
