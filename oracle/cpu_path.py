"""Driver of the multi-threaded CPU restatement of the path (cpu_path.c) --
TEST INFRASTRUCTURE AND CPU BASELINE ONLY.

Only ``bench.py`` (its CPU-baseline leg and its reference arm), ``tests/`` and
``__graft_entry__.build()`` use this module; the product path never imports it.
``build()`` compiles cpu_path.c with gcc and OpenMP into ``oracle/_build/``.

``pipeline()`` runs normalize_cells -> scale_features -> irlba PCA -> kNN on a
count matrix with every host core: the C kernels for normalisation, scaling
and the CenteredMatrix products (FP64, src/normalize.jl:17-38,
src/scaling.jl:18-34,199-272), the oracle's numpy irlba (FP64 CGS2
reorthogonalisation, src/irlba.jl:47-75 defaults) driving them, Z = U diag(s)
(src/embedding.jl:67), and an approximate kNN of the reference's kind in C
(random-projection trees, ntables = 2 d as the reference's default, then one
neighbour-of-neighbour round; its recall against exact search is measured
and reported).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import time
from pathlib import Path

import numpy as np
import scipy.sparse as sp

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpu_path.c"
LIB = HERE / "_build" / "libcpu_path.so"

_lib = None
_P = C.c_void_p
_I64 = C.c_int64
_D = C.c_double


def build() -> Path:
    LIB.parent.mkdir(exist_ok=True)
    if not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        tmp = LIB.with_suffix(".tmp")
        subprocess.run(["gcc", "-O2", "-fopenmp", "-shared", "-fPIC", str(SRC), "-o", str(tmp), "-lm"],
                       check=True)
        tmp.replace(LIB)
    return LIB


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        lib.cp_generate_offsets.argtypes = [_I64, _I64, _P, _P, _P, _P, _D, _D, C.c_uint64, _P, C.c_int]
        lib.cp_generate_offsets.restype = _I64
        lib.cp_generate_fill.argtypes = [_I64, _I64, _P, _P, _P, _P, _D, _D, C.c_uint64, _P, _P, _P,
                                         C.c_int]
        lib.cp_generate_fill.restype = None
        lib.cp_normalize.argtypes = [_I64, _I64, _P, _P, _P, _D, C.c_int, _P, _P, C.c_int]
        lib.cp_normalize.restype = None
        lib.cp_scale.argtypes = [_I64, _P, _P, _P, _I64, _P, _D, _P, _P, _P, _P, _P, _P, C.c_int]
        lib.cp_scale.restype = None
        lib.cp_matvec.argtypes = [_I64, _I64, _P, _P, _P, _P, _P, _P, _P, C.c_int]
        lib.cp_matvec.restype = None
        lib.cp_rmatvec.argtypes = [_I64, _I64, _P, _P, _P, _P, _P, _P, C.c_int]
        lib.cp_rmatvec.restype = None
        lib.cp_cgs2.argtypes = [_I64, _I64, _P, _P, _P, C.c_int]
        lib.cp_cgs2.restype = None
        lib.cp_rotate.argtypes = [_I64, _I64, _I64, _P, _P, _P, C.c_int]
        lib.cp_rotate.restype = None
        lib.cp_knn.argtypes = [_I64, _I64, _P, _I64, _P, _P, C.c_int]
        lib.cp_knn.restype = None
        lib.cp_ann.argtypes = [_I64, _I64, _P, _I64, C.c_int, C.c_int, C.c_uint64, C.c_int, _P, _P,
                               C.c_int]
        lib.cp_ann.restype = None
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def threads() -> int:
    return os.cpu_count() or 1


def generate(n_cells, n_genes, mu_g, s_c, cluster=None, lfc=None, depth=1.0, dispersion=0.2,
             seed=0, nt=0):
    """Seeded NB counts (cells x genes CSC, Int32), the same model as the
    benchmark's device generator (a different random stream)."""
    lib = _load()
    nt = nt or threads()
    mu_g = np.ascontiguousarray(mu_g, np.float64)
    s_c = np.ascontiguousarray(s_c, np.float64)
    cl = None if cluster is None else np.ascontiguousarray(cluster, np.int32)
    lf = None if lfc is None else np.ascontiguousarray(lfc, np.float64)
    toff = np.zeros((nt, n_genes), np.int64)
    nnz = lib.cp_generate_offsets(n_cells, n_genes, _p(mu_g), _p(s_c), _p(cl), _p(lf), depth,
                                  dispersion, seed, _p(toff), nt)
    colptr = np.empty(n_genes + 1, np.int64)
    colptr[:-1] = toff[0]
    colptr[-1] = nnz
    rowidx = np.empty(nnz, np.int32)
    counts = np.empty(nnz, np.int32)
    lib.cp_generate_fill(n_cells, n_genes, _p(mu_g), _p(s_c), _p(cl), _p(lf), depth, dispersion, seed,
                         _p(toff), _p(rowidx), _p(counts), nt)
    return sp.csc_matrix((counts, rowidx, colptr), shape=(n_cells, n_genes))


class Centered:
    """The implicit CenteredMatrix B - 1 mu^T over the feature subset (FP64)."""

    def __init__(self, n_cells, hcolptr, hrow, hval, mu, nt):
        self.m, self.n = n_cells, len(mu)
        self.cp, self.row, self.val, self.mu = hcolptr, hrow, hval, mu
        self.nt = nt
        self.tmp = np.empty(nt * n_cells)
        self.lib = _load()

    def mul(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty(self.m)
        self.lib.cp_matvec(self.m, self.n, _p(self.cp), _p(self.row), _p(self.val), _p(self.mu), _p(x),
                           _p(y), _p(self.tmp), self.nt)
        return y

    def rmul(self, u):
        u = np.ascontiguousarray(u, np.float64)
        y = np.empty(self.n)
        self.lib.cp_rmatvec(self.m, self.n, _p(self.cp), _p(self.row), _p(self.val), _p(self.mu), _p(u),
                            _p(y), self.nt)
        return y


class BasisOps:
    """The irlba basis operations (CGS2, restart rotation) on all cores, for
    column-major bases: passed to the oracle's irlba."""

    def __init__(self, nt):
        self.nt = nt
        self.lib = _load()
        self.tmp = np.empty(nt * 1024)
        self.buf = np.empty(0)

    def cgs2(self, x, Q):
        j = Q.shape[1]
        if j == 0:
            return x
        assert Q.flags.f_contiguous
        x = np.ascontiguousarray(x, np.float64)
        if self.tmp.size < self.nt * j:
            self.tmp = np.empty(self.nt * j)
        self.lib.cp_cgs2(Q.shape[0], j, _p(Q), _p(x), _p(self.tmp), self.nt)
        return x

    def rotate(self, Q, M):
        assert Q.flags.f_contiguous
        n, w = Q.shape
        k = M.shape[1]
        M = np.asfortranarray(M, np.float64)
        if self.buf.size < n * k:
            self.buf = np.empty(n * k)
        self.lib.cp_rotate(n, w, k, _p(Q), _p(M), _p(self.buf), self.nt)


def normalize(X, scale_factor=1e4, log=True, nt=0):
    lib = _load()
    nt = nt or threads()
    X = sp.csc_matrix(X)
    cp = np.ascontiguousarray(X.indptr, np.int64)
    ri = np.ascontiguousarray(X.indices, np.int32)
    ct = np.ascontiguousarray(X.data, np.int32)
    vals = np.empty(X.nnz)
    tot = np.empty(X.shape[0], np.int64)
    lib.cp_normalize(X.shape[0], X.shape[1], _p(cp), _p(ri), _p(ct), scale_factor, int(log), _p(vals),
                     _p(tot), nt)
    return sp.csc_matrix((vals, ri, cp), shape=X.shape), tot


def scale(Xn, features, scale_max=10.0, nt=0):
    """features: 1-based gene indices.  Returns (Centered, mean, std)."""
    lib = _load()
    nt = nt or threads()
    cp = np.ascontiguousarray(Xn.indptr, np.int64)
    ri = np.ascontiguousarray(Xn.indices, np.int32)
    vals = np.ascontiguousarray(Xn.data, np.float64)
    f0 = np.ascontiguousarray(np.asarray(features, np.int64) - 1)
    nf = len(f0)
    nnz_h = int(np.sum(cp[f0 + 1] - cp[f0]))
    hcp = np.empty(nf + 1, np.int64)
    hrow = np.empty(nnz_h, np.int32)
    hval = np.empty(nnz_h)
    mu, mean, std = np.empty(nf), np.empty(nf), np.empty(nf)
    lib.cp_scale(Xn.shape[0], _p(cp), _p(ri), _p(vals), nf, _p(f0), scale_max, _p(hcp), _p(hrow),
                 _p(hval), _p(mu), _p(mean), _p(std), nt)
    return Centered(Xn.shape[0], hcp, hrow, hval, mu, nt), mean, std


def knn(Z, k, nt=0):
    """Exact Euclidean k nearest neighbours (self included, first), 0-based
    indices, by blocked brute force on all cores."""
    lib = _load()
    Z = np.ascontiguousarray(Z, np.float64)
    n, d = Z.shape
    idx = np.empty((n, k), np.int64)
    d2 = np.empty((n, k))
    lib.cp_knn(n, d, _p(Z), k, _p(idx), _p(d2), nt or threads())
    return idx


def ann(Z, k, ntables=None, leaf=64, refine=1, seed=0, nt=0):
    """Approximate k nearest neighbours (self first), 0-based: ntables random-
    projection trees (default 2 d, the reference's default number of tables)
    and one neighbour-of-neighbour round; the stand-in for the reference's
    native approximate search."""
    lib = _load()
    Z = np.ascontiguousarray(Z, np.float64)
    n, d = Z.shape
    idx = np.empty((n, k), np.int64)
    d2 = np.empty((n, k))
    lib.cp_ann(n, d, _p(Z), k, int(ntables or 2 * d), int(leaf), seed, int(refine), _p(idx), _p(d2),
               nt or threads())
    return idx


def pipeline(X, features, npcs=50, k=20, init=None, tol=1e-5, scale_factor=1e4, scale_max=10.0,
             nt=0, approx=True):
    """One pass of the path on the host; returns (stage seconds, Z, info with
    the irlba counts and the neighbour lists).  approx: the random-projection
    forest (the reference's kind of search), else exact brute force."""
    from oracle import severo_oracle as O
    nt = nt or threads()
    t = {}
    t0 = time.perf_counter()
    Xn, _ = normalize(X, scale_factor, True, nt)
    t["normalize"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    S, _, _ = scale(Xn, features, scale_max, nt)
    t["scale"] = time.perf_counter() - t0
    del Xn
    t0 = time.perf_counter()
    if init is None:
        init = np.random.default_rng(0).standard_normal(S.n)
    ops = BasisOps(nt)
    U, s, V, info, it, nmv = O.irlba(S.mul, S.rmul, S.m, S.n, npcs, tol=tol, init=init,
                                     cgs2=ops.cgs2, rotate=ops.rotate)
    Z = U * s                                                        # embedding.jl:67
    t["pca"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    idx = ann(Z, k, nt=nt) if approx else knn(Z, k, nt)
    t["knn"] = time.perf_counter() - t0
    return t, Z, {"iters": int(it), "nmatvec": int(nmv), "sigma": s, "idx": idx}


def recall(Z, idx, k, queries):
    """Fraction of the exact k nearest neighbours (self included) of the query
    rows found in idx."""
    Q = Z[queries]
    D = np.einsum("ij,ij->i", Q, Q)[:, None] + np.einsum("ij,ij->i", Z, Z)[None, :] - 2.0 * (Q @ Z.T)
    D[np.arange(len(queries)), queries] = -1.0
    ex = np.argpartition(D, k - 1, axis=1)[:, :k]
    return float(np.mean([len(set(ex[r]) & set(idx[q])) / k for r, q in enumerate(queries)]))


def run_sizes(params, sizes, nt=0, n_hvf=3000, npcs=50, k=20, seed=0):
    """The path on prefixes of one generated sample: cells 0..n-1 for every n
    in sizes (generation and the feature choice untimed).  params: mapping
    with mu_g, s_c (at least max(sizes) cells), cluster, lfc, depth,
    dispersion.  Returns one record per size: n, nnz, stage seconds, irlba
    iterations and products."""
    nt = nt or threads()
    N = max(sizes)
    cl = params.get("cluster")
    X = generate(N, len(params["mu_g"]), params["mu_g"], params["s_c"][:N],
                 None if cl is None else cl[:N], params.get("lfc"), float(params["depth"]),
                 float(params["dispersion"]), seed, nt)
    # the feature set: a precomputed input of the path (largest normalised variances)
    Xn, _ = normalize(X, 1e4, True, nt)
    m1 = np.asarray(Xn.mean(axis=0)).ravel()
    m2 = np.asarray(Xn.multiply(Xn).mean(axis=0)).ravel()
    hvf = np.sort(np.argsort(-(m2 - m1 * m1), kind="stable")[:n_hvf]) + 1
    del Xn
    Xr = sp.csr_matrix(X)
    del X
    init = np.random.default_rng(seed).standard_normal(len(hvf))
    out = []
    for n in sizes:
        Xs = sp.csc_matrix(Xr[:n])
        t, Z, info = pipeline(Xs, hvf, npcs, k, init=init, nt=nt)
        rec = {"n": int(n), "nnz": int(Xs.nnz), "stages_s": t, "iters": info["iters"],
               "nmatvec": info["nmatvec"]}
        if n == N and n > 1000:
            q = np.random.default_rng(seed + 1).choice(n, 500, replace=False)
            rec["knn_recall"] = recall(Z, info["idx"], k, q)
        out.append(rec)
        del Xs
    return out


def run_in_subprocess(params, sizes, nt=0, timeout=None, **kw):
    """run_sizes in a fresh interpreter whose BLAS is single-threaded, so that
    the OpenMP kernels own the cores (an idle multi-threaded BLAS spinning
    beside them made the irlba 7x slower)."""
    import json
    import sys
    import tempfile
    nt = nt or threads()
    with tempfile.TemporaryDirectory() as td:
        pf = Path(td) / "params.npz"
        np.savez(pf, **{k: v for k, v in params.items() if v is not None})
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS=str(nt), MKL_NUM_THREADS="1")
        cmd = [sys.executable, "-m", "oracle.cpu_path", str(pf), ",".join(str(int(s)) for s in sizes),
               str(nt), json.dumps(kw)]
        r = subprocess.run(cmd, cwd=str(HERE.parent), env=env, capture_output=True, text=True,
                           timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"CPU path failed: {r.stderr[-2000:]}")
        return json.loads(r.stdout.strip().splitlines()[-1])


if __name__ == "__main__":
    import json
    import sys
    pf, sizes, nt = sys.argv[1], [int(s) for s in sys.argv[2].split(",")], int(sys.argv[3])
    kw = json.loads(sys.argv[4]) if len(sys.argv) > 4 else {}
    z = np.load(pf)
    params = {k: z[k] for k in z.files}
    print(json.dumps(run_sizes(params, sizes, nt, **kw)))
