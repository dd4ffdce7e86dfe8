"""GPU parity: count upload (CSC -> device CSR), generator, normalize_cells
(src/normalize.jl:17-55) against the oracle and the reference tests' fixtures."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

G = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())


def _counts(O, n=700, g=900, seed=0, **kw):
    return O.synth_counts(n, g, -1.0, 1.5, depth=0.5, seed=seed, **kw)


def test_upload_builds_sorted_csr(sv, ctx, O):
    X = _counts(O)
    cm = sv.CountMatrix.from_csc(X, ctx)
    assert cm.shape == X.shape and cm.nnz == X.nnz
    back = cm.to_csc()
    assert np.array_equal(back.indptr, X.indptr) and np.array_equal(back.indices, X.indices)
    assert np.array_equal(back.data, X.data)
    R = cm.to_csr()
    ref = X.tocsr()
    ref.sort_indices()
    assert np.array_equal(R.indptr, ref.indptr)
    assert np.array_equal(R.indices, ref.indices)       # columns sorted within rows
    assert np.array_equal(R.data, ref.data)


def test_upload_julia_layout_one_based_int64(sv, ctx):
    # the 10 x 5 literal of test/test_input.jl:47-58 as Julia holds it
    X = sp.csc_matrix(np.array(G["scaling"]["counts"], dtype=np.int64))
    cm = sv.CountMatrix.upload(X.indptr.astype(np.int64) + 1, X.indices.astype(np.int64) + 1,
                               X.data.astype(np.int64), X.shape, index_base=1, ctx=ctx)
    assert (cm.to_csc() != X).nnz == 0


def test_upload_rejects_unsorted_and_out_of_range(sv, ctx):
    cp = np.array([0, 2, 3], dtype=np.int32)
    bad = np.array([1, 0, 2], dtype=np.int32)     # rows not increasing in column 0
    vals = np.array([1, 1, 1], dtype=np.int32)
    with pytest.raises(sv.SeveroGPUError, match="increasing"):
        sv.CountMatrix.upload(cp, bad, vals, (3, 2), ctx=ctx)
    oob = np.array([0, 5, 2], dtype=np.int32)
    with pytest.raises(sv.SeveroGPUError, match="range"):
        sv.CountMatrix.upload(cp, oob, vals, (3, 2), ctx=ctx)
    # the context stays usable
    ok = np.array([0, 1, 2], dtype=np.int32)
    assert sv.CountMatrix.upload(cp, ok, vals, (3, 2), ctx=ctx).nnz == 3


def test_long_rows_sorted(sv, ctx):
    """Rows longer than the shared-memory sort capacity take the global path."""
    rng = np.random.default_rng(4)
    n, g = 40, 20000
    dense_rows = rng.random((n, g)) < 0.5
    dense_rows[:5] = True   # rows of 20000 entries
    X = sp.csc_matrix(dense_rows.astype(np.int32) * rng.integers(1, 9, (n, g)).astype(np.int32))
    X.eliminate_zeros()
    cm = sv.CountMatrix.from_csc(X, ctx)
    R = cm.to_csr()
    ref = X.tocsr()
    ref.sort_indices()
    assert np.array_equal(R.indices, ref.indices) and np.array_equal(R.data, ref.data)


def test_empty_rows_and_columns(sv, ctx, O):
    X = _counts(O, 300, 400, seed=2).tolil()
    X[10, :] = 0
    X[:, 7] = 0
    X = sp.csc_matrix(X)
    X.eliminate_zeros()
    d = sv.normalize_cells(X, scale_factor=1e4, ctx=ctx)
    ref = O.normalize_cells(X, scale_factor=1e4)
    assert np.allclose(d.values_csc(), ref.data, rtol=1e-15, atol=0)
    assert d.cell_totals()[10] == 0


@pytest.mark.parametrize("method", ["relativecounts", "lognormalize"])
def test_normalize_golden(sv, ctx, method):
    # test/test_input.jl:45-75
    C_ = sp.csc_matrix(np.array(G["normalize"]["counts"], dtype=np.int64))
    Q = sv.normalize_cells(C_, method=method, ctx=ctx).to_csc()
    want = G["normalize"]["relative" if method == "relativecounts" else "log"]
    assert np.allclose(Q.toarray(), want, rtol=1e-15, atol=0)
    if method == "relativecounts":
        assert np.allclose(np.asarray(Q.sum(axis=1)).ravel(), 1.0)
        Q10 = sv.normalize_cells(C_, method="relativecounts", scale_factor=10.0, ctx=ctx).to_csc()
        assert np.allclose(Q10.toarray(), G["normalize"]["relative_sf10"], rtol=1e-15)
        assert np.allclose(np.asarray(Q10.sum(axis=1)).ravel(), 10.0)


@pytest.mark.parametrize("dtype,rtol", [("float64", 1e-15), ("float32", 1e-6)])
@pytest.mark.parametrize("method", ["relativecounts", "lognormalize"])
def test_normalize_random(sv, ctx, O, dtype, rtol, method):
    X = _counts(O, seed=11)
    d = sv.normalize_cells(X, method=method, scale_factor=1e4, dtype=dtype, ctx=ctx)
    ref = O.normalize_cells(X, method, 1e4, np.dtype(dtype))
    got = d.values_csc()
    assert got.dtype == np.dtype(dtype)
    assert np.allclose(got, ref.data, rtol=rtol, atol=0)
    # the CSR copy holds the same values in cell-major order
    R = d.counts.to_csr()
    Rv = sp.csr_matrix((d.values_csr(), R.indices, R.indptr), shape=X.shape)
    refr = ref.tocsr()
    refr.sort_indices()
    assert np.allclose(Rv.data, refr.data, rtol=rtol, atol=0)
    assert np.array_equal(d.cell_totals(), np.asarray(X.sum(axis=1)).ravel())


def test_normalize_bf16(sv, ctx, O):
    X = _counts(O, seed=12)
    d = sv.normalize_cells(X, scale_factor=1e4, dtype="bfloat16", ctx=ctx)
    ref32 = O.normalize_cells(X, "lognormalize", 1e4, np.float32).data
    want = O.round_bf16(ref32)
    got = d.values_csc()
    # FP32 log1p may differ by an ulp from numpy's, which can flip one BF16 rounding
    ulp = np.abs(want) * 2.0 ** -7
    assert np.all(np.abs(got - want) <= ulp)
    assert np.mean(got == want) > 0.999


def test_generator_copies_agree(sv, ctx):
    rng = np.random.default_rng(5)
    n, g = 3000, 2000
    mu = rng.lognormal(-1.2, 1.6, g)
    s = rng.lognormal(0, 0.3, n)
    cl = rng.integers(0, 4, n)
    lfc = np.where(rng.random((4, g)) < 0.05, rng.normal(0, 0.8, (4, g)), 0.0)
    cm = sv.CountMatrix.generate(n, g, mu, s, cl, lfc, depth=0.3, dispersion=0.2, seed=9, ctx=ctx)
    A = cm.to_csc()
    B = cm.to_csr()
    assert A.nnz == B.nnz > 0
    assert (A.tocsr() != B).nnz == 0
    # mean count per entry close to the model's mean (NB mean = depth*s*mu*fold)
    mean_model = 0.3 * np.outer(s, mu) * np.exp(lfc[cl])
    assert abs(A.sum() / mean_model.sum() - 1) < 0.02
