"""GPU parity: filter_counts / filter_cells / filter_features
(src/filtering.jl:15-35,98-103) against the oracle, bit for bit."""
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

G = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())


def _same(A, B):
    A = sp.csc_matrix(A)
    B = sp.csc_matrix(B)
    assert A.shape == B.shape
    assert np.array_equal(A.indptr, B.indptr)
    assert np.array_equal(A.indices, B.indices)
    assert np.array_equal(A.data, B.data)


def test_filter_golden(sv, ctx):
    # test/test_input.jl:24-42
    f = G["filter"]
    X = sp.csc_matrix(np.array(f["counts"], dtype=np.int64))
    C = sv.CountMatrix.from_csc(X, ctx=ctx)
    D, ci, fi = sv.filter_counts(C, min_features=f["min_features"], min_cells=f["min_cells"],
                                 min_umi=f["min_umi"])
    assert D.shape == (7, 4)
    assert list(np.nonzero(ci)[0] + 1) == f["cells"]
    assert list(np.nonzero(fi)[0] + 1) == f["genes"]
    assert np.array_equal(D.to_csc().toarray(), np.array(f["filtered"]))
    # the CSR copy is rebuilt consistently
    _same(D.to_csr().tocsc(), D.to_csc())


def test_filter_no_thresholds_keeps_everything(sv, ctx):
    # test/test_input.jl:20-22 (sprand 100 x 10, Poisson(4) values)
    rng = np.random.default_rng(3)
    X = sp.random(100, 10, density=0.1, random_state=4, format="csc",
                  data_rvs=lambda k: rng.poisson(4, k).astype(float)).astype(np.int64)
    C = sv.CountMatrix.from_csc(X, ctx=ctx)
    D, ci, fi = sv.filter_counts(C)
    assert D.shape == (100, 10) and ci.all() and fi.all()
    _same(D.to_csc(), C.to_csc())


@pytest.mark.parametrize("kw", [
    dict(min_cells=3, min_features=20, min_feature_count=0, min_umi=0),
    dict(min_cells=10, min_features=5, min_feature_count=2, min_umi=150),
    dict(min_cells=0, min_features=790, min_feature_count=-1, min_umi=0),
    dict(min_cells=50, min_features=0, min_feature_count=0, min_umi=400),
    dict(min_cells=0, min_features=100000, min_feature_count=0, min_umi=0),   # nothing left
])
def test_filter_counts_matches_oracle(sv, ctx, O, kw):
    X = O.synth_counts(3000, 800, -1.0, 1.5, depth=0.4, seed=41, n_clusters=4)
    C = sv.CountMatrix.from_csc(X, ctx=ctx)
    D, ci, fi = sv.filter_counts(C, **kw)
    R, rci, rfi = O.filter_counts(X, **kw)
    assert np.array_equal(ci, rci) and np.array_equal(fi, rfi)
    assert D.shape == R.shape
    _same(D.to_csc(), R)
    if D.nnz:
        _same(D.to_csr().tocsc(), R)


def test_filter_cells_and_features_wrappers(sv, ctx, O):
    X = O.synth_counts(1500, 400, -1.0, 1.5, depth=0.4, seed=42)
    # explicit stored zeros: copied, but not counted as detected
    X = sp.csc_matrix(X)
    X.data[::7] = 0
    C = sv.CountMatrix.from_csc(X, ctx=ctx)
    D, ci = sv.filter_cells(C, min_features=30, min_feature_count=1)
    R, rci = O.filter_cells(X, min_features=30, min_feature_count=1)
    assert np.array_equal(ci, rci)
    _same(D.to_csc(), R)
    D, fi = sv.filter_features(C, min_cells=40)
    R, rfi = O.filter_features(X, min_cells=40)
    assert np.array_equal(fi, rfi)
    _same(D.to_csc(), R)


def test_select_cells_is_a_row_slice(sv, ctx, O):
    X = O.synth_counts(700, 300, -1.0, 1.5, depth=0.5, seed=43)
    C = sv.CountMatrix.from_csc(X, ctx=ctx)
    D = C.select_cells(120, 455)
    R = sp.csc_matrix(sp.csr_matrix(X)[120:455])
    _same(D.to_csc(), R)
    _same(D.to_csr().tocsc(), R)
