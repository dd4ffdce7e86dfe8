"""GPU parity: exact kNN (replacing the ANN of src/neighbours.jl:19-74; the
cases of test/test_nn.jl:21-96) against the FP64 brute-force oracle."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check_sets(idx1, X, k, include_self, metric, tie_rtol=1e-5, O=None):
    """Index sets equal to the FP64 oracle's except for distance ties within tie_rtol."""
    ridx, rdist = O.knn_exact(X, k, include_self, metric)
    Xd = np.asarray(X, dtype=np.float64)
    if metric == "cosine":
        Xd = Xd / np.linalg.norm(Xd, axis=1, keepdims=True)
    bad = 0
    for i in range(X.shape[0]):
        a = set(idx1[i] - 1)
        b = set(ridx[i])
        if a == b:
            continue
        kth = np.sum((Xd[i] - Xd[ridx[i, -1]]) ** 2)
        for j in a - b:
            dj = np.sum((Xd[i] - Xd[j]) ** 2)
            if abs(dj - kth) > tie_rtol * max(kth, 1e-30):
                bad += 1
    return bad


@pytest.mark.parametrize("metric", ["euclidean", "cosine"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_knn_small_like_reference(sv, ctx, O, metric, dtype):
    # test/test_nn.jl:23-57: 100 x 10 uniform data, k = 4
    X = np.random.default_rng(0).random((100, 10)).astype(dtype)
    idx, dist = sv.ann(X, 4, metric=metric, ctx=ctx)
    assert idx.dtype == np.int32 and dist.dtype == dtype            # :29, :84-93
    assert _check_sets(idx, X, 4, True, metric, O=O) == 0
    assert np.all(idx[:, 0] == np.arange(1, 101))                    # self first
    ridx, rdist = O.knn_exact(X, 4, True, metric)
    assert np.allclose(dist, rdist, rtol=1e-5, atol=1e-6)


def test_knn_view_and_exclude_self(sv, ctx, O):
    # test/test_nn.jl:59-76 (a column view) and include_self = false
    X = np.random.default_rng(1).random((300, 20))
    Z = X[:, :10]
    idx, _ = sv.ann(Z, 7, include_self=False, ctx=ctx)
    assert not np.any(idx == np.arange(1, 301)[:, None])
    assert _check_sets(idx, Z, 7, False, "euclidean", O=O) == 0


@pytest.mark.parametrize("d", [3, 16, 50, 64])
def test_knn_dims(sv, ctx, O, d):
    X = np.random.default_rng(d).standard_normal((2500, d))
    idx, _ = sv.ann(X, 20, ctx=ctx)
    assert _check_sets(idx, X, 20, True, "euclidean", O=O) == 0


def test_knn_k30_gmm(sv, ctx, O):
    rng = np.random.default_rng(7)
    means = rng.normal(0, 4, (12, 50))
    lab = rng.integers(0, 12, 4000)
    X = means[lab] + rng.standard_normal((4000, 50)) / np.sqrt(np.arange(1, 51))
    idx, _ = sv.ann(X.astype(np.float32), 30, ctx=ctx)
    assert _check_sets(idx, X.astype(np.float32), 30, True, "euclidean", O=O) == 0


def test_knn_duplicates_ties_by_index(sv, ctx):
    X = np.repeat(np.arange(10.0)[:, None], 3, axis=0).reshape(30, 1) @ np.ones((1, 4))
    idx, dist = sv.ann(X, 3, ctx=ctx)
    # each point has two exact duplicates: self first, then the duplicates by index
    for i in range(30):
        grp = set(np.where((X == X[i]).all(axis=1))[0] + 1)
        assert set(idx[i]) == grp and idx[i, 0] == i + 1
        assert np.all(dist[i] == 0)


@pytest.mark.parametrize("name,dt", [("FindNeighboursEuclidean64", np.float64),
                                     ("FindNeighboursEuclidean32", np.float32),
                                     ("FindNeighboursCosine64", np.float64),
                                     ("FindNeighboursCosine32", np.float32)])
def test_findneighbours_dropins(sv, O, name, dt):
    """The libcell symbols with the reference's ccall layout (column-major, ldX)."""
    lib = sv._lib.load()
    n, d, k, ld = 400, 12, 6, 450
    Xfull = np.asfortranarray(np.random.default_rng(3).random((ld, 2 * d)).astype(dt))
    idx = np.zeros((n, k), dtype=np.int32, order="F")
    dist = np.zeros((n, k), dtype=dt, order="F")
    getattr(lib, name)(Xfull.ctypes.data_as(C.c_void_p), n, d, ld, k, 2 * d, 1, 1234,
                       idx.ctypes.data_as(C.c_void_p), dist.ctypes.data_as(C.c_void_p))
    X = Xfull[:n, :d]
    metric = "cosine" if "Cosine" in name else "euclidean"
    assert _check_sets(idx, X, k, True, metric, O=O) == 0


def _recall(idx1, X, k, include_self, metric, O):
    ridx, _ = O.knn_exact(X, k, include_self, metric)
    hits = sum(len(set(a - 1) & set(b)) for a, b in zip(idx1, ridx))
    return hits / ridx.size


@pytest.mark.parametrize("n,d,k", [(100, 10, 4), (300, 50, 20), (1000, 50, 20), (4099, 37, 30),
                                   (2600, 64, 16)])
def test_knn_bf16_tensor_cores(sv, ctx, O, n, d, k):
    """BF16 tcgen05 candidates + FP32 exact re-rank: recall against FP64 exact."""
    rng = np.random.default_rng(n + d)
    means = rng.normal(0, 4, (20, d))
    X = means[rng.integers(0, 20, n)] + rng.standard_normal((n, d)) / np.sqrt(np.arange(1, d + 1))
    X = X.astype(np.float32)
    idx, dist = sv.ann(X, k, precision="bf16", ctx=ctx)
    assert np.all(idx[:, 0] == np.arange(1, n + 1))
    assert _recall(idx, X, k, True, "euclidean", O) >= 0.999
    # results agree with the FP32 path except for near-ties
    assert _check_sets(idx, X, k, True, "euclidean", tie_rtol=1e-4, O=O) <= 0.001 * n * k


def test_knn_bf16_exclude_self_and_cosine(sv, ctx, O):
    rng = np.random.default_rng(9)
    X = rng.standard_normal((1500, 24)).astype(np.float32)
    idx, _ = sv.ann(X, 10, include_self=False, precision="bf16", ctx=ctx)
    assert not np.any(idx == np.arange(1, 1501)[:, None])
    assert _recall(idx, X, 10, False, "euclidean", O) >= 0.999
    idx, _ = sv.ann(X, 10, metric="cosine", precision="bf16", ctx=ctx)
    assert _recall(idx, X, 10, True, "cosine", O) >= 0.999


def test_knn_bad_k(sv, ctx):
    with pytest.raises(sv.SeveroGPUError):
        sv.ann(np.zeros((5, 3)), 6, ctx=ctx)


def gmm_points(n, d, ncomp, seed):
    """n points of a ncomp-component Gaussian mixture in d dimensions: means
    ~ N(0, 4^2), unit noise, dimension i scaled by 1/sqrt(i)."""
    rng = np.random.default_rng(seed)
    means = rng.normal(0, 4, (ncomp, d))
    X = means[rng.integers(0, ncomp, n)]
    X += rng.standard_normal((n, d))
    X *= 1.0 / np.sqrt(np.arange(1, d + 1))
    return X.astype(np.float32)


def test_knn_stress_2m_bf16_recall(sv, ctx, O):
    """2,000,000 x 50 FP32 points (60-component mixture), k = 30: BF16 tensor-core
    candidates (64 per point) with the FP32 re-rank against FP64 brute force on
    500 sampled queries; recall@30 >= 0.999."""
    n, d, k = 2_000_000, 50, 30
    X = gmm_points(n, d, 60, 20261205)
    idx, dist = sv.ann(X, k, precision="bf16", ctx=ctx)
    q = np.random.default_rng(5).choice(n, 500, replace=False)
    ref = O.knn_exact_queries(X, q, k)
    hits = sum(len(set(a - 1) & set(b)) for a, b in zip(idx[q], ref))
    assert hits / ref.size >= 0.999, hits / ref.size
    assert np.all(idx[q, 0] == q + 1)
    assert np.all(np.diff(dist[q], axis=1) >= 0)


def test_bounded_wait_runs_out_and_context_survives(sv, ctx, O):
    """The bounded mbarrier wait of the tensor-core kernel, made to run out on
    a barrier that nothing completes (a limit of 10^5 cycles): the call reports
    SV_ERR_DEVICE through the status word, and the context keeps working."""
    lib = sv._lib.load()
    st = lib.sv_selftest_wait_timeout(ctx.h, 100000)
    assert st == sv._lib.SV_ERR_DEVICE
    assert "iteration limit" in sv._lib.last_error()
    X = np.random.default_rng(9).standard_normal((2000, 16))
    idx, _ = sv.ann(X, 5, precision="bf16", ctx=ctx)
    assert _check_sets(idx, X, 5, True, "euclidean", O=O) == 0
