"""GPU parity: irlba (src/irlba.jl:47-99; the cases of test/test_irlba.jl:24-116)
through the drop-in `irlba` symbol (host matvec callbacks) and on the device
matrix; pca (src/embedding.jl:46-94) on the implicit scaled matrix."""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu


def _close(a, b, rtol):
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


def _relerr(X, U, s, V):
    return np.linalg.norm(X - (U * s) @ V.T)


@pytest.mark.parametrize("shape,nu,tol", [((50, 50), 20, 1e-5), ((100, 50), 20, 1e-5)])
def test_irlba_dense_callback(sv, shape, nu, tol):
    rng = np.random.default_rng(10)
    X = rng.standard_normal(shape)
    U, s, V = sv.irlba_callback(lambda x: X @ x, lambda y: X.T @ y, *shape, nu, tol=tol, seed=1)
    ss = np.linalg.svd(X, compute_uv=False)
    assert _close(s, ss[:nu], 1.5e-8)                                       # :29
    assert np.linalg.norm(X.T @ U - V * s) / np.linalg.norm(X) < tol        # :30
    Uf, sf, Vtf = np.linalg.svd(X)
    assert np.isclose(_relerr(X, U, s, V), _relerr(X, Uf[:, :nu], sf[:nu], Vtf[:nu].T), rtol=1.5e-8)


def test_irlba_sparse_callback(sv):
    X = sp.random(2000, 400, density=0.1, random_state=11, format="csc")
    U, s, V = sv.irlba_callback(lambda x: X @ x, lambda y: X.T @ y, 2000, 400, 2, tol=1e-9)
    ss = np.linalg.svd(X.toarray(), compute_uv=False)
    assert _close(s, ss[:2], 1.5e-8)
    assert np.linalg.norm(X.T @ U - V * s) / sp.linalg.norm(X) < 1e-9       # :49


def test_irlba_tall_skinny_vs_transpose(sv, O):
    # test/test_irlba.jl:93-105
    X = np.random.default_rng(12).standard_normal((10000, 10))
    U1, s1, V1 = sv.irlba_callback(lambda x: X @ x, lambda y: X.T @ y, 10000, 10, 2, tol=1e-9)
    U1, V1 = O.svd_flip(U1, V1, u_based=True)
    U2, s2, V2 = sv.irlba_callback(lambda x: X.T @ x, lambda y: X @ y, 10, 10000, 2, tol=1e-9)
    U2, V2 = O.svd_flip(U2, V2, u_based=False)
    assert _close(s1, s2, 1.5e-8)
    assert np.allclose(U1, V2, atol=1e-7) and np.allclose(V1, U2, atol=1e-7)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_irlba_centered_sparse_device(sv, ctx, dtype):
    # test/test_irlba.jl:79-91 with the CenteredMatrix on the device
    X = sp.random(2000, 400, density=0.1, random_state=13, format="csc")
    mu = np.asarray(X.mean(axis=0)).ravel()
    S = sv.CenteredMatrix.from_sparse(X, mu, dtype=dtype, ctx=ctx)
    U, s, V = sv.irlba(S, 2, tol=1e-9, seed=3)
    Q = X.toarray() - mu
    ss = np.linalg.svd(Q, compute_uv=False)
    if dtype == "float64":
        assert _close(s, ss[:2], 1.5e-8)
        assert np.linalg.norm(Q.T @ U - V * s) / np.linalg.norm(Q) < 1e-9
    else:
        # values stored in FP32, products accumulated in FP32
        assert np.max(np.abs(s - ss[:2]) / ss[:2]) < 1e-5


def test_irlba_centered_dense_small(sv, ctx):
    # test/test_irlba.jl:65-77 (20 x 10, nu = 3: work = min(m, n) = 10)
    X = np.random.default_rng(14).standard_normal((20, 10))
    mu = X.mean(axis=0)
    S = sv.CenteredMatrix.from_sparse(sp.csc_matrix(X), mu, ctx=ctx)
    U, s, V = sv.irlba(S, 3, seed=4)
    Q = X - mu
    ss = np.linalg.svd(Q, compute_uv=False)
    assert _close(s, ss[:3], 1.5e-8)
    assert np.linalg.norm(Q.T @ U - V * s) / np.linalg.norm(Q) < 1e-9


def test_irlba_count_matrix(sv, ctx):
    # test/test_irlba.jl:107-115: Poisson(10) counts, CenteredMatrix(X', mu)
    rng = np.random.default_rng(15)
    X = sp.random(3000, 10000, density=0.01, random_state=16, format="csr",
                  data_rvs=lambda k: rng.poisson(10, k).astype(float))
    mu = np.asarray(X.mean(axis=1)).ravel()
    A = sp.csc_matrix(X.T)
    S = sv.CenteredMatrix.from_sparse(A, mu, ctx=ctx)
    U, s, V = sv.irlba(S, 10, seed=5)
    ss = np.linalg.svd(A.toarray() - mu, compute_uv=False)
    assert _close(s, ss[:10], 1.5e-8)


def test_irlba_nonconvergence_reported(sv, ctx):
    X = sp.random(500, 300, density=0.2, random_state=17, format="csc")
    S = sv.CenteredMatrix.from_sparse(X, np.zeros(300), ctx=ctx)
    with pytest.raises(sv.ConvergenceError):
        sv.irlba(S, 20, tol=1e-14, maxit=1)
    # the context remains usable after the failure
    U, s, V = sv.irlba(S, 2, tol=1e-8)
    assert s[0] > s[1] > 0


@pytest.mark.parametrize("dtype,tol_s", [("float64", 1e-9), ("float32", 1e-5), ("bfloat16", 1e-5)])
def test_pca_pipeline(sv, ctx, O, dtype, tol_s):
    X = O.synth_counts(3000, 1500, -1.2, 1.6, depth=0.3, seed=31, n_clusters=6)
    d = sv.normalize_cells(X, scale_factor=1e4, dtype=dtype, ctx=ctx)
    if dtype == "bfloat16":
        ref = O.normalize_cells(X, scale_factor=1e4, dtype=np.float64)
        ref.data = d.values_csc().astype(np.float64)
    else:
        ref = O.normalize_cells(X, scale_factor=1e4, dtype=np.dtype(dtype)).astype(np.float64)
    hvf = O.top_variable_genes(ref, 400)
    S = sv.scale_features(d, scale_max=10.0, features=hvf)
    init = np.random.default_rng(2).standard_normal(400)
    em = sv.pca(S, 20, tol=1e-7, init=init)
    Sr, _, _ = O.scale_features(ref, 10.0, np.float64, hvf)
    Q = Sr.dense()
    Uf, sf, Vtf = np.linalg.svd(Q, full_matrices=False)
    s = em.stdev * np.sqrt(3000 - 1)                              # embedding.jl:68
    rel = np.max(np.abs(s - sf[:20]) / sf[:20])
    assert rel < tol_s, rel
    # Loadings: with tol = 1e-7 the residual of each Ritz pair is at most
    # 1e-7 sigma_1, so a PC whose singular value lies at least 1e-3 sigma_1
    # from its neighbours is within ~1e-4 rad of the exact one; the leading
    # block ending at the widest gap is compared as a subspace.
    d_next = (sf[:20] - sf[1:21]) / sf[0]                 # gap below PC i
    d_prev = np.r_[np.inf, d_next[:-1]]                   # gap above PC i
    sep = np.minimum(d_prev, d_next) >= 1e-3
    assert sep.sum() >= 3, sep
    per_pc = np.arccos(np.clip(np.abs(np.einsum("ij,ji->i", em.basis.T, Vtf[:20].T)), 0.0, 1.0))
    assert per_pc[sep].max() < 1e-4, per_pc
    kk = int(np.argmax(d_next[1:19])) + 2                 # leading block (>= 2 PCs), widest gap
    assert d_next[kk - 1] >= 1e-2, (kk, d_next)
    ang = O.principal_angles(em.basis[:, :kk], Vtf[:kk].T).max()
    assert ang < 1e-4, (kk, ang)
    # coordinates are U diag(s) (embedding.jl:67): Z equals X~ times the loadings
    Z_ref = Q @ em.basis
    zt = 1e-9 if dtype == "float64" else 1e-5
    assert np.linalg.norm(em.coordinates - Z_ref) <= zt * np.linalg.norm(Z_ref)
    assert np.allclose(np.abs(em.coordinates.T @ em.coordinates), np.diag(s ** 2), rtol=1e-6,
                       atol=1e-6 * s[0] ** 2)


@pytest.mark.parametrize("rank", [None, 4])
def test_irlba_graph_replay_matches_direct_launches(sv, ctx, monkeypatch, rank):
    """Each Lanczos cycle over a device matrix is captured once as a CUDA graph
    and replayed; the replay issues the same kernels in the same order as direct
    launches, so the results agree bit for bit (rank 4 < work also exercises the
    breakdown restarts inside the graph)."""
    rng = np.random.default_rng(18)
    if rank is None:
        X = sp.random(5000, 600, density=0.05, random_state=19, format="csc")
    else:
        X = sp.csc_matrix(rng.standard_normal((5000, rank)) @ rng.standard_normal((rank, 600)))
    mu = np.asarray(X.mean(axis=0)).ravel()
    S = sv.CenteredMatrix.from_sparse(X, mu, dtype="float32", ctx=ctx)
    nu = 3
    out = {}
    for mode in ("graph", "direct"):
        if mode == "direct":
            monkeypatch.setenv("SV_NO_GRAPH", "1")
        else:
            monkeypatch.delenv("SV_NO_GRAPH", raising=False)
        l0 = ctx.launches()
        U, s, V, info = sv.irlba(S, nu, tol=1e-8, seed=6, return_info=True)
        out[mode] = (U, s, V, info, ctx.launches() - l0)
    Ug, sg, Vg, ig, lg = out["graph"]
    Ud, sd, Vd, idd, ld = out["direct"]
    assert ig == idd and lg == ld
    assert np.array_equal(sg, sd) and np.array_equal(Ug, Ud) and np.array_equal(Vg, Vd)
    ss = np.linalg.svd(X.toarray() - mu, compute_uv=False)
    assert np.max(np.abs(sg - ss[:nu]) / ss[:nu]) < 1e-5
    if rank is None:
        assert ig["iters"] > 2   # several replays of the restart graphs


def test_feature_side_paths_agree(sv, ctx, O, monkeypatch):
    """The feature-side step in one block per sample (k_vside) and through the
    multi-block CGS kernels give the same embedding (reduction order only)."""
    X = O.synth_counts(3000, 1500, -1.2, 1.6, depth=0.3, seed=33, n_clusters=5)
    d = sv.normalize_cells(X, scale_factor=1e4, dtype="float32", ctx=ctx)
    ref = O.normalize_cells(X, scale_factor=1e4, dtype=np.float32).astype(np.float64)
    hvf = O.top_variable_genes(ref, 400)
    S = sv.scale_features(d, scale_max=10.0, features=hvf)
    init = np.random.default_rng(5).standard_normal(400)
    out = {}
    for mode in ("block", "multi"):
        monkeypatch.setenv("SV_VSIDE", mode)
        out[mode] = sv.pca(S, 10, tol=1e-8, init=init).stdev
    assert np.max(np.abs(out["block"] - out["multi"]) / out["block"]) < 1e-7


def test_caller_provided_outputs(sv, ctx, O):
    """pca(out=Z) and ann(out=(idx, dist)) fill the caller's column-major arrays
    with the same results as freshly allocated ones; wrong shapes are refused."""
    X = O.synth_counts(2500, 1200, -1.2, 1.6, depth=0.3, seed=5, n_clusters=5)
    d = sv.normalize_cells(X, scale_factor=1e4, dtype="float32", ctx=ctx)
    S = sv.scale_features(d, scale_max=10.0, features=np.arange(1, 301))
    init = np.random.default_rng(3).standard_normal(300)
    em = sv.pca(S, 12, tol=1e-8, init=init)
    Z = np.full((2500, 12), np.nan, order="F")
    em2 = sv.pca(S, 12, tol=1e-8, init=init, out=Z)
    assert em2.coordinates is Z and np.array_equal(Z, em.coordinates)
    idx, dist = sv.ann(em, 10, ctx=ctx)
    oi = np.zeros((2500, 10), dtype=np.int32, order="F")
    od = np.zeros((2500, 10), dtype=np.float64, order="F")
    i2, d2 = sv.ann(em2, 10, ctx=ctx, out=(oi, od))
    assert i2 is oi and d2 is od
    assert np.array_equal(oi, idx) and np.array_equal(od, dist)
    with pytest.raises(ValueError):
        sv.pca(S, 12, tol=1e-8, init=init, out=np.zeros((2500, 12)))   # row-major
