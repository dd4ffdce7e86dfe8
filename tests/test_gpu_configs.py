"""GPU parity at the two configurations the reference's CPU path can run, each
checked end to end against the oracle at its stated shape.

C1, the small case: 2,000 cells x 20,000 genes of negative-binomial counts
(gene means LogNormal(-1, 1.5), cell sizes LogNormal(0, 0.3), dispersion 0.2,
~1,000 non-zeros per cell), 2,000 vst features, everything in FP64 as the
reference's default dtype: normalize_cells (log1p, scale 1e4) -> scale_features
(clip 10) -> irlba 50 at the default tol 1e-5 -> kNN 20 -> SNN (prune 1/15).

C2, plain FP32: 100,000 cells x 33,538 genes (gene means LogNormal(-1.2, 1.6),
~2,500 non-zeros per cell) generated on the device, FP32 values, 3,000 vst
features, irlba 50 (FP64-class reorthogonalisation), exact FP32 kNN 20 + SNN.
The singular values and loadings are checked against the eigendecomposition
of the FP64 Gram matrix of the oracle's scaled matrix, the neighbour lists of
2,000 sampled cells against FP64 brute force, and the whole SNN graph bit for
bit.

Bounds: normalised values 1e-15 (FP64) / 1e-6 (FP32) relative; singular values
1e-5 relative; every PC whose singular value lies at least 1e-3 sigma_1 from
both neighbours within 1e-4 rad; kNN sets identical except for distance ties
within 1e-5 relative; SNN bit-exact given the same neighbour lists
(src/normalize.jl:17-38, src/scaling.jl:18-34,199-272, src/irlba.jl:47-75,
src/embedding.jl:46-76, src/neighbours.jl:76-108)."""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

SEP = 1e-3


def _separated(sf, npcs):
    d_next = (sf[:npcs] - sf[1:npcs + 1]) / sf[0]
    d_prev = np.r_[np.inf, d_next[:-1]]
    return np.minimum(d_prev, d_next) >= SEP


def _pc_angles(V, Vref):
    return np.arccos(np.clip(np.abs(np.einsum("ij,ij->j", V, Vref[:, :V.shape[1]])), 0.0, 1.0))


def _exact_queries(Z, q, k):
    """Exact FP64 Euclidean neighbours of the rows q of Z (self included),
    with the distance of each returned neighbour."""
    Q = Z[q]
    D = np.einsum("ij,ij->i", Q, Q)[:, None] + np.einsum("ij,ij->i", Z, Z)[None, :] - 2.0 * (Q @ Z.T)
    D[np.arange(len(q)), q] = -1.0
    part = np.argpartition(D, k - 1, axis=1)[:, :k]
    return part, D


def _knn_mismatches(idx, Z, q, k, tie_rtol=1e-5):
    """Neighbours of the sampled cells that differ from the exact sets by more
    than a distance tie within tie_rtol (relative to the k-th distance)."""
    bad = 0
    for c0 in range(0, len(q), 200):
        qc = q[c0:c0 + 200]
        part, D = _exact_queries(Z, qc, k)
        for r, i in enumerate(qc):
            a = set(idx[i] - 1)
            b = set(part[r])
            if a == b:
                continue
            kth = np.max(D[r, part[r]])
            for j in a - b:
                if abs(D[r, j] - kth) > tie_rtol * max(abs(kth), 1e-30):
                    bad += 1
    return bad


def _same(A, B):
    return (A.shape == B.shape and np.array_equal(A.indptr, B.indptr)
            and np.array_equal(A.indices, B.indices) and np.array_equal(A.data, B.data))


def test_config_small_fp64(sv, ctx, O):
    n, ng, npcs, k = 2000, 20000, 50, 20
    X = O.synth_counts(n, ng, -1.0, 1.5, depth=0.053, seed=20261204)
    assert 900 < X.nnz / n < 1200
    counts = sv.CountMatrix.from_csc(X, ctx)
    hvf, _ = sv.find_variable_features(counts, 2000)
    d = sv.normalize_cells(counts, scale_factor=1e4, dtype="float64", ctx=ctx)
    ref = O.normalize_cells(X, "lognormalize", 1e4, np.float64)
    assert np.allclose(d.values_csc(), ref.data, rtol=1e-15, atol=0)
    S = sv.scale_features(d, scale_max=10.0, features=hvf)
    Sr, mean, std = O.scale_features(ref, 10.0, np.float64, hvf)
    _, gm, gs = S.stats()
    assert np.allclose(gm, mean, rtol=1e-13) and np.allclose(gs, std, rtol=1e-13)
    Q = Sr.dense()
    _, sf, Vtf = np.linalg.svd(Q, full_matrices=False)
    init = np.random.default_rng(1).standard_normal(len(hvf))
    em = sv.pca(S, npcs, tol=1e-5, init=init)                      # the reference default tol
    s = em.stdev * np.sqrt(n - 1)                                   # embedding.jl:68
    assert np.max(np.abs(s - sf[:npcs]) / sf[:npcs]) < 1e-5
    U = em.coordinates / s                                          # embedding.jl:67
    assert np.linalg.norm(Q.T @ U - em.basis * s) / np.linalg.norm(Q) < 1e-5   # test_irlba.jl:30
    sep = _separated(sf, npcs)
    assert sep.sum() >= 2
    assert _pc_angles(em.basis, Vtf.T)[sep].max() < 1e-4
    # kNN 20 on the coordinates (exact FP32 candidates + FP32 re-rank)
    idx, dist = sv.ann(em, k, precision="fp32", ctx=ctx)
    Z = np.ascontiguousarray(em.coordinates)
    assert _knn_mismatches(idx, Z, np.arange(n), k) == 0
    # SNN: bit-exact against the oracle on the same lists, and the device pipeline agrees
    W = sv.jaccard_index(idx, k, prune=1 / 15, dtype=np.float64, ctx=ctx)
    R = O.jaccard_index(O.knn_graph(idx, n), k, 1 / 15, np.float64)
    assert _same(W, R)
    W2 = sv.shared_nearest_neighbours(em, k, prune=1 / 15, ctx=ctx)
    assert _same(W2, W)


def _gram_eigh(Sr, npcs):
    """Singular values, right singular vectors and Frobenius norm of the
    oracle's centred, scaled matrix X~ = B - 1 mu^T from the FP64 Gram matrix
    X~^T X~ = B^T B - c mu^T - mu c^T + n mu mu^T (c = B^T 1), B^T B summed
    over dense row blocks."""
    B = sp.csr_matrix(Sr.A)
    n, m = B.shape
    mu = np.asarray(Sr.mu, dtype=np.float64)
    G = np.zeros((m, m))
    for r0 in range(0, n, 10000):
        Bd = B[r0:r0 + 10000].toarray()
        G += Bd.T @ Bd
    c = np.asarray(B.sum(axis=0)).ravel()
    G -= np.outer(c, mu) + np.outer(mu, c) - n * np.outer(mu, mu)
    lam, W = np.linalg.eigh(G)
    order = np.argsort(-lam)[:npcs + 1]
    return np.sqrt(np.maximum(lam[order], 0.0)), W[:, order], np.sqrt(np.trace(G))


def test_config_plain_fp32_100k(sv, ctx, O):
    n, ng, npcs, k = 100_000, 33_538, 50, 20
    rng = np.random.default_rng(20261205)
    mu_g = rng.lognormal(-1.2, 1.6, ng)
    s_c = rng.lognormal(0.0, 0.3, n)
    counts = sv.CountMatrix.generate(n, ng, mu_g, s_c, depth=0.09, dispersion=0.2, seed=20261205,
                                     ctx=ctx)
    X = counts.to_csc()
    assert 2000 < X.nnz / n < 3000
    hvf, _ = sv.find_variable_features(counts, 3000)
    d = sv.normalize_cells(counts, scale_factor=1e4, dtype="float32", ctx=ctx)
    ref = O.normalize_cells(X, "lognormalize", 1e4, np.float32)
    got = d.values_csc()
    assert np.allclose(got, ref.data, rtol=1e-6, atol=0)
    ref.data = got                                                  # the values the device holds
    S = sv.scale_features(d, scale_max=10.0, features=hvf)
    Sr, _, _ = O.scale_features(ref, 10.0, np.float64, hvf, acc=np.float64)
    sref, Vref, fro = _gram_eigh(Sr, npcs)
    init = np.random.default_rng(2).standard_normal(len(hvf))
    em = sv.pca(S, npcs, tol=1e-5, init=init)
    s = em.stdev * np.sqrt(n - 1)
    assert np.max(np.abs(s - sref[:npcs]) / sref[:npcs]) < 1e-5
    # Ritz residual of every pair (test/test_irlba.jl:30): X~' U - V S, U = Z / s
    U = em.coordinates / s
    R = Sr.rmul(U) - em.basis * s
    assert np.linalg.norm(R) / fro < 1e-5
    # without clusters only the leading PCs stand clear of the noise bulk
    sep = _separated(sref, npcs)
    assert sep.sum() >= 1
    assert _pc_angles(em.basis, Vref)[sep].max() < 1e-4
    # exact FP32 kNN: 2,000 sampled cells against FP64 brute force on the coordinates
    idx, _ = sv.ann(em, k, precision="fp32", ctx=ctx)
    Z = np.ascontiguousarray(em.coordinates)
    q = np.random.default_rng(3).choice(n, 2000, replace=False)
    assert _knn_mismatches(idx, Z, q, k) == 0
    # the whole SNN graph, bit for bit
    W = sv.jaccard_index(idx, k, prune=1 / 15, dtype=np.float64, ctx=ctx)
    R = O.jaccard_index(O.knn_graph(idx, n), k, 1 / 15, np.float64)
    assert _same(W, R)
