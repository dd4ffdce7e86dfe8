"""GPU parity: batched samples (several samples stacked by cells, each scaled,
embedded and searched on its own, in the same launches) against the oracle per
sample and against the single-sample device path."""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

SIZES = [300, 1500, 80, 900, 450]


def _samples(O, nf_genes=600):
    mats = []
    for i, n in enumerate(SIZES):
        X = O.synth_counts(n, nf_genes, -1.0, 1.5, depth=0.3 * (1.0 + 0.4 * i), seed=60 + i, n_clusters=3)
        mats.append(sp.csc_matrix(X))
    off = np.concatenate([[0], np.cumsum(SIZES)])
    return mats, sp.csc_matrix(sp.vstack(mats)), off


@pytest.fixture(scope="module")
def batch_setup(sv, O):
    ctx = sv.Context(0)
    mats, X, off = _samples(O)
    counts = sv.CountMatrix.from_csc(X, ctx=ctx)
    d = sv.normalize_cells(counts, scale_factor=1e4, dtype="float32", ctx=ctx)
    # the moments are compared on the values the device stored (FP32 rounding of
    # the normalisation is tested in test_gpu_normalize.py)
    ref = O.normalize_cells(X, scale_factor=1e4, dtype=np.float32).astype(np.float64)
    ref.data = d.values_csc().astype(np.float64)
    # features that vary in every sample (a feature constant within a sample has
    # std 0 and mu = 0/0 there, as in the reference)
    ok = np.ones(ref.shape[1], bool)
    for s in range(len(SIZES)):
        _, v = O.mean_var(sp.csc_matrix(ref[off[s]:off[s + 1]]))
        ok &= v > 0
    _, var = O.mean_var(ref)
    var[~ok] = -1.0
    hvf = np.sort(np.argsort(-var, kind="stable")[:200]) + 1
    B = sv.Batch.create(d, off, features=hvf, scale_max=10.0)
    return ctx, mats, X, off, counts, d, ref, hvf, B


def test_batch_moments_per_sample(sv, O, batch_setup):
    ctx, mats, X, off, counts, d, ref, hvf, B = batch_setup
    mu, mean, sd = B.stats()
    for s in range(len(SIZES)):
        R = sp.csc_matrix(ref[off[s]:off[s + 1]])
        Sr, m_r, s_r = O.scale_features(R, 10.0, np.float64, hvf)
        # FP64 moments by different summation orders (Welford/Chan on the device)
        assert np.allclose(mean[s], m_r, rtol=1e-11, atol=1e-14)
        assert np.allclose(sd[s], s_r, rtol=1e-11)
        assert np.allclose(mu[s], Sr.mu, rtol=1e-11, atol=1e-14)


def test_batch_pca_matches_single_sample_runs(sv, O, batch_setup):
    ctx, mats, X, off, counts, d, ref, hvf, B = batch_setup
    init = np.random.default_rng(3).standard_normal(len(hvf))
    em = sv.batch_pca(B, 10, tol=1e-7, init=init)
    iters = em.info["iters"]
    assert len(iters) == len(SIZES) and np.all(iters >= 1)
    for s in range(len(SIZES)):
        R = sp.csc_matrix(ref[off[s]:off[s + 1]])
        Sr, _, _ = O.scale_features(R, 10.0, np.float64, hvf)
        sf = np.linalg.svd(Sr.dense(), compute_uv=False)[:10]
        n_s = off[s + 1] - off[s]
        sb = em.stdev[s] * np.sqrt(n_s - 1)
        assert np.max(np.abs(sb - sf) / sf) < 1e-5, s
        # the same sample through the single-sample path
        cs = sv.CountMatrix.from_csc(mats[s], ctx=ctx)
        ds = sv.normalize_cells(cs, scale_factor=1e4, dtype="float32", ctx=ctx)
        S1 = sv.scale_features(ds, scale_max=10.0, features=hvf)
        e1 = sv.pca(S1, 10, tol=1e-7, init=init)
        assert np.max(np.abs(em.stdev[s] - e1.stdev) / e1.stdev) < 1e-6, s
        # coordinates span the same leading subspace (well-separated components)
        Zb = em.coordinates[off[s]:off[s + 1]]
        c = np.abs(np.sum(Zb * e1.coordinates, axis=0)) / (np.linalg.norm(Zb, axis=0) *
                                                          np.linalg.norm(e1.coordinates, axis=0))
        gap = sf[:-1] / sf[1:] - 1
        good = np.nonzero(np.concatenate([[gap[0]], np.minimum(gap[:-1], gap[1:])]) > 0.05)[0]
        assert np.all(c[good] > 1 - 1e-6), (s, c)


@pytest.mark.parametrize("precision", ["bf16", "fp32"])
def test_batch_knn_stays_within_samples(sv, O, batch_setup, precision):
    ctx, mats, X, off, counts, d, ref, hvf, B = batch_setup
    init = np.random.default_rng(4).standard_normal(len(hvf))
    em = sv.batch_pca(B, 10, tol=1e-6, init=init)
    k = 10
    idx, dist, _ = sv.batch_ann(B, em, k, precision=precision)
    Z = em.coordinates
    hits = total = 0
    for s in range(len(SIZES)):
        rows = idx[off[s]:off[s + 1]] - 1
        assert rows.min() >= off[s] and rows.max() < off[s + 1]
        assert np.all(rows[:, 0] == np.arange(off[s], off[s + 1]))      # include_self first
        ref_idx, _ = O.knn_exact(Z[off[s]:off[s + 1]], k)
        for a, b in zip(rows - off[s], ref_idx):
            hits += len(set(a) & set(b))
        total += ref_idx.size
    assert hits / total >= 0.999


def test_batch_rejects_bad_offsets(sv, batch_setup):
    ctx, mats, X, off, counts, d, ref, hvf, B = batch_setup
    with pytest.raises(sv.SeveroGPUError, match="offsets"):
        sv.Batch.create(d, np.array([0, 10, 20]), features=hvf)
    with pytest.raises(sv.SeveroGPUError, match="fewer than two"):
        sv.Batch.create(d, np.array([0, 1, off[-1]]), features=hvf)
