"""GPU parity: scale_features (src/scaling.jl:199-217,335-357) and the implicit
CenteredMatrix products (src/scaling.jl:245-272)."""
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

G = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())


def _dense_of(S, m, n):
    """convert(Matrix, S) through the products: S * e_j for every feature."""
    return S.mul(np.eye(n))


def test_scaling_golden(sv, ctx):
    # test/test_scaling.jl:21-45: S.mu == mean/std, convert(Matrix, S) == (X - mu)/std
    # The reference scales the integer count matrix itself (scaling.jl:335); its
    # CenteredMatrix holds A/std and mean/std, built here with the (A, mu) constructor.
    X = sp.csc_matrix(np.array(G["scaling"]["counts"], dtype=np.int64))
    mu_c = np.array(G["scaling"]["mean"])
    std_c = np.array(G["scaling"]["std"])
    S = sv.CenteredMatrix.from_sparse(X.astype(np.float64) / std_c, mu_c / std_c, ctx=ctx)
    D = _dense_of(S, *S.shape)
    assert np.allclose(D, G["scaling"]["dense"], rtol=1e-13, atol=1e-14)
    assert np.allclose(S.mu, G["scaling"]["mu"], rtol=1e-15)


def test_scale_features_stats_match_oracle(sv, ctx, O):
    X = O.synth_counts(900, 500, -1.0, 1.5, depth=0.5, seed=21)
    d = sv.normalize_cells(X, scale_factor=1e4, ctx=ctx)
    ref = O.normalize_cells(X, scale_factor=1e4)
    hvf = O.top_variable_genes(ref, 150)
    S = sv.scale_features(d, scale_max=10.0, features=hvf)
    Sr, mean, std = O.scale_features(ref, 10.0, np.float64, hvf)
    mu, gm, gs = S.stats()
    assert np.allclose(gm, mean, rtol=1e-13)
    assert np.allclose(gs, std, rtol=1e-13)
    assert np.allclose(mu, Sr.mu, rtol=1e-13)
    assert S.shape == (900, 150) and S.nnz == Sr.A.nnz


@pytest.mark.parametrize("dtype", ["float32", "bfloat16"])
@pytest.mark.parametrize("n_cells", [2000, 300_000])
def test_moments_fp32_bf16_storage(sv, ctx, O, dtype, n_cells):
    """Moments of FP32 / BF16 values (double-float sums on the device, FP64
    merge) against the FP64 oracle on the values actually stored; 300,000
    cells split every column into several parts.  The reference accumulates
    Float32 data in Float32 (src/scaling.jl:40-44): the device's FP64 moments
    differ from that by Float32 rounding only."""
    X = O.synth_counts(n_cells, 60, -0.5, 1.5, depth=0.8, seed=24)
    d = sv.normalize_cells(X, scale_factor=1e4, dtype=dtype, ctx=ctx)
    ref = O.normalize_cells(X, scale_factor=1e4, dtype=np.float32)
    ref.data = d.values_csc().astype(np.float32)          # the stored values (BF16 rounded)
    S = sv.scale_features(d, scale_max=10.0)
    mu, gm, gs = S.stats()
    _, mean, std = O.scale_features(ref.astype(np.float64), 10.0, np.float64)
    assert np.allclose(gm, mean, rtol=1e-13, atol=0)
    assert np.allclose(gs, std, rtol=1e-13, atol=0)
    if n_cells <= 2000 and dtype == "float32":
        _, _, std32 = O.scale_features(ref, 10.0, np.float32)   # the reference's Float32 Welford
        assert np.allclose(gs, std32, rtol=2e-5)


@pytest.mark.parametrize("dtype,rtol", [("float64", 1e-12), ("float32", 2e-6), ("bfloat16", 2e-6)])
@pytest.mark.parametrize("scale_max", [np.inf, 10.0, 0.75])
def test_centered_products(sv, ctx, O, dtype, rtol, scale_max):
    X = O.synth_counts(1200, 700, -1.0, 1.5, depth=0.6, seed=22)
    d = sv.normalize_cells(X, scale_factor=1e4, dtype=dtype, ctx=ctx)
    if dtype == "bfloat16":
        ref = O.normalize_cells(X, scale_factor=1e4, dtype=np.float32)
        ref.data = O.round_bf16(ref.data)
        ref = ref.astype(np.float64)
        # the device stats use the BF16 values actually stored
        ref.data = d.values_csc().astype(np.float64)
    else:
        ref = O.normalize_cells(X, scale_factor=1e4, dtype=np.dtype(dtype)).astype(np.float64)
    hvf = O.top_variable_genes(ref, 300)
    S = sv.scale_features(d, scale_max=scale_max, features=hvf)
    Sr, _, _ = O.scale_features(ref, scale_max, np.float64, hvf)
    Q = Sr.dense()
    if np.isfinite(scale_max) and scale_max < 1:
        assert (Sr.A.data == (scale_max + Sr.mu[np.repeat(np.arange(300), np.diff(Sr.A.indptr))])).any()
    rng = np.random.default_rng(0)
    v = rng.standard_normal(300)
    u = rng.standard_normal(1200)
    y = S.mul(v)
    yr = Q @ v
    assert np.linalg.norm(y - yr) <= rtol * np.linalg.norm(yr) * 10
    z = S.rmul(u)
    zr = Q.T @ u
    assert np.linalg.norm(z - zr) <= rtol * np.linalg.norm(zr) * 10
    # alpha / beta forms and matrix right-hand sides (scaling.jl:259-272)
    V = rng.standard_normal((300, 3))
    Y0 = rng.standard_normal((1200, 3))
    Y = S.mul(V, 2.0, 0.5, Y0)
    assert np.allclose(Y, 2 * Q @ V + 0.5 * Y0, rtol=rtol * 100, atol=rtol * 100 * np.abs(Q @ V).max())


@pytest.mark.parametrize("variant", ["dense", "sparse"])
def test_centered_golden(sv, ctx, variant):
    # test/test_scaling.jl:70-113 (the dense testset uses the same products)
    c = G["centered"]
    S = sv.CenteredMatrix.from_sparse(np.array(c["A"]), np.array(c["mu"]), ctx=ctx)
    assert S.shape == (4, 3)
    r = np.array(c["r"])
    y0 = np.array(c["y0"])
    e = c[variant]
    assert np.allclose(S.mul(r), e["Cr"], rtol=1e-14)
    y = S.mul(r, 2.0, 1.0, y0)
    assert np.allclose(y, e["y1"], rtol=1e-14)
    if variant == "sparse":
        y = S.mul(r, 2.0, 1.0, y)
        assert np.allclose(y, e["y2"], rtol=1e-14)
    assert np.allclose(S.rmul(y), e["Cty"], rtol=1e-14)
    assert np.allclose(S.rmul(y, 2.0, 1.0, r), e["r1"], rtol=1e-14)


@pytest.mark.parametrize("dtype", ["float32", "bfloat16"])
def test_transpose_product_forms_agree(sv, ctx, O, dtype, monkeypatch):
    """X^T u over the row-blocked copy (default), the CSC chunks and the CSR_h
    shared-memory form give the same result (FP32 accumulation order only).
    40,000 cells span three 16,384-cell row blocks."""
    X = O.synth_counts(40000, 600, -1.0, 1.5, depth=0.5, seed=23)
    d = sv.normalize_cells(X, scale_factor=1e4, dtype=dtype, ctx=ctx)
    hvf = np.arange(1, 601, 2)
    u = np.random.default_rng(1).standard_normal(40000)
    out = {}
    for mode in ("rb", "csc", "csr"):
        if mode == "rb":
            monkeypatch.delenv("SV_TPRODUCT", raising=False)
        else:
            monkeypatch.setenv("SV_TPRODUCT", mode)
        S = sv.scale_features(d, scale_max=10.0, features=hvf)
        out[mode] = S.rmul(u)
    ref = out["csc"]
    for mode in ("rb", "csr"):
        assert np.linalg.norm(out[mode] - ref) <= 1e-5 * np.linalg.norm(ref)


def test_scale_rejects_bad_features(sv, ctx, O):
    X = O.synth_counts(50, 40, -1.0, 1.5, depth=0.5, seed=1)
    d = sv.normalize_cells(X, ctx=ctx)
    with pytest.raises(sv.SeveroGPUError, match="out of range"):
        sv.scale_features(d, features=[0, 3])
    with pytest.raises(sv.SeveroGPUError, match="duplicate"):
        sv.scale_features(d, features=[3, 3])
