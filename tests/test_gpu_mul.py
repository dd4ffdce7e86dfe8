"""GPU parity: the sparse products of src/mul.jl (bit-identical to the oracle's
restatement, which accumulates in the reference's order) and the
CenteredMatrix Gram product of src/scaling.jl:274-296."""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu


def test_mul_spvec_bitexact(sv, ctx, O):
    rng = np.random.default_rng(1)
    A = sp.random(9000, 300, density=0.05, random_state=2, format="csc")
    x = sp.random(300, 1, density=0.3, random_state=3, format="csc")
    y0 = rng.standard_normal(9000)
    for alpha, beta in ((1.0, 0.0), (2.0, 0.5), (0.0, 3.0), (-1.5, 1.0)):
        got = sv.sparse_mul_spvec(A, x, alpha, beta, y0, ctx=ctx)
        want = O.mul_spvec(A, x.indices, x.data, alpha, beta, y0)
        assert np.array_equal(got, want), (alpha, beta)


@pytest.mark.parametrize("transa", [False, True])
def test_mul_sparse_bitexact(sv, ctx, O, transa):
    rng = np.random.default_rng(4)
    A = sp.random(200, 150, density=0.05, random_state=5, format="csc")
    B = sp.random(200 if transa else 150, 60, density=0.1, random_state=6, format="csc")
    C0 = rng.standard_normal((150 if transa else 200, 60))
    got = sv.sparse_mul(A, B, 1.5, 0.25, C0, transa=transa, ctx=ctx)
    Aop = sp.csc_matrix(A.T) if transa else A                 # copy(A') (mul.jl:79-80)
    Aop.sort_indices()
    want = O.mul_sparse(Aop, B, 1.5, 0.25, C0)
    assert np.array_equal(got, want)


def test_mul_rejects_out_of_range_index(sv, ctx):
    A = sp.csc_matrix(np.eye(4))
    cp = np.array([0, 1, 2, 3, 4], np.int64)
    rv = np.array([0, 1, 2, 9], np.int64)                    # row 9 of a 4-row matrix
    nz = np.ones(4)
    xi = np.array([3], np.int64)
    xv = np.ones(1)
    y = np.zeros(4)
    lib = sv._lib.load()
    st = lib.sv_sparse_mul_spvec(ctx.h, 4, 4, sv._ptr(cp), sv._ptr(rv), sv._ptr(nz), 1, sv._ptr(xi),
                                 sv._ptr(xv), 0, 1.0, 0.0, sv._ptr(y))
    assert st != 0


@pytest.mark.parametrize("dtype,rtol", [("float64", 1e-12), ("float32", 1e-5)])
def test_centered_gram(sv, ctx, O, dtype, rtol):
    X = O.synth_counts(2500, 600, -0.8, 1.5, depth=0.6, seed=7)
    d = sv.normalize_cells(X, scale_factor=1e4, dtype=dtype, ctx=ctx)
    ref = O.normalize_cells(X, "lognormalize", 1e4, np.dtype(dtype)).astype(np.float64)
    f1, f2 = np.arange(1, 301), np.arange(200, 451)
    S1 = sv.scale_features(d, scale_max=10.0, features=f1)
    S2 = sv.scale_features(d, scale_max=10.0, features=f2)
    R1, _, _ = O.scale_features(ref, 10.0, np.float64, f1)
    R2, _, _ = O.scale_features(ref, 10.0, np.float64, f2)
    for Sl, Sr, Rl, Rr in ((S1, S1, R1, R1), (S1, S2, R1, R2)):
        G = sv.centered_gram(Sl, Sr)
        want = Rl.dense().T @ Rr.dense()
        assert np.linalg.norm(G - want) <= rtol * np.linalg.norm(want)
    C0 = np.random.default_rng(8).standard_normal((300, 300))
    G = sv.centered_gram(S1, None, 0.5, 2.0, C0)
    want = 0.5 * (R1.dense().T @ R1.dense()) + 2.0 * C0
    assert np.linalg.norm(G - want) <= rtol * np.linalg.norm(want)
