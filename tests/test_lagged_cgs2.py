"""The lagged CGS2 of the cell-side Lanczos steps (severo.jl_gb300/csrc/sv_irlba.cu,
k_cgs_lag_tma / k_gdots / k_gcol), restated in FP64 NumPy and compared with
classical Gram-Schmidt applied twice.

Per cell-side step the device forms the first projection's coefficients on the
feature side, c0 = G^T v - beta (cp, 1) with G = A^T W, applies the previous
step's second projection (the pending correction cp) to its column during the
pass, and leaves its own second projection pending; the feature-side product of
a pending column is corrected through G.  The bases and the bidiagonal entries
must be those of plain CGS2 up to rounding.
"""
import numpy as np


def _cgs2(x, Q):
    if Q.shape[1] == 0:
        return x
    x = x - Q @ (Q.T @ x)
    return x - Q @ (Q.T @ x)


def bidiag_cgs2(A, v0, work):
    m, n = A.shape
    W = np.zeros((m, work))
    V = np.zeros((n, work))
    alpha = np.zeros(work)
    beta = np.zeros(work)
    V[:, 0] = v0 / np.linalg.norm(v0)
    y = A @ V[:, 0]
    alpha[0] = np.linalg.norm(y)
    W[:, 0] = y / alpha[0]
    for j in range(work):
        F = A.T @ W[:, j] - alpha[j] * V[:, j]
        F = _cgs2(F, V[:, : j + 1])
        beta[j] = np.linalg.norm(F)
        if j + 1 == work:
            break
        V[:, j + 1] = F / beta[j]
        y = A @ V[:, j + 1] - beta[j] * W[:, j]
        y = _cgs2(y, W[:, : j + 1])
        alpha[j + 1] = np.linalg.norm(y)
        W[:, j + 1] = y / alpha[j + 1]
    return W, V, alpha, beta


def bidiag_lagged(A, v0, work):
    """The device's order of operations on the cell side."""
    m, n = A.shape
    W = np.zeros((m, work))      # column j holds w' (pending) until the next pass corrects it
    V = np.zeros((n, work))
    G = np.zeros((n, work))      # A^T W (corrected columns)
    alpha = np.zeros(work)
    beta = np.zeros(work)
    cp = np.zeros(work)          # pending correction of the last column: w = w' - W[:, :j] cp
    V[:, 0] = v0 / np.linalg.norm(v0)
    y = A @ V[:, 0]
    alpha[0] = np.linalg.norm(y)
    W[:, 0] = y / alpha[0]       # the first column of a run: its norm only, nothing pending
    j = 0
    while True:
        # feature side: F' = A^T w' - alpha v, corrected for the pending part of w'
        F = A.T @ W[:, j] - alpha[j] * V[:, j]
        F = F - G[:, :j] @ cp[:j]                    # k_gcol
        G[:, j] = F + alpha[j] * V[:, j]
        F = _cgs2(F, V[:, : j + 1])
        beta[j] = np.linalg.norm(F)
        if j + 1 == work:
            break
        V[:, j + 1] = F / beta[j]
        jn, pend = j + 1, j
        # the product with the stored (pending) column
        y = A @ V[:, jn] - beta[j] * W[:, pend]
        # k_gdots: first-projection coefficients from the feature side
        c0 = G[:, :jn].T @ V[:, jn]
        c0[:pend] -= beta[j] * cp[:pend]
        c0[pend] -= beta[j]
        # k_cgs_lag: correct the pending column, project once, second dots, norm
        W[:, pend] = W[:, pend] - W[:, :pend] @ cp[:pend]
        x1 = y - W[:, :jn] @ c0
        c1 = W[:, :jn].T @ x1
        nrm = np.sqrt(max(x1 @ x1 - c1 @ c1, 0.0))
        alpha[jn] = nrm
        W[:, jn] = x1 / nrm                         # w' of the new column
        cp[:] = 0
        cp[:jn] = c1 / nrm
        j = jn
    # the last column's pending correction, before the restart rotation
    W[:, j] = W[:, j] - W[:, :j] @ cp[:j]
    return W, V, alpha, beta, G


def _problem(seed, m=3000, n=400):
    rng = np.random.default_rng(seed)
    # a clustered spectrum, as the scaled count matrices have
    U, _ = np.linalg.qr(rng.standard_normal((m, 60)))
    Vt, _ = np.linalg.qr(rng.standard_normal((n, 60)))
    s = np.concatenate([np.linspace(40, 10, 20), np.linspace(3, 2.9, 40)])
    A = (U * s) @ Vt.T + 1e-3 * rng.standard_normal((m, n))
    return A, rng.standard_normal(n)


def test_lagged_cgs2_matches_cgs2():
    for seed in (1, 2):
        A, v0 = _problem(seed)
        W1, V1, a1, b1 = bidiag_cgs2(A, v0, 57)
        W2, V2, a2, b2, G = bidiag_lagged(A, v0, 57)
        assert np.allclose(a1, a2, rtol=1e-10, atol=1e-12 * a1.max())
        assert np.allclose(b1, b2, rtol=1e-10, atol=1e-12 * b1.max())
        assert np.abs(W1 - W2).max() < 1e-9
        assert np.abs(V1 - V2).max() < 1e-9
        # orthonormal bases, and G = A^T W for the settled W
        assert np.abs(W2.T @ W2 - np.eye(57)).max() < 1e-12
        assert np.abs(V2.T @ V2 - np.eye(57)).max() < 1e-12
        assert np.abs(G - A.T @ W2).max() < 1e-9 * np.abs(G).max()


def test_bidiagonal_relation_holds():
    A, v0 = _problem(3)
    W, V, a, b, _ = bidiag_lagged(A, v0, 40)
    B = np.diag(a) + np.diag(b[:-1], 1)
    # A V = W B (exactly, up to rounding) for the first columns
    assert np.abs(A @ V - W @ B).max() < 1e-9 * np.abs(B).max()
