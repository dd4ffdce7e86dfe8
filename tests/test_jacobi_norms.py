"""The restart SVD of the Lanczos bidiagonal (severo.jl_gb300/csrc/sv_irlba.cu,
k_jacobi_svd) restated in FP64 NumPy: one-sided (Hestenes) Jacobi with the pairs
of the circle method, the rotation threshold |a_p . a_q| > tau |a_p| |a_q| with
tau = 1e-12 max(1, m/16), and the squared column norms computed once per sweep
and carried through its rotations by alpha' = alpha - t gamma,
beta' = beta + t gamma instead of being recomputed.

The carried norms only steer the angles and the convergence test; the singular
values come from the final columns.  The tests check that the carried norms stay
those of the rotated columns, that the sweep count and the singular values are
those of the form that recomputes the norms, and that the result is LAPACK's.
"""
import numpy as np
import pytest


def jacobi(B, carried=True, max_sweeps=60):
    m = B.shape[0]
    A = B.astype(np.float64).copy()
    J = np.eye(m)
    mp = m + (m & 1)
    tau = 1e-12 * max(1.0, m / 16.0)
    worst = 0.0
    for sweep in range(max_sweeps):
        rotated = False
        nrm = (A * A).sum(axis=0)
        for rnd in range(mp - 1):
            for pi in range(mp // 2):
                a = 0 if pi == 0 else 1 + (pi - 1 + rnd) % (mp - 1)
                b = 1 + (mp - 2 - pi + rnd) % (mp - 1)
                if a >= m or b >= m:
                    continue
                p, q = min(a, b), max(a, b)
                if carried:
                    al, be = nrm[p], nrm[q]
                else:
                    al, be = A[:, p] @ A[:, p], A[:, q] @ A[:, q]
                ga = A[:, p] @ A[:, q]
                if abs(ga) > tau * np.sqrt(al) * np.sqrt(be) and ga != 0.0:
                    zeta = (be - al) / (2.0 * ga)
                    t = (1.0 if zeta >= 0 else -1.0) / (abs(zeta) + np.hypot(1.0, zeta))
                    c = 1.0 / np.sqrt(1.0 + t * t)
                    s = c * t
                    ap, aq = A[:, p].copy(), A[:, q].copy()
                    A[:, p], A[:, q] = c * ap - s * aq, s * ap + c * aq
                    jp, jq = J[:, p].copy(), J[:, q].copy()
                    J[:, p], J[:, q] = c * jp - s * jq, s * jp + c * jq
                    nrm[p], nrm[q] = al - t * ga, be + t * ga
                    rotated = True
                    if carried:
                        for k in (p, q):
                            true = A[:, k] @ A[:, k]
                            worst = max(worst, abs(nrm[k] - true) / max(true, 1e-300))
        if not rotated:
            break
    s = np.sqrt((A * A).sum(axis=0))
    order = np.argsort(-s, kind="stable")
    return s[order], J[:, order], sweep, worst


def _bidiag_plus(m, seed):
    """An upper bidiagonal with a spike in the last column, as a restarted
    Lanczos cycle's B is, with a clustered spectrum."""
    rng = np.random.default_rng(seed)
    B = np.diag(np.concatenate([np.linspace(40, 10, m // 3), 3 + 1e-3 * rng.random(m - m // 3)]))
    B += np.diag(rng.random(m - 1) * 0.5, 1)
    B[:, -1] += rng.random(m) * 0.1
    return B


@pytest.mark.parametrize("m,seed", [(57, 1), (57, 2), (37, 3), (10, 4)])
def test_carried_norms_follow_the_columns(m, seed):
    B = _bidiag_plus(m, seed)
    s1, J1, sw1, worst = jacobi(B, carried=True)
    s0, J0, sw0, _ = jacobi(B, carried=False)
    # the carried value is the rotated column's squared norm to rounding
    assert worst < 1e-12
    # same convergence and the same singular values as recomputing
    assert abs(sw1 - sw0) <= 1
    assert np.allclose(s1, s0, rtol=1e-14, atol=0)
    ref = np.linalg.svd(B, compute_uv=False)
    assert np.allclose(s1, ref, rtol=1e-13, atol=1e-14 * ref[0])
    assert np.abs(J1.T @ J1 - np.eye(m)).max() < 1e-13
