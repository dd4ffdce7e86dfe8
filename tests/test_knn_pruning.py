"""The tile pruning of the tensor-core kNN (severo.jl_gb300/csrc/sv_knn_tc.cu:
the TMA producer's tile sequence and the epilogue's bound), restated in NumPy.

The points are put in locality order (sorted along the dimension of largest
variance); a CTA of 128 consecutive queries starts at the 256-point tile that
holds them and walks outwards, alternately up and down.  A side stops at the
first tile whose coordinate gap g to the query tile's coordinate range has
g^2 > T, T the largest k-th best squared distance among the CTA's queries: the
gap along one coordinate bounds the distance from below, and the gap only grows
further out.  The restatement recomputes T after every tile (the device reads
it every fourth tile, a larger and so safer bound) and checks that the
neighbour sets are those of brute force while most tiles are skipped.
"""
import numpy as np
import pytest

BM, BN = 128, 256


def pruned_knn(X, k):
    n = X.shape[0]
    dim = int(np.argmax(X.var(axis=0)))
    order = np.argsort(X[:, dim], kind="stable")
    P = X[order]
    coord = P[:, dim]
    ntiles = (n + BN - 1) // BN
    nbr = np.empty((n, k), np.int64)
    visited = 0

    for q0 in range(0, n, BM):
        qend = min(q0 + BM, n)
        Q = P[q0:qend]
        t0 = min(q0 // BN, ntiles - 1)
        qlo, qhi = coord[q0], coord[qend - 1]
        bd = np.full((qend - q0, k), np.inf)
        bi = np.full((qend - q0, k), -1, np.int64)

        def visit(tile):
            s, e = tile * BN, min(tile * BN + BN, n)
            d2 = ((Q[:, None, :] - P[None, s:e, :]) ** 2).sum(-1)
            cd = np.concatenate([bd, d2], axis=1)
            ci = np.concatenate([bi, np.broadcast_to(np.arange(s, e), d2.shape)], axis=1)
            o = np.argsort(cd, axis=1, kind="stable")[:, :k]
            bd[:] = np.take_along_axis(cd, o, axis=1)
            bi[:] = np.take_along_axis(ci, o, axis=1)

        visit(t0)
        visited += 1
        up, dn, turn_up = t0 + 1, t0 - 1, True
        while True:
            T = bd[:, -1].max()
            uo, dok = up < ntiles, dn >= 0
            if uo:
                g = coord[up * BN] - qhi
                if g > 0 and g * g > T:
                    uo = False
            if dok:
                g = qlo - coord[min((dn + 1) * BN, n) - 1]
                if g > 0 and g * g > T:
                    dok = False
            if not uo:
                up = ntiles
            if not dok:
                dn = -1
            if not uo and not dok:
                break
            go_up = uo and (not dok or turn_up)
            if uo and dok:
                turn_up = not turn_up
            if go_up:
                visit(up)
                up += 1
            else:
                visit(dn)
                dn -= 1
            visited += 1
        nbr[order[q0:qend]] = order[bi]
    return nbr, visited, ntiles * ((n + BM - 1) // BM)


@pytest.mark.parametrize("n,d,k,spread,max_frac",
                         [(6000, 8, 20, 4.0, 0.55), (5000, 16, 30, 1.0, 0.85), (3000, 3, 10, 8.0, 0.35)])
def test_pruned_sets_equal_brute_force(n, d, k, spread, max_frac):
    rng = np.random.default_rng(n + d)
    centers = rng.normal(0, spread, (12, d))
    X = centers[rng.integers(0, 12, n)] + rng.standard_normal((n, d))
    X = X / np.sqrt(np.arange(1, d + 1))          # a widest dimension, as PCA scores have
    nbr, visited, total = pruned_knn(X, k)
    D = ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1)
    want = np.argsort(D, axis=1, kind="stable")[:, :k]
    assert all(set(a) == set(b) for a, b in zip(nbr.tolist(), want.tolist()))
    # the bound does skip work (measured 47%, 79% and 29% of the tiles visited)
    assert visited < max_frac * total
