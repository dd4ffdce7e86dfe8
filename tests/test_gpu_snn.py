"""GPU parity: shared-nearest-neighbour Jaccard graphs (src/neighbours.jl:76-108,
127-155,272-278), bit-exact against the oracle given the same neighbour lists."""
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

G = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())


def _same(A, B):
    return (A.shape == B.shape and np.array_equal(A.indptr, B.indptr)
            and np.array_equal(A.indices, B.indices) and np.array_equal(A.data, B.data)
            and A.data.dtype == B.data.dtype)


@pytest.mark.parametrize("case", range(3))
def test_snn_golden(sv, ctx, case):
    s = G["snn"]
    c = s["cases"][case]
    W = sv.jaccard_index(np.array(s["nn_index"]), s["k"], prune=c["prune"], ctx=ctx)
    E = sp.csc_matrix((c["vals"], (np.array(c["rows"]) - 1, np.array(c["cols"]) - 1)), shape=W.shape)
    E.sort_indices()
    assert _same(W, E)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("variant", ["k", "diag"])
def test_snn_random_bitexact(sv, ctx, O, dtype, variant):
    X = np.random.default_rng(5).standard_normal((3000, 8))
    idx, _ = sv.ann(X, 20, ctx=ctx)
    k = 20 if variant == "k" else None
    W = sv.jaccard_index(idx, k, prune=1 / 15, dtype=dtype, ctx=ctx)
    R = O.jaccard_index(O.knn_graph(idx, 3000), k, 1 / 15, dtype)
    assert _same(W, R)
    assert np.all(W.diagonal() == 1)


def test_snn_prune_zero_keeps_all_pairs(sv, ctx, O):
    rng = np.random.default_rng(6)
    idx = np.stack([rng.choice(500, 10, replace=False) for _ in range(500)]).astype(np.int32) + 1
    W = sv.jaccard_index(idx, 10, prune=0.0, ctx=ctx)
    R = O.jaccard_index(O.knn_graph(idx, 500), 10, 0.0)
    assert _same(W, R)


def test_snn_hubs_take_block_and_global_paths(sv, ctx, O):
    """Cells that are neighbours of many cells make long candidate lists."""
    rng = np.random.default_rng(7)
    n, k = 6000, 12
    idx = np.empty((n, k), dtype=np.int32)
    for i in range(n):
        idx[i, 0] = i
        idx[i, 1] = 0                       # a hub every cell points at
        idx[i, 2] = 1 + (i % 3)             # three medium hubs
        idx[i, 3:] = rng.choice(n, k - 3, replace=False)
    idx += 1
    W = sv.jaccard_index(idx, k, prune=1 / 15, ctx=ctx)
    R = O.jaccard_index(O.knn_graph(idx, n), k, 1 / 15)
    assert _same(W, R)


def test_shared_nearest_neighbours_pipeline(sv, ctx, O):
    X = np.random.default_rng(8).standard_normal((2000, 10)).astype(np.float32)
    W = sv.shared_nearest_neighbours(X, 15, prune=1 / 15, ctx=ctx)
    idx, _ = sv.ann(X, 15, ctx=ctx)
    R = O.jaccard_index(O.knn_graph(idx, 2000), 15, 1 / 15, np.float32)
    assert W.dtype == np.float32 and _same(W, R)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_network_handoff_matches_oracle(sv, ctx, O, dtype):
    """Network(snn) (src/modularity.jl:163-194) emitted from the device graph:
    node weights, edge ranges, edges and totw bit-identical to the reference's
    sequential construction."""
    rng = np.random.default_rng(7)
    n, k = 3000, 20
    X = rng.standard_normal((n, 8)).astype(np.float32)
    idx, _ = O.knn_exact(X, k)
    nn = (idx + 1).astype(np.int32)
    A, g = sv.jaccard_index(nn, k, dtype=dtype, ctx=ctx, keep=True)
    nodes, edges, totw = g.network(dtype)
    nw, first, last, en, ew, rt = O.network(A)
    assert np.array_equal(nodes["weight"], nw)
    assert np.array_equal(nodes["first"], first) and np.array_equal(nodes["last"], last)
    assert np.array_equal(edges["node"], en) and np.array_equal(edges["weight"], ew)
    assert totw == rt and type(totw) == type(rt)
    # every self link is dropped: one per node (include_self lists)
    assert len(edges) == A.nnz - n
