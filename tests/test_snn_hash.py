"""The hash-table form of the SNN kernels (severo.jl_gb300/csrc/sv_snn.cu,
snn_column_hash), restated in NumPy and checked against the oracle's
jaccard_index (src/neighbours.jl:88-108).

Per column j the candidates are the reverse neighbours of j's neighbours; a row
occurring c times shares c neighbours with j.  The device counts them in a
table of S = max(32, 32-rounded 1.5 x candidates) 32-bit words, word =
(row + 1) << cb | count with cb the bit length of k, linear probing from a
multiplicative hash, then keeps the words whose weight passes the prune
threshold, pads to a power of two with 0xFFFFFFFF and sorts them (the row is in
the high bits, so word order is row order).  The tests check that the probing
always finds a slot, that counts never carry into the row, that a real word
never equals the padding, and that the result is the oracle's bit for bit
whatever the order in which the candidates arrive.
"""
import numpy as np
import pytest


def _umulhi(a, b):
    return (int(a) * int(b)) >> 32


def column_hash(cands, k, kk, prune, dtype, order_rng=None):
    cb = int(k).bit_length()
    tot = len(cands)
    S = max(32, (3 * tot // 2 + 31) // 32 * 32)
    tab = [0] * S
    cmask = (1 << cb) - 1
    seq = list(cands)
    if order_rng is not None:
        order_rng.shuffle(seq)
    for row in seq:
        key = row + 1
        h = _umulhi((key * 2654435761) & 0xFFFFFFFF, S)
        probes = 0
        while True:
            cur = tab[h]
            if cur == 0:
                tab[h] = (key << cb) | 1
                break
            if (cur >> cb) == key:
                assert (cur & cmask) + 1 <= cmask, "count would carry into the row"
                tab[h] = cur + 1
                break
            h = 0 if h + 1 == S else h + 1
            probes += 1
            assert probes < S, "table full"
    t = dtype.type
    kept = []
    for v in tab:
        if v == 0:
            continue
        c = v & cmask
        w = t(c) / (t(kk) + (t(kk) - t(c)))
        if w > t(prune):
            kept.append(v)
    kept.sort()
    assert all(v != 0xFFFFFFFF for v in kept)
    rows = [(v >> cb) - 1 for v in kept]
    vals = [t(v & cmask) / (t(kk) + (t(kk) - t(v & cmask))) for v in kept]
    return rows, vals


def snn_by_hash(nn, k, prune, dtype, variant_k=True, seed=None):
    n = nn.shape[0]
    N = [sorted(set(int(v) for v in row if 0 <= v < n)) for row in nn]
    R = [[] for _ in range(n)]
    for i in range(n):
        for r in N[i]:
            R[r].append(i)
    rng = np.random.default_rng(seed) if seed is not None else None
    indptr, indices, data = [0], [], []
    for j in range(n):
        cands = [i for r in N[j] for i in R[r]]
        kk = k if variant_k else len(N[j])
        rows, vals = column_hash(cands, k, kk, prune, dtype, rng)
        indices += rows
        data += vals
        indptr.append(len(indices))
    return np.array(indptr), np.array(indices), np.array(data, dtype=dtype)


def _knn(n, k, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, 5))
    X[: n // 10] = X[0]               # a hub: many identical points
    d = ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1)
    return np.argsort(d, axis=1, kind="stable")[:, :k]   # includes self


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("variant_k", [True, False])
def test_hash_form_equals_oracle(O, dtype, variant_k):
    n, k, prune = 600, 12, 1.0 / 15.0
    nn = _knn(n, k, 7)
    G = O.knn_graph(nn + 1, n)
    want = O.jaccard_index(G, k if variant_k else None, prune, dtype)
    for seed in (None, 1, 2):
        p, i, x = snn_by_hash(nn, k, prune, np.dtype(dtype), variant_k, seed)
        assert np.array_equal(p, want.indptr)
        assert np.array_equal(i, want.indices)
        assert x.tobytes() == want.data.astype(dtype).tobytes()


def test_packing_limits():
    """The host picks the packed form when n + 1 < 2^(32 - cb): then every word
    is below the padding value and a count <= k never reaches the row bits."""
    for k in range(1, 65):
        cb = k.bit_length()
        n = (1 << (32 - cb)) - 2          # the largest n that passes the host test
        assert n + 1 < (1 << (32 - cb))
        top = ((n - 1 + 1) << cb) | k      # the largest row and count
        assert top < 0xFFFFFFFF and k <= (1 << cb) - 1
