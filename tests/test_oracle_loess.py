"""The loess surfaces of find_variable_features(:vst) (src/variablefeatures.jl:34-50).

The reference fits log10(std) on log10(mean) with Loess.jl's loess(xs, ys, span)
and evaluates it with predict (variablefeatures.jl:41-42): local quadratic fits at
the vertices of a kd-tree over xs, blended inside each cell.  The oracle restates
that (loess_kdtree_cells, loess_kdtree) beside the fit evaluated directly at every
gene (loess_direct).  These tests pin the kd-tree on hand-worked cases, check that
the library's host-side tree (sv_loess_vertices) is the oracle's bit for bit,
check the surfaces on polynomials and on the zero-width cell that the reference's
nan2zero! works around, and bound how far the vertex surfaces move the vst
metric and the selected genes from the direct fit on synthetic counts.
"""
import ctypes as C
import math

import numpy as np
import pytest

import __graft_entry__ as ge


@pytest.fixture(scope="module")
def lib():
    ge._build_module().build()
    return ge.load_package()._lib


def _tree(lib, xs, span):
    L = lib.load()
    xs = np.ascontiguousarray(xs, dtype=np.float64)
    cap = 4096
    out = np.zeros(cap)
    n = L.sv_loess_vertices(xs.ctypes.data_as(C.c_void_p), len(xs), float(span),
                            out.ctypes.data_as(C.c_void_p), cap)
    assert 0 < n <= cap
    return out[:n]


def test_kdtree_hand_cases(O):
    # n = 20, span 0.5: cells of at most ceil(0.1 * 20) = 2 points; even cells split
    # at the mean of the middle pair, odd cells at their (L div 2)-th smallest point
    b = O.loess_kdtree_cells(np.arange(20.0), 0.5)
    assert b.tolist() == [0, 1, 2, 4.5, 6, 7, 9.5, 11, 12, 14.5, 16, 17, 19]
    b = O.loess_kdtree_cells(np.arange(11.0), 0.5)
    assert b.tolist() == [0, 1, 2, 4, 5, 7.5, 8, 10]
    # a cell of zero width is a leaf whatever its size
    b = O.loess_kdtree_cells(np.array([1.0] * 12 + [2.0, 3.0, 4.0, 5.0]), 0.5)
    assert b[0] == b[1] == 1.0 and b[-1] == 5.0


def test_library_tree_matches_oracle(lib, O):
    rng = np.random.default_rng(3)
    for n, span in [(20, 0.5), (11, 0.5), (1, 0.5), (2, 0.5), (997, 0.5), (5000, 0.3), (4000, 0.75),
                    (12345, 0.5)]:
        xs = np.sort(rng.normal(size=n))
        if n > 100:   # ties, as genes of equal mean give
            xs = np.sort(np.round(xs, 2))
        got = _tree(lib, xs, span)
        want = O.loess_kdtree_cells(xs, span)
        assert got.tobytes() == want.tobytes(), (n, span)
    L = lib.load()
    bad = np.array([1.0, 0.0, 2.0])
    assert L.sv_loess_vertices(bad.ctypes.data_as(C.c_void_p), 3, 0.5, None, 0) == -1


def test_surfaces_on_polynomials(O):
    rng = np.random.default_rng(4)
    x = np.sort(rng.normal(size=600))
    quad = 0.3 * x * x - 0.5 * x + 1.0
    # the local quadratic reproduces a quadratic; so does the Hermite blend of
    # exact vertex values and slopes
    assert np.abs(O.loess_direct(x, quad, 0.5) - quad).max() < 1e-10
    assert np.abs(O.loess_kdtree(x, quad, 0.5, "hermite") - quad).max() < 1e-10
    # the linear blend is exact for a line and meets the direct fit at the vertices
    line = 2.0 * x - 1.0
    assert np.abs(O.loess_kdtree(x, line, 0.5, "linear") - line).max() < 1e-10
    y = np.sin(2 * x) + 0.05 * rng.normal(size=600)
    b = O.loess_kdtree_cells(x, 0.5)
    lin = O.loess_kdtree(x, y, 0.5, "linear")
    direct = O.loess_direct(x, y, 0.5)
    on_vertex = np.isin(x, b)
    assert on_vertex.sum() >= 2
    assert np.allclose(lin[on_vertex], direct[on_vertex], rtol=0, atol=1e-10)


def _singles_and_rich(single, rich, n_cells=400, seed=5):
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    cols = []
    for g in range(single):       # one count in the whole matrix: the lowest mean
        c = np.zeros(n_cells, np.int64)
        c[rng.integers(n_cells)] = 1
        cols.append(c)
    for g in range(rich):
        cols.append(rng.poisson(0.2 + 0.1 * g, n_cells))
    return sp.csc_matrix(np.stack(cols, axis=1))


def test_zero_width_first_cell_gives_metric_zero(O):
    """30% of the non-constant genes at the lowest mean: a split lands on that
    mean, the first cell [min, min] has zero width, the linear blend is 0/0
    there, and nan2zero! leaves those genes an expected std of 0 and a metric of
    0.  The vertex fit at the minimum itself is finite (its q nearest genes
    spread beyond it), so the Hermite blend, which returns a vertex's own fit
    at the vertex, and the direct fit give them a metric."""
    A = _singles_and_rich(36, 84)
    b = O.loess_kdtree_cells(np.sort(np.log10(np.asarray(A.mean(axis=0)).ravel())), 0.5)
    assert b[0] == b[1] and b[2] > b[1]
    m = O.vst_metric(A, 0.5, "interpolate")
    assert np.all(m[:36] == 0.0) and np.all(m[36:] > 0.0)
    assert np.all(O.vst_metric(A, 0.5, "hermite") > 0.0)
    assert np.all(O.vst_metric(A, 0.5, "direct") > 0.0)


def test_flat_vertex_window_gives_metric_zero(O):
    """Over half of the non-constant genes at the lowest mean: the q = n/2
    genes nearest to the vertex at the minimum all sit on it, the weight
    formula is 0/0 there, and every gene whose cell has that vertex gets a
    metric of 0 under both blends; the direct fit (unit weights on a flat
    window) does not."""
    A = _singles_and_rich(70, 50)
    for surf in ("interpolate", "hermite"):
        m = O.vst_metric(A, 0.5, surf)
        assert np.all(m[:70] == 0.0), surf
        assert 0 < np.sum(m[70:] == 0.0) < 50, surf
    assert np.all(O.vst_metric(A, 0.5, "direct") > 0.0)


@pytest.mark.parametrize("n_cells,n_genes,nfeat,seed", [(2000, 6000, 1000, 71)])
def test_surface_difference_bound(O, n_cells, n_genes, nfeat, seed):
    """How far the vertex surfaces move the vst result from the direct fit, on NB
    counts with a realistic mean-variance spread (6,000 genes, clusters): the
    linear blend (the reference's surface) keeps >= 95% of the selected genes
    (measured 97.3%) and moves the metric by a median factor of 1.0003; the
    Hermite blend keeps >= 99.5% (measured 100%)."""
    X = O.synth_counts(n_cells, n_genes, -1.2, 1.6, depth=0.4, seed=seed, n_clusters=6)
    res = {s: O.find_variable_features_vst(X, nfeat, 0.5, s) for s in O.LOESS_SURFACES}
    fd, md = res["direct"]
    for surf, keep, max_log in (("interpolate", 0.95, 0.5), ("hermite", 0.995, 5e-3)):
        f, m = res[surf]
        assert len(set(f) & set(fd)) >= keep * nfeat, surf
        ok = (m > 0) & (md > 0)
        assert np.array_equal(m > 0, md > 0)
        r = np.abs(np.log(m[ok] / md[ok]))
        assert np.median(r) < 1e-3 and r.max() < max_log, surf


def test_unknown_surface_raises(O):
    with pytest.raises(ValueError):
        O.loess_surface(np.arange(5.0), np.arange(5.0), 0.5, "cubic")
    assert math.isnan(O.loess_fit_at(np.zeros(5), np.arange(5.0), 3, 0.0, flat="nan")[0])
