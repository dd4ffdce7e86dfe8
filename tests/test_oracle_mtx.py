"""The MatrixMarket oracle against the format (hand-written files with known
matrices), against scipy's reader on random well-formed files, and the host-side
name handling of the readers (CPU only)."""
import io

import numpy as np
import pytest
import scipy.io
import scipy.sparse as sp

import __graft_entry__ as ge
from oracle import mtx


def mm_text(A, field="integer", rows_are_features=True, shuffle=None, dup=0, crlf=False,
            comments=("% generated",), fmt="{}", seed=0):
    """MatrixMarket text of the cells x genes matrix A (file rows = features when
    rows_are_features); `dup` extra entries split existing counts in two."""
    rng = np.random.default_rng(seed)
    C = sp.coo_matrix(A)
    r, c, v = C.row.astype(np.int64), C.col.astype(np.int64), C.data.astype(np.int64)
    if rows_are_features:
        r, c = c, r
    rows, cols = (A.shape[1], A.shape[0]) if rows_are_features else A.shape
    ent = list(zip(r + 1, c + 1, v))
    for _ in range(dup):
        if not ent:
            break
        i = int(rng.integers(len(ent)))
        a, b, x = ent[i]
        part = int(rng.integers(0, x + 1))
        ent[i] = (a, b, x - part)
        ent.append((a, b, part))
    if shuffle is not None:
        rng.shuffle(ent)
    eol = "\r\n" if crlf else "\n"
    lines = [f"%%MatrixMarket matrix coordinate {field} general", *comments, f"{rows} {cols} {len(ent)}"]
    lines += [f"{a} {b} " + fmt.format(x) for a, b, x in ent]
    return (eol.join(lines) + eol).encode()


def rand_counts(n_cells, n_genes, density, seed):
    rng = np.random.default_rng(seed)
    A = sp.random(n_cells, n_genes, density=density, random_state=rng, format="csc",
                  data_rvs=lambda k: rng.integers(1, 50, k))
    return A.astype(np.int64)


def same(A, B):
    A, B = sp.csc_matrix(A), sp.csc_matrix(B)
    return (A.shape == B.shape and np.array_equal(A.indptr, B.indptr)
            and np.array_equal(A.indices, B.indices) and np.array_equal(A.data, B.data))


def test_known_matrix():
    text = (b"%%MatrixMarket matrix coordinate integer general\n% c\n%\n\n3 4 6\n"
            b"1 1 5\n2 1 3\n3 4 1\n1 1 2\n2 2 0\n3 2 7\n")
    got = mtx.parse(text, rows_are_features=True)
    want = np.array([[7, 3, 0], [0, 0, 7], [0, 0, 0], [0, 0, 1]])
    assert got.shape == (4, 3)
    assert np.array_equal(got.toarray(), want)
    assert got.nnz == 5  # the explicit zero at (gene 2, cell 2) stays stored
    assert got.has_sorted_indices


@pytest.mark.parametrize("seed", range(4))
def test_matches_scipy_reader(seed):
    A = rand_counts(300, 170, 0.05, seed)
    text = mm_text(A, shuffle=True, dup=40, seed=seed)
    got = mtx.parse(text, rows_are_features=True)
    ref = scipy.io.mmread(io.BytesIO(text)).tocsc().T.tocsc()  # features x cells -> cells x genes
    ref.sort_indices()
    assert np.array_equal(got.toarray(), ref.toarray())
    assert same(got, A.tocsc()) or np.array_equal(got.toarray(), A.toarray())


def test_real_field_and_layouts():
    A = rand_counts(50, 40, 0.1, 9)
    for fmt in ("{}.0", "{}e0", "{}.000E+00", "0{}.0"):
        t = mm_text(A, field="real", fmt=fmt, rows_are_features=False, crlf=True)
        assert np.array_equal(mtx.parse(t, rows_are_features=False).toarray(), A.toarray()), fmt


@pytest.mark.parametrize("text,stage", [
    (b"%%MatrixMarket matrix coordinate integer\n1 1 0\n", "header"),
    (b"%MatrixMarket matrix coordinate integer general\n1 1 0\n", "header"),
    (b"%%MatrixMarket vector coordinate integer general\n1 1 0\n", "header"),
    (b"%%MatrixMarket matrix coordinate complex general\n1 1 0\n", "header"),
    (b"%%MatrixMarket matrix coordinate integer symmetric\n1 1 0\n", "header"),
    (b"%%MatrixMarket matrix array integer general\n1 1 0\n", "header"),
    (b"%%MatrixMarket matrix coordinate integer general\n% only comments\n", "header"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2\n", "header"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 2\n1 1 1\n", "entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 2\n1 1 1\n\n2 2 1\n", "entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 1\n", "entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 1 1 1\n", "entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 x 1\n", "entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 1 1.0\n", "entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n3 1 1\n", "range"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n0 1 1\n", "range"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 1 -4\n", "value"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 1 2147483648\n", "value"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 2\n1 1 2147483647\n1 1 1\n", "value"),
    (b"%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 0.5\n", "value"),
    (b"%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 inf\n", "entry"),
])
def test_errors(text, stage):
    with pytest.raises(mtx.MtxOracleError) as e:
        mtx.parse(text)
    assert e.value.stage == stage


def test_no_trailing_newline_and_empty():
    t = b"%%MatrixMarket matrix coordinate integer general\n2 3 2\n1 1 4\n2 3 5"
    assert np.array_equal(mtx.parse(t, rows_are_features=False).toarray(), [[4, 0, 0], [0, 0, 5]])
    t = b"%%MatrixMarket matrix coordinate integer general\n2 3 0\n"
    assert mtx.parse(t).nnz == 0


def test_make_unique_golden():
    """test/test_utils.jl:18-21."""
    sv = ge.load_package()
    assert sv.make_unique(["a", "a", "a"]) == ["a", "a.1", "a.2"]
    assert sv.make_unique(["a", "b", "a", "a.1"]) == ["a", "b", "a.2", "a.1"]


def test_convert_counts_names():
    """convert_counts replaces "_" by "-" before making names unique (src/input.jl:776-790)."""
    sv = ge.load_package()
    nc = sv.convert_counts(None, ["g_1", "g-1", "x"], ["c1", "c2"])
    assert nc.features == ["g-1", "g-1.1", "x"]
    nc = sv.convert_counts(None, ["g_1", "g-1"], ["c1"], unique_features=False)
    assert nc.features == ["g-1", "g-1"]


def test_reader_name_files(tmp_path):
    """Host side of read_10X / read_dge: the feature column of a (gzip) TSV and
    the %%GENES / %%CELL_BARCODES comment lines of a DGE file."""
    import gzip
    sv = ge.load_package()
    rd = sv.readers
    p = tmp_path / "features.tsv.gz"
    with gzip.open(p, "wt") as f:
        f.write("ENSG1\tA_1\tGene Expression\nENSG2\tB\tGene Expression\n\n")
    assert rd._feature_names(str(p), 2) == ["A_1", "B"]
    assert rd._feature_names(str(p), 1) == ["ENSG1", "ENSG2"]
    q = tmp_path / "x.dge.txt"
    q.write_text("%%MatrixMarket matrix coordinate integer general\n%%GENES\tg1\tg2\n\n"
                 "%%CELL_BARCODES\tc1\n%%CELL_BARCODES\tc2\tc3\n% other\n2 3 0\n")
    assert rd._dge_names(str(q)) == (["g1", "g2"], ["c1", "c2", "c3"])
    nc = sv.convert_counts(None, ["A_1", "A-1", "A-1"], ["c"])
    assert nc.features == ["A-1", "A-1.1", "A-1.2"]


def test_bench_text_writer_round_trip():
    """The reader bench's MatrixMarket writer (vectorised digit placement) against
    the C oracle: every field, including values past its digit tables."""
    import bench
    rng = np.random.default_rng(4)
    n = 5000
    gene = rng.integers(1, 28000, n)
    cell = np.sort(rng.integers(1, 1_000_000, n))
    cnt = rng.integers(0, 3000, n)
    cnt[::97] = rng.integers(10 ** 6, 2 ** 31 - 1, cnt[::97].size)
    text = bench.mm_format(gene, cell, cnt, f"%%MatrixMarket matrix coordinate integer general\n"
                                             f"28000 1000000 {n}\n", chunk=1024)
    got = mtx.parse(text, rows_are_features=True)
    want = sp.coo_matrix((cnt, (cell - 1, gene - 1)), shape=(1_000_000, 28000)).tocsc()  # sums repeats
    assert (got != want).nnz == 0
