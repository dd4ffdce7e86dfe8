"""Readers on the device (src/input.jl) against the MatrixMarket oracle: text
parsed in HBM, the cell-major uploads of the HDF5 layouts, and the 10X
directory reader with its names."""
import gzip
import os

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import mtx
from test_oracle_mtx import mm_text, rand_counts

pytestmark = pytest.mark.gpu


def same(A, B):
    A, B = sp.csc_matrix(A), sp.csc_matrix(B)
    return (A.shape == B.shape and np.array_equal(A.indptr, B.indptr)
            and np.array_equal(A.indices, B.indices) and np.array_equal(A.data, B.data))


def check_both_copies(sv, X, ref):
    """CSC and CSR copies of the device matrix equal the oracle entry for entry."""
    got = X.to_csc()
    assert same(got, ref)
    r = sp.csr_matrix(ref)
    r.sort_indices()
    g = X.to_csr()
    assert np.array_equal(g.indptr, r.indptr) and np.array_equal(g.indices, r.indices)
    assert np.array_equal(g.data, r.data)


@pytest.mark.parametrize("seed,rows_are_features,field,crlf", [
    (0, True, "integer", False), (1, False, "integer", True), (2, True, "real", False),
    (3, True, "integer", True)])
def test_parse_matches_oracle(sv, ctx, seed, rows_are_features, field, crlf):
    A = rand_counts(700, 450, 0.04, seed)
    fmt = "{}.0" if field == "real" else "{}"
    text = mm_text(A, field=field, rows_are_features=rows_are_features, shuffle=True, dup=200,
                   crlf=crlf, fmt=fmt, seed=seed)
    ref = mtx.parse(text, rows_are_features)
    X = sv.CountMatrix.parse_mtx(text, rows_are_features, ctx=ctx)
    assert X.shape == ref.shape and X.nnz == ref.nnz
    check_both_copies(sv, X, ref)


@pytest.mark.parametrize("field", ["integer", "real"])
def test_parse_cell_ordered(sv, ctx, field):
    """Entries in cell order with features increasing (the order 10X writes) are
    taken as the cell-major copy directly; one swapped pair or one repeated
    entry sends the file down the general path; both agree with the oracle."""
    A = rand_counts(1500, 700, 0.03, 17).tocsr()
    A.sort_indices()
    fmt = "{}.0" if field == "real" else "{}"
    text = mm_text(A, field=field, fmt=fmt)
    ref = mtx.parse(text, True)
    check_both_copies(sv, sv.CountMatrix.parse_mtx(text, True, ctx=ctx), ref)
    lines = text.split(b"\n")
    k = 3 + len(lines) // 2
    for variant in (lines[:k] + [lines[k + 1], lines[k]] + lines[k + 2:],
                    lines[:k + 1] + [lines[k]] + lines[k + 1:]):
        v = b"\n".join(variant)
        if len(variant) != len(lines):  # a repeated entry: one more entry in the size line
            hdr = lines[2].split()
            v = v.replace(lines[2], b" ".join(hdr[:2] + [str(int(hdr[2]) + 1).encode()]), 1)
        check_both_copies(sv, sv.CountMatrix.parse_mtx(v, True, ctx=ctx), mtx.parse(v, True))


def test_parse_large_with_long_header(sv, ctx):
    """Two million entries over many 4 KB tiles, after a 3 MB comment line (the
    header reader's buffer grows past its first 1 MB)."""
    A = rand_counts(20000, 3000, 0.033, 11)
    names = "\t".join(f"BARCODE{i:07d}" for i in range(200000))
    text = mm_text(A, comments=(f"%%CELL_BARCODES\t{names}", "%"), shuffle=True, seed=3)
    assert len(text) > 20_000_000
    ref = mtx.parse(text, True)
    X = sv.CountMatrix.parse_mtx(text, True, ctx=ctx)
    check_both_copies(sv, X, ref)


def test_edge_shapes(sv, ctx):
    # no trailing newline; an empty matrix; cells and genes with no entries
    t = b"%%MatrixMarket matrix coordinate integer general\n2 3 2\n1 1 4\n2 3 5"
    X = sv.CountMatrix.parse_mtx(t, False, ctx=ctx)
    assert np.array_equal(X.to_csc().toarray(), [[4, 0, 0], [0, 0, 5]])
    t = b"%%MatrixMarket matrix coordinate integer general\n5 4 0\n"
    X = sv.CountMatrix.parse_mtx(t, True, ctx=ctx)
    assert X.shape == (4, 5) and X.nnz == 0
    t = b"%%MatrixMarket matrix coordinate integer general\n  7 9 1\n\t 3   2 \t 0 \n"
    X = sv.CountMatrix.parse_mtx(t, True, ctx=ctx)
    assert X.shape == (9, 7) and X.nnz == 1 and X.to_csc()[1, 2] == 0


@pytest.mark.parametrize("text,match", [
    (b"%%MatrixMarket matrix coordinate integer\n1 1 0\n", "Malformed MatrixMarket header"),
    (b"%MatrixMarket matrix coordinate integer general\n1 1 0\n", "Not a valid MatrixMarket header"),
    (b"%%MatrixMarket vector coordinate integer general\n1 1 0\n", "Unknown MatrixMarket data type"),
    (b"%%MatrixMarket matrix coordinate complex general\n1 1 0\n", "Unsupported field"),
    (b"%%MatrixMarket matrix coordinate integer symmetric\n1 1 0\n", "Unknown matrix symmetry"),
    (b"%%MatrixMarket matrix array integer general\n1 1 0\n", "Unsupported matrix format"),
    (b"%%MatrixMarket matrix coordinate integer general\n% only comments\n", "dimensions"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2\n", "dimensions"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 2\n1 1 1\n", "matrix entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 3\n1 1 1\n", "matrix entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 2\n1 1 1\n\n2 2 1\n", "matrix entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 1\n", "matrix entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 1 1 1\n", "matrix entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 x 1\n", "matrix entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 1 1.0\n", "matrix entry"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n3 1 1\n", "out of range"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n0 1 1\n", "out of range"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 1 -4\n", "not an integer"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 1 2147483648\n", "not an integer"),
    (b"%%MatrixMarket matrix coordinate integer general\n2 2 2\n1 1 2147483647\n1 1 1\n",
     "not an integer"),
    (b"%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 0.5\n", "not an integer"),
    (b"%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 inf\n", "matrix entry"),
])
def test_errors_match_oracle(sv, ctx, text, match):
    with pytest.raises(mtx.MtxOracleError):
        mtx.parse(text)
    with pytest.raises(sv.SeveroGPUError, match=match):
        sv.CountMatrix.parse_mtx(text, True, ctx=ctx)
    # the context stays usable after a rejected file
    ok = b"%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 2 3\n"
    assert sv.CountMatrix.parse_mtx(ok, True, ctx=ctx).nnz == 1


def test_read_10x_directories(sv, ctx, tmp_path):
    A = rand_counts(400, 120, 0.05, 21)
    text = mm_text(A, shuffle=True, dup=30, seed=4)
    ref = mtx.parse(text, True)
    genes = [f"G_{i % 100}" for i in range(120)]
    barcodes = [f"AAAC{i:05d}-1" for i in range(400)]
    v2 = tmp_path / "v2"
    v2.mkdir()
    (v2 / "matrix.mtx").write_bytes(text)
    (v2 / "genes.tsv").write_text("".join(f"ENSG{i}\t{g}\n" for i, g in enumerate(genes)))
    (v2 / "barcodes.tsv").write_text("".join(b + "\n" for b in barcodes))
    v3 = tmp_path / "v3"
    v3.mkdir()
    with gzip.open(v3 / "matrix.mtx.gz", "wb") as f:
        f.write(text)
    with gzip.open(v3 / "features.tsv.gz", "wt") as f:
        f.write("".join(f"ENSG{i}\t{g}\tGene Expression\n" for i, g in enumerate(genes)))
    with gzip.open(v3 / "barcodes.tsv.gz", "wt") as f:
        f.write("".join(b + "\n" for b in barcodes))
    want_features = sv.make_unique([g.replace("_", "-") for g in genes])
    for d in (v2, v3):
        nc = sv.read_10X(str(d), ctx=ctx)
        check_both_copies(sv, nc.counts, ref)
        assert nc.barcodes == barcodes and nc.features == want_features
        assert sv.read_data(str(d), ctx=ctx).shape == (400, 120)
    with pytest.raises(sv.readers.ParseError_10X):
        sv.read_10X(str(tmp_path / "missing"), ctx=ctx)


def test_read_dge(sv, ctx, tmp_path):
    A = rand_counts(30, 20, 0.2, 2)
    genes = [f"g{i}" for i in range(20)]
    cells = [f"c{i}" for i in range(30)]
    text = mm_text(A, comments=("%%GENES\t" + "\t".join(genes), "%%CELL_BARCODES\t" + "\t".join(cells)))
    p = tmp_path / "x.dge.txt.gz"
    with gzip.open(p, "wb") as f:
        f.write(text)
    nc = sv.read_dge(str(p), ctx=ctx)
    assert nc.features == genes and nc.barcodes == cells
    check_both_copies(sv, nc.counts, mtx.parse(text, True))


def test_read_mtx_file_matches_parse(sv, ctx, tmp_path):
    A = rand_counts(5000, 800, 0.05, 8)
    text = mm_text(A, shuffle=True, seed=8)
    p = tmp_path / "m.mtx"
    p.write_bytes(text)
    X = sv.readMM(str(p), rows_are_features=True, ctx=ctx)
    check_both_copies(sv, X, mtx.parse(text, True))
    with pytest.raises(sv.SeveroGPUError, match="cannot open"):
        sv.readMM(str(tmp_path / "nope.mtx"), ctx=ctx)


def test_upload_csr_equals_csc(sv, ctx):
    """The features x barcodes CSC of a 10X HDF5 file (= cells x genes CSR) gives
    the same device matrix as the cells x genes CSC upload."""
    A = rand_counts(900, 300, 0.05, 13).tocsr()
    ref = A.tocsc()
    ref.sort_indices()
    Xr = sv.CountMatrix.upload_csr(A.indptr.astype(np.int64), A.indices.astype(np.int32),
                                   A.data.astype(np.int32), A.shape, ctx=ctx)
    check_both_copies(sv, Xr, ref)
    # unsorted features within cells, Int64 indices, 1-based, Float32 counts
    B = A.copy()
    rng = np.random.default_rng(0)
    for r in range(B.shape[0]):
        s, e = B.indptr[r], B.indptr[r + 1]
        perm = rng.permutation(e - s)
        B.indices[s:e] = B.indices[s:e][perm]
        B.data[s:e] = B.data[s:e][perm]
    Xu = sv.CountMatrix.upload_csr(B.indptr.astype(np.int32) + 1, B.indices.astype(np.int64) + 1,
                                   B.data.astype(np.float32), B.shape, index_base=1, ctx=ctx)
    check_both_copies(sv, Xu, ref)
    # Float64 counts through the CSC upload
    Xc = sv.CountMatrix.upload(ref.indptr, ref.indices, ref.data.astype(np.float64), ref.shape, ctx=ctx)
    check_both_copies(sv, Xc, ref)


@pytest.mark.parametrize("n_cells", [1_000_000, 2_000_000])
def test_upload_large_tiles(sv, ctx, n_cells):
    """The transpose's largest tiles (128 and 256 cells per warp) on a tall
    matrix: both device copies equal scipy's."""
    rng = np.random.default_rng(n_cells)
    n_genes = 70
    rows = rng.integers(0, n_cells, n_genes * n_cells // 10)
    cols = rng.integers(0, n_genes, rows.size)
    A = sp.csc_matrix((rng.integers(1, 9, rows.size).astype(np.int32), (rows, cols)),
                      shape=(n_cells, n_genes))
    A.sum_duplicates()
    A.sort_indices()
    X = sv.CountMatrix.upload(A.indptr.astype(np.int64), A.indices.astype(np.int32),
                              A.data.astype(np.int32), A.shape, ctx=ctx)
    check_both_copies(sv, X, A)


def test_upload_rejects_bad_counts(sv, ctx):
    ptr = np.array([0, 2, 3], np.int64)
    idx = np.array([0, 2, 1], np.int32)
    with pytest.raises(sv.SeveroGPUError, match="not an integer"):
        sv.CountMatrix.upload_csr(ptr, idx, np.array([1.0, 2.5, 3.0]), (2, 3), ctx=ctx)
    with pytest.raises(sv.SeveroGPUError, match="not an integer"):
        sv.CountMatrix.upload_csr(ptr, idx, np.array([1, -2, 3], np.int64), (2, 3), ctx=ctx)
    with pytest.raises(sv.SeveroGPUError, match="duplicate"):
        sv.CountMatrix.upload_csr(ptr, np.array([2, 2, 1], np.int32), np.array([1, 2, 3], np.int32),
                                  (2, 3), ctx=ctx)
    with pytest.raises(sv.SeveroGPUError, match="out of range"):
        sv.CountMatrix.upload_csr(ptr, np.array([0, 3, 1], np.int32), np.array([1, 2, 3], np.int32),
                                  (2, 3), ctx=ctx)
    with pytest.raises(sv.SeveroGPUError, match="pointer"):
        sv.CountMatrix.upload_csr(np.array([0, 4, 3], np.int64), idx, np.array([1, 2, 3], np.int32),
                                  (2, 3), ctx=ctx)
    X = sv.CountMatrix.upload_csr(ptr, idx, np.array([1, 2, 3], np.int32), (2, 3), ctx=ctx)
    assert np.array_equal(X.to_csc().toarray(), [[1, 0, 2], [0, 3, 0]])


def test_read_h5_formats_need_h5py(sv, ctx, tmp_path):
    h5py = pytest.importorskip("h5py")
    A = rand_counts(200, 50, 0.1, 3)
    T = A.T.tocsc()  # features x barcodes
    p = tmp_path / "x.h5"
    with h5py.File(p, "w") as f:
        g = f.create_group("mm10")
        g["indptr"], g["indices"], g["data"] = T.indptr, T.indices, T.data.astype(np.int32)
        g["shape"] = np.array(T.shape)
        g["barcodes"] = np.array([f"c{i}".encode() for i in range(200)])
        f.create_group("mm10/features")["name"] = np.array([f"g{i}".encode() for i in range(50)])
    nc = sv.read_10X_h5(str(p), ctx=ctx)
    ref = A.tocsc()
    ref.sort_indices()
    check_both_copies(sv, nc.counts, ref)
    assert os.path.exists(p)
