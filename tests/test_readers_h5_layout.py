"""The HDF5 file layer of the readers (src/input.jl:158-187 _read_10X_h5,
src/input.jl:210-225 _read_h5, src/input.jl:231-287 _read_h5ad) on the CPU.

h5py is installed on neither machine, so the HDF5 decoding itself cannot run
here.  These tests put an in-memory stand-in for h5py's File / Group / Dataset
in its place and a recording stand-in for the device upload, and check the part
that is this package's: which datasets and attributes are read, how the stored
arrays map onto the cells x genes matrix (a 10X features x barcodes CSC is the
cells x genes CSR; an AnnData csr X is cell-major, a csc X gene-major), the
feature-name slot of the two CellRanger versions, the label clean-up, and the
reference's errors and messages.
"""
import sys
import types

import numpy as np
import pytest
import scipy.sparse as sp

import __graft_entry__ as ge


class _Node:
    def __init__(self, attrs=None):
        self.attrs = dict(attrs or {})


class FakeDataset(_Node):
    def __init__(self, data, attrs=None):
        super().__init__(attrs)
        self._data = data

    def __getitem__(self, key):
        if key == ():
            return self._data
        return self._data[key]


class FakeGroup(_Node):
    def __init__(self, children=None, attrs=None):
        super().__init__(attrs)
        self._children = dict(children or {})

    def _walk(self, path):
        node = self
        for part in [p for p in str(path).split("/") if p]:
            if not isinstance(node, FakeGroup) or part not in node._children:
                return None
            node = node._children[part]
        return node

    def __contains__(self, path):
        return self._walk(path) is not None

    def __getitem__(self, path):
        node = self._walk(path)
        if node is None:
            raise KeyError(path)
        return node


FILES = {}


class FakeFile(FakeGroup):
    def __init__(self, fname, mode="r"):
        root = FILES[str(fname)]
        super().__init__(root._children, root.attrs)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


class Upload:
    """Records what the reader hands to the device loader."""

    def __init__(self, kind, ptr, idx, val, shape):
        self.kind, self.ptr, self.idx, self.val, self.shape = kind, ptr, idx, val, shape

    def dense(self):
        """The cells x genes matrix the device would hold."""
        n_cells, n_genes = self.shape
        if self.kind == "csr":
            return sp.csr_matrix((self.val, self.idx, self.ptr), shape=(n_cells, n_genes)).toarray()
        return sp.csc_matrix((self.val, self.idx, self.ptr), shape=(n_cells, n_genes)).toarray()


class FakeCountMatrix:
    @classmethod
    def upload_csr(cls, rowptr, colidx, nzval, shape, index_base=0, ctx=None):
        assert index_base == 0
        return Upload("csr", rowptr, colidx, nzval, shape)

    @classmethod
    def upload(cls, colptr, rowval, nzval, shape, index_base=0, ctx=None):
        assert index_base == 0
        return Upload("csc", colptr, rowval, nzval, shape)


@pytest.fixture
def readers(monkeypatch):
    fake = types.ModuleType("h5py")
    fake.File, fake.Group, fake.Dataset = FakeFile, FakeGroup, FakeDataset
    monkeypatch.setitem(sys.modules, "h5py", fake)
    R = ge.load_package().readers
    monkeypatch.setattr(R, "_count_matrix", lambda: FakeCountMatrix)
    FILES.clear()
    return R


def _counts(n_cells=7, n_genes=5, seed=0):
    rng = np.random.default_rng(seed)
    A = rng.poisson(0.8, (n_cells, n_genes)).astype(np.int32)
    A[2, :] = 0                       # an empty cell
    return A


def _tenx_file(A, version=3, dataset="mm10"):
    """CellRanger layout: the features x barcodes CSC (0-based) under /dataset,
    shape = (features, barcodes); v3 names under features/name, v2 under gene_names
    with the PyTables attribute on the root."""
    n_cells, n_genes = A.shape
    F = sp.csc_matrix(A.T)            # features x barcodes
    genes = np.array([b"Gene_A", b"Gene_B", b"Gene_A", b"Mt_1", b"Gene_A.1"][:n_genes])
    g = {"indptr": FakeDataset(F.indptr.astype(np.int64)),
         "indices": FakeDataset(F.indices.astype(np.int64)),
         "data": FakeDataset(F.data.astype(np.int32)),
         "shape": FakeDataset(np.array([n_genes, n_cells], np.int32)),
         "barcodes": FakeDataset(np.array([f"AAAC-{c}".encode() for c in range(n_cells)]))}
    attrs = {}
    if version == 3:
        g["features"] = FakeGroup({"name": FakeDataset(genes)})
    else:
        g["gene_names"] = FakeDataset(genes)
        attrs["PYTABLES_FORMAT_VERSION"] = b"2.1"
    return FakeGroup({dataset: FakeGroup(g)}, attrs)


@pytest.mark.parametrize("version", [3, 2])
def test_read_10X_h5_layout(readers, version):
    A = _counts()
    FILES["x.h5"] = _tenx_file(A, version)
    nc = readers.read_10X_h5("x.h5")
    up = nc.counts
    assert up.kind == "csr" and up.shape == A.shape
    assert np.array_equal(up.dense(), A)
    # "_" -> "-", then make_unique (src/input.jl:776-790, src/utils.jl:17-51): the
    # duplicate skips "Gene-A.1", which another feature already has
    assert nc.features == ["Gene-A", "Gene-B", "Gene-A.2", "Mt-1", "Gene-A.1"]
    assert nc.barcodes == [f"AAAC-{c}" for c in range(A.shape[0])]
    assert readers.read_10X_h5("x.h5", unique_features=False).features[2] == "Gene-A"


def test_read_10X_h5_missing_dataset(readers):
    FILES["x.h5"] = _tenx_file(_counts(), 3, dataset="GRCh38")
    with pytest.raises(readers.ParseError_10X, match="Dataset /mm10 does not exist in x.h5"):
        readers.read_10X_h5("x.h5")
    assert readers.read_10X_h5("x.h5", dataset="/GRCh38").counts.shape == (7, 5)


def test_read_h5_layout(readers):
    A = _counts(seed=1)
    F = sp.csc_matrix(A.T)
    FILES["c.h5"] = FakeGroup({"counts": FakeGroup({
        "indptr": FakeDataset(F.indptr), "indices": FakeDataset(F.indices),
        "data": FakeDataset(F.data), "shape": FakeDataset(np.array([A.shape[1], A.shape[0]])),
        "rownames": FakeDataset(np.array([b"g1", b"g2", b"g1", b"g_4", b"g5"])),
        "colnames": FakeDataset(np.array([f"c{c}".encode() for c in range(A.shape[0])]))})})
    nc = readers.read_h5("c.h5")
    assert nc.counts.kind == "csr" and np.array_equal(nc.counts.dense(), A)
    assert nc.features == ["g1", "g2", "g1.1", "g-4", "g5"]
    with pytest.raises(ValueError, match="Dataset /other does not exist"):
        readers.read_h5("c.h5", dataset="/other")


def _h5ad_file(A, fmt="csr", new_attrs=True, compound_index=False):
    n_cells, n_genes = A.shape
    M = sp.csr_matrix(A) if fmt == "csr" else sp.csc_matrix(A)
    if new_attrs:
        attrs = {"shape": np.array([n_cells, n_genes]), "encoding-type": fmt}
    else:
        attrs = {"h5sparse_shape": np.array([n_cells, n_genes]), "h5sparse_format": fmt.encode()}
    X = FakeGroup({"indptr": FakeDataset(M.indptr), "indices": FakeDataset(M.indices),
                   "data": FakeDataset(M.data.astype(np.float32))}, attrs)
    cells = [f"cell_{c}".encode() for c in range(n_cells)]
    genes = [f"G{g % 3}".encode() for g in range(n_genes)]
    if compound_index:                # old AnnData: obs / var as compound datasets
        obs = FakeDataset(np.array([(c,) for c in cells], dtype=[("index", "S16")]))
        var = FakeDataset(np.array([(g,) for g in genes], dtype=[("index", "S16")]))
    else:
        obs = FakeGroup({"_index": FakeDataset(np.array(cells))})
        var = FakeGroup({"_index": FakeDataset(np.array(genes))})
    return FakeGroup({"X": X, "obs": obs, "var": var})


@pytest.mark.parametrize("fmt", ["csr", "csc"])
@pytest.mark.parametrize("new_attrs", [True, False])
@pytest.mark.parametrize("compound_index", [False, True])
def test_read_h5ad_layout(readers, fmt, new_attrs, compound_index):
    A = _counts(6, 5, seed=2)
    FILES["a.h5ad"] = _h5ad_file(A, fmt, new_attrs, compound_index)
    nc = readers.read_h5ad("a.h5ad")
    up = nc.counts
    # csr X -> the cell-major copy; csc X -> the gene-major copy (src/input.jl:267-272)
    assert up.kind == fmt and up.shape == A.shape
    assert np.array_equal(up.dense(), A)
    assert nc.barcodes == [f"cell_{c}" for c in range(6)]
    assert nc.features == ["G0", "G1", "G2", "G0.1", "G1.1"]


def test_read_h5ad_errors(readers):
    FILES["none.h5ad"] = FakeGroup({"obs": FakeGroup()})
    with pytest.raises(ValueError, match="Count data not found in none.h5ad"):
        readers.read_h5ad("none.h5ad")
    f = _h5ad_file(_counts(6, 5))
    f["X"].attrs.pop("shape")
    FILES["noshape.h5ad"] = f
    with pytest.raises(ValueError, match="Cannot read shape information for count matrix in noshape.h5ad"):
        readers.read_h5ad("noshape.h5ad")
    f = _h5ad_file(_counts(6, 5))
    f["X"].attrs.pop("encoding-type")
    FILES["nofmt.h5ad"] = f
    with pytest.raises(ValueError, match="Cannot read format information"):
        readers.read_h5ad("nofmt.h5ad")


def test_read_data_dispatch(readers, tmp_path):
    A = _counts()
    p = tmp_path / "d.h5"
    p.write_bytes(b"")
    FILES[str(p)] = _tenx_file(A)
    assert np.array_equal(readers.read_data(str(p)).counts.dense(), A)
    q = tmp_path / "d.h5ad"
    q.write_bytes(b"")
    FILES[str(q)] = _h5ad_file(A)
    assert np.array_equal(readers.read_data(str(q)).counts.dense(), A)
    with pytest.raises(FileNotFoundError):
        readers.read_data(str(tmp_path / "missing.h5"))
