"""Count-matrix readers (src/input.jl) over the device loaders of libseverogpu.so.

The matrix itself never takes a host-side detour through a transposed copy:

    readMM / read_10X / read_geo / read_dge   MatrixMarket text streamed to HBM and
                                              parsed there (sv_counts_read_mtx)
    read_10X_h5 / read_h5 / read_h5ad         the stored compressed arrays uploaded
                                              as they are (sv_counts_upload_csr /
                                              sv_counts_upload_csc); needs h5py

Feature and barcode names are host strings and are handled here, as in
convert_counts (src/input.jl:776-790) and make_unique! (src/utils.jl:17-51).
"""
from __future__ import annotations

import gzip
import os
from dataclasses import dataclass, field

import numpy as np


class ParseError_10X(Exception):
    """A 10X directory or file that cannot be read (src/input.jl:154-156)."""


class ParseError_H5AD(Exception):
    """An AnnData file that cannot be read (src/input.jl:227-229)."""


@dataclass
class NamedCounts:
    """A device count matrix (cells x genes) with its labels, the NamedCountMatrix
    of src/Severo.jl:27."""
    counts: object
    barcodes: list = field(default_factory=list)
    features: list = field(default_factory=list)

    @property
    def shape(self):
        return self.counts.shape


def make_unique(names, sep="."):
    """Later duplicates get ".1", ".2", ... skipping names already present
    (make_unique!, src/utils.jl:17-51)."""
    names = list(names)
    n = len(names)
    seen = {}
    dup = [False] * n
    for i, x in enumerate(names):
        if x not in seen:
            seen[x] = 1
        else:
            dup[i] = True
    out = list(names)
    for i, x in enumerate(names):
        if dup[i]:
            cnt = seen[x]
            y = f"{x}{sep}{cnt}"
            while y in seen and cnt <= n:
                cnt += 1
                y = f"{x}{sep}{cnt}"
            out[i] = y
            seen[x] = cnt + 1
            seen[y] = 1
    return out


def convert_counts(X, features, barcodes, unique_features=True):
    """Labels a count matrix: "_" in feature names becomes "-", then names are
    made unique (convert_counts, src/input.jl:776-790)."""
    features = [str(f).replace("_", "-") for f in features]
    if unique_features:
        features = make_unique(features)
    return NamedCounts(X, [str(b) for b in barcodes], features)


def _open_text(fname):
    if str(fname).endswith(".gz"):
        return gzip.open(fname, "rt")
    return open(fname, "r")


def _readlines(fname):
    with _open_text(fname) as f:
        return [line.rstrip("\r\n") for line in f]


def _count_matrix():
    from . import CountMatrix
    return CountMatrix


def readMM(fname, rows_are_features=False, ctx=None):
    """A MatrixMarket coordinate file as a device count matrix (readMM,
    src/input.jl:27-115, 125-129).  With rows_are_features=False the file's rows
    are the cells; True transposes the 10X layout (features x barcodes)."""
    return _count_matrix().read_mtx(fname, rows_are_features=rows_are_features, ctx=ctx)


def _feature_names(feature_file, gene_column=2):
    """Column gene_column (1-based) of a tab-separated features / genes file."""
    return [line.split("\t")[gene_column - 1] for line in _readlines(feature_file) if line != ""]


def _read_10X(matrix_file, barcodes_file, feature_file, gene_column=2, ctx=None):
    if not (os.path.isfile(feature_file) and os.path.isfile(barcodes_file) and os.path.isfile(matrix_file)):
        raise ParseError_10X(f"Couldn't locate all components: {feature_file}, {barcodes_file}, {matrix_file}")
    X = _count_matrix().read_mtx(matrix_file, rows_are_features=True, ctx=ctx)
    barcodes = _readlines(barcodes_file)
    features = _feature_names(feature_file, gene_column)
    return X, features, barcodes


def read_10X(dirname, gene_column=2, unique_features=True, ctx=None):
    """A 10X directory (matrix.mtx, genes.tsv or features.tsv, barcodes.tsv;
    gzip-compressed for v3), src/input.jl:634-646 and _read_10X :199-208."""
    if not os.path.isdir(dirname):
        raise ParseError_10X(f"Directory {dirname} does not exist")
    is_v3 = os.path.isfile(os.path.join(dirname, "features.tsv.gz"))
    feature_file = os.path.join(dirname, "features.tsv.gz" if is_v3 else "genes.tsv")
    barcodes_file = os.path.join(dirname, "barcodes.tsv.gz" if is_v3 else "barcodes.tsv")
    matrix_file = os.path.join(dirname, "matrix.mtx.gz" if is_v3 else "matrix.mtx")
    X, features, barcodes = _read_10X(matrix_file, barcodes_file, feature_file, gene_column, ctx)
    return convert_counts(X, features, barcodes, unique_features=unique_features)


def read_geo(prefix, gene_column=2, unique_features=True, ctx=None):
    """GEO-style prefixed 10X files (src/input.jl:668-678)."""
    postfix = ".gz" if os.path.isfile(f"{prefix}matrix.mtx.gz") else ""
    X, features, barcodes = _read_10X(f"{prefix}matrix.mtx{postfix}", f"{prefix}barcodes.tsv{postfix}",
                                      f"{prefix}genes.tsv{postfix}", gene_column, ctx)
    return convert_counts(X, features, barcodes, unique_features=unique_features)


def _dge_names(fname):
    """Gene and barcode names from the %%GENES / %%CELL_BARCODES lines among the
    comments after the banner (parseMM_comments and the loop of _read_dge,
    src/input.jl:66-76,140-148)."""
    genes, barcodes = [], []
    with _open_text(fname) as f:
        f.readline()
        for line in f:
            line = line.rstrip("\r\n")
            if line != "" and line[0] != "%":
                break
            if line.startswith("%%GENES"):
                genes.extend(line.split("\t")[1:])
            elif line.startswith("%%CELL_BARCODES"):
                barcodes.extend(line.split("\t")[1:])
    return genes, barcodes


def read_dge(fname, unique_features=True, ctx=None):
    """A digital gene expression file: MatrixMarket with the gene and barcode
    names in %%GENES / %%CELL_BARCODES comment lines (_read_dge,
    src/input.jl:131-152; the reference's read_dge passes the wrong argument to
    it, this one reads fname)."""
    genes, barcodes = _dge_names(fname)
    X = _count_matrix().read_mtx(fname, rows_are_features=True, ctx=ctx)
    return convert_counts(X, genes, barcodes, unique_features=unique_features)


def _h5py(what):
    try:
        import h5py
    except ImportError as e:
        raise ImportError(f"{what} reads HDF5 through h5py, which is not installed") from e
    return h5py


def _strings(a):
    return [x.decode() if isinstance(x, bytes) else str(x) for x in np.asarray(a).ravel()]


def read_10X_h5(fname, dataset="/mm10", unique_features=True, ctx=None):
    """A 10X CellRanger HDF5 file (_read_10X_h5, src/input.jl:158-187): the
    stored features x barcodes CSC is the cells x genes CSR, uploaded as is."""
    h5py = _h5py("read_10X_h5")
    with h5py.File(fname, "r") as f:
        slot = "/gene_names" if "PYTABLES_FORMAT_VERSION" in f.attrs else "/features/name"
        if dataset not in f:
            raise ParseError_10X(f"Dataset {dataset} does not exist in {fname}")
        g = f[dataset]
        p, i, x = g["indptr"][()], g["indices"][()], g["data"][()]
        dim = g["shape"][()]
        features = _strings(f[dataset + slot][()])
        barcodes = _strings(g["barcodes"][()])
    X = _count_matrix().upload_csr(p, i, x, (int(dim[1]), int(dim[0])), 0, ctx)
    return convert_counts(X, features, barcodes, unique_features=unique_features)


def read_h5(fname, dataset="/counts", unique_features=True, ctx=None):
    """The "/counts" HDF5 layout (_read_h5, src/input.jl:210-225)."""
    h5py = _h5py("read_h5")
    with h5py.File(fname, "r") as f:
        if dataset not in f:
            raise ValueError(f"Dataset {dataset} does not exist in {fname}")
        g = f[dataset]
        p, i, x = g["indptr"][()], g["indices"][()], g["data"][()]
        dim = g["shape"][()]
        features = _strings(g["rownames"][()])
        barcodes = _strings(g["colnames"][()])
    X = _count_matrix().upload_csr(p, i, x, (int(dim[1]), int(dim[0])), 0, ctx)
    return convert_counts(X, features, barcodes, unique_features=unique_features)


def _h5ad_attr(attrs, desc, names, fname):
    for n in names:
        if n in attrs:
            v = attrs[n]
            return v.decode() if isinstance(v, bytes) else v
    raise ValueError(f"Cannot read {desc} information for count matrix in {fname}")


def _h5ad_index(obj):
    import h5py
    if isinstance(obj, h5py.Dataset):
        return _strings(obj[()]["index"])
    return _strings(obj["_index"][()])


def read_h5ad(fname, unique_features=True, ctx=None):
    """An AnnData file (_read_h5ad, src/input.jl:250-287): a csr X is uploaded as
    the cell-major copy, a csc X as the gene-major copy."""
    h5py = _h5py("read_h5ad")
    with h5py.File(fname, "r") as f:
        if "X" not in f:
            raise ValueError(f"Count data not found in {fname}")
        a = f["X"].attrs
        dim = _h5ad_attr(a, "shape", ["shape", "h5sparse_shape"], fname)
        fmt = _h5ad_attr(a, "format", ["encoding-type", "h5sparse_format"], fname)
        p, i, x = f["X/indptr"][()], f["X/indices"][()], f["X/data"][()]
        barcodes = _h5ad_index(f["obs"])
        features = _h5ad_index(f["var"])
    CM = _count_matrix()
    shape = (int(dim[0]), int(dim[1]))
    if fmt in ("csr", "csr_matrix"):
        X = CM.upload_csr(p, i, x, shape, 0, ctx)
    else:
        X = CM.upload(p, i, x, shape, 0, ctx)
    return convert_counts(X, features, barcodes, unique_features=unique_features)


def read_data(path, **kw):
    """Picks the reader from the path (read_data, src/input.jl:734-758): a
    directory is a 10X directory; .h5ad, .h5 and .dge.txt[.gz] files by suffix.
    Loom and CSV files are not read by this package."""
    if not os.path.exists(path):
        raise FileNotFoundError(f"path {path} does not point to anything")
    if os.path.isdir(path):
        return read_10X(path, **kw)
    p = str(path)
    if p.endswith(".h5ad"):
        return read_h5ad(p, **kw)
    if p.endswith(".h5"):
        return read_10X_h5(p, **kw)
    if p.endswith(".dge.txt.gz") or p.endswith(".dge.txt"):
        return read_dge(p, **kw)
    if p.endswith(".mtx") or p.endswith(".mtx.gz"):
        return convert_counts(readMM(p, rows_are_features=True, ctx=kw.get("ctx")), [], [])
    raise ValueError(f"unknown format {path}")
