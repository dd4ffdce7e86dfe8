"""Writes tests/golden/golden.json: the literal fixtures of Severo.jl's own tests for
this path, with the expected values those tests assert, evaluated from the tests'
own right-hand-side expressions (plain dense numpy, independent of the oracle).

Sources (Severo.jl project paths):
  test/test_input.jl:19-43    filter_counts(min_features=1, min_cells=2, min_umi=2)
                              on the 10 x 5 count literal keeps cells 1,2,3,4,5,8,9
                              and genes 1,2,4,5 (:40-42).
  test/test_input.jl:45-101   normalize_cells on the 10 x 5 count literal, after
                              filter_counts(min_features=1, min_cells=2, min_umi=2),
                              whose result the test pins as cells 1,2,3,4,5,8,9 and
                              genes 1,2,4,5 (:40-42).  Expected: row sums 1 and 10
                              (:64,:74), log1p of the relative counts (:70).
  test/test_scaling.jl:20-67  scale_features on the same literal (no filtering):
                              S.mu == mean/std (:43), convert(Matrix, S) ==
                              (X - mean)/std (:44) with scale_max = Inf.
  test/test_scaling.jl:70-113 the 4 x 3 CenteredMatrix with mu, r, y0 and the
                              sequence of mul! calls (y is updated in place).
  test/test_scaling.jl:115-131 grouped mean_var of a sparse vector.
  SNN: hand-built neighbour lists; counts by explicit set intersection.

Run: python tests/golden/make_golden.py
"""
import json
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

X10 = np.array([
    [0, 0, 0, 3, 0],
    [0, 1, 0, 0, 6],
    [5, 0, 0, 0, 0],
    [3, 0, 0, 0, 0],
    [0, 0, 6, 2, 0],
    [0, 0, 0, 0, 0],
    [0, 0, 0, 0, 2],
    [0, 3, 0, 0, 0],
    [0, 0, 0, 0, 3],
    [2, 0, 0, 0, 0],
], dtype=np.int64)


def normalize_fixture():
    cells = np.array([1, 2, 3, 4, 5, 8, 9]) - 1
    genes = np.array([1, 2, 4, 5]) - 1
    C = X10[np.ix_(cells, genes)]
    s = C.sum(axis=1, keepdims=True)
    rel = C / s                       # the test's row-sum identity: rows sum to 1
    out = {
        "counts": C.tolist(),
        "relative": rel.tolist(),
        "relative_sf10": (10.0 * C / s).tolist(),
        "log": np.log1p(rel).tolist(),
    }
    return out


def filter_fixture():
    return {"counts": X10.tolist(), "min_features": 1, "min_cells": 2, "min_umi": 2,
            "cells": [1, 2, 3, 4, 5, 8, 9], "genes": [1, 2, 4, 5],
            "filtered": X10[np.ix_(np.array([1, 2, 3, 4, 5, 8, 9]) - 1,
                                   np.array([1, 2, 4, 5]) - 1)].tolist()}


def scaling_fixture():
    X = X10.astype(np.float64)
    mean = X.mean(axis=0)
    std = X.std(axis=0, ddof=1)
    return {
        "counts": X10.tolist(),
        "mean": mean.tolist(),
        "std": std.tolist(),
        "mu": (mean / std).tolist(),
        "dense": ((X - mean) / std).tolist(),
    }


def centered_fixture():
    A = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1]], dtype=np.float64)
    mu = np.array([0.1, 0.2, 0.3])
    Q = A - mu
    r0 = np.array([0.991, 0.228, 0.291])
    y0 = np.array([0.820, 0.430, 0.264, 0.789])
    # dense testset: y1 = 2Qr + y0 ; C'y1 ; 2Q'y1 + r0
    y1 = 2 * Q @ r0 + y0
    dense = {"Cr": (Q @ r0).tolist(), "y1": y1.tolist(), "Cty": (Q.T @ y1).tolist(),
             "r1": (2 * Q.T @ y1 + r0).tolist()}
    # sparse testset: a second mul!(y, C, r, 2, 1) runs inside @allocated (:106)
    y2 = 2 * Q @ r0 + y1
    sparse = {"Cr": (Q @ r0).tolist(), "y1": y1.tolist(), "y2": y2.tolist(),
              "Cty": (Q.T @ y2).tolist(), "r1": (2 * Q.T @ y2 + r0).tolist()}
    return {"A": A.tolist(), "mu": mu.tolist(), "r": r0.tolist(), "y0": y0.tolist(),
            "dense": dense, "sparse": sparse}


def grouped_fixture():
    idx = [3, 4, 5, 10, 11, 17, 18, 26, 31, 34, 37, 38, 40, 46, 50, 54, 66, 74, 86]
    val = [2, 2, 1, 1, 2, 2, 19, 2, 6, 13, 6, 2, 9, 4, 12, 2, 21, 10, 12]
    x = np.zeros(100)
    x[np.array(idx) - 1] = val
    cases = []
    lbl1 = np.array([1] * 10 + [2] * 90)
    lbl2 = np.random.default_rng(20261203).integers(1, 5, 100)
    for lb, nl in ((lbl1, 2), (lbl2, 4)):
        mu = [float(x[lb == i].mean()) for i in range(1, nl + 1)]
        var = [float(x[lb == i].var(ddof=1)) for i in range(1, nl + 1)]
        n = [int((lb == i).sum()) for i in range(1, nl + 1)]
        cases.append({"labels": lb.tolist(), "nlabels": nl, "mu": mu, "var": var, "n": n})
    return {"n": 100, "idx": idx, "val": val, "cases": cases}


def snn_fixture():
    """Hand-built kNN lists (1-based), expected Jaccard graphs by set intersection."""
    nn = np.array([
        [1, 2, 3],
        [2, 1, 3],
        [3, 1, 4],
        [4, 3, 5],
        [5, 4, 6],
        [6, 5, 4],
        [7, 6, 5],
    ], dtype=np.int64)
    n, k = nn.shape
    N = [set(row) for row in nn]
    out = {"nn_index": nn.tolist(), "k": k, "cases": []}
    for prune in (0.0, 1.0 / 15.0, 0.3):
        rows, cols, vals = [], [], []
        for j in range(n):
            for i in range(n):
                c = len(N[i] & N[j])
                if c == 0:
                    continue
                w = c / (k + (k - c))
                if abs(w) > prune:
                    rows.append(i + 1)
                    cols.append(j + 1)
                    vals.append(w)
        out["cases"].append({"prune": prune, "rows": rows, "cols": cols, "vals": vals})
    return out


def main():
    data = {
        "filter": filter_fixture(),
        "normalize": normalize_fixture(),
        "scaling": scaling_fixture(),
        "centered": centered_fixture(),
        "mean_var_grouped": grouped_fixture(),
        "snn": snn_fixture(),
    }
    (HERE / "golden.json").write_text(json.dumps(data, indent=1))
    print("wrote", HERE / "golden.json")


if __name__ == "__main__":
    main()
