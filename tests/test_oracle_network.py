"""The oracle's Network(snn) (src/modularity.jl:163-194) on the golden SNN graphs."""
import json
from pathlib import Path

import numpy as np
import scipy.sparse as sp

G = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())


def test_network_of_golden_snn(O):
    s = G["snn"]
    n = len(s["nn_index"])
    for case in s["cases"]:
        A = sp.csc_matrix((case["vals"], (np.array(case["rows"]) - 1, np.array(case["cols"]) - 1)),
                          shape=(n, n))
        A.sort_indices()
        nw, first, last, en, ew, totw = O.network(A)
        D = A.toarray()
        off = D - np.diag(np.diag(D))
        assert np.allclose(nw, off.sum(axis=0))
        assert len(en) == A.nnz - np.count_nonzero(np.diag(D))
        assert np.all(last - first + 1 == (off != 0).sum(axis=0))
        assert np.isclose(totw, off.sum())
        assert not np.any(en - 1 == np.repeat(np.arange(n), last - first + 1))
