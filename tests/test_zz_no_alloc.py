"""GPU test of sv_normalize_csc_noalloc, the normalisation entry point that
allocates nothing.  It is there for callers that cannot let the library call
cudaMalloc: a host runtime that keeps the whole device memory budget in its own
pool (Julia's device arrays come from one), or a service that must not allocate
device memory once started.  Its only scratch, the per-cell totals, lives in a
file-scope device array shared by every call, beside a file-scope status word.

Called through the C ABI with caller-owned device arrays; each result is checked
against the existing entry point (sv_normalize_cells, FP32 values) and against
the oracle, within the FP32 normalisation tolerance of the other tests (1e-6
relative), on two calls in a row -- the second on a smaller matrix, so totals
left in the shared array by the first call would show.  A row index out of range
is skipped by the kernels and reported as SV_ERR_ARG.  Collected last, so that a
stop at the first failure has run every other test; it runs alone in a fresh
process as well."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-6


def _device(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _noalloc(sv, torch, indptr, indices, data, shape, method, sf):
    """One call through the C ABI; returns (status, values)."""
    lib = sv._lib.load()
    cp = _device(torch, np.asarray(indptr, dtype=np.int64))
    rv = _device(torch, np.asarray(indices, dtype=np.int32))
    ct = _device(torch, np.asarray(data, dtype=np.int32))
    nnz = len(indices)
    out = torch.full((max(nnz, 1),), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = lib.sv_normalize_csc_noalloc(
        C.c_void_p(cp.data_ptr()), C.c_void_p(rv.data_ptr()), C.c_void_p(ct.data_ptr()),
        shape[0], shape[1], nnz, 0 if method == "lognormalize" else 1, sf,
        C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    torch.cuda.synchronize()
    return st, out[:nnz].cpu().numpy()


def _skip_without_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("method", ["lognormalize", "relativecounts"])
def test_noalloc_matches_allocating_entry_point(sv, ctx, O, method):
    torch = _skip_without_gpu()
    big = O.synth_counts(4000, 1500, -1.0, 1.5, depth=0.5, seed=101)
    small = O.synth_counts(1200, 900, -1.0, 1.5, depth=0.8, seed=102)
    for X in (big, small):                      # two calls in a row
        st, got = _noalloc(sv, torch, X.indptr, X.indices, X.data, X.shape, method, 1e4)
        sv._lib.check(st)
        want = sv.normalize_cells(X, method=method, scale_factor=1e4, dtype="float32",
                                  ctx=ctx).values_csc()
        oracle = O.normalize_cells(X, method, 1e4, np.float32).data
        assert got.dtype == np.float32 and got.shape == want.shape == oracle.shape
        assert np.allclose(got, want, rtol=RTOL, atol=0)
        assert np.allclose(got, oracle, rtol=RTOL, atol=0)


def test_noalloc_reports_row_out_of_range(sv, O):
    """A row index >= n_cells is skipped (no write outside the totals of this
    call's cells) and the call fails with SV_ERR_ARG; the next call is clean."""
    torch = _skip_without_gpu()
    X = O.synth_counts(500, 200, -1.0, 1.5, depth=0.8, seed=103)
    bad = X.indices.copy()
    bad[len(bad) // 2] = X.shape[0]             # one entry names the cell after the last
    st, _ = _noalloc(sv, torch, X.indptr, bad, X.data, X.shape, "lognormalize", 1e4)
    assert st == sv._lib.SV_ERR_ARG
    assert "outside [0, 500)" in sv._lib.last_error()
    st, got = _noalloc(sv, torch, X.indptr, X.indices, X.data, X.shape, "lognormalize", 1e4)
    sv._lib.check(st)
    assert np.allclose(got, O.normalize_cells(X, "lognormalize", 1e4, np.float32).data,
                       rtol=RTOL, atol=0)


def test_noalloc_rejects_too_many_cells(sv):
    lib = sv._lib.load()
    st = lib.sv_normalize_csc_noalloc(None, None, None, 2097153, 10, 0, 0, 1.0, None, None)
    assert st == sv._lib.SV_ERR_ARG
    assert "at most 2097152 cells" in sv._lib.last_error()
