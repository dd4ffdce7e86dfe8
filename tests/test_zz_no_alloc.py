"""GPU test of sv_normalize_csc_noalloc, the normalisation entry point that
allocates nothing (for callers that keep the device memory budget in their own
pool, or record work inside a stream capture, and so cannot let the library call
cudaMalloc).  Its only scratch, the per-cell totals, lives in a file-scope device
array shared by every call.

Called through the C ABI with caller-owned device arrays; each result is checked
against the existing entry point (sv_normalize_cells, FP32 values) within the
FP32 normalisation tolerance of the other tests, on two calls in a row -- the
second on a smaller matrix, so totals left in the shared array by the first call
would show.  Collected last, so that a stop at the first failure has run every
other test; it runs alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _noalloc(sv, torch, X, method, sf):
    lib = sv._lib.load()
    cp = _device(torch, X.indptr.astype(np.int64))
    rv = _device(torch, X.indices.astype(np.int32))
    ct = _device(torch, X.data.astype(np.int32))
    out = torch.empty(X.nnz, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = lib.sv_normalize_csc_noalloc(
        C.c_void_p(cp.data_ptr()), C.c_void_p(rv.data_ptr()), C.c_void_p(ct.data_ptr()),
        X.shape[0], X.shape[1], X.nnz, 0 if method == "lognormalize" else 1, sf,
        C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    sv._lib.check(st)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("method", ["lognormalize", "relativecounts"])
def test_noalloc_matches_allocating_entry_point(sv, ctx, O, method):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    big = O.synth_counts(4000, 1500, -1.0, 1.5, depth=0.5, seed=101)
    small = O.synth_counts(1200, 900, -1.0, 1.5, depth=0.8, seed=102)
    for X in (big, small):                      # two calls in a row
        got = _noalloc(sv, torch, X, method, 1e4)
        want = sv.normalize_cells(X, method=method, scale_factor=1e4, dtype="float32",
                                  ctx=ctx).values_csc()
        assert got.dtype == np.float32 and got.shape == want.shape
        assert np.allclose(got, want, rtol=1e-6, atol=0)


def test_noalloc_rejects_too_many_cells(sv):
    lib = sv._lib.load()
    st = lib.sv_normalize_csc_noalloc(None, None, None, 2097153, 10, 0, 0, 1.0, None, None)
    assert st == sv._lib.SV_ERR_ARG
    assert "at most 2097152 cells" in sv._lib.last_error()
