// normalize_cells over a device CSC without any allocation by the library.
//
// Some callers cannot let a library call cudaMalloc: a host runtime that has
// already reserved the device memory budget in its own pool (a garbage-collected
// language runtime such as Julia's, handing out device arrays from its pool), or
// a service that must not allocate device memory once it has started.  This
// entry point takes the count matrix and the output as device arrays owned by
// the caller and keeps its only scratch -- the per-cell totals -- in the
// file-scope array below, sized for at most SV_NOALLOC_MAX_CELLS cells (16 MiB,
// held by every GPU that loads the library until the process exits), plus one
// file-scope status word.
#include "sv_internal.cuh"

namespace {

constexpr int64_t SV_NOALLOC_MAX_CELLS = 2097152;

// per-cell totals shared by every call on a device
static __device__ __align__(256) unsigned long long g_cell_totals[SV_NOALLOC_MAX_CELLS];
// set to 1 by a call that met a row index outside [0, n_cells)
static __device__ __align__(256) int g_noalloc_status;

struct NoallocSyms {
  unsigned long long* totals = nullptr;
  int* status = nullptr;
};
std::mutex g_sym_mu;
NoallocSyms g_sym[64];   // device addresses of the two arrays, per device ordinal

__global__ void k_totals_scatter(const int32_t* __restrict__ rowidx, const int32_t* __restrict__ cnt,
                                 int64_t nnz, int64_t n_cells,
                                 unsigned long long* __restrict__ totals, int* __restrict__ status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz;
       i += (int64_t)gridDim.x * blockDim.x) {
    int32_t r = rowidx[i];
    if (r < 0 || (int64_t)r >= n_cells) {   // skipped and reported, never written
      *status = 1;
      continue;
    }
    atomicAdd(&totals[r], (unsigned long long)(long long)cnt[i]);
  }
}

// b = (sf * a) / s_cell in FP32 (src/normalize.jl:27), log1p for :lognormalize (:36)
__global__ void k_values_static(const int32_t* __restrict__ rowidx, const int32_t* __restrict__ cnt,
                                int64_t nnz, int64_t n_cells,
                                const unsigned long long* __restrict__ totals, float sf, int log,
                                float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz;
       i += (int64_t)gridDim.x * blockDim.x) {
    int32_t r = rowidx[i];
    if (r < 0 || (int64_t)r >= n_cells) {   // the call fails; leave a defined value
      out[i] = 0.0f;
      continue;
    }
    float v = (sf * (float)cnt[i]) / (float)(long long)totals[r];
    out[i] = log ? log1pf(v) : v;
  }
}

}  // namespace

SV_API int sv_normalize_csc_noalloc(const int64_t* colptr, const int32_t* rowval,
                                    const int32_t* counts, int64_t n_cells, int64_t n_genes,
                                    int64_t nnz, int method, double scale_factor, float* values,
                                    void* stream) {
  SV_TRY
  (void)colptr;   // the values depend on the row of each entry only
  SV_REQUIRE(n_cells >= 1 && n_genes >= 1 && nnz >= 0, "bad sizes");
  if (n_cells > SV_NOALLOC_MAX_CELLS)
    sv_throw(SV_ERR_ARG, "sv_normalize_csc_noalloc handles at most %lld cells (got %lld)",
             (long long)SV_NOALLOC_MAX_CELLS, (long long)n_cells);
  if (method != SV_LOGNORMALIZE && method != SV_RELATIVECOUNTS)
    sv_throw(SV_ERR_ARG, "unknown normalization method: %d", method);
  SV_REQUIRE(nnz == 0 || (rowval && counts && values), "null array");
  int dev = 0;
  SV_CUDA(cudaGetDevice(&dev));
  SV_REQUIRE(dev >= 0 && dev < 64, "device index out of range");
  NoallocSyms sym;
  {
    // once per device, with that device current: the device addresses of the
    // file-scope arrays (their host-side names are not device addresses)
    std::lock_guard<std::mutex> lk(g_sym_mu);
    if (!g_sym[dev].totals) {
      void* p = nullptr;
      void* q = nullptr;
      SV_CUDA(cudaGetSymbolAddress(&p, g_cell_totals));
      SV_CUDA(cudaGetSymbolAddress(&q, g_noalloc_status));
      g_sym[dev].totals = (unsigned long long*)p;
      g_sym[dev].status = (int*)q;
    }
    sym = g_sym[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  // the arrays keep the previous call's contents: clear what this call uses
  SV_CUDA(cudaMemsetAsync(sym.totals, 0, (size_t)n_cells * sizeof(unsigned long long), s));
  SV_CUDA(cudaMemsetAsync(sym.status, 0, sizeof(int), s));
  if (nnz > 0) {
    int blocks = 1216;
    k_totals_scatter<<<blocks, 256, 0, s>>>(rowval, counts, nnz, n_cells, sym.totals, sym.status);
    SV_CUDA(cudaGetLastError());
    k_values_static<<<blocks, 256, 0, s>>>(rowval, counts, nnz, n_cells, sym.totals,
                                           (float)scale_factor, method == SV_LOGNORMALIZE, values);
    SV_CUDA(cudaGetLastError());
    // the status word decides the return code, so the call waits for its work
    int h_status = 0;
    SV_CUDA(cudaMemcpyAsync(&h_status, sym.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    SV_CUDA(cudaStreamSynchronize(s));
    if (h_status)
      sv_throw(SV_ERR_ARG, "sv_normalize_csc_noalloc: a row index is outside [0, %lld)",
               (long long)n_cells);
  }
  SV_CATCH
}
