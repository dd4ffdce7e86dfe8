// Internal definitions shared by the translation units of libseverogpu.so.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <string>
#include <vector>
#include <map>
#include <mutex>
#include <tuple>
#include <algorithm>

#include "../../include/severo_gpu.h"

#define SV_API extern "C" __attribute__((visibility("default")))

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
void sv_set_error(const char* fmt, ...);

struct SvError {
  int code;
};

#define SV_TRY try {
#define SV_CATCH                       \
  }                                    \
  catch (const SvError& e) {           \
    return e.code;                     \
  }                                    \
  catch (...) {                        \
    sv_set_error("unexpected C++ exception"); \
    return SV_ERR_CUDA;                \
  }                                    \
  return SV_OK;

[[noreturn]] void sv_throw(int code, const char* fmt, ...);

#define SV_REQUIRE(cond, ...)                          \
  do {                                                 \
    if (!(cond)) sv_throw(SV_ERR_ARG, __VA_ARGS__);    \
  } while (0)

#define SV_CUDA(call)                                                          \
  do {                                                                         \
    cudaError_t _e = (call);                                                   \
    if (_e != cudaSuccess) {                                                   \
      if (_e == cudaErrorMemoryAllocation) {                                   \
        cudaGetLastError();                                                    \
        sv_throw(SV_ERR_OOM, "%s:%d %s: %s", __FILE__, __LINE__, #call,        \
                 cudaGetErrorString(_e));                                      \
      }                                                                        \
      sv_throw(SV_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,         \
               cudaGetErrorString(_e));                                        \
    }                                                                          \
  } while (0)

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct SvTimedLaunch {
  std::string name;
  cudaEvent_t a, b;
};

struct sv_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  bool profiling = false;
  std::vector<SvTimedLaunch> pending;             // events not yet harvested
  std::map<std::string, std::pair<double, int64_t>> prof;  // name -> (ms, count)
  std::vector<cudaEvent_t> event_pool;
  cudaEvent_t marks[16] = {};
  // device status word written by kernels that detect a bounds / limit failure
  int* d_status = nullptr;
  // small pinned staging buffer for scalar read-backs
  void* h_stage = nullptr;
  size_t h_stage_bytes = 0;
  // two pinned staging buffers for streamed uploads (file readers), kept
  // between calls
  void* h_io[2] = {nullptr, nullptr};
  size_t h_io_bytes = 0;
  cudaEvent_t h_io_ev[2] = {nullptr, nullptr};   // last transfer from / into each buffer
};

void sv_ctx_check(sv_context* ctx);
cudaEvent_t sv_ctx_event(sv_context* ctx);
void sv_ctx_harvest(sv_context* ctx);
void* sv_ctx_stage(sv_context* ctx, size_t bytes);
void sv_check_device_status(sv_context* ctx, const char* where);

// Launch a kernel on the context stream; counts launches and, when profiling
// is on, brackets it with events.
template <typename Kern, typename... Args>
inline void sv_launch(sv_context* ctx, const char* name, Kern kernel, dim3 grid, dim3 block,
                      size_t smem, Args... args) {
  if (grid.x == 0 || grid.y == 0 || grid.z == 0) return;
  cudaEvent_t a = nullptr, b = nullptr;
  if (ctx->profiling) {
    a = sv_ctx_event(ctx);
    b = sv_ctx_event(ctx);
    SV_CUDA(cudaEventRecord(a, ctx->stream));
  }
  kernel<<<grid, block, smem, ctx->stream>>>(args...);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) sv_throw(SV_ERR_CUDA, "launch of %s failed: %s", name, cudaGetErrorString(e));
  ctx->launches++;
  if (ctx->profiling) {
    SV_CUDA(cudaEventRecord(b, ctx->stream));
    ctx->pending.push_back({name, a, b});
  }
}

// ---------------------------------------------------------------------------
// device memory
// ---------------------------------------------------------------------------
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t count) { alloc(count); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count) {
    release();
    n = count;
    // pad so that 16-byte vector loads past the logical end stay inside the allocation
    size_t bytes = (count * sizeof(T) + 64 + 255) & ~size_t(255);
    cudaError_t e = cudaMalloc((void**)&p, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      n = 0;
      sv_throw(SV_ERR_OOM, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    }
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  T* get() const { return p; }
};

// ---------------------------------------------------------------------------
// handles
// ---------------------------------------------------------------------------
struct sv_counts {
  sv_context* ctx = nullptr;
  int64_t n_cells = 0, n_genes = 0, nnz = 0;
  DevBuf<int64_t> csc_colptr;   // n_genes + 1
  DevBuf<int32_t> csc_rowidx;   // nnz
  DevBuf<int32_t> csc_count;    // nnz
  DevBuf<int64_t> csr_rowptr;   // n_cells + 1
  DevBuf<int32_t> csr_colidx;   // nnz
  DevBuf<int32_t> csr_count;    // nnz
};

struct sv_data {
  sv_context* ctx = nullptr;
  const sv_counts* counts = nullptr;
  int dtype = SV_F64;
  int method = SV_LOGNORMALIZE;
  double scale_factor = 1.0;
  DevBuf<unsigned char> csc_val;   // nnz * elem
  DevBuf<unsigned char> csr_val;   // nnz * elem
  DevBuf<int64_t> totals;          // n_cells
};

struct sv_centered {
  sv_context* ctx = nullptr;
  const sv_data* data = nullptr;
  int64_t n_cells = 0, nf = 0, nnz_h = 0;
  int dtype = SV_F64;          // value storage type
  double scale_max = 0;
  DevBuf<int32_t> feat_gene;   // nf: 0-based gene index of each feature
  DevBuf<int64_t> feat_start;  // nf: CSC range of the feature
  DevBuf<int64_t> feat_end;
  DevBuf<double> mean, std_, mu;      // nf (FP64)
  DevBuf<float> mu_h, mu_l;           // nf: mu as double-float (the FP64-free products)
  int grid_csr = 1, grid_csr_df = 1;  // resident blocks of the X v kernels (one wave)
  DevBuf<float> inv_std_f, clip_f;    // nf (FP32 form of the scale / clip)
  DevBuf<double> inv_std_d, clip_d;   // nf (FP64 form, for FP64 data)
  // chunk table of the CSC (X^T u) product
  int64_t n_chunks = 0;
  DevBuf<int32_t> chunk_feat;
  DevBuf<int64_t> chunk_start, chunk_end;
  DevBuf<int64_t> feat_chunk_off;     // nf + 1
  DevBuf<double> chunk_partial;       // n_chunks * block_cols
  int64_t partial_cols = 0;
  // cell-major copy of the feature subset (X v product)
  DevBuf<int64_t> h_rowptr;           // n_cells + 1
  DevBuf<uint16_t> h_col16;           // nnz_h when nf <= 65536
  DevBuf<int32_t> h_col32;            // nnz_h otherwise
  DevBuf<unsigned char> h_val;        // nnz_h * elem
  // scratch for the product prologues
  DevBuf<float> u_f32;                // n_cells
  DevBuf<double> red_partial;         // reduction partials
  DevBuf<double> scal;                // small device scalars
  // row-blocked CSC copy of the subset for X^T u (FP32 / BF16 storage)
  int64_t rb_rows = 0, n_rb = 0;      // rows per block, number of row blocks
  int rb_per_sm = 3;                  // resident blocks per SM of the X^T u kernel
  DevBuf<int64_t> rb_ptr;             // n_rb * nf + 1 entry offsets, ordered (block, feature)
  DevBuf<unsigned long long> rb_idx;  // rows within the block, one coded word per 8 entries
  DevBuf<unsigned char> rb_val;       // value (storage type)
  DevBuf<float> rb_partial;           // n_rb x nf partial sums
  int t_blocks = 0;                   // > 0: X^T u over CSR_h with this many blocks
  DevBuf<unsigned char> t_partial;    // t_blocks x nf partial sums
  // set when the matrix was built by sv_centered_create (owned here)
  sv_counts* own_counts = nullptr;
  sv_data* own_data = nullptr;
};

// Rows of a stacked matrix that holds several independent samples: a block
// schedule covers each sample's rows with contiguous ranges (never crossing a
// sample boundary), the blocks of one sample consecutive.
struct BlkRange {
  int64_t r0, r1;
  int seg, pad;
};

// Several samples stacked by cells over the same genes (one normalised data
// matrix), each scaled with its own moments: the batched path.
struct sv_batch {
  sv_context* ctx = nullptr;
  const sv_data* data = nullptr;
  int64_t nseg = 0, n_cells = 0, nf = 0;
  double scale_max = 0;
  std::vector<int64_t> hoff;          // nseg + 1 cell offsets
  DevBuf<int64_t> off;
  sv_centered* base = nullptr;        // the feature-subset copies of the stacked data
  // per (sample, feature), sample-major: index s * nf + f
  DevBuf<double> mean, std_, mu, inv_d, clip_d;
  DevBuf<float> inv_f, clip_f, mu_h, mu_l;
  // X v: blocks of cells within one sample
  DevBuf<BlkRange> xblk;
  int nxblk = 0;
  int xcells = 0;                     // cells per X v block (autotuned)
  // X^T u: row blocks aligned to the samples
  int64_t n_rb = 0;
  std::vector<int64_t> h_rb_first;    // nseg + 1: first row block of each sample
  DevBuf<int64_t> rb_row0;            // n_rb + 1 first rows
  DevBuf<int> rb_seg;                 // n_rb
  DevBuf<int64_t> rb_first;           // nseg + 1
  DevBuf<int64_t> rb_ptr;             // n_rb * nf + 1
  DevBuf<unsigned long long> rb_idx;
  DevBuf<unsigned char> rb_val;
  DevBuf<float> rb_partial;           // n_rb x nf
  DevBuf<double> upart;               // n_rb sums of u
};

struct sv_embed {
  sv_context* ctx = nullptr;
  int64_t n_cells = 0, npcs = 0, nf = 0;
  DevBuf<double> Z;        // n_cells x npcs column-major (U diag(s))
  DevBuf<double> s;        // npcs
};

struct sv_knn {
  sv_context* ctx = nullptr;
  int64_t n = 0, k = 0;
  DevBuf<int32_t> idx;     // n x k row-major, 0-based
  DevBuf<float> dist;      // n x k row-major, metric distance
};

struct sv_graph {
  sv_context* ctx = nullptr;
  int64_t n = 0, nnz = 0;
  int dtype = SV_F64;
  DevBuf<int64_t> colptr;          // n + 1, 0-based
  DevBuf<int32_t> rowidx;          // nnz, 0-based
  DevBuf<unsigned char> val;       // nnz * elem
};

inline size_t sv_elem_size(int dtype) {
  switch (dtype) {
    case SV_I32: return 4;
    case SV_I64: return 8;
    case SV_F32: return 4;
    case SV_F64: return 8;
    case SV_BF16: return 2;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// shared device helpers
// ---------------------------------------------------------------------------
#define SV_STATUS_OOB 1
#define SV_STATUS_UNSORTED 2
#define SV_STATUS_LIMIT 4
#define SV_STATUS_VALUE 8    // a count that is not an integer in [0, 2^31)
#define SV_STATUS_PARSE 16   // a malformed entry line of a MatrixMarket file

__device__ __forceinline__ void sv_flag(int* status, int bit) { atomicOr(status, bit); }

template <typename T>
__device__ __forceinline__ T sv_warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float sv_load_val(const float* p, int64_t i) { return p[i]; }
__device__ __forceinline__ float sv_load_val(const __nv_bfloat16* p, int64_t i) {
  return __bfloat162float(p[i]);
}
__device__ __forceinline__ double sv_load_val(const double* p, int64_t i) { return p[i]; }
__device__ __forceinline__ double sv_load_val(const int32_t* p, int64_t i) { return (double)p[i]; }

// ---------------------------------------------------------------------------
// host helpers implemented in sv_core.cu
// ---------------------------------------------------------------------------
// out[0..n] = exclusive scan of in[0..n-1]; out[n] = total.  in may equal out
// only if the caller does not need in afterwards.
void sv_scan_i64(sv_context* ctx, const int64_t* in, int64_t* out, int64_t n);
int64_t sv_read_i64(sv_context* ctx, const int64_t* dptr);
void sv_memset(sv_context* ctx, void* p, int v, size_t bytes);
// cuTensorMapEncodeTiled, obtained from the driver through the runtime (no
// link against libcuda)
typedef CUresult (*sv_encode_tiled_fn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                       const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                       const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                       CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
sv_encode_tiled_fn sv_encode_tiled();
// the cell-side restart rotation on the tensor cores (sv_rotate_tc.cu)
bool sv_rotate_tc_supported(int nin, int nout, int64_t ld_in);
void sv_rotate_tc(sv_context* ctx, const float* inh, const float* inl, int64_t ld_in, int64_t len, int nin,
                  const double* M, int nout, float* outh, float* outl, int64_t ld_out, unsigned char* bsl,
                  int* fexp);
// host <-> device copies on the context stream; sv_d2h returns when the data
// are on the host.  Copies of 32 MB or more to or from pageable memory are
// staged through the context's pinned buffers with several host threads.
void sv_h2d(sv_context* ctx, void* dst, const void* src, size_t bytes);
void sv_d2h(sv_context* ctx, void* dst, const void* src, size_t bytes);
// the context's two pinned staging buffers (SV_IO_CHUNK bytes each) and the
// events of their last transfers (wait on them before refilling)
constexpr size_t SV_IO_CHUNK = (size_t)64 << 20;
void sv_ctx_io(sv_context* ctx, void* buf[2], cudaEvent_t ev[2]);
// memcpy split over up to 8 host threads
void sv_parallel_memcpy(void* dst, const void* src, size_t n);
void sv_sync(sv_context* ctx);
int sv_grid_for(sv_context* ctx, int64_t work_items, int per_block, int max_per_sm = 8);
// builds (or rebuilds) the CSR copy of a count matrix from its device CSC copy
// (sv_counts.cu); checks the CSC invariants on the way
void sv_build_csr_from_csc(sv_context* ctx, sv_counts* c);
// transpose of a compressed pattern with its counts, sorted within the output
// segments; checks the source invariants (sv_counts.cu)
void sv_transpose_counts(sv_context* ctx, int64_t n_major, int64_t n_minor, int64_t nnz,
                         const int64_t* ptr, const int32_t* idx, const int32_t* cnt,
                         DevBuf<int64_t>& optr, DevBuf<int32_t>& oidx, DevBuf<int32_t>& ocnt,
                         const char* where);
// sorts the indices within each of the n segments of ptr, counts moving along
void sv_sort_segments(sv_context* ctx, const int64_t* ptr, int64_t n, int32_t* idx, int32_t* cnt);
// converts n host counts of type val_type (SV_I32, SV_I64, SV_F32, SV_F64) into
// device Int32 counts; the wider and floating types must hold integers in
// [0, 2^31) (checked on the device, reported through the context status)
void sv_upload_counts(sv_context* ctx, const void* host, int val_type, int64_t n, int32_t* dst);
// sorts (key, value) pairs by key on the device; the arrays hold n2 entries, n2
// a power of two >= max(n, 2048) (sv_core.cu)
void sv_sort_pairs(sv_context* ctx, unsigned long long* key, int* val, int64_t n, int64_t n2);
