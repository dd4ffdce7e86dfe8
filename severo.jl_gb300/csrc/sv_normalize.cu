// normalize_cells on both copies of the count matrix (src/normalize.jl:17-55).
//
//   K1a  csr: one warp per cell; 128-bit loads of the counts, warp-shuffle sum
//        s_c (integer, normalize.jl:24).  Lane l then evaluates the value of
//        count l + 1 in that cell, f(l + 1, s_c) -- the division and log1p
//        once per lane instead of once per entry -- and the row's values are
//        written with one shuffle per entry (counts above 32 are evaluated
//        directly; the second read of the row hits L1/L2): 509 -> 380 us at
//        100,000 cells.
//   K1b  csc: a flat map over the non-zeros: b = f(a, s[row]) with s gathered
//        from the per-cell totals (10 MB at 1.3M cells, L2-resident).
//
// Every value is the same expression f(a, s) = log1p((sf * a) / s) (or the
// relative count) evaluated in the output type, whichever kernel and path
// computes it.
//
// Algorithmic bytes (HBM): K1a nnz*(4 + v) + 8*(n_cells+1) + 8*n_cells;
// K1b nnz*(4 + 4 + v), v = bytes of the output value type.
#include "sv_internal.cuh"

namespace {

struct NormArgs {
  double sf;
  float sf_f;
  int log;
};

template <typename OutT>
struct NormOp;

template <>
struct NormOp<double> {
  __device__ __forceinline__ static double apply(int a, int64_t s, const NormArgs& p) {
    double v = (p.sf * (double)a) / (double)s;   // normalize.jl:27, evaluated in Float64
    return p.log ? log1p(v) : v;                  // normalize.jl:36
  }
};

template <>
struct NormOp<float> {
  __device__ __forceinline__ static float apply(int a, int64_t s, const NormArgs& p) {
    float v = (p.sf_f * (float)a) / (float)s;     // evaluated in Float32
    return p.log ? log1pf(v) : v;
  }
};

template <>
struct NormOp<__nv_bfloat16> {
  __device__ __forceinline__ static __nv_bfloat16 apply(int a, int64_t s, const NormArgs& p) {
    return __float2bfloat16_rn(NormOp<float>::apply(a, s, p));
  }
};

// Stores 4 consecutive values at out[g..g+3]; elements outside [s, e) are skipped.
template <typename OutT>
__device__ __forceinline__ void store4(OutT* out, int64_t g, int64_t s, int64_t e, const OutT (&v)[4]) {
  if (g >= s && g + 4 <= e) {
    if constexpr (sizeof(OutT) == 4) {
      float4 w;
      w.x = *(const float*)&v[0];
      w.y = *(const float*)&v[1];
      w.z = *(const float*)&v[2];
      w.w = *(const float*)&v[3];
      *(float4*)(out + g) = w;
    } else if constexpr (sizeof(OutT) == 2) {
      uint2 w;
      w.x = (uint32_t)(*(const uint16_t*)&v[0]) | ((uint32_t)(*(const uint16_t*)&v[1]) << 16);
      w.y = (uint32_t)(*(const uint16_t*)&v[2]) | ((uint32_t)(*(const uint16_t*)&v[3]) << 16);
      *(uint2*)(out + g) = w;
    } else {
      double2 w0, w1;
      w0.x = *(const double*)&v[0];
      w0.y = *(const double*)&v[1];
      w1.x = *(const double*)&v[2];
      w1.y = *(const double*)&v[3];
      *(double2*)(out + g) = w0;
      *(double2*)(out + g + 2) = w1;
    }
  } else {
#pragma unroll
    for (int t = 0; t < 4; ++t)
      if (g + t >= s && g + t < e) out[g + t] = v[t];
  }
}

__device__ __forceinline__ void load4(const int32_t* p, int64_t g, int (&v)[4]) {
  int4 w = __ldg((const int4*)(p + g));
  v[0] = w.x;
  v[1] = w.y;
  v[2] = w.z;
  v[3] = w.w;
}

__device__ __forceinline__ float shfl_out(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ double shfl_out(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ __nv_bfloat16 shfl_out(__nv_bfloat16 v, int src) {
  unsigned short u = __bfloat16_as_ushort(v);
  return __ushort_as_bfloat16((unsigned short)__shfl_sync(0xffffffffu, (unsigned)u, src));
}

// K1a: per-cell totals and the CSR values.
template <typename OutT>
__global__ void __launch_bounds__(256) k_norm_csr(const int64_t* __restrict__ rowptr,
                                                  const int32_t* __restrict__ cnt, int64_t n_rows,
                                                  NormArgs p, OutT* __restrict__ out,
                                                  int64_t* __restrict__ totals) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n_rows; r += nwarps) {
    int64_t s = rowptr[r], e = rowptr[r + 1];
    int64_t a0 = s & ~3ll;
    int64_t sum = 0;
    for (int64_t g = a0 + 4 * lane; g < e; g += 128) {
      int v[4];
      load4(cnt, g, v);
#pragma unroll
      for (int t = 0; t < 4; ++t)
        if (g + t >= s && g + t < e) sum += v[t];
    }
    sum = sv_warp_sum(sum);
    if (lane == 0) totals[r] = sum;
    if (e == s) continue;
    const OutT tv = NormOp<OutT>::apply(lane + 1, sum, p);    // the value of count lane + 1
    // every lane takes every pass: the shuffles need the whole warp
    for (int64_t g0 = a0; g0 < e; g0 += 128) {
      const int64_t g = g0 + 4 * lane;
      int v[4] = {0, 0, 0, 0};
      if (g < e) load4(cnt, g, v);
      OutT o[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const bool tabbed = v[t] >= 1 && v[t] <= 32;
        const OutT sh = shfl_out(tv, tabbed ? v[t] - 1 : 0);
        o[t] = tabbed ? sh : NormOp<OutT>::apply(v[t], sum, p);
      }
      if (g < e) store4(out, g, s, e, o);
    }
  }
}

// K1b: flat map over the CSC non-zeros, 4 per thread; s gathered from the
// per-cell totals (10 MB at 1.3M cells, L2-resident).  (Gathering the value
// from a per-cell table of the small counts instead measured slower: 825 vs
// 691 us at 100,000 cells.)
template <typename OutT>
__global__ void __launch_bounds__(256) k_norm_csc(const int32_t* __restrict__ rowidx,
                                                  const int32_t* __restrict__ cnt, int64_t nnz,
                                                  const int64_t* __restrict__ totals, NormArgs p,
                                                  OutT* __restrict__ out) {
  int64_t ngroups = (nnz + 3) >> 2;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ngroups;
       q += (int64_t)gridDim.x * blockDim.x) {
    int64_t g = q << 2;
    int rv[4], cv[4];
    load4(rowidx, g, rv);
    load4(cnt, g, cv);
    OutT o[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      if (g + t < nnz) o[t] = NormOp<OutT>::apply(cv[t], __ldg(totals + rv[t]), p);
      else o[t] = OutT(0.0f);
    }
    store4(out, g, 0, nnz, o);
  }
}

template <typename OutT>
void run_normalize(sv_context* ctx, const sv_counts* c, sv_data* d, NormArgs p) {
  int64_t nnz = c->nnz;
  sv_launch(ctx, "normalize_csr", k_norm_csr<OutT>, dim3(sv_grid_for(ctx, c->n_cells * 32, 256, 8)),
            dim3(256), 0, (const int64_t*)c->csr_rowptr.get(), (const int32_t*)c->csr_count.get(),
            c->n_cells, p, (OutT*)d->csr_val.get(), d->totals.get());
  sv_launch(ctx, "normalize_csc", k_norm_csc<OutT>, dim3(sv_grid_for(ctx, (nnz + 3) / 4, 256, 8)),
            dim3(256), 0, (const int32_t*)c->csc_rowidx.get(), (const int32_t*)c->csc_count.get(),
            nnz, (const int64_t*)d->totals.get(), p, (OutT*)d->csc_val.get());
}

}  // namespace

// Re-runs the normalisation kernels on an existing sv_data (used by the
// benchmark to time the stage with the output buffers already allocated).
void sv_normalize_into(sv_context* ctx, const sv_counts* c, sv_data* d) {
  NormArgs p;
  p.sf = d->scale_factor;
  p.sf_f = (float)d->scale_factor;
  p.log = d->method == SV_LOGNORMALIZE;
  switch (d->dtype) {
    case SV_F64: run_normalize<double>(ctx, c, d, p); break;
    case SV_F32: run_normalize<float>(ctx, c, d, p); break;
    case SV_BF16: run_normalize<__nv_bfloat16>(ctx, c, d, p); break;
    default: sv_throw(SV_ERR_ARG, "unsupported dtype %d", d->dtype);
  }
}

SV_API int sv_normalize_cells(sv_context* ctx, const sv_counts* counts, int method,
                              double scale_factor, int dtype, sv_data** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(out && counts, "null argument");
  SV_REQUIRE(counts->ctx == ctx, "counts handle belongs to another context");
  if (method != SV_LOGNORMALIZE && method != SV_RELATIVECOUNTS)
    sv_throw(SV_ERR_ARG, "unknown normalization method: %d", method);   // normalize.jl:50
  SV_REQUIRE(dtype == SV_F64 || dtype == SV_F32 || dtype == SV_BF16, "dtype must be F64, F32 or BF16");
  auto* d = new sv_data();
  try {
    d->ctx = ctx;
    d->counts = counts;
    d->dtype = dtype;
    d->method = method;
    d->scale_factor = scale_factor;
    size_t es = sv_elem_size(dtype);
    d->csc_val.alloc(counts->nnz * es);
    d->csr_val.alloc(counts->nnz * es);
    d->totals.alloc(counts->n_cells);
    sv_normalize_into(ctx, counts, d);
    sv_sync(ctx);
  } catch (...) {
    delete d;
    throw;
  }
  *out = d;
  SV_CATCH
}

SV_API int sv_data_download_csc(sv_context* ctx, const sv_data* d, void* nzval) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(d && d->ctx == ctx && nzval, "bad handle or null output");
  sv_d2h(ctx, nzval, d->csc_val.get(), d->counts->nnz * sv_elem_size(d->dtype));
  SV_CATCH
}

SV_API int sv_data_download_csr(sv_context* ctx, const sv_data* d, void* nzval) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(d && d->ctx == ctx && nzval, "bad handle or null output");
  sv_d2h(ctx, nzval, d->csr_val.get(), d->counts->nnz * sv_elem_size(d->dtype));
  SV_CATCH
}

SV_API int sv_data_cell_totals(sv_context* ctx, const sv_data* d, int64_t* totals) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(d && d->ctx == ctx && totals, "bad handle or null output");
  sv_d2h(ctx, totals, d->totals.get(), d->counts->n_cells * 8);
  SV_CATCH
}

SV_API int sv_data_free(sv_data* d) {
  if (d) {
    if (d->ctx) cudaSetDevice(d->ctx->device);
    delete d;
  }
  return SV_OK;
}
