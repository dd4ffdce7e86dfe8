// The sparse products of src/mul.jl and the CenteredMatrix Gram product of
// src/scaling.jl:274-296, off the irlba path (they serve the tssvd Gram
// route, src/embedding.jl:30-44).
//
//   sv_sparse_mul_spvec   y = alpha A x + beta y, A CSC (m x n), x sparse
//                         (mul.jl:50-77): blocks own ranges of rows of y; each
//                         walks x's non-zeros in order and, per column, the
//                         column's rows within its range (rows sorted:
//                         binary search), so every y[i] receives its terms
//                         in the reference's order -- bit-identical results.
//   sv_sparse_mul_sparse  C = alpha op(A) B + beta C, dense column-major C
//                         (mul.jl:79-114): one block per column of C, B's
//                         entries of the column in order, the column of A of
//                         each entry spread over the threads (distinct rows),
//                         a barrier between entries -- again the reference's
//                         order per element.  op(A) = A' is the device
//                         transpose of A first (copy(A'), rows sorted).
//   sv_centered_gram      C = alpha Xl~' Xr~ + beta C for two CenteredMatrix
//                         over the same cells (scaling.jl:274-296):
//                         Al' Ar by the same column kernel over the cell-major
//                         copy of Al and the CSC view of Ar, then the rank-1
//                         corrections - mu_l q_r' - (q_l - n mu_l) mu_r'.
// Terms are evaluated as (alpha * a) * b and then added, as the reference
// writes them (explicit roundings: no fused multiply-add).
#include "sv_internal.cuh"

namespace {

__global__ void k_scale_vec(double* __restrict__ y, int64_t n, double beta) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = beta == 0.0 ? 0.0 : __dmul_rn(y[i], beta);
}

constexpr int SPV_ROWS = 4096;   // rows of y per block

// y[r0, r0 + SPV_ROWS) += (alpha * A[i, j]) * x_j over x's non-zeros in order
__global__ void __launch_bounds__(256) k_mul_spvec(const int64_t* __restrict__ colptr,
                                                   const int64_t* __restrict__ rowval,
                                                   const double* __restrict__ nzval, int64_t m,
                                                   int64_t nnzx, const int64_t* __restrict__ xidx,
                                                   const double* __restrict__ xval, double alpha,
                                                   double* __restrict__ y) {
  const int64_t r0 = (int64_t)blockIdx.x * SPV_ROWS;
  const int64_t r1 = r0 + SPV_ROWS < m ? r0 + SPV_ROWS : m;
  __shared__ int64_t range[2];
  for (int64_t jp = 0; jp < nnzx; ++jp) {
    const int64_t j = xidx[jp];
    if (threadIdx.x == 0) {
      int64_t lo = colptr[j], hi = colptr[j + 1];
      int64_t a = lo, b = hi;           // first entry with row >= r0
      while (a < b) {
        int64_t mid = (a + b) >> 1;
        if (rowval[mid] < r0) a = mid + 1;
        else b = mid;
      }
      int64_t c = a, d = hi;            // first entry with row >= r1
      while (c < d) {
        int64_t mid = (c + d) >> 1;
        if (rowval[mid] < r1) c = mid + 1;
        else d = mid;
      }
      range[0] = a;
      range[1] = c;
    }
    __syncthreads();
    const double xv = xval[jp];
    for (int64_t kp = range[0] + threadIdx.x; kp < range[1]; kp += blockDim.x)
      y[rowval[kp]] = __dadd_rn(y[rowval[kp]], __dmul_rn(__dmul_rn(alpha, nzval[kp]), xv));   // mul.jl:71
    __syncthreads();
  }
}

// C[:, col] += (alpha * A[row, j]) * B[j, col] over B's column in order
__global__ void __launch_bounds__(256) k_mul_sparse(const int64_t* __restrict__ acp,
                                                    const int32_t* __restrict__ arv,
                                                    const double* __restrict__ anz,
                                                    const int64_t* __restrict__ bcp,
                                                    const int64_t* __restrict__ brv,
                                                    const double* __restrict__ bnz, int64_t m,
                                                    int64_t n, double alpha, double* __restrict__ C) {
  for (int64_t col = blockIdx.x; col < n; col += gridDim.x) {
    double* cc = C + col * m;
    for (int64_t jp = bcp[col]; jp < bcp[col + 1]; ++jp) {
      const int64_t j = brv[jp];
      const double b = bnz[jp];
      for (int64_t kp = acp[j] + threadIdx.x; kp < acp[j + 1]; kp += blockDim.x)
        cc[arv[kp]] = __dadd_rn(cc[arv[kp]], __dmul_rn(__dmul_rn(alpha, anz[kp]), b));  // mul.jl:107
      __syncthreads();
    }
  }
}

__global__ void k_gather_f64(const double* __restrict__ src, const int32_t* __restrict__ pos, int64_t n,
                             double* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[pos[i]];
}

__global__ void k_iota32(int32_t* __restrict__ a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] = (int32_t)i;
}

__global__ void k_i64_to_i32_checked(const int64_t* __restrict__ in, int64_t n, int64_t base,
                                     int64_t lim, int32_t* __restrict__ out, int* __restrict__ status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = in[i] - base;
    if (v < 0 || v >= lim) {
      sv_flag(status, SV_STATUS_OOB);
      out[i] = 0;
    } else {
      out[i] = (int32_t)v;
    }
  }
}

__global__ void k_sub_base(int64_t* __restrict__ a, int64_t n, int64_t base, int64_t lim,
                           int* __restrict__ status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = a[i] - base;
    if (v < 0 || v >= lim) {
      sv_flag(status, SV_STATUS_OOB);
      a[i] = 0;
    } else {
      a[i] = v;
    }
  }
}

// ---- Gram of CenteredMatrix pairs ---------------------------------------------
// value of a stored entry: min(a * inv_f, clip_f), in the products' precision
template <typename ValT>
__device__ __forceinline__ double gram_val(ValT a, float invf, float clipf, double invd, double clipd);
template <>
__device__ __forceinline__ double gram_val<double>(double a, float, float, double invd, double clipd) {
  const double v = a * invd;
  return v > clipd ? clipd : v;
}
template <>
__device__ __forceinline__ double gram_val<float>(float a, float invf, float clipf, double, double) {
  return (double)fminf(a * invf, clipf);
}
template <>
__device__ __forceinline__ double gram_val<__nv_bfloat16>(__nv_bfloat16 a, float invf, float clipf, double,
                                                          double) {
  return (double)fminf(__bfloat162float(a) * invf, clipf);
}

// G[:, fr] += alpha * sum over the cells c of Ar's column fr (in CSC order) of
// Al[c, :] * Ar[c, fr]: the cell's row of Al (cell-major copy) spread over the
// threads (distinct features), a barrier between cells.
template <typename ValT, typename IdxT>
__global__ void __launch_bounds__(256) k_gram_cols(
    const int64_t* __restrict__ lrowptr, const IdxT* __restrict__ lcol, const ValT* __restrict__ lval,
    const float* __restrict__ linvf, const float* __restrict__ lclipf, const double* __restrict__ linvd,
    const double* __restrict__ lclipd, int64_t nfl, const int64_t* __restrict__ rfs,
    const int64_t* __restrict__ rfe, const int32_t* __restrict__ rrow, const ValT* __restrict__ rval,
    const float* __restrict__ rinvf, const float* __restrict__ rclipf, const double* __restrict__ rinvd,
    const double* __restrict__ rclipd, int64_t nfr, double alpha, double* __restrict__ G) {
  for (int64_t fr = blockIdx.x; fr < nfr; fr += gridDim.x) {
    double* gc = G + fr * nfl;
    for (int64_t jp = rfs[fr]; jp < rfe[fr]; ++jp) {
      const int64_t c = rrow[jp];
      const double b = gram_val<ValT>(rval[jp], rinvf[fr], rclipf[fr], rinvd[fr], rclipd[fr]);
      for (int64_t kp = lrowptr[c] + threadIdx.x; kp < lrowptr[c + 1]; kp += blockDim.x) {
        const int64_t f = (int64_t)lcol[kp];
        gc[f] += alpha * gram_val<ValT>(lval[kp], linvf[f], lclipf[f], linvd[f], lclipd[f]) * b;
      }
      __syncthreads();
    }
  }
}

// q[f] = sum of the stored values of feature f (column order)
template <typename ValT>
__global__ void k_gram_colsum(const int64_t* __restrict__ fs, const int64_t* __restrict__ fe,
                              const ValT* __restrict__ val, const float* __restrict__ invf,
                              const float* __restrict__ clipf, const double* __restrict__ invd,
                              const double* __restrict__ clipd, int64_t nf, double* __restrict__ q) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
       f += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t i = fs[f]; i < fe[f]; ++i) s += gram_val<ValT>(val[i], invf[f], clipf[f], invd[f], clipd[f]);
    q[f] = s;
  }
}

// G[i, j] -= alpha * (mul_i qr_j + (ql_i - n mul_i) mur_j)   (scaling.jl:284-293)
__global__ void k_gram_rank1(double* __restrict__ G, int64_t nfl, int64_t nfr,
                             const double* __restrict__ mul, const double* __restrict__ mur,
                             const double* __restrict__ ql, const double* __restrict__ qr, double n,
                             double alpha) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nfl * nfr;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % nfl, j = e / nfl;
    double g = G[e];
    g += -alpha * mul[i] * qr[j];
    g += -alpha * (ql[i] - n * mul[i]) * mur[j];
    G[e] = g;
  }
}

}  // namespace

SV_API int sv_sparse_mul_spvec(sv_context* ctx, int64_t m, int64_t n, const int64_t* colptr,
                               const int64_t* rowval, const double* nzval, int64_t nnzx,
                               const int64_t* xidx, const double* xval, int index_base, double alpha,
                               double beta, double* y) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(m >= 0 && n >= 0 && nnzx >= 0 && (index_base == 0 || index_base == 1), "bad sizes or base");
  SV_REQUIRE(y || m == 0, "null y");
  SV_REQUIRE(colptr, "null colptr");
  if (n == 0) return SV_OK;                                        // mul.jl:53
  std::vector<int64_t> cp(colptr, colptr + n + 1);
  for (auto& v : cp) v -= index_base;
  const int64_t nnz = cp[n];
  SV_REQUIRE(cp[0] == 0 && nnz >= 0, "colptr does not start at the index base");
  for (int64_t j = 0; j < n; ++j) SV_REQUIRE(cp[j + 1] >= cp[j], "colptr decreases at column %lld", (long long)j);
  DevBuf<double> dy(std::max<int64_t>(m, 1));
  sv_h2d(ctx, dy.get(), y, m * 8);
  if (beta != 1.0)
    sv_launch(ctx, "mul_scale", k_scale_vec, dim3(sv_grid_for(ctx, m, 256)), dim3(256), 0, dy.get(), m, beta);
  if (alpha != 0.0 && nnzx > 0 && nnz > 0) {
    DevBuf<int64_t> dcp(n + 1), drv(nnz), dxi(nnzx);
    DevBuf<double> dnz(nnz), dxv(nnzx);
    sv_h2d(ctx, dcp.get(), cp.data(), (n + 1) * 8);
    sv_h2d(ctx, drv.get(), rowval, nnz * 8);
    sv_h2d(ctx, dnz.get(), nzval, nnz * 8);
    sv_h2d(ctx, dxi.get(), xidx, nnzx * 8);
    sv_h2d(ctx, dxv.get(), xval, nnzx * 8);
    sv_memset(ctx, ctx->d_status, 0, sizeof(int));
    sv_launch(ctx, "mul_check", k_sub_base, dim3(sv_grid_for(ctx, nnz, 256)), dim3(256), 0, drv.get(), nnz,
              (int64_t)index_base, m, ctx->d_status);
    sv_launch(ctx, "mul_check", k_sub_base, dim3(sv_grid_for(ctx, nnzx, 256)), dim3(256), 0, dxi.get(),
              nnzx, (int64_t)index_base, n, ctx->d_status);
    sv_check_device_status(ctx, "sv_sparse_mul_spvec");
    sv_launch(ctx, "mul_spvec", k_mul_spvec, dim3((unsigned)((m + SPV_ROWS - 1) / SPV_ROWS)), dim3(256), 0,
              (const int64_t*)dcp.get(), (const int64_t*)drv.get(), (const double*)dnz.get(), m, nnzx,
              (const int64_t*)dxi.get(), (const double*)dxv.get(), alpha, dy.get());
    sv_d2h(ctx, y, dy.get(), m * 8);
  } else {
    sv_d2h(ctx, y, dy.get(), m * 8);
  }
  SV_CATCH
}

SV_API int sv_sparse_mul_sparse(sv_context* ctx, int64_t m, int64_t k, int64_t n, const int64_t* acolptr,
                                const int64_t* arowval, const double* anzval, int transa,
                                const int64_t* bcolptr, const int64_t* browval, const double* bnzval,
                                int index_base, double alpha, double beta, double* C) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(m >= 0 && k >= 0 && n >= 0 && (index_base == 0 || index_base == 1), "bad sizes or base");
  SV_REQUIRE(C || m * n == 0, "null C");
  SV_REQUIRE(m < (1ll << 31) && k < (1ll << 31), "dimension above 2^31");
  // A as given: m x k (CSC, k + 1 pointers), or k x m when transa (op(A) = A')
  const int64_t amaj = transa ? m : k, amin = transa ? k : m;
  std::vector<int64_t> acp(acolptr, acolptr + amaj + 1), bcp(bcolptr, bcolptr + n + 1);
  for (auto& v : acp) v -= index_base;
  for (auto& v : bcp) v -= index_base;
  const int64_t annz = acp[amaj], bnnz = bcp[n];
  SV_REQUIRE(acp[0] == 0 && bcp[0] == 0 && annz >= 0 && bnnz >= 0, "pointers do not start at the index base");
  for (int64_t j = 0; j < amaj; ++j) SV_REQUIRE(acp[j + 1] >= acp[j], "A's colptr decreases");
  for (int64_t j = 0; j < n; ++j) SV_REQUIRE(bcp[j + 1] >= bcp[j], "B's colptr decreases");
  DevBuf<double> dC(std::max<int64_t>(m * n, 1));
  sv_h2d(ctx, dC.get(), C, m * n * 8);
  if (beta != 1.0)                                                 // mul.jl:97-99
    sv_launch(ctx, "mul_scale", k_scale_vec, dim3(sv_grid_for(ctx, m * n, 256)), dim3(256), 0, dC.get(),
              m * n, beta);
  if (annz > 0 && bnnz > 0) {
    DevBuf<int64_t> dacp(amaj + 1), dbcp(n + 1), dbrv(bnnz), darv64(annz);
    DevBuf<int32_t> darv(annz);
    DevBuf<double> danz(annz), dbnz(bnnz);
    sv_h2d(ctx, dacp.get(), acp.data(), (amaj + 1) * 8);
    sv_h2d(ctx, dbcp.get(), bcp.data(), (n + 1) * 8);
    sv_h2d(ctx, darv64.get(), arowval, annz * 8);
    sv_h2d(ctx, danz.get(), anzval, annz * 8);
    sv_h2d(ctx, dbrv.get(), browval, bnnz * 8);
    sv_h2d(ctx, dbnz.get(), bnzval, bnnz * 8);
    sv_memset(ctx, ctx->d_status, 0, sizeof(int));
    sv_launch(ctx, "mul_check", k_i64_to_i32_checked, dim3(sv_grid_for(ctx, annz, 256)), dim3(256), 0,
              (const int64_t*)darv64.get(), annz, (int64_t)index_base, amin, darv.get(), ctx->d_status);
    sv_launch(ctx, "mul_check", k_sub_base, dim3(sv_grid_for(ctx, bnnz, 256)), dim3(256), 0, dbrv.get(),
              bnnz, (int64_t)index_base, k, ctx->d_status);
    sv_check_device_status(ctx, "sv_sparse_mul_sparse");
    const int64_t* cp_use = dacp.get();
    const int32_t* rv_use = darv.get();
    const double* nz_use = danz.get();
    DevBuf<int64_t> tptr;
    DevBuf<int32_t> tidx, tpos, iota;
    DevBuf<double> tval;
    if (transa) {
      // copy(A') (mul.jl:79-80): the device transpose, rows sorted within columns
      SV_REQUIRE(annz < (1ll << 31), "A has 2^31 or more entries");
      iota.alloc(annz);
      sv_launch(ctx, "mul_iota", k_iota32, dim3(sv_grid_for(ctx, annz, 256)), dim3(256), 0, iota.get(), annz);
      sv_transpose_counts(ctx, amaj, amin, annz, dacp.get(), darv.get(), iota.get(), tptr, tidx, tpos,
                          "sv_sparse_mul_sparse (transpose of A)");
      tval.alloc(annz);
      sv_launch(ctx, "mul_gather", k_gather_f64, dim3(sv_grid_for(ctx, annz, 256)), dim3(256), 0,
                (const double*)danz.get(), (const int32_t*)tpos.get(), annz, tval.get());
      cp_use = tptr.get();
      rv_use = tidx.get();
      nz_use = tval.get();
    }
    if (alpha != 0.0)
      sv_launch(ctx, "mul_sparse", k_mul_sparse, dim3((unsigned)std::min<int64_t>(n, (int64_t)ctx->num_sms * 16)),
                dim3(256), 0, cp_use, rv_use, nz_use, (const int64_t*)dbcp.get(), (const int64_t*)dbrv.get(),
                (const double*)dbnz.get(), m, n, alpha, dC.get());
    sv_d2h(ctx, C, dC.get(), m * n * 8);
  } else {
    sv_d2h(ctx, C, dC.get(), m * n * 8);
  }
  SV_CATCH
}

SV_API int sv_centered_gram(sv_context* ctx, const sv_centered* Sl, const sv_centered* Sr, double alpha,
                            double beta, double* C) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(Sl && Sr && C, "null argument");
  SV_REQUIRE(Sl->ctx == ctx && Sr->ctx == ctx, "matrix handle belongs to another context");
  SV_REQUIRE(Sl->n_cells == Sr->n_cells, "the two matrices have %lld and %lld rows",
             (long long)Sl->n_cells, (long long)Sr->n_cells);
  SV_REQUIRE(Sl->dtype == Sr->dtype, "the two matrices store different value types");
  SV_REQUIRE(Sl->h_rowptr.get() != nullptr, "the left matrix has no cell-major copy");
  const int64_t nfl = Sl->nf, nfr = Sr->nf, n = Sl->n_cells;
  DevBuf<double> G(nfl * nfr), ql(nfl), qr(nfr);
  sv_h2d(ctx, G.get(), C, nfl * nfr * 8);
  sv_launch(ctx, "gram_scale", k_scale_vec, dim3(sv_grid_for(ctx, nfl * nfr, 256)), dim3(256), 0, G.get(),
            nfl * nfr, beta);
  const int32_t* rrow = Sr->data->counts->csc_rowidx.get();
  const int grid = (int)std::min<int64_t>(nfr, (int64_t)ctx->num_sms * 16);
  const bool small = Sl->nf <= 65536;
#define GRAM(VT, IT, COL)                                                                          \
  do {                                                                                             \
  sv_launch(ctx, "gram_cols", k_gram_cols<VT, IT>, dim3(grid), dim3(256), 0,                       \
            (const int64_t*)Sl->h_rowptr.get(), (const IT*)COL, (const VT*)Sl->h_val.get(),         \
            (const float*)Sl->inv_std_f.get(), (const float*)Sl->clip_f.get(),                       \
            (const double*)Sl->inv_std_d.get(), (const double*)Sl->clip_d.get(), nfl,                \
            (const int64_t*)Sr->feat_start.get(), (const int64_t*)Sr->feat_end.get(), rrow,          \
            (const VT*)Sr->data->csc_val.get(), (const float*)Sr->inv_std_f.get(),                   \
            (const float*)Sr->clip_f.get(), (const double*)Sr->inv_std_d.get(),                      \
            (const double*)Sr->clip_d.get(), nfr, alpha, G.get());                                   \
  sv_launch(ctx, "gram_colsum", k_gram_colsum<VT>, dim3(sv_grid_for(ctx, nfl, 256)), dim3(256), 0,  \
            (const int64_t*)Sl->feat_start.get(), (const int64_t*)Sl->feat_end.get(),               \
            (const VT*)Sl->data->csc_val.get(), (const float*)Sl->inv_std_f.get(),                   \
            (const float*)Sl->clip_f.get(), (const double*)Sl->inv_std_d.get(),                      \
            (const double*)Sl->clip_d.get(), nfl, ql.get());                                         \
  sv_launch(ctx, "gram_colsum", k_gram_colsum<VT>, dim3(sv_grid_for(ctx, nfr, 256)), dim3(256), 0,  \
            (const int64_t*)Sr->feat_start.get(), (const int64_t*)Sr->feat_end.get(),               \
            (const VT*)Sr->data->csc_val.get(), (const float*)Sr->inv_std_f.get(),                   \
            (const float*)Sr->clip_f.get(), (const double*)Sr->inv_std_d.get(),                      \
            (const double*)Sr->clip_d.get(), nfr, qr.get());                                          \
  } while (0)
  switch (Sl->dtype) {
    case SV_F64:
      if (small) GRAM(double, uint16_t, Sl->h_col16.get());
      else GRAM(double, int32_t, Sl->h_col32.get());
      break;
    case SV_F32:
      if (small) GRAM(float, uint16_t, Sl->h_col16.get());
      else GRAM(float, int32_t, Sl->h_col32.get());
      break;
    default:
      if (small) GRAM(__nv_bfloat16, uint16_t, Sl->h_col16.get());
      else GRAM(__nv_bfloat16, int32_t, Sl->h_col32.get());
      break;
  }
#undef GRAM
  sv_launch(ctx, "gram_rank1", k_gram_rank1, dim3(sv_grid_for(ctx, nfl * nfr, 256)), dim3(256), 0, G.get(),
            nfl, nfr, (const double*)Sl->mu.get(), (const double*)Sr->mu.get(), (const double*)ql.get(),
            (const double*)qr.get(), (double)n, alpha);
  sv_d2h(ctx, C, G.get(), nfl * nfr * 8);
  SV_CATCH
}
