// Exact k-nearest neighbours (replaces the approximate native FindNeighbours*
// routines that src/neighbours.jl:19-74 calls).
//
// Stage 1 (candidates): every query scans every point.  The distance key is the
// GEMM form |p|^2 - 2 q.p (|q|^2 is constant per query); each query keeps its
// K2 >= 2k smallest keys.  Two implementations:
//   * FP32 CUDA cores (k_knn_fp32): one query per thread, the point tile staged
//     in shared memory and broadcast to the block;
//   * BF16 tcgen05 tensor cores with FP32 accumulation in TMEM (sv_knn_tc.cu).
// Stage 2 (k_rerank): exact FP32 distances sum (q_c - p_c)^2 of the K2
// candidates, sorted by (distance, index); the point itself first when
// include_self, excluded otherwise.
//
// Layout in HBM: points row-major FP32 [n][dp] (dp = d rounded up to 8, zero
// padded) plus FP32 squared norms; candidates [n][K2]; results [n][k] (0-based).
#include "sv_internal.cuh"
#include <float.h>

int sv_knn_tc_candidates(sv_context* ctx, const float* X32, const float* sq, int64_t n, int dp, int d,
                         int K2, int include_self, int32_t* cand,
                         const std::vector<int64_t>* segs);
sv_context* sv_default_context();

namespace {

constexpr int KNN_THREADS = 128;
constexpr int KNN_TILE = 64;

// X (n x d, column-major, leading dim ld, FP32 or FP64) -> row-major FP32 [n][dp]
// (optionally unit-normalised rows for the cosine metric) and squared norms.
template <typename T>
__global__ void k_pack_rows(const T* __restrict__ X, int64_t ld, int64_t n, int d, int dp,
                            int normalise, float* __restrict__ out, float* __restrict__ sq) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double nr = 1.0;
    if (normalise) {
      double s = 0;
      for (int c = 0; c < d; ++c) {
        double v = (double)X[(int64_t)c * ld + i];
        s += v * v;
      }
      nr = s > 0 ? sqrt(s) : 1.0;
    }
    float s2 = 0.f;
    for (int c = 0; c < dp; ++c) {
      float v = c < d ? (float)((double)X[(int64_t)c * ld + i] / nr) : 0.f;
      out[i * dp + c] = v;
      s2 += v * v;
    }
    sq[i] = s2;
  }
}

template <int DP, int K2>
__global__ void __launch_bounds__(KNN_THREADS) k_knn_fp32(const float* __restrict__ X,
                                                          const float* __restrict__ sq, int64_t n,
                                                          int include_self,
                                                          int32_t* __restrict__ cand) {
  __shared__ __align__(16) float tile[KNN_TILE * DP];
  __shared__ float tsq[KNN_TILE];
  __shared__ float kslot[KNN_THREADS][9];
  int64_t qi = (int64_t)blockIdx.x * KNN_THREADS + threadIdx.x;
  bool active = qi < n;
  float q[DP];
#pragma unroll
  for (int c = 0; c < DP; c += 4) {
    float4 v = active ? *(const float4*)(X + qi * DP + c) : make_float4(0, 0, 0, 0);
    q[c] = -2.f * v.x;
    q[c + 1] = -2.f * v.y;
    q[c + 2] = -2.f * v.z;
    q[c + 3] = -2.f * v.w;
  }
  float best[K2];
  int bidx[K2];
#pragma unroll
  for (int t = 0; t < K2; ++t) {
    best[t] = FLT_MAX;
    bidx[t] = -1;
  }
  if (include_self && active) {
    best[0] = -FLT_MAX;
    bidx[0] = (int)qi;
  }
  for (int64_t p0 = 0; p0 < n; p0 += KNN_TILE) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < KNN_TILE * DP / 4; idx += KNN_THREADS) {
      int r = idx / (DP / 4);
      int64_t p = p0 + r;
      float4 v = p < n ? *(const float4*)(X + p * DP + (idx % (DP / 4)) * 4) : make_float4(0, 0, 0, 0);
      *(float4*)(tile + idx * 4) = v;
    }
    for (int r = threadIdx.x; r < KNN_TILE; r += KNN_THREADS) tsq[r] = p0 + r < n ? sq[p0 + r] : FLT_MAX;
    __syncthreads();
    // 8 candidates at a time: 8 independent FMA chains; padded rows have key FLT_MAX
#pragma unroll 1
    for (int r0 = 0; r0 < KNN_TILE; r0 += 8) {
      float acc[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) acc[u] = tsq[r0 + u];
#pragma unroll
      for (int c = 0; c < DP; c += 4) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          float4 v = ((const float4*)(tile + (r0 + u) * DP))[c / 4];
          acc[u] = fmaf(q[c], v.x, acc[u]);
          acc[u] = fmaf(q[c + 1], v.y, acc[u]);
          acc[u] = fmaf(q[c + 2], v.z, acc[u]);
          acc[u] = fmaf(q[c + 3], v.w, acc[u]);
        }
      }
      float thr = best[K2 - 1];
      uint32_t m = 0;
#pragma unroll
      for (int u = 0; u < 8; ++u) m |= (acc[u] < thr ? 1u : 0u) << u;
      if (m) {
        float* slot = kslot[threadIdx.x];
#pragma unroll
        for (int u = 0; u < 8; ++u) slot[u] = acc[u];
        while (m) {
          int u = __ffs(m) - 1;
          m &= m - 1;
          int pid = (int)(p0 + r0 + u);
          float cd = slot[u];
          if (pid == qi || !(cd < best[K2 - 1])) continue;
          int ci = pid;
#pragma unroll
          for (int t = 0; t < K2; ++t) {
            if (cd < best[t]) {
              float td = best[t];
              int ti = bidx[t];
              best[t] = cd;
              bidx[t] = ci;
              cd = td;
              ci = ti;
            }
          }
        }
      }
    }
  }
  if (active) {
#pragma unroll
    for (int t = 0; t < K2; ++t) cand[qi * K2 + t] = bidx[t];
  }
}

// Exact FP32 re-rank: one warp per query; K2 candidates sorted by (d2, index)
// (a bitonic sort over the next power of two, P2, padded with the largest key).
template <int DP>
__global__ void k_rerank(const float* __restrict__ X, int64_t n, const int32_t* __restrict__ cand,
                         int K2, int k, int include_self, int cosine, int32_t* __restrict__ out_idx,
                         float* __restrict__ out_dist) {
  extern __shared__ unsigned long long keys_all[];
  int P2 = 32;
  while (P2 < K2) P2 <<= 1;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long* keys = keys_all + wid * P2;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t qi = warp; qi < n; qi += nwarps) {
    const float* q = X + qi * DP;
    for (int t = lane; t < P2; t += 32) {
      int c = t < K2 ? cand[qi * K2 + t] : -1;
      unsigned long long key = ~0ull;
      if (c >= 0 && c != qi) {
        const float* p = X + (int64_t)c * DP;
        float s = 0.f;
#pragma unroll 8
        for (int j = 0; j < DP; ++j) {
          float df = q[j] - p[j];
          s = fmaf(df, df, s);
        }
        // order-preserving bit pattern of a float (all finite here)
        unsigned int b = __float_as_uint(s);
        b = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
        key = ((unsigned long long)b << 32) | (unsigned int)c;
      }
      keys[t] = key;
    }
    __syncwarp();
    // bitonic sort of the P2 keys by the warp
    for (int kk = 2; kk <= P2; kk <<= 1) {
      for (int j = kk >> 1; j > 0; j >>= 1) {
        for (int i = lane; i < P2; i += 32) {
          int ixj = i ^ j;
          if (ixj > i) {
            unsigned long long a = keys[i], b = keys[ixj];
            bool up = (i & kk) == 0;
            if ((a > b) == up) {
              keys[i] = b;
              keys[ixj] = a;
            }
          }
        }
        __syncwarp();
      }
    }
    // the point itself first when include_self (distance 0), then the others
    int off = include_self ? 1 : 0;
    if (include_self && lane == 0) {
      out_idx[qi * k] = (int32_t)qi;
      out_dist[qi * k] = 0.f;
    }
    for (int t = lane; t + off < k; t += 32) {
      unsigned long long key = keys[t];
      int c = (int)(key & 0xffffffffu);
      unsigned int b = (unsigned int)(key >> 32);
      b = (b & 0x80000000u) ? (b & 0x7fffffffu) : ~b;
      float s = __uint_as_float(b);
      if (s < 0.f) s = 0.f;
      out_idx[qi * k + t + off] = key == ~0ull ? -1 : c;
      out_dist[qi * k + t + off] = cosine ? 0.5f * s : sqrtf(s);
    }
    __syncwarp();
  }
}

template <int DP>
void launch_fp32(sv_context* ctx, const float* X, const float* sq, int64_t n, int K2, int inc,
                 int32_t* cand) {
  dim3 grid((unsigned)((n + KNN_THREADS - 1) / KNN_THREADS));
  if (K2 == 32)
    sv_launch(ctx, "knn_fp32_tiles", k_knn_fp32<DP, 32>, grid, dim3(KNN_THREADS), 0, X, sq, n, inc, cand);
  else
    sv_launch(ctx, "knn_fp32_tiles", k_knn_fp32<DP, 64>, grid, dim3(KNN_THREADS), 0, X, sq, n, inc, cand);
}

template <int DP>
void launch_rerank(sv_context* ctx, const float* X, int64_t n, const int32_t* cand, int K2, int k,
                   int inc, int cosine, int32_t* idx, float* dist) {
  int P2 = 32;
  while (P2 < K2) P2 <<= 1;
  sv_launch(ctx, "knn_rerank", k_rerank<DP>, dim3(sv_grid_for(ctx, n * 32, 256, 8)), dim3(256),
            (size_t)8 * P2 * 8, X, n, cand, K2, k, inc, cosine, idx, dist);
}

// candidate indices of one sample (local, >= 0) -> stacked rows
__global__ void k_add_offset(int32_t* __restrict__ c, int64_t count, int32_t off) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x)
    if (c[e] >= 0) c[e] += off;
}

__global__ void k_to_host_layout(const int32_t* __restrict__ idx, const float* __restrict__ dist,
                                 int64_t n, int k, int32_t* __restrict__ oidx, float* __restrict__ of,
                                 double* __restrict__ od) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * k;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / k;
    int t = (int)(e % k);
    if (oidx) oidx[(int64_t)t * n + i] = idx[e] + 1;   // column-major n x k, 1-based
    if (of) of[(int64_t)t * n + i] = dist[e];
    if (od) od[(int64_t)t * n + i] = (double)dist[e];
  }
}

}  // namespace

// Core: X32 row-major [n][dp] FP32 with norms -> knn handle (row-major, 0-based).
// segs (optional, nseg + 1 row offsets): stacked samples, each point's
// neighbours searched among the points of its own sample only.
static void knn_core(sv_context* ctx, const float* X32, const float* sq, int64_t n, int dp, int d, int k,
                     int include_self, int cosine, int precision, sv_knn* out,
                     const std::vector<int64_t>* segs = nullptr) {
  // candidates per query: at least 2k; the tensor-core stage always keeps 64
  // candidates per query: 32 or 64 from the FP32 tiles, 40 (k <= 20) or 64 from
  // the tensor-core tiles
  int K2 = precision == SV_KNN_BF16 ? (2 * k <= 40 ? 40 : 64) : (2 * k <= 32 ? 32 : 64);
  if (2 * k > 64) sv_throw(SV_ERR_UNSUPPORTED, "k = %d exceeds the supported maximum of 32", k);
  DevBuf<int32_t> cand((size_t)n * K2);
  bool done = false;
  if (precision == SV_KNN_BF16) {
    int st = sv_knn_tc_candidates(ctx, X32, sq, n, dp, d, K2, include_self, cand.get(), segs);
    if (st != SV_OK) sv_throw(st, "tensor-core kNN failed");
    done = true;
  }
  if (!done) {
    // FP32 tiles: one launch per sample (each on its own rows)
    std::vector<int64_t> one = {0, n};
    const std::vector<int64_t>& sg = segs ? *segs : one;
    for (size_t g = 0; g + 1 < sg.size(); ++g) {
      int64_t o = sg[g], ns = sg[g + 1] - sg[g];
      if (ns <= 0) continue;
      const float* Xs = X32 + o * dp;
      const float* qs = sq + o;
      int32_t* cs = cand.get() + o * K2;
      switch (dp) {
        case 8: launch_fp32<8>(ctx, Xs, qs, ns, K2, include_self, cs); break;
        case 16: launch_fp32<16>(ctx, Xs, qs, ns, K2, include_self, cs); break;
        case 24: launch_fp32<24>(ctx, Xs, qs, ns, K2, include_self, cs); break;
        case 32: launch_fp32<32>(ctx, Xs, qs, ns, K2, include_self, cs); break;
        case 40: launch_fp32<40>(ctx, Xs, qs, ns, K2, include_self, cs); break;
        case 48: launch_fp32<48>(ctx, Xs, qs, ns, K2, include_self, cs); break;
        case 56: launch_fp32<56>(ctx, Xs, qs, ns, K2, include_self, cs); break;
        case 64: launch_fp32<64>(ctx, Xs, qs, ns, K2, include_self, cs); break;
        default: sv_throw(SV_ERR_UNSUPPORTED, "padded dimension %d", dp);
      }
      if (o > 0)
        sv_launch(ctx, "knn_offset", k_add_offset, dim3(sv_grid_for(ctx, ns * K2, 256, 4)), dim3(256), 0,
                  cs, ns * K2, (int32_t)o);
    }
  }
  out->n = n;
  out->k = k;
  out->idx.alloc((size_t)n * k);
  out->dist.alloc((size_t)n * k);
  switch (dp) {
#define RR(D) case D: launch_rerank<D>(ctx, X32, n, cand.get(), K2, k, include_self, cosine, out->idx.get(), out->dist.get()); break;
    RR(8) RR(16) RR(24) RR(32) RR(40) RR(48) RR(56) RR(64)
#undef RR
  }
  sv_sync(ctx);
}

static void knn_validate(int64_t n, int64_t d, int64_t k, int metric, int include_self, int precision) {
  SV_REQUIRE(n >= 1 && d >= 1, "bad sizes");
  SV_REQUIRE(n < (1ll << 31), "n exceeds Int32 indices");
  SV_REQUIRE(k >= 1 && k <= (include_self ? n : n - 1), "k must be in 1..n (1..n-1 without self)");
  SV_REQUIRE(metric == SV_EUCLIDEAN || metric == SV_COSINE, "unknown metric");
  SV_REQUIRE(precision == SV_KNN_FP32 || precision == SV_KNN_BF16, "unknown precision");
  if (d > 64) sv_throw(SV_ERR_UNSUPPORTED, "d = %lld > 64 dimensions", (long long)d);
}

static void knn_outputs(sv_context* ctx, sv_knn* h, int dtype, int32_t* nn_index, void* distances) {
  int64_t n = h->n;
  int k = (int)h->k;
  if (!nn_index && !distances) return;
  DevBuf<int32_t> oi(nn_index ? (size_t)n * k : 1);
  DevBuf<unsigned char> od(distances ? (size_t)n * k * (dtype == SV_F64 ? 8 : 4) : 1);
  sv_launch(ctx, "knn_layout", k_to_host_layout, dim3(sv_grid_for(ctx, n * k, 256, 8)), dim3(256), 0,
            (const int32_t*)h->idx.get(), (const float*)h->dist.get(), n, k,
            nn_index ? oi.get() : (int32_t*)nullptr,
            distances && dtype == SV_F32 ? (float*)od.get() : (float*)nullptr,
            distances && dtype == SV_F64 ? (double*)od.get() : (double*)nullptr);
  if (nn_index) sv_d2h(ctx, nn_index, oi.get(), (size_t)n * k * 4);
  if (distances) sv_d2h(ctx, distances, od.get(), (size_t)n * k * (dtype == SV_F64 ? 8 : 4));
}

SV_API int sv_knn_host(sv_context* ctx, const void* X, int dtype, int64_t n, int64_t d, int64_t ldX,
                       int64_t k, int metric, int include_self, int precision, int32_t* nn_index,
                       void* distances, sv_knn** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(X, "X is null");
  SV_REQUIRE(dtype == SV_F32 || dtype == SV_F64, "dtype must be F32 or F64");
  knn_validate(n, d, k, metric, include_self, precision);
  SV_REQUIRE(ldX >= n, "ldX < n");
  int dp = (int)((d + 7) / 8 * 8);
  size_t es = dtype == SV_F64 ? 8 : 4;
  DevBuf<unsigned char> dX((size_t)ldX * (d - 1) * es + (size_t)n * es);
  sv_h2d(ctx, dX.get(), X, ((size_t)ldX * (d - 1) + n) * es);
  DevBuf<float> X32((size_t)n * dp), sq(n);
  if (dtype == SV_F64)
    sv_launch(ctx, "knn_pack", k_pack_rows<double>, dim3(sv_grid_for(ctx, n, 256, 8)), dim3(256), 0,
              (const double*)dX.get(), ldX, n, (int)d, dp, metric == SV_COSINE, X32.get(), sq.get());
  else
    sv_launch(ctx, "knn_pack", k_pack_rows<float>, dim3(sv_grid_for(ctx, n, 256, 8)), dim3(256), 0,
              (const float*)dX.get(), ldX, n, (int)d, dp, metric == SV_COSINE, X32.get(), sq.get());
  auto* h = new sv_knn();
  try {
    h->ctx = ctx;
    knn_core(ctx, X32.get(), sq.get(), n, dp, (int)d, (int)k, include_self, metric == SV_COSINE, precision, h);
    knn_outputs(ctx, h, dtype, nn_index, distances);
  } catch (...) {
    delete h;
    throw;
  }
  if (out) *out = h;
  else delete h;
  SV_CATCH
}

SV_API int sv_knn_embed(sv_context* ctx, const sv_embed* e, int64_t ndims, int64_t k, int metric,
                        int include_self, int precision, int32_t* nn_index, double* distances,
                        sv_knn** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(e && e->ctx == ctx, "bad embedding handle");
  if (ndims <= 0) ndims = e->npcs;
  SV_REQUIRE(ndims <= e->npcs, "ndims exceeds the embedding's components");
  int64_t n = e->n_cells;
  knn_validate(n, ndims, k, metric, include_self, precision);
  int dp = (int)((ndims + 7) / 8 * 8);
  DevBuf<float> X32((size_t)n * dp), sq(n);
  sv_launch(ctx, "knn_pack", k_pack_rows<double>, dim3(sv_grid_for(ctx, n, 256, 8)), dim3(256), 0,
            (const double*)e->Z.get(), n, n, (int)ndims, dp, metric == SV_COSINE, X32.get(), sq.get());
  auto* h = new sv_knn();
  try {
    h->ctx = ctx;
    knn_core(ctx, X32.get(), sq.get(), n, dp, (int)ndims, (int)k, include_self, metric == SV_COSINE, precision, h);
    knn_outputs(ctx, h, SV_F64, nn_index, distances);
  } catch (...) {
    delete h;
    throw;
  }
  if (out) *out = h;
  else delete h;
  SV_CATCH
}

// ann over the PCA coordinates of a batch: every cell's neighbours among the
// cells of its own sample, all samples in the same launches (the tensor-core
// candidate kernel takes one sample per CTA).  Indices are stacked rows
// (1-based), as sv_knn_embed returns them.
SV_API int sv_batch_knn(sv_context* ctx, const sv_batch* b, const sv_embed* e, int64_t ndims, int64_t k,
                        int metric, int include_self, int precision, int32_t* nn_index, double* distances,
                        sv_knn** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(b && b->ctx == ctx, "bad batch handle");
  SV_REQUIRE(e && e->ctx == ctx && e->n_cells == b->n_cells, "bad embedding handle");
  if (ndims <= 0) ndims = e->npcs;
  SV_REQUIRE(ndims <= e->npcs, "ndims exceeds the embedding's components");
  int64_t n = e->n_cells;
  int64_t minc = n;
  for (int64_t s = 0; s < b->nseg; ++s) minc = std::min(minc, b->hoff[s + 1] - b->hoff[s]);
  knn_validate(minc, ndims, k, metric, include_self, precision);
  int dp = (int)((ndims + 7) / 8 * 8);
  DevBuf<float> X32((size_t)n * dp), sq(n);
  sv_launch(ctx, "knn_pack", k_pack_rows<double>, dim3(sv_grid_for(ctx, n, 256, 8)), dim3(256), 0,
            (const double*)e->Z.get(), n, n, (int)ndims, dp, metric == SV_COSINE, X32.get(), sq.get());
  auto* h = new sv_knn();
  try {
    h->ctx = ctx;
    knn_core(ctx, X32.get(), sq.get(), n, dp, (int)ndims, (int)k, include_self, metric == SV_COSINE, precision, h,
             &b->hoff);
    knn_outputs(ctx, h, SV_F64, nn_index, distances);
  } catch (...) {
    delete h;
    throw;
  }
  if (out) *out = h;
  else delete h;
  SV_CATCH
}

SV_API int sv_knn_info(const sv_knn* h, int64_t* n, int64_t* k) {
  SV_TRY
  SV_REQUIRE(h, "null handle");
  if (n) *n = h->n;
  if (k) *k = h->k;
  SV_CATCH
}

SV_API int sv_knn_free(sv_knn* h) {
  if (h) {
    if (h->ctx) cudaSetDevice(h->ctx->device);
    delete h;
  }
  return SV_OK;
}

// ---- drop-ins for the native libcell symbols ------------------------------------
static void find_neighbours(const void* X, int dtype, int n, int d, int ldX, int k, int include_self,
                            int metric, int32_t* nn_index, void* distances) {
  int st;
  try {
    sv_context* ctx = sv_default_context();
    st = sv_knn_host(ctx, X, dtype, n, d, ldX, k, metric, include_self, SV_KNN_FP32, nn_index,
                     distances, nullptr);
  } catch (const SvError& e) {
    st = e.code;
  } catch (...) {
    st = SV_ERR_CUDA;
  }
  if (st != SV_OK && nn_index && n > 0 && k > 0) memset(nn_index, 0, (size_t)n * k * sizeof(int32_t));
}

SV_API void FindNeighboursEuclidean32(const float* X, int n, int d, int ldX, int k, int ntables,
                                      int include_self, int seed, int32_t* nn_index, float* distances) {
  (void)ntables;
  (void)seed;
  find_neighbours(X, SV_F32, n, d, ldX, k, include_self, SV_EUCLIDEAN, nn_index, distances);
}

SV_API void FindNeighboursEuclidean64(const double* X, int n, int d, int ldX, int k, int ntables,
                                      int include_self, int seed, int32_t* nn_index, double* distances) {
  (void)ntables;
  (void)seed;
  find_neighbours(X, SV_F64, n, d, ldX, k, include_self, SV_EUCLIDEAN, nn_index, distances);
}

SV_API void FindNeighboursCosine32(const float* X, int n, int d, int ldX, int k, int ntables,
                                   int include_self, int seed, int32_t* nn_index, float* distances) {
  (void)ntables;
  (void)seed;
  find_neighbours(X, SV_F32, n, d, ldX, k, include_self, SV_COSINE, nn_index, distances);
}

SV_API void FindNeighboursCosine64(const double* X, int n, int d, int ldX, int k, int ntables,
                                   int include_self, int seed, int32_t* nn_index, double* distances) {
  (void)ntables;
  (void)seed;
  find_neighbours(X, SV_F64, n, d, ldX, k, include_self, SV_COSINE, nn_index, distances);
}
