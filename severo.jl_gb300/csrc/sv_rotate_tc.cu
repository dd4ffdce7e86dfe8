// Restart rotation of the cell-side Lanczos basis, W <- W M (W: len x nin
// double-float, column-major; M: nin x nout FP64), on the tensor cores and
// exact to double-float accuracy, by splitting both operands into BF16 digit
// slices (the error-free splitting of Ozaki, Ogita, Oishi and Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59, 2012):
//   row i of W:     x = 2^e_i  sum_s a_s 2^(-7-8s),   a_s integers in [-128, 128]
//   column c of M:  m = 2^f_c  sum_t b_t 2^(-7-8t),   b_t integers in [-128, 128]
// with six slices each (48 bits).  A slice product a_s b_t is a BF16 GEMM
// whose terms are integers of at most 2^14, so a 64-long dot product stays
// below 2^20 and the (at most six) products of one level L = s + t are summed
// exactly in one FP32 tensor-memory accumulator (below 2^23).  Levels L <= 5
// are formed (21 slice products); the rest lies below 2^-48 of the row and
// column scales.  The epilogue combines the levels by Horner in double-float
// and scales by 2^(e_i + f_c - 14).
//
// One CTA per SM, persistent over tiles of 128 rows (MMA M = 128, N = 64
// output columns, K = 64 basis columns); 16 warps, four threads per row (thread
// t: row t mod 128, quarter q = t / 128, which is also the warp's TMEM lane
// quarter and column group).  Per tile: the raw double-float rows (boxes of
// 128 rows x 8 columns, hi and lo) arrive by TMA during the previous tile's
// MMAs and epilogue; each thread cuts 16 columns of its row into slices,
// written in the 128-byte-swizzled K-major layout; one thread issues the
// 21 x 4 MMAs (K = 16 each) and commits; each thread reads 16 output columns
// of its row from the six accumulators, combines and stores them.  Every wait is bounded; on a
// timeout the CTA records SV_STATUS_LIMIT, lets its copies and MMAs land
// (bounded), frees its tensor memory and returns.
#include "sv_internal.cuh"
#include "sv_tc.cuh"

namespace {

using namespace sv_tc;

constexpr int RT_ROWS = 128;          // rows per tile (MMA M)
constexpr int RT_K = 64;              // basis columns, padded (MMA K)
constexpr int RT_N = 64;              // output columns, padded (MMA N)
constexpr int RT_SLICES = 6;
constexpr int RT_THREADS = 512;
constexpr int RT_GC = 8;              // columns per tensor box
constexpr long long RT_TIMEOUT = 4000000000ll;   // cycles (~2 s) per wait
constexpr uint32_t RT_IDESC = idesc_bf16(RT_ROWS, RT_N);

constexpr size_t RT_A_BYTES = (size_t)RT_SLICES * RT_ROWS * RT_K * 2;      // 96 KB
constexpr size_t RT_B_BYTES = (size_t)RT_SLICES * RT_N * RT_K * 2;         // 48 KB
constexpr size_t RT_RAW_BYTES = (size_t)(RT_K / RT_GC) * 2 * RT_GC * RT_ROWS * 4;   // 64 KB
constexpr size_t RT_SMEM = RT_A_BYTES + RT_B_BYTES + RT_RAW_BYTES + 1024;

// byte offset of element (row, k) of a 64-wide K-major BF16 operand in the
// 128-byte-swizzled layout (row r at r * 128, 16-byte chunk j at j ^ (r & 7))
__host__ __device__ __forceinline__ uint32_t sw_off(int row, int k) {
  return (uint32_t)row * 128u + ((uint32_t)((k >> 3) ^ (row & 7)) << 4) + (uint32_t)(k & 7) * 2u;
}

__device__ __forceinline__ float pow2f(int e) {   // 2^e for e in [-126, 127]
  return __int_as_float((127 + e) << 23);
}

// (s, e) = the sum of a and b and its rounding error (two-sum)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float v = s - a;
  e = (a - (s - v)) + (b - v);
}

// Column slices of M: one block per output column c (64 threads, one per basis
// row r): f_c = the exponent of the column's largest entry, digits by exact FP64
// steps, written as BF16 in the swizzled K-major layout of the B operand
// (row = c); columns c >= nout and rows r >= nin are zero.
__global__ void __launch_bounds__(RT_K) k_rotate_tc_bslices(const double* __restrict__ M, int nin, int nout,
                                                            unsigned char* __restrict__ bsl, int* __restrict__ fexp) {
  __shared__ double wmax[2];
  const int c = blockIdx.x, r = threadIdx.x;
  const double x = (c < nout && r < nin) ? M[r + (int64_t)c * nin] : 0.0;
  double a = fabs(x);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
  if ((r & 31) == 0) wmax[r >> 5] = a;
  __syncthreads();
  const double mx = fmax(wmax[0], wmax[1]);
  const int f = mx > 0.0 ? ilogb(mx) + 1 : 0;
  double rem = ldexp(x, -f) * 128.0;   // |rem| < 128 (exact scaling)
  for (int t = 0; t < RT_SLICES; ++t) {
    const double d = rint(rem);
    rem = (rem - d) * 256.0;           // exact: |rem - d| <= 1/2, 53-bit significand
    *(__nv_bfloat16*)(bsl + (size_t)t * RT_N * RT_K * 2 + sw_off(c, r)) = __float2bfloat16_rn((float)d);
  }
  if (r == 0) fexp[c] = f;
}

__global__ void __launch_bounds__(RT_THREADS, 1) k_rotate_tc(
    const __grid_constant__ CUtensorMap mh, const __grid_constant__ CUtensorMap ml, int64_t len, int nin,
    int nout, const unsigned char* __restrict__ bsl, const int* __restrict__ fexp, float* __restrict__ outh,
    float* __restrict__ outl, int64_t ld_out, int* __restrict__ status) {
  extern __shared__ unsigned char rt_dyn[];
  unsigned char* base = (unsigned char*)(((uintptr_t)rt_dyn + 1023) & ~(uintptr_t)1023);
  unsigned char* As = base;                          // RT_SLICES x (128 x 64) BF16
  unsigned char* Bs = As + RT_A_BYTES;               // RT_SLICES x (64 x 64) BF16
  float* raw = (float*)(Bs + RT_B_BYTES);            // groups x {hi, lo} x [8][128]
  __shared__ unsigned long long full, mdone;
  __shared__ uint32_t tbase;
  __shared__ int err;
  __shared__ int fx[RT_N];
  __shared__ float rmx[RT_THREADS / RT_ROWS][RT_ROWS];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int r = tid & (RT_ROWS - 1);    // the thread's row in a tile
  const int qq = tid / RT_ROWS;         // its column quarter (cutting and output)
  const int ngroups = (nin + RT_GC - 1) / RT_GC;
  const uint32_t raw_bytes = (uint32_t)ngroups * 2u * RT_GC * RT_ROWS * 4u;
  const int64_t ntiles = (len + RT_ROWS - 1) / RT_ROWS;

  if (tid == 0) {
    mbar_init(&full, 1);
    mbar_init(&mdone, 1);
    err = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(&tbase, 512);
  for (int i = tid; i < (int)(RT_B_BYTES / 16); i += RT_THREADS)
    ((uint4*)Bs)[i] = ((const uint4*)bsl)[i];
  if (tid < RT_N) fx[tid] = fexp[tid];
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tbase;

  auto issue_raw = [&](int64_t t) {
    mbar_expect_tx(&full, raw_bytes);
    const int x = (int)(t * RT_ROWS);
    for (int g = 0; g < ngroups; ++g) {
      tma_load_2d(raw + (size_t)g * 2 * RT_GC * RT_ROWS, &mh, x, g * RT_GC, &full);
      tma_load_2d(raw + (size_t)g * 2 * RT_GC * RT_ROWS + RT_GC * RT_ROWS, &ml, x, g * RT_GC, &full);
    }
  };
  // thread 0: what is in flight, and the barrier phase it completes
  bool raw_pending = false, mma_pending = false;
  int raw_it = 0;
  if (tid == 0 && (int64_t)blockIdx.x < ntiles) {
    issue_raw(blockIdx.x);
    raw_pending = true;
    raw_it = 0;
  }
  int it = 0;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
    // the tile's raw rows
    if (!mbar_wait_for(&full, (uint32_t)(it & 1), RT_TIMEOUT)) atomicOr(&err, 1);
    __syncthreads();
    if (err) break;
    if (tid == 0) raw_pending = false;
    // this thread's row: exponent (the largest entry, over the row's four
    // threads), then six digit slices of its 16 basis columns
    float mx = 0.f;
    for (int c = 16 * qq; c < 16 * qq + 16 && c < nin; ++c)
      mx = fmaxf(mx, fabsf(raw[(size_t)(c >> 3) * 2 * RT_GC * RT_ROWS + (c & 7) * RT_ROWS + r]));
    rmx[qq][r] = mx;
    __syncthreads();
    mx = fmaxf(fmaxf(rmx[0][r], rmx[1][r]), fmaxf(rmx[2][r], rmx[3][r]));
    const int e = mx > 0.f ? max(-100, min(100, ilogbf(mx) + 1)) : 0;
    const float sc = pow2f(-e) * 128.f;
#pragma unroll 1
    for (int ch = 2 * qq; ch < 2 * qq + 2; ++ch) {
      uint32_t w[RT_SLICES][4];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int c = ch * 8 + j;
        float rh = 0.f, rl = 0.f;
        if (c < nin) {
          const float* p = raw + (size_t)(c >> 3) * 2 * RT_GC * RT_ROWS + (c & 7) * RT_ROWS + r;
          rh = p[0] * sc;                    // exact: scaling by a power of two
          rl = p[RT_GC * RT_ROWS] * sc;
        }
        float dg[RT_SLICES];
#pragma unroll
        for (int s = 0; s < RT_SLICES; ++s) {
          const float d = rintf(rh);
          dg[s] = d;
          float u = rh - d, v = rl;          // u exact (|u| <= 1/2)
          two_sum(u, v, rh, rl);
          rh *= 256.f;
          rl *= 256.f;
        }
#pragma unroll
        for (int s = 0; s < RT_SLICES; ++s) {
          const uint32_t b = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(dg[s]));
          if (j & 1) w[s][j >> 1] |= b << 16;
          else w[s][j >> 1] = b;
        }
      }
#pragma unroll
      for (int s = 0; s < RT_SLICES; ++s)
        *(uint4*)(As + (size_t)s * RT_ROWS * RT_K * 2 + ((uint32_t)r * 128u + ((uint32_t)(ch ^ (r & 7)) << 4))) =
            make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    fence_before();
    __syncthreads();
    fence_after();
    if (tid == 0) {
      // the raw buffer is read: bring the next tile's rows
      if (t + gridDim.x < ntiles) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue_raw(t + gridDim.x);
        raw_pending = true;
        raw_it = it + 1;
      }
      for (int L = 0; L < RT_SLICES; ++L) {
        bool first = true;
        for (int s = 0; s < RT_SLICES; ++s) {
          const int tt = L - s;
          if (tt < 0 || tt >= RT_SLICES) continue;
          const uint32_t a0 = su32(As + (size_t)s * RT_ROWS * RT_K * 2);
          const uint32_t b0 = su32(Bs + (size_t)tt * RT_N * RT_K * 2);
#pragma unroll
          for (int kk = 0; kk < RT_K / 16; ++kk)
            mma_bf16(tmem + (uint32_t)(L * RT_N), sw128_desc(a0 + kk * 32), sw128_desc(b0 + kk * 32), RT_IDESC,
                     (first && kk == 0) ? 0u : 1u);
          first = false;
        }
      }
      mma_commit(&mdone);
      mma_pending = true;
    }
    if (!mbar_wait_for(&mdone, (uint32_t)(it & 1), RT_TIMEOUT)) atomicOr(&err, 1);
    __syncthreads();
    if (err) break;
    if (tid == 0) mma_pending = false;
    fence_after();
    // epilogue: the six levels of this thread's 16 output columns (its warp's
    // lane quarter is its row block, its column group is qq)
    const int64_t row = t * RT_ROWS + r;
    const uint32_t tl = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    if (16 * qq < nout) {
      float h[16], l[16];
      uint32_t v[16];
      tmem_ld16(tl + (uint32_t)((RT_SLICES - 1) * RT_N + 16 * qq), v);
      tmem_ld_wait();
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        h[i] = __uint_as_float(v[i]);
        l[i] = 0.f;
      }
      for (int L = RT_SLICES - 2; L >= 0; --L) {
        tmem_ld16(tl + (uint32_t)(L * RT_N + 16 * qq), v);
        tmem_ld_wait();
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          float s2, e2;
          two_sum(h[i] * 0x1p-8f, __uint_as_float(v[i]), s2, e2);
          h[i] = s2;
          l[i] = l[i] * 0x1p-8f + e2;
        }
      }
      if (row < len) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int c = 16 * qq + i;
          if (c < nout) {
            const float sc2 = pow2f(max(-126, min(127, e + fx[c] - 14)));
            const float hh = h[i] * sc2, ll = l[i] * sc2;
            const float s2 = hh + ll;
            outh[(int64_t)c * ld_out + row] = s2;
            outl[(int64_t)c * ld_out + row] = ll - (s2 - hh);
          }
        }
      }
    }
    fence_before();
    __syncthreads();
    fence_after();
  }
  // a timeout: let the copies and MMAs in flight land (bounded) before freeing
  if (tid == 0) {
    if (raw_pending) mbar_wait_for(&full, (uint32_t)(raw_it & 1), RT_TIMEOUT);
    if (mma_pending) mbar_wait_for(&mdone, (uint32_t)(it & 1), RT_TIMEOUT);
    if (err) atomicOr(status, SV_STATUS_LIMIT);
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0) tmem_free(tmem, 512);
}

}  // namespace

// The cell-side restart rotation on the tensor cores: out[:, c] = in M[:, c] for
// c < nout (in: len x nin double-float with leading dimension ld_in, a multiple
// of 4; out: leading dimension ld_out).  nin, nout <= 64.  bsl (48 KB) and
// fexp (64 ints) are device scratch owned by the caller (no allocation here:
// the call is captured in the Lanczos cycle graphs).
bool sv_rotate_tc_supported(int nin, int nout, int64_t ld_in) {
  return nin >= 1 && nin <= RT_K && nout >= 1 && nout <= RT_N && ld_in % 4 == 0 && !getenv("SV_NO_ROTATE_TC");
}

void sv_rotate_tc(sv_context* ctx, const float* inh, const float* inl, int64_t ld_in, int64_t len, int nin,
                  const double* M, int nout, float* outh, float* outl, int64_t ld_out, unsigned char* bsl,
                  int* fexp) {
  // per call: the attribute belongs to the current device
  SV_CUDA(cudaFuncSetAttribute(k_rotate_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RT_SMEM));
  sv_launch(ctx, "irlba_rotate_tc_b", k_rotate_tc_bslices, dim3(RT_N), dim3(RT_K), 0, M, nin, nout, bsl, fexp);
  CUtensorMap mh, ml;
  cuuint64_t gdim[2] = {(cuuint64_t)len, (cuuint64_t)nin};
  cuuint64_t gstride[1] = {(cuuint64_t)ld_in * 4};
  cuuint32_t box[2] = {(cuuint32_t)RT_ROWS, (cuuint32_t)RT_GC};
  cuuint32_t estr[2] = {1, 1};
  for (int a = 0; a < 2; ++a) {
    CUresult r = sv_encode_tiled()(a ? &ml : &mh, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)(a ? inl : inh), gdim,
                                   gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) sv_throw(SV_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  }
  const int64_t ntiles = (len + RT_ROWS - 1) / RT_ROWS;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, ctx->num_sms));
  sv_launch(ctx, "irlba_rotate", k_rotate_tc, dim3(grid), dim3(RT_THREADS), RT_SMEM, mh, ml, len, nin, nout,
            (const unsigned char*)bsl, (const int*)fexp, outh, outl, ld_out, ctx->d_status);
}
