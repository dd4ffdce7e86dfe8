// irlba on the device: augmented implicitly restarted Lanczos bidiagonalisation
// (Baglama & Reichel, SIAM J. Sci. Comput. 27 (2005)), the routine that
// src/irlba.jl:47-76 reaches through the native `irlba` symbol.
//
//   A V_j = W_j B_j,  A^T W_j = V_j B_j^T + f e_j^T      (A = Xs, m x n)
//
// Both Lanczos bases live in HBM, column-major: W (m x work, the cell side,
// 1.3M x 57 at the atlas size) and V (n x work, the feature side).  They are held
// in double-float form -- each value as an unevaluated sum hi + lo of two FP32
// numbers (about 48 significand bits) -- and all basis arithmetic runs on the
// FP32 pipe with exact two-product / two-sum steps: GB300 executes FP64 at
// 1/57 of its FP32 rate, and the reorthogonalisation and restart rotation are
// the only O(m * work) arithmetic of the method.  Reductions across blocks,
// the norms and the small matrix B are FP64; the SVD of B is double-float.
//
// Every new vector is reorthogonalised against its basis by classical
// Gram-Schmidt applied twice (CGS2).  After `work` steps B (work x work, upper
// triangular) is decomposed by a one-block one-sided Jacobi SVD; the nu
// leading Ritz vectors are kept (thick restart):
//   V <- [V Q_k, f/|f|],  W <- W P_k,  B <- [diag(s_k) rho; 0 ...],
//   rho_i = |f| P[work-1, i]
// and convergence is declared when every |rho_i| < tol * max singular value
// (the residual ||A^T u_i - s_i v_i||).  A cycle (restart, Lanczos steps, SVD)
// is enqueued without host round trips and, over a device operator, captured
// once as a CUDA graph and replayed; the host reads back 2*work+2 doubles per
// cycle to test convergence.
#include "sv_internal.cuh"
#include <math.h>
#include <stdlib.h>

void sv_centered_apply(sv_context* ctx, const sv_centered* S, char trans, const double* x, double* y,
                       double alpha, double beta, const double* csub, const double* z);
bool sv_centered_apply_df(sv_context* ctx, const sv_centered* S, const float* xh, const float* xl,
                          float* yh, float* yl, const double* csub, const float* zh, const float* zl);

namespace {

constexpr int RED_BLOCKS = 608;    // blocks of the tall reductions (4 per SM)
constexpr int MAX_WORK = 96;       // largest Lanczos basis the Jacobi kernel holds in smem

// ---- double-float arithmetic --------------------------------------------------
__device__ __forceinline__ void df_split(double x, float& h, float& l) {
  h = (float)x;
  l = (float)(x - (double)h);
}
__device__ __forceinline__ double df_val(float h, float l) { return (double)h + (double)l; }

// s += a * b: exact product of the high parts (FMA), first-order cross terms,
// two-sum accumulation of the high part
__device__ __forceinline__ void df_fma(float& sh, float& sl, float ah, float al, float bh, float bl) {
  float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  float t = sh + p;
  float v = t - sh;
  float err = (sh - (t - v)) + (p - v);
  sh = t;
  sl += err + e;
}

// (xh, xl) - (sh, sl), renormalised
__device__ __forceinline__ void df_sub(float& xh, float& xl, float sh, float sl) {
  float t = xh - sh;
  float v = t - xh;
  float err = (xh - (t - v)) + (-sh - v);
  float lo = err + xl - sl;
  float h = t + lo;
  xl = lo - (h - t);
  xh = h;
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = sv_warp_sum(v);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0;
  if (wid == 0) {
    r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    r = sv_warp_sum(r);
  }
  return r;  // valid in thread 0
}

// last-block pattern: every block has written its partials; the last one to
// arrive sums them in block order (deterministic) and resets the counter
__device__ __forceinline__ bool last_block(unsigned int* counter, bool* flag_smem) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) *flag_smem = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (*flag_smem) __threadfence();
  return *flag_smem;
}

// One pass of the CGS2 reorthogonalisation of the working vector x against the
// basis Q[:, :ncols] (both double-float), in three fusable parts:
//   UPDATE  x -= Q cin (cin from the previous pass), x written back;
//   DOTS    cout = Q^T x (of the updated x when UPDATE);
//   NORM    *nrm = ||x|| (after the update).
// A CGS2 step is then three launches that read the basis three times: DOTS
// (x taken from the FP64 product y and stored as the working vector), UPDATE +
// DOTS, UPDATE + NORM.  Block of 8 warps over a contiguous row segment, 64 rows
// per iteration (two per lane); warp w owns the columns j = w + 8t, so every
// basis element is loaded once, coalesced, with 4*NJ loads in flight per thread.
// The update sums each row's 8 per-warp partial products through shared memory;
// the dot products accumulate per lane and reduce across lanes once at the end.
// Per-block FP64 partials; the last block reduces them in block order
// (deterministic).  NJ = columns per warp: 8 for bases of up to 64 columns,
// 12 up to MAX_WORK (fewer registers, more resident blocks for the usual
// nu + 7 basis).

// (sh, sl) += (bh, bl), unnormalised
__device__ __forceinline__ void df_acc(float& sh, float& sl, float bh, float bl) {
  float t = sh + bh;
  float v = t - sh;
  float err = (sh - (t - v)) + (bh - v);
  sh = t;
  sl += err + bl;
}

template <int NJ, bool UPDATE, bool DOTS, bool NORM>
__global__ void __launch_bounds__(256) k_cgs_df(const float* __restrict__ Qh,
                                                const float* __restrict__ Ql, int64_t ld, int ncols,
                                                float* __restrict__ xh, float* __restrict__ xl,
                                                const double* __restrict__ y, int64_t len,
                                                const double* __restrict__ cin,
                                                double* __restrict__ part, double* __restrict__ npart,
                                                double* __restrict__ cout, double* __restrict__ nrm,
                                                unsigned int* __restrict__ counter) {
  __shared__ float csh[MAX_WORK], csl[MAX_WORK];
  __shared__ float redh[8][64], redl[8][64];
  __shared__ float xsh[64], xsl[64];
  __shared__ double nsh[32];
  __shared__ bool last;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  if (UPDATE)
    for (int j = tid; j < ncols; j += blockDim.x) df_split(cin[j], csh[j], csl[j]);
  __syncthreads();
  int64_t seg = (len + gridDim.x - 1) / gridDim.x;
  int64_t r0 = (int64_t)blockIdx.x * seg, r1 = min(len, r0 + seg);
  float ah[NJ], al[NJ];
#pragma unroll
  for (int t = 0; t < NJ; ++t) ah[t] = al[t] = 0.f;
  double nacc = 0;
  for (int64_t i0 = r0; i0 < r1; i0 += 64) {
    int64_t ia = i0 + lane, ib = ia + 32;
    bool va = ia < r1, vb = ib < r1;
    float q0h[NJ], q0l[NJ], q1h[NJ], q1l[NJ];
#pragma unroll
    for (int t = 0; t < NJ; ++t) {
      int j = w + 8 * t;
      int64_t o = (int64_t)j * ld + ia;
      q0h[t] = q0l[t] = q1h[t] = q1l[t] = 0.f;
      if (j < ncols) {
        if (va) {
          q0h[t] = Qh[o];
          q0l[t] = Ql[o];
        }
        if (vb) {
          q1h[t] = Qh[o + 32];
          q1l[t] = Ql[o + 32];
        }
      }
    }
    float x0h, x0l, x1h, x1l;
    if (UPDATE) {
      float s0h = 0.f, s0l = 0.f, s1h = 0.f, s1l = 0.f;
#pragma unroll
      for (int t = 0; t < NJ; ++t) {
        int j = w + 8 * t;
        if (j < ncols) {
          df_fma(s0h, s0l, q0h[t], q0l[t], csh[j], csl[j]);
          df_fma(s1h, s1l, q1h[t], q1l[t], csh[j], csl[j]);
        }
      }
      redh[w][lane] = s0h;
      redl[w][lane] = s0l;
      redh[w][lane + 32] = s1h;
      redl[w][lane + 32] = s1l;
      __syncthreads();
      if (tid < 64) {
        int64_t i = i0 + tid;
        float h = 0.f, l = 0.f;
        if (i < r1) {
          float sh = 0.f, sl = 0.f;
#pragma unroll
          for (int u = 0; u < 8; ++u) df_acc(sh, sl, redh[u][tid], redl[u][tid]);
          h = xh[i];
          l = xl[i];
          df_sub(h, l, sh, sl);
          xh[i] = h;
          xl[i] = l;
          if (NORM) {
            double v = df_val(h, l);
            nacc += v * v;
          }
        }
        xsh[tid] = h;
        xsl[tid] = l;
      }
      __syncthreads();
      x0h = xsh[lane];
      x0l = xsl[lane];
      x1h = xsh[lane + 32];
      x1l = xsl[lane + 32];
    } else if (y) {
      // x from the FP64 product; warp 0 stores the working copy
      double ya = va ? y[ia] : 0.0, yb = vb ? y[ib] : 0.0;
      df_split(ya, x0h, x0l);
      df_split(yb, x1h, x1l);
      if (w == 0) {
        if (va) {
          xh[ia] = x0h;
          xl[ia] = x0l;
        }
        if (vb) {
          xh[ib] = x1h;
          xl[ib] = x1l;
        }
      }
    } else {
      x0h = va ? xh[ia] : 0.f;
      x0l = va ? xl[ia] : 0.f;
      x1h = vb ? xh[ib] : 0.f;
      x1l = vb ? xl[ib] : 0.f;
    }
    if (DOTS) {
#pragma unroll
      for (int t = 0; t < NJ; ++t) {
        if (w + 8 * t < ncols) {
          df_fma(ah[t], al[t], q0h[t], q0l[t], x0h, x0l);
          df_fma(ah[t], al[t], q1h[t], q1l[t], x1h, x1l);
        }
      }
    }
  }
  if (DOTS) {
#pragma unroll
    for (int t = 0; t < NJ; ++t) {
      int j = w + 8 * t;
      if (j < ncols) {
        // warp reduction in double-float (FP32 shuffles), one FP64 value per warp
        float h = ah[t], l = al[t];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          float h2 = __shfl_xor_sync(0xffffffffu, h, o);
          float l2 = __shfl_xor_sync(0xffffffffu, l, o);
          float s = h + h2;
          float v = s - h;
          float err = (h - (s - v)) + (h2 - v);
          float lo = err + l + l2;
          h = s + lo;
          l = lo - (h - s);
        }
        if (lane == 0) part[(int64_t)blockIdx.x * ncols + j] = df_val(h, l);
      }
    }
  }
  if (NORM) {
    nacc = block_sum(nacc, nsh);
    if (tid == 0) npart[blockIdx.x] = nacc;
  }
  if (last_block(counter, &last)) {
    if (DOTS) {
      // one warp per column, lanes over blocks (block order fixed: deterministic)
      for (int j = w; j < ncols; j += 8) {
        double s = 0;
        for (unsigned b = lane; b < gridDim.x; b += 32) s += part[(int64_t)b * ncols + j];
        s = sv_warp_sum(s);
        if (lane == 0) cout[j] = s;
      }
    }
    if (NORM && tid == 0) {
      double s = 0;
      for (unsigned b = 0; b < gridDim.x; ++b) s += npart[b];
      *nrm = sqrt(s);
    }
    if (tid == 0) *counter = 0;
  }
}

// FP64 vector -> double-float working vector
__global__ void k_to_df(const double* __restrict__ y, int64_t len, float* __restrict__ xh,
                        float* __restrict__ xl) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    df_split(y[i], xh[i], xl[i]);
}

__device__ __forceinline__ unsigned long long mixbits(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double normal_at(unsigned long long seed, unsigned long long tag, int64_t i) {
  unsigned long long h1 = mixbits(seed ^ mixbits(tag * 0x9E3779B97F4A7C15ull + (unsigned long long)i));
  unsigned long long h2 = mixbits(h1 + 0x632BE59BD9B4E019ull);
  double u1 = ((double)(h1 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  double u2 = ((double)(h2 >> 11)) * (1.0 / 9007199254740992.0);
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);    // Box-Muller
}

// Control block of a Lanczos run, read by the kernels so that a captured cycle
// replays without host-side arguments: [0] breakdown threshold, [1] largest
// Ritz value so far, [2] cycle number (selects the random restart vectors).
#define CTL_THRESH 0
#define CTL_SMAX 1
#define CTL_CYCLE 2
__device__ __forceinline__ unsigned long long breakdown_tag(const double* ctl, unsigned step) {
  return (unsigned long long)ctl[CTL_CYCLE] * 1024ull + step;
}

// Basis column := x / *nrm (double-float) and cur := the same in FP64; the B
// entry := *nrm.  When *nrm < ctl[CTL_THRESH] the Krylov space is (numerically)
// invariant: cur := a random vector, B entry := 0, flag set for k_fix_df, which
// orthonormalises cur against the basis and writes the column.
__global__ void k_scal_df(const float* __restrict__ xh, const float* __restrict__ xl, int64_t len,
                          const double* __restrict__ nrm, const double* __restrict__ ctl,
                          float* __restrict__ colh, float* __restrict__ coll, double* __restrict__ cur,
                          double* __restrict__ bentry, int* __restrict__ flag,
                          unsigned long long seed, unsigned step) {
  double s = *nrm;
  bool brk = !(s >= ctl[CTL_THRESH]);
  unsigned long long tag = breakdown_tag(ctl, step);
  double inv = brk ? 0.0 : 1.0 / s;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (brk) {
      cur[i] = normal_at(seed, tag, i);
    } else {
      double v = df_val(xh[i], xl[i]) * inv;
      cur[i] = v;
      df_split(v, colh[i], coll[i]);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (bentry) *bentry = brk ? 0.0 : s;
    if (brk) *flag = 1;
  }
}

// zero the norm slot (the sub-diagonal scalar the next product uses) when a
// breakdown was flagged; separate launch so every k_scal_df block has read it
__global__ void k_scal_post(double* nrm, const int* flag) {
  if (*flag) *nrm = 0.0;
}

// One block: if *flag, cur <- CGS2(cur, Q[:, :ncols]) normalised (FP64
// arithmetic on the double-float basis), written to the basis column as well;
// clears the flag.  Runs only on a breakdown.
__global__ void k_fix_df(double* __restrict__ cur, int64_t len, const float* __restrict__ Qh,
                         const float* __restrict__ Ql, int64_t ld, int ncols, float* __restrict__ colh,
                         float* __restrict__ coll, int* __restrict__ flag) {
  __shared__ double sh[32];
  __shared__ double cs[MAX_WORK];
  __shared__ double tot;
  if (*flag == 0) return;
  for (int pass = 0; pass < 2; ++pass) {
    for (int j = 0; j < ncols; ++j) {
      double acc = 0;
      for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
        int64_t o = (int64_t)j * ld + i;
        acc += df_val(Qh[o], Ql[o]) * cur[i];
      }
      acc = block_sum(acc, sh);
      if (threadIdx.x == 0) cs[j] = acc;
    }
    __syncthreads();
    for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
      double v = cur[i];
      for (int j = 0; j < ncols; ++j) {
        int64_t o = (int64_t)j * ld + i;
        v -= df_val(Qh[o], Ql[o]) * cs[j];
      }
      cur[i] = v;
    }
    __syncthreads();
  }
  double acc = 0;
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) acc += cur[i] * cur[i];
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) tot = sqrt(acc);
  __syncthreads();
  double s = tot;
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
    double v = cur[i] / s;
    cur[i] = v;
    df_split(v, colh[i], coll[i]);
  }
  __syncthreads();
  if (threadIdx.x == 0) *flag = 0;
}

// The whole feature-side step in one block (the feature side is short: a few
// thousand entries): x = F (FP64 in, double-float working copy in xh/xl); CGS2
// against V[:, :ncols]; *nrm = |x|; when write_col >= 0 the column write_col :=
// x/|x| (double-float, FP64 copy in cur) and *bentry = |x|, or on a breakdown
// (|x| < thresh) a random vector orthonormalised against V[:, :ncols] with
// *bentry = *nrm = 0.  write_col < 0 (last step of a cycle) leaves the residual
// in xh/xl.
__device__ void vside_cgs2(float* __restrict__ xh, float* __restrict__ xl, int64_t len,
                           const float* __restrict__ Vh, const float* __restrict__ Vl, int ncols,
                           double* c, float* ch, float* cl) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int pass = 0; pass < 2 && ncols > 0; ++pass) {
    for (int j = w; j < ncols; j += nw) {
      float ah = 0.f, al = 0.f;
      const float* qh = Vh + (int64_t)j * len;
      const float* ql = Vl + (int64_t)j * len;
      for (int64_t i = lane; i < len; i += 32) df_fma(ah, al, qh[i], ql[i], xh[i], xl[i]);
      double v = sv_warp_sum(df_val(ah, al));
      if (lane == 0) c[j] = v;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < ncols; j += blockDim.x) df_split(c[j], ch[j], cl[j]);
    __syncthreads();
    for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
      float sh_ = 0.f, sl_ = 0.f;
      for (int j = 0; j < ncols; ++j) {
        int64_t o = (int64_t)j * len + i;
        df_fma(sh_, sl_, Vh[o], Vl[o], ch[j], cl[j]);
      }
      float h = xh[i], l = xl[i];
      df_sub(h, l, sh_, sl_);
      xh[i] = h;
      xl[i] = l;
    }
    __syncthreads();
  }
}

__device__ double vside_norm(const float* __restrict__ xh, const float* __restrict__ xl, int64_t len,
                             double* sh, double* tot) {
  double acc = 0;
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
    double v = df_val(xh[i], xl[i]);
    acc += v * v;
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) *tot = sqrt(acc);
  __syncthreads();
  return *tot;
}

__global__ void __launch_bounds__(1024) k_vside(const double* __restrict__ F, int64_t len,
                                                float* __restrict__ Vh, float* __restrict__ Vl,
                                                int ncols, int write_col, double* __restrict__ nrm,
                                                const double* __restrict__ ctl,
                                                double* __restrict__ bentry,
                                                double* __restrict__ cur, float* __restrict__ xh,
                                                float* __restrict__ xl, unsigned long long seed,
                                                unsigned step) {
  __shared__ double c[MAX_WORK];
  __shared__ float ch[MAX_WORK], cl[MAX_WORK];
  __shared__ double sh[32];
  __shared__ double tot;
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) df_split(F[i], xh[i], xl[i]);
  __syncthreads();
  vside_cgs2(xh, xl, len, Vh, Vl, ncols, c, ch, cl);
  double s = vside_norm(xh, xl, len, sh, &tot);
  if (write_col < 0) {
    if (threadIdx.x == 0) *nrm = s;
    return;
  }
  bool brk = !(s >= ctl[CTL_THRESH]);
  if (brk) {
    unsigned long long tag = breakdown_tag(ctl, step);
    for (int64_t i = threadIdx.x; i < len; i += blockDim.x) df_split(normal_at(seed, tag, i), xh[i], xl[i]);
    __syncthreads();
    vside_cgs2(xh, xl, len, Vh, Vl, ncols, c, ch, cl);
    double r = vside_norm(xh, xl, len, sh, &tot);
    double inv = 1.0 / r;
    for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
      double v = df_val(xh[i], xl[i]) * inv;
      cur[i] = v;
      df_split(v, Vh[(int64_t)write_col * len + i], Vl[(int64_t)write_col * len + i]);
    }
    if (threadIdx.x == 0) {
      *nrm = 0.0;
      if (bentry) *bentry = 0.0;
    }
  } else {
    double inv = 1.0 / s;
    for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
      double v = df_val(xh[i], xl[i]) * inv;
      cur[i] = v;
      df_split(v, Vh[(int64_t)write_col * len + i], Vl[(int64_t)write_col * len + i]);
    }
    if (threadIdx.x == 0) {
      *nrm = s;
      if (bentry) *bentry = s;
    }
  }
}

// One-sided (Hestenes) Jacobi SVD of B (m x m, row-major), one block, in
// double-float arithmetic: FP64 runs at 1/57 of the FP32 rate on this part (one
// warp-wide FP64 instruction occupies an SM's FP64 pipe for ~17 cycles), and an
// FP64 block spent ~4 ms per 57 x 57 SVD, so the columns of A = B and the
// accumulated rotations J are held as (hi, lo) FP32 pairs in shared memory and
// updated on the FP32 pipe, and the rotation parameters are formed in FP32 and
// normalised in double-float.
// Columns are paired by the circle method (slot 0 fixed, the others rotating),
// one warp per pair; a pair is rotated while |a_p . a_q| > 1e-13 |a_p| |a_q|
// (the double-float dot products carry ~3e-15 relative error, so the FP64
// threshold of 1e-15 would never be met).  Then s_i = |A e_i|, P_i = A e_i / s_i,
// Q = J, sorted by descending s.
// Outputs: P (m x m col-major), s (m), Q (m x m col-major), summary =
// [s (m), P[m-1, :] (m), rf, sweeps].  Closes the cycle in the control block:
// largest Ritz value so far, the next breakdown threshold eps_b * max(smax, 1)
// and the cycle number.
__device__ __forceinline__ void df_warp_sum(float& h, float& l) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float h2 = __shfl_xor_sync(0xffffffffu, h, o);
    float l2 = __shfl_xor_sync(0xffffffffu, l, o);
    float s = h + h2;
    float v = s - h;
    float err = (h - (s - v)) + (h2 - v);
    float lo = err + l + l2;
    h = s + lo;
    l = lo - (h - s);
  }
}

// (x, y) <- (c x - s y, s x + c y) on double-float entries
__device__ __forceinline__ void df_rot(float& xh, float& xl, float& yh, float& yl, float ch, float cl,
                                       float sh, float sl) {
  float ah = 0.f, al = 0.f, bh = 0.f, bl = 0.f;
  df_fma(ah, al, ch, cl, xh, xl);
  df_fma(ah, al, -sh, -sl, yh, yl);
  df_fma(bh, bl, sh, sl, xh, xl);
  df_fma(bh, bl, ch, cl, yh, yl);
  xh = ah + al;
  xl = al - (xh - ah);
  yh = bh + bl;
  yl = bl - (yh - bh);
}

__global__ void __launch_bounds__(1024) k_jacobi_svd(const double* __restrict__ B, int m,
                                                     double* __restrict__ Pout,
                                                     double* __restrict__ sout,
                                                     double* __restrict__ Qout,
                                                     double* __restrict__ summary,
                                                     const double* __restrict__ rf, int max_sweeps,
                                                     int* __restrict__ status,
                                                     double* __restrict__ ctl, double eps_b) {
  extern __shared__ float smf[];
  float* Ah = smf;              // m*m, column c at [c*m]
  float* Al = Ah + m * m;
  float* Jh = Al + m * m;
  float* Jl = Jh + m * m;
  __shared__ int rotated;
  __shared__ int order[MAX_WORK];
  __shared__ double nrm[MAX_WORK];
  int tid = threadIdx.x;
  for (int idx = tid; idx < m * m; idx += blockDim.x) {
    int r = idx % m, c = idx / m;
    df_split(B[r * m + c], Ah[idx], Al[idx]);
    Jh[idx] = r == c ? 1.f : 0.f;
    Jl[idx] = 0.f;
  }
  __syncthreads();
  int mp = (m + 1) & ~1;   // even number of slots (one dummy when m is odd)
  int npairs = mp / 2;
  int lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    if (tid == 0) rotated = 0;
    __syncthreads();
    for (int round = 0; round < mp - 1; ++round) {
      for (int pi = wid; pi < npairs; pi += nw) {
        int a = pi == 0 ? 0 : 1 + (pi - 1 + round) % (mp - 1);
        int b = 1 + (mp - 2 - pi + round) % (mp - 1);
        if (a >= m || b >= m) continue;
        int p = min(a, b), q = max(a, b);
        float* aph = Ah + p * m;
        float* apl = Al + p * m;
        float* aqh = Ah + q * m;
        float* aql = Al + q * m;
        float alh = 0.f, all = 0.f, beh = 0.f, bel = 0.f, gah = 0.f, gal = 0.f;
        for (int r = lane; r < m; r += 32) {
          float xh = aph[r], xl = apl[r], yh = aqh[r], yl = aql[r];
          df_fma(alh, all, xh, xl, xh, xl);
          df_fma(beh, bel, yh, yl, yh, yl);
          df_fma(gah, gal, xh, xl, yh, yl);
        }
        df_warp_sum(alh, all);
        df_warp_sum(beh, bel);
        df_warp_sum(gah, gal);
        // every lane holds the sums; the test and the angle are FP32 (from
        // double-float sums): the angle only steers convergence, while the
        // orthogonality of the applied rotation comes from normalising (c, s)
        // in double-float
        if (fabsf(gah) > 1e-13f * sqrtf(alh) * sqrtf(beh) && gah != 0.f) {
          // be - al in double-float: close singular values still give an
          // accurate angle
          float dh = beh, dl = bel;
          df_sub(dh, dl, alh, all);
          float zeta = dh / (2.f * gah);
          float t = (zeta >= 0.f ? 1.f : -1.f) / (fabsf(zeta) + hypotf(1.f, zeta));
          float c0 = rsqrtf(1.f + t * t);
          float s0 = c0 * t;
          // q = c0^2 + s0^2 = 1 + d exactly in double-float; (c, s) = (c0, s0) q^(-1/2)
          // with q^(-1/2) = 1 - d/2 (+ O(d^2), d ~ 1e-7)
          float qh = 0.f, ql = 0.f;
          df_fma(qh, ql, c0, 0.f, c0, 0.f);
          df_fma(qh, ql, s0, 0.f, s0, 0.f);
          float d = (qh - 1.f) + ql;
          float fh = 1.f, fl = -0.5f * d;
          float ch = 0.f, cl = 0.f, sh = 0.f, sl = 0.f;
          df_fma(ch, cl, c0, 0.f, fh, fl);
          df_fma(sh, sl, s0, 0.f, fh, fl);
          for (int r = lane; r < m; r += 32) {
            df_rot(aph[r], apl[r], aqh[r], aql[r], ch, cl, sh, sl);
            df_rot(Jh[p * m + r], Jl[p * m + r], Jh[q * m + r], Jl[q * m + r], ch, cl, sh, sl);
          }
          if (lane == 0) rotated = 1;
        }
      }
      __syncthreads();
    }
    if (!rotated) break;
    __syncthreads();
  }
  if (sweep >= max_sweeps && tid == 0) atomicOr(status, SV_STATUS_LIMIT);
  // singular values and ordering
  for (int c = wid; c < m; c += nw) {
    float sh = 0.f, sl = 0.f;
    for (int r = lane; r < m; r += 32) {
      float xh = Ah[c * m + r], xl = Al[c * m + r];
      df_fma(sh, sl, xh, xl, xh, xl);
    }
    df_warp_sum(sh, sl);
    if (lane == 0) nrm[c] = sqrt(df_val(sh, sl));
  }
  __syncthreads();
  if (tid == 0) {
    // stable insertion sort, descending
    for (int i = 0; i < m; ++i) order[i] = i;
    for (int i = 1; i < m; ++i) {
      int v = order[i];
      int t = i - 1;
      while (t >= 0 && nrm[order[t]] < nrm[v]) {
        order[t + 1] = order[t];
        --t;
      }
      order[t + 1] = v;
    }
  }
  __syncthreads();
  for (int idx = tid; idx < m * m; idx += blockDim.x) {
    int r = idx % m, i = idx / m;
    int c = order[i];
    double s = nrm[c];
    double a = df_val(Ah[c * m + r], Al[c * m + r]);
    Pout[i * m + r] = s > 0 ? a / s : (r == i ? 1.0 : 0.0);
    Qout[i * m + r] = df_val(Jh[c * m + r], Jl[c * m + r]);
  }
  for (int i = tid; i < m; i += blockDim.x) {
    double s = nrm[order[i]];
    sout[i] = s;
    summary[i] = s;
    summary[m + i] = s > 0 ? df_val(Ah[order[i] * m + (m - 1)], Al[order[i] * m + (m - 1)]) / s : 0.0;
  }
  if (tid == 0) {
    summary[2 * m] = rf ? *rf : 0.0;
    summary[2 * m + 1] = (double)sweep;
    double smax = fmax(ctl[CTL_SMAX], nrm[order[0]]);
    ctl[CTL_SMAX] = smax;
    ctl[CTL_THRESH] = eps_b * fmax(smax, 1.0);
    ctl[CTL_CYCLE] += 1.0;
  }
}

// Out[:, c] = sum_r In[:, r] * M[r + c*nin] for c < nout (tall x small), In
// double-float; Out double-float (outh/outl) or FP64 (outd).  KB output columns
// per pass; EXACT when KB divides nout (no column guards).  M sits in shared
// memory as (hi, lo) pairs read with one broadcast 8-byte load per term.
template <int KB, bool EXACT>
__global__ void __launch_bounds__(256) k_rotate_df(const float* __restrict__ Inh,
                                                   const float* __restrict__ Inl, int64_t ld_in,
                                                   int64_t len, int nin, const double* __restrict__ M,
                                                   int nout, float* __restrict__ outh,
                                                   float* __restrict__ outl, double* __restrict__ outd,
                                                   int64_t ld_out) {
  extern __shared__ float2 Ms[];   // nin*nout pairs (hi, lo)
  for (int i = threadIdx.x; i < nin * nout; i += blockDim.x) df_split(M[i], Ms[i].x, Ms[i].y);
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x) {
    for (int c0 = 0; c0 < nout; c0 += KB) {
      float ah[KB], al[KB];
#pragma unroll
      for (int t = 0; t < KB; ++t) ah[t] = al[t] = 0.f;
      for (int r = 0; r < nin; ++r) {
        int64_t o = (int64_t)r * ld_in + i;
        float wh = Inh[o], wl = Inl[o];
#pragma unroll
        for (int t = 0; t < KB; ++t)
          if (EXACT || c0 + t < nout) {
            float2 m = Ms[r + (c0 + t) * nin];
            df_fma(ah[t], al[t], wh, wl, m.x, m.y);
          }
      }
#pragma unroll
      for (int t = 0; t < KB; ++t)
        if (EXACT || c0 + t < nout) {
          int64_t o = (int64_t)(c0 + t) * ld_out + i;
          if (outd) {
            outd[o] = df_val(ah[t], al[t]);
          } else {
            // renormalise the pair
            float h = ah[t] + al[t];
            outh[o] = h;
            outl[o] = al[t] - (h - ah[t]);
          }
        }
    }
  }
}

// V[:, k] = F / rf (double-float column + FP64 current vector) and B reset.
__global__ void k_restart_tail(float* __restrict__ vkh, float* __restrict__ vkl,
                               double* __restrict__ vcur, const double* __restrict__ F, int64_t n,
                               const double* __restrict__ summary, int m, int k,
                               double* __restrict__ B) {
  double rf = summary[2 * m];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = F[i] / rf;
    vcur[i] = v;
    df_split(v, vkh[i], vkl[i]);
  }
  if (blockIdx.x == 0) {
    for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
      int r = idx / m, c = idx % m;
      double v = 0;
      if (r < k && c == r) v = summary[r];
      if (r < k && c == k) v = rf * summary[m + r];
      B[idx] = v;
    }
  }
}

__global__ void k_df_to_fp64(const float* __restrict__ h, const float* __restrict__ l, int64_t len,
                             double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = df_val(h[i], l[i]);
}

__global__ void k_axpy_sub(double* __restrict__ y, const double* __restrict__ z,
                           const double* __restrict__ cs, int64_t len) {
  double c = *cs;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] -= c * z[i];
}

__global__ void k_scale_cols(double* __restrict__ X, int64_t len, int ncols,
                             const double* __restrict__ s) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < len * ncols;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int c = (int)(idx / len);
    X[idx] *= s[c];
  }
}

// ---------------------------------------------------------------------------
// operator abstraction: the implicit matrix on the device, or host callbacks
// ---------------------------------------------------------------------------
struct Op {
  virtual ~Op() {}
  // y = A x - (csub ? *csub : 0) * z        (x in R^n, y in R^m)
  virtual void N(const double* x, double* y, const double* csub, const double* z) = 0;
  // y = A^T x - (csub ? *csub : 0) * z      (x in R^m, y in R^n)
  virtual void T(const double* x, double* y, const double* csub, const double* z) = 0;
  // true when N and T only enqueue device work (no host round trip), so that a
  // Lanczos cycle over them can be captured as a CUDA graph
  virtual bool device_only() const { return false; }
  // y = A x - (csub ? *csub : 0) * z with x, z, y double-float vectors (hi, lo);
  // false when the operator has no such form (the FP64 N is used instead)
  virtual bool N_df(const float* xh, const float* xl, float* yh, float* yl, const double* csub,
                    const float* zh, const float* zl) {
    return false;
  }
};

struct CenteredOp : Op {
  sv_context* ctx;
  const sv_centered* S;
  CenteredOp(sv_context* c, const sv_centered* s) : ctx(c), S(s) {}
  void N(const double* x, double* y, const double* csub, const double* z) override {
    sv_centered_apply(ctx, S, 'N', x, y, 1.0, 0.0, csub, z);
  }
  void T(const double* x, double* y, const double* csub, const double* z) override {
    sv_centered_apply(ctx, S, 'T', x, y, 1.0, 0.0, csub, z);
  }
  bool device_only() const override { return true; }
  bool N_df(const float* xh, const float* xl, float* yh, float* yl, const double* csub,
            const float* zh, const float* zl) override {
    return sv_centered_apply_df(ctx, S, xh, xl, yh, yl, csub, zh, zl);
  }
};

struct CallbackOp : Op {
  sv_context* ctx;
  int64_t m, n;
  sv_matmul_fn mm;
  void* data;
  std::vector<double> hx, hy, tmp;
  CallbackOp(sv_context* c, int64_t m_, int64_t n_, sv_matmul_fn f, void* d)
      : ctx(c), m(m_), n(n_), mm(f), data(d), hx(std::max(m_, n_)), hy(std::max(m_, n_)),
        tmp(std::max(m_, n_)) {}
  void run(char trans, const double* x, int64_t lx, double* y, int64_t ly, const double* csub,
           const double* z) {
    sv_d2h(ctx, hx.data(), x, lx * 8);
    mm(hy.data(), trans, hx.data(), tmp.data(), data);
    sv_h2d(ctx, y, hy.data(), ly * 8);
    if (csub)
      sv_launch(ctx, "irlba_axpy", k_axpy_sub, dim3(sv_grid_for(ctx, ly, 256, 4)), dim3(256), 0, y, z,
                csub, ly);
  }
  void N(const double* x, double* y, const double* csub, const double* z) override {
    run('N', x, n, y, m, csub, z);
  }
  void T(const double* x, double* y, const double* csub, const double* z) override {
    run('T', x, m, y, n, csub, z);
  }
};

struct IrlbaResult {
  int info = 1;
  int64_t iters = 0, nmatvec = 0;
};

// One side of the bidiagonalisation: two double-float bases (len x work) --
// the current one and the target of the thick-restart rotation, which swap
// roles every restart -- the double-float working vector and the FP64 copy of
// the current basis vector (the input of the next product).
struct Side {
  int64_t len = 0;
  DevBuf<float> h[2], l[2];     // basis sets
  int set = 0;                  // the current set
  DevBuf<float> xh, xl;         // working vector
  DevBuf<double> cur;           // current basis vector, FP64
  void alloc(int64_t n, int work) {
    len = n;
    for (int t = 0; t < 2; ++t) {
      h[t].alloc(n * work);
      l[t].alloc(n * work);
    }
    xh.alloc(n);
    xl.alloc(n);
    cur.alloc(n);
  }
  float* bh() { return h[set].get(); }
  float* bl() { return l[set].get(); }
  float* ch(int j) { return bh() + (int64_t)j * len; }
  float* cl(int j) { return bl() + (int64_t)j * len; }
  float* th() { return h[1 - set].get(); }
  float* tl() { return l[1 - set].get(); }
  void flip() { set = 1 - set; }
};

// A captured Lanczos cycle: its executable graph and what one replay does.
struct CycleGraph {
  cudaGraphExec_t exec = nullptr;
  int64_t launches = 0, matvecs = 0;
};

// Control-block slots in Lanczos::scal (after the two norm slots).
#define SCAL_S 0        // W-side norm (alpha of the bidiagonal)
#define SCAL_R 1        // V-side norm (beta)
#define SCAL_CTL 2      // control block of the cycles (3 slots)
#define SCAL_CTL0 5     // control block of the start vector: threshold 1e-300

// The Lanczos driver.  m = rows of A (the W side), n = columns (the V side).
struct Lanczos {
  sv_context* ctx;
  Op* op;
  int64_t m, n;
  int nu, work;
  Side Ws, Vs;
  DevBuf<double> ytmp, F, B, P, Q, sig, summary, scal, part, cvec, Ufin, Vfin;
  DevBuf<unsigned int> counter;
  DevBuf<int> flag;
  double* hsum = nullptr;       // pinned copy of the cycle summary
  double eps_b = 0;
  int cgs_blocks = RED_BLOCKS;  // resident blocks of the CGS kernels (one wave)
  // graphs of the first cycle and of restart cycles from basis set 0 / set 1
  CycleGraph graphs[3];

  Lanczos(sv_context* c, Op* o, int64_t m_, int64_t n_, int nu_, int work_)
      : ctx(c), op(o), m(m_), n(n_), nu(nu_), work(work_) {
    Ws.alloc(m, work);
    Vs.alloc(n, work);
    ytmp.alloc(std::max(m, n));
    F.alloc(n);
    B.alloc(work * work);
    P.alloc(work * work);
    Q.alloc(work * work);
    sig.alloc(work);
    summary.alloc(2 * work + 2);
    scal.alloc(8);
    part.alloc((size_t)RED_BLOCKS * (work + 1));
    cvec.alloc(2 * MAX_WORK);
    counter.alloc(4);
    flag.alloc(4);
    sv_memset(ctx, counter.get(), 0, 16);
    sv_memset(ctx, flag.get(), 0, 16);
    sv_memset(ctx, B.get(), 0, work * work * 8);
    SV_CUDA(cudaMallocHost((void**)&hsum, (2 * work + 2) * 8));
    int per_sm = 0;
    if (work <= 64)
      SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cgs_df<8, true, true, false>, 256, 0));
    else
      SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cgs_df<12, true, true, false>, 256, 0));
    cgs_blocks = std::max(1, std::min(RED_BLOCKS, per_sm * ctx->num_sms));
    SV_CUDA(cudaFuncSetAttribute(k_jacobi_svd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 4 * MAX_WORK * MAX_WORK * 4));
    SV_CUDA(cudaFuncSetAttribute(k_rotate_df<10, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 MAX_WORK * MAX_WORK * 8));
    SV_CUDA(cudaFuncSetAttribute(k_rotate_df<8, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 MAX_WORK * MAX_WORK * 8));
    SV_CUDA(cudaFuncSetAttribute(k_rotate_df<16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 MAX_WORK * MAX_WORK * 8));
  }
  ~Lanczos() {
    for (auto& g : graphs)
      if (g.exec) cudaGraphExecDestroy(g.exec);
    if (hsum) cudaFreeHost(hsum);
  }
  Lanczos(const Lanczos&) = delete;
  Lanczos& operator=(const Lanczos&) = delete;

  double* ctl() { return scal.get() + SCAL_CTL; }

  // working vector <- CGS2(y, basis[:, :ncols]) (y FP64; null: the working
  // vector already holds it); *nrm = its norm
  template <int NJ>
  void orth_norm_nj(Side& s, const double* y, int ncols, double* nrm) {
    int g = (int)std::max<int64_t>(1, std::min<int64_t>(cgs_blocks, (s.len + 63) / 64));
    double* c1 = cvec.get();
    double* c2 = cvec.get() + MAX_WORK;
    double* np = part.get() + (size_t)RED_BLOCKS * work;
    if (ncols == 0) {
      if (y) to_working(s, y);
      sv_launch(ctx, "irlba_upd_norm", k_cgs_df<NJ, true, false, true>, dim3(g), dim3(256), 0,
                (const float*)s.bh(), (const float*)s.bl(), s.len, 0, s.xh.get(), s.xl.get(),
                (const double*)nullptr, s.len, (const double*)c1, part.get(), np, c2, nrm, counter.get());
      return;
    }
    sv_launch(ctx, "irlba_dots", k_cgs_df<NJ, false, true, false>, dim3(g), dim3(256), 0,
              (const float*)s.bh(), (const float*)s.bl(), s.len, ncols, s.xh.get(), s.xl.get(), y, s.len,
              (const double*)nullptr, part.get(), np, c1, (double*)nullptr, counter.get());
    sv_launch(ctx, "irlba_upd_dots", k_cgs_df<NJ, true, true, false>, dim3(g), dim3(256), 0,
              (const float*)s.bh(), (const float*)s.bl(), s.len, ncols, s.xh.get(), s.xl.get(),
              (const double*)nullptr, s.len, (const double*)c1, part.get(), np, c2, (double*)nullptr,
              counter.get());
    sv_launch(ctx, "irlba_upd_norm", k_cgs_df<NJ, true, false, true>, dim3(g), dim3(256), 0,
              (const float*)s.bh(), (const float*)s.bl(), s.len, ncols, s.xh.get(), s.xl.get(),
              (const double*)nullptr, s.len, (const double*)c2, part.get(), np, c1, nrm, counter.get());
  }
  void orth_norm(Side& s, const double* y, int ncols, double* nrm) {
    if (work <= 64) orth_norm_nj<8>(s, y, ncols, nrm);
    else orth_norm_nj<12>(s, y, ncols, nrm);
  }

  // basis column j := working vector / *nrm (FP64 copy in cur), breakdown handling
  void scal_fix(Side& s, int j, double* nrm, const double* c, double* bentry, uint64_t seed,
                unsigned step) {
    sv_launch(ctx, "irlba_scal", k_scal_df, dim3(sv_grid_for(ctx, s.len, 256, 4)), dim3(256), 0,
              (const float*)s.xh.get(), (const float*)s.xl.get(), s.len, (const double*)nrm, c,
              s.ch(j), s.cl(j), s.cur.get(), bentry, flag.get(), (unsigned long long)seed, step);
    sv_launch(ctx, "irlba_scal_post", k_scal_post, dim3(1), dim3(1), 0, nrm, (const int*)flag.get());
    sv_launch(ctx, "irlba_fix", k_fix_df, dim3(1), dim3(1024), 0, s.cur.get(), s.len,
              (const float*)s.bh(), (const float*)s.bl(), s.len, j, s.ch(j), s.cl(j), flag.get());
  }

  // the feature-side step in one launch (see k_vside)
  void vside(int ncols, int write_col, double* nrm, const double* c, double* bentry, uint64_t seed,
             unsigned step) {
    if (n > 32768) {   // long feature side: the multi-block kernels
      orth_norm(Vs, F.get(), ncols, nrm);
      if (write_col >= 0) scal_fix(Vs, write_col, nrm, c, bentry, seed, step);
      return;
    }
    sv_launch(ctx, "irlba_vside", k_vside, dim3(1), dim3(1024), 0, (const double*)F.get(), n, Vs.bh(),
              Vs.bl(), ncols, write_col, nrm, c, bentry, Vs.cur.get(), Vs.xh.get(), Vs.xl.get(),
              (unsigned long long)seed, step);
  }

  void to_working(Side& s, const double* y) {
    sv_launch(ctx, "irlba_to_df", k_to_df, dim3(sv_grid_for(ctx, s.len, 256, 4)), dim3(256), 0, y,
              s.len, s.xh.get(), s.xl.get());
  }

  // out = basis * M[:, :nout]: into the other basis set (outd null) or FP64 outd
  void rotate(Side& s, const double* M, int nout, double* outd) {
    auto kern = nout % 10 == 0 ? k_rotate_df<10, true> : nout % 8 == 0 ? k_rotate_df<8, true>
                                                                       : k_rotate_df<16, false>;
    sv_launch(ctx, "irlba_rotate", kern, dim3(sv_grid_for(ctx, s.len, 256, 8)), dim3(256),
              (size_t)work * nout * 8, (const float*)s.bh(), (const float*)s.bl(), s.len, s.len,
              work, M, nout, outd ? (float*)nullptr : s.th(), outd ? (float*)nullptr : s.tl(), outd,
              s.len);
  }

  // One cycle, enqueued on the context stream without any host round trip:
  // for a restart, V <- V Q_k, W <- W P_k, V[:, k] = f/|f| and B reset; the
  // Lanczos steps k..work-1; the SVD of B; its summary copied to hsum.
  // Returns the number of operator products.
  int64_t cycle(bool restart, int k, uint64_t seed) {
    double* s0 = scal.get() + SCAL_S;
    double* s1 = scal.get() + SCAL_R;
    const double* c = ctl();
    int64_t nmv = 0;
    if (restart) {
      rotate(Vs, Q.get(), k, nullptr);
      rotate(Ws, P.get(), k, nullptr);
      Vs.flip();
      Ws.flip();
      df_residual_to_fp64();
      sv_launch(ctx, "irlba_restart", k_restart_tail, dim3(sv_grid_for(ctx, n, 256, 4)), dim3(256), 0,
                Vs.ch(k), Vs.cl(k), Vs.cur.get(), (const double*)F.get(), n,
                (const double*)summary.get(), work, k, B.get());
    }
    unsigned step = 1;
    int j = k;
    // W[:, j] = A V[:, j]; CGS2 against W[:, :j]
    if (op->N_df(Vs.ch(j), Vs.cl(j), Ws.xh.get(), Ws.xl.get(), nullptr, nullptr, nullptr)) {
      orth_norm(Ws, nullptr, j, s0);
    } else {
      op->N(Vs.cur.get(), ytmp.get(), nullptr, nullptr);
      orth_norm(Ws, ytmp.get(), j, s0);
    }
    nmv++;
    scal_fix(Ws, j, s0, c, B.get() + (int64_t)j * work + j, seed, step++);
    while (true) {
      // F = A^T W[:, j] - S V[:, j]; CGS2 against V[:, :j+1]
      op->T(Ws.cur.get(), F.get(), s0, Vs.cur.get());
      nmv++;
      if (j + 1 < work) {
        vside(j + 1, j + 1, s1, c, B.get() + (int64_t)j * work + j + 1, seed, step++);
        // W[:, j+1] = A V[:, j+1] - R W[:, j]
        if (op->N_df(Vs.ch(j + 1), Vs.cl(j + 1), Ws.xh.get(), Ws.xl.get(), s1, Ws.ch(j), Ws.cl(j))) {
          orth_norm(Ws, nullptr, j + 1, s0);
        } else {
          op->N(Vs.cur.get(), ytmp.get(), s1, Ws.cur.get());
          orth_norm(Ws, ytmp.get(), j + 1, s0);
        }
        nmv++;
        scal_fix(Ws, j + 1, s0, c, B.get() + (int64_t)(j + 1) * work + j + 1, seed, step++);
        ++j;
      } else {
        vside(j + 1, -1, s1, c, nullptr, seed, step++);   // residual f and |f|
        break;
      }
    }
    sv_launch(ctx, "irlba_svd", k_jacobi_svd, dim3(1), dim3(1024), (size_t)4 * work * work * 4,
              (const double*)B.get(), work, P.get(), sig.get(), Q.get(), summary.get(),
              (const double*)s1, 60, ctx->d_status, ctl(), eps_b);
    SV_CUDA(cudaMemcpyAsync(hsum, summary.get(), (2 * work + 2) * 8, cudaMemcpyDeviceToHost, ctx->stream));
    return nmv;
  }

  // Enqueue one cycle: replay its graph (captured on first use), or launch it
  // directly when the operator calls back to the host or launches are profiled
  // one by one.
  int64_t enqueue_cycle(bool restart, int k, uint64_t seed, bool graphs_on) {
    if (!graphs_on) return cycle(restart, k, seed);
    CycleGraph& g = graphs[restart ? 1 + Vs.set : 0];
    if (!g.exec) {
      // capturing runs the host side of the cycle (basis sets flip) but
      // launches nothing: the launch count is charged per replay instead
      int64_t l0 = ctx->launches;
      cudaGraph_t graph = nullptr;
      SV_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      try {
        g.matvecs = cycle(restart, k, seed);
      } catch (...) {
        cudaStreamEndCapture(ctx->stream, &graph);
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        ctx->launches = l0;
        throw;
      }
      SV_CUDA(cudaStreamEndCapture(ctx->stream, &graph));
      g.launches = ctx->launches - l0;
      ctx->launches = l0;
      cudaError_t e = cudaGraphInstantiate(&g.exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) {
        g.exec = nullptr;
        SV_CUDA(e);
      }
    } else if (restart) {
      Vs.flip();
      Ws.flip();
    }
    SV_CUDA(cudaGraphLaunch(g.exec, ctx->stream));
    ctx->launches += g.launches;
    return g.matvecs;
  }

  IrlbaResult run(const double* init_host, int maxit, double tol, uint64_t seed) {
    IrlbaResult res;
    eps_b = sqrt(2.220446049250313e-16);
    // control blocks: cycles start at threshold eps_b (smax = 0), the start
    // vector is normalised unless it is zero
    double ctl_init[6] = {eps_b, 0.0, 0.0, 1e-300, 0.0, 0.0};
    sv_h2d(ctx, scal.get() + SCAL_CTL, ctl_init, sizeof(ctl_init));
    sv_h2d(ctx, F.get(), init_host, n * 8);
    vside(0, 0, scal.get() + SCAL_R, scal.get() + SCAL_CTL0, nullptr, seed, 0);
    bool graphs_on = op->device_only() && !ctx->profiling && !getenv("SV_NO_GRAPH");
    const int kr = std::min(nu, work - 1);
    double smax = 0;
    int it = 0;
    for (; it < maxit; ++it) {
      res.nmatvec += enqueue_cycle(it > 0, it > 0 ? kr : 0, seed, graphs_on);
      sv_sync(ctx);
      double rf = hsum[2 * work];
      smax = std::max(smax, hsum[0]);
      int nconv = 0;
      for (int i = 0; i < nu; ++i)
        if (fabs(rf * hsum[work + i]) < tol * smax) ++nconv;
      res.iters = it + 1;
      if (nconv >= nu || rf < eps_b * smax) {
        res.info = 0;
        break;
      }
    }
    if (it >= maxit) res.iters = maxit;
    sv_check_device_status(ctx, "irlba");
    return res;
  }

  // F holds the residual in FP64 only before the first CGS pass; the orthogonalised
  // residual lives in the V-side working vector: bring it back to FP64
  void df_residual_to_fp64() {
    sv_launch(ctx, "irlba_f_fp64", k_df_to_fp64, dim3(sv_grid_for(ctx, n, 256, 4)), dim3(256), 0,
              (const float*)Vs.xh.get(), (const float*)Vs.xl.get(), n, F.get());
  }

  // U = W P[:, :nu], V = V Q[:, :nu] (FP64)
  void finish() {
    Ufin.alloc(m * nu);
    Vfin.alloc(n * nu);
    rotate(Ws, P.get(), nu, Ufin.get());
    rotate(Vs, Q.get(), nu, Vfin.get());
  }
};

int default_work(int64_t m, int64_t n, int64_t nu) {
  // src/irlba.jl:50-58
  int64_t mb = nu + 7;
  if (mb < nu) mb = nu + 1;
  if (mb > std::min(m, n)) mb = std::min(m, n);
  return (int)mb;
}

}  // namespace

static int irlba_core(sv_context* ctx, Op* op, int64_t m, int64_t n, int64_t nu, int64_t work,
                      int64_t maxit, double tol, const double* init, uint64_t seed, double* s_out,
                      double* U, double* V, int64_t* iters, int64_t* nmatvec, sv_embed* emb) {
  SV_REQUIRE(nu >= 1 && nu <= std::min(m, n), "nu must be in 1..min(m, n)");
  if (work <= 0) work = default_work(m, n, nu);
  SV_REQUIRE(work > nu || work == std::min(m, n), "work must exceed nu (or equal min(m, n))");
  SV_REQUIRE(work <= std::min(m, n), "work exceeds min(m, n)");
  if (work > MAX_WORK) sv_throw(SV_ERR_UNSUPPORTED, "work %lld exceeds %d", (long long)work, MAX_WORK);
  SV_REQUIRE(maxit >= 1, "maxit must be >= 1");
  SV_REQUIRE(init != nullptr, "init (length n) is required");
  Lanczos L(ctx, op, m, n, (int)nu, (int)work);
  IrlbaResult r = L.run(init, (int)maxit, tol, seed);
  L.finish();
  if (s_out) sv_d2h(ctx, s_out, L.sig.get(), nu * 8);
  if (U) sv_d2h(ctx, U, L.Ufin.get(), m * nu * 8);
  if (V) sv_d2h(ctx, V, L.Vfin.get(), n * nu * 8);
  if (emb) {
    emb->s.alloc(nu);
    SV_CUDA(cudaMemcpyAsync(emb->s.get(), L.sig.get(), nu * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    emb->Z = std::move(L.Ufin);
    sv_launch(ctx, "pca_scale", k_scale_cols, dim3(sv_grid_for(ctx, m * nu, 256, 8)), dim3(256), 0,
              emb->Z.get(), m, (int)nu, (const double*)emb->s.get());
    sv_sync(ctx);
  }
  if (iters) *iters = r.iters;
  if (nmatvec) *nmatvec = r.nmatvec;
  return r.info;
}

SV_API int sv_irlba(sv_context* ctx, const sv_centered* s, int64_t nu, int64_t work, int64_t maxit,
                    double tol, const double* init, uint64_t seed, double* s_out, double* U,
                    double* V, int64_t* iters, int64_t* nmatvec) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(s && s->ctx == ctx, "bad centered handle");
  CenteredOp op(ctx, s);
  int info = irlba_core(ctx, &op, s->n_cells, s->nf, nu, work, maxit, tol, init, seed, s_out, U, V,
                        iters, nmatvec, nullptr);
  if (info != 0) {
    sv_set_error("convergence failed");   // src/irlba.jl:73
    return SV_ERR_NOCONV;
  }
  SV_CATCH
}

SV_API int sv_pca(sv_context* ctx, const sv_centered* s, int64_t npcs, int64_t maxit, double tol,
                  const double* init, uint64_t seed, sv_embed** out, double* Z, double* stdev,
                  double* loadings, int64_t* iters, int64_t* nmatvec) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(s && s->ctx == ctx, "bad centered handle");
  SV_REQUIRE(npcs >= 1, "npcs must be >= 1");
  int64_t k = std::min(std::min(s->n_cells, s->nf), npcs);   // embedding.jl:48
  if (k > 0.5 * std::min(s->n_cells, s->nf))
    sv_throw(SV_ERR_UNSUPPORTED,
             "npcs > 0.5 min(m, n): the reference switches to a dense svd (embedding.jl:50-53)");
  CenteredOp op(ctx, s);
  auto* e = new sv_embed();
  try {
    e->ctx = ctx;
    e->n_cells = s->n_cells;
    e->npcs = k;
    e->nf = s->nf;
    std::vector<double> sv(k);
    int info = irlba_core(ctx, &op, s->n_cells, s->nf, k, 0, maxit, tol, init, seed, sv.data(),
                          nullptr, loadings, iters, nmatvec, e);
    if (info != 0) {
      delete e;
      sv_set_error("convergence failed");
      return SV_ERR_NOCONV;
    }
    if (Z) sv_d2h(ctx, Z, e->Z.get(), s->n_cells * k * 8);
    if (stdev)
      for (int64_t i = 0; i < k; ++i)
        stdev[i] = sv[i] / sqrt((double)std::max<int64_t>(1, s->n_cells - 1));   // embedding.jl:68
  } catch (...) {
    delete e;
    throw;
  }
  if (out) *out = e;
  else delete e;
  SV_CATCH
}

SV_API int sv_embed_info(const sv_embed* e, int64_t* n_cells, int64_t* npcs) {
  SV_TRY
  SV_REQUIRE(e, "null handle");
  if (n_cells) *n_cells = e->n_cells;
  if (npcs) *npcs = e->npcs;
  SV_CATCH
}

SV_API int sv_embed_free(sv_embed* e) {
  if (e) {
    if (e->ctx) cudaSetDevice(e->ctx->device);
    delete e;
  }
  return SV_OK;
}

// ---- drop-in for the native `irlba` symbol --------------------------------------
static sv_context* g_default_ctx = nullptr;
static std::mutex g_default_mu;

sv_context* sv_default_context() {
  std::lock_guard<std::mutex> lk(g_default_mu);
  if (!g_default_ctx) {
    sv_context* c = nullptr;
    int st = sv_context_create(0, &c);
    if (st != SV_OK) sv_throw(st, "could not create the default context");
    g_default_ctx = c;
  }
  return g_default_ctx;
}

SV_API int irlba(int64_t m, int64_t n, int64_t nu, int64_t work, int64_t maxit, int64_t restart,
                 double tol, double* init, double* s, double* U, double* V, sv_randv_fn randv,
                 sv_matmul_fn matmul, void* data) {
  (void)restart;
  (void)randv;
  SV_TRY
  SV_REQUIRE(matmul != nullptr, "matmul callback is required");
  SV_REQUIRE(m >= 1 && n >= 1, "bad sizes");
  sv_context* ctx = sv_default_context();
  sv_ctx_check(ctx);
  CallbackOp op(ctx, m, n, matmul, data);
  int info = irlba_core(ctx, &op, m, n, nu, work, maxit, tol, init, 0x5EEDull, s, U, V, nullptr,
                        nullptr, nullptr);
  return info == 0 ? 0 : 1;
  SV_CATCH
}
