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
// Gram-Schmidt applied twice (CGS2).  On the cell side (the long one) both
// projections share one pass over the basis per step: the first projection's
// coefficients Q^T (A v) = G^T v come from G = A^T W, kept on the feature side
// from the feature-side products (and rotated with W at a restart); the second
// projection of a step's vector is applied, in place, during the next step's
// pass, which reads the basis anyway, and the products that used the vector in
// between are corrected through G (see k_cgs_lag).  The vector each step adds
// is the CGS2 vector; the pass count drops from three to one.  The feature side
// (a few thousand rows) runs CGS2 directly.  After `work` steps B (work x work, upper
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
#include <string.h>

void sv_centered_apply(sv_context* ctx, const sv_centered* S, char trans, const double* x, double* y,
                       double alpha, double beta, const double* csub, const double* z);
bool sv_centered_apply_df(sv_context* ctx, const sv_centered* S, const float* xh, const float* xl,
                          float* yh, float* yl, const double* csub, const float* zh, const float* zl);
void sv_batch_apply_N_df(sv_context* ctx, const sv_batch* b, const float* xh, const float* xl,
                         float* yh, float* yl, const double* csub, const float* zh, const float* zl,
                         const int* active);
void sv_batch_apply_T(sv_context* ctx, const sv_batch* b, const double* u, double* y,
                      const double* csub, const double* z, const int* active);

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

// Rows of a stacked side: the bases of several independent problems (samples)
// are stacked by rows, sample s owning rows [off[s], off[s+1]); a block schedule
// (BlkRange) covers them, the blocks of sample s being seg_blk[s] ..
// seg_blk[s+1]-1.  One sample is the usual case; the kernels below take the
// schedule in either case.

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
// Per-block FP64 partials; the last block reduces them per sample in block
// order (deterministic); cin / cout hold MAX_WORK coefficients per sample, nrm
// one norm per sample; blocks of inactive samples skip the rows.  NJ = columns per warp: 8 for bases of up to 64 columns,
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
                                                const double* __restrict__ y,
                                                const BlkRange* __restrict__ blk,
                                                const int* __restrict__ seg_blk, int nseg,
                                                const int* __restrict__ active,
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
  const BlkRange br = blk[blockIdx.x];
  const int sg = br.seg;
  if (UPDATE)
    for (int j = tid; j < ncols; j += blockDim.x) df_split(cin[sg * MAX_WORK + j], csh[j], csl[j]);
  __syncthreads();
  int64_t r0 = br.r0, r1 = (active == nullptr || active[sg]) ? br.r1 : br.r0;
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
      // one warp per (sample, column), lanes over the sample's blocks (block
      // order fixed: deterministic)
      for (int pq = w; pq < nseg * ncols; pq += 8) {
        int s2 = pq / ncols, j = pq - s2 * ncols;
        double s = 0;
        for (int b = seg_blk[s2] + lane; b < seg_blk[s2 + 1]; b += 32) s += part[(int64_t)b * ncols + j];
        s = sv_warp_sum(s);
        if (lane == 0) cout[s2 * MAX_WORK + j] = s;
      }
    }
    if (NORM) {
      for (int s2 = tid; s2 < nseg; s2 += blockDim.x) {
        double s = 0;
        for (int b = seg_blk[s2]; b < seg_blk[s2 + 1]; ++b) s += npart[b];
        nrm[s2] = sqrt(s);
      }
    }
    if (tid == 0) *counter = 0;
  }
}

// ---- packed double-float arithmetic -----------------------------------------
// Two independent FP32 lanes per instruction (the f32x2 forms of sm_100 and
// later): each lane is the IEEE FP32 operation of its scalar counterpart, so a
// packed sequence gives bit for bit what the same scalar sequence gives for each
// of the two values, in half the issue slots.
typedef unsigned long long f2_t;
__device__ __forceinline__ f2_t f2_pack(float a, float b) {
  f2_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void f2_unpack(f2_t r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f2_t f2_add(f2_t a, f2_t b) {
  f2_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2_t f2_sub(f2_t a, f2_t b) {
  f2_t d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b) {
  f2_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c) {
  f2_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// df_fma on two accumulator pairs at once with one shared multiplicand a:
// ah, nah = -ah and al broadcast to both lanes.  The product is formed negated
// (pn = -ah*bh, exact negation of the rounded product), which turns df_fma's
// sh + p and p - v into subtractions without a negation instruction.
__device__ __forceinline__ void df_fma2(f2_t& sh, f2_t& sl, f2_t ah, f2_t nah, f2_t al, f2_t bh,
                                        f2_t bl) {
  f2_t pn = f2_mul(nah, bh);
  f2_t e = f2_fma(ah, bh, pn);   // ah*bh - p, exact
  e = f2_fma(ah, bl, e);
  e = f2_fma(al, bh, e);
  f2_t t = f2_sub(sh, pn);       // sh + p
  f2_t v = f2_sub(t, sh);
  f2_t err = f2_sub(sh, f2_sub(t, v));
  err = f2_sub(err, f2_add(pn, v));   // + (p - v)
  sh = t;
  sl = f2_add(sl, f2_add(err, e));
}

// The cell-side step of the lagged CGS2 in one pass over the basis Q (double-
// float, columns 0..ncols-1).  The second projection of a step's new vector is
// carried to the next step's pass, which reads the basis anyway:
//   * column pend (pend >= 0) holds w' = w + Q[:, :pend] cp, the previous
//     step's vector before its second projection; it is corrected in place,
//     w = w' - Q[:, :pend] cp, and used corrected below;
//   * x = y - Q c0, with the first projection's coefficients c0 formed on the
//     feature side (c0 = G^T v - beta (cp, 1), G = A^T Q; k_gdots) instead of a
//     pass over Q;
//   * c1 = Q^T x (the second projection) and |x|^2.
// The last block forms per sample nrm = sqrt(|x|^2 - |c1|^2) -- the norm of
// x - Q c1, by Pythagoras, since x is orthogonal to Q up to c1 -- and
// cp := c1 / nrm, the pending correction of the new basis vector x / nrm.  The
// vector that becomes the basis column is the CGS2 vector (x - Q c1) / nrm;
// only where it is materialised moves.  Layout and reductions as k_cgs_df: 8
// warps, warp w owning columns w + 8t, 64 rows per iteration, per-block FP64
// partials reduced in block order by the last block.
template <int NJ>
__global__ void __launch_bounds__(256) k_cgs_lag(float* __restrict__ Qh, float* __restrict__ Ql,
                                                 int64_t ld, int ncols, int pend,
                                                 float* __restrict__ xh, float* __restrict__ xl,
                                                 const double* __restrict__ y,
                                                 const BlkRange* __restrict__ blk,
                                                 const int* __restrict__ seg_blk, int nseg,
                                                 const int* __restrict__ active,
                                                 const double* __restrict__ c0, double* __restrict__ cp,
                                                 double* __restrict__ part, double* __restrict__ npart,
                                                 double* __restrict__ nrm, unsigned int* __restrict__ counter) {
  // coefficients as packed pairs (both lanes the same value): hi, -hi, lo
  __shared__ f2_t ck[MAX_WORK][3], pk[MAX_WORK][3];
  __shared__ float redh[8][64], redl[8][64], rch[8][64], rcl[8][64];
  __shared__ float xsh[64], xsl[64], wsh[64], wsl[64];
  __shared__ double nsh[32];
  __shared__ bool last;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const BlkRange br = blk[blockIdx.x];
  const int sg = br.seg;
  for (int j = tid; j < ncols; j += blockDim.x) {
    float h, l;
    df_split(c0[sg * MAX_WORK + j], h, l);
    ck[j][0] = f2_pack(h, h);
    ck[j][1] = f2_pack(-h, -h);
    ck[j][2] = f2_pack(l, l);
  }
  for (int j = tid; j < pend; j += blockDim.x) {
    float h, l;
    df_split(cp[sg * MAX_WORK + j], h, l);
    pk[j][0] = f2_pack(h, h);
    pk[j][1] = f2_pack(-h, -h);
    pk[j][2] = f2_pack(l, l);
  }
  __syncthreads();
  const int64_t r0 = br.r0, r1 = (active == nullptr || active[sg]) ? br.r1 : br.r0;
  const int pw = pend >= 0 ? (pend & 7) : -1, pt = pend >= 0 ? (pend >> 3) : -1;
  // dot accumulators: one packed pair per column, lanes = the thread's two rows
  f2_t dh[NJ], dl[NJ];
#pragma unroll
  for (int t = 0; t < NJ; ++t) dh[t] = dl[t] = 0ull;
  float nah = 0.f, nal = 0.f;   // |x|^2, double-float
  for (int64_t i0 = r0; i0 < r1; i0 += 64) {
    const int64_t ia = i0 + lane, ib = ia + 32;
    const bool va = ia < r1, vb = ib < r1;
    // the row of the product this thread finishes below, loaded ahead
    float yh = 0.f, yl = 0.f;
    if (tid < 64 && i0 + tid < r1) {
      if (y) {
        df_split(y[i0 + tid], yh, yl);
      } else {
        yh = xh[i0 + tid];
        yl = xl[i0 + tid];
      }
    }
    f2_t qh[NJ], ql[NJ];
#pragma unroll
    for (int t = 0; t < NJ; ++t) {
      const int j = w + 8 * t;
      const int64_t o = (int64_t)j * ld + ia;
      float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;
      if (j < ncols) {
        if (va) {
          a0 = Qh[o];
          b0 = Ql[o];
        }
        if (vb) {
          a1 = Qh[o + 32];
          b1 = Ql[o + 32];
        }
      }
      qh[t] = f2_pack(a0, a1);
      ql[t] = f2_pack(b0, b1);
    }
    f2_t sh = 0ull, sl = 0ull;   // Q c0 (but the pending column)
    f2_t ph = 0ull, pl = 0ull;   // Q[:, :pend] cp
#pragma unroll
    for (int t = 0; t < NJ; ++t) {
      const int j = w + 8 * t;
      if (j < ncols && j != pend) df_fma2(sh, sl, ck[j][0], ck[j][1], ck[j][2], qh[t], ql[t]);
      if (j < pend) df_fma2(ph, pl, pk[j][0], pk[j][1], pk[j][2], qh[t], ql[t]);
      if (t == pt && w == pw) {
        f2_unpack(qh[t], wsh[lane], wsh[lane + 32]);
        f2_unpack(ql[t], wsl[lane], wsl[lane + 32]);
      }
    }
    f2_unpack(sh, redh[w][lane], redh[w][lane + 32]);
    f2_unpack(sl, redl[w][lane], redl[w][lane + 32]);
    f2_unpack(ph, rch[w][lane], rch[w][lane + 32]);
    f2_unpack(pl, rcl[w][lane], rcl[w][lane + 32]);
    __syncthreads();
    if (tid < 64) {
      const int64_t i = i0 + tid;
      float h = 0.f, l = 0.f, wh = 0.f, wl = 0.f;
      if (i < r1) {
        float uh = 0.f, ul = 0.f;
#pragma unroll
        for (int u = 0; u < 8; ++u) df_acc(uh, ul, redh[u][tid], redl[u][tid]);
        if (pend >= 0) {
          float qh2 = 0.f, ql2 = 0.f;
#pragma unroll
          for (int u = 0; u < 8; ++u) df_acc(qh2, ql2, rch[u][tid], rcl[u][tid]);
          wh = wsh[tid];
          wl = wsl[tid];
          df_sub(wh, wl, qh2, ql2);
          Qh[(int64_t)pend * ld + i] = wh;
          Ql[(int64_t)pend * ld + i] = wl;
          float c0h, c0l, nc0h;
          f2_unpack(ck[pend][0], c0h, nc0h);
          f2_unpack(ck[pend][2], c0l, nc0h);
          df_fma(uh, ul, wh, wl, c0h, c0l);
        }
        h = yh;
        l = yl;
        df_sub(h, l, uh, ul);
        xh[i] = h;
        xl[i] = l;
        df_fma(nah, nal, h, l, h, l);
      }
      xsh[tid] = h;
      xsl[tid] = l;
      wsh[tid] = wh;
      wsl[tid] = wl;
    }
    __syncthreads();
    const float x0h = xsh[lane], x1h = xsh[lane + 32];
    const f2_t xh2 = f2_pack(x0h, x1h), nxh2 = f2_pack(-x0h, -x1h), xl2 = f2_pack(xsl[lane], xsl[lane + 32]);
#pragma unroll
    for (int t = 0; t < NJ; ++t) {
      if (t == pt && w == pw) {
        qh[t] = f2_pack(wsh[lane], wsh[lane + 32]);
        ql[t] = f2_pack(wsl[lane], wsl[lane + 32]);
      }
      if (w + 8 * t < ncols) df_fma2(dh[t], dl[t], xh2, nxh2, xl2, qh[t], ql[t]);
    }
  }
#pragma unroll
  for (int t = 0; t < NJ; ++t) {
    const int j = w + 8 * t;
    if (j < ncols) {
      // the two rows' sums, then across the warp (double-float, FP32 shuffles)
      float h, l, h2, l2;
      f2_unpack(dh[t], h, h2);
      f2_unpack(dl[t], l, l2);
      df_acc(h, l, h2, l2);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        float hs = __shfl_xor_sync(0xffffffffu, h, o);
        float ls = __shfl_xor_sync(0xffffffffu, l, o);
        float s = h + hs;
        float v = s - h;
        float err = (h - (s - v)) + (hs - v);
        float lo = err + l + ls;
        h = s + lo;
        l = lo - (h - s);
      }
      if (lane == 0) part[(int64_t)blockIdx.x * ncols + j] = df_val(h, l);
    }
  }
  const double nacc = block_sum(df_val(nah, nal), nsh);
  if (tid == 0) npart[blockIdx.x] = nacc;
  if (last_block(counter, &last)) {
    // c1 per (sample, column), in block order
    for (int pq = w; pq < nseg * ncols; pq += 8) {
      const int s2 = pq / ncols, j = pq - s2 * ncols;
      double sacc = 0;
      for (int b = seg_blk[s2] + lane; b < seg_blk[s2 + 1]; b += 32) sacc += part[(int64_t)b * ncols + j];
      sacc = sv_warp_sum(sacc);
      if (lane == 0) cp[s2 * MAX_WORK + j] = sacc;
    }
    __syncthreads();
    for (int s2 = tid; s2 < nseg; s2 += blockDim.x) {
      double nsq = 0, csq = 0;
      for (int b = seg_blk[s2]; b < seg_blk[s2 + 1]; ++b) nsq += npart[b];
      for (int j = 0; j < ncols; ++j) csq += cp[s2 * MAX_WORK + j] * cp[s2 * MAX_WORK + j];
      const double r = sqrt(fmax(nsq - csq, 0.0));
      nrm[s2] = r;
      const double inv = r > 0 ? 1.0 / r : 0.0;
      for (int j = 0; j < ncols; ++j) cp[s2 * MAX_WORK + j] *= inv;
    }
    if (tid == 0) *counter = 0;
  }
}

// ---- the same pass with the basis tiles brought in by the tensor-memory
// accelerator ---------------------------------------------------------------
// The basis columns 0..ncols-1 are two 2D tensors (rows x ncols, hi and lo);
// one tensor copy per 8-column group and array lands a box of rows x 8 columns
// column-major ([column][row]).  Rows outside the block's range (the 4-row
// alignment of the copy start) are read but carry x = 0 and are not written;
// columns at or beyond ncols and rows beyond the basis are filled with zeros
// by the copy.  Every wait is bounded: on a timeout the block records
// SV_STATUS_LIMIT, lets its copies land (bounded) and contributes nothing.
// (sh, sl) += (bh, bl) on packed pairs, unnormalised (df_acc per lane)
__device__ __forceinline__ void df_acc2(f2_t& sh, f2_t& sl, f2_t bh, f2_t bl) {
  f2_t t = f2_add(sh, bh);
  f2_t v = f2_sub(t, sh);
  f2_t err = f2_add(f2_sub(sh, f2_sub(t, v)), f2_sub(bh, v));
  sh = t;
  sl = f2_add(sl, f2_add(err, bl));
}
constexpr int LT_GC = 8;   // columns per tensor box
constexpr long long LT_TIMEOUT = 4000000000ll;   // cycles (~2 s) per wait

__device__ __forceinline__ uint32_t lt_su32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ bool lt_try(unsigned long long* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(lt_su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool lt_wait(unsigned long long* b, uint32_t parity) {
  if (lt_try(b, parity)) return true;
  const long long t0 = clock64();
  while (!lt_try(b, parity))
    if (clock64() - t0 > LT_TIMEOUT) return false;
  return true;
}

// The TMA-fed pass.  Eight compute warps in two groups of four and one copy
// warp per block; a tile is 128 rows (32 per warp of a group) x ncols columns;
// the groups take alternate tiles from a ring of NST stages, which the copy warp
// refills as soon as the four warps of the consuming group have released a
// stage (empty barriers).  No block barrier in the main loop:
//   phase 1, lane = row: the lane sums Q c0 and Q[:, :pend] cp over every column
//     of its row (column pairs in packed double-float), corrects the pending
//     column (global and in the tile) and forms x;
//   phase 2, lane = column pair: the lane walks the warp's 32 rows diagonally
//     (row (lane + k) mod 32, so that the 32 lanes read 32 different banks) and
//     accumulates its two dot products in registers across all tiles.
// Per-warp dot products are combined per block in fixed warp order.
constexpr int LR_GROUP = 4;                 // compute warps per tile
constexpr int LR_WARPS = 2 * LR_GROUP;      // compute warps per block
constexpr int LR_ROWS = 32 * LR_GROUP;      // rows per tile
constexpr int LR_STAGES = 3;

template <int NST>
__global__ void __launch_bounds__(32 * (LR_WARPS + 1)) k_cgs_lag_tma(
    const __grid_constant__ CUtensorMap mh, const __grid_constant__ CUtensorMap ml, float* __restrict__ Qh,
    float* __restrict__ Ql, int64_t ld, int ncols, int pend, float* __restrict__ xh, float* __restrict__ xl,
    const double* __restrict__ y, const BlkRange* __restrict__ blk, const int* __restrict__ seg_blk, int nseg,
    const int* __restrict__ active, const double* __restrict__ c0, double* __restrict__ cp,
    double* __restrict__ part, double* __restrict__ npart, double* __restrict__ nrm,
    unsigned int* __restrict__ counter, int* __restrict__ status) {
  extern __shared__ unsigned char lt_dyn[];
  float* tiles = (float*)(((uintptr_t)lt_dyn + 1023) & ~(uintptr_t)1023);
  // coefficients of the column pairs (2q, 2q+1), packed: hi, -hi, lo
  __shared__ f2_t ck[MAX_WORK / 2][3], pk[MAX_WORK / 2][3];
  __shared__ float c0p[2];   // c0 of the pending column (hi, lo)
  __shared__ float xsh[LR_WARPS][32], xsl[LR_WARPS][32];
  __shared__ double wred[LR_WARPS][MAX_WORK];
  __shared__ double nsh[32];
  __shared__ unsigned long long full[NST], empty[NST];
  __shared__ int err;
  __shared__ bool last;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const BlkRange br = blk[blockIdx.x];
  const int sg = br.seg;
  const int npairs = (ncols + 1) >> 1;
  for (int q = tid; q < npairs; q += blockDim.x) {
    float h[2], l[2], ph[2], pl[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int j = 2 * q + u;
      h[u] = l[u] = ph[u] = pl[u] = 0.f;
      // the pending column enters corrected, separately
      if (j < ncols && j != pend) df_split(c0[sg * MAX_WORK + j], h[u], l[u]);
      if (j < pend) df_split(cp[sg * MAX_WORK + j], ph[u], pl[u]);
    }
    ck[q][0] = f2_pack(h[0], h[1]);
    ck[q][1] = f2_pack(-h[0], -h[1]);
    ck[q][2] = f2_pack(l[0], l[1]);
    pk[q][0] = f2_pack(ph[0], ph[1]);
    pk[q][1] = f2_pack(-ph[0], -ph[1]);
    pk[q][2] = f2_pack(pl[0], pl[1]);
  }
  if (tid == 0) {
    c0p[0] = c0p[1] = 0.f;
    if (pend >= 0) df_split(c0[sg * MAX_WORK + pend], c0p[0], c0p[1]);
  }
  const int ngroups = (ncols + LT_GC - 1) / LT_GC;
  const int gfl = 2 * LT_GC * LR_ROWS;   // floats per column group: the hi box, then the lo box
  const int sfl = ngroups * gfl;
  const int64_t r0 = br.r0, r1 = (active == nullptr || active[sg]) ? br.r1 : br.r0;
  const int64_t xs = r0 & ~(int64_t)3;
  const int ntiles = r1 > r0 ? (int)((r1 - xs + LR_ROWS - 1) / LR_ROWS) : 0;
  if (tid == 0) {
    for (int st = 0; st < NST; ++st) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(lt_su32(&full[st])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(lt_su32(&empty[st])), "r"(LR_GROUP)
                   : "memory");
    }
    err = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  float nah = 0.f, nal = 0.f;
  if (w == LR_WARPS) {
    // the copy warp
    if (lane == 0) {
      int t = 0;
      for (; t < ntiles; ++t) {
        const int st = t % NST;
        if (t >= NST && !lt_wait(&empty[st], (uint32_t)(((t / NST) - 1) & 1))) {
          atomicOr(&err, 1);
          break;
        }
        float* dst = tiles + st * sfl;
        const int x = (int)(xs + (int64_t)t * LR_ROWS);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(lt_su32(&full[st])),
                     "r"((uint32_t)sfl * 4u)
                     : "memory");
        for (int g = 0; g < ngroups; ++g) {
          asm volatile(
              "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
                  lt_su32(dst + g * gfl)),
              "l"(&mh), "r"(x), "r"(g * LT_GC), "r"(lt_su32(&full[st]))
              : "memory");
          asm volatile(
              "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
                  lt_su32(dst + g * gfl + LT_GC * LR_ROWS)),
              "l"(&ml), "r"(x), "r"(g * LT_GC), "r"(lt_su32(&full[st]))
              : "memory");
        }
      }
      // the copies in flight land before the block moves on (bounded)
      for (int u = t - NST; u < t; ++u)
        if (u >= 0) lt_wait(&full[u % NST], (uint32_t)((u / NST) & 1));
    }
    __syncwarp();
  } else {
    const int grp = w / LR_GROUP, wi = w % LR_GROUP;
    const int rl = 32 * wi + lane;   // the lane's row within a tile
    // the lane's column pair, four accumulators (row k mod 4)
    f2_t dh = 0ull, dl = 0ull, dh2 = 0ull, dl2 = 0ull, dh3 = 0ull, dl3 = 0ull, dh4 = 0ull, dl4 = 0ull;
    float yh = 0.f, yl = 0.f;
    auto load_y = [&](int t) {
      const int64_t i = xs + (int64_t)t * LR_ROWS + rl;
      yh = yl = 0.f;
      if (t < ntiles && i >= r0 && i < r1) {
        if (y) {
          df_split(y[i], yh, yl);
        } else {
          yh = xh[i];
          yl = xl[i];
        }
      }
    };
    load_y(grp);
    for (int t = grp; t < ntiles; t += 2) {
      const int st = t % NST;
      const int64_t i = xs + (int64_t)t * LR_ROWS + rl;
      const bool valid = i >= r0 && i < r1;
      const float cyh = yh, cyl = yl;
      load_y(t + 2);
      if (!lt_wait(&full[st], (uint32_t)((t / NST) & 1))) {
        atomicOr(&err, 1);
        break;
      }
      float* T = tiles + st * sfl;
      // phase 1: the lane's row (two accumulators per sum: even and odd pairs)
      f2_t uh = 0ull, ul = 0ull, ph = 0ull, pl = 0ull;
      f2_t uh2 = 0ull, ul2 = 0ull, ph2 = 0ull, pl2 = 0ull;
      for (int q = 0; q < npairs; ++q) {
        const int c = 2 * q;
        const float* ch = T + (c >> 3) * gfl + (c & 7) * LR_ROWS + rl;
        const f2_t qh = f2_pack(ch[0], ch[LR_ROWS]);
        const f2_t ql = f2_pack(ch[LT_GC * LR_ROWS], ch[LT_GC * LR_ROWS + LR_ROWS]);
        if (q & 1) {
          df_fma2(uh2, ul2, ck[q][0], ck[q][1], ck[q][2], qh, ql);
          if (c < pend) df_fma2(ph2, pl2, pk[q][0], pk[q][1], pk[q][2], qh, ql);
        } else {
          df_fma2(uh, ul, ck[q][0], ck[q][1], ck[q][2], qh, ql);
          if (c < pend) df_fma2(ph, pl, pk[q][0], pk[q][1], pk[q][2], qh, ql);
        }
      }
      df_acc2(uh, ul, uh2, ul2);
      df_acc2(ph, pl, ph2, pl2);
      float sh, sl, s2h, s2l;
      f2_unpack(uh, sh, s2h);
      f2_unpack(ul, sl, s2l);
      df_acc(sh, sl, s2h, s2l);
      if (pend >= 0) {
        float p1h, p1l, p2h, p2l;
        f2_unpack(ph, p1h, p2h);
        f2_unpack(pl, p1l, p2l);
        df_acc(p1h, p1l, p2h, p2l);
        float* cw = T + (pend >> 3) * gfl + (pend & 7) * LR_ROWS + rl;
        float wh = cw[0], wl = cw[LT_GC * LR_ROWS];
        df_sub(wh, wl, p1h, p1l);
        cw[0] = wh;
        cw[LT_GC * LR_ROWS] = wl;
        if (valid) {
          Qh[(int64_t)pend * ld + i] = wh;
          Ql[(int64_t)pend * ld + i] = wl;
        }
        df_fma(sh, sl, wh, wl, c0p[0], c0p[1]);
      }
      float x_h = 0.f, x_l = 0.f;
      if (valid) {
        x_h = cyh;
        x_l = cyl;
        df_sub(x_h, x_l, sh, sl);
        xh[i] = x_h;
        xl[i] = x_l;
        df_fma(nah, nal, x_h, x_l, x_h, x_l);
      }
      xsh[w][lane] = x_h;
      xsl[w][lane] = x_l;
      __syncwarp();
      // phase 2: the lane's column pair over the warp's 32 rows
      if (lane < npairs) {
        const float* ch = T + ((2 * lane) >> 3) * gfl + ((2 * lane) & 7) * LR_ROWS + 32 * wi;
        for (int k = 0; k < 32; k += 4) {
          f2_t qh[4], ql[4];
          float a[4], b[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int r = (lane + k + u) & 31;
            qh[u] = f2_pack(ch[r], ch[LR_ROWS + r]);
            ql[u] = f2_pack(ch[LT_GC * LR_ROWS + r], ch[LT_GC * LR_ROWS + LR_ROWS + r]);
            a[u] = xsh[w][r];
            b[u] = xsl[w][r];
          }
          df_fma2(dh, dl, f2_pack(a[0], a[0]), f2_pack(-a[0], -a[0]), f2_pack(b[0], b[0]), qh[0], ql[0]);
          df_fma2(dh2, dl2, f2_pack(a[1], a[1]), f2_pack(-a[1], -a[1]), f2_pack(b[1], b[1]), qh[1], ql[1]);
          df_fma2(dh3, dl3, f2_pack(a[2], a[2]), f2_pack(-a[2], -a[2]), f2_pack(b[2], b[2]), qh[2], ql[2]);
          df_fma2(dh4, dl4, f2_pack(a[3], a[3]), f2_pack(-a[3], -a[3]), f2_pack(b[3], b[3]), qh[3], ql[3]);
        }
      }
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(lt_su32(&empty[st])) : "memory");
    }
    df_acc2(dh, dl, dh2, dl2);
    df_acc2(dh3, dl3, dh4, dl4);
    df_acc2(dh, dl, dh3, dl3);
    if (lane < npairs) {
      float h0, h1, l0, l1;
      f2_unpack(dh, h0, h1);
      f2_unpack(dl, l0, l1);
      wred[w][2 * lane] = df_val(h0, l0);
      if (2 * lane + 1 < ncols) wred[w][2 * lane + 1] = df_val(h1, l1);
    }
  }
  __syncthreads();
  if (err) {
    if (tid == 0) atomicOr(status, SV_STATUS_LIMIT);
    nah = nal = 0.f;
  }
  for (int j = tid; j < ncols; j += blockDim.x) {
    double v = 0;
    if (!err)
      for (int u = 0; u < LR_WARPS; ++u) v += wred[u][j];
    part[(int64_t)blockIdx.x * ncols + j] = v;
  }
  const double nacc = block_sum(df_val(nah, nal), nsh);
  if (tid == 0) npart[blockIdx.x] = nacc;
  if (last_block(counter, &last)) {
    for (int pq = w; pq < nseg * ncols; pq += LR_WARPS + 1) {
      const int s2 = pq / ncols, j = pq - s2 * ncols;
      double sacc = 0;
      for (int b = seg_blk[s2] + lane; b < seg_blk[s2 + 1]; b += 32) sacc += part[(int64_t)b * ncols + j];
      sacc = sv_warp_sum(sacc);
      if (lane == 0) cp[s2 * MAX_WORK + j] = sacc;
    }
    __syncthreads();
    for (int s2 = tid; s2 < nseg; s2 += blockDim.x) {
      double nsq = 0, csq = 0;
      for (int b = seg_blk[s2]; b < seg_blk[s2 + 1]; ++b) nsq += npart[b];
      for (int j = 0; j < ncols; ++j) csq += cp[s2 * MAX_WORK + j] * cp[s2 * MAX_WORK + j];
      const double r = sqrt(fmax(nsq - csq, 0.0));
      nrm[s2] = r;
      const double inv = r > 0 ? 1.0 / r : 0.0;
      for (int j = 0; j < ncols; ++j) cp[s2 * MAX_WORK + j] *= inv;
    }
    if (tid == 0) *counter = 0;
  }
}

// First projection coefficients of a cell-side step from the feature side: the
// new vector is y = A v - beta w' (w' the stored, not yet corrected column pend;
// no subtraction when pend < 0), so Q^T y = G^T v - beta Q^T w' with G = A^T Q
// and Q^T w' = (cp, 1, 0...) (w' = w + Q[:, :pend] cp, w a unit vector
// orthogonal to Q[:, :pend]).  Block (column l, sample s); FP64 sums over the
// sample's feature rows.
__global__ void __launch_bounds__(256) k_gdots(const float* __restrict__ Gh, const float* __restrict__ Gl,
                                               int64_t ld, const int64_t* __restrict__ off,
                                               const double* __restrict__ v, int pend,
                                               const double* __restrict__ beta,
                                               const double* __restrict__ cp, const int* __restrict__ active,
                                               double* __restrict__ c0) {
  __shared__ double sh[32];
  const int l = blockIdx.x, sg = blockIdx.y;
  if (active && !active[sg]) return;
  double acc = 0;
  for (int64_t i = off[sg] + threadIdx.x; i < off[sg + 1]; i += blockDim.x) {
    const int64_t o = (int64_t)l * ld + i;
    acc += df_val(Gh[o], Gl[o]) * v[i];
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    if (pend >= 0) acc -= beta[sg] * (l < pend ? cp[sg * MAX_WORK + l] : l == pend ? 1.0 : 0.0);
    c0[sg * MAX_WORK + l] = acc;
  }
}

// After the feature-side product of a cell-side column jn, F = A^T w' - alpha v
// with w' = w + Q[:, :jn] cp not yet corrected: F -= G[:, :jn] cp makes it the
// product of the corrected w, and G[:, jn] := F + alpha v = A^T w.
__global__ void __launch_bounds__(256) k_gcol(float* __restrict__ Gh, float* __restrict__ Gl, int64_t ld,
                                              const BlkRange* __restrict__ blk, const int* __restrict__ active,
                                              int jn, const double* __restrict__ cp,
                                              const double* __restrict__ alpha, const double* __restrict__ v,
                                              double* __restrict__ F) {
  __shared__ double cs[MAX_WORK];
  const BlkRange br = blk[blockIdx.x];
  const int sg = br.seg;
  if (active && !active[sg]) return;
  for (int j = threadIdx.x; j < jn; j += blockDim.x) cs[j] = cp[sg * MAX_WORK + j];
  __syncthreads();
  const double a = alpha[sg];
  for (int64_t i = br.r0 + threadIdx.x; i < br.r1; i += blockDim.x) {
    double corr = 0;
    for (int j = 0; j < jn; ++j) {
      const int64_t o = (int64_t)j * ld + i;
      corr += df_val(Gh[o], Gl[o]) * cs[j];
    }
    const double f = F[i] - corr;
    F[i] = f;
    df_split(f + a * v[i], Gh[(int64_t)jn * ld + i], Gl[(int64_t)jn * ld + i]);
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
#define CTL_N 3          // control-block doubles per sample
__device__ __forceinline__ unsigned long long breakdown_tag(const double* ctl, unsigned step) {
  return (unsigned long long)ctl[CTL_CYCLE] * 1024ull + step;
}

// Basis column := x / nrm[s] (double-float) and cur := the same in FP64; the B
// entry of sample s (B + s*bstride + boff, when B is given) := nrm[s].  When
// nrm[s] < the sample's threshold the Krylov space is (numerically) invariant:
// cur := a random vector, B entry := 0, flag[s] set for k_fix_df, which
// orthonormalises cur against the basis and writes the column.  Rows of sample
// s are indexed from its offset for the random vector (i - off).
__global__ void k_scal_df(const float* __restrict__ xh, const float* __restrict__ xl,
                          const BlkRange* __restrict__ blk, const int* __restrict__ seg_blk,
                          const int64_t* __restrict__ off, const int* __restrict__ active,
                          const double* __restrict__ nrm, const double* __restrict__ ctl,
                          float* __restrict__ colh, float* __restrict__ coll, double* __restrict__ cur,
                          double* __restrict__ B, int64_t boff, int64_t bstride, int* __restrict__ flag,
                          unsigned long long seed, unsigned step) {
  const BlkRange br = blk[blockIdx.x];
  const int sg = br.seg;
  if (active && !active[sg]) return;
  const double* c = ctl + sg * CTL_N;
  double s = nrm[sg];
  bool brk = !(s >= c[CTL_THRESH]);
  unsigned long long tag = breakdown_tag(c, step);
  double inv = brk ? 0.0 : 1.0 / s;
  for (int64_t i = br.r0 + threadIdx.x; i < br.r1; i += blockDim.x) {
    if (brk) {
      cur[i] = normal_at(seed, tag, i - off[sg]);
    } else {
      double v = df_val(xh[i], xl[i]) * inv;
      cur[i] = v;
      df_split(v, colh[i], coll[i]);
    }
  }
  if ((int)blockIdx.x == seg_blk[sg] && threadIdx.x == 0) {
    if (B) B[sg * bstride + boff] = brk ? 0.0 : s;
    if (brk) flag[sg] = 1;
  }
}

// zero the norm slot (the sub-diagonal scalar the next product uses) of every
// sample whose breakdown was flagged, and its pending correction (cp, cell
// side); separate launch so every k_scal_df block has read it
__global__ void k_scal_post(double* nrm, const int* flag, int nseg, double* cp) {
  for (int s = threadIdx.x; s < nseg; s += blockDim.x)
    if (flag[s]) {
      nrm[s] = 0.0;
      // the replacement vector is orthonormalised in full: nothing pending
      if (cp)
        for (int j = 0; j < MAX_WORK; ++j) cp[s * MAX_WORK + j] = 0.0;
    }
}

// One block per sample: if flag[s], cur <- CGS2(cur, Q[:, :ncols]) normalised
// (FP64 arithmetic on the double-float basis) over the sample's rows, written to
// the basis column as well; clears the flag.  Runs only on a breakdown.
__global__ void k_fix_df(double* __restrict__ cur0, const int64_t* __restrict__ off,
                         const float* __restrict__ Qh0, const float* __restrict__ Ql0, int64_t ld,
                         int ncols, float* __restrict__ colh0, float* __restrict__ coll0,
                         int* __restrict__ flags) {
  __shared__ double sh[32];
  __shared__ double cs[MAX_WORK];
  __shared__ double tot;
  const int sg = blockIdx.x;
  int* flag = flags + sg;
  if (*flag == 0) return;
  const int64_t o0 = off[sg], len = off[sg + 1] - o0;
  double* cur = cur0 + o0;
  const float* Qh = Qh0 + o0;
  const float* Ql = Ql0 + o0;
  float* colh = colh0 + o0;
  float* coll = coll0 + o0;
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

// The whole feature-side step of a sample in one block (the feature side is
// short: a few thousand entries), one block per sample: x = F (FP64 in,
// double-float working copy in xh/xl); CGS2 against V[:, :ncols]; nrm[s] = |x|;
// when write_col >= 0 the column write_col := x/|x| (double-float, FP64 copy in
// cur) and the B entry = |x|, or on a breakdown (|x| < threshold) a random vector
// orthonormalised against V[:, :ncols] with B entry = nrm[s] = 0.  write_col < 0
// (last step of a cycle) leaves the residual in xh/xl.
__device__ void vside_cgs2(float* __restrict__ xh, float* __restrict__ xl, int64_t len,
                           const float* __restrict__ Vh, const float* __restrict__ Vl, int64_t ld,
                           int ncols, double* c, float* ch, float* cl) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int pass = 0; pass < 2 && ncols > 0; ++pass) {
    for (int j = w; j < ncols; j += nw) {
      float ah = 0.f, al = 0.f;
      const float* qh = Vh + (int64_t)j * ld;
      const float* ql = Vl + (int64_t)j * ld;
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
        int64_t o = (int64_t)j * ld + i;
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

__global__ void __launch_bounds__(1024) k_vside(const double* __restrict__ F0,
                                                const int64_t* __restrict__ off, int64_t ld,
                                                float* __restrict__ Vh0, float* __restrict__ Vl0,
                                                int ncols, int write_col, double* __restrict__ nrm,
                                                const double* __restrict__ ctl,
                                                double* __restrict__ B, int64_t boff, int64_t bstride,
                                                double* __restrict__ cur0, float* __restrict__ xh0,
                                                float* __restrict__ xl0, const int* __restrict__ active,
                                                unsigned long long seed, unsigned step) {
  __shared__ double c[MAX_WORK];
  __shared__ float ch[MAX_WORK], cl[MAX_WORK];
  __shared__ double sh[32];
  __shared__ double tot;
  const int sg = blockIdx.x;   // one block per sample
  if (active && !active[sg]) return;
  const int64_t o0 = off[sg], len = off[sg + 1] - o0;
  const double* F = F0 + o0;
  float* Vh = Vh0 + o0;
  float* Vl = Vl0 + o0;
  double* cur = cur0 + o0;
  float* xh = xh0 + o0;
  float* xl = xl0 + o0;
  const double* cb = ctl + sg * CTL_N;
  double* bentry = B ? B + sg * bstride + boff : nullptr;
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) df_split(F[i], xh[i], xl[i]);
  __syncthreads();
  vside_cgs2(xh, xl, len, Vh, Vl, ld, ncols, c, ch, cl);
  double s = vside_norm(xh, xl, len, sh, &tot);
  if (write_col < 0) {
    if (threadIdx.x == 0) nrm[sg] = s;
    return;
  }
  bool brk = !(s >= cb[CTL_THRESH]);
  if (brk) {
    unsigned long long tag = breakdown_tag(cb, step);
    for (int64_t i = threadIdx.x; i < len; i += blockDim.x) df_split(normal_at(seed, tag, i), xh[i], xl[i]);
    __syncthreads();
    vside_cgs2(xh, xl, len, Vh, Vl, ld, ncols, c, ch, cl);
    double r = vside_norm(xh, xl, len, sh, &tot);
    double inv = 1.0 / r;
    for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
      double v = df_val(xh[i], xl[i]) * inv;
      cur[i] = v;
      df_split(v, Vh[(int64_t)write_col * ld + i], Vl[(int64_t)write_col * ld + i]);
    }
    if (threadIdx.x == 0) {
      nrm[sg] = 0.0;
      if (bentry) *bentry = 0.0;
    }
  } else {
    double inv = 1.0 / s;
    for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
      double v = df_val(xh[i], xl[i]) * inv;
      cur[i] = v;
      df_split(v, Vh[(int64_t)write_col * ld + i], Vl[(int64_t)write_col * ld + i]);
    }
    if (threadIdx.x == 0) {
      nrm[sg] = s;
      if (bentry) *bentry = s;
    }
  }
}

// One-sided (Hestenes) Jacobi SVD of B (m x m, row-major), one block per sample, in
// double-float arithmetic: FP64 runs at 1/57 of the FP32 rate on this part (one
// warp-wide FP64 instruction occupies an SM's FP64 pipe for ~17 cycles), and an
// FP64 block spent ~4 ms per 57 x 57 SVD, so the columns of A = B and the
// accumulated rotations J are held as (hi, lo) FP32 pairs in shared memory and
// updated on the FP32 pipe, and the rotation parameters are formed in FP32 and
// normalised in double-float.
// Columns are paired by the circle method (slot 0 fixed, the others rotating),
// one warp per pair; a pair is rotated while |a_p . a_q| > tau |a_p| |a_q| with
// tau = 1e-12 max(1, m / 16): a double-float dot product of m terms carries an
// absolute error of about m 2^-48 |a_p| |a_q| (the low parts are summed in FP32),
// so a threshold below that floor (FP64's 1e-15, or 1e-13 for m ~ 40) can keep
// a sweep rotating on rounding noise.  Then s_i = |A e_i|, P_i = A e_i / s_i,
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

__global__ void __launch_bounds__(1024) k_jacobi_svd(const double* __restrict__ B0, int m,
                                                     double* __restrict__ Pout0,
                                                     double* __restrict__ sout0,
                                                     double* __restrict__ Qout0,
                                                     double* __restrict__ summary0,
                                                     const double* __restrict__ rf0, int max_sweeps,
                                                     int* __restrict__ status,
                                                     double* __restrict__ ctl0, double eps_b,
                                                     const int* __restrict__ active) {
  extern __shared__ float smf[];
  // one block per sample
  const int sg = blockIdx.x;
  if (active && !active[sg]) return;
  const double* B = B0 + (int64_t)sg * m * m;
  double* Pout = Pout0 + (int64_t)sg * m * m;
  double* Qout = Qout0 + (int64_t)sg * m * m;
  double* sout = sout0 + (int64_t)sg * m;
  double* summary = summary0 + (int64_t)sg * (2 * m + 2);
  const double* rf = rf0 ? rf0 + sg : nullptr;
  double* ctl = ctl0 + sg * CTL_N;
  float* Ah = smf;              // m*m, column c at [c*m]
  float* Al = Ah + m * m;
  float* Jh = Al + m * m;
  float* Jl = Jh + m * m;
  __shared__ int rotated;
  __shared__ int order[MAX_WORK];
  __shared__ double nrm[MAX_WORK];
  // squared column norms (double-float): computed at the start of a sweep and
  // carried through its rotations by alpha' = alpha - t gamma, beta' = beta +
  // t gamma (exact for the diagonalising angle); they only steer the angles and
  // the convergence test -- the singular values come from the final columns
  __shared__ float cnh[MAX_WORK], cnl[MAX_WORK];
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
  const float tau = 1e-12f * fmaxf(1.f, (float)m / 16.f);
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    if (tid == 0) rotated = 0;
    for (int c = wid; c < m; c += nw) {
      float h = 0.f, l = 0.f;
      for (int r = lane; r < m; r += 32) df_fma(h, l, Ah[c * m + r], Al[c * m + r], Ah[c * m + r], Al[c * m + r]);
      df_warp_sum(h, l);
      if (lane == 0) {
        cnh[c] = h;
        cnl[c] = l;
      }
    }
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
        const float alh = cnh[p], all = cnl[p], beh = cnh[q], bel = cnl[q];
        float gah = 0.f, gal = 0.f;
        for (int r = lane; r < m; r += 32) df_fma(gah, gal, aph[r], apl[r], aqh[r], aql[r]);
        df_warp_sum(gah, gal);
        // every lane holds the sums; the test and the angle are FP32 (from
        // double-float sums): the angle only steers convergence, while the
        // orthogonality of the applied rotation comes from normalising (c, s)
        // in double-float
        if (fabsf(gah) > tau * sqrtf(alh) * sqrtf(beh) && gah != 0.f) {
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
          if (lane == 0) {
            rotated = 1;
            float ah2 = alh, al2 = all, bh2 = beh, bl2 = bel;
            df_fma(ah2, al2, -t, 0.f, gah, gal);
            df_fma(bh2, bl2, t, 0.f, gah, gal);
            cnh[p] = ah2;
            cnl[p] = al2;
            cnh[q] = bh2;
            cnl[q] = bl2;
          }
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
// per pass over a row (KB even; the columns are taken in pairs, one packed
// f32x2 double-float multiply-add per pair and term); gridDim.y blocks share
// the passes of a row range (the short feature side).  M sits in shared memory
// as one float4 (hi c, hi c+1, lo c, lo c+1) per term and column pair, zero
// beyond nout, read with one broadcast 16-byte load.
template <int KB>
__global__ void __launch_bounds__(256) k_rotate_df(const float* __restrict__ Inh,
                                                   const float* __restrict__ Inl, int64_t ld_in,
                                                   const BlkRange* __restrict__ blk,
                                                   const int* __restrict__ sel, int nin,
                                                   const double* __restrict__ M0, int64_t mstride,
                                                   int nout, float* __restrict__ outh,
                                                   float* __restrict__ outl, double* __restrict__ outd,
                                                   int64_t ld_out) {
  static_assert(KB % 2 == 0, "column pairs");
  constexpr int NP = KB / 2;
  extern __shared__ float4 Ms4[];   // nin * (npass * NP)
  const BlkRange br = blk[blockIdx.x];
  if (sel && !sel[br.seg]) return;   // samples not selected keep their rows
  const double* M = M0 + br.seg * mstride;
  const int npass = (nout + KB - 1) / KB;
  const int npair = npass * NP;
  for (int idx = threadIdx.x; idx < nin * npair; idx += blockDim.x) {
    int r = idx % nin, q = idx / nin, c = 2 * q;
    float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f;
    if (c < nout) df_split(M[r + (int64_t)c * nin], h0, l0);
    if (c + 1 < nout) df_split(M[r + (int64_t)(c + 1) * nin], h1, l1);
    Ms4[idx] = make_float4(h0, h1, l0, l1);
  }
  __syncthreads();
  for (int64_t i = br.r0 + threadIdx.x; i < br.r1; i += blockDim.x) {
    for (int ps = blockIdx.y; ps < npass; ps += gridDim.y) {
      f2_t sh[NP], sl[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) sh[q] = sl[q] = 0ull;
      const float4* mrow = Ms4 + (int64_t)ps * NP * nin;
      for (int r = 0; r < nin; ++r) {
        int64_t o = (int64_t)r * ld_in + i;
        float wh = Inh[o], wl = Inl[o];
        f2_t ah = f2_pack(wh, wh), nah = f2_pack(-wh, -wh), al = f2_pack(wl, wl);
#pragma unroll
        for (int q = 0; q < NP; ++q) {
          float4 m = mrow[r + q * nin];
          df_fma2(sh[q], sl[q], ah, nah, al, f2_pack(m.x, m.y), f2_pack(m.z, m.w));
        }
      }
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        // renormalise the pairs
        f2_t h2 = f2_add(sh[q], sl[q]);
        f2_t l2 = f2_sub(sl[q], f2_sub(h2, sh[q]));
        float hv[2], lv[2];
        f2_unpack(h2, hv[0], hv[1]);
        f2_unpack(l2, lv[0], lv[1]);
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          int c = ps * KB + 2 * q + u;
          if (c < nout) {
            int64_t o = (int64_t)c * ld_out + i;
            if (outd) {
              outd[o] = df_val(hv[u], lv[u]);
            } else {
              outh[o] = hv[u];
              outl[o] = lv[u];
            }
          }
        }
      }
    }
  }
}

// V[:, k] = F / rf (double-float column + FP64 current vector) and B reset, per
// sample (blockIdx.y; rows off[s] .. off[s+1]).
__global__ void k_restart_tail(float* __restrict__ vkh, float* __restrict__ vkl,
                               double* __restrict__ vcur, const double* __restrict__ F,
                               const int64_t* __restrict__ off, const double* __restrict__ summary0,
                               int m, int k, double* __restrict__ B0, const int* __restrict__ active) {
  const int sg = blockIdx.y;
  if (active && !active[sg]) return;
  const double* summary = summary0 + (int64_t)sg * (2 * m + 2);
  double* B = B0 + (int64_t)sg * m * m;
  double rf = summary[2 * m];
  for (int64_t i = off[sg] + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < off[sg + 1];
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

// X[r, c] *= s[seg(r) * sstride + c] for the rows of sample blockIdx.y (X
// column-major with leading dimension ld)
__global__ void k_scale_cols(double* __restrict__ X, int64_t ld, const int64_t* __restrict__ off,
                             int ncols, const double* __restrict__ s, int sstride) {
  const int sg = blockIdx.y;
  const int64_t o0 = off[sg], len = off[sg + 1] - o0;
  const double* sc = s + (int64_t)sg * sstride;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < len * ncols;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int c = (int)(idx / len);
    int64_t r = idx - (int64_t)c * len;
    X[(int64_t)c * ld + o0 + r] *= sc[c];
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
  // the driver's per-sample active mask (device), for operators over stacked samples
  virtual void bind_active(const int* active) { (void)active; }
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

// Block-diagonal operator of stacked samples (sv_batch): csub and the vectors
// are per sample; frozen samples are skipped.
struct BatchOp : Op {
  sv_context* ctx;
  const sv_batch* b;
  const int* active = nullptr;
  BatchOp(sv_context* c, const sv_batch* bb) : ctx(c), b(bb) {}
  void N(const double*, double*, const double*, const double*) override {
    sv_throw(SV_ERR_UNSUPPORTED, "batched samples use the double-float product");
  }
  void T(const double* x, double* y, const double* csub, const double* z) override {
    sv_batch_apply_T(ctx, b, x, y, csub, z, active);
  }
  bool device_only() const override { return true; }
  bool N_df(const float* xh, const float* xl, float* yh, float* yl, const double* csub,
            const float* zh, const float* zl) override {
    sv_batch_apply_N_df(ctx, b, xh, xl, yh, yl, csub, zh, zl, active);
    return true;
  }
  void bind_active(const int* a) override { active = a; }
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


// Block schedule of a stacked side: each sample's rows split into contiguous
// ranges, about `target` blocks in total in proportion to the sample sizes (at
// least one per sample); a single sample gets ceil(len / target) rows per block.
static void build_schedule(const std::vector<int64_t>& off, int target, std::vector<BlkRange>& blk,
                           std::vector<int>& seg_blk) {
  int nseg = (int)off.size() - 1;
  int64_t total = std::max<int64_t>(1, off[nseg] - off[0]);
  blk.clear();
  seg_blk.assign(nseg + 1, 0);
  for (int s = 0; s < nseg; ++s) {
    seg_blk[s] = (int)blk.size();
    int64_t ns = off[s + 1] - off[s];
    int64_t nb = nseg == 1 ? target : (int64_t)llround((double)target * (double)ns / (double)total);
    nb = std::max<int64_t>(1, std::min<int64_t>(nb, std::max<int64_t>(1, ns)));
    int64_t per = std::max<int64_t>(1, (ns + nb - 1) / nb);
    for (int64_t r = 0; r < std::max<int64_t>(ns, 1); r += per) {
      BlkRange b;
      b.r0 = off[s] + r;
      b.r1 = off[s] + std::min(ns, r + per);
      b.seg = s;
      b.pad = 0;
      blk.push_back(b);
    }
  }
  seg_blk[nseg] = (int)blk.size();
}

// A device block schedule (see build_schedule).
struct Sched {
  DevBuf<BlkRange> blk;
  DevBuf<int> seg_blk;
  int nblk = 0;
  void build(sv_context* ctx, const std::vector<int64_t>& off, int target) {
    std::vector<BlkRange> hb;
    std::vector<int> hs;
    build_schedule(off, target, hb, hs);
    nblk = (int)hb.size();
    blk.alloc(nblk);
    seg_blk.alloc(hs.size());
    sv_h2d(ctx, blk.get(), hb.data(), nblk * sizeof(BlkRange));
    sv_h2d(ctx, seg_blk.get(), hs.data(), hs.size() * sizeof(int));
  }
};

// One side of the bidiagonalisation: two double-float bases (len x work) --
// the current one and the target of the thick-restart rotation, which swap
// roles every restart -- the double-float working vector and the FP64 copy of
// the current basis vector (the input of the next product).  Rows may stack
// several samples (offsets hoff); `red` schedules the reductions, `rows` the
// row-parallel kernels.
struct Side {
  int64_t len = 0;
  int64_t ld = 0;                // leading dimension of the bases: len rounded up to 4
                                 // rows (16-byte column strides for the tensor copies)
  int nseg = 1;
  int64_t max_seg = 0;           // longest sample
  std::vector<int64_t> hoff;     // nseg + 1 row offsets
  DevBuf<int64_t> off;
  Sched red, rows, lag;   // lag: the cell-side lagged CGS2 pass (cell side only)
  DevBuf<float> h[2], l[2];     // basis sets
  int set = 0;                  // the current set
  DevBuf<float> xh, xl;         // working vector
  DevBuf<double> cur;           // current basis vector, FP64
  void alloc(sv_context* ctx, const std::vector<int64_t>& offsets, int work, int red_target,
             int rows_target) {
    hoff = offsets;
    nseg = (int)hoff.size() - 1;
    len = hoff[nseg];
    ld = (len + 3) & ~(int64_t)3;
    for (int s = 0; s < nseg; ++s) max_seg = std::max(max_seg, hoff[s + 1] - hoff[s]);
    off.alloc(nseg + 1);
    sv_h2d(ctx, off.get(), hoff.data(), (nseg + 1) * 8);
    red.build(ctx, hoff, red_target);
    rows.build(ctx, hoff, rows_target);
    for (int t = 0; t < 2; ++t) {
      h[t].alloc(ld * work);
      l[t].alloc(ld * work);
    }
    xh.alloc(len);
    xl.alloc(len);
    cur.alloc(len);
  }
  float* bh() { return h[set].get(); }
  float* bl() { return l[set].get(); }
  float* ch(int j) { return bh() + (int64_t)j * ld; }
  float* cl(int j) { return bl() + (int64_t)j * ld; }
  float* th() { return h[1 - set].get(); }
  float* tl() { return l[1 - set].get(); }
  void flip() { set = 1 - set; }
};

// A captured Lanczos cycle: its executable graph and what one replay does.
struct CycleGraph {
  cudaGraphExec_t exec = nullptr;
  int64_t launches = 0, matvecs = 0;
};

// Per-sample outcome of a run.
struct IrlbaResult {
  std::vector<int> info;        // 0 converged, 1 not
  std::vector<int64_t> iters;   // cycles until convergence (or maxit)
  int64_t nmatvec = 0;          // operator products (each covers every active sample)
};

// The Lanczos driver.  m = rows of A (the W side), n = columns (the V side);
// with several samples A is block diagonal (sample s: W rows woff[s]..,
// V rows voff[s]..) and every sample runs its own bidiagonalisation in the
// same launches; a sample that converges is finished (U, V written) and
// frozen while the others continue.
struct Lanczos {
  sv_context* ctx;
  Op* op;
  int64_t m, n;
  int nu, work, nseg;
  Side Ws, Vs;
  DevBuf<double> ytmp, F, B, P, Q, sig, summary, scal, part, cvec, Ufin, Vfin;
  // G = A^T W (feature rows x work, double-float), two sets that follow the
  // cell-side basis sets through the restart rotations
  DevBuf<float> gh[2], gl[2];
  // scratch of the tensor-core rotation: the slices of M and their exponents
  DevBuf<unsigned char> rot_b;
  DevBuf<int> rot_f;
  DevBuf<unsigned int> counter;
  DevBuf<int> flag, active, finsel;
  double* hsum = nullptr;       // pinned copy of the cycle summaries
  int* hflags = nullptr;        // pinned staging of the active / finish masks
  double eps_b = 0;
  int cgs_blocks = RED_BLOCKS;  // resident blocks of the CGS kernels (one wave)
  bool vside_multi = false;     // feature side through the multi-block kernels
  bool lag_tma = false;         // the cell-side pass with TMA-fed basis tiles
  // graphs of the first cycle and of restart cycles from basis set 0 / set 1
  CycleGraph graphs[3];

  Lanczos(sv_context* c, Op* o, const std::vector<int64_t>& woff, const std::vector<int64_t>& voff,
          int nu_, int work_)
      : ctx(c), op(o), nu(nu_), work(work_) {
    nseg = (int)woff.size() - 1;
    m = woff[nseg];
    n = voff[nseg];
    int per_sm = 0;
    // one wave of the CGS passes (k_cgs_df; the scaling and fix kernels share
    // the schedule)
    if (work <= 64)
      SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cgs_df<8, true, true, false>, 256, 0));
    else
      SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cgs_df<12, true, true, false>, 256, 0));
    cgs_blocks = std::max(1, std::min(RED_BLOCKS, per_sm * ctx->num_sms));
    auto red_target = [&](int64_t len) {
      return (int)std::max<int64_t>(1, std::min<int64_t>(cgs_blocks, (len + 63) / 64));
    };
    // its own one-wave schedule for the cell-side lagged pass: the TMA-fed form
    // (one block per SM, its ring takes the shared memory) up to 64 basis columns
    int lag_per_sm = 0;
    lag_tma = work <= 64 && !getenv("SV_NO_LAG_TMA");
    if (lag_tma) {
      const size_t dyn = lag_smem(work - 1);
      SV_CUDA(cudaFuncSetAttribute(k_cgs_lag_tma<LR_STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
      SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&lag_per_sm, k_cgs_lag_tma<LR_STAGES>,
                                                            32 * (LR_WARPS + 1), dyn));
    } else if (work <= 64) {
      SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&lag_per_sm, k_cgs_lag<8>, 256, 0));
    } else {
      SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&lag_per_sm, k_cgs_lag<12>, 256, 0));
    }
    const int lag_blocks = std::max(1, std::min(RED_BLOCKS, lag_per_sm * ctx->num_sms));
    auto rows_target = [&](int64_t len) {
      return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->num_sms * 8, (len + 255) / 256));
    };
    Ws.alloc(ctx, woff, work, red_target(m), rows_target(m));
    Vs.alloc(ctx, voff, work, red_target(n), rows_target(n));
    Ws.lag.build(ctx, woff, (int)std::max<int64_t>(1, std::min<int64_t>(lag_blocks, (m + 63) / 64)));
    {
      const char* mode = getenv("SV_VSIDE");
      // one sample: the multi-block kernels (one 1024-thread block per step
      // measured 0.17 ms against ~0.05 ms for the five multi-block launches at
      // 3,000 features); several samples: one block per sample in one launch
      vside_multi = Vs.max_seg > 32768 || (nseg == 1 && Vs.len >= 1024);
      if (mode && strcmp(mode, "multi") == 0) vside_multi = true;
      if (mode && strcmp(mode, "block") == 0 && Vs.max_seg <= 32768) vside_multi = false;
    }
    ytmp.alloc(std::max(m, n));
    F.alloc(n);
    B.alloc((size_t)nseg * work * work);
    P.alloc((size_t)nseg * work * work);
    Q.alloc((size_t)nseg * work * work);
    sig.alloc((size_t)nseg * work);
    summary.alloc((size_t)nseg * (2 * work + 2));
    scal.alloc((size_t)nseg * (2 + 2 * CTL_N));
    int maxblk = std::max(std::max(Ws.red.nblk, Vs.red.nblk), Ws.lag.nblk);
    part.alloc((size_t)maxblk * (work + 1));
    cvec.alloc((size_t)5 * nseg * MAX_WORK);
    for (int t = 0; t < 2; ++t) {
      gh[t].alloc(n * work);
      gl[t].alloc(n * work);
    }
    rot_b.alloc(6 * 64 * 64 * 2);
    rot_f.alloc(64);
    counter.alloc(4);
    flag.alloc(nseg);
    active.alloc(nseg);
    finsel.alloc(nseg);
    Ufin.alloc(m * nu);
    Vfin.alloc(n * nu);
    sv_memset(ctx, counter.get(), 0, 16);
    sv_memset(ctx, flag.get(), 0, nseg * 4);
    sv_memset(ctx, B.get(), 0, (size_t)nseg * work * work * 8);
    SV_CUDA(cudaMallocHost((void**)&hsum, (size_t)nseg * (2 * work + 2) * 8));
    SV_CUDA(cudaMallocHost((void**)&hflags, (size_t)nseg * 4));
    op->bind_active(active.get());
    SV_CUDA(cudaFuncSetAttribute(k_jacobi_svd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 4 * MAX_WORK * MAX_WORK * 4));
    for (auto kern : {k_rotate_df<10>, k_rotate_df<16>, k_rotate_df<26>})
      SV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   MAX_WORK * (MAX_WORK / 2 + 13) * 16));
  }
  ~Lanczos() {
    for (auto& g : graphs)
      if (g.exec) cudaGraphExecDestroy(g.exec);
    if (hsum) cudaFreeHost(hsum);
    if (hflags) cudaFreeHost(hflags);
  }
  Lanczos(const Lanczos&) = delete;
  Lanczos& operator=(const Lanczos&) = delete;

  double* sS() { return scal.get(); }                      // W-side norms (alpha), per sample
  double* sR() { return scal.get() + nseg; }               // V-side norms (beta), per sample
  double* ctl() { return scal.get() + 2 * nseg; }          // cycle control blocks
  double* ctl0() { return scal.get() + 2 * nseg + CTL_N * nseg; }   // start-vector control blocks
  double* c0v() { return cvec.get() + (size_t)2 * nseg * MAX_WORK; }  // first-projection coefficients
  double* cpv() { return cvec.get() + (size_t)3 * nseg * MAX_WORK; }  // pending correction, cell side
  double* scratch() { return cvec.get() + (size_t)4 * nseg * MAX_WORK; }
  float* Gh() { return gh[Ws.set].get(); }
  float* Gl() { return gl[Ws.set].get(); }

  // working vector <- CGS2(y, basis[:, :ncols]) (y FP64; null: the working
  // vector already holds it); nrm[s] = its norm per sample
  template <int NJ>
  void orth_norm_nj(Side& s, const double* y, int ncols, double* nrm) {
    int g = s.red.nblk;
    const BlkRange* bk = s.red.blk.get();
    const int* sb = s.red.seg_blk.get();
    const int* act = active.get();
    double* c1 = cvec.get();
    double* c2 = cvec.get() + (size_t)nseg * MAX_WORK;
    double* np = part.get() + (size_t)g * work;
    if (ncols == 0) {
      if (y) to_working(s, y);
      sv_launch(ctx, "irlba_upd_norm", k_cgs_df<NJ, true, false, true>, dim3(g), dim3(256), 0,
                (const float*)s.bh(), (const float*)s.bl(), s.ld, 0, s.xh.get(), s.xl.get(),
                (const double*)nullptr, bk, sb, nseg, act, (const double*)c1, part.get(), np, c2, nrm,
                counter.get());
      return;
    }
    sv_launch(ctx, "irlba_dots", k_cgs_df<NJ, false, true, false>, dim3(g), dim3(256), 0,
              (const float*)s.bh(), (const float*)s.bl(), s.ld, ncols, s.xh.get(), s.xl.get(), y, bk, sb,
              nseg, act, (const double*)nullptr, part.get(), np, c1, (double*)nullptr, counter.get());
    sv_launch(ctx, "irlba_upd_dots", k_cgs_df<NJ, true, true, false>, dim3(g), dim3(256), 0,
              (const float*)s.bh(), (const float*)s.bl(), s.ld, ncols, s.xh.get(), s.xl.get(),
              (const double*)nullptr, bk, sb, nseg, act, (const double*)c1, part.get(), np, c2,
              (double*)nullptr, counter.get());
    sv_launch(ctx, "irlba_upd_norm", k_cgs_df<NJ, true, false, true>, dim3(g), dim3(256), 0,
              (const float*)s.bh(), (const float*)s.bl(), s.ld, ncols, s.xh.get(), s.xl.get(),
              (const double*)nullptr, bk, sb, nseg, act, (const double*)c2, part.get(), np, c1, nrm,
              counter.get());
  }
  void orth_norm(Side& s, const double* y, int ncols, double* nrm) {
    if (work <= 64) orth_norm_nj<8>(s, y, ncols, nrm);
    else orth_norm_nj<12>(s, y, ncols, nrm);
  }

  // basis column j := working vector / nrm[s] (FP64 copy in cur), breakdown
  // handling; the B entry at offset boff of each sample's B (boff < 0: none)
  void scal_fix(Side& s, int j, double* nrm, const double* c, int64_t boff, uint64_t seed,
                unsigned step) {
    sv_launch(ctx, "irlba_scal", k_scal_df, dim3(s.red.nblk), dim3(256), 0, (const float*)s.xh.get(),
              (const float*)s.xl.get(), (const BlkRange*)s.red.blk.get(), (const int*)s.red.seg_blk.get(),
              (const int64_t*)s.off.get(), (const int*)active.get(), (const double*)nrm, c, s.ch(j),
              s.cl(j), s.cur.get(), boff >= 0 ? B.get() : (double*)nullptr, boff,
              (int64_t)work * work, flag.get(), (unsigned long long)seed, step);
    sv_launch(ctx, "irlba_scal_post", k_scal_post, dim3(1), dim3(64), 0, nrm, (const int*)flag.get(),
              nseg, &s == &Ws ? cpv() : (double*)nullptr);
    sv_launch(ctx, "irlba_fix", k_fix_df, dim3(nseg), dim3(1024), 0, s.cur.get(),
              (const int64_t*)s.off.get(), (const float*)s.bh(), (const float*)s.bl(), s.ld, j, s.ch(j),
              s.cl(j), flag.get());
  }

  // the feature-side step: one block per sample (k_vside), or the multi-block
  // CGS kernels over the feature side (SV_VSIDE=multi|block forces either)
  void vside(int ncols, int write_col, double* nrm, const double* c, int64_t boff, uint64_t seed,
             unsigned step) {
    if (vside_multi) {
      orth_norm(Vs, F.get(), ncols, nrm);
      if (write_col >= 0) scal_fix(Vs, write_col, nrm, c, boff, seed, step);
      return;
    }
    sv_launch(ctx, "irlba_vside", k_vside, dim3(nseg), dim3(1024), 0, (const double*)F.get(),
              (const int64_t*)Vs.off.get(), Vs.ld, Vs.bh(), Vs.bl(), ncols, write_col, nrm, c,
              boff >= 0 ? B.get() : (double*)nullptr, boff, (int64_t)work * work, Vs.cur.get(),
              Vs.xh.get(), Vs.xl.get(), (const int*)active.get(), (unsigned long long)seed, step);
  }

  void to_working(Side& s, const double* y) {
    sv_launch(ctx, "irlba_to_df", k_to_df, dim3(sv_grid_for(ctx, s.len, 256, 4)), dim3(256), 0, y,
              s.len, s.xh.get(), s.xl.get());
  }

  // out = basis * M_s[:, :nout] per sample: into the other basis set (outd null)
  // or FP64 outd (ld = the side's length); only the samples with sel[s] != 0
  void rotate(Side& s, const double* M, int nout, double* outd, const int* sel) {
    // the cell side of one sample into the other basis set: on the tensor cores
    if (&s == &Ws && !outd && nseg == 1 && sv_rotate_tc_supported(work, nout, s.ld)) {
      sv_rotate_tc(ctx, s.bh(), s.bl(), s.ld, s.len, work, M, nout, s.th(), s.tl(), s.ld, rot_b.get(),
                   rot_f.get());
      return;
    }
    // into the other basis set (leading dimension ld) or FP64 outd (len)
    rotate_raw(s.bh(), s.bl(), s.ld, s.rows, M, nout, outd ? (float*)nullptr : s.th(),
               outd ? (float*)nullptr : s.tl(), outd, outd ? s.len : s.ld, sel);
  }
  void rotate_raw(const float* inh, const float* inl, int64_t ld_in, const Sched& rows, const double* M,
                  int nout, float* outh, float* outl, double* outd, int64_t ld_out, const int* sel) {
    // columns per pass: the fewest padded columns, then the fewest passes (at
    // 50 columns 10 per pass measured 1.65 ms per cell-side rotation at the
    // atlas size, 16 and 26 per pass 1.96 and 1.94 ms)
    int kb = 10;
    for (int c : {16, 26})
      if ((nout + c - 1) / c * c <= (nout + kb - 1) / kb * kb) kb = c;
    auto kern = kb == 26 ? k_rotate_df<26> : kb == 16 ? k_rotate_df<16> : k_rotate_df<10>;
    int npass = (nout + kb - 1) / kb;
    // a short side (the features) spreads the passes of its rows over blocks
    int gy = rows.nblk < ctx->num_sms ? npass : 1;
    sv_launch(ctx, "irlba_rotate", kern, dim3(rows.nblk, gy), dim3(256),
              (size_t)work * npass * (kb / 2) * 16, inh, inl, ld_in, (const BlkRange*)rows.blk.get(), sel,
              work, M, (int64_t)work * work, nout, outh, outl, outd, ld_out);
  }

  // The cell-side CGS2 step of column jn in one pass over the basis (k_cgs_lag):
  // first-projection coefficients from G (k_gdots), the pending column pend
  // (the previous step's, or -1) corrected on the way; y: the FP64 product, or
  // null when the product is in the working vector.  s0 = the norm per sample,
  // cp = the new column's pending correction.
  template <int NJ>
  void w_step_nj(int jn, int pend, const double* y) {
    const int g = Ws.lag.nblk;
    sv_launch(ctx, "irlba_gdots", k_gdots, dim3(jn, nseg), dim3(256), 0, (const float*)Gh(),
              (const float*)Gl(), n, (const int64_t*)Vs.off.get(), (const double*)Vs.cur.get(), pend,
              (const double*)sR(), (const double*)cpv(), (const int*)active.get(), c0v());
    if (NJ == 8 && lag_tma) {
      // the basis columns 0..jn-1 as two 2D tensors (rows x jn columns, 16-byte
      // column stride), boxes of 64 rows x 8 columns
      CUtensorMap mh, ml;
      cuuint64_t gdim[2] = {(cuuint64_t)Ws.len, (cuuint64_t)jn};
      cuuint64_t gstride[1] = {(cuuint64_t)Ws.ld * 4};
      cuuint32_t box[2] = {(cuuint32_t)LR_ROWS, (cuuint32_t)LT_GC};
      cuuint32_t estr[2] = {1, 1};
      for (int a = 0; a < 2; ++a) {
        CUresult r = sv_encode_tiled()(a ? &ml : &mh, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, a ? Ws.bl() : Ws.bh(),
                                       gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                       CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) sv_throw(SV_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
      }
      sv_launch(ctx, "irlba_cgs_lag", k_cgs_lag_tma<LR_STAGES>, dim3(g), dim3(32 * (LR_WARPS + 1)), lag_smem(jn),
                mh, ml, Ws.bh(),
                Ws.bl(), Ws.ld, jn, pend, Ws.xh.get(), Ws.xl.get(), y, (const BlkRange*)Ws.lag.blk.get(),
                (const int*)Ws.lag.seg_blk.get(), nseg, (const int*)active.get(), (const double*)c0v(),
                cpv(), part.get(), part.get() + (size_t)g * work, sS(), counter.get(), ctx->d_status);
      return;
    }
    sv_launch(ctx, "irlba_cgs_lag", k_cgs_lag<NJ>, dim3(g), dim3(256), 0, Ws.bh(), Ws.bl(), Ws.ld, jn,
              pend, Ws.xh.get(), Ws.xl.get(), y, (const BlkRange*)Ws.lag.blk.get(),
              (const int*)Ws.lag.seg_blk.get(), nseg, (const int*)active.get(), (const double*)c0v(),
              cpv(), part.get(), part.get() + (size_t)g * work, sS(), counter.get());
  }
  void w_step(int jn, int pend, const double* y) {
    if (work <= 64) w_step_nj<8>(jn, pend, y);
    else w_step_nj<12>(jn, pend, y);
  }
  // dynamic shared memory of the TMA pass over ncols columns (the ring + 1 KB
  // alignment slack)
  static size_t lag_smem(int ncols) {
    return (size_t)LR_STAGES * ((ncols + LT_GC - 1) / LT_GC) * 2 * LT_GC * LR_ROWS * 4 + 1024;
  }
  // F = A^T w' - alpha v of cell-side column jn: corrected for the pending
  // part of w', and G[:, jn] = A^T w
  void g_col(int jn) {
    sv_launch(ctx, "irlba_gcol", k_gcol, dim3(Vs.rows.nblk), dim3(256), 0, Gh(), Gl(), n,
              (const BlkRange*)Vs.rows.blk.get(), (const int*)active.get(), jn, (const double*)cpv(),
              (const double*)sS(), (const double*)Vs.cur.get(), F.get());
  }
  // the pending correction of the last cell-side column, applied in place
  template <int NJ>
  void w_settle_nj(int col) {
    const int g = Ws.red.nblk;
    sv_launch(ctx, "irlba_settle", k_cgs_df<NJ, true, false, true>, dim3(g), dim3(256), 0,
              (const float*)Ws.bh(), (const float*)Ws.bl(), Ws.ld, col, Ws.ch(col), Ws.cl(col),
              (const double*)nullptr, (const BlkRange*)Ws.red.blk.get(), (const int*)Ws.red.seg_blk.get(),
              nseg, (const int*)active.get(), (const double*)cpv(), part.get(),
              part.get() + (size_t)g * work, scratch(), scratch(), counter.get());
  }
  void w_settle(int col) {
    if (work <= 64) w_settle_nj<8>(col);
    else w_settle_nj<12>(col);
  }

  // One cycle, enqueued on the context stream without any host round trip:
  // for a restart, V <- V Q_k, W <- W P_k, V[:, k] = f/|f| and B reset; the
  // Lanczos steps k..work-1; the SVD of B; the summaries copied to hsum.
  // Samples that are no longer active are skipped by every kernel.
  // Returns the number of operator products.
  int64_t cycle(bool restart, int k, uint64_t seed) {
    double* s0 = sS();
    double* s1 = sR();
    const double* c = ctl();
    const int* act = active.get();
    int64_t nmv = 0;
    if (restart) {
      rotate(Vs, Q.get(), k, nullptr, act);
      rotate(Ws, P.get(), k, nullptr, act);
      // G follows W: A^T (W P) = G P
      rotate_raw(Gh(), Gl(), n, Vs.rows, P.get(), k, gh[1 - Ws.set].get(), gl[1 - Ws.set].get(), nullptr, n,
                 act);
      Vs.flip();
      Ws.flip();
      df_residual_to_fp64();
      dim3 grid((unsigned)std::max(1, std::min(sv_grid_for(ctx, Vs.max_seg, 256, 4), 64)), (unsigned)nseg);
      sv_launch(ctx, "irlba_restart", k_restart_tail, grid, dim3(256), 0, Vs.ch(k), Vs.cl(k),
                Vs.cur.get(), (const double*)F.get(), (const int64_t*)Vs.off.get(),
                (const double*)summary.get(), work, k, B.get(), act);
    }
    unsigned step = 1;
    int j = k;
    // W[:, j] = A V[:, j]; CGS2 against W[:, :j] (the first column of a run:
    // its norm only)
    bool pending = false;
    if (op->N_df(Vs.ch(j), Vs.cl(j), Ws.xh.get(), Ws.xl.get(), nullptr, nullptr, nullptr)) {
      if (j == 0) orth_norm(Ws, nullptr, 0, s0);
      else w_step(j, -1, nullptr);
    } else {
      op->N(Vs.cur.get(), ytmp.get(), nullptr, nullptr);
      if (j == 0) orth_norm(Ws, ytmp.get(), 0, s0);
      else w_step(j, -1, ytmp.get());
    }
    pending = j > 0;
    nmv++;
    scal_fix(Ws, j, s0, c, (int64_t)j * work + j, seed, step++);
    while (true) {
      // F = A^T W[:, j] - S V[:, j]; CGS2 against V[:, :j+1]
      op->T(Ws.cur.get(), F.get(), s0, Vs.cur.get());
      nmv++;
      g_col(j);
      if (j + 1 < work) {
        vside(j + 1, j + 1, s1, c, (int64_t)j * work + j + 1, seed, step++);
        // W[:, j+1] = A V[:, j+1] - R W[:, j]
        if (op->N_df(Vs.ch(j + 1), Vs.cl(j + 1), Ws.xh.get(), Ws.xl.get(), s1, Ws.ch(j), Ws.cl(j))) {
          w_step(j + 1, j, nullptr);
        } else {
          op->N(Vs.cur.get(), ytmp.get(), s1, Ws.cur.get());
          w_step(j + 1, j, ytmp.get());
        }
        pending = true;
        nmv++;
        scal_fix(Ws, j + 1, s0, c, (int64_t)(j + 1) * work + j + 1, seed, step++);
        ++j;
      } else {
        vside(j + 1, -1, s1, c, -1, seed, step++);   // residual f and |f|
        break;
      }
    }
    // the last cell-side column's second projection: W is complete for the
    // restart rotation and the final U
    if (pending) w_settle(j);
    sv_launch(ctx, "irlba_svd", k_jacobi_svd, dim3(nseg), dim3(1024), (size_t)4 * work * work * 4,
              (const double*)B.get(), work, P.get(), sig.get(), Q.get(), summary.get(),
              (const double*)s1, 60, ctx->d_status, ctl(), eps_b, act);
    SV_CUDA(cudaMemcpyAsync(hsum, summary.get(), (size_t)nseg * (2 * work + 2) * 8,
                            cudaMemcpyDeviceToHost, ctx->stream));
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

  // U_s = W_s P_s[:, :nu], V_s = V_s Q_s[:, :nu] (FP64) for the samples in hflags
  void finish_selected() {
    sv_h2d(ctx, finsel.get(), hflags, (size_t)nseg * 4);
    rotate(Ws, P.get(), nu, Ufin.get(), finsel.get());
    rotate(Vs, Q.get(), nu, Vfin.get(), finsel.get());
  }

  IrlbaResult run(const double* init_host, int maxit, double tol, uint64_t seed) {
    IrlbaResult res;
    res.info.assign(nseg, 1);
    res.iters.assign(nseg, maxit);
    eps_b = sqrt(2.220446049250313e-16);
    // control blocks: cycles start at threshold eps_b (smax = 0), the start
    // vector is normalised unless it is zero; every sample active
    {
      std::vector<double> ci((size_t)2 * CTL_N * nseg);
      for (int s = 0; s < nseg; ++s) {
        ci[s * CTL_N + CTL_THRESH] = eps_b;
        ci[s * CTL_N + CTL_SMAX] = 0.0;
        ci[s * CTL_N + CTL_CYCLE] = 0.0;
        ci[CTL_N * nseg + s * CTL_N + CTL_THRESH] = 1e-300;
        ci[CTL_N * nseg + s * CTL_N + CTL_SMAX] = 0.0;
        ci[CTL_N * nseg + s * CTL_N + CTL_CYCLE] = 0.0;
      }
      sv_h2d(ctx, ctl(), ci.data(), ci.size() * 8);
      for (int s = 0; s < nseg; ++s) hflags[s] = 1;
      sv_h2d(ctx, active.get(), hflags, (size_t)nseg * 4);
    }
    sv_h2d(ctx, F.get(), init_host, n * 8);
    vside(0, 0, sR(), ctl0(), -1, seed, 0);
    bool graphs_on = op->device_only() && !ctx->profiling && !getenv("SV_NO_GRAPH");
    const int kr = std::min(nu, work - 1);
    std::vector<double> smax(nseg, 0.0);
    std::vector<int> act(nseg, 1);
    int nact = nseg;
    for (int it = 0; it < maxit && nact > 0; ++it) {
      res.nmatvec += enqueue_cycle(it > 0, it > 0 ? kr : 0, seed, graphs_on);
      sv_sync(ctx);
      bool any = false;
      for (int s = 0; s < nseg; ++s) {
        hflags[s] = 0;
        if (!act[s]) continue;
        const double* hs = hsum + (size_t)s * (2 * work + 2);
        double rf = hs[2 * work];
        smax[s] = std::max(smax[s], hs[0]);
        int nconv = 0;
        for (int i = 0; i < nu; ++i)
          if (fabs(rf * hs[work + i]) < tol * smax[s]) ++nconv;
        if (nconv >= nu || rf < eps_b * smax[s]) {
          res.info[s] = 0;
          res.iters[s] = it + 1;
          act[s] = 0;
          hflags[s] = 1;
          --nact;
          any = true;
        }
      }
      if (any) {
        // finish the converged samples now: the next restart skips them
        finish_selected();
        for (int s = 0; s < nseg; ++s) hflags[s] = act[s];
        sv_h2d(ctx, active.get(), hflags, (size_t)nseg * 4);
        sv_sync(ctx);
      }
    }
    if (nact > 0) {
      for (int s = 0; s < nseg; ++s) hflags[s] = act[s];
      finish_selected();
      sv_sync(ctx);
    }
    sv_check_device_status(ctx, "irlba");
    return res;
  }

  // F holds the residual in FP64 only before the first CGS pass; the orthogonalised
  // residual lives in the V-side working vector: bring it back to FP64
  void df_residual_to_fp64() {
    sv_launch(ctx, "irlba_f_fp64", k_df_to_fp64, dim3(sv_grid_for(ctx, n, 256, 4)), dim3(256), 0,
              (const float*)Vs.xh.get(), (const float*)Vs.xl.get(), n, F.get());
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

// irlba over nseg stacked samples (one sample: woff = {0, m}, voff = {0, n}).
// s_out: nseg x nu, U: m x nu, V: n x nu (column-major, stacked rows); emb
// (optional) receives Z = U diag(s) and s.  Returns the number of samples that
// did not converge; iters (nseg) and nmatvec as in the reference.
static int irlba_core(sv_context* ctx, Op* op, const std::vector<int64_t>& woff,
                      const std::vector<int64_t>& voff, int64_t nu, int64_t work, int64_t maxit,
                      double tol, const double* init, uint64_t seed, double* s_out, double* U,
                      double* V, int64_t* iters, int64_t* nmatvec, sv_embed* emb) {
  int nseg = (int)woff.size() - 1;
  int64_t m = woff[nseg], n = voff[nseg];
  int64_t mmin = m, nmin = n;
  for (int s = 0; s < nseg; ++s) {
    mmin = std::min(mmin, woff[s + 1] - woff[s]);
    nmin = std::min(nmin, voff[s + 1] - voff[s]);
  }
  SV_REQUIRE(nu >= 1 && nu <= std::min(mmin, nmin), "nu must be in 1..min(m, n)");
  if (work <= 0) work = default_work(mmin, nmin, nu);
  SV_REQUIRE(work > nu || work == std::min(mmin, nmin), "work must exceed nu (or equal min(m, n))");
  SV_REQUIRE(work <= std::min(mmin, nmin), "work exceeds min(m, n)");
  if (work > MAX_WORK) sv_throw(SV_ERR_UNSUPPORTED, "work %lld exceeds %d", (long long)work, MAX_WORK);
  SV_REQUIRE(maxit >= 1, "maxit must be >= 1");
  SV_REQUIRE(init != nullptr, "init (length n) is required");
  Lanczos L(ctx, op, woff, voff, (int)nu, (int)work);
  IrlbaResult r = L.run(init, (int)maxit, tol, seed);
  if (s_out)
    SV_CUDA(cudaMemcpy2DAsync(s_out, nu * 8, L.sig.get(), work * 8, nu * 8, nseg, cudaMemcpyDeviceToHost,
                              ctx->stream));
  if (U) sv_d2h(ctx, U, L.Ufin.get(), m * nu * 8);
  if (V) sv_d2h(ctx, V, L.Vfin.get(), n * nu * 8);
  if (emb) {
    emb->s.alloc((size_t)nseg * nu);
    SV_CUDA(cudaMemcpy2DAsync(emb->s.get(), nu * 8, L.sig.get(), work * 8, nu * 8, nseg,
                              cudaMemcpyDeviceToDevice, ctx->stream));
    emb->Z = std::move(L.Ufin);
    dim3 grid((unsigned)sv_grid_for(ctx, (m / nseg + 1) * nu, 256, 8), (unsigned)nseg);
    sv_launch(ctx, "pca_scale", k_scale_cols, grid, dim3(256), 0, emb->Z.get(), m,
              (const int64_t*)L.Ws.off.get(), (int)nu, (const double*)emb->s.get(), (int)nu);
  }
  sv_sync(ctx);
  if (iters)
    for (int s = 0; s < nseg; ++s) iters[s] = r.iters[s];
  if (nmatvec) *nmatvec = r.nmatvec;
  int bad = 0;
  for (int s = 0; s < nseg; ++s) bad += r.info[s] != 0;
  return bad;
}

SV_API int sv_irlba(sv_context* ctx, const sv_centered* s, int64_t nu, int64_t work, int64_t maxit,
                    double tol, const double* init, uint64_t seed, double* s_out, double* U,
                    double* V, int64_t* iters, int64_t* nmatvec) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(s && s->ctx == ctx, "bad centered handle");
  CenteredOp op(ctx, s);
  int info = irlba_core(ctx, &op, {0, s->n_cells}, {0, s->nf}, nu, work, maxit, tol, init, seed, s_out,
                        U, V, iters, nmatvec, nullptr);
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
    int info = irlba_core(ctx, &op, {0, s->n_cells}, {0, s->nf}, k, 0, maxit, tol, init, seed,
                          sv.data(), nullptr, loadings, iters, nmatvec, e);
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

// embedding(X, npcs; method=:pca, algorithm=:irlba) for every sample of a batch
// (src/embedding.jl:46-76 per sample), all samples in the same launches.
// Z: n_cells x npcs column-major (the samples' rows stacked), stdev: nseg x
// npcs (sample-major), iters: nseg cycles until convergence.  init is the start
// vector (nf) used for every sample.
SV_API int sv_batch_pca(sv_context* ctx, const sv_batch* b, int64_t npcs, int64_t maxit, double tol,
                        const double* init, uint64_t seed, sv_embed** out, double* Z, double* stdev,
                        int64_t* iters, int64_t* nmatvec) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(b && b->ctx == ctx, "bad batch handle");
  SV_REQUIRE(npcs >= 1, "npcs must be >= 1");
  SV_REQUIRE(init != nullptr, "init (length nf) is required");
  int64_t minc = b->n_cells;
  for (int64_t s = 0; s < b->nseg; ++s) minc = std::min(minc, b->hoff[s + 1] - b->hoff[s]);
  int64_t k = std::min(std::min(minc, b->nf), npcs);
  if (k > 0.5 * std::min(minc, b->nf))
    sv_throw(SV_ERR_UNSUPPORTED,
             "npcs > 0.5 min(m, n) for a sample: the reference switches to a dense svd (embedding.jl:50-53)");
  std::vector<int64_t> voff(b->nseg + 1);
  for (int64_t s = 0; s <= b->nseg; ++s) voff[s] = s * b->nf;
  std::vector<double> init_all((size_t)b->nseg * b->nf);
  for (int64_t s = 0; s < b->nseg; ++s) std::copy(init, init + b->nf, init_all.begin() + s * b->nf);
  BatchOp op(ctx, b);
  auto* e = new sv_embed();
  try {
    e->ctx = ctx;
    e->n_cells = b->n_cells;
    e->npcs = k;
    e->nf = b->nf;
    std::vector<double> sv((size_t)b->nseg * k);
    int bad = irlba_core(ctx, &op, b->hoff, voff, k, 0, maxit, tol, init_all.data(), seed, sv.data(),
                         nullptr, nullptr, iters, nmatvec, e);
    if (Z) sv_d2h(ctx, Z, e->Z.get(), b->n_cells * k * 8);
    if (stdev)
      for (int64_t s = 0; s < b->nseg; ++s) {
        double m1 = (double)std::max<int64_t>(1, b->hoff[s + 1] - b->hoff[s] - 1);
        for (int64_t i = 0; i < k; ++i) stdev[s * k + i] = sv[s * k + i] / sqrt(m1);   // embedding.jl:68
      }
    if (bad) {
      delete e;
      sv_set_error("convergence failed for %d of %lld samples", bad, (long long)b->nseg);
      return SV_ERR_NOCONV;
    }
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
  int info = irlba_core(ctx, &op, {0, m}, {0, n}, nu, work, maxit, tol, init, 0x5EEDull, s, U, V, nullptr,
                        nullptr, nullptr);
  return info == 0 ? 0 : 1;
  SV_CATCH
}
