// scale_features and the CenteredMatrix products (src/scaling.jl:18-44,199-357).
//
// Nothing is densified and no scaled copy is written: the products read the
// normalised values and apply, per element,
//     b = min(a * inv_std_f, clip_f)        clip_f = scale_max + mean_f/std_f
// and the centring as a rank-1 correction:
//     Xs v   = B v  - (mu . v) 1                 (scaling.jl:245-250)
//     Xs^T u = B^T u - (sum u) mu                (scaling.jl:252-257)
//
// Layout in HBM:
//   * the feature (HVF) subset of the CSC copy is a view: per feature its
//     [start, end) range in the full CSC arrays; X^T u walks those ranges in
//     fixed-size chunks (a chunk table built once), one warp per chunk;
//   * X v uses a cell-major copy of the subset (CSR_h): rowptr int64, feature
//     index uint16 (int32 when there are more than 65536 features), value in the
//     data's storage type.  One warp per cell; the per-feature (inv*x, clip*x)
//     pairs are staged in shared memory.
// Algorithmic bytes per product: CSR_h nnz_h*(idx + v) + 8*(n_cells+1) +
// 8*n_cells (y) ; CSC nnz_h*(4 + v) + 4*n_cells (u, FP32) + chunk table.
#include "sv_internal.cuh"

namespace {

constexpr int64_t CHUNK = 4096;   // non-zeros per warp task in the X^T u product

// ---- per-feature moments -----------------------------------------------------
// Mean and unbiased variance of each feature column including its implicit
// zeros (scaling.jl:18-34).  The reference runs Welford over the stored values
// from the state after the n - nnz zeros; here the same two numbers come from
// the sums S1 = sum a and S2 = sum a^2 over the stored values (the zeros add
// nothing): mean = S1 / n, M2 = S2 - S1 * mean, var = M2 / (n - 1).  No
// division per element: the FP64 pipe of this GPU runs at 1/64 of the FP32
// rate, and the former Welford form (one FP64 divide per element) ran at ~1%
// of HBM bandwidth.
//
// FP32 / BF16 values are summed on the FP32 pipe in double-float form (a
// rounded sum and its exact error, Knuth's TwoSum; x^2 exact for BF16, with
// its FMA error term for FP32) over groups of up to 32 elements per thread,
// and each group's (hi, lo) pairs are added into FP64 sums: relative error of
// the sums ~2^-48 per group, of M2 ~2^-47 (1 + mean^2 / var) (3.9e-14 at
// worst on the FP32 test data, 4e-15 for BF16, against FP64 Welford).  FP64
// and Int32 data are summed in FP64.
//
// Work split: each column is cut into parts of at most MOM_PART entries, one
// warp task each (a device-built task table: per column its range and the
// offset of its first task), so dense features form no tail and short ones
// cost one short task; the per-task sums go to `part` and k_moments_finish
// adds a column's parts in order, so the result does not depend on
// scheduling.  With stacked samples (soff: nseg + 1 cell offsets) every
// (sample, feature) pair is a column of its own (the sample's rows of the
// feature, found by binary search in the sorted CSC rows); outputs at index
// s * nf + f.
__device__ __forceinline__ int64_t lower_bound_rows(const int32_t* __restrict__ r, int64_t lo,
                                                    int64_t hi, int64_t key) {
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if ((int64_t)r[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// exact s + e = a + b (TwoSum; explicit roundings so that nothing is contracted)
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

struct DfAcc {
  float h1 = 0.f, l1 = 0.f, h2 = 0.f, l2 = 0.f;
  template <bool EXACT_SQ>
  __device__ __forceinline__ void add(float x) {
    float s, e;
    two_sum_f(h1, x, s, e);
    h1 = s;
    l1 = __fadd_rn(l1, e);
    float p = __fmul_rn(x, x);
    if (!EXACT_SQ) l2 = __fadd_rn(l2, __fmaf_rn(x, x, -p));
    two_sum_f(h2, p, s, e);
    h2 = s;
    l2 = __fadd_rn(l2, e);
  }
  __device__ __forceinline__ void flush(double& S1, double& S2) {
    S1 += (double)h1;
    S1 += (double)l1;
    S2 += (double)h2;
    S2 += (double)l2;
    h1 = l1 = h2 = l2 = 0.f;
  }
};

// the 16-byte vector of each storage type and how its elements are summed
template <typename ValT> struct MomVec;
template <> struct MomVec<__nv_bfloat16> {
  static constexpr int N = 8;
  static __device__ __forceinline__ void add(const uint4& w, DfAcc& acc, double&, double&) {
    const uint32_t u[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      acc.add<true>(__uint_as_float(u[i] << 16));          // low half: the earlier element
      acc.add<true>(__uint_as_float(u[i] & 0xffff0000u));
    }
  }
  static __device__ __forceinline__ void scalar(const __nv_bfloat16* p, int64_t i, DfAcc& acc,
                                                double&, double&) {
    acc.add<true>(__bfloat162float(p[i]));
  }
  static constexpr bool DF = true;
};
template <> struct MomVec<float> {
  static constexpr int N = 4;
  static __device__ __forceinline__ void add(const uint4& w, DfAcc& acc, double&, double&) {
    acc.add<false>(__uint_as_float(w.x));
    acc.add<false>(__uint_as_float(w.y));
    acc.add<false>(__uint_as_float(w.z));
    acc.add<false>(__uint_as_float(w.w));
  }
  static __device__ __forceinline__ void scalar(const float* p, int64_t i, DfAcc& acc, double&,
                                                double&) {
    acc.add<false>(p[i]);
  }
  static constexpr bool DF = true;
};
template <> struct MomVec<double> {
  static constexpr int N = 2;
  static __device__ __forceinline__ void add(const uint4& w, DfAcc&, double& S1, double& S2) {
    double a = __hiloint2double((int)w.y, (int)w.x), b = __hiloint2double((int)w.w, (int)w.z);
    S1 += a;
    S2 = fma(a, a, S2);
    S1 += b;
    S2 = fma(b, b, S2);
  }
  static __device__ __forceinline__ void scalar(const double* p, int64_t i, DfAcc&, double& S1,
                                                double& S2) {
    double a = p[i];
    S1 += a;
    S2 = fma(a, a, S2);
  }
  static constexpr bool DF = false;
};
template <> struct MomVec<int32_t> {
  static constexpr int N = 4;
  static __device__ __forceinline__ void add(const uint4& w, DfAcc&, double& S1, double& S2) {
    const int32_t u[4] = {(int32_t)w.x, (int32_t)w.y, (int32_t)w.z, (int32_t)w.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      double a = (double)u[i];
      S1 += a;
      S2 = fma(a, a, S2);
    }
  }
  static __device__ __forceinline__ void scalar(const int32_t* p, int64_t i, DfAcc&, double& S1,
                                                double& S2) {
    double a = (double)p[i];
    S1 += a;
    S2 = fma(a, a, S2);
  }
  static constexpr bool DF = false;
};

constexpr int MOM_THREADS = 256;
constexpr int MOM_UNROLL = 4;     // 16-byte loads in flight per lane (one group)
constexpr int64_t MOM_PART = 16384;

// per column (s * nf + f): its range and its number of parts
__global__ void k_moments_tasks(const int64_t* __restrict__ fstart, const int64_t* __restrict__ fend,
                                int64_t nf, const int32_t* __restrict__ rowidx,
                                const int64_t* __restrict__ soff, int nseg,
                                int64_t* __restrict__ cs, int64_t* __restrict__ ce,
                                int64_t* __restrict__ nparts) {
  for (int64_t col = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; col < nf * nseg;
       col += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = col % nf;
    const int sg = (int)(col / nf);
    int64_t s = fstart[f], e = fend[f];
    if (soff) {
      const int64_t lo = lower_bound_rows(rowidx, s, e, soff[sg]);
      e = lower_bound_rows(rowidx, lo, e, soff[sg + 1]);
      s = lo;
    }
    cs[col] = s;
    ce[col] = e;
    nparts[col] = e - s > MOM_PART ? (e - s + MOM_PART - 1) / MOM_PART : 1;
  }
}

// one warp per task: the sums of one part of a column
template <typename ValT>
__global__ void __launch_bounds__(MOM_THREADS)
k_moments_part(const ValT* __restrict__ val, const int64_t* __restrict__ cs,
               const int64_t* __restrict__ ce, const int64_t* __restrict__ toff, int64_t ncol,
               double2* __restrict__ part) {
  using V = MomVec<ValT>;
  constexpr int N = V::N;
  const int lane = threadIdx.x & 31;
  const int64_t ntask = toff[ncol];
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t task = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; task < ntask;
       task += nw) {
    // the column of this task: the last col with toff[col] <= task
    int64_t lo = 0, hi = ncol;
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (toff[mid] <= task) lo = mid;
      else hi = mid;
    }
    const int64_t col = lo;
    const int64_t P = toff[col + 1] - toff[col], p = task - toff[col];
    const int64_t s = cs[col], L = ce[col] - s;
    const int64_t a = s + L * p / P, b = s + L * (p + 1) / P;
    double S1 = 0.0, S2 = 0.0;
    DfAcc acc;
    const int64_t va = (a + N - 1) / N, vb = b / N;   // whole 16-byte vectors in [a, b)
    if (va < vb) {
      // head [a, va*N) and tail [vb*N, b): fewer than N elements each
      if (lane < va * N - a) V::scalar(val, a + lane, acc, S1, S2);
      if (lane < b - vb * N) V::scalar(val, vb * N + lane, acc, S1, S2);
      const uint4* vp = reinterpret_cast<const uint4*>(val);
      for (int64_t v0 = va + lane; v0 < vb; v0 += 32 * MOM_UNROLL) {
        uint4 w[MOM_UNROLL];
#pragma unroll
        for (int u = 0; u < MOM_UNROLL; ++u) {
          const int64_t v = v0 + 32 * u;
          if (v < vb) w[u] = __ldg(vp + v);
        }
#pragma unroll
        for (int u = 0; u < MOM_UNROLL; ++u)
          if (v0 + 32 * u < vb) V::add(w[u], acc, S1, S2);
        if (V::DF) acc.flush(S1, S2);
      }
    } else {
      for (int64_t i = a + lane; i < b; i += 32) V::scalar(val, i, acc, S1, S2);
    }
    if (V::DF) acc.flush(S1, S2);
    S1 = sv_warp_sum(S1);
    S2 = sv_warp_sum(S2);
    if (lane == 0) part[task] = make_double2(S1, S2);
  }
}

__global__ void k_moments_finish(const double2* __restrict__ part, const int64_t* __restrict__ toff,
                                 int64_t nf, int nseg, const int64_t* __restrict__ soff, int64_t n_cells,
                                 double scale_max, double* __restrict__ mean_o,
                                 double* __restrict__ std_o, double* __restrict__ mu_o,
                                 float* __restrict__ inv_f, float* __restrict__ clip_f,
                                 double* __restrict__ inv_d, double* __restrict__ clip_d) {
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < nf * nseg;
       o += (int64_t)gridDim.x * blockDim.x) {
    double S1 = 0.0, S2 = 0.0;
    for (int64_t t = toff[o]; t < toff[o + 1]; ++t) {
      const double2 q = part[t];
      S1 += q.x;
      S2 += q.y;
    }
    const int sg = (int)(o / nf);
    const double n = soff ? (double)(soff[sg + 1] - soff[sg]) : (double)n_cells;
    const double meanv = S1 / n;
    const double M2 = fmax(fma(-S1, meanv, S2), 0.0);
    const double var = M2 / (n - 1.0);
    const double sd = sqrt(var);
    const double mu = meanv / sd;                   // scaling.jl:207
    mean_o[o] = meanv;
    std_o[o] = sd;
    mu_o[o] = mu;
    inv_d[o] = 1.0 / sd;                            // a * (1/std): within 1 ulp of a/std
    clip_d[o] = scale_max + mu;                     // scaling.jl:209
    inv_f[o] = (float)(1.0 / sd);
    clip_f[o] = (float)(scale_max + mu);
  }
}

// Per-column moments of a feature set (or of every (sample, feature) pair):
// the two launches above with their partial-sum buffer.
template <typename VT>
void launch_moments(sv_context* ctx, const char* name, const VT* val, const int64_t* fs,
                    const int64_t* fe, int64_t nf, int64_t n_cells, double scale_max, double* mean,
                    double* sd, double* mu, float* invf, float* clipf, double* invd, double* clipd,
                    int64_t nnz_bound, const int32_t* rowidx = nullptr, const int64_t* soff = nullptr,
                    int nseg = 1) {
  const int64_t ncol = nf * nseg;
  DevBuf<int64_t> cs(ncol), ce(ncol), np(ncol + 1), toff(ncol + 1);
  sv_launch(ctx, "moments_tasks", k_moments_tasks, dim3(sv_grid_for(ctx, ncol, 256)), dim3(256), 0,
            fs, fe, nf, rowidx, soff, nseg, cs.get(), ce.get(), np.get());
  sv_scan_i64(ctx, np.get(), toff.get(), ncol);
  // tasks: one per column plus one per MOM_PART entries (the columns hold at
  // most nnz_bound entries together)
  const int64_t tasks_max = ncol + nnz_bound / MOM_PART + 1;
  DevBuf<double2> part((size_t)tasks_max);
  int per_sm = 0;
  SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_moments_part<VT>, MOM_THREADS, 0));
  sv_launch(ctx, name, k_moments_part<VT>,
            dim3(sv_grid_for(ctx, tasks_max * 32, MOM_THREADS, std::max(per_sm, 1))), dim3(MOM_THREADS), 0,
            val, (const int64_t*)cs.get(), (const int64_t*)ce.get(), (const int64_t*)toff.get(), ncol,
            part.get());
  sv_launch(ctx, "moments_finish", k_moments_finish, dim3(sv_grid_for(ctx, ncol, 256)), dim3(256), 0,
            (const double2*)part.get(), (const int64_t*)toff.get(), nf, nseg, soff, n_cells, scale_max,
            mean, sd, mu, invf, clipf, invd, clipd);
  sv_sync(ctx);
}

__global__ void k_feat_ranges(const int32_t* __restrict__ fgene, const int64_t* __restrict__ colptr,
                              int64_t nf, int64_t* __restrict__ fs, int64_t* __restrict__ fe,
                              int32_t* __restrict__ gene_map) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
       f += (int64_t)gridDim.x * blockDim.x) {
    int32_t g = fgene[f];
    fs[f] = colptr[g];
    fe[f] = colptr[g + 1];
    gene_map[g] = (int32_t)f;
  }
}

// ---- CSR_h construction ------------------------------------------------------
__global__ void k_hsub_count(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                             int64_t n_rows, const int32_t* __restrict__ gene_map,
                             int64_t* __restrict__ cnt) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n_rows; r += nwarps) {
    int64_t s = rowptr[r], e = rowptr[r + 1];
    int64_t c = 0;
    for (int64_t i = s + lane; i < e; i += 32) c += __ldg(gene_map + col[i]) >= 0;
    c = sv_warp_sum(c);
    if (lane == 0) cnt[r] = c;
  }
}

template <typename ValT, typename IdxT>
__global__ void k_hsub_write(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                             const ValT* __restrict__ val, int64_t n_rows,
                             const int32_t* __restrict__ gene_map, const int64_t* __restrict__ hrowptr,
                             IdxT* __restrict__ hcol, ValT* __restrict__ hval) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n_rows; r += nwarps) {
    int64_t s = rowptr[r], e = rowptr[r + 1];
    int64_t pos = hrowptr[r];
    for (int64_t i0 = s; i0 < e; i0 += 32) {
      int64_t i = i0 + lane;
      int32_t f = i < e ? __ldg(gene_map + col[i]) : -1;
      unsigned m = __ballot_sync(0xffffffffu, f >= 0);
      if (f >= 0) {
        int64_t p = pos + __popc(m & ((1u << lane) - 1));
        hcol[p] = (IdxT)f;
        hval[p] = val[i];
      }
      pos += __popc(m);
    }
  }
}

// ---- bank-aware order of the product copies --------------------------------------
// The product kernels read a segment (a CSR_h row, or a (row block, feature)
// run of the row-blocked copy) in groups of 32 EPL entries, lane l taking
// entries EPL l .. EPL l + EPL - 1 of the group (from the segment start rounded
// down to EPL; EPL = 8 for the BF16 X v loop, 4 otherwise); for each t the 32
// lanes then gather from a shared-memory table: 8-byte entries per feature for
// X v (bank pair f mod 16), 4-byte entries per row for X^T u (bank row mod 32).
// With sorted indices the gathers serialise on bank conflicts (ncu: ~4 extra
// wavefronts per gather).  So each segment is permuted such that slot p
// (relative to the rounded start) holds an index of class
// c(p) = ((p / EPL) + (NC / EPL) (p mod EPL)) mod NC where possible (NC = 16 or
// 32 classes): the 32 slots of a gather then hold each class 32/NC times.
// Entries of class c fill the c-slots in order of appearance; the surplus of
// over-full classes fills the slots left empty, in slot order.  The segment's
// sum is then taken in another order (a different, equally valid rounding).
// Applied to the CSR_h rows (X v: 1.61 -> 1.52 ms per product at the atlas
// size, for ~16 ms once per scale_features); for the row-blocked runs (NC = 32)
// the product gained 1% and the reordering cost more than it saved.
constexpr int BO_EMPTY = 1024;   // most empty slots a segment may have to be reordered
constexpr int BO_WARPS = 8;
constexpr int XV_EPL16 = 8;      // entries per lane and group of the BF16 X v loop

template <int NC, int EPL>
__device__ __forceinline__ int bo_class(int64_t p) {
  return (int)(((p / EPL) + (NC / EPL) * (p % EPL)) & (NC - 1));
}
// The slots of class c repeat with period EPL NC: EPL of them per period, at
// the offsets EPL ((c - (NC/EPL) t) mod NC) + t (t < EPL).  The kernel keeps
// per class the sorted offsets (the idx-th slot of the class) and, for every
// position x within a period, the number of the class's offsets below x (the
// slots before a position), so that both are table lookups.
// One warp per segment, three passes (class counts; the empty slots; ranks and
// placement), the result written to a second copy (segments with more than
// BO_EMPTY empty slots are copied unchanged).
template <int NC, int EPL, typename VT>
__global__ void __launch_bounds__(BO_WARPS * 32) k_bankorder(const int64_t* __restrict__ ptr,
                                                             int64_t nseg,
                                                             const uint16_t* __restrict__ icol,
                                                             const VT* __restrict__ ival,
                                                             uint16_t* __restrict__ ocol,
                                                             VT* __restrict__ oval) {
  constexpr int PER = EPL * NC;
  __shared__ uint16_t sempty[BO_WARPS][BO_EMPTY];
  __shared__ int cnt[BO_WARPS][NC], run[BO_WARPS][NC];
  __shared__ uint8_t soff[NC][EPL], sbelow[NC][PER + 1];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  for (int i = threadIdx.x; i < NC * (PER + 1); i += blockDim.x) {
    const int c = i / (PER + 1), x = i % (PER + 1);
    int k = 0;
#pragma unroll
    for (int t = 0; t < EPL; ++t) k += (EPL * ((c - (NC / EPL) * t) & (NC - 1)) + t) < x;
    sbelow[c][x] = (uint8_t)k;
  }
  for (int c = threadIdx.x; c < NC; c += blockDim.x) {
    int o[EPL];
#pragma unroll
    for (int t = 0; t < EPL; ++t) o[t] = EPL * ((c - (NC / EPL) * t) & (NC - 1)) + t;
    for (int i = 1; i < EPL; ++i)
      for (int j = i; j > 0 && o[j - 1] > o[j]; --j) {
        const int tmp = o[j];
        o[j] = o[j - 1];
        o[j - 1] = tmp;
      }
    for (int t = 0; t < EPL; ++t) soff[c][t] = (uint8_t)o[t];
  }
  __syncthreads();
  // slots of class c before position X; the idx-th slot of class c
  auto bo_count = [&](int c, int64_t X) -> int64_t { return EPL * (X / PER) + sbelow[c][X % PER]; };
  auto bo_slot = [&](int c, int64_t idx) -> int64_t { return (int64_t)PER * (idx / EPL) + soff[c][idx % EPL]; };
  for (int64_t r = (int64_t)blockIdx.x * BO_WARPS + w; r < nseg; r += (int64_t)gridDim.x * BO_WARPS) {
    const int64_t s = ptr[r], e = ptr[r + 1];
    const int64_t L = e - s;
    if (L <= 0) continue;
    const int64_t P0 = s & (EPL - 1), P1 = P0 + L;
    if (lane < NC) {
      cnt[w][lane] = 0;
      run[w][lane] = 0;
    }
    __syncwarp();
    // pass 1: entries per class
    for (int64_t i0 = 0; i0 < L; i0 += 32) {
      int64_t i = i0 + lane;
      int c = i < L ? (icol[s + i] & (NC - 1)) : NC + lane;
      unsigned same = __match_any_sync(0xffffffffu, c);
      if (i < L && (same & lt) == 0) cnt[w][c] += __popc(same);
      __syncwarp();
    }
    // pass 2: empty slots (classes with fewer entries than slots), in slot order
    int64_t nempty = 0;
    for (int64_t p0 = P0; p0 < P1; p0 += 32) {
      int64_t p = p0 + lane;
      bool emp = false;
      if (p < P1) {
        int c = bo_class<NC, EPL>(p);
        emp = bo_count(c, p) - bo_count(c, P0) >= cnt[w][c];
      }
      unsigned m = __ballot_sync(0xffffffffu, emp);
      int64_t at = nempty + __popc(m & lt);
      if (emp && at < BO_EMPTY) sempty[w][at] = (uint16_t)(p - P0);
      nempty += __popc(m);
    }
    __syncwarp();
    if (nempty > BO_EMPTY || L > 65535) {
      for (int64_t i = lane; i < L; i += 32) {
        ocol[s + i] = icol[s + i];
        oval[s + i] = ival[s + i];
      }
      continue;
    }
    // surplus entries of the classes before c (prefix over the classes)
    int sur = 0;
    if (lane < NC) {
      int64_t slots = bo_count(lane, P1) - bo_count(lane, P0);
      sur = (int)max((int64_t)0, (int64_t)cnt[w][lane] - slots);
    }
    int incl = sur;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int excl = incl - sur;
    // pass 3: rank within the class (order of appearance) and placement
    for (int64_t i0 = 0; i0 < L; i0 += 32) {
      int64_t i = i0 + lane;
      bool v = i < L;
      uint16_t f = v ? icol[s + i] : 0;
      int c = v ? (f & (NC - 1)) : NC + lane;
      unsigned same = __match_any_sync(0xffffffffu, c);
      int base_c = v ? run[w][c] : 0;
      int pre = __shfl_sync(0xffffffffu, excl, c & (NC - 1));
      __syncwarp();
      if (v) {
        int rk = base_c + __popc(same & lt);
        if ((same & lt) == 0) run[w][c] = base_c + __popc(same);
        int64_t slots = bo_count(c, P1) - bo_count(c, P0);
        int64_t q = rk < slots ? bo_slot(c, bo_count(c, P0) + rk) - P0
                               : (int64_t)sempty[w][pre + (rk - slots)];
        ocol[s + q] = f;
        oval[s + q] = ival[s + i];
      }
      __syncwarp();
    }
  }
}

// ---- vector loads of 4 consecutive elements (allocation padded) -------------
__device__ __forceinline__ void ld4(const uint16_t* p, int64_t g, int (&o)[4]) {
  uint2 w = __ldg((const uint2*)(p + g));
  o[0] = w.x & 0xffff;
  o[1] = w.x >> 16;
  o[2] = w.y & 0xffff;
  o[3] = w.y >> 16;
}
__device__ __forceinline__ void ld4(const int32_t* p, int64_t g, int (&o)[4]) {
  int4 w = __ldg((const int4*)(p + g));
  o[0] = w.x;
  o[1] = w.y;
  o[2] = w.z;
  o[3] = w.w;
}
__device__ __forceinline__ void ld4v(const __nv_bfloat16* p, int64_t g, float (&o)[4]) {
  uint2 w = __ldg((const uint2*)(p + g));
  o[0] = __uint_as_float(w.x << 16);
  o[1] = __uint_as_float(w.x & 0xffff0000u);
  o[2] = __uint_as_float(w.y << 16);
  o[3] = __uint_as_float(w.y & 0xffff0000u);
}
__device__ __forceinline__ void ld4v(const float* p, int64_t g, float (&o)[4]) {
  float4 w = __ldg((const float4*)(p + g));
  o[0] = w.x;
  o[1] = w.y;
  o[2] = w.z;
  o[3] = w.w;
}
__device__ __forceinline__ void ld4v(const double* p, int64_t g, double (&o)[4]) {
  double2 a = __ldg((const double2*)(p + g));
  double2 b = __ldg((const double2*)(p + g + 2));
  o[0] = a.x;
  o[1] = a.y;
  o[2] = b.x;
  o[3] = b.y;
}

template <typename ValT>
struct AccOf {
  typedef float type;
};
template <>
struct AccOf<double> {
  typedef double type;
};

// ---- X v over CSR_h ------------------------------------------------------------
// y = alpha * (B x - (mu . x)) + beta * y - (csub ? *csub : 0) * z
// Per-feature table in shared memory.  FP32 form: (P, Q) = (inv*x, clip*x); the
// product term is min(a*P, Q) for x >= 0 and max(a*P, Q) for x < 0 (= min(a*inv,
// clip)*x).  FP64 form: (1/std, clip, x); a * (1/std) is within one ulp of the
// reference's a/std (FP64 division is slow on this part).
// Every block builds the table and mu.x itself from x (a separate one-block
// kernel preparing the table for all blocks measured no faster).
template <typename ValT, typename IdxT>
__global__ void __launch_bounds__(256) k_spmv_csr(
    const int64_t* __restrict__ rowptr, const IdxT* __restrict__ hcol, const ValT* __restrict__ hval,
    int64_t n_rows, int64_t nf, const double* __restrict__ x, const float* __restrict__ inv_f,
    const float* __restrict__ clip_f, const double* __restrict__ inv_d,
    const double* __restrict__ clip_d, const double* __restrict__ mu, double alpha, double beta,
    double* __restrict__ y, const double* __restrict__ csub, const double* __restrict__ z) {
  typedef typename AccOf<ValT>::type AccT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32];
  double mux = 0;
  {
    for (int64_t f = threadIdx.x; f < nf; f += blockDim.x) {
      double xf = x[f];
      if constexpr (sizeof(AccT) == 4) {
        float xs = (float)xf;
        float P = inv_f[f] * xs;
        float Q = xs == 0.f ? 0.f : clip_f[f] * xs;
        ((float2*)smem_raw)[f] = make_float2(P, Q);
      } else {
        double* tab = (double*)smem_raw;
        tab[3 * f] = inv_d[f];
        tab[3 * f + 1] = clip_d[f];
        tab[3 * f + 2] = xf;
      }
      mux += mu[f] * xf;
    }
    mux = sv_warp_sum(mux);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mux;
    __syncthreads();
    if (threadIdx.x < 32) {
      double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
      v = sv_warp_sum(v);
      if (threadIdx.x == 0) red[0] = v;
    }
    __syncthreads();
    mux = red[0];
  }
  double cs = csub ? *csub : 0.0;

  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n_rows; r += nwarps) {
    int64_t s = rowptr[r], e = rowptr[r + 1];
    int64_t a0 = s & ~3ll;
    AccT acc = 0;
    // two 4-element groups per lane in flight; the first load pair is
    // unconditional (a guarded-loop form of the same loads measured 23% slower)
    for (int64_t g = a0 + 4 * lane; g < e; g += 256) {
      int ci[2][4];
      AccT av[2][4];
      bool two = g + 128 < e;
      ld4(hcol, g, ci[0]);
      ld4v(hval, g, av[0]);
      if (two) {
        ld4(hcol, g + 128, ci[1]);
        ld4v(hval, g + 128, av[1]);
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (h == 1 && !two) break;
        int64_t gh = g + 128 * h;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          if (gh + t >= s && gh + t < e) {
            if constexpr (sizeof(AccT) == 4) {
              float2 pq = ((const float2*)smem_raw)[ci[h][t]];
              float rr = av[h][t] * pq.x;
              acc += pq.x >= 0.f ? fminf(rr, pq.y) : fmaxf(rr, pq.y);
            } else {
              const double* tab = (const double*)smem_raw;
              double v = av[h][t] * tab[3 * ci[h][t]];          // scaling.jl:211 (times 1/std)
              double c = tab[3 * ci[h][t] + 1];
              acc += (v > c ? c : v) * tab[3 * ci[h][t] + 2];   // scaling.jl:212
            }
          }
        }
      }
    }
    acc = sv_warp_sum(acc);
    if (lane == 0) {
      double out = alpha * ((double)acc - mux);
      if (beta != 0.0) out += beta * y[r];
      if (z) out -= cs * z[r];
      y[r] = out;
    }
  }
}

// ---- X v for the Lanczos W side, double-float in and out (FP32 storage) -------
// The same row loop as k_spmv_csr with every FP64 operation removed: this part
// issues one warp-wide FP64 instruction per ~17 cycles per SM, and the FP64
// prologue and epilogue of k_spmv_csr kept its FP64 pipe 30% busy.  The vector
// arrives as a double-float basis column (its FP32 high part is the FP32 x of
// the table), mu.x is accumulated in double-float, and the result
//   y = (B x - mu.x) - csub * z      (z a double-float basis column)
// is written as a double-float working vector, ready for reorthogonalisation.
// With stacked samples (blk non-null) block b handles the cells of blk[b] of
// sample s = blk[b].seg with that sample's feature parameters (x, 1/std, clip,
// mu at offset s * nf) and csub[s].
__device__ __forceinline__ void dfx_fma(float& sh, float& sl, float ah, float al, float bh, float bl) {
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

// Prologue shared by the double-float X v kernels: with stacked samples (blk
// non-null) selects block b's row range and sample s = blk[b].seg (false: the
// sample is frozen, nothing to do); builds the per-feature (inv*x, clip*x)
// table in shared memory and returns mu.x and -csub as double-float pairs.
struct XvDf {
  int64_t rb0, rb1;
  float muxh, muxl, csh, csl;
};
__device__ __forceinline__ bool xv_df_prologue(
    unsigned char* smem_raw, int64_t n_rows, int64_t nf, const float* __restrict__ xh,
    const float* __restrict__ xl, const float* __restrict__ inv_f, const float* __restrict__ clip_f,
    const float* __restrict__ mu_h, const float* __restrict__ mu_l, const double* __restrict__ csub,
    const BlkRange* __restrict__ blk, const int* __restrict__ active, XvDf& o) {
  __shared__ float redh[32], redl[32];
  __shared__ float sc[4];
  int sg = 0;
  o.rb0 = 0;
  o.rb1 = n_rows;
  if (blk) {
    const BlkRange br = blk[blockIdx.x];
    sg = br.seg;
    o.rb0 = br.r0;
    o.rb1 = br.r1;
    if (active && !active[sg]) return false;
    const int64_t po = (int64_t)sg * nf;
    xh += po;
    xl += po;
    inv_f += po;
    clip_f += po;
    mu_h += po;
    mu_l += po;
  }
  float mh = 0.f, ml = 0.f;
  for (int64_t f = threadIdx.x; f < nf; f += blockDim.x) {
    float xs = xh[f];
    float P = inv_f[f] * xs;
    float Q = xs == 0.f ? 0.f : clip_f[f] * xs;
    ((float2*)smem_raw)[f] = make_float2(P, Q);
    dfx_fma(mh, ml, mu_h[f], mu_l[f], xs, xl[f]);
  }
  // mu.x: warp reduction in double-float, then warp 0 over the warps
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    float h2 = __shfl_xor_sync(0xffffffffu, mh, off);
    float l2 = __shfl_xor_sync(0xffffffffu, ml, off);
    float t = mh + h2;
    float v = t - mh;
    float err = (mh - (t - v)) + (h2 - v);
    ml = err + ml + l2;
    mh = t;
  }
  if ((threadIdx.x & 31) == 0) {
    redh[threadIdx.x >> 5] = mh;
    redl[threadIdx.x >> 5] = ml;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float h = 0.f, l = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      float t = h + redh[w];
      float v = t - h;
      float err = (h - (t - v)) + (redh[w] - v);
      l += err + redl[w];
      h = t;
    }
    float t = h + l;
    sc[0] = t;
    sc[1] = l - (t - h);
    if (csub) {
      double c = csub[sg];
      sc[2] = (float)c;
      sc[3] = (float)(c - (double)sc[2]);
    } else {
      sc[2] = sc[3] = 0.f;
    }
  }
  __syncthreads();
  o.muxh = sc[0];
  o.muxl = sc[1];
  o.csh = -sc[2];
  o.csl = -sc[3];
  return true;
}

// (acc - mu.x) - csub * z in double-float, written as (yh, yl)
__device__ __forceinline__ void xv_df_store(float acc, const XvDf& p, bool has_z, float zhr, float zlr,
                                            float* __restrict__ yh, float* __restrict__ yl, int64_t r) {
  float h = acc, l = 0.f;
  float t = h - p.muxh;
  float v = t - h;
  float err = (h - (t - v)) + (-p.muxh - v);
  h = t;
  l = err - p.muxl;
  if (has_z) dfx_fma(h, l, p.csh, p.csl, zhr, zlr);
  t = h + l;
  yl[r] = l - (t - h);
  yh[r] = t;
}

template <typename ValT, typename IdxT>
__global__ void __launch_bounds__(256) k_spmv_csr_df(
    const int64_t* __restrict__ rowptr, const IdxT* __restrict__ hcol, const ValT* __restrict__ hval,
    int64_t n_rows, int64_t nf, const float* __restrict__ xh, const float* __restrict__ xl,
    const float* __restrict__ inv_f, const float* __restrict__ clip_f, const float* __restrict__ mu_h,
    const float* __restrict__ mu_l, float* __restrict__ yh, float* __restrict__ yl,
    const double* __restrict__ csub, const float* __restrict__ zh, const float* __restrict__ zl,
    const BlkRange* __restrict__ blk, const int* __restrict__ active) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  XvDf pr;
  if (!xv_df_prologue(smem_raw, n_rows, nf, xh, xl, inv_f, clip_f, mu_h, mu_l, csub, blk, active, pr))
    return;
  const int64_t rb0 = pr.rb0, rb1 = pr.rb1;

  int lane = threadIdx.x & 31;
  int64_t warp, nwarps;
  if (blk) {
    warp = rb0 + (threadIdx.x >> 5);
    nwarps = blockDim.x >> 5;
  } else {
    warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  }
  for (int64_t r = warp; r < rb1; r += nwarps) {
    int64_t s = rowptr[r], e = rowptr[r + 1];
    int64_t a0 = s & ~3ll;
    float acc = 0.f;
    // two 4-element groups per lane in flight, the first load pair
    // unconditional (a loop over guarded groups -- 2 or 4 of them -- measured
    // 20-30% slower at the atlas size)
    if constexpr (sizeof(ValT) == 2 && sizeof(IdxT) == 2) {
      // 16-byte loads of 8 entries per lane and group, two groups (512
      // entries per warp) in flight: a row of ~1,000 entries takes three load
      // rounds instead of five (1.31 -> 1.18 ms per product at the atlas
      // size); 32-bit offsets within the row from its start rounded down to
      // 8 entries; words unpacked at use
      constexpr int E = XV_EPL16;
      const int64_t b0 = s & ~(int64_t)(E - 1);
      const uint16_t* pi = (const uint16_t*)hcol + b0;
      const uint16_t* pv = (const uint16_t*)hval + b0;
      const int ls = (int)(s - b0), le = (int)(e - b0);
      for (int q = E * lane; q < le; q += 64 * E) {
        uint4 ri[2], rv[2];
        const bool two = q + 32 * E < le;
        ri[0] = __ldg((const uint4*)(pi + q));
        rv[0] = __ldg((const uint4*)(pv + q));
        if (two) {
          ri[1] = __ldg((const uint4*)(pi + q + 32 * E));
          rv[1] = __ldg((const uint4*)(pv + q + 32 * E));
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (h == 1 && !two) break;
          const int qh = q + 32 * E * h;
          const unsigned wi[4] = {ri[h].x, ri[h].y, ri[h].z, ri[h].w};
          const unsigned wv[4] = {rv[h].x, rv[h].y, rv[h].z, rv[h].w};
          if (qh >= ls && qh + E <= le) {
            // a group inside the row (all but a row's first and last): no guards
#pragma unroll
            for (int t = 0; t < E; ++t) {
              const int ci = (t & 1) ? (int)(wi[t >> 1] >> 16) : (int)(wi[t >> 1] & 0xffffu);
              const float av = __uint_as_float((t & 1) ? (wv[t >> 1] & 0xffff0000u) : (wv[t >> 1] << 16));
              const float2 pq = ((const float2*)smem_raw)[ci];
              const float rr = av * pq.x;
              acc += pq.x >= 0.f ? fminf(rr, pq.y) : fmaxf(rr, pq.y);
            }
          } else {
#pragma unroll
            for (int t = 0; t < E; ++t) {
              if (qh + t >= ls && qh + t < le) {
                const int ci = (t & 1) ? (int)(wi[t >> 1] >> 16) : (int)(wi[t >> 1] & 0xffffu);
                const float av = __uint_as_float((t & 1) ? (wv[t >> 1] & 0xffff0000u) : (wv[t >> 1] << 16));
                const float2 pq = ((const float2*)smem_raw)[ci];
                const float rr = av * pq.x;
                acc += pq.x >= 0.f ? fminf(rr, pq.y) : fmaxf(rr, pq.y);
              }
            }
          }
        }
      }
    } else
    for (int64_t g = a0 + 4 * lane; g < e; g += 256) {
      int ci[2][4];
      float av[2][4];
      bool two = g + 128 < e;
      ld4(hcol, g, ci[0]);
      ld4v(hval, g, av[0]);
      if (two) {
        ld4(hcol, g + 128, ci[1]);
        ld4v(hval, g + 128, av[1]);
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (h == 1 && !two) break;
        int64_t gh = g + 128 * h;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          if (gh + t >= s && gh + t < e) {
            float2 pq = ((const float2*)smem_raw)[ci[h][t]];
            float rr = av[h][t] * pq.x;
            acc += pq.x >= 0.f ? fminf(rr, pq.y) : fmaxf(rr, pq.y);
          }
        }
      }
    }
    acc = sv_warp_sum(acc);
    if (lane == 0) xv_df_store(acc, pr, zh != nullptr, zh ? zh[r] : 0.f, zh ? zl[r] : 0.f, yh, yl, r);
  }
}

// ---- X^T u over CSR_h (warp per cell, shared-memory accumulation) -----------
// Each block accumulates sum_i min(a_if * inv_f, clip_f) * u_i for its cells into
// a shared array of nf partial sums (shared atomics), then writes the array to
// its row of `partial` (blocks x nf) together with its sum of u; the finish
// kernel adds the block rows in block order (deterministic result).
template <typename ValT, typename IdxT>
__global__ void __launch_bounds__(256) k_spmv_csr_t(
    const int64_t* __restrict__ rowptr, const IdxT* __restrict__ hcol, const ValT* __restrict__ hval,
    int64_t n_rows, int64_t nf, const double* __restrict__ u, const float* __restrict__ inv_f,
    const float* __restrict__ clip_f, const double* __restrict__ inv_d,
    const double* __restrict__ clip_d, void* __restrict__ partial, double* __restrict__ upart) {
  typedef typename AccOf<ValT>::type AccT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32];
  AccT* accs;
  if constexpr (sizeof(AccT) == 4) {
    float2* tab = (float2*)smem_raw;
    accs = (AccT*)(tab + nf);
    for (int64_t f = threadIdx.x; f < nf; f += blockDim.x) {
      tab[f] = make_float2(inv_f[f], clip_f[f]);
      accs[f] = 0;
    }
  } else {
    double2* tab = (double2*)smem_raw;
    accs = (AccT*)(tab + nf);
    for (int64_t f = threadIdx.x; f < nf; f += blockDim.x) {
      tab[f] = make_double2(inv_d[f], clip_d[f]);
      accs[f] = 0;
    }
  }
  __syncthreads();
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double usum = 0;
  for (int64_t r = warp; r < n_rows; r += nwarps) {
    int64_t s = rowptr[r], e = rowptr[r + 1];
    double ud = u[r];
    usum += ud;
    AccT ur = (AccT)ud;
    int64_t a0 = s & ~3ll;
    for (int64_t g = a0 + 4 * lane; g < e; g += 256) {
      int ci[2][4];
      AccT av[2][4];
      bool two = g + 128 < e;
      ld4(hcol, g, ci[0]);
      ld4v(hval, g, av[0]);
      if (two) {
        ld4(hcol, g + 128, ci[1]);
        ld4v(hval, g + 128, av[1]);
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (h == 1 && !two) break;
        int64_t gh = g + 128 * h;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          if (gh + t >= s && gh + t < e) {
            if constexpr (sizeof(AccT) == 4) {
              float2 ic = ((const float2*)smem_raw)[ci[h][t]];
              atomicAdd(&accs[ci[h][t]], fminf(av[h][t] * ic.x, ic.y) * ur);
            } else {
              double2 ic = ((const double2*)smem_raw)[ci[h][t]];
              double v = av[h][t] * ic.x;
              atomicAdd(&accs[ci[h][t]], (v > ic.y ? ic.y : v) * ur);
            }
          }
        }
      }
    }
  }
  // lane 0 of each warp holds the rows' u (all lanes accumulated the same values)
  if (lane != 0) usum = 0;
  usum = sv_warp_sum(usum);
  if (lane == 0) red[threadIdx.x >> 5] = usum;
  __syncthreads();
  AccT* prow = (AccT*)partial + (int64_t)blockIdx.x * nf;
  for (int64_t f = threadIdx.x; f < nf; f += blockDim.x) prow[f] = accs[f];
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    upart[blockIdx.x] = t;
  }
}

template <typename AccT>
__global__ void k_spmv_t_finish(const AccT* __restrict__ partial, int nblocks, int64_t nf,
                                const double* __restrict__ mu, const double* __restrict__ upart,
                                double alpha, double beta, double* __restrict__ y,
                                const double* __restrict__ csub, const double* __restrict__ z) {
  __shared__ double su_s;
  if (threadIdx.x < 32) {
    double v = 0;
    for (int i = threadIdx.x; i < nblocks; i += 32) v += upart[i];
    v = sv_warp_sum(v);
    if (threadIdx.x == 0) su_s = v;
  }
  __syncthreads();
  double su = su_s;
  double cs = csub ? *csub : 0.0;
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
       f += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0;
    for (int b = 0; b < nblocks; ++b) acc += (double)partial[(int64_t)b * nf + f];
    double out = alpha * (acc - mu[f] * su);
    if (beta != 0.0) out += beta * y[f];
    if (z) out -= cs * z[f];
    y[f] = out;
  }
}

// ---- X^T u over the row-blocked CSC copy ---------------------------------------
// The feature subset is stored once more, ordered (row block, feature, row): for
// every block of RB consecutive cells and every feature, the entries of that
// feature in those cells, with the row as a 16-bit offset into the block.  A CTA
// (row block b, feature group g) stages u[b*RB : (b+1)*RB] in shared memory as
// FP32 and gathers from there, so the product streams 4 B per entry (uint16 row +
// BF16 value) and no gather reaches L2.
constexpr int64_t RB_ROWS = 16384;
constexpr int RB_THREADS = 512;

// first row of row block b: b * RB_ROWS, or row0[b] for blocks aligned to
// sample boundaries
__device__ __forceinline__ int64_t rb_first_row(const int64_t* row0, int64_t b) {
  return row0 ? row0[b] : b * RB_ROWS;
}

// The row-blocked copy codes a segment's rows in groups of 8 entries, one
// 64-bit word per group: bits 0-15 the row (within the block) of the group's
// first entry, bits 16 + 6 (t - 1) .. the 6-bit step from entry t - 1 to entry
// t (t = 1..7).  A step longer than 63 between consecutive entries is bridged
// by padding entries (rows r + 63, r + 126, ... and value 0), and every segment
// is padded with value-0 entries to a whole number of groups, so segments
// start on group boundaries.  Padding adds exactly 0 to the product:
// min(0 * (1/sigma), clip) = 0 with clip > 0.
constexpr int RB_GROUP = 8;
__device__ __forceinline__ int rb_pads(int64_t step) { return step > 63 ? (int)((step - 1) / 63) : 0; }

// per (row block, feature), one warp: entries + padding (whole groups), first source entry
__global__ void k_rb_count(const int64_t* __restrict__ fstart, const int64_t* __restrict__ fend,
                           const int32_t* __restrict__ rowidx, int64_t nf, int64_t n_rb,
                           int64_t* __restrict__ cnt, int64_t* __restrict__ src,
                           const int64_t* __restrict__ row0) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t p = warp; p < n_rb * nf; p += nwarps) {
    const int64_t b = p / nf, f = p % nf;
    const int64_t s = fstart[f], e = fend[f];
    const int64_t lo = lower_bound_rows(rowidx, s, e, rb_first_row(row0, b));
    const int64_t hi = lower_bound_rows(rowidx, lo, e, rb_first_row(row0, b + 1));
    int64_t pads = 0;
    for (int64_t t = lo + 1 + lane; t < hi; t += 32) pads += rb_pads((int64_t)rowidx[t] - rowidx[t - 1]);
    pads = sv_warp_sum(pads);
    if (lane == 0) {
      const int64_t n = hi - lo + pads;
      cnt[p] = (n + RB_GROUP - 1) / RB_GROUP * RB_GROUP;
      src[p] = lo;
    }
  }
}

// one warp per (row block, feature): the coded rows (ocode zeroed beforehand,
// bit fields or-ed in) and the values, padding included
template <typename ValT>
__global__ void k_rb_copy(const int64_t* __restrict__ src, const int64_t* __restrict__ dst,
                          const int64_t* __restrict__ fend, const int32_t* __restrict__ rowidx,
                          const ValT* __restrict__ val, int64_t npairs, int64_t nf,
                          unsigned long long* __restrict__ ocode, ValT* __restrict__ oval,
                          const int64_t* __restrict__ row0) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t p = warp; p < npairs; p += nwarps) {
    const int64_t b = p / nf;
    const int64_t first = rb_first_row(row0, b);
    const int64_t s = src[p], d = dst[p], dend = dst[p + 1];
    const int64_t hi = lower_bound_rows(rowidx, s, fend[p % nf], rb_first_row(row0, b + 1));
    // entry q (from d) at row r; the previous entry at row rp
    auto put = [&](int64_t q, int64_t r, int64_t rp, ValT v) {
      const int64_t rel = q - d;
      const int slot = (int)(rel % RB_GROUP);
      const unsigned long long field =
          slot == 0 ? (unsigned long long)r : (unsigned long long)(r - rp) << (16 + 6 * (slot - 1));
      if (field) atomicOr(&ocode[q / RB_GROUP], field);
      oval[q] = v;
    };
    int64_t o = d;
    int64_t last_row = 0;
    for (int64_t t0 = s; t0 < hi; t0 += 32) {
      const int64_t t = t0 + lane;
      int64_t r = 0, rp = 0;
      int k = 0;
      if (t < hi) {
        r = (int64_t)rowidx[t] - first;
        rp = t > s ? (int64_t)rowidx[t - 1] - first : r;
        k = t > s ? rb_pads(r - rp) : 0;
      }
      int incl = t < hi ? k + 1 : 0;
#pragma unroll
      for (int sh = 1; sh < 32; sh <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, sh);
        if (lane >= sh) incl += y;
      }
      const int tot = __shfl_sync(0xffffffffu, incl, 31);
      if (t < hi) {
        int64_t q = o + incl - (k + 1);
        int64_t prev = rp;
        for (int u = 1; u <= k; ++u, ++q) {
          put(q, rp + 63 * u, prev, ValT(0.f));
          prev = rp + 63 * u;
        }
        put(q, r, prev, val[t]);
      }
      const int64_t lr = __shfl_sync(0xffffffffu, r, (tot > 0 ? min(31, (int)(hi - 1 - t0)) : 0));
      if (hi > t0) last_row = lr;
      o += tot;
    }
    // value-0 entries up to the group boundary, at the last row
    for (int64_t q = o + lane; q < dend; q += 32) put(q, last_row, last_row, ValT(0.f));
  }
}

// sum over a segment of whole groups (g0 .. g1) of min(a (1/sigma), clip) u[row];
// two groups per lane in flight, lane-local decoding
template <typename ValT>
__device__ __forceinline__ float rb_seg_dot(const unsigned long long* __restrict__ code,
                                           const ValT* __restrict__ pv, int64_t g0, int64_t g1,
                                           float inv, float clip, const float* us, int lane) {
  float acc = 0.f;
  for (int64_t g = g0 + lane; g < g1; g += 64) {
    unsigned long long c[2];
    uint4 rv[2][sizeof(ValT) == 2 ? 1 : 2];
#pragma unroll
    for (int h = 0; h < 2; ++h)
      if (g + 32 * h < g1) {
        c[h] = __ldg(code + g + 32 * h);
        const uint4* vp = (const uint4*)(pv + (g + 32 * h) * RB_GROUP);
        rv[h][0] = __ldg(vp);
        if constexpr (sizeof(ValT) == 4) rv[h][1] = __ldg(vp + 1);
      }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (g + 32 * h >= g1) break;
      int r = (int)(c[h] & 0xffffu);
      unsigned long long st = c[h] >> 16;
#pragma unroll
      for (int t = 0; t < RB_GROUP; ++t) {
        if (t > 0) {
          r += (int)(st & 63u);
          st >>= 6;
        }
        float a;
        if constexpr (sizeof(ValT) == 2) {
          const unsigned w = (&rv[h][0].x)[t >> 1];
          a = __uint_as_float((t & 1) ? (w & 0xffff0000u) : (w << 16));
        } else {
          a = __uint_as_float((&rv[h][t >> 2].x)[t & 3]);
        }
        acc += fminf(a * inv, clip) * us[r];
      }
    }
  }
  return acc;
}

template <typename ValT>
__global__ void __launch_bounds__(RB_THREADS) k_spmv_rb(
    const int64_t* __restrict__ rb_ptr, const unsigned long long* __restrict__ rb_code,
    const ValT* __restrict__ rb_val, int64_t nf, int64_t n_cells, const float* __restrict__ inv_f,
    const float* __restrict__ clip_f, const float* __restrict__ uf, float* __restrict__ partial,
    const int64_t* __restrict__ row0, const int* __restrict__ rb_seg,
    const int* __restrict__ active) {
  extern __shared__ __align__(16) float us[];
  int64_t b = blockIdx.x;
  int64_t r0, nr;
  if (row0) {
    // blocks aligned to samples: that sample's feature parameters
    int sg = rb_seg[b];
    if (active && !active[sg]) return;
    r0 = row0[b];
    nr = row0[b + 1] - r0;
    inv_f += (int64_t)sg * nf;
    clip_f += (int64_t)sg * nf;
  } else {
    r0 = b * RB_ROWS;
    nr = n_cells - r0 < RB_ROWS ? n_cells - r0 : RB_ROWS;
  }
  for (int64_t i = threadIdx.x; i < RB_ROWS; i += blockDim.x) us[i] = i < nr ? uf[r0 + i] : 0.f;
  __syncthreads();
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int fg = gridDim.y, g = blockIdx.y;
  for (int64_t f = g + (int64_t)fg * w; f < nf; f += (int64_t)fg * nw) {
    int64_t s = rb_ptr[b * nf + f], e = rb_ptr[b * nf + f + 1];
    float inv = inv_f[f], clip = clip_f[f];
    float acc = rb_seg_dot<ValT>(rb_code, rb_val, s / RB_GROUP, e / RB_GROUP, inv, clip, us, lane);
    acc = sv_warp_sum(acc);
    if (lane == 0) partial[b * nf + f] = acc;
  }
}

// The same product for one sample, as a single wave of resident blocks: tasks
// (row block b, feature group g) taken round-robin (b-major), the features of
// a task (g, g + fg, ...) handed to the warps one at a time through a shared
// counter, so that dense and sparse features even out within the block and no
// partial last wave is left (the grid form above ran 3.2 waves of blocks with
// 43% of its warps active).  Same loop and partials as k_spmv_rb.
template <typename ValT>
__global__ void __launch_bounds__(RB_THREADS, 2) k_spmv_rb_waves(
    const int64_t* __restrict__ rb_ptr, const unsigned long long* __restrict__ rb_code,
    const ValT* __restrict__ rb_val, int64_t nf, int64_t n_cells, int64_t n_rb, int fg,
    const float* __restrict__ inv_f, const float* __restrict__ clip_f, const float* __restrict__ uf,
    float* __restrict__ partial) {
  extern __shared__ __align__(16) float us[];
  __shared__ int next_f;
  const int lane = threadIdx.x & 31;
  const int64_t ntask = n_rb * fg;
  for (int64_t task = blockIdx.x; task < ntask; task += gridDim.x) {
    const int64_t b = task / fg;
    const int g = (int)(task % fg);
    const int64_t r0 = b * RB_ROWS;
    const int64_t nr = n_cells - r0 < RB_ROWS ? n_cells - r0 : RB_ROWS;
    __syncthreads();                        // the previous task is done with us and next_f
    for (int64_t i = threadIdx.x; i < RB_ROWS; i += blockDim.x) us[i] = i < nr ? uf[r0 + i] : 0.f;
    if (threadIdx.x == 0) next_f = 0;
    __syncthreads();
    while (true) {
      int fi = 0;
      if (lane == 0) fi = atomicAdd(&next_f, 1);
      fi = __shfl_sync(0xffffffffu, fi, 0);
      const int64_t f = g + (int64_t)fi * fg;
      if (f >= nf) break;
      const int64_t s = rb_ptr[b * nf + f], e = rb_ptr[b * nf + f + 1];
      const float inv = inv_f[f], clip = clip_f[f];
      float acc = rb_seg_dot<ValT>(rb_code, rb_val, s / RB_GROUP, e / RB_GROUP, inv, clip, us, lane);
      acc = sv_warp_sum(acc);
      if (lane == 0) partial[b * nf + f] = acc;
    }
  }
}

// y_f = alpha * (sum_b partial[b][f] - mu_f * sum(u)) + beta*y_f - csub*z_f
__global__ void k_rb_finish(const float* __restrict__ partial, int64_t n_rb, int64_t nf,
                            const double* __restrict__ mu, const double* __restrict__ upart,
                            int nupart, double alpha, double beta, double* __restrict__ y,
                            const double* __restrict__ csub, const double* __restrict__ z) {
  __shared__ double su_s;
  if (threadIdx.x < 32) {
    double v = 0;
    for (int i = threadIdx.x; i < nupart; i += 32) v += upart[i];
    v = sv_warp_sum(v);
    if (threadIdx.x == 0) su_s = v;
  }
  __syncthreads();
  double su = su_s;
  double cs = csub ? *csub : 0.0;
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
       f += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0;
    for (int64_t bb = 0; bb < n_rb; ++bb) acc += (double)partial[bb * nf + f];
    double out = alpha * (acc - mu[f] * su);
    if (beta != 0.0) out += beta * y[f];
    if (z) out -= cs * z[f];
    y[f] = out;
  }
}

// Stacked samples: y[s*nf + f] = sum over the sample's row blocks of
// partial[b][f] - mu[s*nf + f] * (sum of u over the sample) - csub[s] * z[s*nf + f]
// (blockIdx.y = sample).
__global__ void k_rb_finish_seg(const float* __restrict__ partial, const int64_t* __restrict__ rb_first,
                                int64_t nf, const double* __restrict__ mu,
                                const double* __restrict__ upart, double* __restrict__ y,
                                const double* __restrict__ csub, const double* __restrict__ z,
                                const int* __restrict__ active) {
  const int sg = blockIdx.y;
  if (active && !active[sg]) return;
  const int64_t b0 = rb_first[sg], b1 = rb_first[sg + 1];
  double su = 0;
  for (int64_t b = b0; b < b1; ++b) su += upart[b];
  double cs = csub ? csub[sg] : 0.0;
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
       f += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0;
    for (int64_t b = b0; b < b1; ++b) acc += (double)partial[b * nf + f];
    int64_t o = (int64_t)sg * nf + f;
    double out = acc - mu[o] * su;
    if (z) out -= cs * z[o];
    y[o] = out;
  }
}

// u -> FP32 copy and the FP64 sum of u over each sample-aligned row block
__global__ void k_bu_prep(const double* __restrict__ u, const int64_t* __restrict__ row0,
                          float* __restrict__ uf, double* __restrict__ upart) {
  __shared__ double red[32];
  const int64_t b = blockIdx.x;
  double s = 0;
  for (int64_t i = row0[b] + threadIdx.x; i < row0[b + 1]; i += blockDim.x) {
    double v = u[i];
    uf[i] = (float)v;
    s += v;
  }
  s = sv_warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = sv_warp_sum(v);
    if (threadIdx.x == 0) upart[b] = v;
  }
}

// ---- X^T u over the CSC feature ranges ---------------------------------------
// Prologue: u -> FP32 copy and per-block partial sums of u (FP64).
__global__ void k_split_df(const double* __restrict__ x, int64_t n, float* __restrict__ h,
                           float* __restrict__ l) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float a = (float)x[i];
    h[i] = a;
    l[i] = (float)(x[i] - (double)a);
  }
}

__global__ void k_u_prep(const double* __restrict__ u, int64_t n, float* __restrict__ uf,
                         double* __restrict__ part) {
  __shared__ double red[32];
  double s = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = u[i];
    if (uf) uf[i] = (float)v;
    s += v;
  }
  s = sv_warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = sv_warp_sum(v);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}

template <typename ValT>
__global__ void __launch_bounds__(256) k_spmv_csc_chunks(
    const int32_t* __restrict__ rowidx, const ValT* __restrict__ val,
    const int32_t* __restrict__ chunk_feat, const int64_t* __restrict__ cstart,
    const int64_t* __restrict__ cend, int64_t nchunks, const float* __restrict__ inv_f,
    const float* __restrict__ clip_f, const double* __restrict__ std_d,
    const double* __restrict__ clip_d, const float* __restrict__ uf, const double* __restrict__ ud,
    double* __restrict__ partial) {
  typedef typename AccOf<ValT>::type AccT;
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = warp; c < nchunks; c += nwarps) {
    int32_t f = chunk_feat[c];
    int64_t s = cstart[c], e = cend[c];
    int64_t a0 = s & ~3ll;
    AccT acc = 0;
    if constexpr (sizeof(AccT) == 4) {
      float inv = inv_f[f], clip = clip_f[f];
      for (int64_t g = a0 + 4 * lane; g < e; g += 128) {
        int ri[4];
        float av[4];
        ld4(rowidx, g, ri);
        ld4v(val, g, av);
#pragma unroll
        for (int t = 0; t < 4; ++t)
          if (g + t >= s && g + t < e) acc += fminf(av[t] * inv, clip) * __ldg(uf + ri[t]);
      }
    } else {
      double sd = std_d[f], clip = clip_d[f];
      for (int64_t g = a0 + 4 * lane; g < e; g += 128) {
        int ri[4];
        double av[4];
        ld4(rowidx, g, ri);
        ld4v(val, g, av);
#pragma unroll
        for (int t = 0; t < 4; ++t)
          if (g + t >= s && g + t < e) {
            double v = av[t] * sd;   // sd holds 1/std
            acc += (v > clip ? clip : v) * __ldg(ud + ri[t]);
          }
      }
    }
    acc = sv_warp_sum(acc);
    if (lane == 0) partial[c] = (double)acc;
  }
}

// y_f = alpha * (sum of the feature's chunk partials - mu_f * sum(u)) + beta*y_f - csub*z_f
__global__ void k_spmv_csc_finish(const double* __restrict__ partial,
                                  const int64_t* __restrict__ foff, int64_t nf,
                                  const double* __restrict__ mu, const double* __restrict__ upart,
                                  int nupart, double alpha, double beta, double* __restrict__ y,
                                  const double* __restrict__ csub, const double* __restrict__ z) {
  __shared__ double su_s;
  if (threadIdx.x < 32) {
    double v = 0;
    for (int i = threadIdx.x; i < nupart; i += 32) v += upart[i];
    v = sv_warp_sum(v);
    if (threadIdx.x == 0) su_s = v;
  }
  __syncthreads();
  double su = su_s;
  double cs = csub ? *csub : 0.0;
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
       f += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0;
    for (int64_t c = foff[f]; c < foff[f + 1]; ++c) acc += partial[c];
    double out = alpha * (acc - mu[f] * su);
    if (beta != 0.0) out += beta * y[f];
    if (z) out -= cs * z[f];
    y[f] = out;
  }
}

constexpr int UPREP_BLOCKS = 304;

}  // namespace

// ---------------------------------------------------------------------------
// internal product entry points (device vectors), used by irlba too
// ---------------------------------------------------------------------------
void sv_centered_apply(sv_context* ctx, const sv_centered* S, char trans, const double* x, double* y,
                       double alpha, double beta, const double* csub, const double* z) {
  if (trans == 'N') {
    size_t smem = S->dtype == SV_F64 ? (size_t)S->nf * 24 : (size_t)S->nf * 8;
    smem = (smem + 15) & ~(size_t)15;
    int grid = (int)std::max<int64_t>(1, std::min<int64_t>(S->grid_csr, (S->n_cells + 7) / 8));
#define LAUNCH_CSR(VT, IT, COL)                                                                  \
  sv_launch(ctx, "spmv_csr_h", k_spmv_csr<VT, IT>, dim3(grid), dim3(256), smem,                  \
            (const int64_t*)S->h_rowptr.get(), (const IT*)COL, (const VT*)S->h_val.get(),         \
            S->n_cells, S->nf, x, (const float*)S->inv_std_f.get(), (const float*)S->clip_f.get(), \
            (const double*)S->inv_std_d.get(), (const double*)S->clip_d.get(),                    \
            (const double*)S->mu.get(), alpha, beta, y, csub, z)
    bool small = S->nf <= 65536;
    switch (S->dtype) {
      case SV_F64:
        if (small) LAUNCH_CSR(double, uint16_t, S->h_col16.get());
        else LAUNCH_CSR(double, int32_t, S->h_col32.get());
        break;
      case SV_F32:
        if (small) LAUNCH_CSR(float, uint16_t, S->h_col16.get());
        else LAUNCH_CSR(float, int32_t, S->h_col32.get());
        break;
      default:
        if (small) LAUNCH_CSR(__nv_bfloat16, uint16_t, S->h_col16.get());
        else LAUNCH_CSR(__nv_bfloat16, int32_t, S->h_col32.get());
        break;
    }
#undef LAUNCH_CSR
  } else if (S->n_rb > 0) {
    // row-blocked CSC: u staged per row block in shared memory
    sv_centered* Sm = const_cast<sv_centered*>(S);
    sv_launch(ctx, "spmv_csc_uprep", k_u_prep, dim3(UPREP_BLOCKS), dim3(256), 0, x, S->n_cells,
              Sm->u_f32.get(), Sm->red_partial.get());
    // one wave of resident blocks, ~6 tasks (row block, feature group) each,
    // at least 32 features per task
    const int resident = ctx->num_sms * S->rb_per_sm;
    const int fg = (int)std::max<int64_t>(
        1, std::min<int64_t>(std::max<int64_t>(1, S->nf / 32), (6 * resident + S->n_rb - 1) / S->n_rb));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(resident, S->n_rb * fg));
    size_t smem = RB_ROWS * sizeof(float);
    if (S->dtype == SV_F32)
      sv_launch(ctx, "spmv_rb", k_spmv_rb_waves<float>, dim3(grid), dim3(RB_THREADS), smem,
                (const int64_t*)S->rb_ptr.get(), (const unsigned long long*)S->rb_idx.get(),
                (const float*)S->rb_val.get(), S->nf, S->n_cells, S->n_rb, fg,
                (const float*)S->inv_std_f.get(), (const float*)S->clip_f.get(),
                (const float*)Sm->u_f32.get(), Sm->rb_partial.get());
    else
      sv_launch(ctx, "spmv_rb", k_spmv_rb_waves<__nv_bfloat16>, dim3(grid), dim3(RB_THREADS), smem,
                (const int64_t*)S->rb_ptr.get(), (const unsigned long long*)S->rb_idx.get(),
                (const __nv_bfloat16*)S->rb_val.get(), S->nf, S->n_cells, S->n_rb, fg,
                (const float*)S->inv_std_f.get(), (const float*)S->clip_f.get(),
                (const float*)Sm->u_f32.get(), Sm->rb_partial.get());
    sv_launch(ctx, "spmv_rb_finish", k_rb_finish, dim3(sv_grid_for(ctx, S->nf, 256, 4)), dim3(256), 0,
              (const float*)Sm->rb_partial.get(), S->n_rb, S->nf, (const double*)S->mu.get(),
              (const double*)Sm->red_partial.get(), UPREP_BLOCKS, alpha, beta, y, csub, z);
  } else if (S->t_blocks > 0) {
    // warp per cell over CSR_h, shared-memory accumulation per block
    sv_centered* Sm = const_cast<sv_centered*>(S);
    bool f64 = S->dtype == SV_F64;
    size_t smem = (size_t)S->nf * (f64 ? 24 : 12);
    bool small = S->nf <= 65536;
#define LAUNCH_CT(VT, IT, COL)                                                                     \
  sv_launch(ctx, "spmv_csr_t", k_spmv_csr_t<VT, IT>, dim3(S->t_blocks), dim3(256), smem,            \
            (const int64_t*)S->h_rowptr.get(), (const IT*)COL, (const VT*)S->h_val.get(),            \
            S->n_cells, S->nf, x, (const float*)S->inv_std_f.get(), (const float*)S->clip_f.get(),   \
            (const double*)S->inv_std_d.get(), (const double*)S->clip_d.get(),                       \
            (void*)Sm->t_partial.get(), Sm->red_partial.get())
    switch (S->dtype) {
      case SV_F64:
        if (small) LAUNCH_CT(double, uint16_t, S->h_col16.get());
        else LAUNCH_CT(double, int32_t, S->h_col32.get());
        break;
      case SV_F32:
        if (small) LAUNCH_CT(float, uint16_t, S->h_col16.get());
        else LAUNCH_CT(float, int32_t, S->h_col32.get());
        break;
      default:
        if (small) LAUNCH_CT(__nv_bfloat16, uint16_t, S->h_col16.get());
        else LAUNCH_CT(__nv_bfloat16, int32_t, S->h_col32.get());
        break;
    }
#undef LAUNCH_CT
    if (f64)
      sv_launch(ctx, "spmv_t_finish", k_spmv_t_finish<double>, dim3(sv_grid_for(ctx, S->nf, 256, 4)),
                dim3(256), 0, (const double*)Sm->t_partial.get(), S->t_blocks, S->nf,
                (const double*)S->mu.get(), (const double*)Sm->red_partial.get(), alpha, beta, y, csub,
                z);
    else
      sv_launch(ctx, "spmv_t_finish", k_spmv_t_finish<float>, dim3(sv_grid_for(ctx, S->nf, 256, 4)),
                dim3(256), 0, (const float*)Sm->t_partial.get(), S->t_blocks, S->nf,
                (const double*)S->mu.get(), (const double*)Sm->red_partial.get(), alpha, beta, y, csub,
                z);
  } else {
    sv_centered* Sm = const_cast<sv_centered*>(S);
    bool f64 = S->dtype == SV_F64;
    sv_launch(ctx, "spmv_csc_uprep", k_u_prep, dim3(UPREP_BLOCKS), dim3(256), 0, x, S->n_cells,
              f64 ? (float*)nullptr : Sm->u_f32.get(), Sm->red_partial.get());
    int grid = sv_grid_for(ctx, S->n_chunks * 32, 256, 8);
    const sv_data* D = S->data;
    const int32_t* rowidx = D->counts->csc_rowidx.get();
#define LAUNCH_CSC(VT)                                                                            \
  sv_launch(ctx, "spmv_csc_chunks", k_spmv_csc_chunks<VT>, dim3(grid), dim3(256), 0, rowidx,      \
            (const VT*)D->csc_val.get(), (const int32_t*)S->chunk_feat.get(),                     \
            (const int64_t*)S->chunk_start.get(), (const int64_t*)S->chunk_end.get(), S->n_chunks, \
            (const float*)S->inv_std_f.get(), (const float*)S->clip_f.get(),                      \
            (const double*)S->inv_std_d.get(), (const double*)S->clip_d.get(),                    \
            (const float*)Sm->u_f32.get(), x, Sm->chunk_partial.get())
    switch (S->dtype) {
      case SV_F64: LAUNCH_CSC(double); break;
      case SV_F32: LAUNCH_CSC(float); break;
      default: LAUNCH_CSC(__nv_bfloat16); break;
    }
#undef LAUNCH_CSC
    sv_launch(ctx, "spmv_csc_finish", k_spmv_csc_finish, dim3(sv_grid_for(ctx, S->nf, 256, 4)),
              dim3(256), 0, (const double*)S->chunk_partial.get(),
              (const int64_t*)S->feat_chunk_off.get(), S->nf, (const double*)S->mu.get(),
              (const double*)Sm->red_partial.get(), UPREP_BLOCKS, alpha, beta, y, csub, z);
  }
}

// Builds the implicit matrix over the features `fg` (0-based genes) of `data`.
// mu_given == nullptr: per-feature moments (scale_features).  Otherwise the
// CenteredMatrix(A, mu) constructor of src/scaling.jl:224-232: std = 1, no clip.
// X v with double-float input and output (the Lanczos W step): false when the
// matrix stores FP64 values (the FP64 product is used then)
bool sv_centered_apply_df(sv_context* ctx, const sv_centered* S, const float* xh, const float* xl,
                          float* yh, float* yl, const double* csub, const float* zh, const float* zl) {
  if (S->dtype == SV_F64) return false;
  size_t smem = ((size_t)S->nf * 8 + 15) & ~(size_t)15;
  int grid = (int)std::max<int64_t>(1, std::min<int64_t>(S->grid_csr_df, (S->n_cells + 7) / 8));
#define LAUNCH_CSRDF(VT, IT, COL)                                                                \
  sv_launch(ctx, "spmv_csr_h", k_spmv_csr_df<VT, IT>, dim3(grid), dim3(256), smem,               \
            (const int64_t*)S->h_rowptr.get(), (const IT*)COL, (const VT*)S->h_val.get(),         \
            S->n_cells, S->nf, xh, xl, (const float*)S->inv_std_f.get(),                          \
            (const float*)S->clip_f.get(), (const float*)S->mu_h.get(), (const float*)S->mu_l.get(), \
            yh, yl, csub, zh, zl, (const BlkRange*)nullptr, (const int*)nullptr)
  bool small = S->nf <= 65536;
  if (S->dtype == SV_F32) {
    if (small) LAUNCH_CSRDF(float, uint16_t, S->h_col16.get());
    else LAUNCH_CSRDF(float, int32_t, S->h_col32.get());
  } else {
    if (small) LAUNCH_CSRDF(__nv_bfloat16, uint16_t, S->h_col16.get());
    else LAUNCH_CSRDF(__nv_bfloat16, int32_t, S->h_col32.get());
  }
#undef LAUNCH_CSRDF
  return true;
}

// 1-based feature indices (null: every gene) -> 0-based genes, checked
static std::vector<int32_t> feature_genes(const sv_counts* C, const int64_t* features, int64_t nfeatures) {
  SV_REQUIRE(C->n_cells >= 2, "need at least two cells for a variance");
  int64_t nf = features ? nfeatures : C->n_genes;
  SV_REQUIRE(nf >= 1, "no features");
  std::vector<int32_t> fg(nf);
  std::vector<char> seen(C->n_genes, 0);
  for (int64_t f = 0; f < nf; ++f) {
    int64_t g = features ? features[f] - 1 : f;
    SV_REQUIRE(g >= 0 && g < C->n_genes, "feature %lld out of range 1..%lld", (long long)(g + 1),
               (long long)C->n_genes);
    SV_REQUIRE(!seen[g], "duplicate feature %lld", (long long)(g + 1));
    seen[g] = 1;
    fg[f] = (int32_t)g;
  }
  return fg;
}

// Row-blocked CSC copy of the feature subset (the X^T u layout): for every
// (row block, feature) the block's entries of the feature, their rows within
// the block coded in groups of 8 (see k_rb_count) and their values.  Row blocks of RB_ROWS rows, or with
// first rows row0 (n_rb + 1 entries, device) when aligned to samples.
static void rb_build(sv_context* ctx, const sv_counts* C, const sv_data* data, const int64_t* fstart,
                     const int64_t* fend, int64_t nf, int64_t nnz_h, int64_t n_rb, const int64_t* row0,
                     DevBuf<int64_t>& rb_ptr, DevBuf<unsigned long long>& rb_idx, DevBuf<unsigned char>& rb_val,
                     DevBuf<float>& rb_partial) {
  int64_t np = n_rb * nf;
  DevBuf<int64_t> cnt(np + 1), src(np + 1);
  sv_launch(ctx, "scale_rb_count", k_rb_count, dim3(sv_grid_for(ctx, np * 32, 256, 8)), dim3(256), 0, fstart,
            fend, (const int32_t*)C->csc_rowidx.get(), nf, n_rb, cnt.get(), src.get(), row0);
  rb_ptr.alloc(np + 1);
  sv_scan_i64(ctx, cnt.get(), rb_ptr.get(), np);
  const int64_t tot = sv_read_i64(ctx, rb_ptr.get() + np);   // entries + padding
  if (tot < nnz_h)
    sv_throw(SV_ERR_DEVICE, "row-blocked copy size mismatch (%lld vs %lld)", (long long)tot,
             (long long)nnz_h);
  size_t es2 = sv_elem_size(data->dtype);
  rb_idx.alloc(std::max<int64_t>(1, tot / RB_GROUP));
  sv_memset(ctx, rb_idx.get(), 0, std::max<int64_t>(1, tot / RB_GROUP) * 8);
  rb_val.alloc(std::max<int64_t>(1, tot) * es2);
  rb_partial.alloc(std::max<int64_t>(1, np));
  int gridc = sv_grid_for(ctx, np * 32, 256, 8);
  if (data->dtype == SV_F32)
    sv_launch(ctx, "scale_rb_copy", k_rb_copy<float>, dim3(gridc), dim3(256), 0, (const int64_t*)src.get(),
              (const int64_t*)rb_ptr.get(), fend, (const int32_t*)C->csc_rowidx.get(),
              (const float*)data->csc_val.get(), np, nf, rb_idx.get(), (float*)rb_val.get(), row0);
  else
    sv_launch(ctx, "scale_rb_copy", k_rb_copy<__nv_bfloat16>, dim3(gridc), dim3(256), 0,
              (const int64_t*)src.get(), (const int64_t*)rb_ptr.get(), fend,
              (const int32_t*)C->csc_rowidx.get(), (const __nv_bfloat16*)data->csc_val.get(), np, nf,
              rb_idx.get(), (__nv_bfloat16*)rb_val.get(), row0);
  sv_sync(ctx);
}

static sv_centered* make_centered(sv_context* ctx, const sv_data* data, const std::vector<int32_t>& fg,
                                  double scale_max, const double* mu_given, bool want_rb = true) {
  const sv_counts* C = data->counts;
  int64_t nf = (int64_t)fg.size();
  size_t smem_need = data->dtype == SV_F64 ? (size_t)nf * 24 : (size_t)nf * 8;
  if (smem_need > 200 * 1024)
    sv_throw(SV_ERR_UNSUPPORTED, "%lld features exceed the shared-memory feature table",
             (long long)nf);
  auto* S = new sv_centered();
  try {
    S->ctx = ctx;
    S->data = data;
    S->n_cells = C->n_cells;
    S->nf = nf;
    S->dtype = data->dtype;
    S->scale_max = scale_max;
    S->feat_gene.alloc(nf);
    S->feat_start.alloc(nf);
    S->feat_end.alloc(nf);
    sv_h2d(ctx, S->feat_gene.get(), fg.data(), nf * 4);
    DevBuf<int32_t> gene_map(C->n_genes);
    sv_memset(ctx, gene_map.get(), 0xff, C->n_genes * 4);
    sv_launch(ctx, "scale_feat_ranges", k_feat_ranges, dim3(sv_grid_for(ctx, nf, 256)), dim3(256), 0,
              (const int32_t*)S->feat_gene.get(), (const int64_t*)C->csc_colptr.get(), nf,
              S->feat_start.get(), S->feat_end.get(), gene_map.get());
    // moments
    S->mean.alloc(nf);
    S->std_.alloc(nf);
    S->mu.alloc(nf);
    S->inv_std_f.alloc(nf);
    S->clip_f.alloc(nf);
    S->inv_std_d.alloc(nf);
    S->clip_d.alloc(nf);
#define LAUNCH_MOM(VT)                                                                          \
  launch_moments<VT>(ctx, "scale_moments", (const VT*)data->csc_val.get(),                        \
                     (const int64_t*)S->feat_start.get(), (const int64_t*)S->feat_end.get(), nf,   \
                     C->n_cells, scale_max, S->mean.get(), S->std_.get(), S->mu.get(),             \
                     S->inv_std_f.get(), S->clip_f.get(), S->inv_std_d.get(), S->clip_d.get(),      \
                     C->nnz)
    if (!mu_given) {
      switch (data->dtype) {
        case SV_F64: LAUNCH_MOM(double); break;
        case SV_F32: LAUNCH_MOM(float); break;
        default: LAUNCH_MOM(__nv_bfloat16); break;
      }
    } else {
      std::vector<double> one(nf, 1.0), inf(nf, INFINITY);
      std::vector<float> onef(nf, 1.0f), inff(nf, INFINITY);
      sv_h2d(ctx, S->mu.get(), mu_given, nf * 8);
      sv_h2d(ctx, S->mean.get(), mu_given, nf * 8);
      sv_h2d(ctx, S->std_.get(), one.data(), nf * 8);
      sv_h2d(ctx, S->inv_std_d.get(), one.data(), nf * 8);
      sv_h2d(ctx, S->clip_d.get(), inf.data(), nf * 8);
      sv_h2d(ctx, S->inv_std_f.get(), onef.data(), nf * 4);
      sv_h2d(ctx, S->clip_f.get(), inff.data(), nf * 4);
      sv_sync(ctx);
    }
#undef LAUNCH_MOM
    S->mu_h.alloc(nf);
    S->mu_l.alloc(nf);
    sv_launch(ctx, "scale_mu_split", k_split_df, dim3(sv_grid_for(ctx, nf, 256)), dim3(256), 0,
              (const double*)S->mu.get(), nf, S->mu_h.get(), S->mu_l.get());
    // chunk table of the CSC product (built on the host from the nf ranges)
    std::vector<int64_t> hs(nf), he(nf);
    sv_d2h(ctx, hs.data(), S->feat_start.get(), nf * 8);
    sv_d2h(ctx, he.data(), S->feat_end.get(), nf * 8);
    std::vector<int32_t> cf;
    std::vector<int64_t> cs, ce, foff(nf + 1);
    int64_t nnz_h = 0;
    for (int64_t f = 0; f < nf; ++f) {
      foff[f] = (int64_t)cf.size();
      int64_t s = hs[f], e = he[f];
      nnz_h += e - s;
      if (e == s) continue;
      // chunk boundaries on multiples of 4 elements (16-byte aligned vector loads)
      int64_t b = s;
      while (b < e) {
        int64_t nb = ((b + CHUNK) & ~3ll);
        if (nb > e || e - nb < CHUNK / 4) nb = e;
        cf.push_back((int32_t)f);
        cs.push_back(b);
        ce.push_back(nb);
        b = nb;
      }
    }
    foff[nf] = (int64_t)cf.size();
    S->nnz_h = nnz_h;
    S->n_chunks = (int64_t)cf.size();
    S->chunk_feat.alloc(std::max<int64_t>(1, S->n_chunks));
    S->chunk_start.alloc(std::max<int64_t>(1, S->n_chunks));
    S->chunk_end.alloc(std::max<int64_t>(1, S->n_chunks));
    S->chunk_partial.alloc(std::max<int64_t>(1, S->n_chunks));
    S->feat_chunk_off.alloc(nf + 1);
    sv_h2d(ctx, S->chunk_feat.get(), cf.data(), S->n_chunks * 4);
    sv_h2d(ctx, S->chunk_start.get(), cs.data(), S->n_chunks * 8);
    sv_h2d(ctx, S->chunk_end.get(), ce.data(), S->n_chunks * 8);
    sv_h2d(ctx, S->feat_chunk_off.get(), foff.data(), (nf + 1) * 8);
    // cell-major copy of the subset
    DevBuf<int64_t> rc(C->n_cells + 1);
    sv_launch(ctx, "scale_hsub_count", k_hsub_count, dim3(sv_grid_for(ctx, C->n_cells * 32, 256, 8)),
              dim3(256), 0, (const int64_t*)C->csr_rowptr.get(), (const int32_t*)C->csr_colidx.get(),
              C->n_cells, (const int32_t*)gene_map.get(), rc.get());
    S->h_rowptr.alloc(C->n_cells + 1);
    sv_scan_i64(ctx, rc.get(), S->h_rowptr.get(), C->n_cells);
    int64_t tot = sv_read_i64(ctx, S->h_rowptr.get() + C->n_cells);
    if (tot != nnz_h)
      sv_throw(SV_ERR_DEVICE, "subset sizes disagree between copies (%lld vs %lld)", (long long)tot,
               (long long)nnz_h);
    size_t es = sv_elem_size(data->dtype);
    S->h_val.alloc(std::max<int64_t>(1, nnz_h) * es);
    bool small = nf <= 65536;
    if (small) S->h_col16.alloc(std::max<int64_t>(1, nnz_h));
    else S->h_col32.alloc(std::max<int64_t>(1, nnz_h));
    int gridw = sv_grid_for(ctx, C->n_cells * 32, 256, 8);
#define LAUNCH_HW(VT, IT, COL)                                                                  \
  sv_launch(ctx, "scale_hsub_write", k_hsub_write<VT, IT>, dim3(gridw), dim3(256), 0,           \
            (const int64_t*)C->csr_rowptr.get(), (const int32_t*)C->csr_colidx.get(),            \
            (const VT*)data->csr_val.get(), C->n_cells, (const int32_t*)gene_map.get(),          \
            (const int64_t*)S->h_rowptr.get(), (IT*)COL, (VT*)S->h_val.get())
    switch (data->dtype) {
      case SV_F64:
        if (small) LAUNCH_HW(double, uint16_t, S->h_col16.get());
        else LAUNCH_HW(double, int32_t, S->h_col32.get());
        break;
      case SV_F32:
        if (small) LAUNCH_HW(float, uint16_t, S->h_col16.get());
        else LAUNCH_HW(float, int32_t, S->h_col32.get());
        break;
      default:
        if (small) LAUNCH_HW(uint16_t, uint16_t, S->h_col16.get());
        else LAUNCH_HW(uint16_t, int32_t, S->h_col32.get());
        break;
    }
#undef LAUNCH_HW
    if (small && data->dtype != SV_F64 && !getenv("SV_NO_BANKORDER")) {
      // bank-aware order of the rows (into a second copy, then swapped in)
      DevBuf<uint16_t> col2(std::max<int64_t>(1, nnz_h));
      DevBuf<unsigned char> val2(std::max<int64_t>(1, nnz_h) * es);
      int bgrid = ctx->num_sms * 8;
      if (data->dtype == SV_F32)
        sv_launch(ctx, "scale_hsub_order", k_bankorder<16, 4, float>, dim3(bgrid), dim3(BO_WARPS * 32), 0,
                  (const int64_t*)S->h_rowptr.get(), C->n_cells, (const uint16_t*)S->h_col16.get(),
                  (const float*)S->h_val.get(), col2.get(), (float*)val2.get());
      else
        sv_launch(ctx, "scale_hsub_order", k_bankorder<16, XV_EPL16, uint16_t>, dim3(bgrid), dim3(BO_WARPS * 32), 0,
                  (const int64_t*)S->h_rowptr.get(), C->n_cells, (const uint16_t*)S->h_col16.get(),
                  (const uint16_t*)S->h_val.get(), col2.get(), (uint16_t*)val2.get());
      S->h_col16 = std::move(col2);
      S->h_val = std::move(val2);
    }
    S->u_f32.alloc(C->n_cells);
    S->scal.alloc(64);
    // row-blocked CSC copy for X^T u (FP32 / BF16 storage; SV_TPRODUCT=csc or csr
    // selects the other forms)
    {
      const char* mode = getenv("SV_TPRODUCT");
      bool use_rb = want_rb && data->dtype != SV_F64 &&
                    !(mode && (strcmp(mode, "csc") == 0 || strcmp(mode, "csr") == 0));
      if (use_rb) {
        S->rb_rows = RB_ROWS;
        S->n_rb = (C->n_cells + RB_ROWS - 1) / RB_ROWS;
        rb_build(ctx, C, data, S->feat_start.get(), S->feat_end.get(), nf, nnz_h, S->n_rb, nullptr,
                 S->rb_ptr, S->rb_idx, S->rb_val, S->rb_partial);
        SV_CUDA(cudaFuncSetAttribute(k_spmv_rb<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(RB_ROWS * sizeof(float))));
        SV_CUDA(cudaFuncSetAttribute(k_spmv_rb<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(RB_ROWS * sizeof(float))));
        // three 64 KB blocks per SM: prefer the largest shared-memory carve-out
        SV_CUDA(cudaFuncSetAttribute(k_spmv_rb<float>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        SV_CUDA(cudaFuncSetAttribute(k_spmv_rb<__nv_bfloat16>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     100));
        SV_CUDA(cudaFuncSetAttribute(k_spmv_rb_waves<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(RB_ROWS * sizeof(float))));
        SV_CUDA(cudaFuncSetAttribute(k_spmv_rb_waves<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(RB_ROWS * sizeof(float))));
        SV_CUDA(cudaFuncSetAttribute(k_spmv_rb_waves<float>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        SV_CUDA(cudaFuncSetAttribute(k_spmv_rb_waves<__nv_bfloat16>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     100));
        int per = 0;
        if (data->dtype == SV_F32)
          SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_spmv_rb_waves<float>, RB_THREADS,
                                                                RB_ROWS * sizeof(float)));
        else
          SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_spmv_rb_waves<__nv_bfloat16>, RB_THREADS,
                                                                RB_ROWS * sizeof(float)));
        S->rb_per_sm = std::max(1, per);
        sv_sync(ctx);
      }
    }
    // X^T u: CSC chunks by default (measured faster on GB300: the CSR_h form is
    // bound by shared-memory atomics); SV_TPRODUCT=csr selects the warp-per-cell
    // form over CSR_h when its per-block feature arrays fit in shared memory
    {
      size_t tsmem = (size_t)nf * (data->dtype == SV_F64 ? 24 : 12);
      const char* mode = getenv("SV_TPRODUCT");
      bool want_csr = mode && strcmp(mode, "csr") == 0;
      if (want_csr && tsmem <= 200 * 1024) {
        S->t_blocks = ctx->num_sms * 2;
        S->t_partial.alloc((size_t)S->t_blocks * nf * (data->dtype == SV_F64 ? 8 : 4));
        SV_CUDA(cudaFuncSetAttribute(k_spmv_csr_t<double, uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SV_CUDA(cudaFuncSetAttribute(k_spmv_csr_t<double, int32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SV_CUDA(cudaFuncSetAttribute(k_spmv_csr_t<float, uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SV_CUDA(cudaFuncSetAttribute(k_spmv_csr_t<float, int32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SV_CUDA(cudaFuncSetAttribute(k_spmv_csr_t<__nv_bfloat16, uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SV_CUDA(cudaFuncSetAttribute(k_spmv_csr_t<__nv_bfloat16, int32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
      }
      S->red_partial.alloc(std::max<int64_t>(UPREP_BLOCKS, S->t_blocks));
    }
#define SET_SMEM(VT, IT)                                                                         \
  SV_CUDA(cudaFuncSetAttribute(k_spmv_csr<VT, IT>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                               200 * 1024))
    SET_SMEM(double, uint16_t);
    SET_SMEM(double, int32_t);
    SET_SMEM(float, uint16_t);
    SET_SMEM(float, int32_t);
    SET_SMEM(__nv_bfloat16, uint16_t);
    SET_SMEM(__nv_bfloat16, int32_t);
#undef SET_SMEM
    SV_CUDA(cudaFuncSetAttribute(k_spmv_csr_df<float, uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    SV_CUDA(cudaFuncSetAttribute(k_spmv_csr_df<float, int32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    SV_CUDA(cudaFuncSetAttribute(k_spmv_csr_df<__nv_bfloat16, uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    SV_CUDA(cudaFuncSetAttribute(k_spmv_csr_df<__nv_bfloat16, int32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    // the X v kernels loop over rows: one wave of resident blocks (a second,
    // partial wave left SMs idle at the tail)
    {
      size_t tsm = ((size_t)nf * (data->dtype == SV_F64 ? 24 : 8) + 15) & ~(size_t)15;
      size_t tsm_df = ((size_t)nf * 8 + 15) & ~(size_t)15;
      int b1 = 0, b2 = 0;
      bool small16 = nf <= 65536;
      switch (data->dtype) {
        case SV_F64:
          SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
              &b1, small16 ? (const void*)k_spmv_csr<double, uint16_t> : (const void*)k_spmv_csr<double, int32_t>,
              256, tsm));
          break;
        case SV_F32:
          SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
              &b1, small16 ? (const void*)k_spmv_csr<float, uint16_t> : (const void*)k_spmv_csr<float, int32_t>,
              256, tsm));
          SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
              &b2, small16 ? (const void*)k_spmv_csr_df<float, uint16_t> : (const void*)k_spmv_csr_df<float, int32_t>,
              256, tsm_df));
          break;
        default:
          SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
              &b1, small16 ? (const void*)k_spmv_csr<__nv_bfloat16, uint16_t>
                           : (const void*)k_spmv_csr<__nv_bfloat16, int32_t>,
              256, tsm));
          SV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
              &b2, small16 ? (const void*)k_spmv_csr_df<__nv_bfloat16, uint16_t>
                           : (const void*)k_spmv_csr_df<__nv_bfloat16, int32_t>,
              256, tsm_df));
          break;
      }
      S->grid_csr = std::max(1, b1) * ctx->num_sms;
      S->grid_csr_df = std::max(1, b2) * ctx->num_sms;
    }
    sv_sync(ctx);
  } catch (...) {
    delete S;
    throw;
  }
  return S;
}

SV_API int sv_scale_features(sv_context* ctx, const sv_data* data, const int64_t* features,
                             int64_t nfeatures, double scale_max, sv_centered** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(out && data, "null argument");
  SV_REQUIRE(data->ctx == ctx, "data handle belongs to another context");
  const sv_counts* C = data->counts;
  SV_REQUIRE(C->n_cells >= 2, "need at least two cells for a variance");
  std::vector<int32_t> fg = feature_genes(C, features, nfeatures);
  *out = make_centered(ctx, data, fg, scale_max, nullptr);
  SV_CATCH
}

// ---- batched samples ----------------------------------------------------------
// Samples stacked by cells in one data matrix, each scaled with its own
// moments (scale_features per sample, src/scaling.jl:335-357): the feature
// subset copies are those of the stacked matrix; the per-(sample, feature)
// moments, the X v block schedule and the sample-aligned row blocks of X^T u
// are the batch's own.  FP32 / BF16 storage.
// cells per X v block: chosen by timing the candidates on the first batch of a
// given shape (device, cells, features, samples), then reused
static const int BATCH_XCELLS_CAND[] = {128, 256, 512, 1024};
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int64_t, int64_t, int64_t>, int> g_tune;

static void batch_xschedule(sv_context* ctx, sv_batch* B, int cells) {
  std::vector<BlkRange> hb;
  for (int64_t s2 = 0; s2 < B->nseg; ++s2)
    for (int64_t r = B->hoff[s2]; r < B->hoff[s2 + 1]; r += cells) {
      BlkRange b;
      b.r0 = r;
      b.r1 = std::min(B->hoff[s2 + 1], r + cells);
      b.seg = (int)s2;
      b.pad = 0;
      hb.push_back(b);
    }
  B->nxblk = (int)hb.size();
  B->xblk.alloc(hb.size());
  sv_h2d(ctx, B->xblk.get(), hb.data(), hb.size() * sizeof(BlkRange));
  B->xcells = cells;
}

void sv_batch_apply_N_df(sv_context* ctx, const sv_batch* b, const float* xh, const float* xl,
                         float* yh, float* yl, const double* csub, const float* zh, const float* zl,
                         const int* active);

// the autotuner: time every candidate block size on this batch (zero vectors)
static int batch_tune_xcells(sv_context* ctx, sv_batch* B) {
  auto key = std::make_tuple(ctx->device, B->n_cells, B->nf, B->nseg);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) return it->second;
  }
  DevBuf<float> xh((size_t)B->nseg * B->nf), yh(B->n_cells), yl(B->n_cells);
  sv_memset(ctx, xh.get(), 0, (size_t)B->nseg * B->nf * 4);
  cudaEvent_t e0, e1;
  SV_CUDA(cudaEventCreate(&e0));
  SV_CUDA(cudaEventCreate(&e1));
  int best = BATCH_XCELLS_CAND[1];
  float best_ms = 1e30f;
  for (int cand : BATCH_XCELLS_CAND) {
    batch_xschedule(ctx, B, cand);
    sv_batch_apply_N_df(ctx, B, xh.get(), xh.get(), yh.get(), yl.get(), nullptr, nullptr, nullptr, nullptr);
    SV_CUDA(cudaEventRecord(e0, ctx->stream));
    for (int r = 0; r < 3; ++r)
      sv_batch_apply_N_df(ctx, B, xh.get(), xh.get(), yh.get(), yl.get(), nullptr, nullptr, nullptr, nullptr);
    SV_CUDA(cudaEventRecord(e1, ctx->stream));
    SV_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    SV_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best_ms) {
      best_ms = ms;
      best = cand;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = best;
  return best;
}

SV_API int sv_batch_create(sv_context* ctx, const sv_data* data, const int64_t* cell_offsets,
                           int64_t nseg, const int64_t* features, int64_t nfeatures, double scale_max,
                           sv_batch** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(out && data && cell_offsets, "null argument");
  SV_REQUIRE(data->ctx == ctx, "data handle belongs to another context");
  SV_REQUIRE(data->dtype != SV_F64, "batched samples take FP32 or BF16 values");
  const sv_counts* C = data->counts;
  SV_REQUIRE(nseg >= 1, "no samples");
  SV_REQUIRE(cell_offsets[0] == 0 && cell_offsets[nseg] == C->n_cells,
             "cell offsets must run from 0 to the number of cells");
  for (int64_t s = 0; s < nseg; ++s)
    SV_REQUIRE(cell_offsets[s + 1] - cell_offsets[s] >= 2, "sample %lld has fewer than two cells",
               (long long)(s + 1));
  std::vector<int32_t> fg = feature_genes(C, features, nfeatures);
  const int64_t nf = (int64_t)fg.size();
  auto* B = new sv_batch();
  try {
    B->ctx = ctx;
    B->data = data;
    B->nseg = nseg;
    B->n_cells = C->n_cells;
    B->nf = nf;
    B->scale_max = scale_max;
    B->hoff.assign(cell_offsets, cell_offsets + nseg + 1);
    B->off.alloc(nseg + 1);
    sv_h2d(ctx, B->off.get(), cell_offsets, (nseg + 1) * 8);
    B->base = make_centered(ctx, data, fg, scale_max, nullptr, false);
    sv_centered* S = B->base;
    // per-(sample, feature) moments
    size_t sf = (size_t)nseg * nf;
    B->mean.alloc(sf);
    B->std_.alloc(sf);
    B->mu.alloc(sf);
    B->inv_d.alloc(sf);
    B->clip_d.alloc(sf);
    B->inv_f.alloc(sf);
    B->clip_f.alloc(sf);
    B->mu_h.alloc(sf);
    B->mu_l.alloc(sf);
#define LAUNCH_BMOM(VT)                                                                           \
  launch_moments<VT>(ctx, "scale_moments", (const VT*)data->csc_val.get(),                          \
                     (const int64_t*)S->feat_start.get(), (const int64_t*)S->feat_end.get(), nf,     \
                     C->n_cells, scale_max, B->mean.get(), B->std_.get(), B->mu.get(),               \
                     B->inv_f.get(), B->clip_f.get(), B->inv_d.get(), B->clip_d.get(), C->nnz,       \
                     (const int32_t*)C->csc_rowidx.get(), (const int64_t*)B->off.get(), (int)nseg)
    if (data->dtype == SV_F32) LAUNCH_BMOM(float);
    else LAUNCH_BMOM(__nv_bfloat16);
#undef LAUNCH_BMOM
    sv_launch(ctx, "scale_mu_split", k_split_df, dim3(sv_grid_for(ctx, (int64_t)sf, 256)), dim3(256), 0,
              (const double*)B->mu.get(), (int64_t)sf, B->mu_h.get(), B->mu_l.get());
    // X^T u: row blocks of at most RB_ROWS cells, aligned to the samples
    {
      std::vector<int64_t> row0;
      std::vector<int> seg;
      B->h_rb_first.assign(nseg + 1, 0);
      for (int64_t s2 = 0; s2 < nseg; ++s2) {
        B->h_rb_first[s2] = (int64_t)row0.size();
        for (int64_t r = B->hoff[s2]; r < B->hoff[s2 + 1]; r += RB_ROWS) {
          row0.push_back(r);
          seg.push_back((int)s2);
        }
      }
      B->h_rb_first[nseg] = (int64_t)row0.size();
      B->n_rb = (int64_t)row0.size();
      row0.push_back(C->n_cells);
      B->rb_row0.alloc(row0.size());
      B->rb_seg.alloc(seg.size());
      B->rb_first.alloc(nseg + 1);
      sv_h2d(ctx, B->rb_row0.get(), row0.data(), row0.size() * 8);
      sv_h2d(ctx, B->rb_seg.get(), seg.data(), seg.size() * 4);
      sv_h2d(ctx, B->rb_first.get(), B->h_rb_first.data(), (nseg + 1) * 8);
      rb_build(ctx, C, data, S->feat_start.get(), S->feat_end.get(), nf, S->nnz_h, B->n_rb,
               B->rb_row0.get(), B->rb_ptr, B->rb_idx, B->rb_val, B->rb_partial);
      B->upart.alloc(B->n_rb);
      SV_CUDA(cudaFuncSetAttribute(k_spmv_rb<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(RB_ROWS * sizeof(float))));
      SV_CUDA(cudaFuncSetAttribute(k_spmv_rb<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(RB_ROWS * sizeof(float))));
    }
    // X v schedule: cells of one sample per block, the block size tuned once per shape
    batch_xschedule(ctx, B, batch_tune_xcells(ctx, B));
    sv_sync(ctx);
  } catch (...) {
    if (B->base) sv_centered_free(B->base);
    delete B;
    throw;
  }
  *out = B;
  SV_CATCH
}

SV_API int sv_batch_info(const sv_batch* b, int64_t* nseg, int64_t* n_cells, int64_t* nf) {
  SV_TRY
  SV_REQUIRE(b, "null handle");
  if (nseg) *nseg = b->nseg;
  if (n_cells) *n_cells = b->n_cells;
  if (nf) *nf = b->nf;
  SV_CATCH
}

// the X v block size (cells per block) the autotuner chose for this batch's shape
SV_API int sv_batch_tuning(const sv_batch* b, int64_t* cells_per_block) {
  SV_TRY
  SV_REQUIRE(b, "null handle");
  if (cells_per_block) *cells_per_block = b->xcells;
  SV_CATCH
}

// per-(sample, feature) statistics, sample-major (nseg x nf): mu = mean/std,
// mean, std
SV_API int sv_batch_stats(sv_context* ctx, const sv_batch* b, double* mu, double* mean, double* sd) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(b && b->ctx == ctx, "bad batch handle");
  size_t bytes = (size_t)b->nseg * b->nf * 8;
  if (mu) sv_d2h(ctx, mu, b->mu.get(), bytes);
  if (mean) sv_d2h(ctx, mean, b->mean.get(), bytes);
  if (sd) sv_d2h(ctx, sd, b->std_.get(), bytes);
  SV_CATCH
}

SV_API int sv_batch_free(sv_batch* b) {
  if (b) {
    if (b->ctx) cudaSetDevice(b->ctx->device);
    sv_centered_free(b->base);
    delete b;
  }
  return SV_OK;
}

// W step of the batched Lanczos: for every active sample, y = X_s v_s - csub[s] z
// (double-float in and out, stacked)
void sv_batch_apply_N_df(sv_context* ctx, const sv_batch* b, const float* xh, const float* xl,
                         float* yh, float* yl, const double* csub, const float* zh, const float* zl,
                         const int* active) {
  const sv_centered* S = b->base;
  size_t smem = ((size_t)b->nf * 8 + 15) & ~(size_t)15;
#define LAUNCH_BCSR(VT, IT, COL)                                                                  \
  sv_launch(ctx, "spmv_csr_h", k_spmv_csr_df<VT, IT>, dim3(b->nxblk), dim3(256), smem,            \
            (const int64_t*)S->h_rowptr.get(), (const IT*)COL, (const VT*)S->h_val.get(),          \
            b->n_cells, b->nf, xh, xl, (const float*)b->inv_f.get(), (const float*)b->clip_f.get(), \
            (const float*)b->mu_h.get(), (const float*)b->mu_l.get(), yh, yl, csub, zh, zl,         \
            (const BlkRange*)b->xblk.get(), active)
  bool small = b->nf <= 65536;
  if (b->data->dtype == SV_F32) {
    if (small) LAUNCH_BCSR(float, uint16_t, S->h_col16.get());
    else LAUNCH_BCSR(float, int32_t, S->h_col32.get());
  } else {
    if (small) LAUNCH_BCSR(__nv_bfloat16, uint16_t, S->h_col16.get());
    else LAUNCH_BCSR(__nv_bfloat16, int32_t, S->h_col32.get());
  }
#undef LAUNCH_BCSR
}

// V step of the batched Lanczos: for every active sample, y_s = X_s^T u_s -
// csub[s] z_s (FP64, stacked by sample: index s * nf + f)
void sv_batch_apply_T(sv_context* ctx, const sv_batch* b, const double* u, double* y,
                      const double* csub, const double* z, const int* active) {
  sv_batch* bm = const_cast<sv_batch*>(b);
  sv_centered* S = b->base;
  sv_launch(ctx, "spmv_csc_uprep", k_bu_prep, dim3((unsigned)b->n_rb), dim3(256), 0, u,
            (const int64_t*)b->rb_row0.get(), S->u_f32.get(), bm->upart.get());
  int resident = ctx->num_sms * 3;
  int fg = (int)std::max<int64_t>(1, std::min<int64_t>(b->nf, (3 * resident + b->n_rb - 1) / b->n_rb));
  dim3 grid((unsigned)b->n_rb, (unsigned)fg);
  size_t smem = RB_ROWS * sizeof(float);
  if (b->data->dtype == SV_F32)
    sv_launch(ctx, "spmv_rb", k_spmv_rb<float>, grid, dim3(RB_THREADS), smem,
              (const int64_t*)b->rb_ptr.get(), (const unsigned long long*)b->rb_idx.get(), (const float*)b->rb_val.get(),
              b->nf, b->n_cells, (const float*)b->inv_f.get(), (const float*)b->clip_f.get(),
              (const float*)S->u_f32.get(), bm->rb_partial.get(), (const int64_t*)b->rb_row0.get(),
              (const int*)b->rb_seg.get(), active);
  else
    sv_launch(ctx, "spmv_rb", k_spmv_rb<__nv_bfloat16>, grid, dim3(RB_THREADS), smem,
              (const int64_t*)b->rb_ptr.get(), (const unsigned long long*)b->rb_idx.get(),
              (const __nv_bfloat16*)b->rb_val.get(), b->nf, b->n_cells, (const float*)b->inv_f.get(),
              (const float*)b->clip_f.get(), (const float*)S->u_f32.get(), bm->rb_partial.get(),
              (const int64_t*)b->rb_row0.get(), (const int*)b->rb_seg.get(), active);
  dim3 fgrid((unsigned)sv_grid_for(ctx, b->nf, 256, 1), (unsigned)b->nseg);
  sv_launch(ctx, "spmv_rb_finish", k_rb_finish_seg, fgrid, dim3(256), 0, (const float*)bm->rb_partial.get(),
            (const int64_t*)b->rb_first.get(), b->nf, (const double*)b->mu.get(),
            (const double*)bm->upart.get(), y, csub, z, active);
}

sv_counts* sv_counts_upload_positions(sv_context* ctx, int64_t n_rows, int64_t n_cols, int64_t nnz,
                                      const int64_t* colptr, const int64_t* rowval);

namespace {
template <typename T>
__global__ void k_gather_vals(const double* __restrict__ src, const int32_t* __restrict__ pos,
                              int64_t nnz, T* __restrict__ dst_csr, T* __restrict__ dst_csc) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz;
       e += (int64_t)gridDim.x * blockDim.x) {
    dst_csr[e] = (T)src[pos[e]];
    dst_csc[e] = (T)src[e];
  }
}
}  // namespace

SV_API int sv_centered_create(sv_context* ctx, int64_t n_rows, int64_t n_cols, int64_t nnz,
                              const int64_t* colptr, const int64_t* rowval, const double* nzval,
                              const double* mu, int dtype, sv_centered** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(out && colptr && mu && (nnz == 0 || (rowval && nzval)), "null argument");
  SV_REQUIRE(dtype == SV_F64 || dtype == SV_F32, "dtype must be F64 or F32");
  SV_REQUIRE(nnz < (1ll << 31), "nnz must fit Int32 positions");
  sv_counts* C = sv_counts_upload_positions(ctx, n_rows, n_cols, nnz, colptr, rowval);
  sv_data* D = nullptr;
  try {
    D = new sv_data();
    D->ctx = ctx;
    D->counts = C;
    D->dtype = dtype;
    size_t es = sv_elem_size(dtype);
    D->csc_val.alloc(std::max<int64_t>(1, nnz) * es);
    D->csr_val.alloc(std::max<int64_t>(1, nnz) * es);
    DevBuf<double> src(std::max<int64_t>(1, nnz));
    sv_h2d(ctx, src.get(), nzval, nnz * 8);
    if (dtype == SV_F64)
      sv_launch(ctx, "centered_gather", k_gather_vals<double>, dim3(sv_grid_for(ctx, nnz, 256, 8)),
                dim3(256), 0, (const double*)src.get(), (const int32_t*)C->csr_count.get(), nnz,
                (double*)D->csr_val.get(), (double*)D->csc_val.get());
    else
      sv_launch(ctx, "centered_gather", k_gather_vals<float>, dim3(sv_grid_for(ctx, nnz, 256, 8)),
                dim3(256), 0, (const double*)src.get(), (const int32_t*)C->csr_count.get(), nnz,
                (float*)D->csr_val.get(), (float*)D->csc_val.get());
    std::vector<int32_t> fg(n_cols);
    for (int64_t f = 0; f < n_cols; ++f) fg[f] = (int32_t)f;
    sv_centered* S = make_centered(ctx, D, fg, INFINITY, mu);
    S->own_counts = C;
    S->own_data = D;
    *out = S;
  } catch (...) {
    delete D;
    delete C;
    throw;
  }
  SV_CATCH
}

// Per-gene mean and standard deviation (n - 1) of the raw counts, implicit
// zeros included (mean_std on the count matrix, src/scaling.jl:18-44): device
// arrays of n_genes.
void sv_count_moments(sv_context* ctx, const sv_counts* C, double* mean, double* sd) {
  int64_t ng = C->n_genes;
  DevBuf<double> mu(ng), invd(ng), clipd(ng);
  DevBuf<float> invf(ng), clipf(ng);
  launch_moments<int32_t>(ctx, "gene_moments", (const int32_t*)C->csc_count.get(),
                          (const int64_t*)C->csc_colptr.get(), (const int64_t*)C->csc_colptr.get() + 1,
                          ng, C->n_cells, (double)INFINITY, mean, sd, mu.get(), invf.get(),
                          clipf.get(), invd.get(), clipd.get(), C->nnz);
}

SV_API int sv_gene_moments(sv_context* ctx, const sv_data* data, double* mean, double* var) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(data && data->ctx == ctx && (mean || var), "bad argument");
  const sv_counts* C = data->counts;
  SV_REQUIRE(C->n_cells >= 2, "need at least two cells for a variance");
  int64_t ng = C->n_genes;
  DevBuf<int64_t> fs(ng), fe(ng);
  DevBuf<double> m(ng), sd(ng), mu(ng), invd(ng), clipd(ng);
  DevBuf<float> invf(ng), clipf(ng);
  SV_CUDA(cudaMemcpyAsync(fs.get(), C->csc_colptr.get(), ng * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  SV_CUDA(cudaMemcpyAsync(fe.get(), C->csc_colptr.get() + 1, ng * 8, cudaMemcpyDeviceToDevice,
                          ctx->stream));
#define LAUNCH_MOM(VT)                                                                           \
  launch_moments<VT>(ctx, "gene_moments", (const VT*)data->csc_val.get(), (const int64_t*)fs.get(), \
                     (const int64_t*)fe.get(), ng, C->n_cells, (double)INFINITY, m.get(), sd.get(), \
                     mu.get(), invf.get(), clipf.get(), invd.get(), clipd.get(), C->nnz)
  switch (data->dtype) {
    case SV_F64: LAUNCH_MOM(double); break;
    case SV_F32: LAUNCH_MOM(float); break;
    default: LAUNCH_MOM(__nv_bfloat16); break;
  }
#undef LAUNCH_MOM
  if (mean) sv_d2h(ctx, mean, m.get(), ng * 8);
  if (var) {
    std::vector<double> s(ng);
    sv_d2h(ctx, s.data(), sd.get(), ng * 8);
    for (int64_t g = 0; g < ng; ++g) var[g] = s[g] * s[g];
  }
  SV_CATCH
}

SV_API int sv_centered_info(const sv_centered* s, int64_t* n_cells, int64_t* nf, int64_t* nnz) {
  SV_TRY
  SV_REQUIRE(s, "null handle");
  if (n_cells) *n_cells = s->n_cells;
  if (nf) *nf = s->nf;
  if (nnz) *nnz = s->nnz_h;
  SV_CATCH
}

SV_API int sv_centered_stats(sv_context* ctx, const sv_centered* s, double* mu, double* mean,
                             double* sd) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(s && s->ctx == ctx, "bad handle");
  if (mu) sv_d2h(ctx, mu, s->mu.get(), s->nf * 8);
  if (mean) sv_d2h(ctx, mean, s->mean.get(), s->nf * 8);
  if (sd) sv_d2h(ctx, sd, s->std_.get(), s->nf * 8);
  SV_CATCH
}

SV_API int sv_centered_mul(sv_context* ctx, const sv_centered* s, char trans, int64_t ncols,
                           double alpha, const double* x, int64_t ldx, double beta, double* y,
                           int64_t ldy) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(s && s->ctx == ctx, "bad handle");
  SV_REQUIRE(trans == 'N' || trans == 'T', "trans must be 'N' or 'T'");
  SV_REQUIRE(ncols >= 0 && x && y, "bad arguments");
  int64_t nx = trans == 'N' ? s->nf : s->n_cells;
  int64_t ny = trans == 'N' ? s->n_cells : s->nf;
  SV_REQUIRE(ldx >= nx && ldy >= ny, "leading dimension too small");
  DevBuf<double> dx(nx), dy(ny);
  for (int64_t j = 0; j < ncols; ++j) {
    sv_h2d(ctx, dx.get(), x + j * ldx, nx * 8);
    if (beta != 0.0) sv_h2d(ctx, dy.get(), y + j * ldy, ny * 8);
    sv_centered_apply(ctx, s, trans, dx.get(), dy.get(), alpha, beta, nullptr, nullptr);
    sv_d2h(ctx, y + j * ldy, dy.get(), ny * 8);
  }
  SV_CATCH
}

SV_API int sv_centered_free(sv_centered* s) {
  if (s) {
    if (s->ctx) cudaSetDevice(s->ctx->device);
    sv_data* d = s->own_data;
    sv_counts* c = s->own_counts;
    delete s;
    delete d;
    delete c;
  }
  return SV_OK;
}
