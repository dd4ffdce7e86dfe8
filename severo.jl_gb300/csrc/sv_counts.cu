// Count matrix on the device: upload of a Julia SparseMatrixCSC (cells x genes),
// the cell-major (CSR) copy built on the device, and the synthetic generator.
//
// Layout in HBM (both copies resident, as the embedding path reads both):
//   CSC  colptr int64[n_genes+1], rowidx int32[nnz], count int32[nnz]   (gene-major)
//   CSR  rowptr int64[n_cells+1], colidx int32[nnz], count int32[nnz]   (cell-major)
// Indices are 0-based on the device; rows are sorted within columns and columns
// within rows.
#include "sv_internal.cuh"

#include <type_traits>

namespace {

// ---- conversion of the uploaded arrays --------------------------------------
template <typename T>
__global__ void k_colptr_to_i64(const T* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                                int64_t base) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int64_t)in[i] - base;
}

template <typename T>
__global__ void k_idx_to_i32(const T* __restrict__ in, int32_t* __restrict__ out, int64_t n,
                             int64_t base, int64_t limit, int* status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t v = (int64_t)in[i] - base;
    if (v < 0 || v >= limit) {
      sv_flag(status, SV_STATUS_OOB);
      v = 0;
    }
    out[i] = (int32_t)v;
  }
}

// Counts of a wider or floating type to Int32: whole numbers in [0, 2^31) pass,
// anything else (fractions, NaN, out of range) flags SV_STATUS_VALUE.
template <typename T>
__global__ void k_count_to_i32(const T* __restrict__ in, int32_t* __restrict__ out, int64_t n,
                               int* status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    T v = in[i];
    bool ok = v >= (T)0 && v < (T)2147483648.0 && (T)(int64_t)v == v;
    if (!ok) sv_flag(status, SV_STATUS_VALUE);
    out[i] = ok ? (int32_t)v : 0;
  }
}

// Sets bit 1 of *flag when an index is not above its predecessor in the same
// segment, bit 2 when a segment's pointers are out of order or out of range.
__global__ void k_seg_unsorted(const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                               int64_t n, int64_t nnz, int* flag) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n; r += nwarps) {
    int64_t s = ptr[r], e = ptr[r + 1];
    if (s < 0 || e < s || e > nnz) {
      if (lane == 0) atomicOr(flag, 2);
      continue;
    }
    bool bad = false;
    for (int64_t i = s + 1 + lane; i < e; i += 32) bad |= idx[i] <= idx[i - 1];
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(flag, 1);
  }
}

// ---- order-preserving transpose ------------------------------------------------
// The output segments (e.g. cells, for the CSR copy of a CSC) are cut into tiles
// of 2^tshift consecutive segments, one warp per tile.  A warp walks the source
// segments (genes) in order, 32 at a time, one per lane; within such a batch a
// per-output-segment lane mask in shared memory orders the entries that land in
// the same output segment by source segment, so every output segment comes out
// sorted without a sort and without global atomics.  tile_off[t * n_major + m] is
// where source segment m's entries for tile t begin, relative to its start.

constexpr int TR_WARPS = 8;     // tiles (warps) per block
constexpr int TR_MAXT = 256;    // largest tile

// Checks the source invariants (indices in range, strictly increasing within a
// segment) and writes every source segment's tile offsets, segment-major
// (toffm[m * (n_tiles + 1) + t]: a warp's writes land next to each other).
// Warp per segment.
__global__ void k_tr_bounds(const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                            int64_t n_major, int64_t n_minor, int64_t nnz, int tshift, int64_t n_tiles,
                            int32_t* __restrict__ toffm, int* status) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t m = warp; m < n_major; m += nwarps) {
    int64_t s = ptr[m], e = ptr[m + 1];
    if (s < 0 || e < s || e > nnz || e - s > n_minor) {
      if (lane == 0) sv_flag(status, SV_STATUS_OOB);
      continue;
    }
    bool bad = false;
    // four entries per lane per step (16-byte loads from the aligned start);
    // the entry before a lane's first comes from the lane below, or from the
    // previous step's last lane
    const int64_t a0 = s & ~3ll;
    int32_t carry = -1;
    for (int64_t g0 = a0; g0 < e; g0 += 128) {
      const int64_t g = g0 + 4 * lane;
      int4 q = g < e ? *(const int4*)(idx + g) : make_int4(-1, -1, -1, -1);
      int32_t v[4] = {q.x, q.y, q.z, q.w};
      int32_t before = __shfl_up_sync(0xffffffffu, v[3], 1);
      if (lane == 0) before = carry;
      carry = __shfl_sync(0xffffffffu, v[3], 31);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t i = g + u;
        if (i < s || i >= e) continue;
        const int32_t c = v[u];
        const int32_t p = i > s ? (u ? v[u - 1] : before) : -1;
        if (c < 0 || c >= n_minor) {
          sv_flag(status, SV_STATUS_OOB);
          bad = true;
          continue;
        }
        if (i > s && c <= p) {
          sv_flag(status, SV_STATUS_UNSORTED);
          bad = true;
          continue;
        }
        int64_t tc = c >> tshift;
        int64_t tp = (p < 0 || p >= n_minor) ? -1 : (int64_t)(p >> tshift);
        for (int64_t t = tp + 1; t <= tc; ++t) toffm[m * (n_tiles + 1) + t] = (int32_t)(i - s);
      }
    }
    if (__any_sync(0xffffffffu, bad)) continue;
    int64_t last = e > s ? (int64_t)(idx[e - 1] >> tshift) : -1;
    for (int64_t t = last + 1 + lane; t <= n_tiles; t += 32) toffm[m * (n_tiles + 1) + t] = (int32_t)(e - s);
  }
}

// Segment-major tile offsets -> tile-major (the walks read one tile's offsets
// for 32 consecutive segments at a time): a 32 x 32 shared-memory transpose.
__global__ void k_tr_swap(const int32_t* __restrict__ in, int64_t rows, int64_t cols,
                          int32_t* __restrict__ out) {
  __shared__ int32_t tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.x * 32;
  for (int64_t c0 = (int64_t)blockIdx.y * 32; c0 < cols; c0 += (int64_t)gridDim.y * 32) {
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
      int64_t r = r0 + k, c = c0 + threadIdx.x;
      if (r < rows && c < cols) tile[k][threadIdx.x] = in[r * cols + c];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
      int64_t c = c0 + k, r = r0 + threadIdx.x;
      if (r < rows && c < cols) out[c * rows + r] = tile[threadIdx.x][k];
    }
    __syncthreads();
  }
}

// Entries per output segment.  Warp per tile, shared-memory counters; lane l
// walks source segment g0 + l of each batch of 32 (spreading a batch's entries
// evenly over the lanes measured slower: the walk waits on loads, not lanes).
__global__ void __launch_bounds__(TR_WARPS * 32) k_tr_count(
    const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx, int64_t n_major, int64_t n_minor,
    int tshift, int64_t n_tiles, const int32_t* __restrict__ toff, int64_t* __restrict__ seg_cnt) {
  __shared__ int cnt[TR_WARPS][TR_MAXT];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, T = 1 << tshift;
  const int64_t t = (int64_t)blockIdx.x * TR_WARPS + w;
  if (t >= n_tiles) return;
  for (int k = lane; k < T; k += 32) cnt[w][k] = 0;
  __syncwarp();
  const int64_t c0 = t << tshift;
  const int32_t* lo = toff + t * n_major;
  const int32_t* hi = lo + n_major;
  for (int64_t g0 = 0; g0 < n_major; g0 += 32) {
    int64_t g = g0 + lane;
    if (g < n_major) {
      const int64_t base = ptr[g], a = base + lo[g], b = base + hi[g];
#pragma unroll 4
      for (int64_t j = a; j < b; ++j) atomicAdd(&cnt[w][idx[j] - c0], 1);
    }
  }
  __syncwarp();
  for (int k = lane; k < T && c0 + k < n_minor; k += 32) seg_cnt[c0 + k] = cnt[w][k];
}

// Places every entry.  Warp per tile; per batch of 32·H source segments (H per
// lane) an H-word mask per output segment gives each entry its rank among the
// batch's entries of the same output segment.  Wider batches halve the batch
// count each time and lengthen each output row's run per batch, so fewer of its
// stores reach DRAM as partial sectors; with few tiles H = 1 keeps a lane's
// load chain short.  Shared memory (dynamic): per warp T masks of H words and
// T cursors.
template <int H>
__global__ void __launch_bounds__(TR_WARPS * 32) k_tr_write(
    const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx, const int32_t* __restrict__ val,
    int64_t n_major, int64_t n_minor, int tshift, int64_t n_tiles, const int32_t* __restrict__ toff,
    const int64_t* __restrict__ optr, int32_t* __restrict__ oidx, int32_t* __restrict__ oval) {
  extern __shared__ __align__(16) unsigned char tr_smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, T = 1 << tshift;
  int64_t* pos = (int64_t*)tr_smem + (size_t)w * T;
  unsigned* mask = (unsigned*)((int64_t*)tr_smem + (size_t)TR_WARPS * T) + (size_t)w * T * H;
  const int64_t t = (int64_t)blockIdx.x * TR_WARPS + w;
  if (t >= n_tiles) return;
  const int64_t c0 = t << tshift;
  for (int k = lane; k < T; k += 32) {
#pragma unroll
    for (int h = 0; h < H; ++h) mask[k * H + h] = 0u;
    pos[k] = c0 + k < n_minor ? optr[c0 + k] : 0;
  }
  __syncwarp();
  const int32_t* lo = toff + t * n_major;
  const int32_t* hi = lo + n_major;
  const unsigned bit = 1u << lane, below = bit - 1u;
  for (int64_t g0 = 0; g0 < n_major; g0 += 32 * H) {
    int64_t a[H], b[H];
#pragma unroll
    for (int h = 0; h < H; ++h) {
      int64_t g = g0 + 32 * h + lane;
      a[h] = b[h] = 0;
      if (g < n_major) {
        int64_t base = ptr[g];
        a[h] = base + lo[g];
        b[h] = base + hi[g];
      }
    }
#pragma unroll
    for (int h = 0; h < H; ++h) {
#pragma unroll 4
      for (int64_t j = a[h]; j < b[h]; ++j) atomicOr(&mask[(idx[j] - c0) * H + h], bit);
    }
    __syncwarp();
#pragma unroll
    for (int h = 0; h < H; ++h) {
      const int32_t g = (int32_t)(g0 + 32 * h + lane);
#pragma unroll 4
      for (int64_t j = a[h]; j < b[h]; ++j) {
        const int k = idx[j] - (int32_t)c0;
        const unsigned* mk = mask + k * H;
        int r = __popc(mk[h] & below);
#pragma unroll
        for (int u = 0; u < h; ++u) r += __popc(mk[u]);
        const int64_t o = pos[k] + r;
        oidx[o] = g;
        oval[o] = val[j];
      }
    }
    __syncwarp();
    for (int k = lane; k < T; k += 32) {
      int c = 0;
#pragma unroll
      for (int h = 0; h < H; ++h) {
        c += __popc(mask[k * H + h]);
        mask[k * H + h] = 0u;
      }
      pos[k] += c;
    }
    __syncwarp();
  }
}

// Bitonic sort of `n2` (power of two) 64-bit keys held in `buf` by the whole block.
__device__ void block_bitonic_u64(unsigned long long* buf, int n2) {
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        int ixj = i ^ j;
        if (ixj > i) {
          unsigned long long a = buf[i], b = buf[ixj];
          bool up = (i & k) == 0;
          if ((a > b) == up) {
            buf[i] = b;
            buf[ixj] = a;
          }
        }
      }
      __syncthreads();
    }
  }
}

// Sorts each CSR row by column.  Rows that fit `cap` keys are sorted in shared
// memory; longer rows are appended to `long_rows` for the global-memory pass.
__global__ void k_sort_rows_smem(const int64_t* __restrict__ rowptr, int64_t n_rows,
                                 int32_t* __restrict__ col, int32_t* __restrict__ cnt, int cap,
                                 int64_t* __restrict__ long_rows,
                                 unsigned long long* __restrict__ n_long) {
  extern __shared__ unsigned long long skeys[];
  for (int64_t r = blockIdx.x; r < n_rows; r += gridDim.x) {
    int64_t s = rowptr[r], e = rowptr[r + 1];
    int L = e - s < (int64_t)cap + 1 ? (int)(e - s) : cap + 1;
    if (L <= 1) continue;
    if (L > cap) {
      if (threadIdx.x == 0) long_rows[atomicAdd(n_long, 1ull)] = r;
      continue;
    }
    int n2 = 1;
    while (n2 < L) n2 <<= 1;
    for (int i = threadIdx.x; i < n2; i += blockDim.x)
      skeys[i] = i < L ? ((unsigned long long)(uint32_t)col[s + i] << 32) | (uint32_t)cnt[s + i]
                       : ~0ull;
    __syncthreads();
    block_bitonic_u64(skeys, n2);
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
      unsigned long long kv = skeys[i];
      col[s + i] = (int32_t)(kv >> 32);
      cnt[s + i] = (int32_t)(kv & 0xffffffffu);
    }
    __syncthreads();
  }
}

// Long rows: the same bitonic network on a global scratch buffer, one block per row.
__global__ void k_sort_rows_global(const int64_t* __restrict__ rowptr,
                                   const int64_t* __restrict__ long_rows, int64_t n_long,
                                   int32_t* __restrict__ col, int32_t* __restrict__ cnt,
                                   unsigned long long* __restrict__ scratch, int64_t scratch_per_block) {
  unsigned long long* buf = scratch + blockIdx.x * scratch_per_block;
  for (int64_t t = blockIdx.x; t < n_long; t += gridDim.x) {
    int64_t r = long_rows[t];
    int64_t s = rowptr[r], e = rowptr[r + 1];
    int L = (int)(e - s);
    int n2 = 1;
    while (n2 < L) n2 <<= 1;
    for (int i = threadIdx.x; i < n2; i += blockDim.x)
      buf[i] = i < L ? ((unsigned long long)(uint32_t)col[s + i] << 32) | (uint32_t)cnt[s + i] : ~0ull;
    __syncthreads();
    block_bitonic_u64(buf, n2);
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
      unsigned long long kv = buf[i];
      col[s + i] = (int32_t)(kv >> 32);
      cnt[s + i] = (int32_t)(kv & 0xffffffffu);
    }
    __syncthreads();
  }
}

// ---- synthetic negative-binomial generator -----------------------------------
struct GenParams {
  const float* mu_g;     // n_genes, already multiplied by the depth factor
  const float* s_c;      // n_cells
  const int32_t* cl;     // n_cells or null
  const float* fold;     // n_clusters x n_genes (exp of the log fold change) or null
  int64_t n_cells, n_genes;
  float phi, inv_phi;
  unsigned long long seed;
};

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// One count for (cell, gene).  Not inlined so that every kernel that samples
// runs the identical instruction sequence and the CSC and CSR copies agree.
__device__ __noinline__ int nb_sample(const GenParams p, int64_t cell, int64_t gene) {
  float mean = p.mu_g[gene] * p.s_c[cell];
  if (p.fold) mean *= p.fold[(int64_t)p.cl[cell] * p.n_genes + gene];
  unsigned long long h =
      mix64(p.seed ^ mix64((unsigned long long)cell * 0x9E3779B97F4A7C15ull + (unsigned long long)gene));
  float u = ((float)(h >> 40) + 0.5f) * (1.0f / 16777216.0f);
  // P(X = 0) = (1 + phi*mean)^(-1/phi); inversion of the NB cdf from 0 upwards
  float lp = log1pf(p.phi * mean);
  float pk = expf(-p.inv_phi * lp);
  if (u < pk) return 0;
  float ratio = (p.phi * mean) / (1.0f + p.phi * mean);
  float cum = pk;
  int k = 0;
  while (u >= cum && k < 1000000) {
    pk *= ((float)k + p.inv_phi) / (float)(k + 1) * ratio;
    k++;
    cum += pk;
    if (pk < 1e-30f && cum < u) {  // tail underflow: stop at the current count
      break;
    }
  }
  return k;
}

// Pass 1 (cells): non-zeros per cell.  One warp per cell, lanes over genes.
__global__ void k_gen_row_counts(const GenParams p, int64_t* __restrict__ row_nnz) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = warp; c < p.n_cells; c += nwarps) {
    int64_t cntv = 0;
    for (int64_t g = lane; g < p.n_genes; g += 32) cntv += nb_sample(p, c, g) > 0;
    cntv = sv_warp_sum(cntv);
    if (lane == 0) row_nnz[c] = cntv;
  }
}

// Pass 1 (genes): non-zeros per gene.  One block per gene, threads over cells.
__global__ void k_gen_col_counts(const GenParams p, int64_t* __restrict__ col_nnz) {
  __shared__ int64_t red[32];
  for (int64_t g = blockIdx.x; g < p.n_genes; g += gridDim.x) {
    int64_t cntv = 0;
    for (int64_t c = threadIdx.x; c < p.n_cells; c += blockDim.x) cntv += nb_sample(p, c, g) > 0;
    cntv = sv_warp_sum(cntv);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cntv;
    __syncthreads();
    if (threadIdx.x < 32) {
      int64_t v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0;
      v = sv_warp_sum(v);
      if (threadIdx.x == 0) col_nnz[g] = v;
    }
    __syncthreads();
  }
}

// Pass 2 (cells): write the CSR rows in gene order (warp ballot compaction).
__global__ void k_gen_write_csr(const GenParams p, const int64_t* __restrict__ rowptr,
                                int32_t* __restrict__ colidx, int32_t* __restrict__ cnt) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = warp; c < p.n_cells; c += nwarps) {
    int64_t pos = rowptr[c];
    for (int64_t g0 = 0; g0 < p.n_genes; g0 += 32) {
      int64_t g = g0 + lane;
      int v = g < p.n_genes ? nb_sample(p, c, g) : 0;
      unsigned m = __ballot_sync(0xffffffffu, v > 0);
      if (v > 0) {
        int off = __popc(m & ((1u << lane) - 1));
        colidx[pos + off] = (int32_t)g;
        cnt[pos + off] = v;
      }
      pos += __popc(m);
    }
  }
}

// Pass 2 (genes): write the CSC columns in cell order (block-wide compaction).
__global__ void k_gen_write_csc(const GenParams p, const int64_t* __restrict__ colptr,
                                int32_t* __restrict__ rowidx, int32_t* __restrict__ cnt) {
  __shared__ int wsum[32];
  __shared__ int64_t base_s;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t g = blockIdx.x; g < p.n_genes; g += gridDim.x) {
    if (threadIdx.x == 0) base_s = colptr[g];
    __syncthreads();
    for (int64_t c0 = 0; c0 < p.n_cells; c0 += blockDim.x) {
      int64_t c = c0 + threadIdx.x;
      int v = c < p.n_cells ? nb_sample(p, c, g) : 0;
      unsigned m = __ballot_sync(0xffffffffu, v > 0);
      if (lane == 0) wsum[wid] = __popc(m);
      __syncthreads();
      int before = 0, tot = 0;
      for (int w = 0; w < nw; ++w) {
        int x = wsum[w];
        if (w < wid) before += x;
        tot += x;
      }
      int64_t b = base_s;
      if (v > 0) {
        int64_t pos = b + before + __popc(m & ((1u << lane) - 1));
        rowidx[pos] = (int32_t)c;
        cnt[pos] = v;
      }
      __syncthreads();
      if (threadIdx.x == 0) base_s = b + tot;
      __syncthreads();
    }
  }
}

template <typename T>
void upload_idx(sv_context* ctx, const void* host, int64_t n, int64_t base, int64_t limit,
                int32_t* dst) {
  if (n == 0) return;
  DevBuf<T> tmp(n);
  sv_h2d(ctx, tmp.get(), host, n * sizeof(T));
  sv_launch(ctx, "counts_convert_idx", k_idx_to_i32<T>, dim3(sv_grid_for(ctx, n, 256)), dim3(256),
            0, (const T*)tmp.get(), dst, n, base, limit, ctx->d_status);
  sv_sync(ctx);
}

}  // namespace

void sv_upload_counts(sv_context* ctx, const void* host, int val_type, int64_t n, int32_t* dst) {
  if (n == 0) return;
  if (val_type == SV_I32) {
    sv_h2d(ctx, dst, host, n * 4);
    return;
  }
  size_t es = sv_elem_size(val_type);
  DevBuf<unsigned char> tmp(n * es);
  sv_h2d(ctx, tmp.get(), host, n * es);
  dim3 g(sv_grid_for(ctx, n, 256)), b(256);
  if (val_type == SV_I64)
    sv_launch(ctx, "counts_convert_val", k_count_to_i32<int64_t>, g, b, 0, (const int64_t*)tmp.get(),
              dst, n, ctx->d_status);
  else if (val_type == SV_F32)
    sv_launch(ctx, "counts_convert_val", k_count_to_i32<float>, g, b, 0, (const float*)tmp.get(), dst,
              n, ctx->d_status);
  else
    sv_launch(ctx, "counts_convert_val", k_count_to_i32<double>, g, b, 0, (const double*)tmp.get(),
              dst, n, ctx->d_status);
  sv_sync(ctx);
}

// Sorts the indices of each segment of a compressed pattern (ptr over n
// segments) in place, counts moving with their indices.  Segments that fit
// 8192 keys are sorted in shared memory, longer ones in a global pass.
void sv_sort_segments(sv_context* ctx, const int64_t* ptr, int64_t n, int32_t* idx, int32_t* cnt) {
  const int cap = 8192;
  DevBuf<int64_t> long_rows(n + 1);
  DevBuf<unsigned long long> n_long(1);
  sv_memset(ctx, n_long.get(), 0, sizeof(unsigned long long));
  SV_CUDA(cudaFuncSetAttribute(k_sort_rows_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               cap * 8));
  sv_launch(ctx, "counts_sort_rows", k_sort_rows_smem, dim3(sv_grid_for(ctx, n, 1, 16)),
            dim3(256), (size_t)cap * 8, ptr, n, idx, cnt, cap, long_rows.get(), n_long.get());
  int64_t nl = sv_read_i64(ctx, (const int64_t*)n_long.get());
  if (nl > 0) {
    // longest segment bounds the scratch per block
    std::vector<int64_t> rp(n + 1);
    sv_d2h(ctx, rp.data(), ptr, (n + 1) * sizeof(int64_t));
    int64_t maxlen = 0;
    for (int64_t r = 0; r < n; ++r) maxlen = std::max(maxlen, rp[r + 1] - rp[r]);
    int64_t n2 = 1;
    while (n2 < maxlen) n2 <<= 1;
    int blocks = (int)std::min<int64_t>(nl, (int64_t)ctx->num_sms * 2);
    DevBuf<unsigned long long> scratch((size_t)blocks * n2);
    sv_launch(ctx, "counts_sort_rows_long", k_sort_rows_global, dim3(blocks), dim3(1024), 0, ptr,
              (const int64_t*)long_rows.get(), nl, idx, cnt, scratch.get(), n2);
    sv_sync(ctx);
  }
  sv_sync(ctx);
}

// Transpose of a compressed pattern with its counts: the n_major segments of
// (ptr, idx, cnt) become n_minor segments (optr, oidx, ocnt) whose indices are
// the former segment numbers, sorted within each segment.  The source
// invariants (indices in range, strictly increasing within a segment) are
// checked on the way and reported as SV_ERR_ARG naming `where`.
void sv_transpose_counts(sv_context* ctx, int64_t n_major, int64_t n_minor, int64_t nnz,
                         const int64_t* ptr, const int32_t* idx, const int32_t* cnt,
                         DevBuf<int64_t>& optr, DevBuf<int32_t>& oidx, DevBuf<int32_t>& ocnt,
                         const char* where) {
  // tile size: enough warps to fill the device (~8 tiles per SM slot), tile
  // offsets bounded to ~2 GB
  int tshift = 8;
  while (tshift > 5 && ((n_minor + (1ll << tshift) - 1) >> tshift) < (int64_t)ctx->num_sms * 48) --tshift;
  while (tshift < 8 && (((n_minor + (1ll << tshift) - 1) >> tshift) + 1) * n_major * 4 > (2ll << 30)) ++tshift;
  const int64_t n_tiles = (n_minor + (1ll << tshift) - 1) >> tshift;
  DevBuf<int32_t> toff((size_t)(n_tiles + 1) * (size_t)n_major);
  {
    DevBuf<int32_t> toffm((size_t)(n_tiles + 1) * (size_t)n_major);
    sv_launch(ctx, "counts_transpose_bounds", k_tr_bounds, dim3(sv_grid_for(ctx, n_major * 32, 256)),
              dim3(256), 0, ptr, idx, n_major, n_minor, nnz, tshift, n_tiles, toffm.get(), ctx->d_status);
    sv_check_device_status(ctx, where);
    const int64_t ty = (n_tiles + 1 + 31) / 32;
    sv_launch(ctx, "counts_transpose_bounds", k_tr_swap, dim3((unsigned)((n_major + 31) / 32),
              (unsigned)(ty < 65535 ? ty : 65535)), dim3(32, 8), 0, (const int32_t*)toffm.get(), n_major,
              n_tiles + 1, toff.get());
  }
  const dim3 gt((unsigned)((n_tiles + TR_WARPS - 1) / TR_WARPS)), bt(TR_WARPS * 32);
  DevBuf<int64_t> seg(n_minor + 1);
  sv_launch(ctx, "counts_transpose_count", k_tr_count, gt, bt, 0, ptr, idx, n_major, n_minor, tshift,
            n_tiles, (const int32_t*)toff.get(), seg.get());
  optr.alloc(n_minor + 1);
  sv_scan_i64(ctx, seg.get(), optr.get(), n_minor);
  oidx.alloc(nnz);
  ocnt.alloc(nnz);
  // batch width: 256 source segments with many tiles, 32 with few
  const int T = 1 << tshift;
  const bool wide = n_tiles >= (int64_t)ctx->num_sms * 32;
  const int H = wide ? 8 : 1;
  const size_t smem = (size_t)TR_WARPS * T * (8 + 4 * H);
  if (wide) {
    SV_CUDA(cudaFuncSetAttribute(k_tr_write<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    sv_launch(ctx, "counts_transpose_write", k_tr_write<8>, gt, bt, smem, ptr, idx, cnt, n_major, n_minor,
              tshift, n_tiles, (const int32_t*)toff.get(), (const int64_t*)optr.get(), oidx.get(),
              ocnt.get());
  } else {
    sv_launch(ctx, "counts_transpose_write", k_tr_write<1>, gt, bt, smem, ptr, idx, cnt, n_major, n_minor,
              tshift, n_tiles, (const int32_t*)toff.get(), (const int64_t*)optr.get(), oidx.get(),
              ocnt.get());
  }
  sv_sync(ctx);
}

// Builds the CSR copy from the CSC copy already on the device.
void sv_build_csr_from_csc(sv_context* ctx, sv_counts* c) {
  sv_transpose_counts(ctx, c->n_genes, c->n_cells, c->nnz, c->csc_colptr.get(), c->csc_rowidx.get(),
                      c->csc_count.get(), c->csr_rowptr, c->csr_colidx, c->csr_count,
                      "sv_counts_upload_csc");
}

// Uploads one compressed copy (n_major segments over n_minor indices) from host
// arrays of the declared types, converting to the device layout (0-based int64
// pointers, int32 indices and counts) and checking ranges and values.
static void upload_compressed(sv_context* ctx, int64_t n_major, int64_t n_minor, int64_t nnz,
                              const void* ptr, int ptr_type, const void* idx, int idx_type,
                              const void* val, int val_type, int index_base, DevBuf<int64_t>& optr,
                              DevBuf<int32_t>& oidx, DevBuf<int32_t>& ocnt, const char* where) {
  optr.alloc(n_major + 1);
  {
    size_t es = ptr_type == SV_I32 ? 4 : 8;
    DevBuf<unsigned char> tmp((n_major + 1) * es);
    sv_h2d(ctx, tmp.get(), ptr, (n_major + 1) * es);
    dim3 g(sv_grid_for(ctx, n_major + 1, 256)), b(256);
    if (ptr_type == SV_I32)
      sv_launch(ctx, "counts_colptr", k_colptr_to_i64<int32_t>, g, b, 0, (const int32_t*)tmp.get(),
                optr.get(), n_major + 1, (int64_t)index_base);
    else
      sv_launch(ctx, "counts_colptr", k_colptr_to_i64<int64_t>, g, b, 0, (const int64_t*)tmp.get(),
                optr.get(), n_major + 1, (int64_t)index_base);
    int64_t first = sv_read_i64(ctx, optr.get());
    int64_t last = sv_read_i64(ctx, optr.get() + n_major);
    SV_REQUIRE(first == 0 && last == nnz, "%s: pointer[0] must equal index_base and pointer[end] nnz+base",
               where);
  }
  oidx.alloc(nnz);
  ocnt.alloc(nnz);
  if (idx_type == SV_I32 && index_base == 0) {
    sv_h2d(ctx, oidx.get(), idx, nnz * 4);
  } else if (idx_type == SV_I32) {
    upload_idx<int32_t>(ctx, idx, nnz, index_base, n_minor, oidx.get());
  } else {
    upload_idx<int64_t>(ctx, idx, nnz, index_base, n_minor, oidx.get());
  }
  sv_upload_counts(ctx, val, val_type, nnz, ocnt.get());
  sv_check_device_status(ctx, where);
}

static void check_upload_args(int64_t n_cells, int64_t n_genes, int64_t nnz, const void* ptr,
                              int ptr_type, const void* idx, int idx_type, const void* val,
                              int val_type, int index_base) {
  SV_REQUIRE(n_cells >= 1 && n_genes >= 1 && nnz >= 0, "bad sizes");
  SV_REQUIRE(n_cells < (1ll << 31) && n_genes < (1ll << 31), "dimension exceeds Int32 indices");
  SV_REQUIRE(ptr_type == SV_I32 || ptr_type == SV_I64, "pointer type must be SV_I32 or SV_I64");
  SV_REQUIRE(ptr_type == SV_I64 || nnz < (1ll << 31), "nnz >= 2^31 needs Int64 pointers");
  SV_REQUIRE(idx_type == SV_I32 || idx_type == SV_I64, "index type must be SV_I32 or SV_I64");
  SV_REQUIRE(val_type == SV_I32 || val_type == SV_I64 || val_type == SV_F32 || val_type == SV_F64,
             "val_type must be SV_I32, SV_I64, SV_F32 or SV_F64");
  SV_REQUIRE(index_base == 0 || index_base == 1, "index_base must be 0 or 1");
  SV_REQUIRE(ptr && (nnz == 0 || (idx && val)), "null array");
}

SV_API int sv_counts_upload_csc(sv_context* ctx, int64_t n_cells, int64_t n_genes, int64_t nnz,
                                const void* colptr, int colptr_type, const void* rowval,
                                int idx_type, const void* nzval, int val_type, int index_base,
                                sv_counts** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(out, "out is null");
  check_upload_args(n_cells, n_genes, nnz, colptr, colptr_type, rowval, idx_type, nzval, val_type,
                    index_base);
  auto* c = new sv_counts();
  try {
    c->ctx = ctx;
    c->n_cells = n_cells;
    c->n_genes = n_genes;
    c->nnz = nnz;
    upload_compressed(ctx, n_genes, n_cells, nnz, colptr, colptr_type, rowval, idx_type, nzval,
                      val_type, index_base, c->csc_colptr, c->csc_rowidx, c->csc_count,
                      "sv_counts_upload_csc");
    sv_build_csr_from_csc(ctx, c);
  } catch (...) {
    delete c;
    throw;
  }
  *out = c;
  SV_CATCH
}

SV_API int sv_counts_upload_csr(sv_context* ctx, int64_t n_cells, int64_t n_genes, int64_t nnz,
                                const void* rowptr, int rowptr_type, const void* colidx,
                                int idx_type, const void* nzval, int val_type, int index_base,
                                sv_counts** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(out, "out is null");
  check_upload_args(n_cells, n_genes, nnz, rowptr, rowptr_type, colidx, idx_type, nzval, val_type,
                    index_base);
  auto* c = new sv_counts();
  try {
    c->ctx = ctx;
    c->n_cells = n_cells;
    c->n_genes = n_genes;
    c->nnz = nnz;
    upload_compressed(ctx, n_cells, n_genes, nnz, rowptr, rowptr_type, colidx, idx_type, nzval,
                      val_type, index_base, c->csr_rowptr, c->csr_colidx, c->csr_count,
                      "sv_counts_upload_csr");
    // Files store each cell's features in the order they were written; the
    // transpose below requires them increasing, so unsorted cells are sorted.
    DevBuf<int> unsorted(1);
    sv_memset(ctx, unsorted.get(), 0, sizeof(int));
    sv_launch(ctx, "counts_check_sorted", k_seg_unsorted, dim3(sv_grid_for(ctx, n_cells * 32, 256)),
              dim3(256), 0, (const int64_t*)c->csr_rowptr.get(), (const int32_t*)c->csr_colidx.get(),
              n_cells, nnz, unsorted.get());
    int flag = 0;
    sv_d2h(ctx, &flag, unsorted.get(), sizeof(int));
    SV_REQUIRE(!(flag & 2), "sv_counts_upload_csr: row pointers are not increasing");
    if (flag) sv_sort_segments(ctx, c->csr_rowptr.get(), n_cells, c->csr_colidx.get(), c->csr_count.get());
    sv_transpose_counts(ctx, n_cells, n_genes, nnz, c->csr_rowptr.get(), c->csr_colidx.get(),
                        c->csr_count.get(), c->csc_colptr, c->csc_rowidx, c->csc_count,
                        "sv_counts_upload_csr");
  } catch (...) {
    delete c;
    throw;
  }
  *out = c;
  SV_CATCH
}

// Pattern-only upload used by sv_centered_create: "counts" hold the CSC position
// of each entry, so that after the transpose the CSR copy carries, per entry, the
// index of its value in the CSC order.
sv_counts* sv_counts_upload_positions(sv_context* ctx, int64_t n_rows, int64_t n_cols, int64_t nnz,
                                      const int64_t* colptr, const int64_t* rowval) {
  std::vector<int32_t> pos(std::max<int64_t>(1, nnz));
  for (int64_t i = 0; i < nnz; ++i) pos[i] = (int32_t)i;
  sv_counts* c = nullptr;
  int st = sv_counts_upload_csc(ctx, n_rows, n_cols, nnz, colptr, SV_I64, rowval, SV_I64, pos.data(),
                                SV_I32, 0, &c);
  if (st != SV_OK) sv_throw(st, "pattern upload failed");
  return c;
}

SV_API int sv_counts_generate(sv_context* ctx, int64_t n_cells, int64_t n_genes, const float* mu_g,
                              const float* s_c, const int32_t* cluster, const float* lfc,
                              int32_t n_clusters, double depth, double dispersion, uint64_t seed,
                              sv_counts** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(out && mu_g && s_c, "null argument");
  SV_REQUIRE(n_cells >= 1 && n_genes >= 1 && n_cells < (1ll << 31) && n_genes < (1ll << 31),
             "bad sizes");
  SV_REQUIRE(dispersion > 0, "dispersion must be > 0");
  SV_REQUIRE((n_clusters > 0) == (cluster != nullptr && lfc != nullptr),
             "cluster and lfc must both be given with n_clusters > 0");
  std::vector<float> mu_h(n_genes);
  for (int64_t g = 0; g < n_genes; ++g) mu_h[g] = (float)(mu_g[g] * depth);
  DevBuf<float> d_mu(n_genes), d_s(n_cells), d_fold;
  DevBuf<int32_t> d_cl;
  sv_h2d(ctx, d_mu.get(), mu_h.data(), n_genes * 4);
  sv_h2d(ctx, d_s.get(), s_c, n_cells * 4);
  GenParams p{};
  p.mu_g = d_mu.get();
  p.s_c = d_s.get();
  if (n_clusters > 0) {
    std::vector<float> fold((size_t)n_clusters * n_genes);
    for (size_t i = 0; i < fold.size(); ++i) fold[i] = expf(lfc[i]);
    for (int64_t i = 0; i < n_cells; ++i)
      SV_REQUIRE(cluster[i] >= 0 && cluster[i] < n_clusters, "cluster id out of range");
    d_fold.alloc(fold.size());
    d_cl.alloc(n_cells);
    sv_h2d(ctx, d_fold.get(), fold.data(), fold.size() * 4);
    sv_h2d(ctx, d_cl.get(), cluster, n_cells * 4);
    p.fold = d_fold.get();
    p.cl = d_cl.get();
  }
  p.n_cells = n_cells;
  p.n_genes = n_genes;
  p.phi = (float)dispersion;
  p.inv_phi = (float)(1.0 / dispersion);
  p.seed = seed;
  auto* c = new sv_counts();
  try {
    c->ctx = ctx;
    c->n_cells = n_cells;
    c->n_genes = n_genes;
    DevBuf<int64_t> rn(n_cells + 1), cn(n_genes + 1);
    sv_launch(ctx, "gen_row_counts", k_gen_row_counts, dim3(sv_grid_for(ctx, n_cells * 32, 256, 16)),
              dim3(256), 0, p, rn.get());
    sv_launch(ctx, "gen_col_counts", k_gen_col_counts, dim3(sv_grid_for(ctx, n_genes, 1, 8)),
              dim3(1024), 0, p, cn.get());
    c->csr_rowptr.alloc(n_cells + 1);
    c->csc_colptr.alloc(n_genes + 1);
    sv_scan_i64(ctx, rn.get(), c->csr_rowptr.get(), n_cells);
    sv_scan_i64(ctx, cn.get(), c->csc_colptr.get(), n_genes);
    int64_t nnz_r = sv_read_i64(ctx, c->csr_rowptr.get() + n_cells);
    int64_t nnz_c = sv_read_i64(ctx, c->csc_colptr.get() + n_genes);
    if (nnz_r != nnz_c)
      sv_throw(SV_ERR_DEVICE, "generator: row and column totals disagree (%lld vs %lld)",
               (long long)nnz_r, (long long)nnz_c);
    c->nnz = nnz_r;
    c->csr_colidx.alloc(c->nnz);
    c->csr_count.alloc(c->nnz);
    c->csc_rowidx.alloc(c->nnz);
    c->csc_count.alloc(c->nnz);
    sv_launch(ctx, "gen_write_csr", k_gen_write_csr, dim3(sv_grid_for(ctx, n_cells * 32, 256, 16)),
              dim3(256), 0, p, (const int64_t*)c->csr_rowptr.get(), c->csr_colidx.get(),
              c->csr_count.get());
    sv_launch(ctx, "gen_write_csc", k_gen_write_csc, dim3(sv_grid_for(ctx, n_genes, 1, 8)), dim3(1024),
              0, p, (const int64_t*)c->csc_colptr.get(), c->csc_rowidx.get(), c->csc_count.get());
    sv_sync(ctx);
  } catch (...) {
    delete c;
    throw;
  }
  *out = c;
  SV_CATCH
}

SV_API int sv_counts_info(const sv_counts* c, int64_t* n_cells, int64_t* n_genes, int64_t* nnz) {
  SV_TRY
  SV_REQUIRE(c, "null handle");
  if (n_cells) *n_cells = c->n_cells;
  if (n_genes) *n_genes = c->n_genes;
  if (nnz) *nnz = c->nnz;
  SV_CATCH
}

SV_API int sv_counts_download_csc(sv_context* ctx, const sv_counts* c, int64_t* colptr,
                                  int32_t* rowval, int32_t* counts) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(c && c->ctx == ctx, "handle does not belong to this context");
  if (colptr) sv_d2h(ctx, colptr, c->csc_colptr.get(), (c->n_genes + 1) * 8);
  if (rowval) sv_d2h(ctx, rowval, c->csc_rowidx.get(), c->nnz * 4);
  if (counts) sv_d2h(ctx, counts, c->csc_count.get(), c->nnz * 4);
  SV_CATCH
}

SV_API int sv_counts_download_csr(sv_context* ctx, const sv_counts* c, int64_t* rowptr,
                                  int32_t* colidx, int32_t* counts) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(c && c->ctx == ctx, "handle does not belong to this context");
  if (rowptr) sv_d2h(ctx, rowptr, c->csr_rowptr.get(), (c->n_cells + 1) * 8);
  if (colidx) sv_d2h(ctx, colidx, c->csr_colidx.get(), c->nnz * 4);
  if (counts) sv_d2h(ctx, counts, c->csr_count.get(), c->nnz * 4);
  SV_CATCH
}

SV_API int sv_counts_free(sv_counts* c) {
  if (c) {
    if (c->ctx) cudaSetDevice(c->ctx->device);
    delete c;
  }
  return SV_OK;
}
