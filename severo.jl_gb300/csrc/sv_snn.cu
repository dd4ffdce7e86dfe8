// Shared-nearest-neighbour graph (src/neighbours.jl:76-108,127-155,272-278).
//
// nn graph G (column j = the sorted, de-duplicated neighbours N(j) of cell j,
// neighbours.jl:79); integer counts c_ij = |N(i) & N(j)| = (G^T G)_ij
// (neighbours.jl:89, Bool x Bool accumulates to Int); weight
// w = c / (k + (k - c)) evaluated in the output type T (neighbours.jl:90-91, or
// k = |N(j)| = diag for the variant of :96-108); entries with w <= prune dropped
// (droptol!, :92).  Output: CSC, rows sorted per column.
//
// Per column j the candidate rows are the reverse neighbours of its neighbours,
// cand(j) = concat_{r in N(j)} R(r) with R(r) = {i : r in N(i)}; each i appears
// once per shared neighbour, so its count is its multiplicity in cand(j).
// Columns are processed by one warp (<= 1024 candidates), one block (<= 16384)
// or one block over a global scratch buffer (larger hubs).  The warp and block
// forms count the candidates in a shared-memory hash table (row and count
// packed in one 32-bit word, open addressing, at least 1.5 times as many slots
// as candidates), keep the entries whose weight passes the prune threshold, and
// sort only those by row; the hub form (and rows or k too large for the
// packing) sorts all candidates and reads the counts as run lengths.  Two
// passes: count the kept entries, scan, write.  All integer work; the one
// division is IEEE-correctly rounded.
#include "sv_internal.cuh"
#include <limits.h>

namespace {

constexpr int CAP_WARP = 1024;
constexpr int CAP_BLOCK = 16384;
constexpr int SNN_BLOCK = 256;
constexpr int SLOTS_WARP = 3 * CAP_WARP / 2;     // hash slots per warp (load <= 2/3)
constexpr int SLOTS_BLOCK = 3 * CAP_BLOCK / 2;   // hash slots per block

// nn (n x k row-major 0-based) -> G (n x k row-major, sorted unique, -1 padded), gcnt
__global__ void k_snn_graph(const int32_t* __restrict__ nn, int64_t n, int k,
                            int32_t* __restrict__ G, int32_t* __restrict__ gcnt,
                            unsigned long long* __restrict__ rcnt, int* status) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    int32_t* g = G + j * k;
    int m = 0;
    for (int t = 0; t < k; ++t) {
      int32_t v = nn[j * k + t];
      if (v < 0 || v >= n) {
        if (v != -1) sv_flag(status, SV_STATUS_OOB);
        continue;
      }
      // insertion into the sorted prefix, dropping duplicates (sparse() ORs them)
      int p = m;
      while (p > 0 && g[p - 1] > v) --p;
      if (p > 0 && g[p - 1] == v) continue;
      for (int q = m; q > p; --q) g[q] = g[q - 1];
      g[p] = v;
      ++m;
    }
    for (int t = m; t < k; ++t) g[t] = -1;
    gcnt[j] = m;
    for (int t = 0; t < m; ++t) atomicAdd(&rcnt[g[t]], 1ull);
  }
}

__global__ void k_u64_i64(const unsigned long long* a, int64_t* b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (int64_t)a[i];
}

__global__ void k_snn_reverse(const int32_t* __restrict__ G, const int32_t* __restrict__ gcnt,
                              int64_t n, int k, unsigned long long* __restrict__ cursor,
                              int32_t* __restrict__ rlist) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    int m = gcnt[j];
    for (int t = 0; t < m; ++t) {
      int32_t r = G[j * k + t];
      rlist[atomicAdd(&cursor[r], 1ull)] = (int32_t)j;
    }
  }
}

// candidate totals per column and classification into the three work lists
__global__ void k_snn_classify(const int32_t* __restrict__ G, const int32_t* __restrict__ gcnt,
                               const int64_t* __restrict__ rptr, int64_t n, int k,
                               int32_t* __restrict__ lists, unsigned long long* __restrict__ lcnt,
                               unsigned long long* __restrict__ maxtot) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    int m = gcnt[j];
    int64_t tot = 0;
    for (int t = 0; t < m; ++t) {
      int32_t r = G[j * k + t];
      tot += rptr[r + 1] - rptr[r];
    }
    int cls = tot <= CAP_WARP ? 0 : (tot <= CAP_BLOCK ? 1 : 2);
    unsigned long long pos = atomicAdd(&lcnt[cls], 1ull);
    lists[(int64_t)cls * n + pos] = (int32_t)j;
    if (cls == 2) atomicMax(maxtot, (unsigned long long)tot);
  }
}

struct WarpG {
  __device__ int rank() const { return threadIdx.x & 31; }
  __device__ int size() const { return 32; }
  __device__ void sync() const { __syncwarp(); }
};
struct BlockG {
  __device__ int rank() const { return threadIdx.x; }
  __device__ int size() const { return blockDim.x; }
  __device__ void sync() const { __syncthreads(); }
};

template <typename Grp>
__device__ void group_bitonic(int32_t* buf, int n2, const Grp& g) {
  for (int kk = 2; kk <= n2; kk <<= 1) {
    for (int j = kk >> 1; j > 0; j >>= 1) {
      for (int i = g.rank(); i < n2; i += g.size()) {
        int ixj = i ^ j;
        if (ixj > i) {
          int32_t a = buf[i], b = buf[ixj];
          bool up = (i & kk) == 0;
          if ((a > b) == up) {
            buf[i] = b;
            buf[ixj] = a;
          }
        }
      }
      g.sync();
    }
  }
}

// bitonic sort of n2 (a power of two) unsigned words, ascending
template <typename Grp>
__device__ void group_bitonic_u32(uint32_t* buf, int n2, const Grp& g) {
  for (int kk = 2; kk <= n2; kk <<= 1) {
    for (int j = kk >> 1; j > 0; j >>= 1) {
      for (int i = g.rank(); i < n2; i += g.size()) {
        int ixj = i ^ j;
        if (ixj > i) {
          uint32_t a = buf[i], b = buf[ixj];
          bool up = (i & kk) == 0;
          if ((a > b) == up) {
            buf[i] = b;
            buf[ixj] = a;
          }
        }
      }
      g.sync();
    }
  }
}

template <typename T>
struct Wt {
  __device__ static T w(int c, int kk) {
    T x = (T)c, kt = (T)kk;
    return x / (kt + (kt - x));   // neighbours.jl:90 (and :103)
  }
};

// Process one column with a group: gather candidates into buf, sort, count runs,
// keep w > prune.  WRITE=false: returns the kept count (valid in rank 0 for
// BlockG; in every lane for WarpG).  WRITE=true: writes rows/values at `base`.
template <typename T, bool WRITE, typename Grp>
__device__ int64_t snn_column(int64_t j, const int32_t* __restrict__ G, const int32_t* __restrict__ gcnt,
                              const int64_t* __restrict__ rptr, const int32_t* __restrict__ rlist,
                              int k, int kparam, T prune, int32_t* buf, int* wsum, const Grp& g,
                              int64_t base, int32_t* __restrict__ orow, T* __restrict__ oval) {
  int m = gcnt[j];
  // gather
  int tot = 0;
  for (int t = 0; t < m; ++t) {
    int32_t r = G[j * k + t];
    int64_t s = rptr[r], e = rptr[r + 1];
    for (int64_t q = s + g.rank(); q < e; q += g.size()) buf[tot + (q - s)] = rlist[q];
    tot += (int)(e - s);
  }
  int n2 = 1;
  while (n2 < tot) n2 <<= 1;
  for (int i = tot + g.rank(); i < n2; i += g.size()) buf[i] = INT_MAX;
  g.sync();
  group_bitonic(buf, n2, g);
  int kk = kparam >= 0 ? kparam : m;
  // runs: position p starts a run when buf[p] != buf[p-1]
  int64_t kept_total = 0;
  for (int p0 = 0; p0 < tot; p0 += g.size()) {
    int p = p0 + g.rank();
    bool keep = false;
    int32_t row = 0;
    T wv = 0;
    if (p < tot && (p == 0 || buf[p] != buf[p - 1])) {
      row = buf[p];
      int c = 1;
      while (p + c < tot && buf[p + c] == row) ++c;
      if (kparam < 0) kk = gcnt[j];
      wv = Wt<T>::w(c, kk);
      keep = wv > prune;                      // droptol!: |w| > prune kept
    }
    // group-wide exclusive prefix of `keep`
    int before, chunk;
    if (g.size() == 32) {
      unsigned msk = __ballot_sync(0xffffffffu, keep);
      before = __popc(msk & ((1u << (threadIdx.x & 31)) - 1));
      chunk = __popc(msk);
    } else {
      unsigned msk = __ballot_sync(0xffffffffu, keep);
      int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      if (lane == 0) wsum[wid] = __popc(msk);
      __syncthreads();
      before = __popc(msk & ((1u << lane) - 1));
      chunk = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        if (w < wid) before += wsum[w];
        chunk += wsum[w];
      }
      __syncthreads();
    }
    if (WRITE && keep) {
      orow[base + kept_total + before] = row;
      oval[base + kept_total + before] = wv;
    }
    kept_total += chunk;
  }
  g.sync();
  return kept_total;
}

// group-wide exclusive prefix of a flag: (before, total)
template <typename Grp>
__device__ __forceinline__ void group_prefix(bool flag, int* wsum, const Grp& g, int& before, int& chunk) {
  unsigned msk = __ballot_sync(0xffffffffu, flag);
  if (g.size() == 32) {
    before = __popc(msk & ((1u << (threadIdx.x & 31)) - 1));
    chunk = __popc(msk);
    return;
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) wsum[wid] = __popc(msk);
  __syncthreads();
  before = __popc(msk & ((1u << lane) - 1));
  chunk = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
    if (w < wid) before += wsum[w];
    chunk += wsum[w];
  }
  __syncthreads();
}

// Column j counted in a hash table `tab` of 1.5 * (candidates) slots or more:
// word = (row + 1) << cb | count (cb bits hold any count <= k; 0 = empty).
// WRITE=false: the kept count; WRITE=true: the kept entries written at `base`
// in row order.  Same weights and threshold as snn_column.
template <typename T, bool WRITE, typename Grp>
__device__ int64_t snn_column_hash(int64_t j, const int32_t* __restrict__ G, const int32_t* __restrict__ gcnt,
                                   const int64_t* __restrict__ rptr, const int32_t* __restrict__ rlist, int k,
                                   int kparam, T prune, int cb, uint32_t* tab, int* wsum, const Grp& g,
                                   int64_t base, int32_t* __restrict__ orow, T* __restrict__ oval,
                                   int* status) {
  const int m = gcnt[j];
  int tot = 0;
  for (int t = 0; t < m; ++t) {
    const int32_t r = G[j * k + t];
    tot += (int)(rptr[r + 1] - rptr[r]);
  }
  // a multiple of 32, load at most 2/3; never above the table (tot <= CAP)
  const int S = max(32, (3 * tot / 2 + 31) / 32 * 32);
  const uint32_t cmask = (1u << cb) - 1u;
  for (int i = g.rank(); i < S; i += g.size()) tab[i] = 0u;
  g.sync();
  for (int t = 0; t < m; ++t) {
    const int32_t r = G[j * k + t];
    const int64_t s0 = rptr[r], e0 = rptr[r + 1];
    for (int64_t q = s0 + g.rank(); q < e0; q += g.size()) {
      const uint32_t key = (uint32_t)rlist[q] + 1u;
      uint32_t h = __umulhi(key * 2654435761u, (uint32_t)S);
      int probes = 0;
      while (true) {
        uint32_t cur = tab[h];
        if (cur == 0u) {
          cur = atomicCAS(&tab[h], 0u, (key << cb) | 1u);
          if (cur == 0u) break;
        }
        if ((cur >> cb) == key) {
          atomicAdd(&tab[h], 1u);
          break;
        }
        h = h + 1 == (uint32_t)S ? 0u : h + 1;
        if (++probes >= S) {   // cannot happen with S > candidates
          sv_flag(status, SV_STATUS_LIMIT);
          break;
        }
      }
    }
  }
  g.sync();
  const int kk = kparam >= 0 ? kparam : m;
  // compact the kept entries to the front, in place (each chunk is read before
  // it is written, and writes land at or before the slots already read)
  int nk = 0;
  for (int c0 = 0; c0 < S; c0 += g.size()) {
    const int i = c0 + g.rank();
    const uint32_t v = i < S ? tab[i] : 0u;
    bool keep = false;
    if (v != 0u) keep = Wt<T>::w((int)(v & cmask), kk) > prune;   // droptol!: |w| > prune kept
    int before, chunk;
    group_prefix(keep, wsum, g, before, chunk);
    if (WRITE) {
      g.sync();   // every read of this chunk before any write
      if (keep) tab[nk + before] = v;
    }
    nk += chunk;
  }
  if (!WRITE) {
    g.sync();
    return nk;
  }
  int n2 = 1;
  while (n2 < nk) n2 <<= 1;
  for (int i = nk + g.rank(); i < n2; i += g.size()) tab[i] = 0xFFFFFFFFu;
  g.sync();
  group_bitonic_u32(tab, n2, g);
  for (int p = g.rank(); p < nk; p += g.size()) {
    const uint32_t v = tab[p];
    orow[base + p] = (int32_t)((v >> cb) - 1u);
    oval[base + p] = Wt<T>::w((int)(v & cmask), kk);
  }
  g.sync();
  return nk;
}

template <typename T, bool WRITE>
__global__ void __launch_bounds__(SNN_BLOCK) k_snn_warp(
    const int32_t* __restrict__ list, int64_t nlist, const int32_t* __restrict__ G,
    const int32_t* __restrict__ gcnt, const int64_t* __restrict__ rptr,
    const int32_t* __restrict__ rlist, int k, int kparam, T prune, int64_t* __restrict__ kept,
    const int64_t* __restrict__ colptr, int32_t* __restrict__ orow, T* __restrict__ oval, int cb,
    int* status) {
  extern __shared__ int32_t sbuf[];   // SLOTS_WARP words per warp
  int wid = threadIdx.x >> 5;
  int32_t* buf = sbuf + wid * SLOTS_WARP;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  WarpG g;
  for (int64_t t = warp; t < nlist; t += nwarps) {
    int64_t j = list[t];
    int64_t base = WRITE ? colptr[j] : 0;
    int64_t c = cb > 0 ? snn_column_hash<T, WRITE>(j, G, gcnt, rptr, rlist, k, kparam, prune, cb,
                                                   (uint32_t*)buf, nullptr, g, base, orow, oval, status)
                       : snn_column<T, WRITE>(j, G, gcnt, rptr, rlist, k, kparam, prune, buf, nullptr, g,
                                              base, orow, oval);
    if (!WRITE && g.rank() == 0) kept[j] = c;
  }
}

template <typename T, bool WRITE>
__global__ void __launch_bounds__(1024) k_snn_block(
    const int32_t* __restrict__ list, int64_t nlist, const int32_t* __restrict__ G,
    const int32_t* __restrict__ gcnt, const int64_t* __restrict__ rptr,
    const int32_t* __restrict__ rlist, int k, int kparam, T prune, int64_t* __restrict__ kept,
    const int64_t* __restrict__ colptr, int32_t* __restrict__ orow, T* __restrict__ oval,
    int32_t* __restrict__ gscratch, int64_t scratch_per_block, int cb, int* status) {
  extern __shared__ int32_t dbuf[];
  __shared__ int wsum[32];
  int32_t* buf = gscratch ? gscratch + blockIdx.x * scratch_per_block : dbuf;
  BlockG g;
  for (int64_t t = blockIdx.x; t < nlist; t += gridDim.x) {
    int64_t j = list[t];
    int64_t base = WRITE ? colptr[j] : 0;
    int64_t c = cb > 0 ? snn_column_hash<T, WRITE>(j, G, gcnt, rptr, rlist, k, kparam, prune, cb,
                                                   (uint32_t*)buf, wsum, g, base, orow, oval, status)
                       : snn_column<T, WRITE>(j, G, gcnt, rptr, rlist, k, kparam, prune, buf, wsum, g,
                                              base, orow, oval);
    if (!WRITE && threadIdx.x == 0) kept[j] = c;
    __syncthreads();
  }
}

template <typename T>
void snn_run(sv_context* ctx, const int32_t* nn, int64_t n, int k, int64_t kparam, double prune_d,
             sv_graph* out) {
  T prune = (T)prune_d;   // convert(T, prune)
  DevBuf<int32_t> G((size_t)n * k), gcnt(n);
  DevBuf<unsigned long long> rc(n + 1);
  sv_memset(ctx, rc.get(), 0, (n + 1) * 8);
  int gridt = sv_grid_for(ctx, n, 256, 8);
  sv_launch(ctx, "snn_graph", k_snn_graph, dim3(gridt), dim3(256), 0, nn, n, k, G.get(), gcnt.get(),
            rc.get(), ctx->d_status);
  sv_check_device_status(ctx, "snn");
  DevBuf<int64_t> rc64(n + 1), rptr(n + 1);
  sv_launch(ctx, "snn_cvt", k_u64_i64, dim3(gridt), dim3(256), 0, (const unsigned long long*)rc.get(),
            rc64.get(), n);
  sv_scan_i64(ctx, rc64.get(), rptr.get(), n);
  int64_t nent = sv_read_i64(ctx, rptr.get() + n);
  DevBuf<int32_t> rlist(std::max<int64_t>(1, nent));
  // cursors = rptr
  SV_CUDA(cudaMemcpyAsync(rc.get(), rptr.get(), n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  sv_launch(ctx, "snn_reverse", k_snn_reverse, dim3(gridt), dim3(256), 0, (const int32_t*)G.get(),
            (const int32_t*)gcnt.get(), n, k, rc.get(), rlist.get());
  DevBuf<int32_t> lists((size_t)3 * n);
  DevBuf<unsigned long long> lcnt(4);
  sv_memset(ctx, lcnt.get(), 0, 32);
  sv_launch(ctx, "snn_classify", k_snn_classify, dim3(gridt), dim3(256), 0, (const int32_t*)G.get(),
            (const int32_t*)gcnt.get(), (const int64_t*)rptr.get(), n, k, lists.get(), lcnt.get(),
            lcnt.get() + 3);
  unsigned long long hl[4];
  sv_d2h(ctx, hl, lcnt.get(), 32);
  int64_t nl[3] = {(int64_t)hl[0], (int64_t)hl[1], (int64_t)hl[2]};
  int64_t maxtot = (int64_t)hl[3];
  int64_t big_n2 = 1;
  while (big_n2 < maxtot) big_n2 <<= 1;
  int big_blocks = (int)std::min<int64_t>(std::max<int64_t>(nl[2], 1), (int64_t)ctx->num_sms);
  DevBuf<int32_t> gscratch(nl[2] > 0 ? (size_t)big_blocks * big_n2 : 1);
  DevBuf<int64_t> kept(n + 1);
  out->colptr.alloc(n + 1);
  size_t es = sizeof(T);
  // count bits of the hash words: any count <= k; rows + 1 in the remaining bits
  int cb = 32 - __builtin_clz((unsigned)k);
  if ((uint64_t)(n + 1) >= (1ull << (32 - cb))) cb = 0;   // does not fit: the sorting form
  const size_t warp_smem = (size_t)(SNN_BLOCK / 32) * SLOTS_WARP * 4;
  const size_t block_smem = (size_t)(cb > 0 ? SLOTS_BLOCK : CAP_BLOCK) * 4;
  for (auto kern : {k_snn_warp<T, false>, k_snn_warp<T, true>})
    SV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)warp_smem));
  for (auto kern : {k_snn_block<T, false>, k_snn_block<T, true>})
    SV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)block_smem));
  for (int pass = 0; pass < 2; ++pass) {
    bool W = pass == 1;
    int32_t* orow = W ? out->rowidx.get() : nullptr;
    T* oval = W ? (T*)out->val.get() : nullptr;
    const int64_t* cp = W ? (const int64_t*)out->colptr.get() : nullptr;
    int gw = sv_grid_for(ctx, nl[0] * 32, SNN_BLOCK, 4);
    int gb = (int)std::min<int64_t>(std::max<int64_t>(nl[1], 1), (int64_t)ctx->num_sms * 2);
    if (W) {
      sv_launch(ctx, "snn_columns_warp", k_snn_warp<T, true>, dim3(nl[0] ? gw : 0), dim3(SNN_BLOCK),
                warp_smem, (const int32_t*)lists.get(), nl[0], (const int32_t*)G.get(),
                (const int32_t*)gcnt.get(), (const int64_t*)rptr.get(), (const int32_t*)rlist.get(), k,
                (int)kparam, prune, kept.get(), cp, orow, oval, cb, ctx->d_status);
      sv_launch(ctx, "snn_columns_block", k_snn_block<T, true>, dim3(nl[1] ? gb : 0), dim3(1024),
                block_smem, (const int32_t*)lists.get() + n, nl[1], (const int32_t*)G.get(),
                (const int32_t*)gcnt.get(), (const int64_t*)rptr.get(), (const int32_t*)rlist.get(), k,
                (int)kparam, prune, kept.get(), cp, orow, oval, (int32_t*)nullptr, (int64_t)0, cb,
                ctx->d_status);
      sv_launch(ctx, "snn_columns_big", k_snn_block<T, true>, dim3(nl[2] ? big_blocks : 0), dim3(1024),
                (size_t)0, (const int32_t*)lists.get() + 2 * n, nl[2], (const int32_t*)G.get(),
                (const int32_t*)gcnt.get(), (const int64_t*)rptr.get(), (const int32_t*)rlist.get(), k,
                (int)kparam, prune, kept.get(), cp, orow, oval, gscratch.get(), big_n2, 0, ctx->d_status);
    } else {
      sv_launch(ctx, "snn_columns_warp", k_snn_warp<T, false>, dim3(nl[0] ? gw : 0), dim3(SNN_BLOCK),
                warp_smem, (const int32_t*)lists.get(), nl[0], (const int32_t*)G.get(),
                (const int32_t*)gcnt.get(), (const int64_t*)rptr.get(), (const int32_t*)rlist.get(), k,
                (int)kparam, prune, kept.get(), cp, orow, oval, cb, ctx->d_status);
      sv_launch(ctx, "snn_columns_block", k_snn_block<T, false>, dim3(nl[1] ? gb : 0), dim3(1024),
                block_smem, (const int32_t*)lists.get() + n, nl[1], (const int32_t*)G.get(),
                (const int32_t*)gcnt.get(), (const int64_t*)rptr.get(), (const int32_t*)rlist.get(), k,
                (int)kparam, prune, kept.get(), cp, orow, oval, (int32_t*)nullptr, (int64_t)0, cb,
                ctx->d_status);
      sv_launch(ctx, "snn_columns_big", k_snn_block<T, false>, dim3(nl[2] ? big_blocks : 0), dim3(1024),
                (size_t)0, (const int32_t*)lists.get() + 2 * n, nl[2], (const int32_t*)G.get(),
                (const int32_t*)gcnt.get(), (const int64_t*)rptr.get(), (const int32_t*)rlist.get(), k,
                (int)kparam, prune, kept.get(), cp, orow, oval, gscratch.get(), big_n2, 0, ctx->d_status);
      sv_scan_i64(ctx, kept.get(), out->colptr.get(), n);
      out->nnz = sv_read_i64(ctx, out->colptr.get() + n);
      out->rowidx.alloc(std::max<int64_t>(1, out->nnz));
      out->val.alloc(std::max<int64_t>(1, out->nnz) * es);
    }
  }
  sv_sync(ctx);
  sv_check_device_status(ctx, "snn");
}

__global__ void k_nn_from_host_layout(const int32_t* __restrict__ in, int64_t n, int k,
                                      int32_t* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * k;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e % n;
    int t = (int)(e / n);
    out[i * k + t] = in[e] - 1;   // column-major 1-based -> row-major 0-based
  }
}

__global__ void k_graph_out(const int64_t* __restrict__ cp, const int32_t* __restrict__ ri,
                            int64_t n, int64_t nnz, int64_t* __restrict__ ocp,
                            int64_t* __restrict__ ori) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n + 1 + nnz;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i <= n) {
      if (ocp) ocp[i] = cp[i] + 1;
    } else if (ori) {
      ori[i - n - 1] = (int64_t)ri[i - n - 1] + 1;
    }
  }
}

void snn_dispatch(sv_context* ctx, const int32_t* nn, int64_t n, int k, int64_t kparam, double prune,
                  int dtype, sv_graph* g) {
  g->ctx = ctx;
  g->n = n;
  g->dtype = dtype;
  if (dtype == SV_F64) snn_run<double>(ctx, nn, n, k, kparam, prune, g);
  else snn_run<float>(ctx, nn, n, k, kparam, prune, g);
}


// ---- hand-off to Louvain: Network(snn) of src/modularity.jl:163-194 ----------
// Julia's isbits layouts of Edge{T} (node::Int64, weight::T) and Node{T}
// (weight::T, edges::UnitRange{Int64}), written directly so that the caller's
// Vector{Edge{T}} / Vector{Node{T}} are filled without a host rebuild.
template <typename T>
struct JlEdge {
  int64_t node;
  T weight;
};
template <typename T>
struct JlNode {
  T weight;
  int64_t first, last;
};
static_assert(sizeof(JlEdge<double>) == 16 && sizeof(JlEdge<float>) == 16, "Edge{T} layout");
static_assert(sizeof(JlNode<double>) == 24 && sizeof(JlNode<float>) == 24, "Node{T} layout");

// non-self entries per column (rows are sorted; at most one self entry)
__global__ void k_net_count(const int64_t* __restrict__ cp, const int32_t* __restrict__ ri, int64_t n,
                            int64_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t c = 0;
    for (int64_t e = cp[i]; e < cp[i + 1]; ++e) c += ri[e] != i;
    cnt[i] = c;
  }
}

// one thread per column, in column order: the node weight is accumulated in T
// in the same order as the reference's loop (bit-identical)
template <typename T>
__global__ void k_net_write(const int64_t* __restrict__ cp, const int32_t* __restrict__ ri,
                            const T* __restrict__ val, int64_t n, const int64_t* __restrict__ off,
                            JlNode<T>* __restrict__ nodes, JlEdge<T>* __restrict__ edges) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t o = off[i];
    T w = T(0);
    for (int64_t e = cp[i]; e < cp[i + 1]; ++e) {
      if (ri[e] == i) continue;
      w += val[e];
      JlEdge<T> ed;
      ed.node = (int64_t)ri[e] + 1;
      ed.weight = val[e];
      edges[o++] = ed;
    }
    JlNode<T> nd;
    nd.weight = w;
    nd.first = off[i] + 1;
    nd.last = o;
    nodes[i] = nd;
  }
}

// totw: the sequential sum over all edges in order (the reference accumulates
// edge by edge); one warp loads 32 edges at a time, lane 0 adds them in order
template <typename T>
__global__ void k_net_total(const JlEdge<T>* __restrict__ edges, int64_t nedges, T* __restrict__ tot) {
  int lane = threadIdx.x & 31;
  T s = T(0);
  for (int64_t b = 0; b < nedges; b += 32) {
    T v = b + lane < nedges ? edges[b + lane].weight : T(0);
    int m = nedges - b < 32 ? (int)(nedges - b) : 32;
    for (int j = 0; j < m; ++j) {
      T x = __shfl_sync(0xffffffffu, v, j);
      if (lane == 0) s += x;
    }
  }
  if (lane == 0) *tot = s;
}

}  // namespace

SV_API int sv_snn_host(sv_context* ctx, const int32_t* nn_index, int64_t n, int64_t k, int64_t k_param,
                       double prune, int dtype, sv_graph** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(out && nn_index, "null argument");
  SV_REQUIRE(n >= 1 && n < (1ll << 31) && k >= 1 && k <= 1024, "bad sizes");
  SV_REQUIRE(dtype == SV_F32 || dtype == SV_F64, "dtype must be F32 or F64");
  DevBuf<int32_t> raw((size_t)n * k), nn((size_t)n * k);
  sv_h2d(ctx, raw.get(), nn_index, (size_t)n * k * 4);
  sv_launch(ctx, "snn_layout", k_nn_from_host_layout, dim3(sv_grid_for(ctx, n * k, 256, 8)), dim3(256),
            0, (const int32_t*)raw.get(), n, (int)k, nn.get());
  auto* g = new sv_graph();
  try {
    snn_dispatch(ctx, nn.get(), n, (int)k, k_param, prune, dtype, g);
  } catch (...) {
    delete g;
    throw;
  }
  *out = g;
  SV_CATCH
}

SV_API int sv_snn_knn(sv_context* ctx, const sv_knn* knn, int64_t k_param, double prune, int dtype,
                      sv_graph** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(out && knn && knn->ctx == ctx, "bad argument");
  SV_REQUIRE(dtype == SV_F32 || dtype == SV_F64, "dtype must be F32 or F64");
  auto* g = new sv_graph();
  try {
    snn_dispatch(ctx, knn->idx.get(), knn->n, (int)knn->k, k_param, prune, dtype, g);
  } catch (...) {
    delete g;
    throw;
  }
  *out = g;
  SV_CATCH
}

SV_API int sv_graph_info(const sv_graph* g, int64_t* n, int64_t* nnz) {
  SV_TRY
  SV_REQUIRE(g, "null handle");
  if (n) *n = g->n;
  if (nnz) *nnz = g->nnz;
  SV_CATCH
}

SV_API int sv_graph_download(sv_context* ctx, const sv_graph* g, int64_t* colptr, int64_t* rowval,
                             void* nzval) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(g && g->ctx == ctx, "bad handle");
  if (colptr || rowval) {
    DevBuf<int64_t> ocp(g->n + 1), ori(std::max<int64_t>(1, g->nnz));
    sv_launch(ctx, "snn_out", k_graph_out, dim3(sv_grid_for(ctx, g->n + 1 + g->nnz, 256, 8)), dim3(256),
              0, (const int64_t*)g->colptr.get(), (const int32_t*)g->rowidx.get(), g->n, g->nnz,
              colptr ? ocp.get() : (int64_t*)nullptr, rowval ? ori.get() : (int64_t*)nullptr);
    if (colptr) sv_d2h(ctx, colptr, ocp.get(), (g->n + 1) * 8);
    if (rowval) sv_d2h(ctx, rowval, ori.get(), g->nnz * 8);
  }
  if (nzval) sv_d2h(ctx, nzval, g->val.get(), g->nnz * sv_elem_size(g->dtype));
  SV_CATCH
}

SV_API int sv_graph_network(sv_context* ctx, const sv_graph* g, int64_t* nedges, void* nodes,
                            void* edges, void* totw) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(g && g->ctx == ctx, "bad handle");
  SV_REQUIRE(nedges, "nedges is required");
  DevBuf<int64_t> cnt(g->n + 1), off(g->n + 1);
  sv_launch(ctx, "snn_net_count", k_net_count, dim3(sv_grid_for(ctx, g->n, 256, 8)), dim3(256), 0,
            (const int64_t*)g->colptr.get(), (const int32_t*)g->rowidx.get(), g->n, cnt.get());
  sv_scan_i64(ctx, cnt.get(), off.get(), g->n);
  int64_t ne = sv_read_i64(ctx, off.get() + g->n);
  *nedges = ne;
  if (!nodes && !edges && !totw) return SV_OK;
  bool f64 = g->dtype == SV_F64;
  DevBuf<unsigned char> dn((size_t)g->n * 24), de((size_t)std::max<int64_t>(1, ne) * 16), dt(8);
  if (f64) {
    sv_launch(ctx, "snn_net_write", k_net_write<double>, dim3(sv_grid_for(ctx, g->n, 256, 8)), dim3(256),
              0, (const int64_t*)g->colptr.get(), (const int32_t*)g->rowidx.get(),
              (const double*)g->val.get(), g->n, (const int64_t*)off.get(), (JlNode<double>*)dn.get(),
              (JlEdge<double>*)de.get());
    sv_launch(ctx, "snn_net_total", k_net_total<double>, dim3(1), dim3(32), 0,
              (const JlEdge<double>*)de.get(), ne, (double*)dt.get());
  } else {
    sv_launch(ctx, "snn_net_write", k_net_write<float>, dim3(sv_grid_for(ctx, g->n, 256, 8)), dim3(256),
              0, (const int64_t*)g->colptr.get(), (const int32_t*)g->rowidx.get(),
              (const float*)g->val.get(), g->n, (const int64_t*)off.get(), (JlNode<float>*)dn.get(),
              (JlEdge<float>*)de.get());
    sv_launch(ctx, "snn_net_total", k_net_total<float>, dim3(1), dim3(32), 0,
              (const JlEdge<float>*)de.get(), ne, (float*)dt.get());
  }
  if (nodes) sv_d2h(ctx, nodes, dn.get(), (size_t)g->n * 24);
  if (edges) sv_d2h(ctx, edges, de.get(), (size_t)ne * 16);
  if (totw) sv_d2h(ctx, totw, dt.get(), f64 ? 8 : 4);
  sv_sync(ctx);
  SV_CATCH
}

SV_API int sv_graph_free(sv_graph* g) {
  if (g) {
    if (g->ctx) cudaSetDevice(g->ctx->device);
    delete g;
  }
  return SV_OK;
}
