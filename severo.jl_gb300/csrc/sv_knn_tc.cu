// BF16 tensor-core (tcgen05) candidate stage of the exact kNN.
//
// Distances in the GEMM form key(q, p) = |p|^2 - 2 q.p over BF16-rounded
// coordinates (K padded to 64 = one 128-byte swizzle row), FP32 accumulation in
// tensor memory.  One CTA per block of 128 queries streams every point tile of
// 256 points:
//   warp 0      TMA producer (one thread): the query tile once, point tiles into
//               a 4-stage ring (cp.async.bulk.tensor, 128B swizzle, mbarriers);
//   warp 1      MMA issuer (one thread): 4 x tcgen05.mma.kind::f16 (K = 16 each)
//               per tile into one of two 256-column TMEM accumulators;
//   warps 2..9  epilogue: tcgen05.ld of their lane quarter (= 32 queries) and
//               column half (128 points), key = |p|^2 - 2 acc, and a register
//               top-KH per (query, half): KH = 20 for k <= 20 (the 40
//               candidates of the atlas's k = 20), 32 up to k = 32.
// The 2 KH candidates per query then go through the exact FP32 re-rank
// (sv_knn.cu).  Every mbarrier wait is bounded: on a timeout the kernel records
// an error, drains its own outstanding copies and MMAs (bounded as well),
// releases its tensor memory and returns.
#include "sv_internal.cuh"
#include "sv_tc.cuh"
#include <cuda.h>
#include <float.h>

namespace {

using namespace sv_tc;

constexpr int BM = 128;            // queries per CTA (MMA M)
constexpr int BN = 256;            // points per tile (MMA N)
constexpr int BK = 64;             // padded dimension (BF16 elements, 128 bytes)
constexpr int STAGES = 4;
constexpr int EPI_WARPS = 8;
constexpr int THREADS = (2 + EPI_WARPS) * 32;
constexpr int KH_MAX = 32;         // most candidates kept per (query, column half)
constexpr long long TIMEOUT = 4000000000ll;   // cycles (~2 s) per wait
constexpr int RING = 16;           // tile-sequence slots (> STAGES + 2 tiles in flight)
constexpr uint32_t END = 0xffffffffu;   // tile id of the end-of-sequence slot

struct __align__(1024) Smem {
  __nv_bfloat16 A[BM * BK];              // 16 KB
  __nv_bfloat16 B[STAGES][BN * BK];      // 4 x 32 KB
  // per-epilogue-thread key slot for two chunks, written with 16-byte stores
  // (row stride 68 words: eight threads per wavefront on distinct banks)
  float keys[EPI_WARPS * 32][68];
  unsigned long long full[STAGES];
  unsigned long long empty[STAGES];
  unsigned long long tfull[2];
  unsigned long long tempty[2];
  unsigned long long abar;
  unsigned long long drain;
  // the tile sequence chosen by the producer: slot t % RING holds (t << 32 | tile)
  unsigned long long seq[RING];
  // per epilogue warp, the largest (threshold + |q|^2 + margin) of its queries
  float wmax[EPI_WARPS];
  uint32_t tmem_base;
  int err;
};

static_assert(sizeof(Smem) + 1024 <= 232448, "the CTA's shared memory (with the alignment slack) fits");

// The tile of sequence position t (its slot carries the tag t).  Bounded: on a
// timeout the CTA aborts and the end of the sequence is returned.
__device__ __forceinline__ uint32_t seq_tile(unsigned long long* seq, int t, int* err) {
  volatile unsigned long long* p = seq + (t & (RING - 1));
  unsigned long long v = *p;
  if ((uint32_t)(v >> 32) == (uint32_t)t) return (uint32_t)v;
  long long t0 = clock64();
  while ((uint32_t)((v = *p) >> 32) != (uint32_t)t) {
    if (*(volatile int*)err || clock64() - t0 > TIMEOUT) {
      atomicOr(err, 1);
      return END;
    }
  }
  return (uint32_t)v;
}

// Bounded wait.  Returns false when the CTA is aborting (timeout here or elsewhere).
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, uint32_t parity, int* err,
                                          long long limit = TIMEOUT) {
  if (mbar_try(b, parity)) return true;
  long long t0 = clock64();
  while (!mbar_try(b, parity)) {
    if (*(volatile int*)err) return false;
    if (clock64() - t0 > limit) {
      atomicOr(err, 1);
      return false;
    }
  }
  return true;
}

// The bounded wait on its own: one warp waits on a barrier that nothing
// arrives at, with a limit of `limit` cycles; the wait runs out, the kernel
// records SV_STATUS_LIMIT in *status and returns.  No copy or MMA is in
// flight, so nothing needs draining.
__global__ void k_wait_timeout_selftest(long long limit, int* status) {
  __shared__ unsigned long long bar;
  __shared__ int err;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    err = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (!mbar_wait(&bar, 0, &err, limit)) {
    if (threadIdx.x == 0) atomicOr(status, SV_STATUS_LIMIT);
    return;
  }
  // unreachable: nothing arrives at the barrier
}

// instruction descriptor: D f32, A/B bf16, both K-major, M = 128, N = 256
constexpr uint32_t IDESC = idesc_bf16(BM, BN);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  sv_tc::mma_bf16(d_tmem, a, b, IDESC, acc);
}

// Keys of one 32-column chunk (in place) and the mask of those below thr.
// FOLD: acc holds D = q.p - |p|^2/2; the chunk is rejected by one compare of its
// maximum (key < thr  <=>  D > -thr/2, exact: scaling by powers of two), and
// only a surviving chunk is converted to keys -2 D.  Otherwise key = |p|^2 - 2 acc.
template <bool FOLD>
__device__ __forceinline__ uint32_t chunk_mask(float (&acc)[32], const float* __restrict__ pn, int64_t col0,
                                               int64_t n, float thr) {
  uint32_t m = 0;
  if constexpr (FOLD) {
    // columns past the last point read zero rows (TMA fill): never candidates
    if (col0 + 32 > n) {
#pragma unroll
      for (int i = 0; i < 32; ++i)
        if (col0 + i >= n) acc[i] = -FLT_MAX;
    }
    float thrD = -0.5f * thr;
    float t16[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) t16[i] = fmaxf(acc[2 * i], acc[2 * i + 1]);
#pragma unroll
    for (int w2 = 8; w2 >= 1; w2 >>= 1)
#pragma unroll
      for (int i = 0; i < w2; ++i) t16[i] = fmaxf(t16[i], t16[i + w2]);
    if (t16[0] > thrD) {
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        acc[i] = -2.0f * acc[i];
        m |= (acc[i] < thr ? 1u : 0u) << i;
      }
    }
  } else {
    const float4* np = (const float4*)pn;   // squared norms of the chunk's points (padded)
#pragma unroll
    for (int i4 = 0; i4 < 8; ++i4) {
      float4 v = __ldg(np + i4);
      float pv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        int i = 4 * i4 + u;
        acc[i] = fmaf(-2.0f, acc[i], pv[u]);
        m |= (acc[i] < thr ? 1u : 0u) << i;
      }
    }
    // columns past the point range (another sample's points) are no candidates
    if (col0 + 32 > n) m &= col0 >= n ? 0u : (0xffffffffu >> (32 - (int)(n - col0)));
  }
  return m;
}

// The j-th point tile a CTA visits: with the points in locality order, the
// tiles nearest to the CTA's own queries first (alternately above and below),
// so that the top-k thresholds fall early and later tiles rarely hold a
// candidate; otherwise in order.
__device__ __forceinline__ int tile_at(int j, int t0, int ntiles, bool around) {
  if (!around) return j;
  int L = t0, R = ntiles - 1 - t0, k = min(L, R);
  if (j == 0) return t0;
  if (j <= 2 * k) {
    int m = (j + 1) >> 1;
    return (j & 1) ? t0 + m : t0 - m;
  }
  return R > L ? t0 + (j - k) : t0 - (j - k);
}

// FOLD: |p|^2 is part of the MMA (see k_pack_fold): the accumulator is
// D = q.p - |p|^2 / 2 and key = -2 D, so no norm is loaded in the epilogue and a
// 32-candidate chunk is rejected by one compare of its maximum D.
template <bool FOLD, int KH>
__global__ void __launch_bounds__(THREADS, 1)
    k_knn_tc(const __grid_constant__ CUtensorMap tmapA, const __grid_constant__ CUtensorMap tmapB,
             const float* __restrict__ sqpad, int64_t n, int ntiles, int32_t* __restrict__ cand,
             int* __restrict__ status, const int64_t* __restrict__ sched, int around,
             const float* __restrict__ coord, const float* __restrict__ nrm,
             const unsigned* __restrict__ pmax) {
  extern __shared__ unsigned char smem_raw[];
  Smem* s = (Smem*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // queries q0 .. min(q0 + BM, qend) against the points [p0, pend): the whole
  // set, or one sample of stacked samples (sched: 4 values per CTA)
  int64_t q0 = (int64_t)blockIdx.x * BM, qend = n, p0 = 0, pend = n;
  if (sched) {
    q0 = sched[4 * blockIdx.x];
    qend = sched[4 * blockIdx.x + 1];
    p0 = sched[4 * blockIdx.x + 2];
    pend = sched[4 * blockIdx.x + 3];
    ntiles = (int)((pend - p0 + BN - 1) / BN);
  }
  // the point tile that holds this CTA's first query
  int64_t tq = (q0 - p0) / BN;
  const int t0 = tq < 0 ? 0 : (tq > ntiles - 1 ? ntiles - 1 : (int)tq);

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&s->full[i], 1);
      mbar_init(&s->empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&s->tfull[i], 1);
      mbar_init(&s->tempty[i], EPI_WARPS);
    }
    mbar_init(&s->abar, 1);
    mbar_init(&s->drain, 1);
    for (int i = 0; i < RING; ++i) s->seq[i] = ~0ull;
    for (int i = 0; i < EPI_WARPS; ++i) s->wmax[i] = __int_as_float(0x7f800000);
    s->err = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     su32(&s->tmem_base)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  uint32_t tmem = s->tmem_base;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    // Chooses the tile sequence.  With the points in locality order (coord: the
    // sort coordinate of every point, as the BF16 operand holds it) a tile whose
    // coordinate gap to this CTA's queries already exceeds every query's
    // current threshold is skipped, and so is every tile beyond it: the squared
    // gap bounds the squared distance of the operands from below.
    if (lane == 0) {
      int issued = 0;
      bool ok = true;
      mbar_expect_tx(&s->abar, BM * BK * 2);
      tma_load_2d(s->A, &tmapA, 0, (int)q0, &s->abar);
      const bool prune = coord != nullptr;
      float qlo = 0.f, qhi = 0.f;
      if (prune) {
        int64_t ql = q0 + BM < qend ? q0 + BM : qend;
        qlo = coord[q0];
        qhi = coord[ql - 1];
      }
      int up = t0 + 1, dn = t0 - 1;
      // first coordinate of the next tile above, last of the next tile below
      // (loaded one step ahead of their use)
      auto lo_of = [&](int u) { return u < ntiles ? coord[p0 + (int64_t)u * BN] : 0.f; };
      auto hi_of = [&](int v) {
        int64_t hi = p0 + (int64_t)(v + 1) * BN;
        return v >= 0 ? coord[(hi < pend ? hi : pend) - 1] : 0.f;
      };
      float lo_up = prune ? lo_of(up) : 0.f, hi_dn = prune ? hi_of(dn) : 0.f;
      bool turn_up = true;
      int t = 0;
      for (;; ++t) {
        int tile;
        if (!prune) {
          if (t >= ntiles) break;
          tile = tile_at(t, t0, ntiles, around);
        } else if (t == 0) {
          tile = t0;
        } else {
          volatile float* wm = s->wmax;
          float T = wm[0];
#pragma unroll
          for (int e = 1; e < EPI_WARPS; ++e) T = fmaxf(T, wm[e]);
          bool uo = up < ntiles, dok = dn >= 0;
          if (uo) {
            float g = lo_up - qhi;
            if (g > 0.f && g * g > T) uo = false;
          }
          if (dok) {
            float g = qlo - hi_dn;
            if (g > 0.f && g * g > T) dok = false;
          }
          if (!uo) up = ntiles;   // the gap only grows further out
          if (!dok) dn = -1;
          if (!uo && !dok) break;
          bool go_up = uo && (!dok || turn_up);
          if (uo && dok) turn_up = !turn_up;
          if (go_up) {
            tile = up++;
            lo_up = lo_of(up);
          } else {
            tile = dn--;
            hi_dn = hi_of(dn);
          }
        }
        int st = t % STAGES;
        uint32_t ph = (t / STAGES) & 1;
        if (!mbar_wait(&s->empty[st], ph ^ 1, &s->err)) {
          ok = false;
          break;
        }
        ((volatile unsigned long long*)s->seq)[t & (RING - 1)] = ((unsigned long long)t << 32) | (uint32_t)tile;
        mbar_expect_tx(&s->full[st], BN * BK * 2);
        tma_load_2d(s->B[st], &tmapB, 0, (int)(p0 + (int64_t)tile * BN), &s->full[st]);
        issued = t + 1;
      }
      // end of the sequence: a stage that completes without a copy
      bool sent = false;
      if (ok) {
        int st = issued % STAGES;
        uint32_t ph = (issued / STAGES) & 1;
        if (mbar_wait(&s->empty[st], ph ^ 1, &s->err)) {
          ((volatile unsigned long long*)s->seq)[issued & (RING - 1)] =
              ((unsigned long long)issued << 32) | END;
          mbar_arrive(&s->full[st]);
          sent = true;
        }
      }
      // drain: every issued copy has landed before the CTA may exit (the tile
      // that shared the end slot's stage was consumed before the end was written)
      {
        long long c0 = clock64();
        while (!mbar_try(&s->abar, 0) && clock64() - c0 < TIMEOUT) {
        }
      }
      int first = issued - STAGES + (sent ? 1 : 0);
      for (int tt = first < 0 ? 0 : first; tt < issued; ++tt) {
        int st = tt % STAGES;
        uint32_t ph = (tt / STAGES) & 1;
        long long c0 = clock64();
        while (!mbar_try(&s->full[st], ph) && clock64() - c0 < TIMEOUT) {
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      bool ok = mbar_wait(&s->abar, 0, &s->err);
      uint32_t a_base = su32(s->A);
      for (int t = 0; ok; ++t) {
        int st = t % STAGES;
        uint32_t ph = (t / STAGES) & 1;
        int ab = t & 1;
        uint32_t aph = (t >> 1) & 1;
        if (!mbar_wait(&s->tempty[ab], aph ^ 1, &s->err)) break;
        if (!mbar_wait(&s->full[st], ph, &s->err)) break;
        if (seq_tile(s->seq, t, &s->err) == END) {
          mbar_arrive(&s->tfull[ab]);   // the epilogue reads the end too
          break;
        }
        fence_after();
        uint32_t b_base = su32(s->B[st]);
        uint32_t d = tmem + (uint32_t)(ab * BN);
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk)
          mma_bf16(d, sw128_desc(a_base + kk * 32), sw128_desc(b_base + kk * 32), kk > 0 ? 1u : 0u);
        mma_commit(&s->empty[st]);
        mma_commit(&s->tfull[ab]);
      }
      // all MMAs issued by this thread complete before the drain barrier fires
      mma_commit(&s->drain);
      long long t0 = clock64();
      while (!mbar_try(&s->drain, 0) && clock64() - t0 < TIMEOUT) {
      }
    }
  } else {
    // ---------------- epilogue ----------------
    int ew = warp - 2;
    int quarter = warp & 3;            // TMEM lane quarter this warp may access
    int half = ew >> 2;                // column half: warps 2..5 -> 0, 6..9 -> 1
    int row = quarter * 32 + lane;
    int64_t q = q0 + row;
    float best[KH];
    int bidx[KH];
#pragma unroll
    for (int i = 0; i < KH; ++i) {
      best[i] = FLT_MAX;
      bidx[i] = -1;
    }
    uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
    // pruning bound of this query: threshold + |q|^2 + a margin for the FP32
    // accumulation of the MMA (2^-15 (|q|^2 + max |p|^2), several times its bound)
    float qn = 0.f;
    if (coord && q < qend) qn = nrm[q] + 0x1p-15f * (nrm[q] + __uint_as_float(*pmax));
    for (int t = 0;; ++t) {
      int ab = t & 1;
      uint32_t aph = (t >> 1) & 1;
      bool ok = mbar_wait(&s->tfull[ab], aph, &s->err);
      if (!__all_sync(0xffffffffu, ok)) break;   // warp-uniform: the TMEM loads are .aligned
      fence_after();
      const uint32_t tile = seq_tile(s->seq, t, &s->err);
      if (__any_sync(0xffffffffu, tile == END)) break;   // warp-uniform (a timed-out lane sees END)
      int64_t j0 = p0 + (int64_t)tile * BN + half * (BN / 2);
      uint32_t tbase = tmem + lane_off + (uint32_t)(ab * BN + half * (BN / 2));
      // two chunks per TMEM round trip: both loads are issued before one wait
#pragma unroll 1
      for (int c = 0; c < BN / 2 / 32; c += 2) {
        uint32_t r0[32], r1[32];
        float a0[32], a1[32];
        __syncwarp();
        tmem_ld32(tbase + c * 32, r0);
        tmem_ld32(tbase + (c + 1) * 32, r1);
        tmem_ld_wait();
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          a0[i] = __uint_as_float(r0[i]);
          a1[i] = __uint_as_float(r1[i]);
        }
        if (c + 2 == BN / 2 / 32) {
          // accumulator values are in registers: release the buffer to the MMA warp
          fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&s->tempty[ab]);
        }
        float thr = best[KH - 1];
        int64_t cbase = j0 + c * 32;
        uint32_t m0 = chunk_mask<FOLD>(a0, sqpad + cbase, cbase, pend, thr);
        uint32_t m1 = chunk_mask<FOLD>(a1, sqpad + cbase + 32, cbase + 32, pend, thr);
        if (m0 | m1) {
          // rare: park the keys in this thread's shared slot and insert one by one
          // (one copy of the insertion code keeps the loop small in the I-cache)
          float* slot = s->keys[threadIdx.x - 64];
          // (parking is not rare per warp: with 32 queries a warp, about half of
          // the chunk pairs have a candidate for some query)
          if (m0) {
#pragma unroll
            for (int i = 0; i < 32; i += 4)
              *(float4*)(slot + i) = make_float4(a0[i], a0[i + 1], a0[i + 2], a0[i + 3]);
          }
          if (m1) {
#pragma unroll
            for (int i = 0; i < 32; i += 4)
              *(float4*)(slot + 32 + i) = make_float4(a1[i], a1[i + 1], a1[i + 2], a1[i + 3]);
          }
          unsigned long long m = (unsigned long long)m0 | ((unsigned long long)m1 << 32);
          while (m) {
            int i = __ffsll((long long)m) - 1;
            m &= m - 1;
            float cd = slot[i];
            if (!(cd < best[KH - 1])) continue;
            int ci = (int)(cbase + i);
#pragma unroll
            for (int u = 0; u < KH; ++u) {
              if (cd < best[u]) {
                float tf = best[u];
                int ti = bidx[u];
                best[u] = cd;
                bidx[u] = ci;
                cd = tf;
                ci = ti;
              }
            }
          }
        }
      }
      if (coord && (t & 3) == 3) {
        // every fourth tile; keys only fall, so a stale (larger) bound read by
        // the producer is safe
        float v = q < qend ? best[KH - 1] + qn : -FLT_MAX;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) ((volatile float*)s->wmax)[ew] = v;
      }
    }
    if (q < qend) {
      int32_t* o = cand + q * (2 * KH) + half * KH;
#pragma unroll
      for (int i = 0; i < KH; ++i) o[i] = (bidx[i] >= p0 && bidx[i] < pend) ? bidx[i] : -1;
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512)
                 : "memory");
  }
  if (threadIdx.x == 0 && s->err) atomicOr(status, SV_STATUS_LIMIT);
}

// FP32 row-major [n][dp] -> BF16 row-major [n][64] (zero padded) and the FP32 squared
// norms of the rounded rows, padded with FLT_MAX up to npad.
__global__ void k_pack_bf16(const float* __restrict__ X, int64_t n, int dp, int64_t npad,
                            __nv_bfloat16* __restrict__ Xb, float* __restrict__ sq,
                            const int* __restrict__ perm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npad;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i >= n) {
      sq[i] = FLT_MAX;
      continue;
    }
    float s = 0.f;
    const int64_t src = perm ? perm[i] : i;
    for (int c = 0; c < BK; ++c) {
      float v = c < dp ? X[src * dp + c] : 0.f;
      __nv_bfloat16 b = __float2bfloat16_rn(v);
      Xb[i * BK + c] = b;
      float r = __bfloat162float(b);
      s = fmaf(r, r, s);
    }
    sq[i] = s;
  }
}

// Operands with |p|^2 folded into the product (d + 3 <= 64): queries carry -1/2 in
// columns d..d+2, points carry |p|^2 split into three BF16 parts (hi, mid, lo,
// summing to the FP32 norm of the rounded row to ~2^-24), so that the MMA yields
// D = q.p - |p|^2/2 and the key |p|^2 - 2 q.p is -2 D.
// With coord: also the sort coordinate (column dim) and |p|^2 of the BF16
// operand row, and the largest |p|^2 (float bits; all values >= 0).
__global__ void k_pack_fold(const float* __restrict__ X, int64_t n, int dp, int d,
                            __nv_bfloat16* __restrict__ Xq, __nv_bfloat16* __restrict__ Xp,
                            const int* __restrict__ perm, int dim, float* __restrict__ coord,
                            float* __restrict__ nrm, unsigned* __restrict__ pmax) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    const int64_t src = perm ? perm[i] : i;
    for (int c = 0; c < BK; ++c) {
      float v = c < d ? X[src * dp + c] : 0.f;
      __nv_bfloat16 b = __float2bfloat16_rn(v);
      Xq[i * BK + c] = b;
      Xp[i * BK + c] = b;
      float r = __bfloat162float(b);
      s = fmaf(r, r, s);
    }
    if (coord) {
      coord[i] = __bfloat162float(__float2bfloat16_rn(X[src * dp + dim]));
      nrm[i] = s;
      atomicMax(pmax, __float_as_uint(s));
    }
    __nv_bfloat16 p1 = __float2bfloat16_rn(s);
    float r1 = s - __bfloat162float(p1);
    __nv_bfloat16 p2 = __float2bfloat16_rn(r1);
    __nv_bfloat16 p3 = __float2bfloat16_rn(r1 - __bfloat162float(p2));
    __nv_bfloat16 mh = __float2bfloat16_rn(-0.5f);
    Xq[i * BK + d] = mh;
    Xq[i * BK + d + 1] = mh;
    Xq[i * BK + d + 2] = mh;
    Xp[i * BK + d] = p1;
    Xp[i * BK + d + 1] = p2;
    Xp[i * BK + d + 2] = p3;
  }
}

// ---- locality order of the points ----------------------------------------------
// Per-dimension sums and sums of squares (FP64, atomics: only the choice of the
// widest dimension depends on them).
__global__ void k_dim_moments(const float* __restrict__ X, int64_t n, int dp, double* __restrict__ acc) {
  __shared__ double s1[256], s2[256];
  const int c = threadIdx.x % dp, r0 = threadIdx.x / dp, rstep = blockDim.x / dp;
  double a = 0, b = 0;
  if (r0 < rstep)
    for (int64_t i = blockIdx.x * (int64_t)rstep + r0; i < n; i += (int64_t)gridDim.x * rstep) {
      double v = X[i * dp + c];
      a += v;
      b += v * v;
    }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  __syncthreads();
  if (threadIdx.x < dp) {
    double ta = 0, tb = 0;
    for (int r = 0; r < rstep; ++r) {
      ta += s1[r * dp + threadIdx.x];
      tb += s2[r * dp + threadIdx.x];
    }
    atomicAdd(acc + threadIdx.x, ta);
    atomicAdd(acc + dp + threadIdx.x, tb);
  }
}

// sort key: sample in the high word, the coordinate (order-preserving bits) low
__global__ void k_locality_keys(const float* __restrict__ X, int dp, int dim, const int64_t* __restrict__ off,
                                int nseg, int64_t n, unsigned long long* __restrict__ key, int* __restrict__ val) {
  const int sg = blockIdx.y;
  const int64_t a = off ? off[sg] : 0, b = off ? off[sg + 1] : n;
  for (int64_t i = a + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < b;
       i += (int64_t)gridDim.x * blockDim.x) {
    unsigned u = __float_as_uint(X[i * dp + dim]);
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    key[i] = ((unsigned long long)sg << 32) | u;
    val[i] = (int)i;
  }
}

// candidates found in locality order -> original point and query indices
__global__ void k_cand_unperm(const int32_t* __restrict__ cs, const int* __restrict__ perm, int64_t n, int K2,
                              int32_t* __restrict__ co) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * K2;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t q = e / K2;
    int t = (int)(e - q * K2);
    int32_t c = cs[e];
    co[(int64_t)perm[q] * K2 + t] = c >= 0 ? perm[c] : -1;
  }
}

}  // namespace

int sv_knn_tc_candidates(sv_context* ctx, const float* X32, const float* sq_unused, int64_t n, int dp,
                         int d, int K2, int include_self, int32_t* cand, const std::vector<int64_t>* segs) {
  (void)sq_unused;
  (void)include_self;   // the re-rank places or removes the point itself
  try {
    if (dp > BK) sv_throw(SV_ERR_UNSUPPORTED, "tensor-core kNN handles up to %d dimensions", BK);
    if (K2 != 40 && K2 != 2 * KH_MAX)
      sv_throw(SV_ERR_UNSUPPORTED, "tensor-core kNN keeps 40 or %d candidates", 2 * KH_MAX);
    if (n >= (1ll << 31) - BN) sv_throw(SV_ERR_UNSUPPORTED, "too many points");
    int ntiles = (int)((n + BN - 1) / BN);
    // one spare tile of padding: a sample's last tile may start anywhere
    int64_t npad = (int64_t)(ntiles + 1) * BN;
    bool fold = d + 3 <= BK && !getenv("SV_KNN_NOFOLD");
    // locality order: the points sorted (within each sample) along their widest
    // dimension, and every CTA visiting the tiles around its own queries first
    bool around = !getenv("SV_KNN_NOSORT") && n >= 4 * BN;
    // tiles beyond every query's reach are skipped (locality order, folded norms)
    const bool prune = around && fold && !getenv("SV_KNN_NOPRUNE");
    DevBuf<int> perm;
    int dim = 0;
    if (around) {
      int nseg = segs ? (int)segs->size() - 1 : 1;
      DevBuf<double> mom(2 * dp);
      sv_memset(ctx, mom.get(), 0, 2 * dp * 8);
      sv_launch(ctx, "knn_order", k_dim_moments, dim3(sv_grid_for(ctx, n, 256, 2)), dim3(256 / dp * dp), 0,
                X32, n, dp, mom.get());
      std::vector<double> hm(2 * dp);
      sv_d2h(ctx, hm.data(), mom.get(), 2 * dp * 8);
      double best = -1;
      for (int c = 0; c < d; ++c) {
        double mean = hm[c] / (double)n, var = hm[dp + c] / (double)n - mean * mean;
        if (var > best) {
          best = var;
          dim = c;
        }
      }
      int64_t n2 = 2048;
      while (n2 < n) n2 <<= 1;
      DevBuf<unsigned long long> key(n2);
      perm.alloc(n2);
      DevBuf<int64_t> doff;
      if (segs) {
        doff.alloc(segs->size());
        sv_h2d(ctx, doff.get(), segs->data(), segs->size() * 8);
      }
      dim3 kg((unsigned)sv_grid_for(ctx, segs ? n / nseg + 1 : n, 256, 4), (unsigned)nseg);
      sv_launch(ctx, "knn_order", k_locality_keys, kg, dim3(256), 0, X32, dp, dim,
                segs ? (const int64_t*)doff.get() : (const int64_t*)nullptr, nseg, n, key.get(), perm.get());
      sv_sort_pairs(ctx, key.get(), perm.get(), n, n2);
    }
    const int* pm = around ? (const int*)perm.get() : (const int*)nullptr;
    DevBuf<__nv_bfloat16> Xq((size_t)n * BK), Xp;
    DevBuf<float> sq(npad);
    DevBuf<float> coord, nrm;
    DevBuf<unsigned> pmax;
    if (prune) {
      coord.alloc(n);
      nrm.alloc(n);
      pmax.alloc(1);
      sv_memset(ctx, pmax.get(), 0, sizeof(unsigned));
    }
    if (fold) {
      Xp.alloc((size_t)n * BK);
      sv_launch(ctx, "knn_pack_fold", k_pack_fold, dim3(sv_grid_for(ctx, n, 256, 8)), dim3(256), 0, X32,
                n, dp, d, Xq.get(), Xp.get(), pm, dim, coord.get(), nrm.get(), pmax.get());
    } else {
      sv_launch(ctx, "knn_pack_bf16", k_pack_bf16, dim3(sv_grid_for(ctx, npad, 256, 8)), dim3(256), 0,
                X32, n, dp, npad, Xq.get(), sq.get(), pm);
    }
    DevBuf<int32_t> cand_sorted(around ? (size_t)n * K2 : 1);
    int32_t* cout = around ? cand_sorted.get() : cand;
    // row-major BF16 operands, 64 elements (128 bytes, one swizzle row) wide: the
    // query box is 128 rows, the point box 256 rows
    CUtensorMap tmapA, tmapB;
    cuuint64_t gdim[2] = {(cuuint64_t)BK, (cuuint64_t)n};
    cuuint64_t gstride[1] = {(cuuint64_t)BK * 2};
    cuuint32_t boxA[2] = {(cuuint32_t)BK, (cuuint32_t)BM};
    cuuint32_t boxB[2] = {(cuuint32_t)BK, (cuuint32_t)BN};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = sv_encode_tiled()(&tmapA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, Xq.get(), gdim, gstride,
                             boxA, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) sv_throw(SV_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    r = sv_encode_tiled()(&tmapB, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, fold ? Xp.get() : Xq.get(), gdim,
                    gstride, boxB, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) sv_throw(SV_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    size_t smem = sizeof(Smem) + 1024;
    int nblocks = (int)((n + BM - 1) / BM);
    // stacked samples: every CTA takes 128 queries of one sample against that
    // sample's points
    DevBuf<int64_t> sched;
    if (segs) {
      std::vector<int64_t> hs;
      for (size_t g = 0; g + 1 < segs->size(); ++g)
        for (int64_t q = (*segs)[g]; q < (*segs)[g + 1]; q += BM) {
          hs.push_back(q);
          hs.push_back((*segs)[g + 1]);
          hs.push_back((*segs)[g]);
          hs.push_back((*segs)[g + 1]);
        }
      nblocks = (int)(hs.size() / 4);
      sched.alloc(hs.size());
      sv_h2d(ctx, sched.get(), hs.data(), hs.size() * 8);
    }
#define KNN_TC(FOLD, KHV, CO, NR, PM)                                                                \
  do {                                                                                              \
    SV_CUDA(cudaFuncSetAttribute(k_knn_tc<FOLD, KHV>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                 (int)smem));                                                       \
    sv_launch(ctx, "knn_tc_tiles", k_knn_tc<FOLD, KHV>, dim3(nblocks), dim3(THREADS), smem, tmapA,   \
              tmapB, (const float*)sq.get(), n, ntiles, cout, ctx->d_status,                        \
              (const int64_t*)sched.get(), (int)around, CO, NR, PM);                               \
  } while (0)
    // 20 candidates per column half (40 per query) for k <= 20, else 32
    if (fold) {
      if (K2 == 40)
        KNN_TC(true, 20, (const float*)coord.get(), (const float*)nrm.get(), (const unsigned*)pmax.get());
      else
        KNN_TC(true, 32, (const float*)coord.get(), (const float*)nrm.get(), (const unsigned*)pmax.get());
    } else {
      if (K2 == 40)
        KNN_TC(false, 20, (const float*)nullptr, (const float*)nullptr, (const unsigned*)nullptr);
      else
        KNN_TC(false, 32, (const float*)nullptr, (const float*)nullptr, (const unsigned*)nullptr);
    }
#undef KNN_TC
    if (around)
      sv_launch(ctx, "knn_unperm", k_cand_unperm, dim3(sv_grid_for(ctx, n * K2, 256, 8)), dim3(256), 0,
                (const int32_t*)cand_sorted.get(), pm, n, K2, cand);
    sv_check_device_status(ctx, "tensor-core kNN");
  } catch (const SvError& e) {
    return e.code;
  }
  return SV_OK;
}

// Runs the bounded mbarrier wait of the tensor-core kNN kernel against a
// barrier that never completes, with a limit of `cycles` clock cycles
// (1 .. 2^32); returns SV_ERR_DEVICE (the wait ran out, recorded through the
// context's status word) with the context still usable.  A self-test of the
// timeout path that needs no fault: no copy or MMA is involved.
SV_API int sv_selftest_wait_timeout(sv_context* ctx, long long cycles) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(cycles >= 1 && cycles <= (1ll << 32), "cycles out of range");
  sv_launch(ctx, "selftest_wait_timeout", k_wait_timeout_selftest, dim3(1), dim3(32), 0, cycles,
            ctx->d_status);
  sv_check_device_status(ctx, "sv_selftest_wait_timeout");
  SV_CATCH
}
