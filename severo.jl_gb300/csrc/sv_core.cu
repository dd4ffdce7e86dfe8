// Context, error reporting, profiling, pinned-memory helpers and the device-wide
// scan used by the other translation units.
#include "sv_internal.cuh"

#include <thread>
#include <stdarg.h>

static thread_local std::string g_last_error;

void sv_set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  if (getenv("SV_LOG")) fprintf(stderr, "[severo_gpu] %s\n", buf);
}

void sv_throw(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  if (getenv("SV_LOG")) fprintf(stderr, "[severo_gpu] %s\n", buf);
  throw SvError{code};
}

SV_API int sv_version(void) { return 100; }

SV_API int sv_last_error(char* buf, size_t len) {
  if (buf && len) {
    size_t n = g_last_error.size() < len - 1 ? g_last_error.size() : len - 1;
    memcpy(buf, g_last_error.data(), n);
    buf[n] = 0;
  }
  return (int)g_last_error.size();
}

void sv_ctx_check(sv_context* ctx) {
  if (!ctx) sv_throw(SV_ERR_ARG, "null context");
  SV_CUDA(cudaSetDevice(ctx->device));
}

cudaEvent_t sv_ctx_event(sv_context* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  SV_CUDA(cudaEventCreate(&e));
  return e;
}

void sv_ctx_harvest(sv_context* ctx) {
  if (ctx->pending.empty()) return;
  SV_CUDA(cudaStreamSynchronize(ctx->stream));
  for (auto& t : ctx->pending) {
    float ms = 0.f;
    SV_CUDA(cudaEventElapsedTime(&ms, t.a, t.b));
    auto& slot = ctx->prof[t.name];
    slot.first += ms;
    slot.second += 1;
    ctx->event_pool.push_back(t.a);
    ctx->event_pool.push_back(t.b);
  }
  ctx->pending.clear();
}

void* sv_ctx_stage(sv_context* ctx, size_t bytes) {
  if (bytes > ctx->h_stage_bytes) {
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    ctx->h_stage = nullptr;
    size_t b = bytes < 4096 ? 4096 : bytes;
    SV_CUDA(cudaMallocHost(&ctx->h_stage, b));
    ctx->h_stage_bytes = b;
  }
  return ctx->h_stage;
}

void sv_sync(sv_context* ctx) { SV_CUDA(cudaStreamSynchronize(ctx->stream)); }

void sv_memset(sv_context* ctx, void* p, int v, size_t bytes) {
  if (bytes) SV_CUDA(cudaMemsetAsync(p, v, bytes, ctx->stream));
}

sv_encode_tiled_fn sv_encode_tiled() {
  static sv_encode_tiled_fn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    SV_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p)
      sv_throw(SV_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available from the driver");
    fn = (sv_encode_tiled_fn)p;
  }
  return fn;
}

void sv_parallel_memcpy(void* dst, const void* src, size_t n) {
  const size_t PART = (size_t)4 << 20;
  int t = (int)std::min<size_t>(std::min<size_t>(8, std::max(1u, std::thread::hardware_concurrency())),
                                (n + PART - 1) / PART);
  if (t <= 1) {
    memcpy(dst, src, n);
    return;
  }
  size_t per = (n + t - 1) / t;
  std::vector<std::thread> th;
  for (int i = 0; i < t; ++i) {
    size_t a = (size_t)i * per, b = std::min(n, a + per);
    if (a >= b) break;
    th.emplace_back([=] { memcpy((char*)dst + a, (const char*)src + a, b - a); });
  }
  for (auto& x : th) x.join();
}

void sv_ctx_io(sv_context* ctx, void* buf[2], cudaEvent_t ev[2]) {
  const size_t CH = SV_IO_CHUNK;
  if (ctx->h_io_bytes < CH) {
    for (void*& p : ctx->h_io) {
      if (p) cudaFreeHost(p);
      p = nullptr;
    }
    ctx->h_io_bytes = 0;
    for (void*& p : ctx->h_io) SV_CUDA(cudaMallocHost(&p, CH));
    ctx->h_io_bytes = CH;
  }
  for (int b = 0; b < 2; ++b) {
    if (!ctx->h_io_ev[b]) SV_CUDA(cudaEventCreateWithFlags(&ctx->h_io_ev[b], cudaEventDisableTiming));
    buf[b] = ctx->h_io[b];
    ev[b] = ctx->h_io_ev[b];
  }
}

// Large copies to or from pageable host memory go through the context's two
// pinned buffers, the host side copied by several threads: a single-threaded
// staging copy (what the driver does for pageable memory) runs at a few GB/s
// when the destination pages are touched for the first time.
static bool pageable(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  return a.type == cudaMemoryTypeUnregistered;
}

static const size_t SV_STAGE_MIN = (size_t)32 << 20;

void sv_h2d(sv_context* ctx, void* dst, const void* src, size_t bytes) {
  if (!bytes) return;
  if (bytes < SV_STAGE_MIN || !pageable(src)) {
    SV_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return;
  }
  void* pin[2];
  cudaEvent_t ev[2];
  sv_ctx_io(ctx, pin, ev);
  int b = 0;
  for (size_t off = 0; off < bytes; off += SV_IO_CHUNK, b ^= 1) {
    size_t n = std::min(SV_IO_CHUNK, bytes - off);
    SV_CUDA(cudaEventSynchronize(ev[b]));
    sv_parallel_memcpy(pin[b], (const char*)src + off, n);
    SV_CUDA(cudaMemcpyAsync((char*)dst + off, pin[b], n, cudaMemcpyHostToDevice, ctx->stream));
    SV_CUDA(cudaEventRecord(ev[b], ctx->stream));
  }
}

void sv_d2h(sv_context* ctx, void* dst, const void* src, size_t bytes) {
  if (!bytes) return;
  if (bytes < SV_STAGE_MIN || !pageable(dst)) {
    SV_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    sv_sync(ctx);
    return;
  }
  void* pin[2];
  cudaEvent_t ev[2];
  sv_ctx_io(ctx, pin, ev);
  // chunk i lands in pin[i & 1]; its host copy overlaps the transfer of chunk i + 1
  const size_t nch = (bytes + SV_IO_CHUNK - 1) / SV_IO_CHUNK;
  auto issue = [&](size_t i) {
    size_t off = i * SV_IO_CHUNK, n = std::min(SV_IO_CHUNK, bytes - off);
    SV_CUDA(cudaMemcpyAsync(pin[i & 1], (const char*)src + off, n, cudaMemcpyDeviceToHost, ctx->stream));
    SV_CUDA(cudaEventRecord(ev[i & 1], ctx->stream));
  };
  SV_CUDA(cudaEventSynchronize(ev[0]));
  SV_CUDA(cudaEventSynchronize(ev[1]));
  issue(0);
  for (size_t i = 0; i < nch; ++i) {
    if (i + 1 < nch) issue(i + 1);
    SV_CUDA(cudaEventSynchronize(ev[i & 1]));
    size_t off = i * SV_IO_CHUNK, n = std::min(SV_IO_CHUNK, bytes - off);
    sv_parallel_memcpy((char*)dst + off, pin[i & 1], n);
  }
  sv_sync(ctx);
}

int64_t sv_read_i64(sv_context* ctx, const int64_t* dptr) {
  int64_t* h = (int64_t*)sv_ctx_stage(ctx, sizeof(int64_t));
  SV_CUDA(cudaMemcpyAsync(h, dptr, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  sv_sync(ctx);
  return *h;
}

void sv_check_device_status(sv_context* ctx, const char* where) {
  int* h = (int*)sv_ctx_stage(ctx, sizeof(int));
  SV_CUDA(cudaMemcpyAsync(h, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  sv_sync(ctx);
  int st = *h;
  if (st) {
    SV_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
    if (st & SV_STATUS_PARSE)
      sv_throw(SV_ERR_ARG, "%s: could not read a matrix entry (three fields per line expected)", where);
    if (st & SV_STATUS_UNSORTED)
      sv_throw(SV_ERR_ARG,
               "%s: indices are not strictly increasing within a column (unsorted or duplicate entries)",
               where);
    if (st & SV_STATUS_OOB) sv_throw(SV_ERR_ARG, "%s: an index is out of range", where);
    if (st & SV_STATUS_VALUE)
      sv_throw(SV_ERR_ARG, "%s: a count is not an integer in [0, 2^31)", where);
    sv_throw(SV_ERR_DEVICE, "%s: a device-side iteration limit was reached (status %d)", where, st);
  }
}

int sv_grid_for(sv_context* ctx, int64_t work_items, int per_block, int max_per_sm) {
  int64_t blocks = (work_items + per_block - 1) / per_block;
  int64_t cap = (int64_t)ctx->num_sms * max_per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

SV_API int sv_context_create(int device, sv_context** out) {
  SV_TRY
  SV_REQUIRE(out != nullptr, "out is null");
  int ndev = 0;
  SV_CUDA(cudaGetDeviceCount(&ndev));
  SV_REQUIRE(device >= 0 && device < ndev, "device %d not present (%d devices)", device, ndev);
  SV_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  SV_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10)
    sv_throw(SV_ERR_UNSUPPORTED, "device %d is sm_%d%d; this library is built for sm_103a",
             device, prop.major, prop.minor);
  sv_context* ctx = new sv_context();
  ctx->device = device;
  ctx->num_sms = prop.multiProcessorCount;
  cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete ctx;
    sv_throw(SV_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  for (int i = 0; i < 16; ++i) SV_CUDA(cudaEventCreate(&ctx->marks[i]));
  SV_CUDA(cudaMalloc((void**)&ctx->d_status, 256));
  SV_CUDA(cudaMemsetAsync(ctx->d_status, 0, 256, ctx->stream));
  SV_CUDA(cudaStreamSynchronize(ctx->stream));
  *out = ctx;
  SV_CATCH
}

SV_API int sv_context_destroy(sv_context* ctx) {
  if (!ctx) return SV_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& t : ctx->pending) {
    cudaEventDestroy(t.a);
    cudaEventDestroy(t.b);
  }
  for (auto e : ctx->event_pool) cudaEventDestroy(e);
  for (int i = 0; i < 16; ++i)
    if (ctx->marks[i]) cudaEventDestroy(ctx->marks[i]);
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  for (void* p : ctx->h_io)
    if (p) cudaFreeHost(p);
  for (cudaEvent_t e : ctx->h_io_ev)
    if (e) cudaEventDestroy(e);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return SV_OK;
}

SV_API int sv_synchronize(sv_context* ctx) {
  SV_TRY
  sv_ctx_check(ctx);
  sv_sync(ctx);
  SV_CATCH
}

SV_API int sv_host_register(void* ptr, size_t bytes) {
  SV_TRY
  SV_REQUIRE(ptr && bytes, "null pointer or zero size");
  SV_CUDA(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
  SV_CATCH
}

SV_API int sv_host_unregister(void* ptr) {
  SV_TRY
  SV_CUDA(cudaHostUnregister(ptr));
  SV_CATCH
}

SV_API int sv_host_alloc(void** ptr, size_t bytes) {
  SV_TRY
  SV_REQUIRE(ptr, "null out pointer");
  SV_CUDA(cudaMallocHost(ptr, bytes ? bytes : 1));
  SV_CATCH
}

SV_API int sv_host_free(void* ptr) {
  SV_TRY
  if (ptr) SV_CUDA(cudaFreeHost(ptr));
  SV_CATCH
}

SV_API int sv_mark(sv_context* ctx, int slot) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(slot >= 0 && slot < 16, "slot %d out of range", slot);
  SV_CUDA(cudaEventRecord(ctx->marks[slot], ctx->stream));
  SV_CATCH
}

SV_API int sv_elapsed_ms(sv_context* ctx, int a, int b, double* ms) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(a >= 0 && a < 16 && b >= 0 && b < 16 && ms, "bad slots");
  SV_CUDA(cudaEventSynchronize(ctx->marks[b]));
  float f = 0;
  SV_CUDA(cudaEventElapsedTime(&f, ctx->marks[a], ctx->marks[b]));
  *ms = f;
  SV_CATCH
}

SV_API int sv_launch_count(sv_context* ctx, int64_t* count) {
  SV_TRY
  SV_REQUIRE(ctx && count, "null argument");
  *count = ctx->launches;
  SV_CATCH
}

SV_API int sv_profile_enable(sv_context* ctx, int enable) {
  SV_TRY
  sv_ctx_check(ctx);
  sv_ctx_harvest(ctx);
  ctx->profiling = enable != 0;
  SV_CATCH
}

SV_API int sv_profile_reset(sv_context* ctx) {
  SV_TRY
  sv_ctx_check(ctx);
  sv_ctx_harvest(ctx);
  ctx->prof.clear();
  SV_CATCH
}

SV_API int sv_profile_query(sv_context* ctx, const char* sub, double* total_ms, int64_t* launches) {
  SV_TRY
  sv_ctx_check(ctx);
  sv_ctx_harvest(ctx);
  double t = 0;
  int64_t c = 0;
  for (auto& kv : ctx->prof) {
    if (!sub || strstr(kv.first.c_str(), sub)) {
      t += kv.second.first;
      c += kv.second.second;
    }
  }
  if (total_ms) *total_ms = t;
  if (launches) *launches = c;
  SV_CATCH
}

SV_API int sv_profile_report(sv_context* ctx, char* buf, size_t len) {
  SV_TRY
  sv_ctx_check(ctx);
  sv_ctx_harvest(ctx);
  std::string s;
  char line[256];
  for (auto& kv : ctx->prof) {
    snprintf(line, sizeof line, "%s %lld %.6f\n", kv.first.c_str(), (long long)kv.second.second,
             kv.second.first);
    s += line;
  }
  if (buf && len) {
    size_t n = s.size() < len - 1 ? s.size() : len - 1;
    memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
  return (int)s.size();
  SV_CATCH
}

SV_API int sv_device_memory(sv_context* ctx, size_t* free_b, size_t* total_b) {
  SV_TRY
  sv_ctx_check(ctx);
  size_t f = 0, t = 0;
  SV_CUDA(cudaMemGetInfo(&f, &t));
  if (free_b) *free_b = f;
  if (total_b) *total_b = t;
  SV_CATCH
}

// ---------------------------------------------------------------------------
// device-wide exclusive scan of int64 (three phases, recursive on block sums)
// ---------------------------------------------------------------------------
namespace {
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t* total) {
  __shared__ int64_t warp_sums[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t w = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_sums[lane] = w;
  }
  __syncthreads();
  int64_t prefix = (wid > 0 ? warp_sums[wid - 1] : 0) + x - v;
  *total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return prefix;
}

__global__ void k_scan_tiles(const int64_t* __restrict__ in, int64_t* __restrict__ out,
                             int64_t* __restrict__ tile_sums, int64_t n) {
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
  int64_t vals[SCAN_ITEMS];
  int64_t local = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    int64_t idx = base + i;
    vals[i] = idx < n ? in[idx] : 0;
    local += vals[i];
  }
  int64_t total;
  int64_t pre = block_exclusive_scan(local, &total);
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    int64_t idx = base + i;
    if (idx < n) out[idx] = pre;
    pre += vals[i];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void k_scan_add(int64_t* __restrict__ out, const int64_t* __restrict__ tile_pre,
                           int64_t n) {
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
  int64_t add = tile_pre[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    int64_t idx = base + i;
    if (idx < n) out[idx] += add;
  }
}

__global__ void k_scan_total(int64_t* out, const int64_t* tile_pre, int64_t ntiles, int64_t n) {
  // out[n] = total = exclusive prefix of the (virtual) tile after the last one
  out[n] = tile_pre[ntiles];
}
}  // namespace

void sv_scan_i64(sv_context* ctx, const int64_t* in, int64_t* out, int64_t n) {
  if (n <= 0) {
    sv_memset(ctx, out, 0, sizeof(int64_t));
    return;
  }
  int64_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  DevBuf<int64_t> sums(ntiles);
  sv_launch(ctx, "scan_tiles", k_scan_tiles, dim3((unsigned)ntiles), dim3(SCAN_THREADS), 0, in,
            out, sums.get(), n);
  if (ntiles == 1) {
    sv_launch(ctx, "scan_total", k_scan_total, dim3(1), dim3(1), 0, out,
              (const int64_t*)sums.get() - 1, (int64_t)1, n);
    sv_sync(ctx);
    return;
  }
  DevBuf<int64_t> pre(ntiles + 1);
  sv_scan_i64(ctx, sums.get(), pre.get(), ntiles);  // pre[ntiles] = total
  sv_launch(ctx, "scan_add", k_scan_add, dim3((unsigned)ntiles), dim3(SCAN_THREADS), 0, out,
            (const int64_t*)pre.get(), n);
  sv_launch(ctx, "scan_total", k_scan_total, dim3(1), dim3(1), 0, out, (const int64_t*)pre.get(),
            ntiles, n);
  // the temporaries are released on return: finish their last use first
  sv_sync(ctx);
}

// ---- bitonic sort of (key, value) pairs ------------------------------------------
// Sorts n pairs by key (ascending; equal keys in no particular order) in place,
// padding to a power of two with the largest key.  Strides below 1024 run in
// shared memory (2048 pairs per block), larger strides one launch each.
namespace {

__global__ void k_bitonic_pad(unsigned long long* __restrict__ key, int* __restrict__ val, int64_t n,
                              int64_t n2) {
  for (int64_t i = n + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2;
       i += (int64_t)gridDim.x * blockDim.x) {
    key[i] = ~0ull;
    val[i] = -1;
  }
}

__device__ __forceinline__ void bitonic_cas(unsigned long long& ka, int& va, unsigned long long& kb, int& vb,
                                            bool up) {
  if ((ka > kb) == up) {
    unsigned long long tk = ka;
    ka = kb;
    kb = tk;
    int tv = va;
    va = vb;
    vb = tv;
  }
}

// one global step: stride j of the merge of size k
__global__ void k_bitonic_global(unsigned long long* __restrict__ key, int* __restrict__ val, int64_t n2,
                                 int64_t k, int64_t j) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n2 / 2;
       t += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = (t / j) * 2 * j + (t % j);
    int64_t l = i + j;
    bool up = (i & k) == 0;
    unsigned long long ka = key[i], kb = key[l];
    int va = val[i], vb = val[l];
    bitonic_cas(ka, va, kb, vb, up);
    key[i] = ka;
    key[l] = kb;
    val[i] = va;
    val[l] = vb;
  }
}

// every stride j <= 1024 of the merges of size k (kfrom .. kto) in shared memory,
// 2048 pairs per block
__global__ void __launch_bounds__(1024) k_bitonic_smem(unsigned long long* __restrict__ key,
                                                       int* __restrict__ val, int64_t kfrom, int64_t kto,
                                                       int64_t jfrom) {
  __shared__ unsigned long long sk[2048];
  __shared__ int sv[2048];
  int64_t base = (int64_t)blockIdx.x * 2048;
  for (int i = threadIdx.x; i < 2048; i += blockDim.x) {
    sk[i] = key[base + i];
    sv[i] = val[base + i];
  }
  __syncthreads();
  for (int64_t k = kfrom; k <= kto; k <<= 1) {
    for (int64_t j = (k == kfrom ? jfrom : k >> 1); j > 0; j >>= 1) {
      int t = threadIdx.x;
      int i = (int)((t / j) * 2 * j + (t % j));
      int l = i + (int)j;
      bool up = ((base + i) & k) == 0;
      bitonic_cas(sk[i], sv[i], sk[l], sv[l], up);
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < 2048; i += blockDim.x) {
    key[base + i] = sk[i];
    val[base + i] = sv[i];
  }
}

}  // namespace

// key / val hold n2 >= n entries (n2 = next power of two, at least 2048)
void sv_sort_pairs(sv_context* ctx, unsigned long long* key, int* val, int64_t n, int64_t n2) {
  if (n2 > n)
    sv_launch(ctx, "sort_pad", k_bitonic_pad, dim3(sv_grid_for(ctx, n2 - n, 256)), dim3(256), 0, key, val, n,
              n2);
  int64_t blocks = n2 / 2048;
  // merges of size up to 2048 entirely in shared memory
  sv_launch(ctx, "sort_smem", k_bitonic_smem, dim3((unsigned)blocks), dim3(1024), 0, key, val, (int64_t)2,
            (int64_t)2048, (int64_t)1);
  for (int64_t k = 4096; k <= n2; k <<= 1) {
    for (int64_t j = k >> 1; j >= 2048; j >>= 1)
      sv_launch(ctx, "sort_global", k_bitonic_global, dim3(sv_grid_for(ctx, n2 / 2, 256)), dim3(256), 0, key,
                val, n2, k, j);
    sv_launch(ctx, "sort_smem", k_bitonic_smem, dim3((unsigned)blocks), dim3(1024), 0, key, val, k, k,
              (int64_t)1024);
  }
}
