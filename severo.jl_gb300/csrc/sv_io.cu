// MatrixMarket count matrices parsed on the device (readMM, src/input.jl:27-115;
// _read_10X :199-208 and _read_dge :131-152 read the same format).
//
// The host reads the banner, the comment lines and the size line, then streams
// the entry section, byte for byte as it lies in the file, into HBM through two
// pinned staging buffers.  The device finds the line ends (one warp per 4 KB
// tile, two passes: count, then place), parses one entry line per thread, and
// builds the cells x genes count matrix with its CSR and CSC copies.  As in
// sparse(I, J, V) (src/input.jl:113), entries that name the same position are
// summed and explicit zeros are kept; as in read_10X, a file whose rows are
// features is transposed so that its columns become the cells.
//
// Counts are stored as Int32: values must be whole numbers in [0, 2^31), the
// range convert_counts (src/input.jl:776-780) converts real-valued files into.
#include "sv_internal.cuh"

#include <dlfcn.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <atomic>
#include <cerrno>
#include <memory>
#include <thread>

namespace {

constexpr int64_t TILE = 4096;  // text bytes per warp in the line-end passes

// ---- device: line ends -----------------------------------------------------
// 16-bit mask of the newline bytes of a 16-byte chunk, bit j = byte j
__device__ __forceinline__ unsigned nl_mask(uint4 v) {
  unsigned m = 0;
  uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    uint32_t e = __vcmpeq4(w[k], 0x0a0a0a0au) & 0x80808080u;
    unsigned b = ((e >> 7) & 1u) | ((e >> 14) & 2u) | ((e >> 21) & 4u) | ((e >> 28) & 8u);
    m |= b << (4 * k);
  }
  return m;
}

// newlines per tile; the text buffer is zero-padded to whole tiles
__global__ void k_nl_count(const uint4* __restrict__ txt, int64_t n_tiles, int64_t* __restrict__ cnt) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = warp; t < n_tiles; t += nwarps) {
    const uint4* p = txt + t * (TILE / 16);
    int c = 0;
#pragma unroll
    for (int it = 0; it < TILE / 512; ++it) c += __popc(nl_mask(p[it * 32 + lane]));
    c = sv_warp_sum(c);
    if (lane == 0) cnt[t] = c;
  }
}

// byte offsets of the first `need` newlines, in file order
__global__ void k_nl_pos(const uint4* __restrict__ txt, int64_t n_tiles,
                         const int64_t* __restrict__ tile_off, int64_t need,
                         int64_t* __restrict__ nlpos) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = warp; t < n_tiles; t += nwarps) {
    int64_t run = tile_off[t];
    if (run >= need) continue;
    const uint4* p = txt + t * (TILE / 16);
    for (int it = 0; it < TILE / 512; ++it) {
      unsigned m = nl_mask(p[it * 32 + lane]);
      int c = __popc(m), incl = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      int64_t k = run + incl - c;
      int64_t byte0 = t * TILE + it * 512 + lane * 16;
      while (m) {
        int j = __ffs(m) - 1;
        if (k < need) nlpos[k] = byte0 + j;
        ++k;
        m &= m - 1;
      }
      run += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
}

// ---- device: one entry line per thread ---------------------------------------
// Whitespace as split() treats it in ASCII text.
__device__ __forceinline__ bool is_ws(unsigned c) {
  return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f';
}

struct Cursor {
  const unsigned char* t;
  int64_t i, end;
  __device__ unsigned peek() const { return i < end ? t[i] : 0u; }
  __device__ void skip_ws() {
    while (i < end && is_ws(t[i])) ++i;
  }
  __device__ bool at_token_end() const { return i >= end || is_ws(t[i]); }
};

// [+-]digits as an Int64 (parse(Int64, s)); false on a malformed token or overflow
__device__ bool parse_int(Cursor& c, long long& out) {
  bool neg = false;
  unsigned ch = c.peek();
  if (ch == '+' || ch == '-') {
    neg = ch == '-';
    ++c.i;
  }
  unsigned long long v = 0;
  int nd = 0;
  while (c.i < c.end) {
    unsigned d = c.t[c.i] - '0';
    if (d > 9) break;
    if (v > (9223372036854775807ull - d) / 10) return false;
    v = v * 10 + d;
    ++nd;
    ++c.i;
  }
  if (nd == 0 || !c.at_token_end()) return false;
  out = neg ? -(long long)v : (long long)v;
  return true;
}

// A decimal real token ([+-]digits[.digits][(e|E)[+-]digits]) that must hold a
// whole number: evaluated exactly as mantissa x 10^exponent.  Returns 0 on
// success, 1 for a malformed token, 2 for a value that is not a whole number in
// [0, 2^31).
__device__ int parse_real_count(Cursor& c, long long& out) {
  bool neg = false;
  unsigned ch = c.peek();
  if (ch == '+' || ch == '-') {
    neg = ch == '-';
    ++c.i;
  }
  unsigned long long m = 0;
  int sig = 0, nd = 0;
  long long e10 = 0;
  bool lost = false;  // a non-zero digit beyond 19 significant digits
  while (c.i < c.end) {
    unsigned d = c.t[c.i] - '0';
    if (d > 9) break;
    ++nd;
    ++c.i;
    if (sig < 19) {
      m = m * 10 + d;
      if (m) ++sig;
    } else {
      ++e10;
      lost |= d != 0;
    }
  }
  if (c.peek() == '.') {
    ++c.i;
    while (c.i < c.end) {
      unsigned d = c.t[c.i] - '0';
      if (d > 9) break;
      ++nd;
      ++c.i;
      if (sig < 19) {
        m = m * 10 + d;
        if (m) ++sig;
        --e10;
      } else {
        lost |= d != 0;
      }
    }
  }
  if (nd == 0) return 1;
  ch = c.peek();
  if (ch == 'e' || ch == 'E') {
    ++c.i;
    bool eneg = false;
    ch = c.peek();
    if (ch == '+' || ch == '-') {
      eneg = ch == '-';
      ++c.i;
    }
    long long x = 0;
    int ne = 0;
    while (c.i < c.end) {
      unsigned d = c.t[c.i] - '0';
      if (d > 9) break;
      if (x < 100000000) x = x * 10 + d;
      ++ne;
      ++c.i;
    }
    if (ne == 0) return 1;
    e10 += eneg ? -x : x;
  }
  if (!c.at_token_end()) return 1;
  if (m == 0) {
    out = 0;
    return lost ? 2 : 0;
  }
  if (lost || neg) return 2;
  while (e10 < 0) {
    if (m % 10) return 2;
    m /= 10;
    ++e10;
  }
  while (e10 > 0) {
    if (m >= 2147483648ull) return 2;
    m *= 10;
    --e10;
  }
  if (m >= 2147483648ull) return 2;
  out = (long long)m;
  return 0;
}

__global__ void k_parse_entries(const unsigned char* __restrict__ txt, int64_t len,
                                const int64_t* __restrict__ nlpos, int64_t n_nl, int64_t entries,
                                int real_field, int rows_are_features, int64_t n_rows,
                                int64_t n_cols, int32_t* __restrict__ cell, int32_t* __restrict__ gene,
                                int32_t* __restrict__ val, int* status) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < entries;
       e += (int64_t)gridDim.x * blockDim.x) {
    Cursor c{txt, e == 0 ? 0 : nlpos[e - 1] + 1, e < n_nl ? nlpos[e] : len};
    long long r = 0, q = 0, v = 0;
    bool ok = true;
    int vst = 0;
    c.skip_ws();
    ok = parse_int(c, r);
    if (ok) {
      c.skip_ws();
      ok = parse_int(c, q);
    }
    if (ok) {
      c.skip_ws();
      if (real_field) {
        vst = parse_real_count(c, v);
        ok = vst != 1;
      } else {
        ok = parse_int(c, v);
        if (ok && (v < 0 || v >= 2147483648ll)) vst = 2;
      }
    }
    if (ok) {
      c.skip_ws();
      ok = c.i >= c.end;
    }
    int32_t ci = 0, gi = 0, vi = 0;
    if (!ok) {
      sv_flag(status, SV_STATUS_PARSE);
    } else if (r < 1 || r > n_rows || q < 1 || q > n_cols) {
      sv_flag(status, SV_STATUS_OOB);
    } else if (vst) {
      sv_flag(status, SV_STATUS_VALUE);
    } else {
      ci = (int32_t)(rows_are_features ? q - 1 : r - 1);
      gi = (int32_t)(rows_are_features ? r - 1 : q - 1);
      vi = (int32_t)v;
    }
    cell[e] = ci;
    gene[e] = gi;
    val[e] = vi;
  }
}

// ---- device: coordinates to the compressed copies ------------------------------
__global__ void k_coo_hist(const int32_t* __restrict__ cell, int64_t n,
                           unsigned long long* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[cell[i]], 1ull);
}

__global__ void k_u64_i64(const unsigned long long* __restrict__ in, int64_t* __restrict__ out,
                          int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int64_t)in[i];
}

__global__ void k_i64_u64(const int64_t* __restrict__ in, unsigned long long* __restrict__ out,
                          int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (unsigned long long)in[i];
}

__global__ void k_coo_scatter(const int32_t* __restrict__ cell, const int32_t* __restrict__ gene,
                              const int32_t* __restrict__ val, int64_t n,
                              unsigned long long* __restrict__ cursor, int32_t* __restrict__ col,
                              int32_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long pos = atomicAdd(&cursor[cell[i]], 1ull);
    col[pos] = gene[i];
    cnt[pos] = val[i];
  }
}

// Sets *flag unless the entries are in cell order with strictly increasing
// features within each cell (the order 10X writes): then they already are the
// cell-major copy.
__global__ void k_coo_unsorted(const int32_t* __restrict__ cell, const int32_t* __restrict__ gene,
                               int64_t n, int* flag) {
  bool bad = false;
  for (int64_t e = 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    int32_t c0 = cell[e - 1], c1 = cell[e];
    bad |= c1 < c0 || (c1 == c0 && gene[e] <= gene[e - 1]);
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) *flag = 1;
}

// distinct columns per (sorted) row
__global__ void k_dup_len(const int64_t* __restrict__ ptr, const int32_t* __restrict__ col, int64_t n,
                          int64_t* __restrict__ len) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n; r += nwarps) {
    int64_t s = ptr[r], e = ptr[r + 1];
    long long h = 0;
    for (int64_t i = s + lane; i < e; i += 32) h += i == s || col[i] != col[i - 1];
    h = sv_warp_sum(h);
    if (lane == 0) len[r] = h;
  }
}

// one entry per distinct column, its counts summed (sparse(I, J, V) combines with +)
__global__ void k_dup_write(const int64_t* __restrict__ ptr, const int32_t* __restrict__ col,
                            const int32_t* __restrict__ cnt, int64_t n,
                            const int64_t* __restrict__ nptr, int32_t* __restrict__ ocol,
                            int32_t* __restrict__ ocnt, int* status) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n; r += nwarps) {
    int64_t s = ptr[r], e = ptr[r + 1], dst = nptr[r];
    for (int64_t b = s; b < e; b += 32) {
      int64_t i = b + lane;
      bool head = i < e && (i == s || col[i] != col[i - 1]);
      unsigned m = __ballot_sync(0xffffffffu, head);
      if (head) {
        long long sum = cnt[i];
        for (int64_t j = i + 1; j < e && col[j] == col[i]; ++j) sum += cnt[j];
        if (sum >= 2147483648ll) {
          sv_flag(status, SV_STATUS_VALUE);
          sum = 0;
        }
        int64_t o = dst + __popc(m & ((1u << lane) - 1u));
        ocol[o] = col[i];
        ocnt[o] = (int32_t)sum;
      }
      dst += __popc(m);
    }
  }
}

// ---- host: byte sources ----------------------------------------------------------
struct Source {
  virtual ~Source() {}
  // up to n bytes into dst; 0 at the end of the input
  virtual size_t read(void* dst, size_t n) = 0;
  // bytes left to read when known, else -1
  virtual int64_t remaining() const { return -1; }
};

// Runs part(i, a, b) over [0, n) split into up to 8 host threads (parallel
// reads of a file into the staging buffers).
template <typename F>
void split_copy(size_t n, F part) {
  const size_t PART = (size_t)8 << 20;
  int t = (int)std::min<size_t>(std::min<size_t>(8, std::max(1u, std::thread::hardware_concurrency())),
                                (n + PART - 1) / PART);
  if (t <= 1) {
    part(0, 0, n);
    return;
  }
  size_t per = (n + t - 1) / t;
  std::vector<std::thread> th;
  for (int i = 0; i < t; ++i) {
    size_t a = (size_t)i * per, b = std::min(n, a + per);
    if (a >= b) break;
    th.emplace_back([=] { part(i, a, b); });
  }
  for (auto& x : th) x.join();
}

struct MemSource : Source {
  const char* p;
  size_t n, pos = 0;
  MemSource(const char* p_, size_t n_) : p(p_), n(n_) {}
  size_t read(void* dst, size_t k) override {
    k = std::min(k, n - pos);
    sv_parallel_memcpy(dst, p + pos, k);
    pos += k;
    return k;
  }
  int64_t remaining() const override { return (int64_t)(n - pos); }
};

struct FileSource : Source {
  int fd = -1;
  bool regular = false;
  int64_t size = -1, pos = 0;
  explicit FileSource(const char* path) {
    fd = ::open(path, O_RDONLY);
    if (fd < 0) sv_throw(SV_ERR_ARG, "cannot open %s", path);
    struct stat st;
    if (fstat(fd, &st) == 0 && S_ISREG(st.st_mode)) {
      regular = true;
      size = st.st_size;
    }
  }
  ~FileSource() override {
    if (fd >= 0) ::close(fd);
  }
  size_t read(void* dst, size_t k) override {
    if (!regular) {  // pipes and devices: one sequential read
      ssize_t r;
      do r = ::read(fd, dst, k); while (r < 0 && errno == EINTR);
      if (r < 0) sv_throw(SV_ERR_ARG, "read error");
      pos += r;
      return (size_t)r;
    }
    k = (size_t)std::min<int64_t>((int64_t)k, std::max<int64_t>(0, size - pos));
    std::atomic<int> bad{0};
    const int64_t base = pos;
    split_copy(k, [&, base](int, size_t a, size_t b) {
      while (a < b) {
        ssize_t r = ::pread(fd, (char*)dst + a, b - a, (off_t)(base + (int64_t)a));
        if (r < 0 && errno == EINTR) continue;
        if (r <= 0) {
          bad = 1;
          return;
        }
        a += (size_t)r;
      }
    });
    if (bad) sv_throw(SV_ERR_ARG, "read error (the file changed or could not be read)");
    pos += (int64_t)k;
    return k;
  }
  int64_t remaining() const override { return regular ? size - pos : -1; }
};

// gzip through the system zlib, loaded when a gzip file is first read
struct Zlib {
  void* h = nullptr;
  void* (*open)(const char*, const char*) = nullptr;
  int (*read)(void*, void*, unsigned) = nullptr;
  int (*close)(void*) = nullptr;
  int (*buffer)(void*, unsigned) = nullptr;
};

Zlib* zlib() {
  static Zlib z;
  static std::once_flag once;
  std::call_once(once, [] {
    void* h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) return;
    z.open = (void* (*)(const char*, const char*))dlsym(h, "gzopen");
    z.read = (int (*)(void*, void*, unsigned))dlsym(h, "gzread");
    z.close = (int (*)(void*))dlsym(h, "gzclose");
    z.buffer = (int (*)(void*, unsigned))dlsym(h, "gzbuffer");
    if (z.open && z.read && z.close) z.h = h;
  });
  return z.h ? &z : nullptr;
}

struct GzSource : Source {
  Zlib* z;
  void* g = nullptr;
  explicit GzSource(const char* path) {
    z = zlib();
    if (!z) sv_throw(SV_ERR_UNSUPPORTED, "reading %s needs libz.so.1, which could not be loaded", path);
    g = z->open(path, "rb");
    if (!g) sv_throw(SV_ERR_ARG, "cannot open %s", path);
    if (z->buffer) z->buffer(g, 1u << 20);
  }
  ~GzSource() override {
    if (g) z->close(g);
  }
  size_t read(void* dst, size_t k) override {
    size_t tot = 0;
    while (tot < k) {
      unsigned ask = (unsigned)std::min<size_t>(k - tot, (size_t)1 << 30);
      int r = z->read(g, (char*)dst + tot, ask);
      if (r < 0) sv_throw(SV_ERR_ARG, "corrupt gzip stream");
      if (r == 0) break;
      tot += (size_t)r;
    }
    return tot;
  }
};

// Buffered line reader for the banner, comments and size line; whatever it has
// read beyond them is handed to the entry-section upload.
struct Head {
  Source& src;
  std::vector<char> buf;
  size_t pos = 0, len = 0;
  bool eof = false;
  explicit Head(Source& s) : src(s), buf(1 << 20) {}
  bool fill() {
    if (eof) return false;
    if (pos > 0) {
      memmove(buf.data(), buf.data() + pos, len - pos);
      len -= pos;
      pos = 0;
    }
    if (len == buf.size()) buf.resize(buf.size() * 2);
    size_t r = src.read(buf.data() + len, buf.size() - len);
    if (r == 0) eof = true;
    len += r;
    return r > 0;
  }
  // the next line without its "\n" or "\r\n"; false at the end of the input
  bool line(std::string& out) {
    size_t searched = 0;
    for (;;) {
      const char* b = buf.data();
      const void* nl = memchr(b + pos + searched, '\n', len - pos - searched);
      if (nl) {
        size_t e = (const char*)nl - b;
        out.assign(b + pos, e - pos);
        pos = e + 1;
        break;
      }
      searched = len - pos;
      if (!fill()) {
        if (pos == len) return false;
        out.assign(buf.data() + pos, len - pos);
        pos = len;
        break;
      }
    }
    if (!out.empty() && out.back() == '\r') out.pop_back();
    return true;
  }
};

std::vector<std::string> split_ws(const std::string& s) {
  std::vector<std::string> t;
  size_t i = 0;
  auto ws = [](char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f' || c == '\n'; };
  while (i < s.size()) {
    while (i < s.size() && ws(s[i])) ++i;
    size_t j = i;
    while (j < s.size() && !ws(s[j])) ++j;
    if (j > i) t.push_back(s.substr(i, j - i));
    i = j;
  }
  return t;
}

std::string lower(std::string s) {
  for (auto& c : s) c = (char)tolower((unsigned char)c);
  return s;
}

bool to_i64(const std::string& s, long long& v) {
  if (s.empty()) return false;
  size_t i = 0;
  bool neg = false;
  if (s[0] == '+' || s[0] == '-') {
    neg = s[0] == '-';
    i = 1;
  }
  if (i == s.size()) return false;
  unsigned long long x = 0;
  for (; i < s.size(); ++i) {
    unsigned d = (unsigned char)s[i] - '0';
    if (d > 9 || x > (9223372036854775807ull - d) / 10) return false;
    x = x * 10 + d;
  }
  v = neg ? -(long long)x : (long long)x;
  return true;
}

struct MMHeader {
  bool real = false;
  long long rows = 0, cols = 0, entries = 0;
};

// parseMM_header, skipMM_comments and the size line of readMM (src/input.jl:27-56,58-64,78-96)
MMHeader read_header(Head& h) {
  MMHeader m;
  std::string line;
  if (!h.line(line)) line.clear();
  auto tk = split_ws(line);
  if (tk.size() != 5) sv_throw(SV_ERR_ARG, "Malformed MatrixMarket header: %.200s", line.c_str());
  if (tk[0] != "%%MatrixMarket") sv_throw(SV_ERR_ARG, "Not a valid MatrixMarket header: %.200s", line.c_str());
  std::string obj = lower(tk[1]), format = lower(tk[2]), field = lower(tk[3]), symm = lower(tk[4]);
  if (obj != "matrix")
    sv_throw(SV_ERR_ARG, "Unknown MatrixMarket data type: %s (only \"matrix\" is supported)", obj.c_str());
  if (field == "real")
    m.real = true;
  else if (field != "integer")
    sv_throw(SV_ERR_ARG, "Unsupported field %s (only real and integer are supported)", field.c_str());
  if (symm != "general")
    sv_throw(SV_ERR_ARG, "Unknown matrix symmetry: %s (only \"general\" is supported)", symm.c_str());
  if (format != "coordinate")
    sv_throw(SV_ERR_ARG, "Unsupported matrix format: %s (only \"coordinate\" is supported)",
             format.c_str());
  for (;;) {
    if (!h.line(line)) sv_throw(SV_ERR_ARG, "Could not read in matrix dimensions: end of input");
    if (!line.empty() && line[0] != '%') break;
  }
  tk = split_ws(line);
  if (tk.size() != 3 || !to_i64(tk[0], m.rows) || !to_i64(tk[1], m.cols) || !to_i64(tk[2], m.entries))
    sv_throw(SV_ERR_ARG, "Could not read in matrix dimensions: %.200s", line.c_str());
  return m;
}

// Streams the entry section into a device buffer through two pinned staging
// buffers (the copy of one overlaps the read into the other).  The buffer is
// zero-padded to whole tiles.
DevBuf<unsigned char> upload_text(sv_context* ctx, Head& h, int64_t& len_out) {
  const size_t CH = SV_IO_CHUNK;
  int64_t known = h.src.remaining();
  int64_t cap = known >= 0 ? (int64_t)(h.len - h.pos) + known : std::max<int64_t>(CH, 4 * (int64_t)(h.len - h.pos));
  cap = (cap + TILE - 1) / TILE * TILE + TILE;
  DevBuf<unsigned char> d(cap);
  void* pin[2];
  cudaEvent_t ev[2];
  sv_ctx_io(ctx, pin, ev);
  int64_t len = 0;
  try {
    for (int b = 0;; b ^= 1) {
      SV_CUDA(cudaEventSynchronize(ev[b]));
      size_t n = 0;
      if (h.pos < h.len) {
        n = std::min(CH, h.len - h.pos);
        memcpy(pin[b], h.buf.data() + h.pos, n);
        h.pos += n;
      }
      while (n < CH) {
        size_t r = h.src.read((char*)pin[b] + n, CH - n);
        if (r == 0) break;
        n += r;
      }
      if (n == 0) break;
      if (len + (int64_t)n + TILE > cap) {
        // unknown size (gzip): grow by doubling
        int64_t ncap = std::max<int64_t>(2 * cap, len + (int64_t)n + 2 * TILE);
        ncap = (ncap + TILE - 1) / TILE * TILE;
        DevBuf<unsigned char> nd(ncap);
        if (len) SV_CUDA(cudaMemcpyAsync(nd.get(), d.get(), len, cudaMemcpyDeviceToDevice, ctx->stream));
        sv_sync(ctx);
        d = std::move(nd);
        cap = ncap;
      }
      SV_CUDA(cudaMemcpyAsync(d.get() + len, pin[b], n, cudaMemcpyHostToDevice, ctx->stream));
      SV_CUDA(cudaEventRecord(ev[b], ctx->stream));
      len += (int64_t)n;
    }
    sv_sync(ctx);
  } catch (...) {
    cudaStreamSynchronize(ctx->stream);  // no transfer from the staging buffers left in flight
    throw;
  }
  // zero the rest of the last tile (at least one tile is scanned)
  int64_t padded = std::max<int64_t>(1, (len + TILE - 1) / TILE) * TILE;
  sv_memset(ctx, d.get() + len, 0, (size_t)(padded - len));
  len_out = len;
  return d;
}

sv_counts* read_mm(sv_context* ctx, Source& src, int rows_are_features, const char* where) {
  Head h(src);
  MMHeader m = read_header(h);
  SV_REQUIRE(m.rows >= 1 && m.cols >= 1 && m.entries >= 0, "%s: bad matrix dimensions %lld x %lld, %lld entries",
             where, m.rows, m.cols, m.entries);
  const int64_t n_cells = rows_are_features ? m.cols : m.rows;
  const int64_t n_genes = rows_are_features ? m.rows : m.cols;
  SV_REQUIRE(n_cells < (1ll << 31) && n_genes < (1ll << 31), "%s: dimension exceeds Int32 indices", where);
  int64_t len = 0;
  DevBuf<unsigned char> txt = upload_text(ctx, h, len);
  const int64_t entries = m.entries;
  // the coordinates are allocated once the text is known to hold the entries
  DevBuf<int32_t> cell, gene, val;
  if (entries == 0) {
    cell.alloc(0);
    gene.alloc(0);
    val.alloc(0);
  } else {
    const int64_t n_tiles = std::max<int64_t>(1, (len + TILE - 1) / TILE);
    DevBuf<int64_t> tcnt(n_tiles + 1), toff(n_tiles + 1);
    dim3 gw(sv_grid_for(ctx, n_tiles * 32, 256)), bw(256);
    sv_launch(ctx, "mtx_line_count", k_nl_count, gw, bw, 0, (const uint4*)txt.get(), n_tiles, tcnt.get());
    sv_scan_i64(ctx, tcnt.get(), toff.get(), n_tiles);
    const int64_t n_nl = sv_read_i64(ctx, toff.get() + n_tiles);
    SV_REQUIRE(n_nl >= entries - 1, "%s: Could not read matrix entry: the input holds fewer than %lld entry lines",
               where, (long long)entries);
    const int64_t need = std::min<int64_t>(n_nl, entries);
    cell.alloc(entries);
    gene.alloc(entries);
    val.alloc(entries);
    DevBuf<int64_t> nlpos(std::max<int64_t>(1, need));
    sv_launch(ctx, "mtx_line_ends", k_nl_pos, gw, bw, 0, (const uint4*)txt.get(), n_tiles,
              (const int64_t*)toff.get(), need, nlpos.get());
    sv_launch(ctx, "mtx_parse", k_parse_entries, dim3(sv_grid_for(ctx, entries, 256)), dim3(256), 0,
              (const unsigned char*)txt.get(), len, (const int64_t*)nlpos.get(), need, entries,
              (int)m.real, rows_are_features, (int64_t)m.rows, (int64_t)m.cols, cell.get(), gene.get(),
              val.get(), ctx->d_status);
    sv_check_device_status(ctx, where);
  }
  txt.release();

  auto* c = new sv_counts();
  try {
    c->ctx = ctx;
    c->n_cells = n_cells;
    c->n_genes = n_genes;
    // cell-major order with the features of each cell sorted
    DevBuf<unsigned long long> hist(n_cells + 1);
    DevBuf<int64_t> p0(n_cells + 1), h64(n_cells + 1);
    sv_memset(ctx, hist.get(), 0, (n_cells + 1) * sizeof(unsigned long long));
    dim3 ge(sv_grid_for(ctx, entries, 256)), gc(sv_grid_for(ctx, n_cells, 256)), b(256);
    sv_launch(ctx, "mtx_hist", k_coo_hist, ge, b, 0, (const int32_t*)cell.get(), entries, hist.get());
    sv_launch(ctx, "mtx_hist", k_u64_i64, gc, b, 0, (const unsigned long long*)hist.get(), h64.get(), n_cells);
    DevBuf<int> unsorted(1);
    sv_memset(ctx, unsorted.get(), 0, sizeof(int));
    sv_launch(ctx, "mtx_order", k_coo_unsorted, ge, b, 0, (const int32_t*)cell.get(),
              (const int32_t*)gene.get(), entries, unsorted.get());
    int flag = 0;
    sv_d2h(ctx, &flag, unsorted.get(), sizeof(int));
    if (!flag) {
      // already the cell-major copy: no scatter, sort or merge
      c->csr_rowptr.alloc(n_cells + 1);
      sv_scan_i64(ctx, h64.get(), c->csr_rowptr.get(), n_cells);
      c->nnz = entries;
      c->csr_colidx = std::move(gene);
      c->csr_count = std::move(val);
      cell.release();
      sv_transpose_counts(ctx, n_cells, n_genes, c->nnz, c->csr_rowptr.get(), c->csr_colidx.get(),
                          c->csr_count.get(), c->csc_colptr, c->csc_rowidx, c->csc_count, where);
      sv_sync(ctx);
      return c;
    }
    DevBuf<int32_t> col(entries), cnt(entries);
    sv_scan_i64(ctx, h64.get(), p0.get(), n_cells);
    sv_launch(ctx, "mtx_hist", k_i64_u64, gc, b, 0, (const int64_t*)p0.get(), hist.get(), n_cells);
    sv_launch(ctx, "mtx_scatter", k_coo_scatter, ge, b, 0, (const int32_t*)cell.get(),
              (const int32_t*)gene.get(), (const int32_t*)val.get(), entries, hist.get(), col.get(),
              cnt.get());
    cell.release();
    gene.release();
    val.release();
    sv_sort_segments(ctx, p0.get(), n_cells, col.get(), cnt.get());
    // sum entries that name the same position
    dim3 gr(sv_grid_for(ctx, n_cells * 32, 256));
    sv_launch(ctx, "mtx_dedup", k_dup_len, gr, b, 0, (const int64_t*)p0.get(), (const int32_t*)col.get(),
              n_cells, h64.get());
    c->csr_rowptr.alloc(n_cells + 1);
    sv_scan_i64(ctx, h64.get(), c->csr_rowptr.get(), n_cells);
    c->nnz = sv_read_i64(ctx, c->csr_rowptr.get() + n_cells);
    if (c->nnz == entries) {
      c->csr_colidx = std::move(col);
      c->csr_count = std::move(cnt);
    } else {
      c->csr_colidx.alloc(c->nnz);
      c->csr_count.alloc(c->nnz);
      sv_launch(ctx, "mtx_dedup", k_dup_write, gr, b, 0, (const int64_t*)p0.get(), (const int32_t*)col.get(),
                (const int32_t*)cnt.get(), n_cells, (const int64_t*)c->csr_rowptr.get(), c->csr_colidx.get(),
                c->csr_count.get(), ctx->d_status);
      sv_check_device_status(ctx, where);
    }
    sv_transpose_counts(ctx, n_cells, n_genes, c->nnz, c->csr_rowptr.get(), c->csr_colidx.get(),
                        c->csr_count.get(), c->csc_colptr, c->csc_rowidx, c->csc_count, where);
    sv_sync(ctx);
  } catch (...) {
    delete c;
    throw;
  }
  return c;
}

bool ends_with(const char* s, const char* suf) {
  size_t a = strlen(s), b = strlen(suf);
  return a >= b && strcmp(s + a - b, suf) == 0;
}

}  // namespace

SV_API int sv_counts_read_mtx(sv_context* ctx, const char* path, int rows_are_features, sv_counts** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(path && out, "null argument");
  SV_REQUIRE(rows_are_features == 0 || rows_are_features == 1, "rows_are_features must be 0 or 1");
  std::unique_ptr<Source> src;
  if (ends_with(path, ".gz"))
    src.reset(new GzSource(path));
  else
    src.reset(new FileSource(path));
  *out = read_mm(ctx, *src, rows_are_features, "sv_counts_read_mtx");
  SV_CATCH
}

SV_API int sv_counts_parse_mtx(sv_context* ctx, const char* text, int64_t len, int rows_are_features,
                               sv_counts** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(out && (text || len == 0) && len >= 0, "bad argument");
  SV_REQUIRE(rows_are_features == 0 || rows_are_features == 1, "rows_are_features must be 0 or 1");
  MemSource src(text, (size_t)len);
  *out = read_mm(ctx, src, rows_are_features, "sv_counts_parse_mtx");
  SV_CATCH
}
