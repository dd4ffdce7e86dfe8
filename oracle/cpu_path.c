/* Multi-threaded CPU restatement of the embedding path -- TEST INFRASTRUCTURE
 * AND CPU BASELINE ONLY.
 *
 * Only bench.py's CPU-baseline leg and its reference arm (through
 * oracle/cpu_path.py) and tests/ load this file's library; the product path
 * (libseverogpu.so) never calls into it.
 *
 * The reference runs this path in single-threaded Julia (the SparseArrays
 * stdlib products) around a native irlba; this restatement follows the same
 * arithmetic in FP64 and spreads it over the host's cores with OpenMP, so that
 * the GPU is compared with a CPU baseline that uses the whole host:
 *   cp_generate_*    seeded negative-binomial counts (the benchmark's synthetic
 *                    input; not part of the timed path)
 *   cp_normalize     per-cell totals and log1p((sf * a) / s)
 *                    (src/normalize.jl:17-38), parallel over genes
 *   cp_scale         the feature subset, per-feature Welford mean / variance
 *                    with the implicit zeros in FP64 (src/scaling.jl:18-34) and
 *                    the clipped values min(a / std, scale_max + mean / std)
 *                    (src/scaling.jl:199-217), parallel over features
 *   cp_matvec        X~ x  = B x - (mu . x) 1   (src/scaling.jl:245-250): the
 *                    CSC column scatter of the stdlib, each thread into its own
 *                    accumulator, then summed over the threads
 *   cp_rmatvec       X~' u = B' u - (sum u) mu  (src/scaling.jl:252-257): the
 *                    CSC column gather, parallel over features
 *   cp_cgs2, cp_rotate  the irlba basis operations (CGS2, restart rotation)
 *   cp_knn           exact kNN by blocked brute force (the reference calls an
 *                    approximate native search instead)
 * The Lanczos iteration (irlba) is the oracle's numpy restatement driving these
 * kernels.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int nthreads_of(int nt) {
#ifdef _OPENMP
  return nt > 0 ? nt : omp_get_max_threads();
#else
  (void)nt;
  return 1;
#endif
}

/* ---- counter-based random numbers: splitmix64 of (seed, stream, counter) ---- */
static inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
typedef struct {
  uint64_t key, ctr;
} rng_t;
static inline double u01(rng_t* r) { /* (0, 1) */
  uint64_t x = mix64(r->key ^ mix64(r->ctr++));
  return ((double)(x >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
/* NegBinomial(size r, mean m) by inversion of its probability function:
 * P(0) = (r / (r + m))^r, P(k + 1) = P(k) (k + r) / (k + 1) q with q = m / (r + m);
 * one uniform per draw, and for the usual small means one comparison. */
static int64_t nb_draw(rng_t* rg, double r, double m) {
  if (m <= 0.0) return 0;
  const double q = m / (r + m);
  double pk = exp(r * log1p(-q)), f = pk;
  const double u = u01(rg);
  int64_t k = 0;
  while (u > f && k < 10000000) {
    pk *= (k + r) / (double)(k + 1) * q;
    ++k;
    f += pk;
    if (pk == 0.0 && f < u) break;   /* the tail underflowed: stop at the last k */
  }
  return k;
}

/* Cells x genes counts NB(mean = depth s_c mu_g exp(lfc[cluster_c][g]), dispersion
 * phi, i.e. size 1/phi), one random stream per cell,
 * in two passes that draw the same numbers.  Pass 1 (this function) counts the
 * non-zeros of each thread's block of cells per gene and turns the counts into
 * each thread's first position within each gene's column of the CSC (toff:
 * nt x n_genes); it returns the number of non-zeros.  colptr[g] is toff[0][g]. */
int64_t cp_generate_offsets(int64_t n_cells, int64_t n_genes, const double* mu_g, const double* s_c,
                            const int32_t* cluster, const double* lfc, double depth, double phi,
                            uint64_t seed, int64_t* toff, int nt) {
  nt = nthreads_of(nt);
  const double shape = 1.0 / phi;
  memset(toff, 0, (size_t)nt * (size_t)n_genes * sizeof(int64_t));
  const int64_t per = (n_cells + nt - 1) / nt;
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    const int t = omp_get_thread_num();
#else
    const int t = 0;
#endif
    const int64_t c0 = t * per, c1 = c0 + per < n_cells ? c0 + per : n_cells;
    int64_t* cnt = toff + (size_t)t * (size_t)n_genes;
    for (int64_t c = c0; c < c1; ++c) {
      rng_t r = {mix64(seed ^ 0x5EEDull) ^ (uint64_t)c * 0xD1B54A32D192ED03ull, 0};
      const double* fc = (cluster && lfc) ? lfc + (size_t)cluster[c] * (size_t)n_genes : NULL;
      for (int64_t g = 0; g < n_genes; ++g) {
        double mean = depth * s_c[c] * mu_g[g];
        if (fc) mean *= exp(fc[g]);
        if (nb_draw(&r, shape, mean) > 0) cnt[g]++;
      }
    }
  }
  int64_t total = 0;
  for (int64_t g = 0; g < n_genes; ++g) {
    int64_t off = 0;
    for (int t = 0; t < nt; ++t) {
      int64_t v = toff[(size_t)t * (size_t)n_genes + g];
      toff[(size_t)t * (size_t)n_genes + g] = total + off;
      off += v;
    }
    total += off;
  }
  return total;
}

/* Pass 2 with the per-thread offsets of cp_generate_offsets (advanced in
 * place): fills the CSC rows (sorted within each gene) and counts. */
void cp_generate_fill(int64_t n_cells, int64_t n_genes, const double* mu_g, const double* s_c,
                      const int32_t* cluster, const double* lfc, double depth, double phi,
                      uint64_t seed, int64_t* toff, int32_t* rowidx, int32_t* counts, int nt) {
  nt = nthreads_of(nt);
  const double shape = 1.0 / phi;
  const int64_t per = (n_cells + nt - 1) / nt;
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    const int t = omp_get_thread_num();
#else
    const int t = 0;
#endif
    const int64_t c0 = t * per, c1 = c0 + per < n_cells ? c0 + per : n_cells;
    int64_t* pos = toff + (size_t)t * (size_t)n_genes;
    for (int64_t c = c0; c < c1; ++c) {
      rng_t r = {mix64(seed ^ 0x5EEDull) ^ (uint64_t)c * 0xD1B54A32D192ED03ull, 0};
      const double* fc = (cluster && lfc) ? lfc + (size_t)cluster[c] * (size_t)n_genes : NULL;
      for (int64_t g = 0; g < n_genes; ++g) {
        double mean = depth * s_c[c] * mu_g[g];
        if (fc) mean *= exp(fc[g]);
        int64_t x = nb_draw(&r, shape, mean);
        if (x > 0) {
          rowidx[pos[g]] = (int32_t)c;
          counts[pos[g]] = (int32_t)(x < 2147483647 ? x : 2147483647);
          pos[g]++;
        }
      }
    }
  }
}

/* normalize_cells: totals[c] = sum of cell c's counts (integer, normalize.jl:24);
 * values[i] = (sf * a) / s (normalize.jl:27), log1p'd for :lognormalize (:36). */
void cp_normalize(int64_t n_cells, int64_t n_genes, const int64_t* colptr, const int32_t* rowidx,
                  const int32_t* counts, double sf, int log_norm, double* values, int64_t* totals,
                  int nt) {
  nt = nthreads_of(nt);
  int64_t* part = (int64_t*)calloc((size_t)nt * (size_t)n_cells, sizeof(int64_t));
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    const int t = omp_get_thread_num();
#else
    const int t = 0;
#endif
    int64_t* s = part + (size_t)t * (size_t)n_cells;
#pragma omp for schedule(dynamic, 64)
    for (int64_t g = 0; g < n_genes; ++g)
      for (int64_t i = colptr[g]; i < colptr[g + 1]; ++i) s[rowidx[i]] += counts[i];
#pragma omp for schedule(static)
    for (int64_t c = 0; c < n_cells; ++c) {
      int64_t v = 0;
      for (int u = 0; u < nt; ++u) v += part[(size_t)u * (size_t)n_cells + c];
      totals[c] = v;
    }
#pragma omp for schedule(dynamic, 64)
    for (int64_t g = 0; g < n_genes; ++g)
      for (int64_t i = colptr[g]; i < colptr[g + 1]; ++i) {
        double b = (sf * (double)counts[i]) / (double)totals[rowidx[i]];
        values[i] = log_norm ? log1p(b) : b;
      }
  }
  free(part);
}

/* scale_features over the features feats (0-based genes): the subset CSC
 * (hcolptr[nf + 1] filled here; hrow / hval sized by the caller), per-feature
 * Welford moments from the state after the implicit zeros (scaling.jl:18-34),
 * mu = mean / std (:207) and the stored values min(a / std, scale_max + mu)
 * (:209-212). */
void cp_scale(int64_t n_cells, const int64_t* colptr, const int32_t* rowidx, const double* values,
              int64_t nf, const int64_t* feats, double scale_max, int64_t* hcolptr, int32_t* hrow,
              double* hval, double* mu_out, double* mean_out, double* std_out, int nt) {
  nt = nthreads_of(nt);
  hcolptr[0] = 0;
  for (int64_t f = 0; f < nf; ++f) hcolptr[f + 1] = hcolptr[f] + (colptr[feats[f] + 1] - colptr[feats[f]]);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 4)
  for (int64_t f = 0; f < nf; ++f) {
    const int64_t s = colptr[feats[f]], e = colptr[feats[f] + 1];
    double count = (double)(n_cells - (e - s)), mu = 0.0, m2 = 0.0;
    for (int64_t i = s; i < e; ++i) {
      const double v = values[i];
      count += 1.0;
      const double delta = v - mu;
      mu += delta / count;
      m2 += delta * (v - mu);
    }
    const double sd = sqrt(m2 / (double)(n_cells - 1));
    const double muf = mu / sd, clip = scale_max + muf;
    mean_out[f] = mu;
    std_out[f] = sd;
    mu_out[f] = muf;
    const int64_t o = hcolptr[f];
    for (int64_t i = s; i < e; ++i) {
      const double v = values[i] / sd;
      hrow[o + (i - s)] = rowidx[i];
      hval[o + (i - s)] = v > clip ? clip : v;
    }
  }
}

/* y = B x - (mu . x) 1 over the subset CSC (n_cells x nf); tmp holds nt * n_cells
 * doubles (one accumulator per thread). */
void cp_matvec(int64_t n_cells, int64_t nf, const int64_t* hcolptr, const int32_t* hrow,
               const double* hval, const double* mu, const double* x, double* y, double* tmp,
               int nt) {
  nt = nthreads_of(nt);
  double mux = 0.0;
  for (int64_t f = 0; f < nf; ++f) mux += mu[f] * x[f];
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    const int t = omp_get_thread_num();
#else
    const int t = 0;
#endif
    double* acc = tmp + (size_t)t * (size_t)n_cells;
    memset(acc, 0, (size_t)n_cells * sizeof(double));
#pragma omp for schedule(dynamic, 8)
    for (int64_t f = 0; f < nf; ++f) {
      const double xf = x[f];
      for (int64_t i = hcolptr[f]; i < hcolptr[f + 1]; ++i) acc[hrow[i]] += hval[i] * xf;
    }
#pragma omp for schedule(static)
    for (int64_t c = 0; c < n_cells; ++c) {
      double v = 0.0;
      for (int u = 0; u < nt; ++u) v += tmp[(size_t)u * (size_t)n_cells + c];
      y[c] = v - mux;
    }
  }
}

/* y_f = sum_i B_if u_i - (sum u) mu_f */
void cp_rmatvec(int64_t n_cells, int64_t nf, const int64_t* hcolptr, const int32_t* hrow,
                const double* hval, const double* mu, const double* u, double* y, int nt) {
  nt = nthreads_of(nt);
  double su = 0.0;
#pragma omp parallel for num_threads(nt) reduction(+ : su) schedule(static)
  for (int64_t c = 0; c < n_cells; ++c) su += u[c];
#pragma omp parallel for num_threads(nt) schedule(dynamic, 8)
  for (int64_t f = 0; f < nf; ++f) {
    double v = 0.0;
    for (int64_t i = hcolptr[f]; i < hcolptr[f + 1]; ++i) v += hval[i] * u[hrow[i]];
    y[f] = v - su * mu[f];
  }
}

/* Classical Gram-Schmidt twice against the first j columns of the column-major
 * basis Q (n rows, leading dimension n): x <- x - Q (Q' x), two times.  tmp
 * holds nt * j doubles (one partial Q' x per thread). */
void cp_cgs2(int64_t n, int64_t j, const double* Q, double* x, double* tmp, int nt) {
  if (j <= 0) return;
  nt = nthreads_of(nt);
  double* c = (double*)malloc((size_t)j * sizeof(double));
  for (int pass = 0; pass < 2; ++pass) {
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
      const int t = omp_get_thread_num(), T = omp_get_num_threads();
#else
      const int t = 0, T = 1;
#endif
      const int64_t per = (n + T - 1) / T, r0 = t * per, r1 = r0 + per < n ? r0 + per : n;
      double* ct = tmp + (size_t)t * (size_t)j;
      for (int64_t q = 0; q < j; ++q) {
        const double* col = Q + (size_t)q * (size_t)n;
        double v = 0.0;
        for (int64_t i = r0; i < r1; ++i) v += col[i] * x[i];
        ct[q] = v;
      }
#pragma omp barrier
#pragma omp single
      for (int64_t q = 0; q < j; ++q) {
        double v = 0.0;
        for (int u = 0; u < T; ++u) v += tmp[(size_t)u * (size_t)j + q];
        c[q] = v;
      }
      for (int64_t q = 0; q < j; ++q) {
        const double* col = Q + (size_t)q * (size_t)n;
        const double cq = c[q];
        for (int64_t i = r0; i < r1; ++i) x[i] -= col[i] * cq;
      }
    }
  }
  free(c);
}

/* The restart rotation Q[:, :k] <- Q[:, :w] M (M: w x k column-major), by
 * blocks of rows; buf holds n * k doubles. */
void cp_rotate(int64_t n, int64_t w, int64_t k, double* Q, const double* M, double* buf, int nt) {
  nt = nthreads_of(nt);
  const int64_t RB = 256;
#pragma omp parallel for num_threads(nt) schedule(static)
  for (int64_t b = 0; b < (n + RB - 1) / RB; ++b) {
    const int64_t i0 = b * RB, i1 = i0 + RB < n ? i0 + RB : n;
    for (int64_t c = 0; c < k; ++c) {
      double* o = buf + (size_t)c * (size_t)n;
      for (int64_t i = i0; i < i1; ++i) o[i] = 0.0;
      for (int64_t t = 0; t < w; ++t) {
        const double m = M[t + c * w];
        const double* col = Q + (size_t)t * (size_t)n;
        for (int64_t i = i0; i < i1; ++i) o[i] += col[i] * m;
      }
    }
  }
#pragma omp parallel for num_threads(nt) schedule(static)
  for (int64_t c = 0; c < k; ++c)
    memcpy(Q + (size_t)c * (size_t)n, buf + (size_t)c * (size_t)n, (size_t)n * sizeof(double));
}

/* Exact Euclidean k nearest neighbours of every row of Z (n x d, row-major,
 * FP64), the row itself included, by brute force: squared distances
 * |q|^2 + |p|^2 - 2 q.p over blocks of 4 queries x 1024 points (the points
 * transposed once so that the inner loop runs over points), a sorted list of
 * the k best per query.  idx (n x k, 0-based) and dist2 (squared distances),
 * nearest first. */
void cp_knn(int64_t n, int64_t d, const double* Z, int64_t k, int64_t* idx, double* dist2, int nt) {
  nt = nthreads_of(nt);
  enum { QB = 4, PB = 1024 };
  double* ZT = (double*)malloc((size_t)n * (size_t)d * sizeof(double));
  double* sq = (double*)malloc((size_t)n * sizeof(double));
#pragma omp parallel for num_threads(nt) schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double s = 0.0;
    for (int64_t t = 0; t < d; ++t) {
      const double v = Z[i * d + t];
      ZT[t * n + i] = v;
      s += v * v;
    }
    sq[i] = s;
  }
#pragma omp parallel num_threads(nt)
  {
    double* acc = (double*)malloc((size_t)QB * PB * sizeof(double));
#pragma omp for schedule(dynamic, 4)
    for (int64_t q0 = 0; q0 < n; q0 += QB) {
      const int nq = (int)(q0 + QB <= n ? QB : n - q0);
      for (int a = 0; a < nq; ++a)
        for (int64_t r = 0; r < k; ++r) {
          dist2[(q0 + a) * k + r] = INFINITY;
          idx[(q0 + a) * k + r] = -1;
        }
      for (int64_t j0 = 0; j0 < n; j0 += PB) {
        const int np_ = (int)(j0 + PB <= n ? PB : n - j0);
        for (int64_t x = 0; x < (int64_t)QB * PB; ++x) acc[x] = 0.0;
        for (int64_t t = 0; t < d; ++t) {
          const double* row = ZT + t * n + j0;
          const double c0 = Z[q0 * d + t];
          const double c1 = nq > 1 ? Z[(q0 + 1) * d + t] : 0.0;
          const double c2 = nq > 2 ? Z[(q0 + 2) * d + t] : 0.0;
          const double c3 = nq > 3 ? Z[(q0 + 3) * d + t] : 0.0;
          double* a0 = acc;
          double* a1 = acc + PB;
          double* a2 = acc + 2 * PB;
          double* a3 = acc + 3 * PB;
          for (int j = 0; j < np_; ++j) {
            const double p = row[j];
            a0[j] += c0 * p;
            a1[j] += c1 * p;
            a2[j] += c2 * p;
            a3[j] += c3 * p;
          }
        }
        for (int a = 0; a < nq; ++a) {
          const int64_t q = q0 + a;
          double* bd = dist2 + q * k;
          int64_t* bi = idx + q * k;
          const double* ac = acc + (size_t)a * PB;
          for (int j = 0; j < np_; ++j) {
            double dv = sq[q] + sq[j0 + j] - 2.0 * ac[j];
            if (j0 + j == q) dv = -1.0;          /* the query itself comes first */
            if (dv < bd[k - 1]) {
              int64_t r = k - 1;
              while (r > 0 && bd[r - 1] > dv) {
                bd[r] = bd[r - 1];
                bi[r] = bi[r - 1];
                --r;
              }
              bd[r] = dv;
              bi[r] = j0 + j;
            }
          }
        }
      }
      for (int a = 0; a < nq; ++a) dist2[(q0 + a) * k] = 0.0;
    }
    free(acc);
  }
  free(ZT);
  free(sq);
}

/* ---- approximate kNN: random-projection forest + one neighbour-of-neighbour
 * round.  The reference calls a native approximate search parameterised by
 * `ntables` random tables (src/neighbours.jl:19-74, default ntables = 2 d);
 * its code is not available, so this is a stand-in of the same class, sized
 * by the same parameter: ntables random-projection trees (each node split at
 * the median of a random Gaussian direction, leaves of at most `leaf` points),
 * all pairs within a leaf as candidates, then the neighbours of each point's
 * neighbours.  Distances exact (FP64); lists nearest first, self first. */
static inline double gauss(rng_t* r) {
  double a = u01(r), b = u01(r);
  return sqrt(-2.0 * log(a)) * cos(6.283185307179586 * b);
}

static inline double sqdist(const double* a, const double* b, int64_t d) {
  double s0 = 0.0, s1 = 0.0;
  int64_t t = 0;
  for (; t + 1 < d; t += 2) {
    const double x = a[t] - b[t], y = a[t + 1] - b[t + 1];
    s0 += x * x;
    s1 += y * y;
  }
  if (t < d) {
    const double x = a[t] - b[t];
    s0 += x * x;
  }
  return s0 + s1;
}

static inline void knn_insert(double* bd, int64_t* bi, int64_t k, double dv, int64_t j) {
  if (dv >= bd[k - 1]) return;
  for (int64_t r = 0; r < k; ++r)
    if (bi[r] == j) return;
  int64_t r = k - 1;
  while (r > 0 && bd[r - 1] > dv) {
    bd[r] = bd[r - 1];
    bi[r] = bi[r - 1];
    --r;
  }
  bd[r] = dv;
  bi[r] = j;
}

/* the m-th smallest key of key[lo, hi) moved to position m (Hoare selection),
 * values permuted alongside */
static void select_kth(double* key, int32_t* val, int64_t lo, int64_t hi, int64_t m) {
  hi -= 1;
  while (lo < hi) {
    const double pivot = key[(lo + hi) / 2];
    int64_t i = lo, j = hi;
    while (i <= j) {
      while (key[i] < pivot) ++i;
      while (key[j] > pivot) --j;
      if (i <= j) {
        double tk = key[i]; key[i] = key[j]; key[j] = tk;
        int32_t tv = val[i]; val[i] = val[j]; val[j] = tv;
        ++i;
        --j;
      }
    }
    if (m <= j) hi = j;
    else if (m >= i) lo = i;
    else return;
  }
}

void cp_ann(int64_t n, int64_t d, const double* Z, int64_t k, int ntables, int leaf, uint64_t seed,
            int refine, int64_t* idx, double* dist2, int nt) {
  nt = nthreads_of(nt);
  if (leaf < 2) leaf = 2;
  for (int64_t i = 0; i < n; ++i)
    for (int64_t r = 0; r < k; ++r) {
      dist2[i * k + r] = INFINITY;
      idx[i * k + r] = -1;
    }
  for (int64_t i = 0; i < n; ++i) {
    dist2[i * k] = 0.0;
    idx[i * k] = i;
  }
  /* leaves hold at least leaf / 2 points: at most 2 n / leaf + 2 of them, two
   * offsets each */
  const int64_t maxleaves = 4 * (n / leaf + 2);
  int32_t* order = (int32_t*)malloc((size_t)ntables * (size_t)n * sizeof(int32_t));
  int64_t* lofs = (int64_t*)malloc((size_t)ntables * (size_t)maxleaves * sizeof(int64_t));
  int64_t* nleaf = (int64_t*)calloc((size_t)ntables, sizeof(int64_t));
  /* phase 1: the trees, one per task */
#pragma omp parallel num_threads(nt)
  {
    double* key = (double*)malloc((size_t)n * sizeof(double));
    double* dir = (double*)malloc((size_t)d * sizeof(double));
    int64_t* stack = (int64_t*)malloc((size_t)(2 * maxleaves + 64) * sizeof(int64_t));
#pragma omp for schedule(dynamic, 1)
    for (int t = 0; t < ntables; ++t) {
      int32_t* ord = order + (size_t)t * (size_t)n;
      int64_t* lo_ = lofs + (size_t)t * (size_t)maxleaves;
      rng_t rg = {mix64(seed ^ 0xA11ull) ^ (uint64_t)(t + 1) * 0x9E3779B97F4A7C15ull, 0};
      for (int64_t i = 0; i < n; ++i) ord[i] = (int32_t)i;
      int64_t sp = 0, nl = 0;
      stack[sp++] = 0;
      stack[sp++] = n;
      while (sp > 0) {
        const int64_t hi = stack[--sp], lo = stack[--sp];
        if (hi - lo <= leaf) {
          lo_[nl++] = lo;            /* leaves in order of completion; end = next start */
          lo_[nl++] = hi;
          continue;
        }
        for (int64_t u = 0; u < d; ++u) dir[u] = gauss(&rg);
        for (int64_t i = lo; i < hi; ++i) {
          const double* z = Z + (size_t)ord[i] * (size_t)d;
          double s = 0.0;
          for (int64_t u = 0; u < d; ++u) s += z[u] * dir[u];
          key[i] = s;
        }
        const int64_t mid = lo + (hi - lo) / 2;
        select_kth(key, ord, lo, hi, mid);
        stack[sp++] = lo;
        stack[sp++] = mid;
        stack[sp++] = mid;
        stack[sp++] = hi;
      }
      nleaf[t] = nl / 2;
    }
    free(key);
    free(dir);
    free(stack);
  }
  /* phase 2: all pairs within each leaf; a point lies in one leaf per tree, so
   * the leaves of a tree update disjoint lists */
  for (int t = 0; t < ntables; ++t) {
    const int32_t* ord = order + (size_t)t * (size_t)n;
    const int64_t* lo_ = lofs + (size_t)t * (size_t)maxleaves;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 16)
    for (int64_t l = 0; l < nleaf[t]; ++l) {
      const int64_t a = lo_[2 * l], b = lo_[2 * l + 1];
      for (int64_t x = a; x < b; ++x) {
        const int64_t i = ord[x];
        for (int64_t y = x + 1; y < b; ++y) {
          const int64_t j = ord[y];
          const double dv = sqdist(Z + (size_t)i * (size_t)d, Z + (size_t)j * (size_t)d, d);
          knn_insert(dist2 + i * k, idx + i * k, k, dv, j);
          knn_insert(dist2 + j * k, idx + j * k, k, dv, i);
        }
      }
    }
  }
  free(order);
  free(lofs);
  free(nleaf);
  /* phase 3: neighbours of neighbours, from a snapshot of the lists */
  for (int round = 0; round < refine; ++round) {
    int64_t* snap = (int64_t*)malloc((size_t)n * (size_t)k * sizeof(int64_t));
    memcpy(snap, idx, (size_t)n * (size_t)k * sizeof(int64_t));
#pragma omp parallel for num_threads(nt) schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i)
      for (int64_t r = 1; r < k; ++r) {
        const int64_t j = snap[i * k + r];
        if (j < 0) continue;
        for (int64_t s = 1; s < k; ++s) {
          const int64_t c = snap[j * k + s];
          if (c < 0 || c == i) continue;
          knn_insert(dist2 + i * k, idx + i * k, k,
                     sqdist(Z + (size_t)i * (size_t)d, Z + (size_t)c * (size_t)d, d), c);
        }
      }
    free(snap);
  }
}
