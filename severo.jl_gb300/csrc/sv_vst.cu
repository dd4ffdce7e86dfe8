// find_variable_features(:vst) (src/variablefeatures.jl:19-50,128-160) on the
// device-resident counts: per-gene mean and std of the counts, a local
// quadratic regression of log10(std) on log10(mean) over the non-constant
// genes, the expected std 10^fit, and the variance of the standardised counts
// clipped at sqrt(n_cells); the nfeatures genes of largest variance.
//
// The regression is loess (Cleveland 1979; Cleveland & Grosse 1991): the local
// fit at a point x0 takes the q = floor(span * n) nearest genes in log10(mean)
// (a contiguous window of the sorted values), tricube weights and weighted
// least squares in x - x0, FP64.  The reference calls Loess.jl's
// loess(xs, ys, span) and predict (variablefeatures.jl:41-42), which fits at
// the vertices of a kd-tree over xs and blends the two vertex fits of the
// cell holding each gene.  Three surfaces:
//   SV_LOESS_INTERPOLATE  kd-tree vertices, linear blend (NaN in a cell of
//                         zero width, or at a vertex whose q nearest genes
//                         all share its x: the reference's nan2zero! makes
//                         the expected std 0 and the metric 0 there)
//   SV_LOESS_HERMITE      kd-tree vertices, cubic Hermite blend of the fits'
//                         values and slopes
//   SV_LOESS_DIRECT       the local fit evaluated at every gene
// The kd-tree (a few dozen vertices) is built on the host from the sorted x;
// the fits and the blend run on the device.
#include "sv_internal.cuh"
#include <math.h>

void sv_count_moments(sv_context* ctx, const sv_counts* C, double* mean, double* sd);

namespace {

// One block per evaluation point x0 (any value in [x[0], x[n-1]]): the window
// [a, a + q) is the first a with x0 - x[a] <= x[a + q] - x0 (binary search:
// the difference falls with a); the block's threads stride over the window
// summing the weighted moments, then one thread solves the normal equations of
// the quadratic in x - x0.  val = its value at x0, slope (may be null) = its
// derivative.  A window of zero width gives unit weights, or NaN when
// flat_nan is set (the 0/0 of the weight formula).
constexpr int LOESS_THREADS = 256;
__global__ void __launch_bounds__(LOESS_THREADS)
    k_loess(const double* __restrict__ xs, const double* __restrict__ ys, int64_t n, int64_t q,
            const double* __restrict__ x0s, int64_t m, int flat_nan, double* __restrict__ val,
            double* __restrict__ slope) {
  __shared__ double part[LOESS_THREADS / 32][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t i = blockIdx.x; i < m; i += gridDim.x) {
    const double x0 = x0s[i];
    int64_t lo = 0, hi = n - q;   // answer in [0, n - q]
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if ((x0 - xs[mid]) > (xs[mid + q] - x0)) lo = mid + 1;
      else hi = mid;
    }
    const int64_t a = lo;
    const double dq = fmax(x0 - xs[a], xs[a + q - 1] - x0);
    if (dq <= 0 && flat_nan) {
      if (threadIdx.x == 0) {
        val[i] = nan("");
        if (slope) slope[i] = nan("");
      }
      continue;
    }
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};   // s0..s4, r0..r2
    for (int64_t j = a + threadIdx.x; j < a + q; j += LOESS_THREADS) {
      double t = xs[j] - x0;
      double w = 1.0;
      if (dq > 0) {
        double u = fabs(t) / dq;
        double c = 1.0 - u * u * u;
        w = c * c * c;
      }
      double wt = w * t, wt2 = wt * t, y = ys[j];
      acc[0] += w;
      acc[1] += wt;
      acc[2] += wt2;
      acc[3] += wt2 * t;
      acc[4] += wt2 * t * t;
      acc[5] += w * y;
      acc[6] += wt * y;
      acc[7] += wt2 * y;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = sv_warp_sum(acc[k]);
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < 8; ++k) part[warp][k] = acc[k];
    __syncthreads();
    if (threadIdx.x == 0) {
      double S[8];
      for (int k = 0; k < 8; ++k) {
        S[k] = 0;
        for (int w = 0; w < LOESS_THREADS / 32; ++w) S[k] += part[w][k];
      }
      // [s0 s1 s2; s1 s2 s3; s2 s3 s4] b = r: Gaussian elimination, partial pivoting
      double M[3][4] = {{S[0], S[1], S[2], S[5]}, {S[1], S[2], S[3], S[6]}, {S[2], S[3], S[4], S[7]}};
      for (int c = 0; c < 3; ++c) {
        int p = c;
        for (int r = c + 1; r < 3; ++r)
          if (fabs(M[r][c]) > fabs(M[p][c])) p = r;
        if (p != c)
          for (int k = 0; k < 4; ++k) {
            double tmp = M[c][k];
            M[c][k] = M[p][k];
            M[p][k] = tmp;
          }
        for (int r = c + 1; r < 3; ++r) {
          double f = M[c][c] != 0.0 ? M[r][c] / M[c][c] : 0.0;
          for (int k = c; k < 4; ++k) M[r][k] -= f * M[c][k];
        }
      }
      double b2 = M[2][2] != 0.0 ? M[2][3] / M[2][2] : 0.0;
      double b1 = M[1][1] != 0.0 ? (M[1][3] - M[1][2] * b2) / M[1][1] : 0.0;
      double b0 = M[0][0] != 0.0 ? (M[0][3] - M[0][1] * b1 - M[0][2] * b2) / M[0][0] : 0.0;
      val[i] = b0;
      if (slope) slope[i] = b1;
    }
    __syncthreads();   // part is reused by the next point
  }
}

// One thread per point z of xs: the first leaf k whose upper bound bnd[k + 1]
// is >= z (the leaf the tree's descent reaches, left when z <= split), then the
// blend of the fits at its bounds (vval / vslope indexed like bnd).
__global__ void k_loess_blend(const double* __restrict__ xs, int64_t n, const double* __restrict__ bnd,
                              int64_t nb, const double* __restrict__ vval, const double* __restrict__ vslope,
                              int hermite, double* __restrict__ fit) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double z = xs[i];
    int64_t lo = 1, hi = nb - 1;   // first index in [1, nb - 1] with bnd >= z
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if (bnd[mid] < z) lo = mid + 1;
      else hi = mid;
    }
    int64_t k = lo - 1;
    double x0 = bnd[k], x1 = bnd[k + 1], f0 = vval[k], f1 = vval[k + 1];
    double h = x1 - x0;
    double y;
    if (!hermite) {
      double u = (z - x0) / h;     // 0/0 = NaN in a cell of zero width
      y = (1.0 - u) * f0 + u * f1;
    } else if (z == x0) {
      y = f0;
    } else if (z == x1) {
      y = f1;
    } else {
      double t = (z - x0) / h, t2 = t * t, t3 = t2 * t;
      y = (2 * t3 - 3 * t2 + 1) * f0 + (t3 - 2 * t2 + t) * h * vslope[k] + (-2 * t3 + 3 * t2) * f1 +
          (t3 - t2) * h * vslope[k + 1];
    }
    fit[i] = y;
  }
}

// The leaf bounds b_0 <= ... <= b_L of the kd-tree over the sorted xs (leaf i
// is [b_i, b_i+1]): a cell of L points is split when L > ceil(cell * span * n)
// and it has a positive width, at the (L div 2)-th smallest of its points for
// odd L, at the mean of the (L/2)-th and (L/2 + 1)-th for even L, the smaller
// half going left.
std::vector<double> loess_kdtree_bounds(const std::vector<double>& xs, double span) {
  const int64_t n = (int64_t)xs.size();
  const double cell = 0.2;
  const int64_t cutoff = (int64_t)ceil((cell * span) * (double)n);
  std::vector<double> b{xs[0]};
  struct Node {
    int64_t s, e;
    double lo, hi;
  };
  std::vector<Node> stack{{0, n, xs[0], xs[n - 1]}};
  while (!stack.empty()) {
    Node c = stack.back();
    stack.pop_back();
    const int64_t L = c.e - c.s;
    if (L <= cutoff || c.hi - c.lo <= 0) {
      b.push_back(c.hi);
      continue;
    }
    const int64_t mid = L / 2;
    const double med = (L & 1) ? xs[c.s + mid - 1] : (xs[c.s + mid - 1] + xs[c.s + mid]) / 2;
    stack.push_back({c.s + mid, c.e, med, c.hi});
    stack.push_back({c.s, c.s + mid, c.lo, med});
  }
  return b;
}

// one warp per gene: sum of min((x - mu) / esd, vmax)^2 over the stored
// counts plus the implicit zeros' share, / (n - 1).  The square depends on the
// count only: lane l holds it for the count l + 1, and a stored count in
// 1..32 (nearly all of them) reads it from that lane instead of dividing.
__global__ void k_vst_var(const int64_t* __restrict__ colptr, const int32_t* __restrict__ cnt,
                          int64_t n_genes, int64_t n_cells, const double* __restrict__ mu,
                          const double* __restrict__ esd, double vmax, double* __restrict__ out) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t g = warp; g < n_genes; g += nwarps) {
    double e = esd[g];
    if (e == 0.0) {
      if (lane == 0) out[g] = 0.0;
      continue;
    }
    double m = mu[g];
    double zl = fmin(((double)(lane + 1) - m) / e, vmax);
    double tab = zl * zl;
    int64_t s = colptr[g], t = colptr[g + 1];
    double acc = 0;
    for (int64_t b = s; b < t; b += 32) {   // every lane runs every round (the shuffle)
      int64_t i = b + lane;
      int c = i < t ? cnt[i] : 1;
      double z2 = __shfl_sync(0xffffffffu, tab, (int)(((unsigned)c - 1u) & 31u));
      if (c < 1 || c > 32) {
        double z = fmin(((double)c - m) / e, vmax);
        z2 = z * z;
      }
      if (i < t) acc += z2;
    }
    acc = sv_warp_sum(acc);
    if (lane == 0) {
      double z0 = fmin((0.0 - m) / e, vmax);
      out[g] = (acc + (double)(n_cells - (t - s)) * z0 * z0) / (double)(n_cells - 1);
    }
  }
}

}  // namespace

SV_API int sv_find_variable_features_vst_surface(sv_context* ctx, const sv_counts* C, int64_t nfeatures,
                                                 double loess_span, int surface, int64_t* features,
                                                 double* metric) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(C && C->ctx == ctx, "bad count-matrix handle");
  SV_REQUIRE(C->n_cells >= 2, "need at least two cells for a variance");
  SV_REQUIRE(nfeatures >= 0 && nfeatures <= C->n_genes, "nfeatures must be in 0..n_genes");
  SV_REQUIRE(loess_span > 0, "loess span must be positive");
  SV_REQUIRE(surface == SV_LOESS_INTERPOLATE || surface == SV_LOESS_HERMITE || surface == SV_LOESS_DIRECT,
             "unknown loess surface");
  const int64_t ng = C->n_genes;
  DevBuf<double> mean(ng), sd(ng);
  sv_count_moments(ctx, C, mean.get(), sd.get());
  std::vector<double> hm(ng), hs(ng);
  sv_d2h(ctx, hm.data(), mean.get(), ng * 8);
  sv_d2h(ctx, hs.data(), sd.get(), ng * 8);
  // non-constant genes, sorted by log10(mean) (ties by gene index)
  std::vector<int64_t> nc;
  for (int64_t g = 0; g < ng; ++g)
    if (hs[g] > 0) nc.push_back(g);
  int64_t n = (int64_t)nc.size();
  std::vector<double> esd(hs);
  if (n > 0) {
    std::vector<double> lx(n), ly(n);
    for (int64_t i = 0; i < n; ++i) {
      lx[i] = log10(hm[nc[i]]);
      ly[i] = log10(hs[nc[i]]);
    }
    std::vector<int64_t> ord(n);
    for (int64_t i = 0; i < n; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return lx[a] < lx[b]; });
    std::vector<double> xs(n), ys(n), fit(n);
    for (int64_t i = 0; i < n; ++i) {
      xs[i] = lx[ord[i]];
      ys[i] = ly[ord[i]];
    }
    int64_t q = std::max<int64_t>(3, std::min<int64_t>(n, (int64_t)floor((double)n * loess_span)));
    if (q > n) q = n;
    DevBuf<double> dx(n), dy(n), df(n);
    sv_h2d(ctx, dx.get(), xs.data(), n * 8);
    sv_h2d(ctx, dy.get(), ys.data(), n * 8);
    if (surface == SV_LOESS_DIRECT) {
      sv_launch(ctx, "vst_loess", k_loess, dim3(sv_grid_for(ctx, n, 1, 8)), dim3(LOESS_THREADS), 0,
                (const double*)dx.get(), (const double*)dy.get(), n, q, (const double*)dx.get(), n, 0,
                df.get(), (double*)nullptr);
    } else {
      std::vector<double> bnd = loess_kdtree_bounds(xs, loess_span);
      const int64_t nb = (int64_t)bnd.size();   // >= 2: the extremes
      DevBuf<double> db(nb), dv(nb), ds(nb);
      sv_h2d(ctx, db.get(), bnd.data(), nb * 8);
      sv_launch(ctx, "vst_loess_vertices", k_loess, dim3(sv_grid_for(ctx, nb, 1, 8)), dim3(LOESS_THREADS), 0,
                (const double*)dx.get(), (const double*)dy.get(), n, q, (const double*)db.get(), nb, 1,
                dv.get(), ds.get());
      sv_launch(ctx, "vst_loess_blend", k_loess_blend, dim3(sv_grid_for(ctx, n, 128, 4)), dim3(128), 0,
                (const double*)dx.get(), n, (const double*)db.get(), nb, (const double*)dv.get(),
                (const double*)ds.get(), surface == SV_LOESS_HERMITE ? 1 : 0, df.get());
    }
    sv_d2h(ctx, fit.data(), df.get(), n * 8);
    for (int64_t i = 0; i < n; ++i) {
      double e = pow(10.0, fit[i]);
      esd[nc[ord[i]]] = std::isnan(e) ? 0.0 : e;   // variablefeatures.jl:46-47
    }
  }
  DevBuf<double> desd(ng), dout(ng);
  sv_h2d(ctx, desd.get(), esd.data(), ng * 8);
  sv_launch(ctx, "vst_var", k_vst_var, dim3(sv_grid_for(ctx, ng * 32, 256, 8)), dim3(256), 0,
            (const int64_t*)C->csc_colptr.get(), (const int32_t*)C->csc_count.get(), ng, C->n_cells,
            (const double*)mean.get(), (const double*)desd.get(), sqrt((double)C->n_cells), dout.get());
  std::vector<double> hv(ng);
  sv_d2h(ctx, hv.data(), dout.get(), ng * 8);
  if (metric) std::copy(hv.begin(), hv.end(), metric);
  if (features && nfeatures > 0) {
    // partialsortperm(metric, 1:nfeatures, rev=true): largest first, ties by index
    std::vector<int64_t> idx(ng);
    for (int64_t g = 0; g < ng; ++g) idx[g] = g;
    std::partial_sort(idx.begin(), idx.begin() + nfeatures, idx.end(), [&](int64_t a, int64_t b) {
      return hv[a] > hv[b] || (hv[a] == hv[b] && a < b);
    });
    for (int64_t i = 0; i < nfeatures; ++i) features[i] = idx[i] + 1;
  }
  SV_CATCH
}

SV_API int sv_find_variable_features_vst(sv_context* ctx, const sv_counts* C, int64_t nfeatures,
                                         double loess_span, int64_t* features, double* metric) {
  return sv_find_variable_features_vst_surface(ctx, C, nfeatures, loess_span, SV_LOESS_INTERPOLATE, features,
                                               metric);
}

SV_API int64_t sv_loess_vertices(const double* xs, int64_t n, double loess_span, double* bounds, int64_t cap) {
  if (!xs || n < 1 || !(loess_span > 0) || (cap > 0 && !bounds)) return SV_ERR_ARG;
  for (int64_t i = 1; i < n; ++i)
    if (!(xs[i - 1] <= xs[i])) return SV_ERR_ARG;
  try {
    std::vector<double> v(xs, xs + n);
    std::vector<double> b = loess_kdtree_bounds(v, loess_span);
    for (int64_t i = 0; i < (int64_t)b.size() && i < cap; ++i) bounds[i] = b[i];
    return (int64_t)b.size();
  } catch (const std::bad_alloc&) {
    return SV_ERR_OOM;
  }
}
