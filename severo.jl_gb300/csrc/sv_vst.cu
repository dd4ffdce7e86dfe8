// find_variable_features(:vst) (src/variablefeatures.jl:19-50,128-160) on the
// device-resident counts: per-gene mean and std of the counts, a local
// quadratic regression of log10(std) on log10(mean) over the non-constant
// genes, the expected std 10^fit, and the variance of the standardised counts
// clipped at sqrt(n_cells); the nfeatures genes of largest variance.
//
// The regression is loess (Cleveland 1979; Cleveland & Grosse 1991) evaluated
// directly at every gene: the q = floor(span * n) nearest genes in log10(mean)
// (a contiguous window of the sorted values), tricube weights, weighted least
// squares in x - x0, FP64.  The reference calls Loess.jl, whose default
// interpolates this fit between kd-tree vertices; that interpolation is not
// restated, so the metric agrees with the reference to the interpolation error.
#include "sv_internal.cuh"
#include <math.h>

void sv_count_moments(sv_context* ctx, const sv_counts* C, double* mean, double* sd);

namespace {

// One thread per evaluation point (sorted x): the window [a, a + q) is the
// first a with x0 - x[a] <= x[a + q] - x0 (binary search: the difference falls
// with a), then the weighted normal equations of the quadratic.
__global__ void k_loess(const double* __restrict__ xs, const double* __restrict__ ys, int64_t n, int64_t q,
                        double* __restrict__ fit) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double x0 = xs[i];
    int64_t lo = 0, hi = n - q;   // answer in [0, n - q]
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if ((x0 - xs[mid]) > (xs[mid + q] - x0)) lo = mid + 1;
      else hi = mid;
    }
    int64_t a = lo;
    double dq = fmax(x0 - xs[a], xs[a + q - 1] - x0);
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0, r0 = 0, r1 = 0, r2 = 0;
    for (int64_t j = a; j < a + q; ++j) {
      double t = xs[j] - x0;
      double w = 1.0;
      if (dq > 0) {
        double u = fabs(t) / dq;
        double c = 1.0 - u * u * u;
        w = c * c * c;
      }
      double wt = w * t, wt2 = wt * t;
      s0 += w;
      s1 += wt;
      s2 += wt2;
      s3 += wt2 * t;
      s4 += wt2 * t * t;
      r0 += w * ys[j];
      r1 += wt * ys[j];
      r2 += wt2 * ys[j];
    }
    // [s0 s1 s2; s1 s2 s3; s2 s3 s4] b = r: Gaussian elimination, partial pivoting
    double M[3][4] = {{s0, s1, s2, r0}, {s1, s2, s3, r1}, {s2, s3, s4, r2}};
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
    fit[i] = b0;
  }
}

// one warp per gene: sum of min((x - mu) / esd, vmax)^2 over the stored
// counts plus the implicit zeros' share, / (n - 1)
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
    int64_t s = colptr[g], t = colptr[g + 1];
    double acc = 0;
    for (int64_t i = s + lane; i < t; i += 32) {
      double z = fmin(((double)cnt[i] - m) / e, vmax);
      acc += z * z;
    }
    acc = sv_warp_sum(acc);
    if (lane == 0) {
      double z0 = fmin((0.0 - m) / e, vmax);
      out[g] = (acc + (double)(n_cells - (t - s)) * z0 * z0) / (double)(n_cells - 1);
    }
  }
}

}  // namespace

SV_API int sv_find_variable_features_vst(sv_context* ctx, const sv_counts* C, int64_t nfeatures,
                                         double loess_span, int64_t* features, double* metric) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(C && C->ctx == ctx, "bad count-matrix handle");
  SV_REQUIRE(C->n_cells >= 2, "need at least two cells for a variance");
  SV_REQUIRE(nfeatures >= 0 && nfeatures <= C->n_genes, "nfeatures must be in 0..n_genes");
  SV_REQUIRE(loess_span > 0, "loess span must be positive");
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
    sv_launch(ctx, "vst_loess", k_loess, dim3(sv_grid_for(ctx, n, 128, 4)), dim3(128), 0,
              (const double*)dx.get(), (const double*)dy.get(), n, q, df.get());
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
