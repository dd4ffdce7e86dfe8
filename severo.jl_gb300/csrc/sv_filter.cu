// filter_counts on the device (src/filtering.jl:15-35,98-103): cells, then
// genes, removed from a resident count matrix without a host round trip.
//
//   detected(c) = #{g : A[c, g] > min_feature_count}   (implicit zeros count
//                 when min_feature_count < 0, as sum(>(t), A, dims=2) tests them)
//   keep cell   = detected >= min_features  and, when min_umi > 0, sum_g A[c, g] > min_umi
//   keep gene   = #{kept c : A[c, g] > 0} >= min_cells       (on the filtered cells)
//
// The result is a new count matrix: the kept rows renumbered in order, the kept
// genes' columns compacted in order (stored entries, explicit zeros included,
// are copied as they are), and its CSR copy rebuilt on the device.
#include "sv_internal.cuh"

namespace {

// one warp per cell over the CSR copy
__global__ void k_filter_cells(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ cnt,
                               int64_t n_cells, int64_t n_genes, int64_t min_feature_count,
                               int64_t min_features, int64_t min_umi, unsigned char* __restrict__ keep,
                               int64_t* __restrict__ keep64) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = warp; c < n_cells; c += nwarps) {
    int64_t s = rowptr[c], e = rowptr[c + 1];
    long long det = 0, umi = 0;
    for (int64_t i = s + lane; i < e; i += 32) {
      int32_t v = cnt[i];
      det += (int64_t)v > min_feature_count;
      umi += v;
    }
    det = sv_warp_sum(det);
    umi = sv_warp_sum(umi);
    if (lane == 0) {
      if (min_feature_count < 0) det += n_genes - (e - s);
      bool k = det >= min_features && (min_umi <= 0 || umi > min_umi);
      keep[c] = k;
      keep64[c] = k;
    }
  }
}

// one warp per gene over the CSC copy: cells (kept, count > 0) and kept entries
__global__ void k_filter_genes(const int64_t* __restrict__ colptr, const int32_t* __restrict__ rowidx,
                               const int32_t* __restrict__ cnt, int64_t n_genes,
                               const unsigned char* __restrict__ cell_keep, int64_t min_cells,
                               unsigned char* __restrict__ keep, int64_t* __restrict__ keep64,
                               int64_t* __restrict__ newlen) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t g = warp; g < n_genes; g += nwarps) {
    int64_t s = colptr[g], e = colptr[g + 1];
    long long cells = 0, kept = 0;
    for (int64_t i = s + lane; i < e; i += 32) {
      bool k = cell_keep[rowidx[i]];
      kept += k;
      cells += k && cnt[i] > 0;
    }
    cells = sv_warp_sum(cells);
    kept = sv_warp_sum(kept);
    if (lane == 0) {
      bool k = cells >= min_cells;
      keep[g] = k;
      keep64[g] = k;
      newlen[g] = k ? kept : 0;
    }
  }
}

// one warp per kept gene: copy its kept entries in order (warp ballot
// compaction), rows renumbered; writes the new column pointer
__global__ void k_filter_write(const int64_t* __restrict__ colptr, const int32_t* __restrict__ rowidx,
                               const int32_t* __restrict__ cnt, int64_t n_genes,
                               const unsigned char* __restrict__ cell_keep,
                               const int64_t* __restrict__ cell_new,
                               const unsigned char* __restrict__ gene_keep,
                               const int64_t* __restrict__ gene_new, const int64_t* __restrict__ start,
                               int64_t* __restrict__ out_colptr, int32_t* __restrict__ out_row,
                               int32_t* __restrict__ out_cnt) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t g = warp; g < n_genes; g += nwarps) {
    if (!gene_keep[g]) continue;
    int64_t dst = start[g];
    if (lane == 0) out_colptr[gene_new[g]] = dst;
    int64_t s = colptr[g], e = colptr[g + 1];
    for (int64_t b = s; b < e; b += 32) {
      int64_t i = b + lane;
      int32_t r = i < e ? rowidx[i] : 0;
      bool k = i < e && cell_keep[r];
      unsigned m = __ballot_sync(0xffffffffu, k);
      if (k) {
        int64_t o = dst + __popc(m & ((1u << lane) - 1u));
        out_row[o] = (int32_t)cell_new[r];
        out_cnt[o] = cnt[i];
      }
      dst += __popc(m);
    }
  }
}

__global__ void k_set_i64(int64_t* p, int64_t v) { *p = v; }

}  // namespace

// The compaction shared by filter_counts and select_cells: rows with
// ckeep[c] (device mask, ck64 its 0/1 copy), genes passing min_cells.
static sv_counts* compact(sv_context* ctx, const sv_counts* A, DevBuf<unsigned char>& ckeep,
                          DevBuf<int64_t>& ck64, int64_t min_cells, DevBuf<unsigned char>& gkeep) {
  const int64_t nc = A->n_cells, ng = A->n_genes;
  DevBuf<int64_t> cnew(nc + 1), gk64(ng + 1), gnew(ng + 1), glen(ng + 1), gstart(ng + 1);
  sv_scan_i64(ctx, ck64.get(), cnew.get(), nc);
  sv_launch(ctx, "filter_genes", k_filter_genes, dim3(sv_grid_for(ctx, ng * 32, 256)), dim3(256), 0,
            (const int64_t*)A->csc_colptr.get(), (const int32_t*)A->csc_rowidx.get(),
            (const int32_t*)A->csc_count.get(), ng, (const unsigned char*)ckeep.get(), min_cells,
            gkeep.get(), gk64.get(), glen.get());
  sv_scan_i64(ctx, gk64.get(), gnew.get(), ng);
  sv_scan_i64(ctx, glen.get(), gstart.get(), ng);
  int64_t nc2 = sv_read_i64(ctx, cnew.get() + nc);
  int64_t ng2 = sv_read_i64(ctx, gnew.get() + ng);
  int64_t nnz2 = sv_read_i64(ctx, gstart.get() + ng);
  auto* c = new sv_counts();
  try {
    c->ctx = ctx;
    c->n_cells = nc2;
    c->n_genes = ng2;
    c->nnz = nnz2;
    c->csc_colptr.alloc(ng2 + 1);
    c->csc_rowidx.alloc(std::max<int64_t>(1, nnz2));
    c->csc_count.alloc(std::max<int64_t>(1, nnz2));
    sv_launch(ctx, "filter_write", k_filter_write, dim3(sv_grid_for(ctx, ng * 32, 256)), dim3(256), 0,
              (const int64_t*)A->csc_colptr.get(), (const int32_t*)A->csc_rowidx.get(),
              (const int32_t*)A->csc_count.get(), ng, (const unsigned char*)ckeep.get(),
              (const int64_t*)cnew.get(), (const unsigned char*)gkeep.get(), (const int64_t*)gnew.get(),
              (const int64_t*)gstart.get(), c->csc_colptr.get(), c->csc_rowidx.get(), c->csc_count.get());
    sv_launch(ctx, "filter_write", k_set_i64, dim3(1), dim3(1), 0, c->csc_colptr.get() + ng2, nnz2);
    sv_build_csr_from_csc(ctx, c);
  } catch (...) {
    delete c;
    throw;
  }
  return c;
}

__global__ void k_range_mask(int64_t n, int64_t r0, int64_t r1, unsigned char* __restrict__ keep,
                             int64_t* __restrict__ keep64) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    bool k = i >= r0 && i < r1;
    keep[i] = k;
    keep64[i] = k;
  }
}

// The cells [r0, r1) of a count matrix as a count matrix of their own (all
// genes kept), e.g. one sample of samples stacked by cells.
SV_API int sv_counts_select_cells(sv_context* ctx, const sv_counts* A, int64_t r0, int64_t r1,
                                  sv_counts** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(A && A->ctx == ctx && out, "bad argument");
  SV_REQUIRE(0 <= r0 && r0 < r1 && r1 <= A->n_cells, "cell range out of bounds");
  DevBuf<unsigned char> ckeep(A->n_cells), gkeep(A->n_genes);
  DevBuf<int64_t> ck64(A->n_cells + 1);
  sv_launch(ctx, "filter_cells", k_range_mask, dim3(sv_grid_for(ctx, A->n_cells, 256)), dim3(256), 0,
            A->n_cells, r0, r1, ckeep.get(), ck64.get());
  *out = compact(ctx, A, ckeep, ck64, 0, gkeep);
  sv_sync(ctx);
  SV_CATCH
}

SV_API int sv_filter_counts(sv_context* ctx, const sv_counts* A, int64_t min_cells,
                            int64_t min_features, int64_t min_feature_count, int64_t min_umi,
                            uint8_t* cells_kept, uint8_t* genes_kept, sv_counts** out) {
  SV_TRY
  sv_ctx_check(ctx);
  SV_REQUIRE(A && A->ctx == ctx, "bad count-matrix handle");
  SV_REQUIRE(out, "out is required");
  const int64_t nc = A->n_cells, ng = A->n_genes;
  DevBuf<unsigned char> ckeep(nc), gkeep(ng);
  DevBuf<int64_t> ck64(nc + 1);
  sv_launch(ctx, "filter_cells", k_filter_cells, dim3(sv_grid_for(ctx, nc * 32, 256)), dim3(256), 0,
            (const int64_t*)A->csr_rowptr.get(), (const int32_t*)A->csr_count.get(), nc, ng,
            min_feature_count, min_features, min_umi, ckeep.get(), ck64.get());
  sv_counts* c = compact(ctx, A, ckeep, ck64, min_cells, gkeep);
  try {
    if (cells_kept) sv_d2h(ctx, cells_kept, ckeep.get(), nc);
    if (genes_kept) sv_d2h(ctx, genes_kept, gkeep.get(), ng);
    sv_sync(ctx);
  } catch (...) {
    delete c;
    throw;
  }
  *out = c;
  SV_CATCH
}
