/*
 * severo_gpu.h -- C ABI of libseverogpu.so, the GB300 (sm_103a) implementation of
 * Severo.jl's embedding hot path:
 *
 *   normalize_cells -> scale_features (implicit centre / scale / clip)
 *   -> irlba PCA over the CenteredMatrix products -> nearest_neighbours
 *   -> shared_nearest_neighbours / jaccard_index
 *
 * Every entry point is plain C: pointers, sizes and enums, no C++ or torch types.
 * All functions except the four FindNeighbours* compatibility symbols return an
 * int status (SV_OK = 0, negative on failure) and never throw or abort; the
 * message of the most recent failure on the calling thread is available through
 * sv_last_error().  Host pointers passed in are read (or written) before the call
 * returns; device-resident results live in opaque handles owned by the caller
 * and released with the matching *_free function.
 *
 * Matrix orientation follows Severo.jl: count / data matrices are cells x genes
 * (src/Severo.jl:26-32), handed over as Julia SparseMatrixCSC arrays (one column
 * per gene; row indices are cells).  Dense host matrices are column-major, as in
 * Julia.  Neighbour indices at the boundary are 1-based Int32, as returned by the
 * native FindNeighbours* routines (src/neighbours.jl:22,37-39).
 *
 * A context owns one CUDA stream on one device.  Handles created from a context
 * are used with that context only, and one context is not re-entrant: calls on
 * the same context must not overlap in time.  Different contexts are independent.
 */
#ifndef SEVERO_GPU_H
#define SEVERO_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------- */
#define SV_OK               0
#define SV_ERR_ARG         -1   /* invalid argument (size, pointer, enum, index range) */
#define SV_ERR_OOM         -2   /* device or pinned-host allocation failed               */
#define SV_ERR_CUDA        -3   /* a CUDA runtime error                                   */
#define SV_ERR_NOCONV      -4   /* irlba did not converge within maxit restarts           */
#define SV_ERR_UNSUPPORTED -5   /* a size or combination this build does not handle       */
#define SV_ERR_STATE       -6   /* handle used with the wrong context or in a bad state   */
#define SV_ERR_DEVICE      -7   /* a kernel reported a bounds / iteration-limit failure   */

/* ---- element types ---------------------------------------------------------- */
#define SV_I32   1
#define SV_I64   2
#define SV_F32   3
#define SV_F64   4
#define SV_BF16  5   /* storage type of the mixed-precision form (values only) */

/* ---- normalisation methods (src/normalize.jl:45-51) ------------------------- */
#define SV_LOGNORMALIZE   0
#define SV_RELATIVECOUNTS 1

/* ---- kNN metric and distance-kernel precision ------------------------------ */
#define SV_EUCLIDEAN 0
#define SV_COSINE    1
#define SV_KNN_FP32  0   /* FP32 CUDA-core distance tiles                           */
#define SV_KNN_BF16  1   /* BF16 tcgen05 distance tiles, FP32 accumulation in TMEM  */

typedef struct sv_context  sv_context;
typedef struct sv_counts   sv_counts;    /* device CSC + CSR copies of a count matrix  */
typedef struct sv_data     sv_data;      /* normalised values over both copies         */
typedef struct sv_centered sv_centered;  /* implicit CenteredMatrix over a feature set */
typedef struct sv_embed    sv_embed;     /* device-resident PCA result                 */
typedef struct sv_knn      sv_knn;       /* device-resident neighbour lists            */
typedef struct sv_graph    sv_graph;     /* device-resident SNN graph (CSC)            */
typedef struct sv_batch    sv_batch;     /* samples stacked by cells, scaled per sample */

/* ---- context, errors, diagnostics ----------------------------------------- */
int  sv_version(void);                                   /* 100 * major + minor */
int  sv_last_error(char* buf, size_t len);               /* copies the message, returns its length */
int  sv_context_create(int device, sv_context** out);
int  sv_context_destroy(sv_context* ctx);
int  sv_synchronize(sv_context* ctx);
/* Pin (page-lock) caller memory so that uploads run at full link speed. */
int  sv_host_register(void* ptr, size_t bytes);
int  sv_host_unregister(void* ptr);
int  sv_host_alloc(void** ptr, size_t bytes);            /* pinned host allocation */
int  sv_host_free(void* ptr);
/* Device time between two marks on the context stream (CUDA events). */
int  sv_mark(sv_context* ctx, int slot);                 /* slot 0..15 */
int  sv_elapsed_ms(sv_context* ctx, int slot_a, int slot_b, double* ms);
/* Number of kernels this library launched on the context since creation. */
int  sv_launch_count(sv_context* ctx, int64_t* count);
/* Per-kernel timing with CUDA events around each launch (off by default). */
int  sv_profile_enable(sv_context* ctx, int enable);
int  sv_profile_reset(sv_context* ctx);
/* Sum of device time (ms) and number of launches of kernels whose name contains
 * `name_substring`.  Synchronises the context. */
int  sv_profile_query(sv_context* ctx, const char* name_substring, double* total_ms, int64_t* launches);
/* Writes "name launches total_ms" lines for every kernel seen into buf. */
int  sv_profile_report(sv_context* ctx, char* buf, size_t len);
int  sv_device_memory(sv_context* ctx, size_t* free_bytes, size_t* total_bytes);
/* Self-test of the bounded waits of the tensor-core kNN kernel: one warp waits
 * on an mbarrier that nothing completes, with a limit of `cycles` (1 .. 2^32)
 * clock cycles; the wait runs out and the call returns SV_ERR_DEVICE through
 * the context's status word, the context staying usable (no reference
 * counterpart: it exercises this library's failure path without a fault). */
int  sv_selftest_wait_timeout(sv_context* ctx, long long cycles);

/* ---- count matrix ------------------------------------------------------------
 * sv_counts_upload_csc replaces holding the CountMatrix of src/Severo.jl:26-27
 * in host memory: it copies a cells x genes SparseMatrixCSC (colptr, rowval,
 * nzval, each SV_I32 or SV_I64 as declared by its *_type, nzval also SV_F32 or
 * SV_F64; index_base 0 or 1, 1 for Julia's arrays) to the device and builds
 * the cell-major (CSR) copy there.
 * Row indices must be strictly increasing within each column (Julia's
 * invariant); this is checked on the device and reported as SV_ERR_ARG. */
int sv_counts_upload_csc(sv_context* ctx, int64_t n_cells, int64_t n_genes, int64_t nnz,
                         const void* colptr, int colptr_type, const void* rowval,
                         int rowval_type, const void* nzval, int val_type, int index_base,
                         sv_counts** out);
/* sv_counts_upload_csr takes the cell-major arrays as the file formats store
 * them: the features x barcodes CSC of a 10X CellRanger HDF5 file
 * (src/input.jl:158-187) and of the "/counts" HDF5 layout (:210-225), or the
 * cells x genes CSR of an AnnData X (:250-287), which the reference turns into
 * a cells x genes SparseMatrixCSC on the host with copy(X').  Here the arrays
 * go to the device as they are and the gene-major (CSC) copy is built there.
 * Features may be unsorted within a cell (they are sorted on the device);
 * duplicate features within a cell are SV_ERR_ARG.  For both uploads the counts
 * may be SV_I32, SV_I64, SV_F32 or SV_F64; wider and floating types must hold
 * whole numbers in [0, 2^31) (convert_counts, src/input.jl:776-780, converts
 * real-valued files to Int32), else SV_ERR_ARG. */
int sv_counts_upload_csr(sv_context* ctx, int64_t n_cells, int64_t n_genes, int64_t nnz,
                         const void* rowptr, int rowptr_type, const void* colidx,
                         int colidx_type, const void* nzval, int val_type, int index_base,
                         sv_counts** out);
/* MatrixMarket coordinate files (readMM, src/input.jl:27-115, as _read_10X
 * reads matrix.mtx[.gz], :199-208), parsed on the device: the entry section is
 * streamed to HBM as it lies in the file and parsed there, one line per thread.
 * rows_are_features = 1 for the 10X layout (features x barcodes; the reference
 * transposes it with copy(X')), 0 when the file's rows are the cells.  Entries
 * naming the same position are summed and explicit zeros kept, as
 * sparse(I, J, V) does.  Header errors carry the reference's messages; a
 * malformed entry line, an index outside the declared size or a count that is
 * not a whole number in [0, 2^31) is SV_ERR_ARG.  Paths ending in ".gz" are
 * read through libz.so.1 (SV_ERR_UNSUPPORTED when it cannot be loaded).
 * sv_counts_parse_mtx reads the same format from len bytes of host memory. */
int sv_counts_read_mtx(sv_context* ctx, const char* path, int rows_are_features, sv_counts** out);
int sv_counts_parse_mtx(sv_context* ctx, const char* text, int64_t len, int rows_are_features,
                        sv_counts** out);
/* Synthetic negative-binomial counts generated on the device (benchmarks).
 * Cells x genes; mean depth * s_c * mu_g * exp(lfc[cluster(c), g]); variance
 * mean + dispersion * mean^2.  mu_g (n_genes), s_c (n_cells), cluster ids
 * (n_cells, may be NULL) and lfc (n_clusters x n_genes row-major, may be NULL)
 * are host arrays. Counter-based hashing of (seed, cell, gene) makes the CSC and
 * CSR copies identical entry for entry. */
int sv_counts_generate(sv_context* ctx, int64_t n_cells, int64_t n_genes,
                       const float* mu_g, const float* s_c, const int32_t* cluster,
                       const float* lfc, int32_t n_clusters, double depth,
                       double dispersion, uint64_t seed, sv_counts** out);
int sv_counts_info(const sv_counts* c, int64_t* n_cells, int64_t* n_genes, int64_t* nnz);
/* Copies the CSC arrays back (0-based int64 colptr, int32 rowval, int32 counts). */
int sv_counts_download_csc(sv_context* ctx, const sv_counts* c, int64_t* colptr,
                           int32_t* rowval, int32_t* counts);
/* Copies the CSR arrays back (0-based int64 rowptr, int32 colidx, int32 counts). */
int sv_counts_download_csr(sv_context* ctx, const sv_counts* c, int64_t* rowptr,
                           int32_t* colidx, int32_t* counts);
int sv_counts_free(sv_counts* c);

/* ---- filter_counts (src/filtering.jl:15-35,98-103) --------------------------
 * Cells first: a cell is kept when at least min_features of its genes have a
 * count > min_feature_count (implicit zeros included in the test) and, when
 * min_umi > 0, its count total is > min_umi.  Then genes: kept when at least
 * min_cells of the kept cells have a count > 0.  *out is a new count matrix
 * (kept rows and columns, in order, stored entries copied as they are);
 * cells_kept (n_cells) / genes_kept (n_genes) receive the 0/1 masks the
 * reference returns as CI / FI (either may be NULL).  filter_cells is
 * min_cells = 0; filter_features is the cell thresholds at 0. */
int sv_filter_counts(sv_context* ctx, const sv_counts* counts, int64_t min_cells,
                     int64_t min_features, int64_t min_feature_count, int64_t min_umi,
                     uint8_t* cells_kept, uint8_t* genes_kept, sv_counts** out);
/* The cells [r0, r1) (0-based, end exclusive) of a count matrix as a count
 * matrix of their own, every gene kept (one sample of samples stacked by cells). */
int sv_counts_select_cells(sv_context* ctx, const sv_counts* counts, int64_t r0, int64_t r1,
                           sv_counts** out);

/* ---- find_variable_features(:vst) (src/variablefeatures.jl:19-50,128-160) ----
 * Per-gene mean and std (n - 1) of the counts; over the genes with std > 0 a
 * local quadratic regression (loess, span loess_span, tricube weights) of
 * log10(std) on log10(mean); expected std 10^fit (NaN -> 0); metric = variance
 * of min((x - mean)/expected std, sqrt(n_cells)) over all cells (implicit
 * zeros included).  features receives the nfeatures genes of largest metric
 * (1-based, largest first, ties by index); metric (n_genes) may be NULL.
 * surface selects how the fit is evaluated at the genes:
 *   SV_LOESS_INTERPOLATE  fits at the vertices of the kd-tree that Loess.jl's
 *                         loess builds (cells of at most ceil(0.2 span n)
 *                         genes), blended linearly inside each cell: the
 *                         loess / predict calls of variablefeatures.jl:41-42
 *   SV_LOESS_HERMITE      the same vertices, cubic Hermite blend of the
 *                         vertex fits' values and slopes
 *   SV_LOESS_DIRECT       the local fit evaluated at every gene
 * sv_find_variable_features_vst is the call with SV_LOESS_INTERPOLATE. */
#define SV_LOESS_INTERPOLATE 0
#define SV_LOESS_HERMITE     1
#define SV_LOESS_DIRECT      2
int sv_find_variable_features_vst(sv_context* ctx, const sv_counts* counts, int64_t nfeatures,
                                  double loess_span, int64_t* features, double* metric);
int sv_find_variable_features_vst_surface(sv_context* ctx, const sv_counts* counts, int64_t nfeatures,
                                          double loess_span, int surface, int64_t* features,
                                          double* metric);
/* The leaf bounds b_0 <= b_1 <= ... of that kd-tree over n sorted values xs
 * (leaf i is [b_i, b_i+1]; b_0 and the last are the extremes): writes
 * min(count, cap) of them and returns the count, or SV_ERR_ARG (xs unsorted,
 * n < 1, span <= 0).  Host only: needs no device. */
int64_t sv_loess_vertices(const double* xs, int64_t n, double loess_span, double* bounds, int64_t cap);

/* ---- normalize_cells (src/normalize.jl:17-55,76-79) -------------------------
 * method SV_LOGNORMALIZE or SV_RELATIVECOUNTS; value dtype SV_F64 (the
 * reference default), SV_F32 or SV_BF16 (values computed in FP32 and stored
 * rounded to BF16).  b = (scale_factor * a) / s_cell in dtype (normalize.jl:27),
 * then log1p for SV_LOGNORMALIZE (normalize.jl:36).  Both the CSC and the CSR
 * copy receive values; the sparsity pattern is the counts'. */
int sv_normalize_cells(sv_context* ctx, const sv_counts* counts, int method,
                       double scale_factor, int dtype, sv_data** out);
/* normalize_cells for callers that cannot let this library allocate device
 * memory.  No counterpart in the reference: it exists for hosts that keep the
 * whole device memory budget in their own pool (a language runtime such as
 * Julia's, which hands out device arrays from its pool and would otherwise
 * compete with the library's cudaMalloc) and for services that must not
 * allocate device memory once started.  Inputs and output are device arrays
 * owned by the caller: a 0-based cells x genes CSC (colptr int64
 * [n_genes + 1], rowval and counts int32 [nnz]) and values (FP32 [nnz], CSC
 * order, the same numbers as the SV_F32 form of sv_normalize_cells).  The
 * per-cell totals live in a file-scope device array of 2,097,152 entries
 * (16 MiB on every GPU that loads the library, until the process exits); more
 * cells are rejected with SV_ERR_ARG.  Nothing is allocated: no cudaMalloc, no
 * cudaFree.  The first call on a device looks up the array's device address
 * with that device current and keeps it for the life of the process (a
 * cudaDeviceReset on that device makes the kept address stale).  Work runs on
 * `stream` (a cudaStream_t, NULL for the legacy default stream); the call waits
 * for it, because a row index outside [0, n_cells) -- skipped by the kernels,
 * its value set to 0 -- is reported as SV_ERR_ARG.  Every call on a device
 * shares the array: calls that overlap on the GPU (other streams, other host
 * threads) race and corrupt each other's totals. */
int sv_normalize_csc_noalloc(const int64_t* colptr, const int32_t* rowval, const int32_t* counts,
                             int64_t n_cells, int64_t n_genes, int64_t nnz, int method,
                             double scale_factor, float* values, void* stream);
/* Copies the CSC values (in the data's dtype; BF16 as uint16 bit patterns). */
int sv_data_download_csc(sv_context* ctx, const sv_data* d, void* nzval);
int sv_data_download_csr(sv_context* ctx, const sv_data* d, void* nzval);
/* Per-cell totals s_c (normalize.jl:24), int64. */
int sv_data_cell_totals(sv_context* ctx, const sv_data* d, int64_t* totals);
int sv_data_free(sv_data* d);

/* ---- scale_features (src/scaling.jl:199-217,335-357) ------------------------
 * features: 1-based gene indices (nfeatures of them, no duplicates), or NULL
 * for all genes (src/scaling.jl:338-340).  Per feature, FP64 mean and unbiased
 * variance with the implicit zeros (scaling.jl:18-34); mu = mean/std
 * (scaling.jl:207); the represented matrix is
 *     Xs[c, f] = min(a[c, f] / std_f, scale_max + mu_f) - mu_f   (a != 0)
 *     Xs[c, f] = -mu_f                                            (a == 0)
 * (scaling.jl:209-212,219-233).  Nothing is densified: the products below apply
 * the scaling, clip and centring on the fly. scale_max may be +Inf. */
int sv_scale_features(sv_context* ctx, const sv_data* data, const int64_t* features,
                      int64_t nfeatures, double scale_max, sv_centered** out);
/* CenteredMatrix(A, mu) (src/scaling.jl:224-232) for an arbitrary sparse A
 * (n_rows x n_cols CSC, 0-based int64 colptr / rowval, FP64 values stored as
 * dtype SV_F64 or SV_F32) and centring vector mu (n_cols): the represented
 * matrix is A - 1 mu^T (no scaling, no clip).  Used by the reference's
 * CenteredMatrix and irlba tests (test/test_scaling.jl:70-113,
 * test/test_irlba.jl:65-115). */
int sv_centered_create(sv_context* ctx, int64_t n_rows, int64_t n_cols, int64_t nnz,
                       const int64_t* colptr, const int64_t* rowval, const double* nzval,
                       const double* mu, int dtype, sv_centered** out);
/* Per-gene mean and unbiased variance over all genes of a data matrix, with the
 * implicit zeros (the statistics of src/scaling.jl:132-142 on every column); the
 * input of highly-variable-feature selection (src/variablefeatures.jl). */
int sv_gene_moments(sv_context* ctx, const sv_data* data, double* mean, double* var);
int sv_centered_info(const sv_centered* s, int64_t* n_cells, int64_t* n_features, int64_t* nnz);
/* mu (= mean/std, the reference's S.mu), mean and std per feature (FP64). */
int sv_centered_stats(sv_context* ctx, const sv_centered* s, double* mu, double* mean, double* std);
/* y = alpha * op(Xs) * x + beta * y  (src/scaling.jl:245-272 mul! family).
 * trans 'N': x is n_features x ncols, y is n_cells x ncols;
 * trans 'T': x is n_cells x ncols, y is n_features x ncols.  Host FP64,
 * column-major with leading dimensions ldx / ldy. */
int sv_centered_mul(sv_context* ctx, const sv_centered* s, char trans, int64_t ncols,
                    double alpha, const double* x, int64_t ldx, double beta,
                    double* y, int64_t ldy);
int sv_centered_free(sv_centered* s);
/* The Gram product of two CenteredMatrix over the same cells (the Adjoint x
 * CenteredMatrix mul! of src/scaling.jl:274-296, used by the tssvd route of
 * src/embedding.jl:30-44): C = alpha Xl~' Xr~ + beta C, C host column-major
 * FP64 (nf_l x nf_r, in/out), computed as Al' Ar - mu_l q_r' - (q_l - n mu_l)
 * mu_r' with q = the column sums of the stored values. */
int sv_centered_gram(sv_context* ctx, const sv_centered* left, const sv_centered* right, double alpha,
                     double beta, double* C);

/* ---- sparse products of src/mul.jl ------------------------------------------
 * Host CSC arrays (Julia layout; index_base 0 or 1), FP64 values, computed on
 * the device in the reference's order of accumulation (bit-identical results).
 * y = alpha A x + beta y, A m x n, x a sparse vector of nnzx (index, value)
 * pairs (mul.jl:50-77); y host FP64 (m, in/out). */
int sv_sparse_mul_spvec(sv_context* ctx, int64_t m, int64_t n, const int64_t* colptr,
                        const int64_t* rowval, const double* nzval, int64_t nnzx, const int64_t* xidx,
                        const double* xval, int index_base, double alpha, double beta, double* y);
/* C = alpha op(A) B + beta C (mul.jl:79-114), C host column-major FP64 m x n
 * (in/out), B k x n CSC; A m x k CSC, or with transa != 0 A is k x m and
 * op(A) = A' (the reference multiplies by copy(A'), formed here on the device). */
int sv_sparse_mul_sparse(sv_context* ctx, int64_t m, int64_t k, int64_t n, const int64_t* acolptr,
                         const int64_t* arowval, const double* anzval, int transa,
                         const int64_t* bcolptr, const int64_t* browval, const double* bnzval,
                         int index_base, double alpha, double beta, double* C);

/* ---- irlba (src/irlba.jl:47-99) ---------------------------------------------
 * Truncated SVD of the implicit matrix, all Lanczos vectors in HBM.
 * nu singular triplets; work = Lanczos basis size (the reference passes nu + 7
 * clamped to [nu + 1, min(m, n)], irlba.jl:50-58; pass 0 for that default);
 * maxit restarts; tol: converged when every ||Xs^T u_i - s_i v_i|| is below
 * tol * s_max; init: start vector on the feature side (length n_features,
 * irlba.jl:62-64); seed: for the random vectors drawn on an invariant subspace.
 * Outputs (host, column-major FP64, any may be NULL): s (nu), U (n_cells x nu),
 * V (n_features x nu).  iters / nmatvec report the restarts and products used.
 * Returns SV_ERR_NOCONV if maxit is reached (the reference raises
 * "convergence failed", irlba.jl:73); outputs then hold the last iterate. */
int sv_irlba(sv_context* ctx, const sv_centered* s, int64_t nu, int64_t work, int64_t maxit,
             double tol, const double* init, uint64_t seed, double* s_out, double* U,
             double* V, int64_t* iters, int64_t* nmatvec);

/* pca / embedding with algorithm = :irlba (src/embedding.jl:46-94,202-212):
 * runs sv_irlba and keeps coordinates Z = U diag(s) (n_cells x npcs) on the
 * device for kNN.  Host outputs (NULL to skip): Z (n_cells x npcs, column-major
 * FP64), stdev = s / sqrt(max(1, n_cells - 1)) (npcs), loadings = V
 * (n_features x npcs). */
int sv_pca(sv_context* ctx, const sv_centered* s, int64_t npcs, int64_t maxit, double tol,
           const double* init, uint64_t seed, sv_embed** out, double* Z, double* stdev,
           double* loadings, int64_t* iters, int64_t* nmatvec);
int sv_embed_info(const sv_embed* e, int64_t* n_cells, int64_t* npcs);
int sv_embed_free(sv_embed* e);

/* Drop-in for the native `irlba` symbol that src/irlba.jl:66-71 calls:
 *   int irlba(BlasInt m, BlasInt n, BlasInt nu, BlasInt work, BlasInt maxit,
 *             BlasInt restart, double tol, double* init, double* s, double* U,
 *             double* V, randv, matmul, void* data)
 * with BlasInt = int64_t (ILP64, deps/build.jl:17-57).  The matrix is only known
 * through the caller's callback matmul(y, trans, x, temp, data) ('T' = 84:
 * y = A' x, x in R^m, y in R^n; otherwise y = A x), invoked on the calling
 * thread with host FP64 vectors; reorthogonalisation, the restart SVD and all
 * basis updates run on the device (context 0 of device 0, created on first use).
 * randv(y, n, data) fills y with standard normals for restarts on an invariant
 * subspace.  restart > 0 (warm restart) is accepted and treated as a cold start,
 * which the reference's own test marks as broken (test/test_irlba.jl:60-62).
 * Returns 0 on convergence, 1 when maxit is reached, < 0 on errors. */
typedef void (*sv_randv_fn)(double* y, int n, void* data);
typedef void (*sv_matmul_fn)(double* y, char trans, double* x, double* temp, void* data);
int irlba(int64_t m, int64_t n, int64_t nu, int64_t work, int64_t maxit, int64_t restart,
          double tol, double* init, double* s, double* U, double* V,
          sv_randv_fn randv, sv_matmul_fn matmul, void* data);

/* ---- nearest neighbours (src/neighbours.jl:19-86) ---------------------------
 * Exact k-nearest neighbours of the n points (rows) of X (n x d, column-major,
 * leading dimension ldX >= n; dtype SV_F32 or SV_F64; host memory).
 * include_self != 0 puts each point first in its own list; otherwise it is
 * excluded.  precision SV_KNN_FP32 or SV_KNN_BF16 (candidates from BF16
 * tensor-core distances, then an FP32 exact re-rank of the best 2k).
 * Outputs (host, NULL to skip): nn_index (n x k column-major, 1-based Int32,
 * ascending distance, ties by index) and distances (n x k column-major, in
 * dtype: Euclidean distance, or 1 - cosine similarity for SV_COSINE). */
int sv_knn_host(sv_context* ctx, const void* X, int dtype, int64_t n, int64_t d, int64_t ldX,
                int64_t k, int metric, int include_self, int precision,
                int32_t* nn_index, void* distances, sv_knn** out);
/* Same, on the device-resident PCA coordinates (dims 1..ndims of the embedding). */
int sv_knn_embed(sv_context* ctx, const sv_embed* e, int64_t ndims, int64_t k, int metric,
                 int include_self, int precision, int32_t* nn_index, double* distances,
                 sv_knn** out);
int sv_knn_info(const sv_knn* k, int64_t* n, int64_t* kk);
int sv_knn_free(sv_knn* k);

/* ---- batched samples ------------------------------------------------------------
 * No single counterpart in the reference: several samples, stacked by cells in
 * one count matrix over the same genes (sample s = cells cell_offsets[s] ..
 * cell_offsets[s+1]-1), each taken through scale_features, pca and ann as the
 * reference would take it on its own (src/scaling.jl:335-357,
 * src/embedding.jl:46-76, src/neighbours.jl:19-74), with one launch per stage
 * covering every sample.  normalize_cells works per cell, so sv_normalize_cells
 * of the stacked counts is already per sample.  Values FP32 or BF16.
 * sv_batch_create: per-(sample, feature) moments and the implicit scaled
 * matrices (features as in sv_scale_features).  sv_batch_stats: sample-major
 * (nseg x nf) mu, mean, std.  sv_batch_pca: the irlba of every sample in the same
 * launches (each converges and is finished on its own); Z is n_cells x npcs
 * column-major (samples' rows stacked), stdev nseg x npcs, iters nseg; init (nf)
 * is every sample's start vector; SV_ERR_NOCONV when a sample did not converge.
 * sv_batch_knn: each cell's k neighbours among the cells of its own sample;
 * indices are 1-based stacked rows. */
int sv_batch_create(sv_context* ctx, const sv_data* data, const int64_t* cell_offsets, int64_t nseg,
                    const int64_t* features, int64_t nfeatures, double scale_max, sv_batch** out);
int sv_batch_info(const sv_batch* b, int64_t* nseg, int64_t* n_cells, int64_t* nf);
int sv_batch_stats(sv_context* ctx, const sv_batch* b, double* mu, double* mean, double* sd);
int sv_batch_pca(sv_context* ctx, const sv_batch* b, int64_t npcs, int64_t maxit, double tol,
                 const double* init, uint64_t seed, sv_embed** out, double* Z, double* stdev,
                 int64_t* iters, int64_t* nmatvec);
int sv_batch_knn(sv_context* ctx, const sv_batch* b, const sv_embed* e, int64_t ndims, int64_t k,
                 int metric, int include_self, int precision, int32_t* nn_index, double* distances,
                 sv_knn** out);
/* The cells per block of the batched X v product, chosen on the first batch of
 * each shape by timing the candidates 128, 256, 512, 1024. */
int sv_batch_tuning(const sv_batch* b, int64_t* cells_per_block);
int sv_batch_free(sv_batch* b);

/* Drop-ins for the native libcell symbols of src/neighbours.jl:37-72 (the Julia
 * side declares every X / distances pointer as Ptr{Float64}; the element type is
 * the one in the name).  The search is exact, so ntables and seed are accepted
 * and ignored.  void return as in the reference: failures leave nn_index
 * filled with 0 and are reported through sv_last_error(). */
void FindNeighboursEuclidean32(const float* X, int n, int d, int ldX, int k, int ntables,
                               int include_self, int seed, int32_t* nn_index, float* distances);
void FindNeighboursEuclidean64(const double* X, int n, int d, int ldX, int k, int ntables,
                               int include_self, int seed, int32_t* nn_index, double* distances);
void FindNeighboursCosine32(const float* X, int n, int d, int ldX, int k, int ntables,
                            int include_self, int seed, int32_t* nn_index, float* distances);
void FindNeighboursCosine64(const double* X, int n, int d, int ldX, int k, int ntables,
                            int include_self, int seed, int32_t* nn_index, double* distances);

/* ---- shared nearest neighbours (src/neighbours.jl:76-108,127-155,272-278) ----
 * Builds the kNN graph of src/neighbours.jl:79 (column j holds the neighbours
 * of cell j), counts c_ij = |N(i) & N(j)| in integers, weights
 * w = c / (k + (k - c)) in dtype (SV_F32 or SV_F64) with k = k_param, or, when
 * k_param < 0, k = |N(j)| of the column (the diag variant, neighbours.jl:96-108),
 * and keeps w > prune (prune converted to dtype; droptol!, neighbours.jl:92).
 * The result is an n x n CSC with sorted rows, bit-identical to the reference's
 * given the same neighbour lists.
 * sv_snn_host takes nn_index as the caller holds it (n x k column-major, 1-based
 * Int32); sv_snn_knn takes a device-resident kNN result. */
int sv_snn_host(sv_context* ctx, const int32_t* nn_index, int64_t n, int64_t k,
                int64_t k_param, double prune, int dtype, sv_graph** out);
int sv_snn_knn(sv_context* ctx, const sv_knn* knn, int64_t k_param, double prune, int dtype,
               sv_graph** out);
int sv_graph_info(const sv_graph* g, int64_t* n, int64_t* nnz);
/* Copies the graph out as a Julia SparseMatrixCSC: colptr (n + 1) and rowval
 * (nnz) as 1-based Int64, nzval (nnz) in the graph's dtype.  Any may be NULL. */
int sv_graph_download(sv_context* ctx, const sv_graph* g, int64_t* colptr, int64_t* rowval,
                      void* nzval);
/* Hand-off to Louvain: the arrays of Network(snn) (src/modularity.jl:163-194)
 * written in Julia's isbits layouts, so that the caller's Vector{Node{T}} and
 * Vector{Edge{T}} receive them without a host rebuild:
 *   Edge{T}: { int64 node (1-based); T weight; }                 16 bytes
 *   Node{T}: { T weight; int64 first; int64 last; }              24 bytes
 *            (weight = sum of the column's non-self weights, in column order;
 *             edges first:last, 1-based, empty when first > last)
 * Self links are excluded; *totw (T) is the sum of all edge weights taken edge
 * by edge in order, as the reference accumulates it (tot_self is zero).  Call
 * with nodes = edges = totw = NULL to obtain *nedges first. */
int sv_graph_network(sv_context* ctx, const sv_graph* g, int64_t* nedges, void* nodes,
                     void* edges, void* totw);
int sv_graph_free(sv_graph* g);

#ifdef __cplusplus
}
#endif
#endif /* SEVERO_GPU_H */
