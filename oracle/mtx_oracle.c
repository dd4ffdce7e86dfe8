/* CPU oracle for the MatrixMarket reader -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/ and the CPU-baseline leg of bench.py load this file's library;
 * the product path (libseverogpu.so) never calls into it.
 *
 * A single-threaded C restatement of how Severo.jl reads a MatrixMarket count
 * file, line by line as the reference does:
 *   parseMM_header            src/input.jl:27-56   (banner, 5 fields, checks in order)
 *   skipMM_comments           src/input.jl:58-64   (empty lines and '%' lines)
 *   readMM                    src/input.jl:78-115  (size line, one entry per line,
 *                                                    exactly three fields)
 *   sparse(r, c, v, m, n)     src/input.jl:113     (duplicates summed, zeros kept:
 *                                                    Julia's SparseArrays stdlib)
 *   copy(X')                  src/input.jl:207     (features x barcodes -> cells x genes)
 * giving the cells x genes CSC with rows sorted within each column.  The
 * construction follows the stdlib's counting-sort shape: entries bucketed by
 * cell in file order, duplicates merged per cell with a last-touch marker over
 * the genes, then one transpose that leaves rows sorted.
 *
 * Counts are whole numbers in [0, 2^31) (the Int32 range convert_counts,
 * src/input.jl:776-780, converts real files into); a real-field token is read
 * exactly as mantissa x 10^exponent, so a decimal that is not a whole number is
 * rejected even where Float64 rounding would make it one.
 *
 * Parity is unpinned against the reference itself: its tests hold no
 * MatrixMarket fixture and Julia cannot run here.  It is pinned to the format
 * (hand-written files with known matrices in tests/) and to scipy's reader on
 * well-formed files.
 */
#include <ctype.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int64_t n_cells, n_genes, nnz;
  int64_t* colptr;  /* n_genes + 1 */
  int32_t* rowidx;  /* nnz, 0-based cells */
  int32_t* val;     /* nnz */
  char err[256];
} mtx_oracle_result;

typedef struct {
  const char* p;
  int64_t n, pos;
} Text;

/* next line without "\n" / "\r\n"; returns 0 at the end of the input */
static int next_line(Text* t, const char** s, int64_t* len) {
  if (t->pos >= t->n) return 0;
  const char* b = t->p + t->pos;
  const char* nl = memchr(b, '\n', (size_t)(t->n - t->pos));
  int64_t l = nl ? nl - b : t->n - t->pos;
  t->pos += l + (nl ? 1 : 0);
  if (l > 0 && b[l - 1] == '\r') --l;
  *s = b;
  *len = l;
  return 1;
}

static int is_ws(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f' || c == '\n'; }

/* splits [s, s+len) on whitespace into at most maxtok tokens; returns the count */
static int split(const char* s, int64_t len, const char** tok, int64_t* tl, int maxtok) {
  int n = 0;
  int64_t i = 0;
  while (i < len) {
    while (i < len && is_ws(s[i])) ++i;
    int64_t j = i;
    while (j < len && !is_ws(s[j])) ++j;
    if (j > i) {
      if (n < maxtok) {
        tok[n] = s + i;
        tl[n] = j - i;
      }
      ++n;
    }
    i = j;
  }
  return n;
}

static int tok_eq_ci(const char* t, int64_t l, const char* w) {
  int64_t k = (int64_t)strlen(w);
  if (k != l) return 0;
  for (int64_t i = 0; i < l; ++i)
    if (tolower((unsigned char)t[i]) != w[i]) return 0;
  return 1;
}

static int parse_i64(const char* t, int64_t l, long long* out) {
  int64_t i = 0;
  int neg = 0;
  if (l > 0 && (t[0] == '+' || t[0] == '-')) {
    neg = t[0] == '-';
    i = 1;
  }
  if (i == l) return 0;
  unsigned long long v = 0;
  for (; i < l; ++i) {
    unsigned d = (unsigned char)t[i] - '0';
    if (d > 9 || v > (9223372036854775807ull - d) / 10) return 0;
    v = v * 10 + d;
  }
  *out = neg ? -(long long)v : (long long)v;
  return 1;
}

/* 0 ok, 1 malformed, 2 not a whole number in [0, 2^31) */
static int parse_real_count(const char* t, int64_t l, long long* out) {
  int64_t i = 0;
  int neg = 0;
  if (l > 0 && (t[0] == '+' || t[0] == '-')) {
    neg = t[0] == '-';
    i = 1;
  }
  /* collect the significant digits as a decimal string and the exponent */
  char dig[4096];
  int nd = 0, any = 0, lost = 0; /* lost: a non-zero digit beyond the buffer */
  long long e10 = 0;
  for (; i < l && isdigit((unsigned char)t[i]); ++i) {
    any = 1;
    if (nd == 0 && t[i] == '0') continue;
    if (nd < (int)sizeof(dig)) {
      dig[nd++] = t[i];
    } else {
      ++e10;
      lost |= t[i] != '0';
    }
  }
  if (i < l && t[i] == '.') {
    ++i;
    for (; i < l && isdigit((unsigned char)t[i]); ++i) {
      any = 1;
      if (nd == 0 && t[i] == '0') {
        --e10;
      } else if (nd < (int)sizeof(dig)) {
        dig[nd++] = t[i];
        --e10;
      } else {
        lost |= t[i] != '0';
      }
    }
  }
  if (!any) return 1;
  if (i < l && (t[i] == 'e' || t[i] == 'E')) {
    ++i;
    int eneg = 0;
    if (i < l && (t[i] == '+' || t[i] == '-')) {
      eneg = t[i] == '-';
      ++i;
    }
    if (i == l) return 1;
    long long x = 0;
    for (; i < l; ++i) {
      if (!isdigit((unsigned char)t[i])) return 1;
      if (x < 100000000) x = x * 10 + (t[i] - '0');
    }
    e10 += eneg ? -x : x;
  }
  if (i != l) return 1;
  /* value = digits x 10^e10; trailing zeros move into the exponent */
  while (nd > 0 && dig[nd - 1] == '0') {
    --nd;
    ++e10;
  }
  if (nd == 0) {
    *out = 0;
    return lost ? 2 : 0;
  }
  if (lost || neg || e10 < 0) return 2;
  if (nd + e10 > 10) return 2;
  long long v = 0;
  for (int k = 0; k < nd; ++k) v = v * 10 + (dig[k] - '0');
  for (long long k = 0; k < e10; ++k) v *= 10;
  if (v >= 2147483648ll) return 2;
  *out = v;
  return 0;
}

static int fail(mtx_oracle_result* r, int code, const char* msg) {
  snprintf(r->err, sizeof(r->err), "%s", msg);
  return code;
}

void mtx_oracle_free(mtx_oracle_result* r) {
  free(r->colptr);
  free(r->rowidx);
  free(r->val);
  r->colptr = NULL;
  r->rowidx = NULL;
  r->val = NULL;
}

/* 0 on success; 1 header, 2 entry line, 3 index range, 4 count value */
int mtx_oracle_parse(const char* text, int64_t len, int rows_are_features, mtx_oracle_result* r) {
  memset(r, 0, sizeof(*r));
  Text t = {text, len, 0};
  const char* s;
  int64_t l;
  const char* tok[6];
  int64_t tl[6];
  if (!next_line(&t, &s, &l)) l = 0, s = text;
  if (split(s, l, tok, tl, 6) != 5) return fail(r, 1, "Malformed MatrixMarket header");
  if (!(tl[0] == 14 && memcmp(tok[0], "%%MatrixMarket", 14) == 0))
    return fail(r, 1, "Not a valid MatrixMarket header");
  if (!tok_eq_ci(tok[1], tl[1], "matrix")) return fail(r, 1, "Unknown MatrixMarket data type");
  int real = 0;
  if (tok_eq_ci(tok[3], tl[3], "real")) real = 1;
  else if (!tok_eq_ci(tok[3], tl[3], "integer")) return fail(r, 1, "Unsupported field");
  if (!tok_eq_ci(tok[4], tl[4], "general")) return fail(r, 1, "Unknown matrix symmetry");
  if (!tok_eq_ci(tok[2], tl[2], "coordinate")) return fail(r, 1, "Unsupported matrix format");
  for (;;) {
    if (!next_line(&t, &s, &l)) return fail(r, 1, "Could not read in matrix dimensions");
    if (l > 0 && s[0] != '%') break;
  }
  long long rows, cols, entries;
  if (split(s, l, tok, tl, 6) != 3 || !parse_i64(tok[0], tl[0], &rows) ||
      !parse_i64(tok[1], tl[1], &cols) || !parse_i64(tok[2], tl[2], &entries))
    return fail(r, 1, "Could not read in matrix dimensions");
  if (rows < 1 || cols < 1 || entries < 0) return fail(r, 1, "bad matrix dimensions");
  const int64_t nc = rows_are_features ? cols : rows, ng = rows_are_features ? rows : cols;
  int32_t* ec = malloc(sizeof(int32_t) * (entries + 1));
  int32_t* eg = malloc(sizeof(int32_t) * (entries + 1));
  int64_t* ev = malloc(sizeof(int64_t) * (entries + 1));
  int rc = 0;
  for (long long e = 0; e < entries && rc == 0; ++e) {
    if (!next_line(&t, &s, &l)) l = 0, s = text;
    long long a, b, v = 0;
    if (split(s, l, tok, tl, 6) != 3 || !parse_i64(tok[0], tl[0], &a) || !parse_i64(tok[1], tl[1], &b)) {
      rc = fail(r, 2, "Could not read matrix entry");
      break;
    }
    int vs = 0;
    if (real) {
      vs = parse_real_count(tok[2], tl[2], &v);
      if (vs == 1) rc = fail(r, 2, "Could not read matrix entry");
    } else if (!parse_i64(tok[2], tl[2], &v)) {
      rc = fail(r, 2, "Could not read matrix entry");
    } else if (v < 0 || v >= 2147483648ll) {
      vs = 2;
    }
    if (rc) break;
    if (a < 1 || a > rows || b < 1 || b > cols) {
      rc = fail(r, 3, "index out of range");
      break;
    }
    if (vs) {
      rc = fail(r, 4, "count is not an integer in [0, 2^31)");
      break;
    }
    ec[e] = (int32_t)(rows_are_features ? b - 1 : a - 1);
    eg[e] = (int32_t)(rows_are_features ? a - 1 : b - 1);
    ev[e] = v;
  }
  if (rc) {
    free(ec), free(eg), free(ev);
    return rc;
  }
  /* bucket by cell in file order */
  int64_t* cp = calloc(nc + 1, sizeof(int64_t));
  for (long long e = 0; e < entries; ++e) cp[ec[e] + 1]++;
  for (int64_t c = 0; c < nc; ++c) cp[c + 1] += cp[c];
  int64_t* cur = malloc(sizeof(int64_t) * (nc + 1));
  memcpy(cur, cp, sizeof(int64_t) * (nc + 1));
  int32_t* bg = malloc(sizeof(int32_t) * (entries + 1));
  int64_t* bv = malloc(sizeof(int64_t) * (entries + 1));
  for (long long e = 0; e < entries; ++e) {
    int64_t p = cur[ec[e]]++;
    bg[p] = eg[e];
    bv[p] = ev[e];
  }
  free(ec), free(eg), free(ev), free(cur);
  /* merge duplicates per cell (last-touch marker over genes) */
  int64_t* mark = malloc(sizeof(int64_t) * (ng + 1));
  for (int64_t g = 0; g < ng; ++g) mark[g] = -1;
  int64_t* np = calloc(nc + 1, sizeof(int64_t));
  int64_t w = 0;
  for (int64_t c = 0; c < nc; ++c) {
    int64_t start = w;
    for (int64_t p = cp[c]; p < cp[c + 1]; ++p) {
      int32_t g = bg[p];
      if (mark[g] >= start) {
        bv[mark[g]] += bv[p];
      } else {
        mark[g] = w;
        bg[w] = g;
        bv[w] = bv[p];
        ++w;
      }
    }
    np[c + 1] = w;
  }
  free(mark), free(cp);
  for (int64_t p = 0; p < w; ++p)
    if (bv[p] >= 2147483648ll) {
      free(np), free(bg), free(bv);
      return fail(r, 4, "count is not an integer in [0, 2^31)");
    }
  /* transpose to genes: cells visited in order leave rows sorted */
  r->n_cells = nc;
  r->n_genes = ng;
  r->nnz = w;
  r->colptr = calloc(ng + 1, sizeof(int64_t));
  r->rowidx = malloc(sizeof(int32_t) * (w + 1));
  r->val = malloc(sizeof(int32_t) * (w + 1));
  for (int64_t p = 0; p < w; ++p) r->colptr[bg[p] + 1]++;
  for (int64_t g = 0; g < ng; ++g) r->colptr[g + 1] += r->colptr[g];
  int64_t* gc = malloc(sizeof(int64_t) * (ng + 1));
  memcpy(gc, r->colptr, sizeof(int64_t) * (ng + 1));
  for (int64_t c = 0; c < nc; ++c)
    for (int64_t p = np[c]; p < np[c + 1]; ++p) {
      int64_t q = gc[bg[p]]++;
      r->rowidx[q] = (int32_t)c;
      r->val[q] = (int32_t)bv[p];
    }
  free(gc), free(np), free(bg), free(bv);
  return 0;
}
