/*
 * cacg_io.c -- the reference's input files on the host: Matrix Market
 * matrices, comma-separated right-hand sides, and the 1-D row-block split
 * of both that the reference's ranks use.
 *
 *   cacg_read_mtx       src/readMTX.c:8-135 (readMtx_info_and_coo) followed by
 *                       src/matrixType.c:4-52 (Converter_Coo2Csr)
 *   cacg_csr_row_block  src/SparseMatrixDistribution.c:7-205
 *   cacg_read_csv       src/common.c:16-48 (parseCSV)
 *   cacg_dense_row_block src/GetRHS.c:124-208 (GenVector_ReadCSV, the split)
 *
 * Same inputs, same outputs; where the reference calls exit() or assert()
 * these return CACG_ERR_ARG (or CACG_ERR_OOM) and leave the outputs zeroed.
 * The banner and size-line rules are those of the Matrix Market exchange
 * format (NIST), which the reference reads through its vendored mmio.c.
 */
#include <ctype.h>
#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cacg.h"

/* ------------------------------------------------------------ Matrix Market */

enum { MM_REAL, MM_INTEGER, MM_PATTERN, MM_COMPLEX };
enum { MM_GENERAL, MM_SYMMETRIC, MM_SKEW, MM_HERMITIAN };

static void lower(char *s) {
    for (; *s; ++s) *s = (char)tolower((unsigned char)*s);
}

/* "%%MatrixMarket matrix <format> <field> <symmetry>" (tokens after the first
 * are case-insensitive); returns 0 and the codes, or -1. */
static int parse_banner(const char *line, int *coordinate, int *field, int *sym) {
    char b[128], obj[128], fmt[128], fld[128], sy[128];
    if (sscanf(line, "%127s %127s %127s %127s %127s", b, obj, fmt, fld, sy) != 5) return -1;
    if (strncmp(b, "%%MatrixMarket", 14) != 0) return -1;
    lower(obj);
    lower(fmt);
    lower(fld);
    lower(sy);
    if (strcmp(obj, "matrix") != 0) return -1;
    if (strcmp(fmt, "coordinate") == 0)
        *coordinate = 1;
    else if (strcmp(fmt, "array") == 0)
        *coordinate = 0;
    else
        return -1;
    if (strcmp(fld, "real") == 0)
        *field = MM_REAL;
    else if (strcmp(fld, "integer") == 0)
        *field = MM_INTEGER;
    else if (strcmp(fld, "pattern") == 0)
        *field = MM_PATTERN;
    else if (strcmp(fld, "complex") == 0)
        *field = MM_COMPLEX;
    else
        return -1;
    if (strcmp(sy, "general") == 0)
        *sym = MM_GENERAL;
    else if (strcmp(sy, "symmetric") == 0)
        *sym = MM_SYMMETRIC;
    else if (strcmp(sy, "skew-symmetric") == 0)
        *sym = MM_SKEW;
    else if (strcmp(sy, "hermitian") == 0)
        *sym = MM_HERMITIAN;
    else
        return -1;
    /* combinations the format rules out */
    if (!*coordinate && *field == MM_PATTERN) return -1;
    if ((*field == MM_REAL || *field == MM_INTEGER) && *sym == MM_HERMITIAN) return -1;
    if (*field == MM_PATTERN && (*sym == MM_HERMITIAN || *sym == MM_SKEW)) return -1;
    return 0;
}

/* next whitespace-separated token as long / double; 0 on success */
static int next_long(FILE *f, long *v) { return fscanf(f, " %ld", v) == 1 ? 0 : -1; }
static int next_double(FILE *f, double *v) { return fscanf(f, " %lf", v) == 1 ? 0 : -1; }

void cacg_csr_free(csrType_local *m) {
    if (!m) return;
    free(m->row_start);
    free(m->col_idx);
    free(m->csrdata);
    memset(m, 0, sizeof *m);
}

/* COO (0-based) -> CSR by a counting sort on the row index that keeps the
 * entries of a row in COO order (src/matrixType.c:4-52). */
static int coo_to_csr(long nrows, long ncols, long nnz, const long *I, const long *J,
                      const double *V, csrType_local *out) {
    long *rs = (long *)calloc((size_t)nrows + 1, sizeof(long));
    long *ci = (long *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(long));
    double *cv = (double *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(double));
    if (!rs || !ci || !cv) {
        free(rs);
        free(ci);
        free(cv);
        return CACG_ERR_OOM;
    }
    for (long e = 0; e < nnz; ++e) rs[I[e] + 1]++;
    for (long r = 0; r < nrows; ++r) rs[r + 1] += rs[r];
    long *fill = (long *)malloc((size_t)(nrows > 0 ? nrows : 1) * sizeof(long));
    if (!fill) {
        free(rs);
        free(ci);
        free(cv);
        return CACG_ERR_OOM;
    }
    memcpy(fill, rs, (size_t)nrows * sizeof(long));
    for (long e = 0; e < nnz; ++e) {
        const long d = fill[I[e]]++;
        ci[d] = J[e];
        cv[d] = V[e];
    }
    free(fill);
    out->num_rows = nrows;
    out->num_cols = ncols;
    out->nnz = nnz;
    out->start = 0;
    out->row_start = rs;
    out->col_idx = ci;
    out->csrdata = cv;
    return CACG_OK;
}

int cacg_read_mtx(const char *path, csrType_local *out) {
    if (!out) return CACG_ERR_ARG;
    memset(out, 0, sizeof *out);
    if (!path) return CACG_ERR_ARG;
    FILE *f = fopen(path, "r");
    if (!f) return CACG_ERR_ARG;
    char line[1025];
    int coordinate = 0, field = 0, sym = 0;
    if (!fgets(line, sizeof line, f) || parse_banner(line, &coordinate, &field, &sym) != 0) {
        fclose(f);
        return CACG_ERR_ARG; /* not a Matrix Market banner */
    }
    if (!coordinate || field == MM_COMPLEX) {
        fclose(f);
        return CACG_ERR_UNSUPPORTED; /* src/readMTX.c:32-38: coordinate real/integer/pattern only */
    }
    /* size line: skip comment lines and blank lines, then "M N nnz" */
    long M = -1, N = -1, nz = -1;
    for (;;) {
        if (!fgets(line, sizeof line, f)) {
            fclose(f);
            return CACG_ERR_ARG;
        }
        if (line[0] == '%') continue;
        const char *p = line;
        while (*p && isspace((unsigned char)*p)) ++p;
        if (!*p) continue;
        if (sscanf(p, "%ld %ld %ld", &M, &N, &nz) != 3 || M < 0 || N < 0 || nz < 0) {
            fclose(f);
            return CACG_ERR_ARG;
        }
        break;
    }
    long *I = (long *)malloc((size_t)(nz > 0 ? nz : 1) * sizeof(long));
    long *J = (long *)malloc((size_t)(nz > 0 ? nz : 1) * sizeof(long));
    double *V = (double *)malloc((size_t)(nz > 0 ? nz : 1) * sizeof(double));
    int rc = (I && J && V) ? CACG_OK : CACG_ERR_OOM;
    long offd = 0;
    for (long e = 0; rc == CACG_OK && e < nz; ++e) {
        long i, j;
        double v = 1.0; /* pattern entries read as 1.0 */
        if (next_long(f, &i) || next_long(f, &j) ||
            (field != MM_PATTERN && next_double(f, &v))) {
            rc = CACG_ERR_ARG; /* short or malformed entry */
            break;
        }
        if (i < 1 || i > M || j < 1 || j > N) {
            rc = CACG_ERR_ARG; /* the reference would index out of bounds */
            break;
        }
        I[e] = i - 1;
        J[e] = j - 1;
        V[e] = v;
        if (i != j) ++offd;
    }
    fclose(f);
    if (rc == CACG_OK && sym == MM_SYMMETRIC) {
        /* each off-diagonal entry is followed by its mirror image, in file
         * order (src/readMTX.c:96-133) */
        const long tot = nz + offd;
        long *I2 = (long *)malloc((size_t)(tot > 0 ? tot : 1) * sizeof(long));
        long *J2 = (long *)malloc((size_t)(tot > 0 ? tot : 1) * sizeof(long));
        double *V2 = (double *)malloc((size_t)(tot > 0 ? tot : 1) * sizeof(double));
        if (!I2 || !J2 || !V2) {
            free(I2);
            free(J2);
            free(V2);
            rc = CACG_ERR_OOM;
        } else {
            long q = 0;
            for (long e = 0; e < nz; ++e) {
                I2[q] = I[e];
                J2[q] = J[e];
                V2[q++] = V[e];
                if (I[e] != J[e]) {
                    I2[q] = J[e];
                    J2[q] = I[e];
                    V2[q++] = V[e];
                }
            }
            free(I);
            free(J);
            free(V);
            I = I2;
            J = J2;
            V = V2;
            nz = tot;
        }
    }
    if (rc == CACG_OK) rc = coo_to_csr(M, N, nz, I, J, V, out);
    free(I);
    free(J);
    free(V);
    return rc;
}

/* rows of rank `myid` of `numprocs`: n / numprocs each, the last rank also
 * the remainder (src/SparseMatrixDistribution.c:72-78, src/GetRHS.c:147-150) */
static void row_block(long n, int myid, int numprocs, long *first, long *count) {
    const long per = n / numprocs;
    *first = (long)myid * per;
    *count = myid == numprocs - 1 ? n - per * (numprocs - 1) : per;
}

int cacg_csr_row_block(const csrType_local *A, int myid, int numprocs, csrType_local *local) {
    if (!local) return CACG_ERR_ARG;
    memset(local, 0, sizeof *local);
    if (!A || !A->row_start || numprocs < 1 || myid < 0 || myid >= numprocs || A->num_rows < 0)
        return CACG_ERR_ARG;
    long r0, nr;
    row_block(A->num_rows, myid, numprocs, &r0, &nr);
    const long e0 = A->row_start[r0], e1 = A->row_start[r0 + nr];
    long *rs = (long *)malloc((size_t)(nr + 1) * sizeof(long));
    long *ci = (long *)malloc((size_t)(e1 - e0 > 0 ? e1 - e0 : 1) * sizeof(long));
    double *cv = (double *)malloc((size_t)(e1 - e0 > 0 ? e1 - e0 : 1) * sizeof(double));
    if (!rs || !ci || !cv) {
        free(rs);
        free(ci);
        free(cv);
        return CACG_ERR_OOM;
    }
    for (long r = 0; r <= nr; ++r) rs[r] = A->row_start[r0 + r] - e0;
    if (e1 > e0) {
        memcpy(ci, A->col_idx + e0, (size_t)(e1 - e0) * sizeof(long));
        memcpy(cv, A->csrdata + e0, (size_t)(e1 - e0) * sizeof(double));
    }
    local->num_rows = nr;
    local->num_cols = A->num_cols;
    local->nnz = e1 - e0;
    local->start = r0;
    local->row_start = rs;
    local->col_idx = ci;
    local->csrdata = cv;
    return CACG_OK;
}

/* ------------------------------------------------------------------- CSV */

int cacg_read_csv(const char *path, int64_t rows, int64_t cols, double *out,
                  int64_t *rows_read) {
    if (rows_read) *rows_read = 0;
    if (!path || !out || rows < 0 || cols < 1) return CACG_ERR_ARG;
    memset(out, 0, (size_t)rows * (size_t)cols * sizeof(double));
    FILE *f = fopen(path, "r");
    if (!f) return CACG_ERR_ARG;
    size_t cap = 4096;
    char *buf = (char *)malloc(cap);
    if (!buf) {
        fclose(f);
        return CACG_ERR_OOM;
    }
    int rc = CACG_OK;
    int64_t r = 0;
    while (r < rows) {
        /* one whole line, however long */
        size_t len = 0;
        int got = 0;
        for (;;) {
            if (!fgets(buf + len, (int)(cap - len), f)) break;
            got = 1;
            len += strlen(buf + len);
            if (len > 0 && buf[len - 1] == '\n') break;
            if (len + 1 < cap) continue; /* end of file without a newline */
            char *nb = (char *)realloc(buf, cap * 2);
            if (!nb) {
                rc = CACG_ERR_OOM;
                break;
            }
            buf = nb;
            cap *= 2;
        }
        if (rc != CACG_OK || !got) break;
        /* fields: first split on ',', then on ',' and '\n'; an empty field
         * ends the line (src/common.c:29-37) */
        int64_t c = 0;
        char *save = NULL;
        char *tok = strtok_r(buf, ",", &save);
        for (; tok && *tok; tok = strtok_r(NULL, ",\n", &save)) {
            if (c < cols) out[r * cols + c] = atof(tok);
            ++c;
        }
        if (c != cols) {
            rc = CACG_ERR_ARG; /* the reference asserts */
            break;
        }
        ++r;
    }
    free(buf);
    fclose(f);
    if (rc != CACG_OK) {
        memset(out, 0, (size_t)rows * (size_t)cols * sizeof(double));
        return rc;
    }
    if (rows_read) *rows_read = r;
    return CACG_OK;
}

void cacg_dense_free(denseType *d) {
    if (!d) return;
    free(d->data);
    memset(d, 0, sizeof *d);
}

int cacg_dense_row_block(const double *global, int64_t rows, int64_t cols, int myid,
                         int numprocs, denseType *local) {
    if (!local) return CACG_ERR_ARG;
    memset(local, 0, sizeof *local);
    if (!global || rows < 0 || cols < 1 || numprocs < 1 || myid < 0 || myid >= numprocs)
        return CACG_ERR_ARG;
    long r0, nr;
    row_block((long)rows, myid, numprocs, &r0, &nr);
    double *d = (double *)malloc((size_t)(nr * cols > 0 ? nr * cols : 1) * sizeof(double));
    if (!d) return CACG_ERR_OOM;
    if (nr > 0) memcpy(d, global + (size_t)r0 * cols, (size_t)(nr * cols) * sizeof(double));
    local->local_num_row = nr;
    local->local_num_col = (long)cols;
    local->global_num_row = (long)rows;
    local->global_num_col = (long)cols;
    /* src/GetRHS.c:202: element offset of the block, in rows x cols units */
    local->start_idx = (long)myid * (long)cols * ((long)rows / numprocs);
    local->data = d;
    return CACG_OK;
}
