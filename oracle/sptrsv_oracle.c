/*
 * CPU oracle for the sync-free sparse triangular solve.
 *
 * TEST INFRASTRUCTURE ONLY: the CUDA library's results are compared with
 * it. Only the test suite, the smoke check and the benchmark's CPU-baseline
 * leg load it. The library (the CUDA path) never links or calls it, and there
 * is no CPU fallback.
 *
 * It restates, in plain C, the reference's serial algorithm for this path
 * (harunsasmaz/Benchmark-SpTRSV, directory SpTRSV_cuda/):
 *   - in-degree analyser ............ sptrsv_syncfree_serialref.h:6-23
 *   - serial sync-free executor ..... sptrsv_syncfree_serialref.h:25-108
 *   - CSR<->CSC transposition ....... tranpose.h:6-43 (+ utils.h:375-391 scan)
 *   - level-set construction ........ findlevel.h:6-69
 *   - level statistics .............. findlevel.h:71-147
 *   - manufactured right-hand side .. main.cu:347-358 (CSC SpMV b = L x)
 *   - L1-relative validation ........ sptrsv_syncfree_serialref.h:194-204
 *
 * Floating-point operations are written in the reference's order (product,
 * then sum, then one true division per unknown) and the file is compiled with
 * -ffp-contract=off, so results are bit-identical on x86-64 and AArch64 and
 * bit-identical to the reference compiled with the same flag.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>

#define ORACLE_FORWARD 0
#define ORACLE_BACKWARD 1

/* Row histogram of the CSC row indices; the count includes the diagonal.
 * sptrsv_syncfree_serialref.h:6-23 */
void oracle_analyser(const int *row_idx, int m, int nnz, int *in_degree)
{
    memset(in_degree, 0, sizeof(int) * (size_t)m);
    for (int e = 0; e < nnz; ++e)
        in_degree[row_idx[e]] += 1;
}

/* Serial sync-free executor. Unknowns are finished in dependency order
 * (0..n-1 forward, n-1..0 backward); each finished unknown pushes x*L(row,col)
 * into the partial sums of the rows below (above) it and bumps their arrival
 * counters. x and b are row-major n x rhs. Returns 0, or 1 when an arrival
 * counter disagrees with the analysed in-degree at the moment its unknown is
 * solved (the serial form of the reference's wait loop, which would spin
 * forever on such input). sptrsv_syncfree_serialref.h:25-108 */
#define ORACLE_EXECUTOR(NAME, T)                                                    \
int NAME(const int *col_ptr, const int *row_idx, const T *val,                      \
         const int *in_degree, int m, int n, int substitution, int rhs,             \
         const T *b, T *x)                                                          \
{                                                                                   \
    int *arrived = (int *)calloc((size_t)m, sizeof(int));                           \
    T *partial = (T *)calloc((size_t)m * (size_t)rhs, sizeof(T));                   \
    int bad = 0;                                                                    \
    for (int step = 0; step < n; ++step) {                                          \
        const int col = substitution == ORACLE_FORWARD ? step : n - 1 - step;       \
        const int first = col_ptr[col], last = col_ptr[col + 1] - 1;                \
        const int diag = substitution == ORACLE_FORWARD ? first : last;             \
        if (arrived[col] != in_degree[col] - 1) bad = 1;                            \
        for (int k = 0; k < rhs; ++k) {                                             \
            const size_t p = (size_t)col * rhs + k;                                 \
            x[p] = (b[p] - partial[p]) / val[diag];                                 \
        }                                                                           \
        const int lo = substitution == ORACLE_FORWARD ? first + 1 : first;          \
        const int hi = substitution == ORACLE_FORWARD ? last : last - 1;            \
        for (int e = lo; e <= hi; ++e) {                                            \
            const int row = row_idx[e];                                             \
            for (int k = 0; k < rhs; ++k) {                                         \
                const T prod = x[(size_t)col * rhs + k] * val[e];                   \
                partial[(size_t)row * rhs + k] = partial[(size_t)row * rhs + k] + prod; \
            }                                                                       \
            arrived[row] += 1;                                                      \
        }                                                                           \
    }                                                                               \
    free(arrived);                                                                  \
    free(partial);                                                                  \
    return bad;                                                                     \
}

ORACLE_EXECUTOR(oracle_executor_f64, double)
ORACLE_EXECUTOR(oracle_executor_f32, float)

/* Compressed-format transposition: histogram of the minor index, exclusive
 * scan, then an in-order scatter, so every output segment lists its entries
 * in increasing major index. tranpose.h:6-43 */
void oracle_transpose_f64(int m, int n, int nnz, const int *ptr, const int *idx,
                          const double *val, int *out_idx, int *out_ptr,
                          double *out_val)
{
    memset(out_ptr, 0, sizeof(int) * (size_t)(n + 1));
    for (int e = 0; e < nnz; ++e)
        out_ptr[idx[e]] += 1;
    int run = 0;
    for (int c = 0; c <= n; ++c) {   /* exclusive scan, utils.h:375-391 */
        const int cnt = out_ptr[c];
        out_ptr[c] = run;
        run += cnt;
    }
    int *fill = (int *)malloc(sizeof(int) * (size_t)(n + 1));
    memcpy(fill, out_ptr, sizeof(int) * (size_t)(n + 1));
    for (int r = 0; r < m; ++r) {
        for (int e = ptr[r]; e < ptr[r + 1]; ++e) {
            const int c = idx[e];
            out_idx[fill[c]] = r;
            if (val && out_val) out_val[fill[c]] = val[e];
            fill[c] += 1;
        }
    }
    free(fill);
}

/* Level sets by breadth-first peeling of the in-degree: level 0 holds the
 * unknowns whose only entry in their row is the diagonal; visiting a level
 * decrements the in-degree of every row its columns touch, and a row whose
 * count drops to one joins the next level. findlevel.h:6-69 */
int oracle_findlevel(const int *col_ptr, const int *row_idx, const int *row_ptr,
                     int m, int *nlevel, int *level_ptr, int *level_item)
{
    int *deg = (int *)malloc(sizeof(int) * (size_t)m);
    for (int i = 0; i < m; ++i) deg[i] = row_ptr[i + 1] - row_ptr[i];
    int tail = 0;
    level_ptr[0] = 0;
    for (int i = 0; i < m; ++i)
        if (deg[i] == 1) level_item[tail++] = i;
    level_ptr[1] = tail;
    int lv = 1;
    while (level_ptr[lv] != m) {
        const int before = tail;
        for (int q = level_ptr[lv - 1]; q < level_ptr[lv]; ++q) {
            const int node = level_item[q];
            for (int e = col_ptr[node]; e < col_ptr[node + 1]; ++e) {
                const int v = row_idx[e];
                deg[v] -= 1;
                if (deg[v] == 1) level_item[tail++] = v;
            }
        }
        ++lv;
        level_ptr[lv] = tail;
        if (tail == before) { free(deg); *nlevel = lv; return 1; } /* cyclic or malformed */
    }
    *nlevel = lv;
    free(deg);
    return 0;
}

/* Level count and per-level parallelism (min, m/nlevel, max) of a square CSC
 * triangle, as findlevel_csc reports them. findlevel.h:71-147 */
int oracle_findlevel_csc(const int *col_ptr, const int *row_idx, int m, int n, int nnz,
                         int *nlevel, int *pmin, int *pavg, int *pmax)
{
    if (m != n) return -1;
    int *row_ptr = (int *)malloc(sizeof(int) * (size_t)(m + 1));
    int *col_idx = (int *)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    oracle_transpose_f64(n, m, nnz, col_ptr, row_idx, NULL, col_idx, row_ptr, NULL);
    int *lptr = (int *)malloc(sizeof(int) * (size_t)(m + 1));
    int *litem = (int *)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    int nl = 0;
    const int rc = oracle_findlevel(col_ptr, row_idx, row_ptr, m, &nl, lptr, litem);
    int lo = lptr[1] - lptr[0], hi = lo;
    for (int l = 1; l < nl; ++l) {
        const int cnt = lptr[l + 1] - lptr[l];
        if (cnt > hi) hi = cnt;
        else if (cnt < lo) lo = cnt;   /* same else-if as the reference */
    }
    *pmin = lo;
    *pmax = hi;
    *pavg = nl > 0 ? m / nl : 0;
    *nlevel = nl;
    free(row_ptr); free(col_idx); free(lptr); free(litem);
    return rc;
}

/* b = L * x for a CSC matrix and row-major n x rhs vectors. main.cu:347-358 */
void oracle_csc_spmv_f64(const int *col_ptr, const int *row_idx, const double *val,
                         int m, int n, int rhs, const double *x, double *b)
{
    memset(b, 0, sizeof(double) * (size_t)m * (size_t)rhs);
    for (int c = 0; c < n; ++c)
        for (int e = col_ptr[c]; e < col_ptr[c + 1]; ++e) {
            const int r = row_idx[e];
            for (int k = 0; k < rhs; ++k) {
                const double prod = val[e] * x[(size_t)c * rhs + k];
                b[(size_t)r * rhs + k] = b[(size_t)r * rhs + k] + prod;
            }
        }
}

/* sum|x - x_ref| / sum|x_ref| (the plain sum when x_ref is all zero).
 * sptrsv_syncfree_serialref.h:194-204 */
double oracle_l1_rel_err_f64(const double *x, const double *x_ref, long long len)
{
    double ref = 0.0, res = 0.0;
    for (long long i = 0; i < len; ++i) {
        ref += fabs(x_ref[i]);
        res += fabs(x[i] - x_ref[i]);
    }
    return ref == 0.0 ? res : res / ref;
}
