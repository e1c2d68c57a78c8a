/* The reference's call site (SpTRSV_cuda/main.cu:376-378) compiled against
 * libsptrsv_gb300 instead of sptrsv_syncfree_cuda.h: plain C, host arrays, the
 * reference's argument list and return convention.
 *
 *   cc drop_in.c -I<repo>/include -L<repo>/benchmark-sptrsv_gb300/_build -lsptrsv_gb300 \
 *      -Wl,-rpath,<repo>/benchmark-sptrsv_gb300/_build -o drop_in && ./drop_in
 *
 * Builds the unit-lower triangle of a tridiagonal-plus-band matrix (n = 2000,
 * values 1..10 as the reference's -mtx path draws them), b = L * x_ref with
 * x_ref in 1..10 and two right-hand sides, solves forward and backward
 * (upper = the transpose), and exits 0 when both pass the reference's
 * L1-relative check. */
#include <stdio.h>
#include <stdlib.h>

#include "sptrsv_gb300.h"

static unsigned lcg(unsigned* s) {
  *s = *s * 1664525u + 1013904223u;
  return *s >> 8;
}

/* CSC of a unit-diagonal triangle: column j holds j itself and rows j+1, j+7
 * (lower) or j-1, j-7 (upper) where they exist; rows ascending per column. */
static int build(int n, int upper, int* col_ptr, int* row_idx, double* val, unsigned* seed) {
  int nnz = 0;
  for (int j = 0; j < n; ++j) {
    col_ptr[j] = nnz;
    int rows[3], k = 0;
    if (upper) {
      if (j - 7 >= 0) rows[k++] = j - 7;
      if (j - 1 >= 0) rows[k++] = j - 1;
      rows[k++] = j;
    } else {
      rows[k++] = j;
      if (j + 1 < n) rows[k++] = j + 1;
      if (j + 7 < n) rows[k++] = j + 7;
    }
    for (int t = 0; t < k; ++t) {
      row_idx[nnz] = rows[t];
      val[nnz] = rows[t] == j ? 1.0 : (double)(lcg(seed) % 10 + 1);
      ++nnz;
    }
  }
  col_ptr[n] = nnz;
  return nnz;
}

int main(void) {
  const int n = 2000, rhs = 2;
  int* col_ptr = malloc(sizeof(int) * (n + 1));
  int* row_idx = malloc(sizeof(int) * 3 * n);
  double* val = malloc(sizeof(double) * 3 * n);
  double* x_ref = malloc(sizeof(double) * n * rhs);
  double* b = malloc(sizeof(double) * n * rhs);
  double* x = malloc(sizeof(double) * n * rhs);
  unsigned seed = 12345u;
  int failures = 0;
  for (int substitution = SPTRSV_SUBSTITUTION_FORWARD; substitution <= SPTRSV_SUBSTITUTION_BACKWARD;
       ++substitution) {
    const int nnz = build(n, substitution == SPTRSV_SUBSTITUTION_BACKWARD, col_ptr, row_idx, val, &seed);
    for (int i = 0; i < n * rhs; ++i) {
      x_ref[i] = (double)(lcg(&seed) % 10 + 1);
      b[i] = 0.0;
      x[i] = 0.0;
    }
    for (int j = 0; j < n; ++j)   /* b = L * x_ref (CSC SpMV, row-major rhs as main.cu:347-358) */
      for (int e = col_ptr[j]; e < col_ptr[j + 1]; ++e)
        for (int k = 0; k < rhs; ++k) b[row_idx[e] * rhs + k] += val[e] * x_ref[j * rhs + k];
    double gflops = 0.0;
    const int rc = sptrsv_syncfree_cuda(col_ptr, row_idx, val, n, n, nnz, substitution, rhs,
                                        SPTRSV_OPT_WARP_AUTO, x, b, x_ref, &gflops);
    double num = 0.0, den = 0.0;
    for (int i = 0; i < n * rhs; ++i) {
      num += x[i] > x_ref[i] ? x[i] - x_ref[i] : x_ref[i] - x[i];
      den += x_ref[i] > 0 ? x_ref[i] : -x_ref[i];
    }
    const double l1 = num / den;
    printf("%s: status %d, L1 relative error %.3e, %.3f GFLOPS\n",
           substitution == SPTRSV_SUBSTITUTION_FORWARD ? "forward" : "backward", rc, l1, gflops);
    if (rc != 0 || !(l1 < 1e-4)) ++failures;
  }
  /* the reference's own error convention: m != n is rejected with -1 */
  if (sptrsv_syncfree_cuda(col_ptr, row_idx, val, n, n + 1, 3 * n, 0, rhs, SPTRSV_OPT_WARP_AUTO, x, b, x_ref,
                           NULL) != -1)
    ++failures;
  free(col_ptr);
  free(row_idx);
  free(val);
  free(x_ref);
  free(b);
  free(x);
  printf(failures ? "drop-in FAILED\n" : "drop-in ok\n");
  return failures ? 1 : 0;
}
