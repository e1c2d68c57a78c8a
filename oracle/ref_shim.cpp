/*
 * Build shim that compiles the reference's own serial sources, where they lie
 * in the reference checkout, into C-callable wrappers for the test suite.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle). Nothing in the library links it.
 * Compiled twice by oracle/Makefile, with VALUE_TYPE=double (REF_SFX=_f64)
 * and VALUE_TYPE=float (REF_SFX=_f32); the reference's functions are wrapped
 * in an anonymous namespace so the two precisions do not collide.
 *
 * Wrapped reference functions (SpTRSV_cuda/):
 *   sptrsv_syncfree_analyser  sptrsv_syncfree_serialref.h:6-23
 *   sptrsv_syncfree_executor  sptrsv_syncfree_serialref.h:25-108
 *   matrix_transposition      tranpose.h:6-43
 *   findlevel / findlevel_csc findlevel.h:6-69, 71-147
 *   mmio_info / mmio_data     mmio_highlevel.h:8-134, 137-296 (Matrix Market
 *                             reader, with mmio.h)
 */
#include <time.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <sys/time.h>

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define WRAP(name) CAT(name, REF_SFX)

namespace {
/* tranpose.h calls exclusive_scan, which the reference defines in utils.h
 * next to CUDA-only code; this is a plain in-place exclusive prefix sum. */
template <typename T>
void exclusive_scan(T *a, int len)
{
    T run = 0;
    for (int i = 0; i < len; ++i) { T v = a[i]; a[i] = run; run += v; }
}
#include "common.h"
#include "sptrsv_syncfree_serialref.h"
#include "tranpose.h"
#include "findlevel.h"
#include "mmio_highlevel.h"
}

extern "C" {
int WRAP(ref_analyser)(const int *row_idx, int m, int n, int nnz, int *in_degree)
{
    return sptrsv_syncfree_analyser(row_idx, m, n, nnz, in_degree);
}
int WRAP(ref_executor)(const int *col_ptr, const int *row_idx, const VALUE_TYPE *val,
                       const int *in_degree, int m, int n, int substitution, int rhs,
                       const VALUE_TYPE *b, VALUE_TYPE *x)
{
    return sptrsv_syncfree_executor(col_ptr, row_idx, val, in_degree, m, n,
                                    substitution, rhs, b, x);
}
void WRAP(ref_transpose)(int m, int n, int nnz, const int *ptr, const int *idx,
                         const VALUE_TYPE *val, int *out_idx, int *out_ptr,
                         VALUE_TYPE *out_val)
{
    matrix_transposition(m, n, nnz, ptr, idx, val, out_idx, out_ptr, out_val);
}
int WRAP(ref_findlevel)(const int *col_ptr, const int *row_idx, const int *row_ptr,
                        int m, int *nlevel, int *level_ptr, int *level_item)
{
    return findlevel(col_ptr, row_idx, row_ptr, m, nlevel, level_ptr, level_item);
}
int WRAP(ref_findlevel_csc)(const int *col_ptr, const int *row_idx, const VALUE_TYPE *val,
                            int m, int n, int nnz, int *nlevel, int *pmin, int *pavg,
                            int *pmax)
{
    return findlevel_csc(col_ptr, row_idx, val, m, n, nnz, nlevel, pmin, pavg, pmax);
}
int WRAP(ref_mmio_info)(int *m, int *n, int *nnz, int *is_symmetric, const char *filename)
{
    return mmio_info(m, n, nnz, is_symmetric, const_cast<char *>(filename));
}
int WRAP(ref_mmio_data)(int *row_ptr, int *col_idx, VALUE_TYPE *val, const char *filename)
{
    return mmio_data(row_ptr, col_idx, val, const_cast<char *>(filename));
}
}
