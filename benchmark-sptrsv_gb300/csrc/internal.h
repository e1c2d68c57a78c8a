// Library-internal declarations shared by the .cu translation units and the
// C-ABI layer. Nothing here is exported.
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "common.cuh"

namespace sptrsv {

// Structural defects found by the validation kernels (bitmask).
enum StructFlags : int {
  SF_BAD_PTR = 1,         // column pointers not monotone or not [0, nnz]
  SF_ROW_RANGE = 2,       // a row index outside [0, n)
  SF_UNSORTED = 4,        // rows not strictly ascending inside a column
  SF_MISSING_DIAG = 8,    // column without its diagonal entry
  SF_WRONG_TRIANGLE = 16, // entry on the wrong side of the diagonal
  SF_ZERO_DIAG = 32,      // zero (or non-finite) diagonal value
};

// Executor families.
enum Sched : int { SCHED_AUTO = 0, SCHED_PUSH = 1, SCHED_PULL = 2, SCHED_LEVELSET = 3 };

struct ExecConfig {
  int sched = SCHED_PULL;
  int lanes = 1;          // lanes per unknown (1, 2, 4, 8, 16, 32)
  int chunk = 1024;       // positions per CTA work unit
  int smem_tier = 1;      // resolve in-chunk dependencies through shared memory
  int exact = 0;          // oracle-order arithmetic (pull only)
  int block = 256;        // threads per CTA (64, 128 or 256)
  int ctas_per_sm = 0;    // resident CTAs per SM (0: as many as fit)
  unsigned sleep_max = 0; // backoff cap of global polls in ns (0: spin)
  int staged = 1;         // one right-hand side: TMA-staged chunk executor
  int emax = 0;           // staged: dependency entries per chunk (0: automatic)
  int stages = 2;         // staged: chunk buffers in the producer/consumer ring
  int wsync = 0;          // unstaged one-rhs pull: warp-synchronous lanes (k_pull_wsync)
  int split = 0;          // warp-synchronous, fast arithmetic: split lists longer than this (0: never)
  int wsync_batch = 4;    // warp-synchronous one rhs, fast arithmetic: dependencies per lane per iteration
  int opt = 3;            // push, many rhs: the reference's lane mode (1 entries, 2 rhs, 3 automatic rule)
  int rhs_tile = 0;       // many rhs: right-hand sides per lane (1, 2, 4; 0: automatic)
  int one_batch = 0;      // importer executor: every list fits one lockstep batch (no batch reloads)
};

// Lane group of the many-rhs executors: G lanes per unknown (a power of two,
// 4..32), each covering `rpl` right-hand sides, with G * rpl >= rhs when
// rhs <= 128. rhs_tile = 0 picks one right-hand side per lane up to 32 and two
// beyond; otherwise rpl = rhs_tile where that keeps G >= 4 (else the next
// smaller tile).
inline int multi_group(int rhs, int rhs_tile, int* rpl_out) {
  int rpl = rhs_tile > 0 ? rhs_tile : (rhs <= 32 ? 1 : 2);
  if (rpl != 1 && rpl != 2 && rpl != 4) rpl = 1;
  while (rpl > 1 && (rhs + rpl - 1) / rpl < 4) rpl >>= 1;
  if (rpl < 2 && rhs > 32) rpl = 2;
  if (rpl < 4 && rhs > 64) rpl = 4;
  const int need = (rhs + rpl - 1) / rpl;
  int g = 4;
  while (g < need && g < 32) g <<= 1;
  if (rpl_out) *rpl_out = rpl;
  return g;
}

// Work units of the staged executor: chunk k covers walk indices
// [start[k], start[k+1]) (positions for a forward walk, reversed positions for
// the adjoint walk), holds at most cmax unknowns and emax dependency entries,
// and is processed in one mode (0 thread per unknown, 1 warp per unknown,
// 2 warp per unknown reading its list from global memory).
struct ChunkTable {
  int nchunks = 0, cmax = 0, emax = 0;
  int* start = nullptr;   // device [nchunks+1]
  int* mode = nullptr;    // device [nchunks]
};

// Work units of the split-list warp-synchronous executor: a walk's dependency
// lists cut into k <= 32 interleaved pieces of about `split` entries (piece j
// of an unknown covers entries lo, lo + k, lo + 2k, ... below hi, lo = list
// start + j; k = the number of adjacent lanes holding the unknown),
// 32 pieces per warp segment with no unknown straddling two segments (padding
// pieces have walk -1). A chunk holds at most ceil(chunk/32) segments (one
// per warp when chunk = threads per CTA) and never crosses a multiple of
// `chunk` walk indices (so chunks stay inside order blocks of that size).
struct PieceTable {
  int split = 0, chunk = 0, nseg = 0, nchunks = 0;
  int* walk = nullptr;    // device [nseg*32]
  int* row = nullptr;     // device [nseg*32] row of the unknown (perm of its position; 0 for padding)
  int* lo = nullptr;      // device [nseg*32] first entry (list start + piece index)
  int* hi = nullptr;      // device [nseg*32] end of the list
  int* cseg = nullptr;    // device [nchunks+1] first segment of each chunk
  int* cbase = nullptr;   // device [nchunks] first walk index of each chunk
  unsigned char* seg_split = nullptr;  // device [nseg] 1 if an unknown of the segment spans several lanes
};

// Imported dependencies of a forward walk in work units (the units of a
// blocked layout, else ranges of `chunk` positions): unit c covers positions
// [start[c], start[c+1]) and reads the positions q[ptr[c] .. ptr[c+1])
// (sorted) from other units; dep_slot[e] = shared-memory slot of dependency e
// (in-unit: its position minus the unit start; imported: width + its index in
// the unit's list, width = the longest unit).
//
// The unit pipeline (ring > 0) keeps only a ring of `ring` slots (a power of
// two) per unit: an in-unit dependency fewer than ring - 32 positions back
// reads slot (position - unit start) mod ring, and every other dependency,
// in-unit ones further back included, is imported into slot ring + index.
// Each unit is cut into segments (runs of at most 32 consecutive positions,
// one lane each; segment g covers [segs[g], segs[g+1])) and the segments into
// stages of at most pmax positions, emax list entries and smax segments: unit
// c owns stages ustage[c] .. ustage[c+1]-1; stage k covers positions
// [stab[2k].x, stab[2k].y), list entries [stab[2k].z, stab[2k].w) and
// segments [stab[2k+1].x, stab[2k+1].y).
struct ImportTable {
  int chunk = 0, nchunks = 0, width = 0, max_imports = 0;
  int* start = nullptr;     // device [nchunks+1]
  int* ptr = nullptr;       // device [nchunks+1]
  int* q = nullptr;         // device [total imports]
  int* dep_slot = nullptr;  // device [ndep + padding]
  int ring = 0, ring_cap = 0, pmax = 0, emax = 0, smax = 0, stages = 0, nstages = 0;
  int* ustage = nullptr;    // device [nchunks+1]
  int4* stab = nullptr;     // device [2*nstages]
  int* segs = nullptr;      // device [segments+1 + padding] first position of each segment
};

// Solve-time description of one right-hand-side block. Element (i, k) of b
// (x) lives at i*si + k*sk.
template <typename T>
struct VecView {
  const T* b;
  T* x;
  long long b_si, b_sk, x_si, x_sk;
};

// Device arrays describing one analysed triangle in "position" space:
// position p is the p-th unknown in the execution schedule, row perm[p].
struct Layout {
  int n = 0;
  int ndep = 0;
  int* perm = nullptr;       // [n] position -> row
  int* iperm = nullptr;      // [n] row -> position
  // pull layout (dependencies of each position, diagonal excluded; listed in
  // the order the serial executor accumulates them)
  int* dep_ptr = nullptr;    // [n+1]
  int* dep_pos = nullptr;    // [ndep]
  int* dep_src = nullptr;    // [ndep] CSC entry index (for value staging)
  int* dep_col = nullptr;    // [ndep] column (unknown) of the dependency
  int* diag_src = nullptr;   // [n]
  // push layout (dependents of each position, diagonal excluded), listed in the
  // order the serial executor applied to the transpose accumulates them
  int* out_ptr = nullptr;    // [n+1]
  int* out_pos = nullptr;    // [ndep]
  int* out_src = nullptr;    // [ndep]
  // the same lists in ready order, for the fast executors: dependencies by
  // ascending position, dependents by descending position (the adjoint walk)
  int* dep_pos_f = nullptr;  // [ndep]
  int* dep_src_f = nullptr;  // [ndep]
  int* out_pos_f = nullptr;  // [ndep]
  int* out_src_f = nullptr;  // [ndep]
  // level sets in position space (valid when the schedule is pure level order)
  int nlevels = 0;
  std::vector<int> level_ptr_host;
  int* level_ptr = nullptr;  // [nlevels+1] (positions)
};

template <typename T>
struct Values {
  T* dep_val = nullptr;  // [ndep]
  T* dep_w = nullptr;    // [ndep] values scaled by the reciprocal of the row's diagonal (ready order)
  T* out_val = nullptr;  // [ndep]
  T* out_w = nullptr;    // [ndep] values scaled by the reciprocal of the owning position's diagonal (ready order)
  T* diag = nullptr;     // [n]
  T* rcp = nullptr;      // [n] correctly rounded 1/diag
};

// Independent triangles sharing one index space (a batch): unknown c belongs
// to system sys_of[c], whose unknowns are [sys_off[s], sys_off[s] + sys_n[s])
// and which is solved forward (dir 0, lower) or backward (dir 1, upper). A
// single system has count 1, null arrays and a uniform `substitution`.
struct SysDesc {
  int count = 1;
  int substitution = 0;
  const unsigned char* dir = nullptr;
  const int* sys_of = nullptr;
  const int* sys_off = nullptr;
  const int* sys_n = nullptr;
};

// ---------------------------------------------------------------- analysis
cudaError_t launch_validate_ptr(const int* col_ptr, int n, int nnz, int* flags, cudaStream_t s);
// safe on any column pointers: a column with an out-of-range or decreasing pair is
// flagged SF_BAD_PTR and its rows are not read (nnz = length of row_idx)
cudaError_t launch_validate_rows(const int* col_ptr, const int* row_idx, int n, int nnz, const SysDesc& sd,
                                 int* flags, cudaStream_t s);
// batch: merge per-system CSC arrays (local indices, concatenated) into one
// block-diagonal CSC and fill the per-unknown system/direction arrays
cudaError_t launch_batch_merge(const int* col_ptr_cat, const int* row_idx_cat, int count, const int* sys_off,
                               const int* sys_eoff, const int* sys_sub, int n, int nnz, int* col_ptr, int* row_idx,
                               unsigned char* dir, int* sys_of, int* flags, cudaStream_t s);
// natural execution order: forward systems ascending, backward systems descending
cudaError_t launch_nat_rows(const SysDesc& sd, int n, int* rows_nat, cudaStream_t s);
// rows outside [0, m) are skipped; with `bad` set they also raise SF_ROW_RANGE there
cudaError_t launch_in_degree(const int* row_idx, int m, int nnz, int* in_degree, cudaStream_t s,
                             int* bad = nullptr);
// exclusive scan of `count` ints; out may alias in; out[count] receives the total when with_total.
cudaError_t exclusive_scan_int(const int* in, int* out, int count, bool with_total, cudaStream_t s);
size_t radix_sort_temp_bytes(int count);
// Stable LSD radix sort of (key, value) pairs on the low `key_bits` bits.
cudaError_t radix_sort_pairs(const unsigned* keys_in, const int* vals_in, unsigned* keys_out,
                             int* vals_out, int count, int key_bits, void* temp, cudaStream_t s);
cudaError_t launch_iota(int* out, int count, int start, int step, cudaStream_t s);
cudaError_t launch_expand_cols(const int* col_ptr, int n, int* col_of, cudaStream_t s);
cudaError_t launch_copy_keys(const int* in, unsigned* out, int count, cudaStream_t s);
cudaError_t launch_gather_int(const int* src, const int* idx, int* out, int count, cudaStream_t s);
cudaError_t launch_levels(const int* col_ptr, const int* row_idx, const int* in_degree, int n,
                          int* cnt_scratch, int* front_a, int* front_b, int* depth, int* level_sizes,
                          DeviceCtl* ctl, unsigned long long timeout_ns, cudaStream_t s);
// mode 0: level; 1: (natural block, system) of blocked orders; 2: the level
// stretched to a target of max_depth keys, floor(level * max(D_s, max_depth) /
// D_s) with D_s = sys_depth[system]
cudaError_t launch_schedule_keys(const int* rows, const int* depth, int n, const SysDesc& sd, int block,
                                 int mode, unsigned* keys, cudaStream_t s, const int* sys_depth = nullptr,
                                 int max_depth = 0);
cudaError_t launch_sys_depth(const int* depth, const int* sys_of, int n, int* sys_depth, cudaStream_t s);
cudaError_t launch_inverse_perm(const int* perm, int n, int* iperm, cudaStream_t s);
// key = 0 for rows with more than `threshold` dependencies, 1 otherwise
cudaError_t launch_long_keys(const int* rows, const int* in_degree, int n, int threshold, unsigned* keys,
                             cudaStream_t s);
cudaError_t launch_dep_counts(const int* perm, const int* in_degree, int n, int* counts, cudaStream_t s);
cudaError_t launch_out_counts(const int* perm, const int* col_ptr, int n, int* counts, cudaStream_t s);
cudaError_t launch_fill_pull(const int* perm, const int* iperm, const int* csr_ptr, const int* csr_col,
                             const int* csr_src, const int* dep_ptr, int n, const SysDesc& sd,
                             int* dep_pos, int* dep_src, int* dep_col, int* diag_src, cudaStream_t s);
cudaError_t launch_fill_push(const int* perm, const int* iperm, const int* col_ptr, const int* row_idx,
                             const int* out_ptr, int n, const SysDesc& sd, int* out_pos, int* out_src,
                             cudaStream_t s);
// count += off-diagonal entries whose row and column share a block of `block`
// unknowns in the natural execution order.
cudaError_t launch_block_locality(const int* row, const int* col, int nnz, int n, int block, bool backward,
                                  unsigned long long* count, cudaStream_t s);
// count[0] += unknowns with two or more dependencies on the level just before
// their own, count[1] += unknowns with any dependency (CSR rows, depth per row).
cudaError_t launch_coarrival(const int* row_ptr, const int* col, const int* depth, int n, unsigned long long* count,
                             cudaStream_t s);
// Sorts every list [ptr[p], ptr[p+1]) of (pos, src) by pos (descending when asked).
cudaError_t launch_sort_lists(const int* ptr, const int* pos, const int* src, int n, int count, bool descending,
                              int* pos_out, int* src_out, cudaStream_t s);
template <typename TV, typename T>
cudaError_t launch_stage_values(const Layout& L, const TV* val, Values<T>& V, int* flags, cudaStream_t s);

// ---------------------------------------------------------------- execution
// Transposed (adjoint) solve request: optional fused gradient w.r.t. the values.
template <typename T>
struct AdjointArgs {
  T* grad = nullptr;       // [nnz] CSC order, or null
  const T* xf = nullptr;   // forward solution (row-indexed, strides below)
  long long xf_si = 0, xf_sk = 0;
};
template <typename T>
cudaError_t launch_pull(const Layout& L, const Values<T>& V, int rhs, const VecView<T>& v, T* xw,
                        DeviceCtl* ctl, const ExecConfig& cfg, unsigned long long timeout_ns,
                        int num_sms, cudaStream_t s, const AdjointArgs<T>* adj = nullptr,
                        const PieceTable* pc = nullptr);
template <typename T>
cudaError_t launch_push(const Layout& L, const Values<T>& V, int rhs, const VecView<T>& v, T* left_sum,
                        unsigned* counters, DeviceCtl* ctl, const ExecConfig& cfg,
                        unsigned long long timeout_ns, int num_sms, cudaStream_t s);
template <typename T>
cudaError_t launch_levelset(const Layout& L, const Values<T>& V, int rhs, const VecView<T>& v, T* xw,
                            DeviceCtl* ctl, const ExecConfig& cfg, unsigned long long timeout_ns,
                            cudaStream_t s);
size_t pull_smem_bytes(int chunk, int rhs, size_t elem);
size_t imported_smem_bytes(int chunk, int max_imports, size_t elem);
// warp-synchronous one-rhs forward pull with an importer warp per CTA (blocked layouts)
template <typename T>
cudaError_t launch_pull_imported(const Layout& L, const Values<T>& V, const VecView<T>& v, T* xw, DeviceCtl* ctl,
                                 const ExecConfig& cfg, unsigned long long timeout_ns, int num_sms, cudaStream_t s,
                                 const ImportTable& im);
// unit pipeline: consumer, importer and bulk-copy loader warp per unit (blocked layouts);
// c0 = workspace of n + 16 elements for the first terms
size_t unit_smem_bytes(int ring, int max_imports, int pmax, int emax, int smax, int stages, size_t elem);
template <typename T>
cudaError_t launch_pull_unit(const Layout& L, const Values<T>& V, const VecView<T>& v, T* xw, T* c0, DeviceCtl* ctl,
                             const ExecConfig& cfg, unsigned long long timeout_ns, int num_sms, cudaStream_t s,
                             const ImportTable& im);
size_t staged_smem_bytes(int cmax, int emax, size_t elem, bool smem_tier, int stages);
template <typename T>
cudaError_t launch_pull_staged(const Layout& L, const Values<T>& V, const ChunkTable& tab, const VecView<T>& v, T* xw,
                               DeviceCtl* ctl, const ExecConfig& cfg, unsigned long long timeout_ns, int num_sms,
                               cudaStream_t s, const AdjointArgs<T>* adj);

template <typename T>
cudaError_t launch_grad_values(const int* csc_row, const int* csc_col, int nnz, int rhs, const T* lambda,
                               const T* x, long long si, long long sk, T* dval, cudaStream_t s);

// out (cols x rows, row-major) = transpose of in (rows x cols, row-major)
template <typename T>
cudaError_t launch_transpose(const T* in, T* out, int rows, int cols, cudaStream_t s);

// ---------------------------------------------------------------- mixed precision
// Fused first refinement step (exec_refine.cu): one pass computing the FP32
// solution x0, the FP64 residual and the FP32 correction d together; writes
// x = x0 + d (FP64, strides si/sk) and stats[0..2] = max |d|, max |x|, max |x0|
// (ordered bits; zero them first). xw: n*rhs 64-bit words set to all ones.
// wsplit (optional): (hi, lo) float pairs of v64.dep_w; given, the residual runs
// in double-float on the FP32 pipe instead of FP64 (launch_split_weights fills it)
cudaError_t launch_refine_fused(const Layout& L, const Values<float>& v32, const Values<double>& v64, int rhs,
                                const double* b, double* x, long long si, long long sk, unsigned long long* xw,
                                unsigned long long* stats, DeviceCtl* ctl, const ExecConfig& cfg,
                                unsigned long long timeout_ns, int num_sms, cudaStream_t s,
                                const float2* wsplit = nullptr);
cudaError_t launch_split_weights(const double* w, long long count, float2* out, cudaStream_t s);
// The same fused step (double-float residual, one right-hand side, b and x
// vectors) on a blocked layout, with an importer warp per CTA (the table of
// launch_pull_imported)
cudaError_t launch_refine_fused_imported(const Layout& L, const Values<double>& v64, const float2* wsplit,
                                         const double* b, double* x, unsigned long long* xw,
                                         unsigned long long* stats, DeviceCtl* ctl, const ExecConfig& cfg,
                                         unsigned long long timeout_ns, int num_sms, cudaStream_t s,
                                         const ImportTable& im);
cudaError_t launch_cast_d2f(const double* in, float* out, long long count, cudaStream_t s);
cudaError_t launch_residual(const Layout& L, const Values<double>& V, int rhs, const double* b, const double* x,
                            long long si, long long sk, float* r, cudaStream_t s);
cudaError_t launch_update(double* x, const float* d, long long count, unsigned long long* stats, bool first,
                          cudaStream_t s);

// Kernel-level surface of the reference: in-degree countdown counters owned by
// the caller, natural column order, one warp per column. A row index outside
// [0, m) is never written through: the kernel records DEV_BAD_INPUT and stops.
// With `gate` set, the kernel does nothing but record DEV_BAD_INPUT when
// *gate is non-zero (structural flags found by validation earlier in the stream).
template <typename T>
cudaError_t launch_ref_executor(const int* col_ptr, const int* row_idx, const T* val, int* in_degree,
                                T* left_sum, int m, int substitution, int rhs, int opt, const T* b, T* x,
                                DeviceCtl* ctl, unsigned long long timeout_ns, cudaStream_t s,
                                const int* gate = nullptr);

}  // namespace sptrsv
