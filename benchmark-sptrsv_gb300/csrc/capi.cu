// C ABI: handles, analysis pipeline, solve dispatch, status mapping, and the
// reference-compatible host entry point.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/sptrsv_gb300.h"
#include "internal.h"

using namespace sptrsv;

namespace {

int g_verbose = 0;
int g_bench_repeat = 100;  // BENCH_REPEAT of the reference (common.h:13-15)
constexpr int kLongDeps = 32;  // dependency lists longer than this are solved by a whole warp

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct sptrsv_gb300_handle_s {
  int device = 0;
  int num_sms = 0;
  // options
  ExecConfig cfg;
  int order_block = INT_MAX;   // level order: the fastest schedule on both deep and wide DAGs measured
  long long timeout_ms = 1000;
  int sync_check = 1;
  int sched_option = SCHED_AUTO;
  int lanes_option = 0;    // 0: automatic
  int chunk_option = 0;    // 0: automatic
  int block_option = 0;    // 0: automatic
  long long backoff_ns = 256;
  int ctas_per_sm = 0;
  int staged = 1;
  int emax_option = 0;
  int stages_option = 2;
  int fused_grad = 0;
  int wsync = 0;
  int split = 32;
  int wsync_batch = 0;   // 0: automatic (auto_wsync_batch)
  int opt_option = SPTRSV_OPT_WARP_AUTO;  // push, many rhs: the reference's lane mode
  int rhs_tile_option = 0;                // many rhs: right-hand sides per lane (0: automatic)
  int stretch_option = 1;                 // batches in level order: levels stretched to the batch depth
  unsigned long long user_set = 0;  // options the caller set explicitly (bit = option id)
  // executor settings chosen from the analysis for SPTRSV_SCHED_AUTO (one rhs)
  struct AutoPlan {
    bool valid = false;
    int order_block = INT_MAX, chunk = 256, block = 256, ctas = 2, backoff = 0, staged = 0, wsync = 1;
    int split_fwd = 0, split_adj = 0;  // split length for the forward / transposed walk (0: none)
    double locality = 0.0;
    double coarrive = 0.0;  // short lists: share of unknowns with >= 2 dependencies on the preceding level
  } plan;
  // analysis
  bool analysed = false;
  int n = 0, nnz = 0, substitution = 0;
  int nlevels = 0, pmin = 0, pavg = 0, pmax = 0, max_in_degree = 0;
  double analysis_ms = 0.0;
  std::vector<int> level_sizes_host;
  // batch (several independent triangles in one index space)
  int batch_count = 1;
  std::vector<int> sys_off_host, sys_n_host, sys_sub_host;
  unsigned char* sys_dir = nullptr;
  int* sys_of = nullptr;
  int* sys_off = nullptr;
  int* sys_n = nullptr;
  int* csc_ptr = nullptr;   // owned copy of the structure
  int* csc_row = nullptr;
  int* csc_col = nullptr;   // column of every CSC entry
  int* in_degree = nullptr;
  int* depth = nullptr;
  int* csr_ptr = nullptr;
  int* csr_col = nullptr;
  int* csr_src = nullptr;
  int* level_item = nullptr;
  int* level_ptr_nat = nullptr;
  Layout layout;
  int layout_block = -1;
  int layout_stretched = 0;        // the layout's level order is stretched per system (batches)
  std::vector<int> layout_units;   // blocked layouts: start positions of the units (+ n), else empty
  std::vector<int> dep_cnt_host;   // dependencies per position
  std::vector<int> out_cnt_host;   // dependents per position
  int max_dep_cnt = 0, max_out_cnt = 0;
  ChunkTable tab_fwd, tab_adj;
  PieceTable pc_fwd, pc_adj;
  ImportTable imports;
  int import_option = 1;   // importer warp on blocked layouts (SPTRSV_OPTION_IMPORT)
  ImportTable pipe;        // unit pipeline tables (ring slots, stages)
  int pipe_option = 0;     // SPTRSV_OPTION_UNIT_PIPELINE: 0 off, 1 on, else the ring cap
  int fused_refine = 2;    // SPTRSV_OPTION_FUSED_REFINE: first refinement step fused into the FP32 pass
                           // (2: residual in double-float on the FP32 pipe, 1: in FP64, 0: separate passes)
  // staged values
  Values<double> v64;
  Values<float> v32;
  bool staged64 = false, staged32 = false;
  // workspace
  DevBuf xw, left_sum, counters, r32, d32, stats;
  DevBuf tb, tx;  // row-major staging of column-major blocks of many right-hand sides
  DevBuf c0;      // unit pipeline: first term b/d of every position
  DevBuf wsplit;  // fused refinement in double-float: (hi, lo) float pairs of the FP64 weights
  bool wsplit_ok = false;
  DeviceCtl* ctl = nullptr;
  int* flags = nullptr;
  int* host_pinned = nullptr;  // 4 ints
  int last_sched = 0;
  bool last_pipe = false;  // the last one-rhs solve ran the unit pipeline
  size_t device_bytes = 0;
  int profile = 0;
  cudaEvent_t ev_exec[2] = {nullptr, nullptr};
  bool ev_recorded = false;
};

namespace {

#define CUDA_TRY(...)                                \
  do {                                               \
    cudaError_t e_ = (__VA_ARGS__);                  \
    if (e_ != cudaSuccess) return map_cuda_error(e_); \
  } while (0)

#define ST_TRY(...)                \
  do {                             \
    int s_ = (__VA_ARGS__);        \
    if (s_ != SPTRSV_OK) return s_; \
  } while (0)

int map_cuda_error(cudaError_t e) {
  cudaGetLastError();  // clear a non-sticky error so later launches are not blamed for it
  if (e == cudaErrorMemoryAllocation) return SPTRSV_ERR_OOM;
  return SPTRSV_ERR_CUDA;
}

// Every array gets 16 spare elements so the executors' bulk copies, widened
// to 16-byte boundaries, never read past an allocation.
template <typename T>
int dev_alloc(sptrsv_gb300_handle_s* h, T** p, size_t count) {
  *p = nullptr;
  count += 16;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * count);
  if (e != cudaSuccess) return map_cuda_error(e);
  h->device_bytes += sizeof(T) * count;
  return SPTRSV_OK;
}

template <typename T>
void dev_free(T** p) {
  if (*p) cudaFree(*p);
  *p = nullptr;
}

int bits_for(long long maxval) {
  int b = 1;
  while (b < 32 && (1LL << b) <= maxval) ++b;
  return b;
}

void free_table(ChunkTable& t) {
  if (t.start) cudaFree(t.start);
  if (t.mode) cudaFree(t.mode);
  t = ChunkTable();
}

void free_pieces(PieceTable& t) {
  if (t.walk) cudaFree(t.walk);
  if (t.row) cudaFree(t.row);
  if (t.lo) cudaFree(t.lo);
  if (t.hi) cudaFree(t.hi);
  if (t.cseg) cudaFree(t.cseg);
  if (t.cbase) cudaFree(t.cbase);
  if (t.seg_split) cudaFree(t.seg_split);
  t = PieceTable();
}

void free_imports(ImportTable& t) {
  if (t.start) cudaFree(t.start);
  if (t.ptr) cudaFree(t.ptr);
  if (t.q) cudaFree(t.q);
  if (t.dep_slot) cudaFree(t.dep_slot);
  if (t.ustage) cudaFree(t.ustage);
  if (t.stab) cudaFree(t.stab);
  if (t.segs) cudaFree(t.segs);
  t = ImportTable();
}

void free_layout(Layout& L) {
  dev_free(&L.perm);
  dev_free(&L.iperm);
  dev_free(&L.dep_ptr);
  dev_free(&L.dep_pos);
  dev_free(&L.dep_src);
  dev_free(&L.dep_col);
  dev_free(&L.diag_src);
  dev_free(&L.out_ptr);
  dev_free(&L.out_pos);
  dev_free(&L.out_src);
  dev_free(&L.dep_pos_f);
  dev_free(&L.dep_src_f);
  dev_free(&L.out_pos_f);
  dev_free(&L.out_src_f);
  dev_free(&L.level_ptr);
  L = Layout();
}

template <typename T>
void free_values(Values<T>& V) {
  dev_free(&V.dep_val);
  dev_free(&V.dep_w);
  dev_free(&V.out_w);
  dev_free(&V.out_val);
  dev_free(&V.diag);
  dev_free(&V.rcp);
}

void free_analysis(sptrsv_gb300_handle_s* h) {
  dev_free(&h->sys_dir);
  dev_free(&h->sys_of);
  dev_free(&h->sys_off);
  dev_free(&h->sys_n);
  h->batch_count = 1;
  h->sys_off_host.clear();
  h->sys_n_host.clear();
  h->sys_sub_host.clear();
  dev_free(&h->csc_ptr);
  dev_free(&h->csc_row);
  dev_free(&h->csc_col);
  dev_free(&h->in_degree);
  dev_free(&h->depth);
  dev_free(&h->csr_ptr);
  dev_free(&h->csr_col);
  dev_free(&h->csr_src);
  dev_free(&h->level_item);
  dev_free(&h->level_ptr_nat);
  free_layout(h->layout);
  free_table(h->tab_fwd);
  free_table(h->tab_adj);
  free_pieces(h->pc_fwd);
  free_pieces(h->pc_adj);
  free_imports(h->imports);
  free_imports(h->pipe);
  free_values(h->v64);
  free_values(h->v32);
  h->staged64 = h->staged32 = false;
  h->wsplit_ok = false;
  h->analysed = false;
  h->layout_block = -1;
}

void free_buf(DevBuf& b) {
  if (b.p) cudaFree(b.p);
  b = DevBuf();
}

int ensure_buf(sptrsv_gb300_handle_s* h, DevBuf& b, size_t bytes, int fill_zero, cudaStream_t s) {
  if (b.bytes >= bytes && b.p) return SPTRSV_OK;
  // Growing: make sure nothing in flight still uses the old buffer.
  CUDA_TRY(cudaStreamSynchronize(s));
  free_buf(b);
  CUDA_TRY(cudaMalloc(&b.p, bytes));
  b.bytes = bytes;
  h->device_bytes += bytes;
  if (fill_zero) CUDA_TRY(cudaMemsetAsync(b.p, 0, bytes, s));
  return SPTRSV_OK;
}

SysDesc sys_desc(const sptrsv_gb300_handle_s* h) {
  SysDesc d;
  d.count = h->batch_count;
  d.substitution = h->substitution;
  d.dir = h->sys_dir;
  d.sys_of = h->sys_of;
  d.sys_off = h->sys_off;
  d.sys_n = h->sys_n;
  return d;
}

unsigned long long timeout_ns(const sptrsv_gb300_handle_s* h) {
  return static_cast<unsigned long long>(h->timeout_ms) * 1000000ull;
}

// Clears the control block and the self-cleaning push workspace after a
// failed launch left them dirty.
int reset_after_failure(sptrsv_gb300_handle_s* h, cudaStream_t s) {
  cudaGetLastError();
  CUDA_TRY(cudaMemsetAsync(h->ctl, 0, sizeof(DeviceCtl), s));
  if (h->left_sum.p) CUDA_TRY(cudaMemsetAsync(h->left_sum.p, 0, h->left_sum.bytes, s));
  if (h->counters.p) CUDA_TRY(cudaMemsetAsync(h->counters.p, 0, h->counters.bytes, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return SPTRSV_OK;
}

int read_device_code(sptrsv_gb300_handle_s* h, cudaStream_t s, int* code) {
  CUDA_TRY(cudaMemcpyAsync(h->host_pinned, &h->ctl->code, sizeof(int), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  *code = h->host_pinned[0];
  return SPTRSV_OK;
}

int check_device(sptrsv_gb300_handle_s* h, cudaStream_t s) {
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return map_cuda_error(e);
  int code = 0;
  ST_TRY(read_device_code(h, s, &code));
  if (code != DEV_OK) {
    ST_TRY(reset_after_failure(h, s));
    return code == DEV_TIMEOUT ? SPTRSV_ERR_TIMEOUT : SPTRSV_ERR_CUDA;
  }
  return SPTRSV_OK;
}

int read_flags(sptrsv_gb300_handle_s* h, cudaStream_t s, int* flags) {
  CUDA_TRY(cudaMemcpyAsync(h->host_pinned + 1, h->flags, sizeof(int), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  *flags = h->host_pinned[1];
  return SPTRSV_OK;
}

// Builds the position-space layout for the given order block.
// Batches in level order (not for the level-set executor, which needs whole
// levels): each system's levels stretched to the batch's depth.
bool want_stretch(const sptrsv_gb300_handle_s* h, int block) {
  return h->batch_count > 1 && block >= h->n && h->stretch_option && h->sched_option != SCHED_LEVELSET;
}

int build_layout(sptrsv_gb300_handle_s* h, int block, cudaStream_t s) {
  free_layout(h->layout);
  free_table(h->tab_fwd);
  free_table(h->tab_adj);
  free_pieces(h->pc_fwd);
  free_pieces(h->pc_adj);
  free_imports(h->imports);
  free_imports(h->pipe);
  free_values(h->v64);
  free_values(h->v32);
  h->staged64 = h->staged32 = false;
  h->wsplit_ok = false;
  Layout& L = h->layout;
  const int n = h->n;
  const int ndep = h->nnz - n;
  L.n = n;
  L.ndep = ndep;
  ST_TRY(dev_alloc(h, &L.perm, n));
  ST_TRY(dev_alloc(h, &L.iperm, n));
  ST_TRY(dev_alloc(h, &L.dep_ptr, (size_t)n + 1));
  ST_TRY(dev_alloc(h, &L.out_ptr, (size_t)n + 1));
  ST_TRY(dev_alloc(h, &L.dep_pos, ndep));
  ST_TRY(dev_alloc(h, &L.dep_src, ndep));
  ST_TRY(dev_alloc(h, &L.dep_col, ndep));
  ST_TRY(dev_alloc(h, &L.out_pos, ndep));
  ST_TRY(dev_alloc(h, &L.out_src, ndep));
  ST_TRY(dev_alloc(h, &L.dep_pos_f, ndep));
  ST_TRY(dev_alloc(h, &L.dep_src_f, ndep));
  ST_TRY(dev_alloc(h, &L.out_pos_f, ndep));
  ST_TRY(dev_alloc(h, &L.out_src_f, ndep));
  ST_TRY(dev_alloc(h, &L.diag_src, n));

  const bool level_order = block >= n;
  const bool stretched = want_stretch(h, block);
  h->layout_units.clear();
  if (n > 0) {
    // natural order rows
    int* rows_nat = nullptr;
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&rows_nat), sizeof(int) * n, s));
    const SysDesc sd = sys_desc(h);
    CUDA_TRY(launch_nat_rows(sd, n, rows_nat, s));
    if (block <= 1) {
      CUDA_TRY(cudaMemcpyAsync(L.perm, rows_nat, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
    } else {
      unsigned *keys = nullptr, *keys_sorted = nullptr;
      int* rows_lv = nullptr;
      void* temp = nullptr;
      CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&keys), sizeof(unsigned) * n, s));
      CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&keys_sorted), sizeof(unsigned) * n, s));
      CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&rows_lv), sizeof(int) * n, s));
      CUDA_TRY(cudaMallocAsync(&temp, radix_sort_temp_bytes(n), s));
      // long dependency lists first inside each level (so chunks of one mode form), then
      // level order, then (blocked orders) the natural block
      int* rows_ls = nullptr;
      CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&rows_ls), sizeof(int) * n, s));
      CUDA_TRY(launch_long_keys(rows_nat, h->in_degree, n, kLongDeps, keys, s));
      CUDA_TRY(radix_sort_pairs(keys, rows_nat, keys_sorted, rows_ls, n, 1, temp, s));
      if (stretched) {
        // every system's levels spread over 65 % of the batch's depth (or its
        // own depth, if deeper), so a deep system's chain does not queue behind
        // the shallow systems' wide levels, and the shallow systems' work is
        // done before the deep chain's last third runs on its own. On the
        // 512-system batch (depth 22,729): 24.9 ms in global level order, 19.3
        // stretched to the whole depth, 18.7 to 55-70 % of it, 19.7 to 40 %
        int* sys_depth = nullptr;
        CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&sys_depth), sizeof(int) * h->batch_count, s));
        CUDA_TRY(cudaMemsetAsync(sys_depth, 0, sizeof(int) * h->batch_count, s));
        CUDA_TRY(launch_sys_depth(h->depth, h->sys_of, n, sys_depth, s));
        const int target = static_cast<int>(((long long)h->nlevels * 13 + 19) / 20);  // 65 %
        CUDA_TRY(launch_schedule_keys(rows_ls, h->depth, n, sd, block, 2, keys, s, sys_depth, target));
        CUDA_TRY(cudaFreeAsync(sys_depth, s));
      } else {
        CUDA_TRY(launch_schedule_keys(rows_ls, h->depth, n, sd, block, 0, keys, s));
      }
      CUDA_TRY(radix_sort_pairs(keys, rows_ls, keys_sorted, level_order ? L.perm : rows_lv, n,
                                bits_for(h->nlevels - 1), temp, s));
      CUDA_TRY(cudaFreeAsync(rows_ls, s));
      if (!level_order) {
        CUDA_TRY(launch_schedule_keys(rows_lv, h->depth, n, sd, block, 1, keys, s));
        int max_sys = 0;
        for (int v : h->sys_n_host) max_sys = std::max(max_sys, v);
        if (h->sys_n_host.empty()) max_sys = n;
        const long long max_key = (long long)((max_sys - 1) / block + 1) * h->batch_count;
        if (max_key > 0xFFFFFFFFLL) return SPTRSV_ERR_UNSUPPORTED;
        CUDA_TRY(radix_sort_pairs(keys, rows_lv, keys_sorted, L.perm, n, bits_for(max_key - 1), temp, s));
        // units of the blocked order (one system's natural block): contiguous
        // position ranges, the work units of the importer executor
        std::vector<unsigned> ks(n);
        CUDA_TRY(cudaMemcpyAsync(ks.data(), keys_sorted, sizeof(unsigned) * (size_t)n, cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        h->layout_units.clear();
        for (int i = 0; i < n; ++i)
          if (i == 0 || ks[i] != ks[i - 1]) h->layout_units.push_back(i);
        h->layout_units.push_back(n);
      }
      CUDA_TRY(cudaFreeAsync(keys, s));
      CUDA_TRY(cudaFreeAsync(keys_sorted, s));
      CUDA_TRY(cudaFreeAsync(rows_lv, s));
      CUDA_TRY(cudaFreeAsync(temp, s));
    }
    CUDA_TRY(cudaFreeAsync(rows_nat, s));
    CUDA_TRY(launch_inverse_perm(L.perm, n, L.iperm, s));
    CUDA_TRY(launch_dep_counts(L.perm, h->in_degree, n, L.dep_ptr, s));
    CUDA_TRY(exclusive_scan_int(L.dep_ptr, L.dep_ptr, n, true, s));
    CUDA_TRY(launch_out_counts(L.perm, h->csc_ptr, n, L.out_ptr, s));
    CUDA_TRY(exclusive_scan_int(L.out_ptr, L.out_ptr, n, true, s));
    CUDA_TRY(launch_fill_pull(L.perm, L.iperm, h->csr_ptr, h->csr_col, h->csr_src, L.dep_ptr, n, sd,
                              L.dep_pos, L.dep_src, L.dep_col, L.diag_src, s));
    CUDA_TRY(launch_fill_push(L.perm, L.iperm, h->csc_ptr, h->csc_row, L.out_ptr, n, sd, L.out_pos,
                              L.out_src, s));
    CUDA_TRY(launch_sort_lists(L.dep_ptr, L.dep_pos, L.dep_src, n, ndep, false, L.dep_pos_f, L.dep_src_f, s));
    CUDA_TRY(launch_sort_lists(L.out_ptr, L.out_pos, L.out_src, n, ndep, true, L.out_pos_f, L.out_src_f, s));
    std::vector<int> ptr((size_t)n + 1);
    CUDA_TRY(cudaMemcpyAsync(ptr.data(), L.dep_ptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    h->dep_cnt_host.resize(n);
    h->max_dep_cnt = 0;
    for (int p = 0; p < n; ++p) {
      h->dep_cnt_host[p] = ptr[p + 1] - ptr[p];
      h->max_dep_cnt = std::max(h->max_dep_cnt, h->dep_cnt_host[p]);
    }
    CUDA_TRY(cudaMemcpyAsync(ptr.data(), L.out_ptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    h->out_cnt_host.resize(n);
    h->max_out_cnt = 0;
    for (int p = 0; p < n; ++p) {
      h->out_cnt_host[p] = ptr[p + 1] - ptr[p];
      h->max_out_cnt = std::max(h->max_out_cnt, h->out_cnt_host[p]);
    }
  }
  if (level_order && !stretched) {
    L.nlevels = h->nlevels;
    L.level_ptr_host.assign(h->nlevels + 1, 0);
    for (int l = 0; l < h->nlevels; ++l) L.level_ptr_host[l + 1] = L.level_ptr_host[l] + h->level_sizes_host[l];
    ST_TRY(dev_alloc(h, &L.level_ptr, (size_t)h->nlevels + 1));
    CUDA_TRY(cudaMemcpyAsync(L.level_ptr, L.level_ptr_host.data(), sizeof(int) * (h->nlevels + 1),
                             cudaMemcpyHostToDevice, s));
  }
  CUDA_TRY(cudaStreamSynchronize(s));
  h->layout_block = block;
  h->layout_stretched = stretched ? 1 : 0;
  return SPTRSV_OK;
}

// Chunk table over a walk: counts[i] = dependency entries of the i-th unknown
// walked. A chunk ends at cmax unknowns, at emax entries, or where the mode
// changes; an unknown with more than emax entries forms a mode-2 chunk alone.
int build_table(sptrsv_gb300_handle_s* h, ChunkTable& t, const std::vector<int>& counts, bool reversed, int cmax,
                int emax) {
  free_table(t);
  const int n = static_cast<int>(counts.size());
  auto cnt = [&](int i) { return counts[reversed ? n - 1 - i : i]; };
  auto mode_of = [&](int c) { return c > emax ? 2 : (c > kLongDeps ? 1 : 0); };
  std::vector<int> start, mode;
  start.reserve(n / (cmax > 0 ? cmax : 1) + 16);
  int i = 0;
  while (i < n) {
    const int m0 = mode_of(cnt(i));
    start.push_back(i);
    mode.push_back(m0);
    if (m0 == 2) {
      ++i;
      continue;
    }
    long long e = 0;
    const int first = i;
    while (i < n && i - first < cmax) {
      const int c = cnt(i);
      if (mode_of(c) != m0 || e + c > emax) break;
      e += c;
      ++i;
    }
  }
  start.push_back(n);
  t.nchunks = static_cast<int>(mode.size());
  t.cmax = cmax;
  t.emax = emax;
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.start), sizeof(int) * start.size()));
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.mode), sizeof(int) * (mode.size() ? mode.size() : 1)));
  CUDA_TRY(cudaMemcpy(t.start, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice));
  if (!mode.empty()) CUDA_TRY(cudaMemcpy(t.mode, mode.data(), sizeof(int) * mode.size(), cudaMemcpyHostToDevice));
  h->device_bytes += sizeof(int) * (start.size() + mode.size());
  return SPTRSV_OK;
}

int ensure_table(sptrsv_gb300_handle_s* h, bool adj, int cmax, int emax) {
  ChunkTable& t = adj ? h->tab_adj : h->tab_fwd;
  if (t.start && t.cmax == cmax && t.emax == emax) return SPTRSV_OK;
  return build_table(h, t, adj ? h->out_cnt_host : h->dep_cnt_host, adj, cmax, emax);
}

// Piece table over a walk (see PieceTable): lists longer than `split` entries
// are cut into k = min(32, ceil(len/split)) interleaved slices (piece j takes
// entries j, j+k, j+2k, ... of the ready-ordered list), so the latest entries
// spread over all the pieces instead of piling up in the last one.
int build_pieces(sptrsv_gb300_handle_s* h, PieceTable& t, const std::vector<int>& counts, bool reversed, int split,
                 int chunk, cudaStream_t s) {
  free_pieces(t);
  const int n = static_cast<int>(counts.size());
  std::vector<long long> start((size_t)n + 1, 0);
  for (int p = 0; p < n; ++p) start[p + 1] = start[p] + counts[p];
  std::vector<int> walk, lo, hi;
  walk.reserve((size_t)n + n / 8 + 32);
  lo.reserve(walk.capacity());
  hi.reserve(walk.capacity());
  auto pad = [&]() {
    while (walk.size() % 32) {
      walk.push_back(-1);
      lo.push_back(0);
      hi.push_back(0);
    }
  };
  std::vector<int> cseg, cbase;
  std::vector<unsigned char> seg_split_host;
  const size_t seg_cap = static_cast<size_t>(std::max(1, (chunk + 31) / 32));
  // a reverse walk is shifted so that its chunk boundaries fall on multiples of
  // `chunk` positions (the order blocks of a blocked layout)
  const int shift = reversed ? (chunk - n % chunk) % chunk : 0;
  for (int i = 0; i < n; ++i) {
    const int p = reversed ? n - 1 - i : i;
    const long long c = counts[p], e0 = start[p];
    const int k = (split > 0 && c > split) ? static_cast<int>(std::min<long long>(32, (c + split - 1) / split)) : 1;
    const bool seg_full = walk.size() % 32 + k > 32;
    const size_t first = seg_full ? (walk.size() + 31) / 32 * 32 : walk.size();
    const size_t segs_after = (first + k - 1) / 32 + 1;  // segments in use once i is placed
    if ((i + shift) % chunk == 0 || i == 0 || (!cseg.empty() && segs_after - cseg.back() > seg_cap)) {
      pad();  // a chunk starts on a fresh segment
      cseg.push_back(static_cast<int>(walk.size() / 32));
      cbase.push_back(i);
    } else if (seg_full) {
      pad();
    }
    if (k > 1) {  // this unknown spans lanes of the segment it starts (after any padding above)
      const size_t sg = walk.size() / 32;
      if (seg_split_host.size() <= sg) seg_split_host.resize(sg + 1, 0);
      seg_split_host[sg] = 1;
    }
    for (int j = 0; j < k; ++j) {  // piece j: entries e0 + j, e0 + j + k, ... (interleaved)
      walk.push_back(i);
      lo.push_back(static_cast<int>(e0 + j));
      hi.push_back(static_cast<int>(e0 + c));
    }
  }
  pad();
  t.split = split;
  t.chunk = chunk;
  t.nseg = static_cast<int>(walk.size() / 32);
  t.nchunks = static_cast<int>(cseg.size());
  cseg.push_back(t.nseg);
  const size_t np = walk.size() > 0 ? walk.size() : 1;
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.walk), sizeof(int) * np));
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.row), sizeof(int) * np));
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.lo), sizeof(int) * np));
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.hi), sizeof(int) * np));
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.cseg), sizeof(int) * cseg.size()));
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.cbase), sizeof(int) * (cbase.empty() ? 1 : cbase.size())));
  seg_split_host.resize(t.nseg > 0 ? t.nseg : 1, 0);
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.seg_split), seg_split_host.size()));
  CUDA_TRY(cudaMemcpy(t.seg_split, seg_split_host.data(), seg_split_host.size(), cudaMemcpyHostToDevice));
  if (!cbase.empty())
    CUDA_TRY(cudaMemcpy(t.cbase, cbase.data(), sizeof(int) * cbase.size(), cudaMemcpyHostToDevice));
  if (!walk.empty()) {
    CUDA_TRY(cudaMemcpy(t.walk, walk.data(), sizeof(int) * walk.size(), cudaMemcpyHostToDevice));
    // row of each piece's unknown: perm gathered on the device (padding reads position 0)
    std::vector<int> posv(walk.size());
    for (size_t i = 0; i < walk.size(); ++i)
      posv[i] = walk[i] < 0 ? 0 : (reversed ? n - 1 - walk[i] : walk[i]);
    int* pos_dev = nullptr;
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&pos_dev), sizeof(int) * posv.size()));
    cudaError_t err = cudaMemcpyAsync(pos_dev, posv.data(), sizeof(int) * posv.size(), cudaMemcpyHostToDevice, s);
    if (err == cudaSuccess) err = launch_gather_int(h->layout.perm, pos_dev, t.row, static_cast<int>(posv.size()), s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    cudaFree(pos_dev);
    CUDA_TRY(err);
    CUDA_TRY(cudaMemcpy(t.lo, lo.data(), sizeof(int) * walk.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(t.hi, hi.data(), sizeof(int) * walk.size(), cudaMemcpyHostToDevice));
  }
  CUDA_TRY(cudaMemcpy(t.cseg, cseg.data(), sizeof(int) * cseg.size(), cudaMemcpyHostToDevice));
  h->device_bytes += sizeof(int) * (4 * np + cseg.size() + cbase.size());
  return SPTRSV_OK;
}

int ensure_pieces(sptrsv_gb300_handle_s* h, bool adj, int split, int chunk, cudaStream_t s) {
  PieceTable& t = adj ? h->pc_adj : h->pc_fwd;
  if (t.walk && t.split == split && t.chunk == chunk) return SPTRSV_OK;
  return build_pieces(h, t, adj ? h->out_cnt_host : h->dep_cnt_host, adj, split, chunk, s);
}

// Import table of the forward walk for chunks of `chunk` positions (see
// ImportTable). When a chunk's window and imports do not fit one CTA's shared
// memory only the sizes are recorded (no device arrays; the caller checks).
// ring_cap = 0: the importer kernel's table (a window as wide as the longest
// unit). ring_cap > 0: the unit pipeline's (ring slots, far dependencies
// imported, stages of at most pmax positions and emax entries).
int build_import_table(sptrsv_gb300_handle_s* h, ImportTable& t, int chunk, size_t elem, int ring_cap, int pmax,
                       int emax, int stages, cudaStream_t s) {
  free_imports(t);
  const int smax = std::max(4, pmax / 8);  // segments per stage
  const Layout& L = h->layout;
  const int n = L.n;
  const int ndep = L.ndep;
  std::vector<int> ptr((size_t)n + 1), pos(ndep > 0 ? (size_t)ndep : 1);
  CUDA_TRY(cudaMemcpyAsync(ptr.data(), L.dep_ptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToHost, s));
  if (ndep > 0)
    CUDA_TRY(cudaMemcpyAsync(pos.data(), L.dep_pos_f, sizeof(int) * (size_t)ndep, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  // work units: the blocked layout's units (one system's natural block), or
  // consecutive ranges of `chunk` positions
  std::vector<int> starts = h->layout_units;
  if (starts.empty())
    for (int b = 0; b <= n; b += chunk) starts.push_back(std::min(b, n));
  if (starts.back() != n) starts.push_back(n);
  const int nchunks = static_cast<int>(starts.size()) - 1;
  int width = 1;  // shared-memory window: the longest unit
  for (int c = 0; c < nchunks; ++c) width = std::max(width, starts[c + 1] - starts[c]);
  int ring = 0;
  if (ring_cap > 0) {
    ring = 64;
    while (ring < width && ring < ring_cap) ring *= 2;
  }
  const int win = ring > 0 ? ring : width;  // first import slot
  // a dependency reads the ring when it is in the unit and (with wrapping) fewer
  // than ring - 32 positions back
  auto in_ring = [&](int p, int qe, int base, int len) {
    return qe >= base && (ring == 0 || len <= ring || p - qe < ring - 32);
  };
  std::vector<int> cptr((size_t)nchunks + 1, 0), q, slot((size_t)std::max(ndep, 1) + 16, -1), ext;
  std::vector<int> ustage, segs, useg;
  std::vector<int4> stab;  // two per stage: {lo, hi, e0, e1}, {first segment, end segment, 0, 0}
  int max_imp = 0;
  bool stages_fit = true;
  for (int c = 0; c < nchunks; ++c) {
    const int base = starts[c], end = starts[c + 1], len = end - base;
    ext.clear();
    for (int p = base; p < end; ++p)
      for (int e = ptr[p]; e < ptr[p + 1]; ++e)
        if (!in_ring(p, pos[e], base, len)) ext.push_back(pos[e]);
    std::sort(ext.begin(), ext.end());
    ext.erase(std::unique(ext.begin(), ext.end()), ext.end());
    for (int p = base; p < end; ++p)
      for (int e = ptr[p]; e < ptr[p + 1]; ++e) {
        const int qe = pos[e];
        slot[e] = in_ring(p, qe, base, len)
                      ? (ring > 0 ? (qe - base) & (ring - 1) : qe - base)
                      : win + static_cast<int>(std::lower_bound(ext.begin(), ext.end(), qe) - ext.begin());
      }
    q.insert(q.end(), ext.begin(), ext.end());
    cptr[c + 1] = static_cast<int>(q.size());
    max_imp = std::max(max_imp, static_cast<int>(ext.size()));
    if (ring > 0) {
      // segments: runs of at most 32 consecutive positions (one lane each) whose
      // lists fit a stage buffer. (Ending runs early at level boundaries was
      // measured: no faster on 32-wide levels, slower on narrower ones.)
      useg.clear();
      int first = base;
      for (int p = base + 1; p < end; ++p) {
        if (p - first >= 32 || ptr[p + 1] - ptr[first] > emax) {
          useg.push_back(first);
          first = p;
        }
      }
      useg.push_back(first);
      // stages: runs of whole segments with at most pmax positions, emax list
      // entries and smax segments
      ustage.push_back(static_cast<int>(stab.size() / 2));
      const int sg_base = static_cast<int>(segs.size());
      const int nsu = static_cast<int>(useg.size());
      for (int i = 0; i < nsu;) {
        const int lo = useg[i];
        int j = i;
        while (j < nsu) {
          const int hi = j + 1 < nsu ? useg[j + 1] : end;
          if (hi - lo > pmax || ptr[hi] - ptr[lo] > emax || j + 1 - i > smax) break;
          ++j;
        }
        if (j == i) {  // one segment's lists exceed a stage buffer
          stages_fit = false;
          break;
        }
        const int hi = j < nsu ? useg[j] : end;
        stab.push_back(make_int4(lo, hi, ptr[lo], ptr[hi]));
        stab.push_back(make_int4(sg_base + i, sg_base + j, 0, 0));
        i = j;
      }
      segs.insert(segs.end(), useg.begin(), useg.end());
    }
  }
  t.chunk = chunk;
  t.width = width;
  t.max_imports = max_imp;
  t.ring = ring;
  t.ring_cap = ring_cap;
  t.pmax = pmax;
  t.emax = emax;
  t.stages = stages;
  t.smax = smax;
  if (ring > 0) {
    ustage.push_back(static_cast<int>(stab.size() / 2));
    segs.push_back(n);
    if (!stages_fit || unit_smem_bytes(ring, max_imp, pmax, emax, smax, stages, elem) > 220 * 1024)
      return SPTRSV_OK;  // recorded: does not fit
  } else if (imported_smem_bytes(width, max_imp, elem) > 220 * 1024) {
    return SPTRSV_OK;  // recorded: does not fit
  }
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.start), sizeof(int) * starts.size()));
  CUDA_TRY(cudaMemcpy(t.start, starts.data(), sizeof(int) * starts.size(), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.ptr), sizeof(int) * cptr.size()));
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.q), sizeof(int) * (q.empty() ? 1 : q.size())));
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.dep_slot), sizeof(int) * slot.size()));
  CUDA_TRY(cudaMemcpy(t.ptr, cptr.data(), sizeof(int) * cptr.size(), cudaMemcpyHostToDevice));
  if (!q.empty()) CUDA_TRY(cudaMemcpy(t.q, q.data(), sizeof(int) * q.size(), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(t.dep_slot, slot.data(), sizeof(int) * slot.size(), cudaMemcpyHostToDevice));
  if (ring > 0) {
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.ustage), sizeof(int) * ustage.size()));
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.stab), sizeof(int4) * std::max<size_t>(stab.size(), 2)));
    segs.resize(segs.size() + 16, n);  // bulk copies read up to 16 bytes past a slice
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&t.segs), sizeof(int) * segs.size()));
    CUDA_TRY(cudaMemcpy(t.ustage, ustage.data(), sizeof(int) * ustage.size(), cudaMemcpyHostToDevice));
    if (!stab.empty()) CUDA_TRY(cudaMemcpy(t.stab, stab.data(), sizeof(int4) * stab.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(t.segs, segs.data(), sizeof(int) * segs.size(), cudaMemcpyHostToDevice));
    t.nstages = static_cast<int>(stab.size() / 2);
    h->device_bytes += sizeof(int) * (ustage.size() + segs.size()) + sizeof(int4) * stab.size();
  }
  t.chunk = chunk;
  t.nchunks = nchunks;
  t.max_imports = max_imp;
  h->device_bytes += sizeof(int) * (starts.size() + cptr.size() + q.size() + slot.size());
  return SPTRSV_OK;
}

int build_imports(sptrsv_gb300_handle_s* h, int chunk, size_t elem, cudaStream_t s) {
  return build_import_table(h, h->imports, chunk, elem, 0, 0, 0, 0, s);
}

// Largest per-chunk entry budget whose ring of stage buffers (plus the
// shared-memory tier) fits one CTA's shared memory; 0 if none does.
constexpr size_t kSmemCap = 220 * 1024;
int fit_emax(int cmax, size_t elem, int stages, bool tier, int want) {
  int e = want;
  while (e >= 64) {
    if (staged_smem_bytes(cmax, e, elem, tier, stages) <= kSmemCap) return e;
    e = e * 3 / 4;
  }
  return 0;
}

int auto_emax(int cmax, size_t elem, int stages, bool tier) {
  // aim at ~180 KB for the whole ring so another CTA may share the SM when chunks are small
  int want = std::max(4096, 8 * cmax);
  while (want > 64 && staged_smem_bytes(cmax, want, elem, tier, stages) > 180 * 1024) want = want * 3 / 4;
  return fit_emax(cmax, elem, stages, tier, want);
}

// True when option `opt` follows the analysis-driven plan: automatic schedule
// and not set by the caller.
bool planned(const sptrsv_gb300_handle_s* h, int opt) {
  return h->sched_option == SCHED_AUTO && h->plan.valid && !(h->user_set & (1ull << opt));
}

int effective_block(const sptrsv_gb300_handle_s* h) {
  if (h->sched_option == SCHED_LEVELSET) return INT_MAX;
  if (planned(h, SPTRSV_OPTION_ORDER_BLOCK)) return h->plan.order_block;
  return h->order_block;
}

// Automatic one-rhs executor plan. Wide level sets (or a batch): global level
// order, warp-synchronous lanes, one CTA of 256 threads per SM (fewer polling
// warps, measured faster than full occupancy). Deep, narrow DAGs whose
// dependencies stay local in the natural order (>= 96 % of the entries inside
// blocks of 32 level widths): level order inside such blocks, one CTA per
// block with in-block hops through shared memory. Measured on 160k-row band
// systems with 1-16 entries per column and bands of 100-2000 rows: blocked
// orders won at 965-976 permille local (band 100: 2.84 vs 4.33 ms with two
// entries, 13.1 vs 17.5 with twelve), and lost at 925-953 (band 300: 3.83 vs
// 2.77 ms with four entries, 13.6 vs 9.1 with sixteen; band 2000 with two:
// 1.93 vs 0.40 ms), where too many hops leave the block and the wider levels
// are better spread over every SM.
//
// Lists are split over lanes only where a few lists are far longer than the
// rest: > 5 % of the entries in lists longer than max(32, 4 x the mean list
// length). Splitting pays for heavy-tailed lists (power-law backward walks:
// 2.19 vs 32.5 ms at 4M rows, 63 vs 301 ms at 1M) and costs where most lists
// are long and alike, since a warp then holds fewer unknowns and pays suffix
// sums (band systems with 30-100 entries per row, power-law forward walks:
// 1.5-1.9x slower split, e.g. 243 vs 128 ms on a 2M-row band of width 500).
//
// Residency in level order follows the average level width: one CTA of 256
// threads per SM below 1,536 unknowns per level (fewer lanes polling ahead of
// the wave: 1M-row band 1.109 vs 1.139 ms, 500k-row band 2.21 vs 2.68 ms),
// two up to 8,192 (4M-row power-law 1.68 vs 1.76 ms forward, 2.19 vs 2.60
// backward), three beyond (a 4M-row band with 17,468 per level 0.51 vs 0.60).
double long_share(const std::vector<int>& ptr, int cut) {
  long long all = 0, lng = 0;
  for (size_t i = 0; i + 1 < ptr.size(); ++i) {
    const int c = ptr[i + 1] - ptr[i] - 1;  // entries without the diagonal
    if (c <= 0) continue;
    all += c;
    if (c > cut) lng += c;
  }
  return all ? static_cast<double>(lng) / static_cast<double>(all) : 0.0;
}

int make_plan(sptrsv_gb300_handle_s* h, const std::vector<int>& row_ptr, cudaStream_t s) {
  auto& P = h->plan;
  P = sptrsv_gb300_handle_s::AutoPlan();
  const int n = h->n, nnz = h->nnz, nl = h->nlevels;
  if (n > 0) {
    std::vector<int> col_ptr((size_t)n + 1);
    CUDA_TRY(cudaMemcpyAsync(col_ptr.data(), h->csc_ptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    const int cut = std::max<int>(32, static_cast<int>(4.0 * (double)(nnz - n) / (double)n));
    P.split_fwd = long_share(row_ptr, cut) > 0.05 ? 32 : 0;
    P.split_adj = long_share(col_ptr, cut) > 0.05 ? 8 : 0;  // the reverse walk measured best with short pieces
    if (h->batch_count == 1 && nl > 0) {
      const long long width = ((long long)n + nl - 1) / nl;
      P.ctas = width < 1536 ? 1 : (width < 8192 ? 2 : 3);
    }
    if (nnz > n && (long long)(nnz - n) <= 3LL * (long long)n) {
      unsigned long long* d_count = nullptr;
      CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&d_count), 2 * sizeof(unsigned long long), s));
      CUDA_TRY(cudaMemsetAsync(d_count, 0, 2 * sizeof(unsigned long long), s));
      CUDA_TRY(launch_coarrival(h->csr_ptr, h->csr_col, h->depth, n, d_count, s));
      unsigned long long count[2] = {0, 0};
      CUDA_TRY(cudaMemcpyAsync(count, d_count, sizeof(count), cudaMemcpyDeviceToHost, s));
      CUDA_TRY(cudaStreamSynchronize(s));
      CUDA_TRY(cudaFree(d_count));
      P.coarrive = count[1] ? static_cast<double>(count[0]) / static_cast<double>(count[1]) : 0.0;
    }
  }
  if (n > 0 && nl >= 256 && h->batch_count == 1 && nnz > n) {
    const long long width = ((long long)n + nl - 1) / nl;
    if (width <= 4096) {
      const int blk = static_cast<int>(std::min<long long>(24576, std::max<long long>(2048, (32 * width + 31) / 32 * 32)));
      unsigned long long* d_count = nullptr;
      CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&d_count), sizeof(unsigned long long), s));
      CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), s));
      CUDA_TRY(launch_block_locality(h->csc_row, h->csc_col, nnz, n, blk, h->substitution == 1, d_count, s));
      unsigned long long count = 0;
      CUDA_TRY(cudaMemcpyAsync(&count, d_count, sizeof(count), cudaMemcpyDeviceToHost, s));
      CUDA_TRY(cudaStreamSynchronize(s));
      CUDA_TRY(cudaFree(d_count));
      P.locality = static_cast<double>(count) / static_cast<double>(nnz - n);
      if (P.locality >= 0.96) {
        P.order_block = blk;
        P.chunk = blk;
        P.block = 128;
        P.ctas = 0;
        P.backoff = 0;
      }
    }
  }
  P.valid = true;
  return SPTRSV_OK;
}

int ensure_layout(sptrsv_gb300_handle_s* h, cudaStream_t s) {
  const int want = effective_block(h);
  const int have = h->layout_block;
  const bool same = ((want >= h->n && have >= h->n) || want == have) &&
                    (want_stretch(h, want) ? 1 : 0) == h->layout_stretched;
  if (same && h->layout.perm != nullptr) return SPTRSV_OK;
  if (h->n == 0 && have >= 0) return SPTRSV_OK;
  return build_layout(h, want, s);
}

template <typename TV, typename T>
int stage(sptrsv_gb300_handle_s* h, Values<T>& V, const TV* val, cudaStream_t s, bool check) {
  const Layout& L = h->layout;
  if (!V.dep_val) {
    ST_TRY(dev_alloc(h, &V.dep_val, L.ndep));
    ST_TRY(dev_alloc(h, &V.dep_w, L.ndep));
    ST_TRY(dev_alloc(h, &V.out_w, L.ndep));
    ST_TRY(dev_alloc(h, &V.out_val, L.ndep));
    ST_TRY(dev_alloc(h, &V.diag, L.n));
    ST_TRY(dev_alloc(h, &V.rcp, L.n));
  }
  if (check) CUDA_TRY(cudaMemsetAsync(h->flags, 0, sizeof(int), s));
  CUDA_TRY(launch_stage_values<TV, T>(L, val, V, h->flags, s));
  if (check) {
    int f = 0;
    ST_TRY(read_flags(h, s, &f));
    if (f & SF_ZERO_DIAG) return SPTRSV_ERR_BAD_STRUCTURE;
  }
  return SPTRSV_OK;
}

int stage_values(sptrsv_gb300_handle_s* h, const void* d_val, int dtype, cudaStream_t s, bool check) {
  if (dtype == SPTRSV_DTYPE_F64) {
    ST_TRY(stage<double, double>(h, h->v64, static_cast<const double*>(d_val), s, check));
    ST_TRY(stage<double, float>(h, h->v32, static_cast<const double*>(d_val), s, false));
    h->staged64 = h->staged32 = true;
    h->wsplit_ok = false;
  } else if (dtype == SPTRSV_DTYPE_F32) {
    ST_TRY(stage<float, float>(h, h->v32, static_cast<const float*>(d_val), s, check));
    h->staged32 = true;
    h->staged64 = false;
  } else {
    return SPTRSV_ERR_INVALID;
  }
  return SPTRSV_OK;
}

// Unit pipeline tables for this order block (built on first use); true when
// they exist and the CTA's shared memory holds them for element type T.
template <typename T>
bool pipe_ready(sptrsv_gb300_handle_s* h, int chunk, cudaStream_t s) {
  const int ring_cap = h->pipe_option == 1 ? 8192 : h->pipe_option;
  const int emax = h->emax_option > 0 ? h->emax_option : 2048;
  const int pmax = std::min(512, std::max(32, (emax / 4) & ~31));  // at most the kernel's 512
  const int stages = (h->user_set & (1ull << SPTRSV_OPTION_STAGES)) ? h->stages_option : 3;
  ImportTable& t = h->pipe;
  if (t.chunk != chunk || t.ring_cap != ring_cap || t.emax != emax || t.pmax != pmax || t.stages != stages) {
    if (build_import_table(h, t, chunk, sizeof(T), ring_cap, pmax, emax, stages, s) != SPTRSV_OK) {
      free_imports(t);
      return false;
    }
  }
  return t.ustage != nullptr &&
         unit_smem_bytes(t.ring, t.max_imports, t.pmax, t.emax, t.smax, t.stages, sizeof(T)) <= 220 * 1024;
}

// Dependencies a lane loads per lockstep iteration (one rhs) when the caller
// left it open. Forward walks over lists averaging more than 3 entries: one
// (the shortest iteration; ready-ordered lists let the earlier entries land
// long before the last). Shorter lists: two when at least half of the unknowns
// have two or more dependencies on the level just before their own, which
// land in the same iteration (the mesh triangle in level order: 16.1 ms with
// two, 18.6 with one), else one (160k-row bands with 1 / 2 entries per column
// 0.087 / 1.79 ms with two, 0.072 / 1.42 with one; a 1M-row band with 3
// entries 6.42 vs 5.37 ms; a 20k-row chain on the importer executor 5.24 vs
// 4.02 ms). Split lists and the transposed walk: two.
int auto_wsync_batch(const sptrsv_gb300_handle_s* h, bool adj, bool split) {
  if (adj || split) return 2;
  if ((long long)(h->nnz - h->n) > 3LL * (long long)h->n) return 1;
  return h->plan.coarrive >= 0.5 ? 2 : 1;
}

// Automatic executor settings for a request.
ExecConfig pick_config(const sptrsv_gb300_handle_s* h, int rhs) {
  ExecConfig c = h->cfg;
  c.sched = h->sched_option == SCHED_AUTO ? SCHED_PULL : h->sched_option;
  c.lanes = h->lanes_option > 0 ? h->lanes_option : 1;
  c.block = h->block_option > 0 ? h->block_option : 256;
  // one-rhs: one unknown per consumer thread per chunk; many rhs: one unknown per
  // lane group (the group width the multi-rhs executors pick for this rhs)
  c.opt = h->opt_option;
  c.rhs_tile = h->rhs_tile_option;
  const int group = multi_group(rhs, c.rhs_tile, nullptr);
  c.chunk = h->chunk_option > 0 ? h->chunk_option : (rhs == 1 ? 224 : std::max(1, c.block / group));
  c.sleep_max = static_cast<unsigned>(h->backoff_ns);
  c.ctas_per_sm = h->ctas_per_sm;
  c.staged = h->staged;
  c.emax = h->emax_option;
  c.stages = h->stages_option;
  c.wsync = h->wsync;
  c.split = h->split;
  c.wsync_batch = h->wsync_batch;  // 0: chosen per solve (solve_typed)
  if (rhs == 1 && h->sched_option == SCHED_AUTO && h->plan.valid) {
    if (planned(h, SPTRSV_OPTION_CHUNK)) c.chunk = h->plan.chunk;
    if (planned(h, SPTRSV_OPTION_BLOCK)) c.block = h->plan.block;
    if (planned(h, SPTRSV_OPTION_CTAS_PER_SM)) c.ctas_per_sm = h->plan.ctas;
    if (planned(h, SPTRSV_OPTION_BACKOFF_NS)) c.sleep_max = static_cast<unsigned>(h->plan.backoff);
    if (planned(h, SPTRSV_OPTION_STAGED)) c.staged = h->plan.staged;
    if (planned(h, SPTRSV_OPTION_WARP_SYNC)) c.wsync = h->plan.wsync;
  } else if (rhs > 1 && h->sched_option == SCHED_AUTO && h->plan.valid) {
    // many rhs: warp-synchronous lane groups (up to 64 rhs), one unknown per group
    // per chunk; two CTAs per SM up to 8 rhs (the 1M-row band system at 4 / 8 rhs:
    // 1.025 / 1.027 ms against 1.073 / 1.064 with one or with every CTA that
    // fits), every CTA that fits beyond (16 rhs: 1.13 ms against 1.45 with two)
    if (planned(h, SPTRSV_OPTION_WARP_SYNC)) c.wsync = rhs <= 64 ? 1 : 0;
    if (planned(h, SPTRSV_OPTION_CTAS_PER_SM)) c.ctas_per_sm = rhs <= 8 ? 2 : 0;
    if (planned(h, SPTRSV_OPTION_BACKOFF_NS)) c.sleep_max = 0u;  // spinning measured 1-3 % faster at 16 and 64 rhs
    // a blocked layout: one CTA per order block (small chunks would hand the
    // blocks out one after another); the shared-memory tier does not fit there
    if (planned(h, SPTRSV_OPTION_CHUNK) && h->layout_block > 0 && h->layout_block < h->n) {
      c.chunk = h->layout_block;
      c.ctas_per_sm = 0;
      c.sleep_max = 0u;
    }
  }
  return c;
}

template <typename T>
int solve_typed(sptrsv_gb300_handle_s* h, const Values<T>& V, int rhs, int layout, const T* b, T* x,
                cudaStream_t s, const AdjointArgs<T>* adj = nullptr, bool allow_check = true) {
  const int n = h->n;
  VecView<T> v{};
  v.b = b;
  v.x = x;
  if (layout == SPTRSV_LAYOUT_ROW_MAJOR) {
    v.b_si = v.x_si = rhs;
    v.b_sk = v.x_sk = 1;
  } else {
    v.b_si = v.x_si = 1;
    v.b_sk = v.x_sk = n;
  }
  ExecConfig c = pick_config(h, rhs);
  if (adj) c.sched = SCHED_PULL;  // the transposed solve walks the analysis in reverse with the pull executor
  h->last_sched = c.sched;
  h->last_pipe = false;
  const size_t elems = (size_t)n * (size_t)rhs;
  if (c.sched == SCHED_PUSH) {
    ST_TRY(ensure_buf(h, h->left_sum, elems * sizeof(T), 1, s));
    ST_TRY(ensure_buf(h, h->counters, (size_t)n * sizeof(unsigned), 1, s));
  } else {
    ST_TRY(ensure_buf(h, h->xw, elems * sizeof(T), 0, s));
    if (c.sched != SCHED_LEVELSET) CUDA_TRY(cudaMemsetAsync(h->xw.p, 0xFF, elems * sizeof(T), s));
  }
  if (h->profile) {
    if (!h->ev_exec[0]) {
      CUDA_TRY(cudaEventCreate(&h->ev_exec[0]));
      CUDA_TRY(cudaEventCreate(&h->ev_exec[1]));
    }
    CUDA_TRY(cudaEventRecord(h->ev_exec[0], s));
  }
  if (c.sched == SCHED_PUSH) {
    CUDA_TRY(launch_push<T>(h->layout, V, rhs, v, static_cast<T*>(h->left_sum.p),
                            static_cast<unsigned*>(h->counters.p), h->ctl, c, timeout_ns(h), h->num_sms, s));
  } else if (c.sched == SCHED_LEVELSET) {
    CUDA_TRY(launch_levelset<T>(h->layout, V, rhs, v, static_cast<T*>(h->xw.p), h->ctl, c, timeout_ns(h), s));
  } else if (rhs == 1 && c.staged &&
             (c.emax > 0 ? fit_emax(c.chunk, sizeof(T), c.stages, c.smem_tier, c.emax) == c.emax
                         : auto_emax(c.chunk, sizeof(T), c.stages, c.smem_tier) > 0)) {
    const int emax = c.emax > 0 ? c.emax : auto_emax(c.chunk, sizeof(T), c.stages, c.smem_tier);
    ST_TRY(ensure_table(h, adj != nullptr, c.chunk, emax));
    CUDA_TRY(launch_pull_staged<T>(h->layout, V, adj ? h->tab_adj : h->tab_fwd, v, static_cast<T*>(h->xw.p), h->ctl,
                                   c, timeout_ns(h), h->num_sms, s, adj));
  } else if (rhs == 1 && c.wsync && !c.exact && !adj && h->pipe_option && h->layout_block < n &&
             c.chunk == h->layout_block && c.smem_tier && pipe_ready<T>(h, c.chunk, s)) {
    // blocked layout: one consumer warp per unit reads everything from shared
    // memory; a loader warp streams the unit's stages, an importer warp its
    // external dependencies
    if (c.wsync_batch == 0) c.wsync_batch = 2;
    ST_TRY(ensure_buf(h, h->c0, ((size_t)n + 16) * sizeof(T), 0, s));
    CUDA_TRY(launch_pull_unit<T>(h->layout, V, v, static_cast<T*>(h->xw.p), static_cast<T*>(h->c0.p), h->ctl, c,
                                 timeout_ns(h), h->num_sms, s, h->pipe));
    h->last_pipe = true;
  } else if (rhs == 1 && c.wsync && !c.exact && !adj && h->import_option && h->layout_block < n &&
             c.chunk == h->layout_block && c.smem_tier &&
             !(c.split > 0 && h->max_dep_cnt > c.split) &&
             (h->imports.chunk == c.chunk || build_imports(h, c.chunk, sizeof(T), s) == SPTRSV_OK) &&
             h->imports.ptr != nullptr &&
             imported_smem_bytes(h->imports.width, h->imports.max_imports, sizeof(T)) <= 220 * 1024) {
    // blocked layout: an importer warp per CTA brings the chunk's external dependencies
    // into shared memory
    if (c.wsync_batch == 0) c.wsync_batch = auto_wsync_batch(h, false, false);
    c.one_batch = h->max_dep_cnt <= c.wsync_batch ? 1 : 0;
    CUDA_TRY(launch_pull_imported<T>(h->layout, V, v, static_cast<T*>(h->xw.p), h->ctl, c, timeout_ns(h),
                                     h->num_sms, s, h->imports));
  } else {
    const PieceTable* pc = nullptr;
    if (rhs == 1 && planned(h, SPTRSV_OPTION_SPLIT)) c.split = adj ? h->plan.split_adj : h->plan.split_fwd;
    const int longest = adj ? h->max_out_cnt : h->max_dep_cnt;
    if (rhs == 1 && c.wsync && !c.exact && c.split > 0 && longest > c.split && !(adj && adj->grad)) {
      ST_TRY(ensure_pieces(h, adj != nullptr, c.split, c.chunk, s));
      pc = adj ? &h->pc_adj : &h->pc_fwd;
    }
    if (c.wsync_batch == 0) c.wsync_batch = auto_wsync_batch(h, adj != nullptr, pc != nullptr);
    CUDA_TRY(launch_pull<T>(h->layout, V, rhs, v, static_cast<T*>(h->xw.p), h->ctl, c, timeout_ns(h), h->num_sms,
                            s, adj, pc));
  }
  if (h->profile) {
    CUDA_TRY(cudaEventRecord(h->ev_exec[1], s));
    h->ev_recorded = true;
  }
  if (h->sync_check && allow_check) return check_device(h, s);
  return SPTRSV_OK;
}

// Control blocks (ticket, done counter, error code) of the kernel-level
// executor, one per (device, stream): calls on one stream are ordered by the
// stream, and calls on different streams, from any host threads, never share
// a block. A block is allocated at the first call on its stream and kept
// until exit (a later stream that reuses the handle value reuses the block,
// which is as safe: the block is idle between calls on that stream).
std::mutex g_raw_mutex;
std::map<std::pair<int, cudaStream_t>, DeviceCtl*> g_raw_ctl;

int raw_ctl(cudaStream_t s, DeviceCtl** out) {
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_raw_mutex);
  DeviceCtl*& c = g_raw_ctl[std::make_pair(dev, s)];
  if (!c) {
    DeviceCtl* fresh = nullptr;
    if (cudaMalloc(reinterpret_cast<void**>(&fresh), sizeof(DeviceCtl)) != cudaSuccess) {
      cudaGetLastError();
      g_raw_ctl.erase(std::make_pair(dev, s));
      return SPTRSV_ERR_OOM;
    }
    CUDA_TRY(cudaMemset(fresh, 0, sizeof(DeviceCtl)));
    c = fresh;
  }
  *out = c;
  return SPTRSV_OK;
}

}  // namespace

extern "C" {

const char* sptrsv_gb300_status_string(int status) {
  switch (status) {
    case SPTRSV_OK: return "ok";
    case SPTRSV_ERR_NOT_SQUARE: return "matrix is not square";
    case SPTRSV_ERR_BAD_STRUCTURE: return "malformed triangular CSC structure or zero diagonal";
    case SPTRSV_ERR_INVALID: return "invalid argument";
    case SPTRSV_ERR_CUDA: return "CUDA runtime error";
    case SPTRSV_ERR_TIMEOUT: return "bounded device wait ran out";
    case SPTRSV_ERR_OOM: return "device out of memory";
    case SPTRSV_ERR_STATE: return "call out of order";
    case SPTRSV_ERR_NOT_CONVERGED: return "iterative refinement did not converge";
    case SPTRSV_ERR_UNSUPPORTED: return "unsupported request";
    default: return "unknown status";
  }
}

int sptrsv_gb300_version(void) { return SPTRSV_GB300_VERSION; }

void sptrsv_gb300_set_verbose(int verbose) { g_verbose = verbose; }
void sptrsv_gb300_set_bench_repeat(int repeat) { g_bench_repeat = repeat > 0 ? repeat : 1; }

int sptrsv_gb300_create(sptrsv_handle_t* handle) {
  if (!handle) return SPTRSV_ERR_INVALID;
  *handle = nullptr;
  auto* h = new (std::nothrow) sptrsv_gb300_handle_s();
  if (!h) return SPTRSV_ERR_OOM;
  cudaError_t e = cudaGetDevice(&h->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&h->ctl), sizeof(DeviceCtl));
  if (e == cudaSuccess) e = cudaMemset(h->ctl, 0, sizeof(DeviceCtl));
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&h->flags), sizeof(int));
  if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&h->host_pinned), 4 * sizeof(int));
  if (e != cudaSuccess) {
    if (h->ctl) cudaFree(h->ctl);
    if (h->flags) cudaFree(h->flags);
    delete h;
    return map_cuda_error(e);
  }
  *handle = h;
  return SPTRSV_OK;
}

int sptrsv_gb300_destroy(sptrsv_handle_t h) {
  if (!h) return SPTRSV_ERR_INVALID;
  cudaDeviceSynchronize();
  free_analysis(h);
  free_buf(h->xw);
  free_buf(h->left_sum);
  free_buf(h->counters);
  free_buf(h->r32);
  free_buf(h->d32);
  free_buf(h->stats);
  free_buf(h->tb);
  free_buf(h->tx);
  free_buf(h->c0);
  free_buf(h->wsplit);
  if (h->ctl) cudaFree(h->ctl);
  if (h->flags) cudaFree(h->flags);
  if (h->host_pinned) cudaFreeHost(h->host_pinned);
  if (h->ev_exec[0]) cudaEventDestroy(h->ev_exec[0]);
  if (h->ev_exec[1]) cudaEventDestroy(h->ev_exec[1]);
  delete h;
  return SPTRSV_OK;
}

static int set_option_value(sptrsv_handle_t h, int option, long long value);

int sptrsv_gb300_set_option(sptrsv_handle_t h, int option, long long value) {
  if (!h) return SPTRSV_ERR_INVALID;
  const int st = set_option_value(h, option, value);
  if (st == SPTRSV_OK && option >= 0 && option < 64) h->user_set |= 1ull << option;
  return st;
}

static int set_option_value(sptrsv_handle_t h, int option, long long value) {
  switch (option) {
    case SPTRSV_OPTION_SCHEDULE:
      if (value < SCHED_AUTO || value > SCHED_LEVELSET) return SPTRSV_ERR_INVALID;
      h->sched_option = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_LANES:
      if (!(value == 0 || value == 1 || value == 2 || value == 4 || value == 8 || value == 16 || value == 32))
        return SPTRSV_ERR_INVALID;
      h->lanes_option = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_CHUNK:
      if (value < 0 || value > (1 << 20)) return SPTRSV_ERR_INVALID;
      h->chunk_option = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_SMEM_TIER:
      h->cfg.smem_tier = value != 0;
      return SPTRSV_OK;
    case SPTRSV_OPTION_EXACT:
      h->cfg.exact = value != 0;
      return SPTRSV_OK;
    case SPTRSV_OPTION_ORDER_BLOCK:
      if (value < 1) return SPTRSV_ERR_INVALID;
      h->order_block = value > INT_MAX ? INT_MAX : static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_TIMEOUT_MS:
      if (value < 1) return SPTRSV_ERR_INVALID;
      h->timeout_ms = value;
      return SPTRSV_OK;
    case SPTRSV_OPTION_SYNC_CHECK:
      h->sync_check = value != 0;
      return SPTRSV_OK;
    case SPTRSV_OPTION_PROFILE:
      h->profile = value != 0;
      return SPTRSV_OK;
    case SPTRSV_OPTION_BLOCK:
      if (!(value == 0 || value == 64 || value == 128 || value == 256)) return SPTRSV_ERR_INVALID;
      h->block_option = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_BACKOFF_NS:
      if (value < 0 || value > 100000) return SPTRSV_ERR_INVALID;
      h->backoff_ns = value;
      return SPTRSV_OK;
    case SPTRSV_OPTION_CTAS_PER_SM:
      if (value < 0 || value > 32) return SPTRSV_ERR_INVALID;
      h->ctas_per_sm = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_STAGED:
      h->staged = value != 0;
      return SPTRSV_OK;
    case SPTRSV_OPTION_STAGE_ENTRIES:
      if (value < 0 || value > (1 << 16)) return SPTRSV_ERR_INVALID;
      h->emax_option = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_STAGES:
      if (value < 2 || value > 4) return SPTRSV_ERR_INVALID;
      h->stages_option = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_FUSED_GRAD:
      h->fused_grad = value != 0;
      return SPTRSV_OK;
    case SPTRSV_OPTION_WARP_SYNC:
      h->wsync = value != 0;
      return SPTRSV_OK;
    case SPTRSV_OPTION_SPLIT:
      if (value < 0 || (value > 0 && value < 4) || value > (1 << 20)) return SPTRSV_ERR_INVALID;
      h->split = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_WSYNC_BATCH:
      if (!(value == 0 || value == 1 || value == 2 || value == 4)) return SPTRSV_ERR_INVALID;
      h->wsync_batch = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_IMPORT:
      h->import_option = value != 0;
      return SPTRSV_OK;
    case SPTRSV_OPTION_UNIT_PIPELINE:
      if (!(value == 0 || value == 1 || (value >= 128 && value <= 8192 && (value & (value - 1)) == 0)))
        return SPTRSV_ERR_INVALID;
      h->pipe_option = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_FUSED_REFINE:
      if (value < 0 || value > 2) return SPTRSV_ERR_INVALID;
      h->fused_refine = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_OPT:
      if (value < SPTRSV_OPT_WARP_NNZ || value > SPTRSV_OPT_WARP_AUTO) return SPTRSV_ERR_INVALID;
      h->opt_option = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_RHS_TILE:
      if (!(value == 0 || value == 1 || value == 2 || value == 4)) return SPTRSV_ERR_INVALID;
      h->rhs_tile_option = static_cast<int>(value);
      return SPTRSV_OK;
    case SPTRSV_OPTION_STRETCH:
      h->stretch_option = value != 0;
      return SPTRSV_OK;
    default:
      return SPTRSV_ERR_INVALID;
  }
}

int sptrsv_gb300_get_option(sptrsv_handle_t h, int option, long long* value) {
  if (!h || !value) return SPTRSV_ERR_INVALID;
  switch (option) {
    case SPTRSV_OPTION_SCHEDULE: *value = h->sched_option; break;
    case SPTRSV_OPTION_LANES: *value = h->lanes_option; break;
    case SPTRSV_OPTION_CHUNK: *value = h->chunk_option; break;
    case SPTRSV_OPTION_SMEM_TIER: *value = h->cfg.smem_tier; break;
    case SPTRSV_OPTION_EXACT: *value = h->cfg.exact; break;
    case SPTRSV_OPTION_ORDER_BLOCK: *value = h->order_block; break;
    case SPTRSV_OPTION_TIMEOUT_MS: *value = h->timeout_ms; break;
    case SPTRSV_OPTION_SYNC_CHECK: *value = h->sync_check; break;
    case SPTRSV_OPTION_PROFILE: *value = h->profile; break;
    case SPTRSV_OPTION_BLOCK: *value = h->block_option; break;
    case SPTRSV_OPTION_BACKOFF_NS: *value = h->backoff_ns; break;
    case SPTRSV_OPTION_CTAS_PER_SM: *value = h->ctas_per_sm; break;
    case SPTRSV_OPTION_STAGED: *value = h->staged; break;
    case SPTRSV_OPTION_STAGE_ENTRIES: *value = h->emax_option; break;
    case SPTRSV_OPTION_STAGES: *value = h->stages_option; break;
    case SPTRSV_OPTION_FUSED_GRAD: *value = h->fused_grad; break;
    case SPTRSV_OPTION_WARP_SYNC: *value = h->wsync; break;
    case SPTRSV_OPTION_SPLIT: *value = h->split; break;
    case SPTRSV_OPTION_WSYNC_BATCH: *value = h->wsync_batch; break;
    case SPTRSV_OPTION_IMPORT: *value = h->import_option; break;
    case SPTRSV_OPTION_UNIT_PIPELINE: *value = h->pipe_option; break;
    case SPTRSV_OPTION_FUSED_REFINE: *value = h->fused_refine; break;
    case SPTRSV_OPTION_OPT: *value = h->opt_option; break;
    case SPTRSV_OPTION_RHS_TILE: *value = h->rhs_tile_option; break;
    case SPTRSV_OPTION_STRETCH: *value = h->stretch_option; break;
    default: return SPTRSV_ERR_INVALID;
  }
  return SPTRSV_OK;
}

}  // extern "C"

namespace {
// The analysis pipeline on a CSC structure already described by h->n, nnz,
// substitution and (for batches) the system arrays.
int analyse_core(sptrsv_handle_t h, const int* d_colPtr, const int* d_rowIdx, cudaStream_t s) {
  const int n = h->n, nnz = h->nnz, substitution = h->substitution;
  (void)substitution;
  const SysDesc sd0 = sys_desc(h);
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  CUDA_TRY(cudaEventRecord(e0, s));

  // 1. structure validation (pointers first, then rows)
  CUDA_TRY(cudaMemsetAsync(h->flags, 0, sizeof(int), s));
  CUDA_TRY(launch_validate_ptr(d_colPtr, n, nnz, h->flags, s));
  int f = 0;
  ST_TRY(read_flags(h, s, &f));
  if (f) return SPTRSV_ERR_BAD_STRUCTURE;
  CUDA_TRY(launch_validate_rows(d_colPtr, d_rowIdx, n, nnz, sd0, h->flags, s));
  ST_TRY(read_flags(h, s, &f));
  if (f) return SPTRSV_ERR_BAD_STRUCTURE;

  // 2. owned copy of the structure, in-degree analyser
  ST_TRY(dev_alloc(h, &h->csc_ptr, (size_t)n + 1));
  ST_TRY(dev_alloc(h, &h->csc_row, nnz));
  CUDA_TRY(cudaMemcpyAsync(h->csc_ptr, d_colPtr, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToDevice, s));
  if (nnz) CUDA_TRY(cudaMemcpyAsync(h->csc_row, d_rowIdx, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToDevice, s));
  ST_TRY(dev_alloc(h, &h->in_degree, n));
  CUDA_TRY(cudaMemsetAsync(h->in_degree, 0, sizeof(int) * (size_t)(n > 0 ? n : 1), s));
  CUDA_TRY(launch_in_degree(h->csc_row, n, nnz, h->in_degree, s));

  // 3. CSR transpose by a stable sort of the CSC entries on their row
  ST_TRY(dev_alloc(h, &h->csr_ptr, (size_t)n + 1));
  ST_TRY(dev_alloc(h, &h->csr_col, nnz));
  ST_TRY(dev_alloc(h, &h->csr_src, nnz));
  CUDA_TRY(exclusive_scan_int(h->in_degree, h->csr_ptr, n, true, s));
  if (nnz > 0) {
    unsigned *keys = nullptr, *keys_sorted = nullptr;
    int *iota = nullptr, *col_of = nullptr;
    void* temp = nullptr;
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&keys), sizeof(unsigned) * nnz, s));
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&keys_sorted), sizeof(unsigned) * nnz, s));
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&iota), sizeof(int) * nnz, s));
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&col_of), sizeof(int) * nnz, s));
    CUDA_TRY(cudaMallocAsync(&temp, radix_sort_temp_bytes(nnz), s));
    CUDA_TRY(launch_copy_keys(h->csc_row, keys, nnz, s));
    CUDA_TRY(launch_iota(iota, nnz, 0, 1, s));
    CUDA_TRY(radix_sort_pairs(keys, iota, keys_sorted, h->csr_src, nnz, bits_for(n - 1), temp, s));
    CUDA_TRY(launch_expand_cols(h->csc_ptr, n, col_of, s));
    CUDA_TRY(launch_gather_int(col_of, h->csr_src, h->csr_col, nnz, s));
    ST_TRY(dev_alloc(h, &h->csc_col, nnz));
    CUDA_TRY(cudaMemcpyAsync(h->csc_col, col_of, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToDevice, s));
    CUDA_TRY(cudaFreeAsync(keys, s));
    CUDA_TRY(cudaFreeAsync(keys_sorted, s));
    CUDA_TRY(cudaFreeAsync(iota, s));
    CUDA_TRY(cudaFreeAsync(col_of, s));
    CUDA_TRY(cudaFreeAsync(temp, s));
  }

  // 4. level sets
  ST_TRY(dev_alloc(h, &h->depth, n));
  h->nlevels = 0;
  h->level_sizes_host.clear();
  if (n > 0) {
    int *cnt = nullptr, *fa = nullptr, *fb = nullptr, *sizes = nullptr;
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&cnt), sizeof(int) * n, s));
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&fa), sizeof(int) * n, s));
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&fb), sizeof(int) * n, s));
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&sizes), sizeof(int) * ((size_t)n + 5), s));
    CUDA_TRY(launch_levels(h->csc_ptr, h->csc_row, h->in_degree, n, cnt, fa, fb, h->depth, sizes, h->ctl,
                           timeout_ns(h), s));
    int code = 0;
    ST_TRY(read_device_code(h, s, &code));
    if (code != DEV_OK) {
      ST_TRY(reset_after_failure(h, s));
      return SPTRSV_ERR_TIMEOUT;
    }
    int nl = 0;
    CUDA_TRY(cudaMemcpyAsync(h->host_pinned + 2, sizes + n + 1 + 3, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    nl = h->host_pinned[2];
    if (nl < 1 || nl > n) return SPTRSV_ERR_BAD_STRUCTURE;
    h->level_sizes_host.resize(nl);
    CUDA_TRY(cudaMemcpy(h->level_sizes_host.data(), sizes, sizeof(int) * nl, cudaMemcpyDeviceToHost));
    long long total = 0;
    for (int l = 0; l < nl; ++l) total += h->level_sizes_host[l];
    if (total != n) return SPTRSV_ERR_BAD_STRUCTURE;
    h->nlevels = nl;
    // findlevel_csc statistics (findlevel.h:123-136)
    int lo = h->level_sizes_host[0], hi = lo;
    for (int l = 1; l < nl; ++l) {
      const int c = h->level_sizes_host[l];
      if (c > hi) hi = c;
      else if (c < lo) lo = c;
    }
    h->pmin = lo;
    h->pmax = hi;
    h->pavg = n / nl;
    CUDA_TRY(cudaFreeAsync(cnt, s));
    CUDA_TRY(cudaFreeAsync(fa, s));
    CUDA_TRY(cudaFreeAsync(fb, s));
    CUDA_TRY(cudaFreeAsync(sizes, s));

    // level items: rows sorted by (level, row)
    ST_TRY(dev_alloc(h, &h->level_item, n));
    ST_TRY(dev_alloc(h, &h->level_ptr_nat, (size_t)nl + 1));
    std::vector<int> lp(nl + 1, 0);
    for (int l = 0; l < nl; ++l) lp[l + 1] = lp[l] + h->level_sizes_host[l];
    CUDA_TRY(cudaMemcpyAsync(h->level_ptr_nat, lp.data(), sizeof(int) * (nl + 1), cudaMemcpyHostToDevice, s));
    unsigned *keys = nullptr, *keys_sorted = nullptr;
    int* iota = nullptr;
    void* temp = nullptr;
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&keys), sizeof(unsigned) * n, s));
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&keys_sorted), sizeof(unsigned) * n, s));
    CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&iota), sizeof(int) * n, s));
    CUDA_TRY(cudaMallocAsync(&temp, radix_sort_temp_bytes(n), s));
    CUDA_TRY(launch_iota(iota, n, 0, 1, s));
    CUDA_TRY(launch_schedule_keys(iota, h->depth, n, SysDesc(), 1, 0, keys, s));
    CUDA_TRY(radix_sort_pairs(keys, iota, keys_sorted, h->level_item, n, bits_for(nl - 1), temp, s));
    CUDA_TRY(cudaFreeAsync(keys, s));
    CUDA_TRY(cudaFreeAsync(keys_sorted, s));
    CUDA_TRY(cudaFreeAsync(iota, s));
    CUDA_TRY(cudaFreeAsync(temp, s));
  }
  // max in-degree, from the CSR row pointers
  h->max_in_degree = 0;
  std::vector<int> rp(n > 0 ? (size_t)n + 1 : 0);
  if (n > 0) {
    CUDA_TRY(cudaMemcpyAsync(rp.data(), h->csr_ptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    for (int i = 0; i < n; ++i) h->max_in_degree = std::max(h->max_in_degree, rp[i + 1] - rp[i]);
  }
  h->analysed = true;
  // 5. execution plan, schedule and layouts
  ST_TRY(make_plan(h, rp, s));
  ST_TRY(build_layout(h, effective_block(h), s));
  CUDA_TRY(cudaEventRecord(e1, s));
  CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  h->analysis_ms = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return SPTRSV_OK;
}
}  // namespace

extern "C" {

int sptrsv_gb300_analyse(sptrsv_handle_t h, int m, int n, int nnz, const int* d_colPtr, const int* d_rowIdx,
                         int substitution, void* stream) {
  if (!h) return SPTRSV_ERR_INVALID;
  if (m != n) return SPTRSV_ERR_NOT_SQUARE;
  if (n < 0 || nnz < 0 || (substitution != 0 && substitution != 1)) return SPTRSV_ERR_INVALID;
  if (nnz < n) return SPTRSV_ERR_BAD_STRUCTURE;  // a diagonal per column at least
  if (n > 0 && (!d_colPtr || (nnz > 0 && !d_rowIdx))) return SPTRSV_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  free_analysis(h);
  h->n = n;
  h->nnz = nnz;
  h->substitution = substitution;
  return analyse_core(h, d_colPtr, d_rowIdx, s);
}

int sptrsv_gb300_analyse_batch(sptrsv_handle_t h, int count, const int* h_n, const int* h_nnz,
                               const int* h_substitution, const int* d_colPtr, const int* d_rowIdx, void* stream) {
  if (!h || count < 1 || !h_n || !h_nnz || !h_substitution) return SPTRSV_ERR_INVALID;
  long long total_n = 0, total_nnz = 0;
  for (int i = 0; i < count; ++i) {
    if (h_n[i] < 0 || h_nnz[i] < h_n[i] || (h_substitution[i] != 0 && h_substitution[i] != 1))
      return h_n[i] >= 0 && h_nnz[i] < h_n[i] ? SPTRSV_ERR_BAD_STRUCTURE : SPTRSV_ERR_INVALID;
    total_n += h_n[i];
    total_nnz += h_nnz[i];
  }
  if (total_n > INT_MAX || total_nnz > INT_MAX) return SPTRSV_ERR_UNSUPPORTED;
  if (total_n > 0 && (!d_colPtr || (total_nnz > 0 && !d_rowIdx))) return SPTRSV_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  free_analysis(h);
  const int n = static_cast<int>(total_n), nnz = static_cast<int>(total_nnz);
  h->n = n;
  h->nnz = nnz;
  h->substitution = h_substitution[0];
  h->batch_count = count;
  std::vector<int> off(count), eoff(count);
  long long ro = 0, eo = 0;
  for (int i = 0; i < count; ++i) {
    off[i] = static_cast<int>(ro);
    eoff[i] = static_cast<int>(eo);
    ro += h_n[i];
    eo += h_nnz[i];
  }
  h->sys_off_host = off;
  h->sys_n_host.assign(h_n, h_n + count);
  h->sys_sub_host.assign(h_substitution, h_substitution + count);
  ST_TRY(dev_alloc(h, &h->sys_dir, n));
  ST_TRY(dev_alloc(h, &h->sys_of, n));
  ST_TRY(dev_alloc(h, &h->sys_off, count));
  ST_TRY(dev_alloc(h, &h->sys_n, count));
  int *d_eoff = nullptr, *d_sub = nullptr, *g_ptr = nullptr, *g_row = nullptr;
  CUDA_TRY(cudaMemcpyAsync(h->sys_off, off.data(), sizeof(int) * count, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(h->sys_n, h_n, sizeof(int) * count, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&d_eoff), sizeof(int) * count, s));
  CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&d_sub), sizeof(int) * count, s));
  CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&g_ptr), sizeof(int) * ((size_t)n + 1), s));
  CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&g_row), sizeof(int) * ((size_t)nnz + 1), s));
  CUDA_TRY(cudaMemcpyAsync(d_eoff, eoff.data(), sizeof(int) * count, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(d_sub, h_substitution, sizeof(int) * count, cudaMemcpyHostToDevice, s));
  // per-system pointers must start at 0 and end at their nnz: checked by the merged validation
  CUDA_TRY(cudaMemsetAsync(h->flags, 0, sizeof(int), s));
  CUDA_TRY(launch_batch_merge(d_colPtr, d_rowIdx, count, h->sys_off, d_eoff, d_sub, n, nnz, g_ptr, g_row, h->sys_dir,
                              h->sys_of, h->flags, s));
  int mf = 0;
  ST_TRY(read_flags(h, s, &mf));
  const int st = mf ? SPTRSV_ERR_BAD_STRUCTURE : analyse_core(h, g_ptr, g_row, s);
  cudaFreeAsync(d_eoff, s);
  cudaFreeAsync(d_sub, s);
  cudaFreeAsync(g_ptr, s);
  cudaFreeAsync(g_row, s);
  cudaStreamSynchronize(s);
  return st;
}

int sptrsv_gb300_batch_count(sptrsv_handle_t h, int* count) {
  if (!h || !count) return SPTRSV_ERR_INVALID;
  *count = h->batch_count;
  return h->analysed ? SPTRSV_OK : SPTRSV_ERR_STATE;
}

int sptrsv_gb300_get_info(sptrsv_handle_t h, sptrsv_info* info) {
  if (!h || !info) return SPTRSV_ERR_INVALID;
  std::memset(info, 0, sizeof(*info));
  info->n = h->n;
  info->nnz = h->nnz;
  info->substitution = h->substitution;
  info->nlevels = h->nlevels;
  info->parallelism_min = h->pmin;
  info->parallelism_avg = h->pavg;
  info->parallelism_max = h->pmax;
  info->max_in_degree = h->max_in_degree;
  ExecConfig c = pick_config(h, 1);
  info->schedule = h->last_sched ? h->last_sched : c.sched;
  info->lanes = c.lanes;
  info->chunk = c.chunk;
  info->order_block = h->layout_block;
  info->analysis_ms = h->analysis_ms;
  info->device_bytes = h->device_bytes;
  info->block = c.block;
  info->warp_sync = c.wsync;
  info->staged = c.staged;
  info->split = planned(h, SPTRSV_OPTION_SPLIT) ? h->plan.split_fwd : c.split;
  info->locality_permille = static_cast<int>(h->plan.locality * 1000.0 + 0.5);
  info->unit_pipeline = h->last_pipe ? 1 : 0;
  if (c.wsync_batch > 0) {
    info->wsync_batch = c.wsync_batch;
  } else {
    // the forward walk of a plain solve: the importer executor on a blocked
    // layout, else the level-order executor with or without split lists
    const bool imported = c.wsync && !c.exact && h->import_option && h->layout_block < h->n &&
                          c.chunk == h->layout_block && c.smem_tier && !(c.split > 0 && h->max_dep_cnt > c.split);
    const bool split = !imported && c.wsync && !c.exact && info->split > 0 && h->max_dep_cnt > info->split;
    info->wsync_batch = auto_wsync_batch(h, false, split);
  }
  info->coarrive_permille = static_cast<int>(h->plan.coarrive * 1000.0 + 0.5);
  return h->analysed ? SPTRSV_OK : SPTRSV_ERR_STATE;
}

int sptrsv_gb300_levels(sptrsv_handle_t h, int* d_levelPtr, int* d_levelItem, void* stream) {
  if (!h) return SPTRSV_ERR_INVALID;
  if (!h->analysed) return SPTRSV_ERR_STATE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (h->n == 0) return SPTRSV_OK;
  if (d_levelPtr)
    CUDA_TRY(cudaMemcpyAsync(d_levelPtr, h->level_ptr_nat, sizeof(int) * (h->nlevels + 1), cudaMemcpyDeviceToDevice, s));
  if (d_levelItem)
    CUDA_TRY(cudaMemcpyAsync(d_levelItem, h->level_item, sizeof(int) * h->n, cudaMemcpyDeviceToDevice, s));
  return SPTRSV_OK;
}

int sptrsv_gb300_csr(sptrsv_handle_t h, int* d_rowPtr, int* d_colIdx, int* d_srcIdx, void* stream) {
  if (!h) return SPTRSV_ERR_INVALID;
  if (!h->analysed) return SPTRSV_ERR_STATE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (d_rowPtr)
    CUDA_TRY(cudaMemcpyAsync(d_rowPtr, h->csr_ptr, sizeof(int) * ((size_t)h->n + 1), cudaMemcpyDeviceToDevice, s));
  if (h->nnz > 0 && d_colIdx)
    CUDA_TRY(cudaMemcpyAsync(d_colIdx, h->csr_col, sizeof(int) * (size_t)h->nnz, cudaMemcpyDeviceToDevice, s));
  if (h->nnz > 0 && d_srcIdx)
    CUDA_TRY(cudaMemcpyAsync(d_srcIdx, h->csr_src, sizeof(int) * (size_t)h->nnz, cudaMemcpyDeviceToDevice, s));
  return SPTRSV_OK;
}

int sptrsv_gb300_set_values(sptrsv_handle_t h, const void* d_val, int dtype, void* stream) {
  if (!h || (!d_val && h->nnz > 0)) return SPTRSV_ERR_INVALID;
  if (!h->analysed) return SPTRSV_ERR_STATE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ST_TRY(ensure_layout(h, s));
  return stage_values(h, d_val, dtype, s, true);
}

// Column-major blocks of many right-hand sides are solved through row-major
// staging (transpose in, solve, transpose out): the executors then read and
// write whole rows of the block with coalesced accesses. Measured worthwhile
// from 32 right-hand sides for plain solves, and always for refinement
// (whose FP32 solves and residual run on internal buffers).
constexpr int kColMajorStageRhs = 32;

bool stage_col_major(const sptrsv_gb300_handle_s* h, int rhs, int layout, int min_rhs) {
  return layout == SPTRSV_LAYOUT_COL_MAJOR && rhs >= min_rhs && rhs > 1 && h->n > 0;
}

int sptrsv_gb300_solve(sptrsv_handle_t h, const void* d_val, int dtype, int rhs, int layout, const void* d_b,
                       void* d_x, void* stream) {
  if (!h) return SPTRSV_ERR_INVALID;
  if (!h->analysed) return SPTRSV_ERR_STATE;
  if (rhs < 1 || (layout != SPTRSV_LAYOUT_ROW_MAJOR && layout != SPTRSV_LAYOUT_COL_MAJOR)) return SPTRSV_ERR_INVALID;
  if (dtype != SPTRSV_DTYPE_F64 && dtype != SPTRSV_DTYPE_F32) return SPTRSV_ERR_INVALID;
  if (h->n == 0) return SPTRSV_OK;
  if (!d_b || !d_x) return SPTRSV_ERR_INVALID;
  if ((long long)h->n * rhs > INT_MAX) return SPTRSV_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (stage_col_major(h, rhs, layout, kColMajorStageRhs)) {
    const size_t elem = dtype == SPTRSV_DTYPE_F64 ? sizeof(double) : sizeof(float);
    const size_t bytes = (size_t)h->n * rhs * elem;
    ST_TRY(ensure_buf(h, h->tb, bytes, 0, s));
    ST_TRY(ensure_buf(h, h->tx, bytes, 0, s));
    if (dtype == SPTRSV_DTYPE_F64) {
      CUDA_TRY(launch_transpose<double>(static_cast<const double*>(d_b), static_cast<double*>(h->tb.p), rhs, h->n, s));
    } else {
      CUDA_TRY(launch_transpose<float>(static_cast<const float*>(d_b), static_cast<float*>(h->tb.p), rhs, h->n, s));
    }
    const int st = sptrsv_gb300_solve(h, d_val, dtype, rhs, SPTRSV_LAYOUT_ROW_MAJOR, h->tb.p, h->tx.p, stream);
    if (st != SPTRSV_OK) return st;
    if (dtype == SPTRSV_DTYPE_F64) {
      CUDA_TRY(launch_transpose<double>(static_cast<const double*>(h->tx.p), static_cast<double*>(d_x), h->n, rhs, s));
    } else {
      CUDA_TRY(launch_transpose<float>(static_cast<const float*>(h->tx.p), static_cast<float*>(d_x), h->n, rhs, s));
    }
    return SPTRSV_OK;
  }
  const int before = h->layout_block;
  ST_TRY(ensure_layout(h, s));
  if (d_val) {
    ST_TRY(stage_values(h, d_val, dtype, s, h->sync_check != 0));
  } else if (h->layout_block != before) {
    return SPTRSV_ERR_STATE;  // schedule changed since the values were staged
  }
  if (dtype == SPTRSV_DTYPE_F64) {
    if (!h->staged64) return SPTRSV_ERR_STATE;
    return solve_typed<double>(h, h->v64, rhs, layout, static_cast<const double*>(d_b), static_cast<double*>(d_x), s);
  }
  if (!h->staged32) return SPTRSV_ERR_STATE;
  return solve_typed<float>(h, h->v32, rhs, layout, static_cast<const float*>(d_b), static_cast<float*>(d_x), s);
}

int sptrsv_gb300_solve_refine(sptrsv_handle_t h, const double* d_val, int rhs, int layout, const double* d_b,
                              double* d_x, double tol, int max_iter, int* iters, double* est, void* stream) {
  if (iters) *iters = 0;
  if (est) *est = NAN;
  if (!h) return SPTRSV_ERR_INVALID;
  if (!h->analysed) return SPTRSV_ERR_STATE;
  if (rhs < 1 || max_iter < 1 || (layout != SPTRSV_LAYOUT_ROW_MAJOR && layout != SPTRSV_LAYOUT_COL_MAJOR))
    return SPTRSV_ERR_INVALID;
  if (h->n == 0) return SPTRSV_OK;
  if (!d_b || !d_x) return SPTRSV_ERR_INVALID;
  if ((long long)h->n * rhs > INT_MAX) return SPTRSV_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (stage_col_major(h, rhs, layout, 2)) {
    const size_t bytes = (size_t)h->n * rhs * sizeof(double);
    ST_TRY(ensure_buf(h, h->tb, bytes, 0, s));
    ST_TRY(ensure_buf(h, h->tx, bytes, 0, s));
    CUDA_TRY(launch_transpose<double>(d_b, static_cast<double*>(h->tb.p), rhs, h->n, s));
    const int st = sptrsv_gb300_solve_refine(h, d_val, rhs, SPTRSV_LAYOUT_ROW_MAJOR, static_cast<double*>(h->tb.p),
                                             static_cast<double*>(h->tx.p), tol, max_iter, iters, est, stream);
    if (st != SPTRSV_OK && st != SPTRSV_ERR_NOT_CONVERGED) return st;
    CUDA_TRY(launch_transpose<double>(static_cast<const double*>(h->tx.p), d_x, h->n, rhs, s));
    return st;
  }
  const int before = h->layout_block;
  ST_TRY(ensure_layout(h, s));
  if (d_val) {
    ST_TRY(stage_values(h, d_val, SPTRSV_DTYPE_F64, s, h->sync_check != 0));
  } else if (h->layout_block != before) {
    return SPTRSV_ERR_STATE;
  }
  if (!h->staged64 || !h->staged32) return SPTRSV_ERR_STATE;
  const long long count = (long long)h->n * rhs;
  ST_TRY(ensure_buf(h, h->r32, sizeof(float) * count, 0, s));
  ST_TRY(ensure_buf(h, h->d32, sizeof(float) * count, 0, s));
  ST_TRY(ensure_buf(h, h->stats, 4 * sizeof(unsigned long long), 1, s));
  const long long si = layout == SPTRSV_LAYOUT_ROW_MAJOR ? rhs : 1;
  const long long sk = layout == SPTRSV_LAYOUT_ROW_MAJOR ? 1 : h->n;
  float* r32 = static_cast<float*>(h->r32.p);
  float* d32 = static_cast<float*>(h->d32.p);
  auto* stats = static_cast<unsigned long long*>(h->stats.p);
  const bool checked = tol > 0.0;
  double prev = 0.0, xmax = 0.0, estimate = NAN;
  unsigned long long host_stats[3] = {0, 0, 0};
  int it = 0, first = 1;
  bool converged = false;
  ExecConfig fc = pick_config(h, rhs);
  bool fuse = h->fused_refine && fc.sched == SCHED_PULL && !fc.exact && rhs <= 64;
  if (fuse && rhs == 1) {
    // the fused pass gives every unknown one lane: where the plain solve would
    // spread long lists over lanes (split executor), separate passes are faster
    const int split = planned(h, SPTRSV_OPTION_SPLIT) ? h->plan.split_fwd : fc.split;
    if (split > 0 && h->max_dep_cnt > split) fuse = false;
  }
  if (fuse) {
    // X_0, the FP64 residual and the first FP32 correction in one pass: X = X_0 + D_1
    // the plain solve's rule (160k-row bands with 1 / 2 entries per column and a
    // 1M-row band with 3: 0.101 / 1.95 / 6.40 ms refined with two dependencies
    // per iteration, 0.082 / 1.54 / 5.62 with one; the mesh triangle with two:
    // 0.28 vs 0.61 ms)
    if (rhs == 1 && fc.wsync_batch == 0) fc.wsync_batch = auto_wsync_batch(h, false, false);
    // level order: one CTA of 256 threads per SM for one right-hand side on one
    // system, two up to 4 right-hand sides (and for batches); beyond, three with
    // the FP64 residual and every CTA that fits (four) with the double-float
    // one, which holds fewer registers (measured on the 1M-row band system and
    // the 512-system batch: the pass reads more per dependency than a plain
    // solve, and fewer polling warps paid with few right-hand sides — rhs 1:
    // 1.19 ms with one, 1.21 with two; rhs 4: 1.245 with two, 1.29 with one; at
    // 16 / 64 the double-float pass took 1.34 / 2.78 ms with three and 1.23 /
    // 2.43 ms with four)
    if (h->sched_option == SCHED_AUTO && planned(h, SPTRSV_OPTION_CTAS_PER_SM) && h->layout_block >= h->n)
      fc.ctas_per_sm = rhs <= 4 ? (rhs == 1 && h->batch_count == 1 ? 1 : 2) : (h->fused_refine == 2 ? 0 : 3);
    ST_TRY(ensure_buf(h, h->xw, sizeof(unsigned long long) * count, 0, s));
    CUDA_TRY(cudaMemsetAsync(h->xw.p, 0xFF, sizeof(unsigned long long) * count, s));
    CUDA_TRY(cudaMemsetAsync(stats, 0, 3 * sizeof(unsigned long long), s));
    h->last_sched = SCHED_PULL;
    h->last_pipe = false;
    if (h->profile) {
      if (!h->ev_exec[0]) {
        CUDA_TRY(cudaEventCreate(&h->ev_exec[0]));
        CUDA_TRY(cudaEventCreate(&h->ev_exec[1]));
      }
      CUDA_TRY(cudaEventRecord(h->ev_exec[0], s));
    }
    const float2* wsplit = nullptr;
    if (h->fused_refine == 2) {
      // the residual in double-float: (hi, lo) pairs of the FP64 weights, once per staging
      const long long ndep = h->layout.ndep;
      if (!h->wsplit_ok) {
        ST_TRY(ensure_buf(h, h->wsplit, sizeof(float2) * (size_t)(ndep + 16), 0, s));
        CUDA_TRY(launch_split_weights(h->v64.dep_w, ndep, static_cast<float2*>(h->wsplit.p), s));
        h->wsplit_ok = true;
      }
      wsplit = static_cast<const float2*>(h->wsplit.p);
    }
    // one right-hand side on a blocked layout: the importer-warp variant (as the
    // plain solve's k_pull_wsync_imp) keeps the cross-block polls out of the
    // consumer warps' lockstep iterations
    const bool imported = wsplit && rhs == 1 && fc.wsync && h->import_option && h->layout_block < h->n &&
                          fc.chunk == h->layout_block && fc.smem_tier &&
                          (h->imports.chunk == fc.chunk || build_imports(h, fc.chunk, 8, s) == SPTRSV_OK) &&
                          h->imports.ptr != nullptr &&
                          imported_smem_bytes(h->imports.width, h->imports.max_imports, 8) <= 220 * 1024;
    if (imported) {
      fc.one_batch = h->max_dep_cnt <= fc.wsync_batch ? 1 : 0;
      CUDA_TRY(launch_refine_fused_imported(h->layout, h->v64, wsplit, d_b, d_x,
                                            static_cast<unsigned long long*>(h->xw.p), stats, h->ctl, fc,
                                            timeout_ns(h), h->num_sms, s, h->imports));
    } else {
      CUDA_TRY(launch_refine_fused(h->layout, h->v32, h->v64, rhs, d_b, d_x, si, sk,
                                   static_cast<unsigned long long*>(h->xw.p), stats, h->ctl, fc, timeout_ns(h),
                                   h->num_sms, s, wsplit));
    }
    if (h->profile) {
      CUDA_TRY(cudaEventRecord(h->ev_exec[1], s));
      h->ev_recorded = true;
    }
    first = 2;
    it = 1;
    if (checked) {
      CUDA_TRY(cudaMemcpyAsync(host_stats, stats, sizeof(host_stats), cudaMemcpyDeviceToHost, s));
      CUDA_TRY(cudaStreamSynchronize(s));
      double dmax = 0.0, x0max = 0.0;
      std::memcpy(&dmax, &host_stats[0], sizeof(double));
      std::memcpy(&xmax, &host_stats[1], sizeof(double));
      std::memcpy(&x0max, &host_stats[2], sizeof(double));
      // D_0 = X_0, D_1 = the fused correction
      estimate = (x0max > 0.0 && xmax > 0.0) ? dmax * (dmax / x0max) / xmax : (dmax == 0.0 ? 0.0 : INFINITY);
      converged = estimate <= tol;
      prev = dmax;
    }
  } else {
    // X_0 = FP32 solve of (float) B
    CUDA_TRY(launch_cast_d2f(d_b, r32, count, s));
    ST_TRY(solve_typed<float>(h, h->v32, rhs, layout, r32, d32, s, nullptr, false));
    CUDA_TRY(cudaMemsetAsync(stats, 0, 2 * sizeof(unsigned long long), s));
    CUDA_TRY(launch_update(d_x, d32, count, stats, true, s));
    if (checked) {
      CUDA_TRY(cudaMemcpyAsync(host_stats, stats, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
      CUDA_TRY(cudaStreamSynchronize(s));
      std::memcpy(&prev, &host_stats[1], sizeof(double));
      xmax = prev;
    }
  }
  int steps = first - 1;  // refinement steps done
  for (it = first; !converged && it <= max_iter; ++it) {
    CUDA_TRY(launch_residual(h->layout, h->v64, rhs, d_b, d_x, si, sk, r32, s));
    ST_TRY(solve_typed<float>(h, h->v32, rhs, layout, r32, d32, s, nullptr, false));
    CUDA_TRY(cudaMemsetAsync(stats, 0, 2 * sizeof(unsigned long long), s));
    CUDA_TRY(launch_update(d_x, d32, count, stats, false, s));
    steps = it;
    if (!checked) continue;
    CUDA_TRY(cudaMemcpyAsync(host_stats, stats, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    double dmax = 0.0;
    std::memcpy(&dmax, &host_stats[0], sizeof(double));
    std::memcpy(&xmax, &host_stats[1], sizeof(double));
    estimate = (prev > 0.0 && xmax > 0.0) ? dmax * (dmax / prev) / xmax : (dmax == 0.0 ? 0.0 : INFINITY);
    if (estimate <= tol) {
      converged = true;
      break;
    }
    prev = dmax;
  }
  if (iters) *iters = steps;
  if (est) *est = estimate;
  if (h->sync_check || checked) ST_TRY(check_device(h, s));
  if (checked && !converged) return SPTRSV_ERR_NOT_CONVERGED;
  return SPTRSV_OK;
}

int sptrsv_gb300_solve_adjoint(sptrsv_handle_t h, const void* d_val, int dtype, int rhs, int layout, const void* d_g,
                               void* d_lambda, const void* d_x, void* d_dval, void* stream) {
  if (!h) return SPTRSV_ERR_INVALID;
  if (!h->analysed) return SPTRSV_ERR_STATE;
  if (rhs < 1 || (layout != SPTRSV_LAYOUT_ROW_MAJOR && layout != SPTRSV_LAYOUT_COL_MAJOR)) return SPTRSV_ERR_INVALID;
  if (dtype != SPTRSV_DTYPE_F64 && dtype != SPTRSV_DTYPE_F32) return SPTRSV_ERR_INVALID;
  if (h->n == 0) return SPTRSV_OK;
  if (!d_g || !d_lambda || (d_dval && !d_x)) return SPTRSV_ERR_INVALID;
  if (h->sched_option == SCHED_LEVELSET) return SPTRSV_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int before = h->layout_block;
  ST_TRY(ensure_layout(h, s));
  if (d_val) {
    ST_TRY(stage_values(h, d_val, dtype, s, h->sync_check != 0));
  } else if (h->layout_block != before) {
    return SPTRSV_ERR_STATE;
  }
  const long long si = layout == SPTRSV_LAYOUT_ROW_MAJOR ? rhs : 1;
  const long long sk = layout == SPTRSV_LAYOUT_ROW_MAJOR ? 1 : h->n;
  if (d_dval && !h->fused_grad) {
    // transposed solve first, then one pass over the stored pattern for the gradient
    const int saved = h->sync_check;
    h->sync_check = 0;
    int st = sptrsv_gb300_solve_adjoint(h, nullptr, dtype, rhs, layout, d_g, d_lambda, nullptr, nullptr, stream);
    h->sync_check = saved;
    if (st != SPTRSV_OK) return st;
    return sptrsv_gb300_grad_values(h, dtype, rhs, layout, d_lambda, d_x, d_dval, stream);
  }
  if (dtype == SPTRSV_DTYPE_F64) {
    if (!h->staged64) return SPTRSV_ERR_STATE;
    AdjointArgs<double> adj;
    adj.grad = static_cast<double*>(d_dval);
    adj.xf = static_cast<const double*>(d_x);
    adj.xf_si = si;
    adj.xf_sk = sk;
    return solve_typed<double>(h, h->v64, rhs, layout, static_cast<const double*>(d_g), static_cast<double*>(d_lambda),
                               s, &adj);
  }
  if (!h->staged32) return SPTRSV_ERR_STATE;
  AdjointArgs<float> adj;
  adj.grad = static_cast<float*>(d_dval);
  adj.xf = static_cast<const float*>(d_x);
  adj.xf_si = si;
  adj.xf_sk = sk;
  return solve_typed<float>(h, h->v32, rhs, layout, static_cast<const float*>(d_g), static_cast<float*>(d_lambda), s,
                            &adj);
}

int sptrsv_gb300_grad_values(sptrsv_handle_t h, int dtype, int rhs, int layout, const void* d_lambda, const void* d_x,
                             void* d_dval, void* stream) {
  if (!h) return SPTRSV_ERR_INVALID;
  if (!h->analysed) return SPTRSV_ERR_STATE;
  if (rhs < 1 || (layout != SPTRSV_LAYOUT_ROW_MAJOR && layout != SPTRSV_LAYOUT_COL_MAJOR)) return SPTRSV_ERR_INVALID;
  if (h->nnz == 0) return SPTRSV_OK;
  if (!d_lambda || !d_x || !d_dval) return SPTRSV_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long si = layout == SPTRSV_LAYOUT_ROW_MAJOR ? rhs : 1;
  const long long sk = layout == SPTRSV_LAYOUT_ROW_MAJOR ? 1 : h->n;
  if (dtype == SPTRSV_DTYPE_F64)
    CUDA_TRY(launch_grad_values<double>(h->csc_row, h->csc_col, h->nnz, rhs, static_cast<const double*>(d_lambda),
                                        static_cast<const double*>(d_x), si, sk, static_cast<double*>(d_dval), s));
  else if (dtype == SPTRSV_DTYPE_F32)
    CUDA_TRY(launch_grad_values<float>(h->csc_row, h->csc_col, h->nnz, rhs, static_cast<const float*>(d_lambda),
                                       static_cast<const float*>(d_x), si, sk, static_cast<float*>(d_dval), s));
  else
    return SPTRSV_ERR_INVALID;
  if (h->sync_check) return check_device(h, s);
  return SPTRSV_OK;
}

// ---------------------------------------------------------------- CUDA graphs
namespace {
struct GraphBox {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};
}  // namespace

int sptrsv_gb300_graph_create(sptrsv_handle_t h, int kind, int dtype, int rhs, int layout, const void* d_b, void* d_x,
                              int count, void** graph, void* stream) {
  if (!h || !graph || count < 1 || (kind != 0 && kind != 1)) return SPTRSV_ERR_INVALID;
  *graph = nullptr;
  if (!h->analysed) return SPTRSV_ERR_STATE;
  if (kind == 1 && dtype != SPTRSV_DTYPE_F64) return SPTRSV_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int saved_check = h->sync_check, saved_profile = h->profile;
  // one eager run sizes every workspace and table, so the capture allocates nothing
  int st = kind == 0 ? sptrsv_gb300_solve(h, nullptr, dtype, rhs, layout, d_b, d_x, stream)
                     : sptrsv_gb300_solve_refine(h, nullptr, rhs, layout, static_cast<const double*>(d_b),
                                                 static_cast<double*>(d_x), 0.0, count, nullptr, nullptr, stream);
  if (st != SPTRSV_OK) return st;
  CUDA_TRY(cudaStreamSynchronize(s));
  cudaStream_t cs = nullptr;
  CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  h->sync_check = 0;
  h->profile = 0;
  GraphBox* box = new (std::nothrow) GraphBox();
  cudaError_t e = box ? cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) : cudaErrorMemoryAllocation;
  if (e == cudaSuccess) {
    if (kind == 0) {
      for (int i = 0; i < count && st == SPTRSV_OK; ++i)
        st = sptrsv_gb300_solve(h, nullptr, dtype, rhs, layout, d_b, d_x, cs);
    } else {
      st = sptrsv_gb300_solve_refine(h, nullptr, rhs, layout, static_cast<const double*>(d_b),
                                     static_cast<double*>(d_x), 0.0, count, nullptr, nullptr, cs);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    if (st == SPTRSV_OK && e2 == cudaSuccess) {
      box->graph = g;
      e = cudaGraphInstantiate(&box->exec, g, 0);
    } else {
      if (g) cudaGraphDestroy(g);
      e = e2 != cudaSuccess ? e2 : cudaSuccess;
    }
  }
  h->sync_check = saved_check;
  h->profile = saved_profile;
  cudaStreamDestroy(cs);
  if (st != SPTRSV_OK || e != cudaSuccess || !box || !box->exec) {
    if (box) {
      if (box->exec) cudaGraphExecDestroy(box->exec);
      if (box->graph) cudaGraphDestroy(box->graph);
      delete box;
    }
    cudaGetLastError();
    return st != SPTRSV_OK ? st : map_cuda_error(e != cudaSuccess ? e : cudaErrorUnknown);
  }
  *graph = box;
  return SPTRSV_OK;
}

int sptrsv_gb300_graph_launch(void* graph, void* stream) {
  if (!graph) return SPTRSV_ERR_INVALID;
  CUDA_TRY(cudaGraphLaunch(static_cast<GraphBox*>(graph)->exec, static_cast<cudaStream_t>(stream)));
  return SPTRSV_OK;
}

int sptrsv_gb300_graph_destroy(void* graph) {
  if (!graph) return SPTRSV_ERR_INVALID;
  auto* box = static_cast<GraphBox*>(graph);
  if (box->exec) cudaGraphExecDestroy(box->exec);
  if (box->graph) cudaGraphDestroy(box->graph);
  delete box;
  return SPTRSV_OK;
}

// ---------------------------------------------------------------- autotuner
int sptrsv_gb300_tune(sptrsv_handle_t h, const void* d_val, int dtype, int rhs, int layout, const void* d_b, void* d_x,
                      int reps, double* best_ms, void* stream) {
  if (!h || !d_val || !d_b || !d_x || reps < 1) return SPTRSV_ERR_INVALID;
  if (!h->analysed) return SPTRSV_ERR_STATE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  struct Cand {
    int sched, order_block, chunk, staged, backoff, ctas, lanes, stages, wsync, block, split, batch = 0;
    int smem = 1, opt = SPTRSV_OPT_WARP_AUTO, tile = 0;
  };
  const int n = h->n;
  const int big = INT_MAX;
  std::vector<Cand> cands;
  const int sp = 32;  // split length of the warp-synchronous candidates
  // Order blocks from the analysis: blocks of 16, 32 and 64 average level
  // widths (the automatic plan's locality test uses 32), multiples of 32
  // unknowns, kept between 1024 and 32768 and below n; plus the plan's own.
  std::vector<int> blocks;
  if (n > 0 && h->nlevels > 0) {
    const long long width = ((long long)n + h->nlevels - 1) / h->nlevels;
    for (int f : {16, 32, 64}) {
      long long b = (f * width + 31) / 32 * 32;
      b = std::min<long long>(32768, std::max<long long>(1024, b));
      if (b < n && std::find(blocks.begin(), blocks.end(), (int)b) == blocks.end()) blocks.push_back((int)b);
    }
    if (h->plan.valid && h->plan.order_block < n &&
        std::find(blocks.begin(), blocks.end(), h->plan.order_block) == blocks.end())
      blocks.push_back(h->plan.order_block);
  }
  if (rhs == 1) {
    // staged warp-specialised executor, level order
    for (int bo : {0, 256}) cands.push_back({SCHED_PULL, big, 224, 1, bo, 0, 1, 2, 0, 256, sp});
    // warp-synchronous executor (long lists split over lanes): level order, and
    // blocked orders for deep narrow DAGs
    for (int ch : {128, 256}) cands.push_back({SCHED_PULL, big, ch, 0, 128, 1, 1, 2, 1, ch, sp});
    cands.push_back({SCHED_PULL, big, 256, 0, 128, 1, 1, 2, 1, 256, 0});
    for (int bt : {1, 2, 4}) cands.push_back({SCHED_PULL, big, 256, 0, 128, 1, 1, 2, 1, 256, sp, bt});
    for (int ct : {2, 3}) {
      cands.push_back({SCHED_PULL, big, 256, 0, 0, ct, 1, 2, 1, 256, sp});
      cands.push_back({SCHED_PULL, big, 256, 0, 0, ct, 1, 2, 1, 256, 0});
      cands.push_back({SCHED_PULL, big, 128, 0, 0, ct, 1, 2, 1, 128, sp});
    }
    // in-chunk dependencies through global memory only (no shared-memory tier)
    cands.push_back({SCHED_PULL, big, 256, 0, 0, 2, 1, 2, 1, 256, sp, 0, 0});
    for (int ob : blocks) {
      cands.push_back({SCHED_PULL, ob, ob, 0, 0, 0, 1, 2, 1, 128, sp});
      for (int bt : {1, 2, 4}) cands.push_back({SCHED_PULL, ob, ob, 0, 0, 0, 1, 2, 1, 128, sp, bt});
    }
    // thread-per-unknown executor, level order
    cands.push_back({SCHED_PULL, big, 256, 0, 128, 1, 1, 2, 0, 256, sp});
    cands.push_back({SCHED_LEVELSET, big, 256, 0, 256, 1, 8, 2, 0, 256, sp});
    cands.push_back({SCHED_PUSH, 1024, 1024, 0, 256, 0, 1, 2, 0, 256, sp});
    cands.push_back({SCHED_PUSH, 1024, 1024, 0, 256, 0, 1, 2, 0, 256, sp, 0, 0});
  } else {
    // chunk 0 = one unknown per lane group; right-hand-side tiles (1, 2, 4 per lane)
    for (int bo : {64, 512}) cands.push_back({SCHED_PULL, big, 0, 0, bo, 0, 1, 2, 1, 256, sp});
    std::vector<int> groups;   // distinct (lanes, right-hand sides per lane) pairs
    for (int tile : {1, 2, 4}) {
      int rpl = 1;
      const int key = multi_group(rhs, tile, &rpl) * 8 + rpl;
      if (std::find(groups.begin(), groups.end(), key) != groups.end()) continue;
      groups.push_back(key);
      for (int ct : {1, 2, 3})
        cands.push_back({SCHED_PULL, big, 0, 0, 0, ct, 1, 2, 1, 256, sp, 0, 1, SPTRSV_OPT_WARP_AUTO, tile});
    }
    cands.push_back({SCHED_PULL, big, 0, 0, 0, 0, 1, 2, 1, 256, sp, 0, 0});   // global-memory tier only
    for (int ob : blocks) cands.push_back({SCHED_PULL, ob, ob, 0, 0, 0, 1, 2, 1, 256, sp});
    cands.push_back({SCHED_PULL, big, 0, 0, 256, 0, 1, 2, 0, 256, sp});
    cands.push_back({SCHED_LEVELSET, big, 256, 0, 256, 1, 8, 2, 0, 256, sp});
    // the reference's scheme with its three lane modes
    for (int o : {SPTRSV_OPT_WARP_NNZ, SPTRSV_OPT_WARP_RHS, SPTRSV_OPT_WARP_AUTO})
      cands.push_back({SCHED_PUSH, big, 0, 0, 256, 0, 1, 2, 0, 256, sp, 0, 1, o, 0});
  }
  (void)n;
  const int saved_check = h->sync_check, saved_profile = h->profile;
  h->sync_check = 0;
  h->profile = 0;
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  double best = 1e300;
  int best_i = -1;
  for (size_t i = 0; i < cands.size(); ++i) {
    const Cand& c = cands[i];
    h->sched_option = c.sched;
    h->order_block = c.order_block;
    h->chunk_option = c.chunk;
    h->staged = c.staged;
    h->backoff_ns = c.backoff;
    h->ctas_per_sm = c.ctas;
    h->lanes_option = c.lanes;
    h->stages_option = c.stages;
    h->wsync = c.wsync;
    h->block_option = c.block;
    h->split = c.split;
    h->wsync_batch = c.batch;
    h->cfg.smem_tier = c.smem;
    h->opt_option = c.opt;
    h->rhs_tile_option = c.tile;
    int st = sptrsv_gb300_solve(h, d_val, dtype, rhs, layout, d_b, d_x, stream);
    if (st == SPTRSV_OK) st = check_device(h, s);
    if (st != SPTRSV_OK) continue;  // a candidate that fails (or times out) is skipped
    std::vector<float> t;
    for (int r = 0; r < reps && st == SPTRSV_OK; ++r) {
      cudaEventRecord(e0, s);
      st = sptrsv_gb300_solve(h, nullptr, dtype, rhs, layout, d_b, d_x, stream);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      t.push_back(ms);
    }
    if (st == SPTRSV_OK) st = check_device(h, s);
    if (st != SPTRSV_OK || t.empty()) continue;
    std::sort(t.begin(), t.end());
    const double med = t[t.size() / 2];
    if (med < best) {
      best = med;
      best_i = static_cast<int>(i);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  h->sync_check = saved_check;
  h->profile = saved_profile;
  if (best_i < 0) return SPTRSV_ERR_CUDA;
  const Cand& c = cands[best_i];
  h->sched_option = c.sched;
  h->order_block = c.order_block;
  h->chunk_option = c.chunk;
  h->staged = c.staged;
  h->backoff_ns = c.backoff;
  h->ctas_per_sm = c.ctas;
  h->lanes_option = c.lanes;
  h->stages_option = c.stages;
  h->wsync = c.wsync;
  h->block_option = c.block;
  h->split = c.split;
  h->wsync_batch = c.batch;
  h->cfg.smem_tier = c.smem;
  h->opt_option = c.opt;
  h->rhs_tile_option = c.tile;
  ST_TRY(ensure_layout(h, s));
  ST_TRY(stage_values(h, d_val, dtype, s, false));
  if (best_ms) *best_ms = best;
  return SPTRSV_OK;
}

int sptrsv_gb300_check(sptrsv_handle_t h, void* stream) {
  if (!h) return SPTRSV_ERR_INVALID;
  return check_device(h, static_cast<cudaStream_t>(stream));
}

int sptrsv_gb300_exec_ms(sptrsv_handle_t h, double* ms) {
  if (!h || !ms) return SPTRSV_ERR_INVALID;
  if (!h->ev_recorded) return SPTRSV_ERR_STATE;
  CUDA_TRY(cudaEventSynchronize(h->ev_exec[1]));
  float t = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&t, h->ev_exec[0], h->ev_exec[1]));
  *ms = t;
  return SPTRSV_OK;
}

// ---------------------------------------------------------------- kernel-level surface
int sptrsv_gb300_analyser(const int* d_cscRowIdx, int m, int nnz, int* d_graphInDegree, void* stream) {
  if (m < 0 || nnz < 0 || (m > 0 && !d_graphInDegree) || (nnz > 0 && !d_cscRowIdx)) return SPTRSV_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (m > 0) CUDA_TRY(cudaMemsetAsync(d_graphInDegree, 0, sizeof(int) * (size_t)m, s));
  CUDA_TRY(launch_in_degree(d_cscRowIdx, m, nnz, d_graphInDegree, s));
  return SPTRSV_OK;
}

int sptrsv_gb300_executor(const int* d_cscColPtr, const int* d_cscRowIdx, const double* d_cscVal,
                          int* d_graphInDegree, double* d_left_sum, int m, int substitution, int rhs, int opt,
                          const double* d_b, double* d_x, void* stream) {
  if (m < 0 || rhs < 1 || (substitution != 0 && substitution != 1)) return SPTRSV_ERR_INVALID;
  if (m > 0 && (!d_cscColPtr || !d_cscRowIdx || !d_cscVal || !d_graphInDegree || !d_left_sum || !d_b || !d_x))
    return SPTRSV_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DeviceCtl* ctl = nullptr;
  ST_TRY(raw_ctl(s, &ctl));
  CUDA_TRY(launch_ref_executor<double>(d_cscColPtr, d_cscRowIdx, d_cscVal, d_graphInDegree, d_left_sum, m,
                                       substitution, rhs, opt, d_b, d_x, ctl, 1000000000ull, s));
  int code = 0;
  CUDA_TRY(cudaMemcpyAsync(&code, &ctl->code, sizeof(int), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (code != DEV_OK) {
    // the kernel resets its ticket and done words on exit; clear the error code
    CUDA_TRY(cudaMemsetAsync(ctl, 0, sizeof(DeviceCtl), s));
    CUDA_TRY(cudaStreamSynchronize(s));
    return code == DEV_BAD_INPUT ? SPTRSV_ERR_BAD_STRUCTURE : SPTRSV_ERR_TIMEOUT;
  }
  return SPTRSV_OK;
}

// ---------------------------------------------------------------- reference-compatible entry
int sptrsv_gb300_syncfree_host(const int* cscColPtrTR, const int* cscRowIdxTR, const double* cscValTR, int m, int n,
                               int nnzTR, int substitution, int rhs, int opt, double* x, const double* b,
                               const double* x_ref, double* gflops, double* solve_ms, double* analysis_ms,
                               double* l1_err) {
  if (m != n) {
    if (g_verbose) printf("This is not a square matrix, return.\n");
    return SPTRSV_ERR_NOT_SQUARE;
  }
  if (n < 0 || nnzTR < 0 || rhs < 1 || !x || !b || (n > 0 && (!cscColPtrTR || !cscRowIdxTR || !cscValTR)))
    return SPTRSV_ERR_INVALID;
  int *d_ptr = nullptr, *d_row = nullptr, *d_indeg = nullptr;
  double *d_val = nullptr, *d_b = nullptr, *d_x = nullptr;
  sptrsv_handle_t h = nullptr;
  int st = SPTRSV_OK;
  const size_t vec = (size_t)n * (size_t)rhs;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double t_solve = 0.0, t_an = 0.0;
  auto fail = [&](int code) { st = code; };
  do {
    if (cudaMalloc(&d_ptr, sizeof(int) * ((size_t)n + 1)) != cudaSuccess) { fail(SPTRSV_ERR_OOM); break; }
    if (cudaMalloc(&d_row, sizeof(int) * (nnzTR ? nnzTR : 1)) != cudaSuccess) { fail(SPTRSV_ERR_OOM); break; }
    if (cudaMalloc(&d_val, sizeof(double) * (nnzTR ? nnzTR : 1)) != cudaSuccess) { fail(SPTRSV_ERR_OOM); break; }
    if (cudaMalloc(&d_b, sizeof(double) * (vec ? vec : 1)) != cudaSuccess) { fail(SPTRSV_ERR_OOM); break; }
    if (cudaMalloc(&d_x, sizeof(double) * (vec ? vec : 1)) != cudaSuccess) { fail(SPTRSV_ERR_OOM); break; }
    if (cudaMalloc(&d_indeg, sizeof(int) * (n ? n : 1)) != cudaSuccess) { fail(SPTRSV_ERR_OOM); break; }
    cudaMemcpy(d_ptr, cscColPtrTR, sizeof(int) * ((size_t)n + 1), cudaMemcpyHostToDevice);
    if (nnzTR) {
      cudaMemcpy(d_row, cscRowIdxTR, sizeof(int) * nnzTR, cudaMemcpyHostToDevice);
      cudaMemcpy(d_val, cscValTR, sizeof(double) * nnzTR, cudaMemcpyHostToDevice);
    }
    if (vec) cudaMemcpy(d_b, b, sizeof(double) * vec, cudaMemcpyHostToDevice);
    if (vec) cudaMemset(d_x, 0, sizeof(double) * vec);
    if (cudaGetLastError() != cudaSuccess) { fail(SPTRSV_ERR_CUDA); break; }
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // analysis time: the in-degree analyser, averaged like the reference (:456-483)
    for (int i = 0; i < g_bench_repeat; ++i) {
      float ms = 0.f;
      cudaEventRecord(e0, 0);
      int r = sptrsv_gb300_analyser(d_row, m, nnzTR, d_indeg, nullptr);
      cudaEventRecord(e1, 0);
      cudaEventSynchronize(e1);
      cudaEventElapsedTime(&ms, e0, e1);
      t_an += ms;
      if (r != SPTRSV_OK) { fail(r); break; }
    }
    if (st != SPTRSV_OK) break;
    t_an /= g_bench_repeat;
    if (g_verbose) printf("cuda syncfree SpTRSV analysis on L used %4.2f ms\n", t_an);
    if ((st = sptrsv_gb300_create(&h)) != SPTRSV_OK) break;
    // the reference's lane mode for many right-hand sides (used by the push
    // schedule, the reference's own scheme; out-of-range values keep AUTO)
    if (opt >= SPTRSV_OPT_WARP_NNZ && opt <= SPTRSV_OPT_WARP_AUTO) sptrsv_gb300_set_option(h, SPTRSV_OPTION_OPT, opt);
    if ((st = sptrsv_gb300_analyse(h, m, n, nnzTR, d_ptr, d_row, substitution, nullptr)) != SPTRSV_OK) break;
    if ((st = sptrsv_gb300_set_values(h, d_val, SPTRSV_DTYPE_F64, nullptr)) != SPTRSV_OK) break;
    for (int i = 0; i < g_bench_repeat; ++i) {
      float ms = 0.f;
      cudaEventRecord(e0, 0);
      int r = sptrsv_gb300_solve(h, nullptr, SPTRSV_DTYPE_F64, rhs, SPTRSV_LAYOUT_ROW_MAJOR, d_b, d_x, nullptr);
      cudaEventRecord(e1, 0);
      cudaEventSynchronize(e1);
      cudaEventElapsedTime(&ms, e0, e1);
      t_solve += ms;
      if (r != SPTRSV_OK) { fail(r); break; }
    }
    if (st != SPTRSV_OK) break;
    t_solve /= g_bench_repeat;
    const double flop = 2.0 * (double)rhs * (double)nnzTR;
    const double gf = t_solve > 0 ? flop / (1e6 * t_solve) : 0.0;
    if (gflops) *gflops = gf;
    if (g_verbose) printf("cuda syncfree SpTRSV solve used %4.2f ms, throughput is %4.2f gflops\n", t_solve, gf);
    if (vec && cudaMemcpy(x, d_x, sizeof(double) * vec, cudaMemcpyDeviceToHost) != cudaSuccess) {
      fail(SPTRSV_ERR_CUDA);
      break;
    }
    double err = NAN;
    if (x_ref) {
      double ref = 0.0, res = 0.0;
      for (size_t i = 0; i < vec; ++i) {
        ref += std::fabs(x_ref[i]);
        res += std::fabs(x[i] - x_ref[i]);
      }
      err = ref == 0.0 ? res : res / ref;
      if (g_verbose) {
        if (err < 1e-4)
          printf("cuda syncfree SpTRSV executor passed! |x-xref|/|xref| = %8.2e\n", err);
        else
          printf("cuda syncfree SpTRSV executor _NOT_ passed! |x-xref|/|xref| = %8.2e\n", err);
      }
    }
    if (l1_err) *l1_err = err;
  } while (false);
  if (solve_ms) *solve_ms = t_solve;
  if (analysis_ms) *analysis_ms = t_an;
  if (h) sptrsv_gb300_destroy(h);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(d_ptr);
  cudaFree(d_row);
  cudaFree(d_val);
  cudaFree(d_b);
  cudaFree(d_x);
  cudaFree(d_indeg);
  return st;
}

int sptrsv_syncfree_cuda(const int* cscColPtrTR, const int* cscRowIdxTR, const double* cscValTR, int m, int n,
                         int nnzTR, int substitution, int rhs, int opt, double* x, const double* b,
                         const double* x_ref, double* gflops) {
  return sptrsv_gb300_syncfree_host(cscColPtrTR, cscRowIdxTR, cscValTR, m, n, nnzTR, substitution, rhs, opt, x, b,
                                    x_ref, gflops, nullptr, nullptr, nullptr);
}

}  // extern "C"
