// Structural analysis on the device: CSC validation, the in-degree analyser,
// prefix scans, a stable radix sort, level sets, and the position-space
// layouts the executors read.
#include <algorithm>
#include <cstdio>

#include "internal.h"

namespace sptrsv {

namespace {
constexpr int kThreads = 256;

inline int grid_for(long long count, int threads = kThreads, int cap = 1 << 20) {
  long long g = (count + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return static_cast<int>(g);
}
}  // namespace

__device__ __forceinline__ int dir_of(const SysDesc& d, long long c) {
  return d.dir ? static_cast<int>(d.dir[c]) : d.substitution;
}

// ------------------------------------------------------------ validation
__global__ void k_validate_ptr(const int* __restrict__ col_ptr, int n, int nnz, int* flags) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c <= n; c += stride) {
    const int v = col_ptr[c];
    bool bad = v < 0 || v > nnz;
    if (c == 0 && v != 0) bad = true;
    if (c == n && v != nnz) bad = true;
    if (c < n && col_ptr[c + 1] < v) bad = true;
    if (bad) atomicOr(flags, SF_BAD_PTR);
  }
}

// One thread per column. A column whose pointers are not an in-range,
// non-decreasing pair is flagged SF_BAD_PTR and its rows are not read, so the
// kernel is safe on any column-pointer array (nnz = length of row_idx).
__global__ void k_validate_rows(const int* __restrict__ col_ptr, const int* __restrict__ row_idx, int n, int nnz,
                                SysDesc sd, int* flags) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += stride) {
    const int substitution = dir_of(sd, c);
    const int beg = col_ptr[c], end = col_ptr[c + 1];
    int f = 0;
    if (beg < 0 || end < beg || end > nnz) {
      f |= SF_BAD_PTR;
    } else if (beg == end) {
      f |= SF_MISSING_DIAG;
    } else {
      int prev = -1;
      bool has_diag = false;
      for (int e = beg; e < end; ++e) {
        const int r = row_idx[e];
        if (r < 0 || r >= n) { f |= SF_ROW_RANGE; break; }
        if (r <= prev) f |= SF_UNSORTED;
        prev = r;
        if (r == c) has_diag = true;
        if (substitution == 0 ? r < c : r > c) f |= SF_WRONG_TRIANGLE;
      }
      if (!(f & SF_ROW_RANGE)) {
        if (!has_diag) f |= SF_MISSING_DIAG;
        // The diagonal must open a forward column and close a backward one.
        const int edge = substitution == 0 ? row_idx[beg] : row_idx[end - 1];
        if (has_diag && edge != c) f |= SF_UNSORTED;
      }
    }
    if (f) atomicOr(flags, f);
  }
}

cudaError_t launch_validate_ptr(const int* col_ptr, int n, int nnz, int* flags, cudaStream_t s) {
  k_validate_ptr<<<grid_for((long long)n + 1), kThreads, 0, s>>>(col_ptr, n, nnz, flags);
  return cudaGetLastError();
}
cudaError_t launch_validate_rows(const int* col_ptr, const int* row_idx, int n, int nnz, const SysDesc& sd,
                                 int* flags, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_validate_rows<<<grid_for(n), kThreads, 0, s>>>(col_ptr, row_idx, n, nnz, sd, flags);
  return cudaGetLastError();
}

// ------------------------------------------------------------ batches
__device__ __forceinline__ int upper_bound_sys(const int* off, int count, long long v) {
  // largest s with off[s] <= v
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= v) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void k_batch_cols(const int* __restrict__ col_ptr_cat, int count, const int* __restrict__ sys_off,
                             const int* __restrict__ sys_eoff, const int* __restrict__ sys_sub, int n, int nnz,
                             int* col_ptr, unsigned char* dir, int* sys_of, int* flags) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  if (blockIdx.x == 0 && threadIdx.x == 0) col_ptr[n] = nnz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += stride) {
    const int sy = upper_bound_sys(sys_off, count, c);
    const long long local = c - sys_off[sy];
    const int len = (sy + 1 < count ? sys_off[sy + 1] : n) - sys_off[sy];
    const int* cp = col_ptr_cat + sys_off[sy] + sy;
    const int enz = (sy + 1 < count ? sys_eoff[sy + 1] : nnz) - sys_eoff[sy];
    if (local == 0 && (cp[0] != 0 || cp[len] != enz)) atomicOr(flags, SF_BAD_PTR);
    col_ptr[c] = sys_eoff[sy] + cp[local];
    dir[c] = static_cast<unsigned char>(sys_sub[sy]);
    sys_of[c] = sy;
  }
}
__global__ void k_batch_rows(const int* __restrict__ row_idx_cat, int count, const int* __restrict__ sys_off,
                             const int* __restrict__ sys_eoff, int n, int nnz, int* row_idx, int* flags) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nnz; e += stride) {
    const int sy = upper_bound_sys(sys_eoff, count, e);
    const int local = row_idx_cat[e];
    const int len = (sy + 1 < count ? sys_off[sy + 1] : n) - sys_off[sy];
    if (local < 0 || local >= len) atomicOr(flags, SF_ROW_RANGE);
    row_idx[e] = sys_off[sy] + local;
  }
}
cudaError_t launch_batch_merge(const int* col_ptr_cat, const int* row_idx_cat, int count, const int* sys_off,
                               const int* sys_eoff, const int* sys_sub, int n, int nnz, int* col_ptr, int* row_idx,
                               unsigned char* dir, int* sys_of, int* flags, cudaStream_t s) {
  k_batch_cols<<<grid_for(n > 0 ? n : 1), kThreads, 0, s>>>(col_ptr_cat, count, sys_off, sys_eoff, sys_sub, n, nnz,
                                                            col_ptr, dir, sys_of, flags);
  if (nnz > 0)
    k_batch_rows<<<grid_for(nnz), kThreads, 0, s>>>(row_idx_cat, count, sys_off, sys_eoff, n, nnz, row_idx, flags);
  return cudaGetLastError();
}

__device__ __forceinline__ void nat_of(const SysDesc& sd, int n, long long r, long long* off, long long* nat) {
  if (!sd.sys_of) {
    *off = 0;
    *nat = sd.substitution == 0 ? r : n - 1 - r;
    return;
  }
  const int sy = sd.sys_of[r];
  *off = sd.sys_off[sy];
  const long long local = r - *off;
  *nat = sd.dir[r] == 0 ? local : sd.sys_n[sy] - 1 - local;
}

__global__ void k_nat_rows(SysDesc sd, int n, int* rows_nat) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += stride) {
    long long off, nat;
    nat_of(sd, n, r, &off, &nat);
    rows_nat[off + nat] = static_cast<int>(r);
  }
}
cudaError_t launch_nat_rows(const SysDesc& sd, int n, int* rows_nat, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_nat_rows<<<grid_for(n), kThreads, 0, s>>>(sd, n, rows_nat);
  return cudaGetLastError();
}

// ------------------------------------------------------------ in-degree analyser
// inDeg[row] += 1 for every stored entry, diagonal included
// (reference: SpTRSV_cuda/sptrsv_syncfree_cuda.h:8-19). The caller zeroes inDeg.
// A row index outside [0, m) is skipped (never written) and, when `bad` is
// given, raises SF_ROW_RANGE there.
__global__ void k_in_degree(const int* __restrict__ row_idx, int m, int nnz, int* in_degree, int* bad) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nnz; e += stride) {
    const int r = row_idx[e];
    if (static_cast<unsigned>(r) < static_cast<unsigned>(m)) {
      atomicAdd(&in_degree[r], 1);
    } else if (bad) {
      atomicOr(bad, SF_ROW_RANGE);
    }
  }
}
cudaError_t launch_in_degree(const int* row_idx, int m, int nnz, int* in_degree, cudaStream_t s, int* bad) {
  if (nnz == 0) return cudaSuccess;
  k_in_degree<<<grid_for(nnz), kThreads, 0, s>>>(row_idx, m, nnz, in_degree, bad);
  return cudaGetLastError();
}

// ------------------------------------------------------------ exclusive scan
namespace {
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    int w = lane < nw ? s_warp[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < nw) s_warp[lane] = wi - w;
    if (lane == nw - 1) s_warp[32] = wi;
  }
  __syncthreads();
  const int excl = incl - v + s_warp[warp];
  *total = s_warp[32];
  __syncthreads();
  return excl;
}

__global__ void k_scan_tile_sums(const int* __restrict__ in, int count, int* sums) {
  __shared__ int s_warp[33];
  const long long base = (long long)blockIdx.x * kScanTile;
  int acc = 0;
  for (int i = 0; i < kScanItems; ++i) {
    const long long idx = base + (long long)i * kScanThreads + threadIdx.x;
    if (idx < count) acc += in[idx];
  }
  int total;
  block_exclusive_scan(acc, s_warp, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void k_scan_tiles(const int* __restrict__ in, int* out, int count, const int* __restrict__ carry,
                             int* total_out) {
  __shared__ int s_vals[kScanTile];
  __shared__ int s_warp[33];
  const long long base = (long long)blockIdx.x * kScanTile;
  for (int i = 0; i < kScanItems; ++i) {
    const int li = i * kScanThreads + threadIdx.x;
    const long long idx = base + li;
    s_vals[li] = idx < count ? in[idx] : 0;
  }
  __syncthreads();
  int local[kScanItems];
  int acc = 0;
  for (int i = 0; i < kScanItems; ++i) {
    local[i] = s_vals[threadIdx.x * kScanItems + i];
    acc += local[i];
  }
  int total;
  int run = block_exclusive_scan(acc, s_warp, &total) + (carry ? carry[blockIdx.x] : 0);
  for (int i = 0; i < kScanItems; ++i) {
    s_vals[threadIdx.x * kScanItems + i] = run;
    run += local[i];
  }
  __syncthreads();
  for (int i = 0; i < kScanItems; ++i) {
    const int li = i * kScanThreads + threadIdx.x;
    const long long idx = base + li;
    if (idx < count) out[idx] = s_vals[li];
  }
  if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == kScanThreads - 1) {
    *total_out = run;  // last thread's running value after its items = grand total
  }
}
}  // namespace

cudaError_t exclusive_scan_int(const int* in, int* out, int count, bool with_total, cudaStream_t s) {
  if (count <= 0) {
    if (with_total) return cudaMemsetAsync(out, 0, sizeof(int), s);
    return cudaSuccess;
  }
  const int tiles = (count + kScanTile - 1) / kScanTile;
  int* total_ptr = with_total ? out + count : nullptr;
  if (tiles == 1) {
    k_scan_tiles<<<1, kScanThreads, 0, s>>>(in, out, count, nullptr, total_ptr);
    return cudaGetLastError();
  }
  int* sums = nullptr;
  cudaError_t err = cudaMallocAsync(reinterpret_cast<void**>(&sums), sizeof(int) * (size_t)(tiles + 1), s);
  if (err != cudaSuccess) return err;
  k_scan_tile_sums<<<tiles, kScanThreads, 0, s>>>(in, count, sums);
  err = cudaGetLastError();
  if (err == cudaSuccess) err = exclusive_scan_int(sums, sums, tiles, false, s);
  if (err == cudaSuccess) {
    k_scan_tiles<<<tiles, kScanThreads, 0, s>>>(in, out, count, sums, total_ptr);
    err = cudaGetLastError();
  }
  cudaError_t e2 = cudaFreeAsync(sums, s);
  return err != cudaSuccess ? err : e2;
}

// ------------------------------------------------------------ stable radix sort
namespace {
constexpr int kRsThreads = 256;
constexpr int kRsItems = 8;
constexpr int kRsTile = kRsThreads * kRsItems;
constexpr int kRsBins = 256;

__global__ void k_rs_hist(const unsigned* __restrict__ keys, int count, int shift, int* hist, int nblocks) {
  __shared__ int s_h[kRsBins];
  s_h[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kRsTile;
  for (int i = 0; i < kRsItems; ++i) {
    const long long idx = base + (long long)i * kRsThreads + threadIdx.x;
    if (idx < count) atomicAdd(&s_h[(keys[idx] >> shift) & 0xFFu], 1);
  }
  __syncthreads();
  hist[threadIdx.x * nblocks + blockIdx.x] = s_h[threadIdx.x];
}

// Stable scatter: elements are ranked in index order within the tile (iteration
// by iteration, warp by warp, lane by lane), so equal digits keep input order.
__global__ void k_rs_scatter(const unsigned* __restrict__ keys_in, const int* __restrict__ vals_in,
                             unsigned* keys_out, int* vals_out, int count, int shift,
                             const int* __restrict__ offsets, int nblocks) {
  constexpr int kWarps = kRsThreads / 32;
  __shared__ int s_cnt[kWarps][kRsBins];
  __shared__ int s_off[kWarps][kRsBins];
  __shared__ int s_run[kRsBins];
  __shared__ int s_base[kRsBins];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  s_run[threadIdx.x] = 0;
  s_base[threadIdx.x] = offsets[threadIdx.x * nblocks + blockIdx.x];
  const long long base = (long long)blockIdx.x * kRsTile;
  for (int it = 0; it < kRsItems; ++it) {
    for (int w = 0; w < kWarps; ++w) s_cnt[w][threadIdx.x] = 0;
    __syncthreads();
    const long long idx = base + (long long)it * kRsThreads + threadIdx.x;
    const bool valid = idx < count;
    unsigned key = 0;
    int val = 0;
    int digit = kRsBins;  // out-of-range elements form their own group
    if (valid) {
      key = keys_in[idx];
      val = vals_in[idx];
      digit = static_cast<int>((key >> shift) & 0xFFu);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    const int leader = __ffs(peers) - 1;
    if (valid && lane == leader) s_cnt[warp][digit] = __popc(peers);
    __syncthreads();
    {
      int run = s_run[threadIdx.x];
      for (int w = 0; w < kWarps; ++w) {
        s_off[w][threadIdx.x] = run;
        run += s_cnt[w][threadIdx.x];
      }
      s_run[threadIdx.x] = run;
    }
    __syncthreads();
    if (valid) {
      const int pos = s_base[digit] + s_off[warp][digit] + rank;
      keys_out[pos] = key;
      vals_out[pos] = val;
    }
    __syncthreads();
  }
}
}  // namespace

size_t radix_sort_temp_bytes(int count) {
  const size_t nblocks = (size_t)((count + kRsTile - 1) / kRsTile);
  // histogram (+1 for the scan total), ping-pong keys and values
  return ((nblocks * kRsBins + 1) * sizeof(int) + 255) / 256 * 256 + (size_t)count * 8 + 512;
}

cudaError_t radix_sort_pairs(const unsigned* keys_in, const int* vals_in, unsigned* keys_out, int* vals_out,
                             int count, int key_bits, void* temp, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  const int nblocks = (count + kRsTile - 1) / kRsTile;
  int* hist = static_cast<int*>(temp);
  const size_t hist_bytes = (((size_t)nblocks * kRsBins + 1) * sizeof(int) + 255) / 256 * 256;
  unsigned* k_tmp = reinterpret_cast<unsigned*>(static_cast<char*>(temp) + hist_bytes);
  int* v_tmp = reinterpret_cast<int*>(k_tmp + count);
  int passes = (key_bits + 7) / 8;
  if (passes < 1) passes = 1;
  // Ping-pong so that the last pass lands in the output arrays.
  const unsigned* src_k = keys_in;
  const int* src_v = vals_in;
  for (int p = 0; p < passes; ++p) {
    const bool to_out = ((passes - 1 - p) % 2) == 0;
    unsigned* dk = to_out ? keys_out : k_tmp;
    int* dv = to_out ? vals_out : v_tmp;
    k_rs_hist<<<nblocks, kRsThreads, 0, s>>>(src_k, count, p * 8, hist, nblocks);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    err = exclusive_scan_int(hist, hist, nblocks * kRsBins, false, s);
    if (err != cudaSuccess) return err;
    k_rs_scatter<<<nblocks, kRsThreads, 0, s>>>(src_k, src_v, dk, dv, count, p * 8, hist, nblocks);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    src_k = dk;
    src_v = dv;
  }
  return cudaSuccess;
}

// ------------------------------------------------------------ small helpers
__global__ void k_iota(int* out, int count, int start, int step) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride)
    out[i] = start + static_cast<int>(i) * step;
}
cudaError_t launch_iota(int* out, int count, int start, int step, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_iota<<<grid_for(count), kThreads, 0, s>>>(out, count, start, step);
  return cudaGetLastError();
}

__global__ void k_expand_cols(const int* __restrict__ col_ptr, int n, int* col_of) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += stride)
    for (int e = col_ptr[c]; e < col_ptr[c + 1]; ++e) col_of[e] = static_cast<int>(c);
}
cudaError_t launch_expand_cols(const int* col_ptr, int n, int* col_of, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_expand_cols<<<grid_for(n), kThreads, 0, s>>>(col_ptr, n, col_of);
  return cudaGetLastError();
}

__global__ void k_copy_keys(const int* __restrict__ in, unsigned* out, int count) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride)
    out[i] = static_cast<unsigned>(in[i]);
}
cudaError_t launch_copy_keys(const int* in, unsigned* out, int count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_copy_keys<<<grid_for(count), kThreads, 0, s>>>(in, out, count);
  return cudaGetLastError();
}

__global__ void k_gather_int(const int* __restrict__ src, const int* __restrict__ idx, int* out, int count) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride)
    out[i] = src[idx[i]];
}
cudaError_t launch_gather_int(const int* src, const int* idx, int* out, int count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_gather_int<<<grid_for(count), kThreads, 0, s>>>(src, idx, out, count);
  return cudaGetLastError();
}

// ------------------------------------------------------------ ready-order lists
// The fast (non-exact) executors consume a dependency list in batches and only
// move to the next batch once the current one has arrived. Listing each
// position's dependencies in the order they complete (ascending position for a
// forward walk, descending for the reverse walk) leaves only the final batch
// waiting on the last publication, instead of whatever followed it in the
// serial (column) order.
__global__ void k_rank_keys(const int* __restrict__ pos, int count, int n, int descending, unsigned* keys) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride)
    keys[i] = static_cast<unsigned>(descending ? n - 1 - pos[i] : pos[i]);
}
__global__ void k_owner_keys(const int* __restrict__ owner, const int* __restrict__ idx, int count, unsigned* keys) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride)
    keys[i] = static_cast<unsigned>(owner[idx[i]]);
}

cudaError_t launch_sort_lists(const int* ptr, const int* pos, const int* src, int n, int count, bool descending,
                              int* pos_out, int* src_out, cudaStream_t s) {
  if (count <= 0 || n <= 0) return cudaSuccess;
  int bits = 1;
  while (bits < 31 && (1u << bits) <= static_cast<unsigned>(n - 1)) ++bits;
  unsigned *k1 = nullptr, *k2 = nullptr;
  int *v1 = nullptr, *v2 = nullptr;
  void* temp = nullptr;
  auto run = [&]() -> cudaError_t {
    cudaError_t err;
    if ((err = cudaMallocAsync(reinterpret_cast<void**>(&k1), sizeof(unsigned) * count, s)) != cudaSuccess) return err;
    if ((err = cudaMallocAsync(reinterpret_cast<void**>(&k2), sizeof(unsigned) * count, s)) != cudaSuccess) return err;
    if ((err = cudaMallocAsync(reinterpret_cast<void**>(&v1), sizeof(int) * count, s)) != cudaSuccess) return err;
    if ((err = cudaMallocAsync(reinterpret_cast<void**>(&v2), sizeof(int) * count, s)) != cudaSuccess) return err;
    if ((err = cudaMallocAsync(&temp, radix_sort_temp_bytes(count), s)) != cudaSuccess) return err;
    // entries by position of the dependency, then (stable) by owning position
    k_rank_keys<<<grid_for(count), kThreads, 0, s>>>(pos, count, n, descending ? 1 : 0, k1);
    if ((err = launch_iota(v1, count, 0, 1, s)) != cudaSuccess) return err;
    if ((err = radix_sort_pairs(k1, v1, k2, v2, count, bits, temp, s)) != cudaSuccess) return err;
    if ((err = launch_expand_cols(ptr, n, v1, s)) != cudaSuccess) return err;
    k_owner_keys<<<grid_for(count), kThreads, 0, s>>>(v1, v2, count, k1);
    if ((err = radix_sort_pairs(k1, v2, k2, v1, count, bits, temp, s)) != cudaSuccess) return err;
    if ((err = launch_gather_int(pos, v1, pos_out, count, s)) != cudaSuccess) return err;
    if ((err = launch_gather_int(src, v1, src_out, count, s)) != cudaSuccess) return err;
    return cudaGetLastError();
  };
  const cudaError_t err = run();
  // temporaries are released on every path (stream-ordered after their last use)
  if (k1) cudaFreeAsync(k1, s);
  if (k2) cudaFreeAsync(k2, s);
  if (v1) cudaFreeAsync(v1, s);
  if (v2) cudaFreeAsync(v2, s);
  if (temp) cudaFreeAsync(temp, s);
  return err;
}

// ------------------------------------------------------------ schedule heuristics
// Off-diagonal entries whose row and column fall in the same block of `block`
// unknowns of the natural execution order (ascending for a forward solve,
// descending for a backward one): how much of the DAG a blocked order keeps
// inside one CTA.
__global__ void k_block_locality(const int* __restrict__ row, const int* __restrict__ col, int nnz, int n,
                                 int block, int backward, unsigned long long* count) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned local = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nnz; i += stride) {
    const int r = row[i], c = col[i];
    if (r == c) continue;
    const int pr = backward ? n - 1 - r : r, pc = backward ? n - 1 - c : c;
    local += (pr / block == pc / block) ? 1u : 0u;
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, (unsigned long long)local);
}

cudaError_t launch_block_locality(const int* row, const int* col, int nnz, int n, int block, bool backward,
                                  unsigned long long* count, cudaStream_t s) {
  if (nnz <= 0) return cudaSuccess;
  k_block_locality<<<grid_for(nnz), kThreads, 0, s>>>(row, col, nnz, n, block, backward ? 1 : 0, count);
  return cudaGetLastError();
}

// Unknowns with two or more dependencies on the level just before their own
// (count[0]; in a warp-synchronous loop those dependencies land in the same
// iteration) and unknowns with any dependency (count[1]), over the CSR rows
// (diagonal included in each row and skipped here).
__global__ void k_coarrival(const int* __restrict__ row_ptr, const int* __restrict__ col,
                            const int* __restrict__ depth, int n, unsigned long long* count) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned co = 0, any = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int prev = depth[i] - 1;
    int k = 0, deps = 0;
    for (int e = row_ptr[i]; e < row_ptr[i + 1]; ++e) {
      const int c = col[e];
      if (c == i) continue;
      ++deps;
      k += depth[c] == prev ? 1 : 0;
    }
    co += k >= 2 ? 1u : 0u;
    any += deps > 0 ? 1u : 0u;
  }
  for (int o = 16; o > 0; o >>= 1) {
    co += __shfl_xor_sync(0xffffffffu, co, o);
    any += __shfl_xor_sync(0xffffffffu, any, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (co) atomicAdd(&count[0], (unsigned long long)co);
    if (any) atomicAdd(&count[1], (unsigned long long)any);
  }
}

cudaError_t launch_coarrival(const int* row_ptr, const int* col, const int* depth, int n, unsigned long long* count,
                             cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_coarrival<<<grid_for(n), kThreads, 0, s>>>(row_ptr, col, depth, n, count);
  return cudaGetLastError();
}

// ------------------------------------------------------------ level sets
// Breadth-first peeling of the in-degree, one grid barrier per level
// (the level definition of SpTRSV_cuda/findlevel.h:6-69): level 0 holds rows
// whose only entry is the diagonal; a row joins level l+1 when the last of its
// dependencies is visited at level l. Cooperative launch (all CTAs resident).
__global__ void k_levels(const int* __restrict__ col_ptr, const int* __restrict__ row_idx,
                         const int* __restrict__ in_degree, int n, int* cnt, int* front_a, int* front_b,
                         int* depth, int* level_sizes, DeviceCtl* ctl, unsigned long long timeout_ns,
                         int* tails /* [4]: three rotating tails + level count */, unsigned smin, unsigned smax) {
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = tid; i < n; i += stride) {
    const int d = in_degree[i];
    cnt[i] = d;
    if (d == 1) {
      const int slot = atomicAdd(&tails[0], 1);
      front_a[slot] = static_cast<int>(i);
      depth[i] = 0;
    }
  }
  if (!grid_barrier(ctl, timeout_ns, smin, smax)) return;
  int* cur = front_a;
  int* nxt = front_b;
  for (int level = 0;; ++level) {
    const int cur_tail = level % 3, nxt_tail = (level + 1) % 3, free_tail = (level + 2) % 3;
    const int size = *reinterpret_cast<volatile int*>(&tails[cur_tail]);
    if (size == 0) {
      if (tid == 0) tails[3] = level;
      break;
    }
    if (tid == 0) {
      level_sizes[level] = size;
      tails[free_tail] = 0;
    }
    // one warp per frontier node, lanes over the node's column entries
    const long long warp = tid >> 5;
    const long long nwarps = stride >> 5;
    const int lane = static_cast<int>(tid & 31);
    for (long long q = warp; q < size; q += nwarps) {
      const int node = cur[q];
      for (int e = col_ptr[node] + lane; e < col_ptr[node + 1]; e += 32) {
        const int r = row_idx[e];
        if (r == node) continue;
        const int old = atomicSub(&cnt[r], 1);
        if (old == 2) {
          const int slot = atomicAdd(&tails[nxt_tail], 1);
          nxt[slot] = r;
          depth[r] = level + 1;
        }
      }
    }
    if (!grid_barrier(ctl, timeout_ns, smin, smax)) return;
    int* t = cur;
    cur = nxt;
    nxt = t;
  }
}

cudaError_t launch_levels(const int* col_ptr, const int* row_idx, const int* in_degree, int n, int* cnt_scratch,
                          int* front_a, int* front_b, int* depth, int* level_sizes, DeviceCtl* ctl,
                          unsigned long long timeout_ns, cudaStream_t s) {
  // tails live right after level_sizes[n+1]
  int* tails = level_sizes + n + 1;
  cudaError_t err = cudaMemsetAsync(tails, 0, 4 * sizeof(int), s);
  if (err != cudaSuccess) return err;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // one CTA per SM and a short back-off in the per-level grid barrier: deep
  // DAGs pay one barrier per level (2M-row mesh, 2,827 levels: analysis 41.1
  // ms with four CTAs per SM and 32-256 ns back-off, 36.4 with this; a
  // 200k-row chain 973 vs 694 ms; wide power-law levels unchanged)
  unsigned smin = 16, smax = 64;
  int grid = sms;
  void* args[] = {(void*)&col_ptr, (void*)&row_idx, (void*)&in_degree, (void*)&n, (void*)&cnt_scratch,
                  (void*)&front_a, (void*)&front_b, (void*)&depth, (void*)&level_sizes, (void*)&ctl,
                  (void*)&timeout_ns, (void*)&tails, (void*)&smin, (void*)&smax};
  return cudaLaunchCooperativeKernel((void*)k_levels, dim3(grid), dim3(kThreads), args, 0, s);
}

// ------------------------------------------------------------ schedule
// mode 0: key = depth (level order); mode 1: key = natural position / block
// (second, stable pass of the blocked level order).
// mode 0: key = depth (level order); mode 1: key = (natural position inside its
// system / block) * count + system (second, stable pass of the blocked level
// order; batches interleave their systems block by block).
__global__ void k_schedule_keys(const int* __restrict__ rows, const int* __restrict__ depth, int n, SysDesc sd,
                                int block, int mode, unsigned* keys, const int* __restrict__ sys_depth,
                                int max_depth) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int r = rows[i];
    if (mode == 0) {
      keys[i] = static_cast<unsigned>(depth[r]);
    } else if (mode == 2) {
      // the level stretched to max(D_s, T) keys, T = max_depth (the stretch
      // target): floor(level * max(D_s, T) / D_s) grows strictly with the
      // level inside system s
      const long long ds = sys_depth[sd.sys_of[r]] > 0 ? sys_depth[sd.sys_of[r]] : 1;
      const long long span = ds > max_depth ? ds : max_depth;
      keys[i] = static_cast<unsigned>((long long)depth[r] * span / ds);
    } else {
      long long off, nat;
      nat_of(sd, n, r, &off, &nat);
      const long long sy = sd.sys_of ? sd.sys_of[r] : 0;
      keys[i] = static_cast<unsigned>((nat / block) * sd.count + sy);
    }
  }
}
cudaError_t launch_schedule_keys(const int* rows, const int* depth, int n, const SysDesc& sd, int block, int mode,
                                 unsigned* keys, cudaStream_t s, const int* sys_depth, int max_depth) {
  if (n <= 0) return cudaSuccess;
  k_schedule_keys<<<grid_for(n), kThreads, 0, s>>>(rows, depth, n, sd, block, mode, keys, sys_depth, max_depth);
  return cudaGetLastError();
}

// sys_depth[s] = 1 + the deepest level of system s (zeroed by the caller)
__global__ void k_sys_depth(const int* __restrict__ depth, const int* __restrict__ sys_of, int n, int* sys_depth) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += stride)
    atomicMax(&sys_depth[sys_of[r]], depth[r] + 1);
}
cudaError_t launch_sys_depth(const int* depth, const int* sys_of, int n, int* sys_depth, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_sys_depth<<<grid_for(n), kThreads, 0, s>>>(depth, sys_of, n, sys_depth);
  return cudaGetLastError();
}

__global__ void k_long_keys(const int* __restrict__ rows, const int* __restrict__ in_degree, int n, int threshold,
                            unsigned* keys) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
    keys[i] = in_degree[rows[i]] - 1 > threshold ? 0u : 1u;
}
cudaError_t launch_long_keys(const int* rows, const int* in_degree, int n, int threshold, unsigned* keys,
                             cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_long_keys<<<grid_for(n), kThreads, 0, s>>>(rows, in_degree, n, threshold, keys);
  return cudaGetLastError();
}

__global__ void k_inverse_perm(const int* __restrict__ perm, int n, int* iperm) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += stride)
    iperm[perm[p]] = static_cast<int>(p);
}
cudaError_t launch_inverse_perm(const int* perm, int n, int* iperm, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_inverse_perm<<<grid_for(n), kThreads, 0, s>>>(perm, n, iperm);
  return cudaGetLastError();
}

__global__ void k_dep_counts(const int* __restrict__ perm, const int* __restrict__ in_degree, int n, int* counts) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += stride)
    counts[p] = in_degree[perm[p]] - 1;
}
cudaError_t launch_dep_counts(const int* perm, const int* in_degree, int n, int* counts, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_dep_counts<<<grid_for(n), kThreads, 0, s>>>(perm, in_degree, n, counts);
  return cudaGetLastError();
}

__global__ void k_out_counts(const int* __restrict__ perm, const int* __restrict__ col_ptr, int n, int* counts) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += stride) {
    const int c = perm[p];
    counts[p] = col_ptr[c + 1] - col_ptr[c] - 1;
  }
}
cudaError_t launch_out_counts(const int* perm, const int* col_ptr, int n, int* counts, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_out_counts<<<grid_for(n), kThreads, 0, s>>>(perm, col_ptr, n, counts);
  return cudaGetLastError();
}

// Dependencies of position p in the order the serial executor accumulates
// them: ascending column for a forward solve, descending for a backward one
// (SpTRSV_cuda/sptrsv_syncfree_serialref.h:76-103 and :105-133).
__global__ void k_fill_pull(const int* __restrict__ perm, const int* __restrict__ iperm,
                            const int* __restrict__ csr_ptr, const int* __restrict__ csr_col,
                            const int* __restrict__ csr_src, const int* __restrict__ dep_ptr, int n,
                            SysDesc sd, int* dep_pos, int* dep_src, int* dep_col, int* diag_src) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += stride) {
    const int r = perm[p];
    const int substitution = dir_of(sd, r);
    const int beg = csr_ptr[r], end = csr_ptr[r + 1];
    int out = dep_ptr[p];
    if (substitution == 0) {
      for (int k = beg; k < end - 1; ++k, ++out) {
        dep_pos[out] = iperm[csr_col[k]];
        dep_src[out] = csr_src[k];
        dep_col[out] = csr_col[k];
      }
      diag_src[p] = csr_src[end - 1];
    } else {
      for (int k = end - 1; k > beg; --k, ++out) {
        dep_pos[out] = iperm[csr_col[k]];
        dep_src[out] = csr_src[k];
        dep_col[out] = csr_col[k];
      }
      diag_src[p] = csr_src[beg];
    }
  }
}
cudaError_t launch_fill_pull(const int* perm, const int* iperm, const int* csr_ptr, const int* csr_col,
                             const int* csr_src, const int* dep_ptr, int n, const SysDesc& sd, int* dep_pos,
                             int* dep_src, int* dep_col, int* diag_src, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_fill_pull<<<grid_for(n), kThreads, 0, s>>>(perm, iperm, csr_ptr, csr_col, csr_src, dep_ptr, n, sd,
                                                dep_pos, dep_src, dep_col, diag_src);
  return cudaGetLastError();
}

// Dependents of position p (its column's off-diagonal entries), listed in the
// order the serial executor run on the transpose accumulates them: descending
// row for a lower triangle (its transpose is solved backward), ascending for an
// upper one. The push executor is order-agnostic; the adjoint solve relies on it.
__global__ void k_fill_push(const int* __restrict__ perm, const int* __restrict__ iperm,
                            const int* __restrict__ col_ptr, const int* __restrict__ row_idx,
                            const int* __restrict__ out_ptr, int n, SysDesc sd, int* out_pos, int* out_src) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += stride) {
    const int c = perm[p];
    const int substitution = dir_of(sd, c);
    int out = out_ptr[p];
    if (substitution == 0) {
      for (int e = col_ptr[c + 1] - 1; e > col_ptr[c]; --e, ++out) {
        out_pos[out] = iperm[row_idx[e]];
        out_src[out] = e;
      }
    } else {
      for (int e = col_ptr[c]; e < col_ptr[c + 1] - 1; ++e, ++out) {
        out_pos[out] = iperm[row_idx[e]];
        out_src[out] = e;
      }
    }
  }
}
cudaError_t launch_fill_push(const int* perm, const int* iperm, const int* col_ptr, const int* row_idx,
                             const int* out_ptr, int n, const SysDesc& sd, int* out_pos, int* out_src,
                             cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_fill_push<<<grid_for(n), kThreads, 0, s>>>(perm, iperm, col_ptr, row_idx, out_ptr, n, sd, out_pos,
                                                out_src);
  return cudaGetLastError();
}

// ------------------------------------------------------------ value staging
template <typename TV, typename T>
__global__ void k_stage_edges(const TV* __restrict__ val, const int* __restrict__ src, T* out, int count) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride)
    out[i] = static_cast<T>(val[src[i]]);
}
template <typename TV, typename T>
__global__ void k_stage_diag(const TV* __restrict__ val, const int* __restrict__ diag_src, T* diag, T* rcp, int n,
                             int* flags) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += stride) {
    const T d = static_cast<T>(val[diag_src[p]]);
    diag[p] = d;
    rcp[p] = T(1) / d;
    if (!(d != T(0)) || !isfinite(d)) atomicOr(flags, SF_ZERO_DIAG);
  }
}

// w = v * (1/diag of the dependent row): x_p = b_p/d_p - sum_j w_j x_j needs one
// fused multiply-add per dependency once the reciprocal is folded in. The scaled
// lists follow the ready order (src_f), the plain ones the serial order.
template <typename TV, typename T>
__global__ void k_stage_scaled(const int* __restrict__ ptr, const TV* __restrict__ val, const int* __restrict__ src_f,
                               const T* __restrict__ rcp, T* w, int n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += stride) {
    const T r = rcp[p];
    for (int e = ptr[p]; e < ptr[p + 1]; ++e) w[e] = static_cast<T>(val[src_f[e]]) * r;
  }
}

template <typename TV, typename T>
cudaError_t launch_stage_values(const Layout& L, const TV* val, Values<T>& V, int* flags, cudaStream_t s) {
  if (L.ndep > 0) {
    k_stage_edges<TV, T><<<grid_for(L.ndep), kThreads, 0, s>>>(val, L.dep_src, V.dep_val, L.ndep);
    k_stage_edges<TV, T><<<grid_for(L.ndep), kThreads, 0, s>>>(val, L.out_src, V.out_val, L.ndep);
  }
  if (L.n > 0) k_stage_diag<TV, T><<<grid_for(L.n), kThreads, 0, s>>>(val, L.diag_src, V.diag, V.rcp, L.n, flags);
  if (L.n > 0 && L.ndep > 0) {
    k_stage_scaled<TV, T><<<grid_for(L.n), kThreads, 0, s>>>(L.dep_ptr, val, L.dep_src_f, V.rcp, V.dep_w, L.n);
    k_stage_scaled<TV, T><<<grid_for(L.n), kThreads, 0, s>>>(L.out_ptr, val, L.out_src_f, V.rcp, V.out_w, L.n);
  }
  return cudaGetLastError();
}

template cudaError_t launch_stage_values<double, double>(const Layout&, const double*, Values<double>&, int*,
                                                          cudaStream_t);
template cudaError_t launch_stage_values<double, float>(const Layout&, const double*, Values<float>&, int*,
                                                         cudaStream_t);
template cudaError_t launch_stage_values<float, float>(const Layout&, const float*, Values<float>&, int*,
                                                        cudaStream_t);

}  // namespace sptrsv
