// Allocation-free sync-free solve for callers that may not allocate device
// memory themselves: code running under a host framework that owns the whole
// device-memory budget (its caching allocator or a fixed pool must see every
// byte), and latency-critical loops that cannot accept the device-wide
// synchronisation a cudaMalloc/cudaFree can imply. The handle API allocates
// its analysis products and workspace; this entry point instead keeps its
// scratch (in-degree counters, partial sums, control words) in one
// file-scope device array that every GPU loading the library holds until the
// process exits.
//
// Limits and rules:
//  * at most kNoAllocMaxN unknowns, one right-hand side, FP64;
//  * the structure is validated on the device in the same stream before the
//    solve (column pointers, row range, order, diagonal placement, triangle);
//    malformed input returns SPTRSV_ERR_BAD_STRUCTURE and nothing past the
//    scratch array is ever written;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, once per device, with that device current); make
//    that first call before any stream capture;
//  * every call shares the array: the call clears what must start at zero,
//    and calls whose work overlaps on the GPU (other streams, other threads)
//    race on it — serialise them;
//  * no cudaMalloc, cudaFree or allocating library routine is called.
#include <mutex>

#include "../../include/sptrsv_gb300.h"
#include "internal.h"

namespace sptrsv {
namespace {

constexpr int kNoAllocMaxN = SPTRSV_NOALLOC_MAX_N;
constexpr size_t kCtlBytes = 256;     // DeviceCtl, then the structural flags word at kFlagsOffset
constexpr size_t kFlagsOffset = 128;
static_assert(sizeof(DeviceCtl) <= kFlagsOffset, "control block overlaps the flags word");
constexpr size_t kCounterBytes = sizeof(int) * (size_t)kNoAllocMaxN;
constexpr size_t kSumBytes = sizeof(double) * (size_t)kNoAllocMaxN;
constexpr size_t kScratchBytes = kCtlBytes + kCounterBytes + kSumBytes;

// [control block, flags | in-degree counters | partial sums]
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[64] = {nullptr};

// Device address of the scratch array for the current device (looked up once).
int scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SPTRSV_ERR_CUDA;
  if (dev < 0 || dev >= 64) return SPTRSV_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return SPTRSV_ERR_CUDA;
    }
    g_scratch_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_addr[dev];
  return SPTRSV_OK;
}

}  // namespace
}  // namespace sptrsv

extern "C" int sptrsv_gb300_solve_noalloc(const int* d_colPtr, const int* d_rowIdx, const double* d_val, int n,
                                          int nnz, int substitution, const double* d_b, double* d_x, void* stream) {
  using namespace sptrsv;
  if (n < 0 || nnz < 0 || (substitution != 0 && substitution != 1)) return SPTRSV_ERR_INVALID;
  if (n > kNoAllocMaxN) return SPTRSV_ERR_UNSUPPORTED;  // beyond the fixed scratch array
  if (n == 0) return SPTRSV_OK;
  if (!d_colPtr || !d_rowIdx || !d_val || !d_b || !d_x || nnz < n) return SPTRSV_ERR_INVALID;
  unsigned char* scratch = nullptr;
  const int st = scratch_for_current_device(&scratch);
  if (st != SPTRSV_OK) return st;
  auto* ctl = reinterpret_cast<DeviceCtl*>(scratch);
  auto* flags = reinterpret_cast<int*>(scratch + kFlagsOffset);
  auto* counters = reinterpret_cast<int*>(scratch + kCtlBytes);
  auto* left_sum = reinterpret_cast<double*>(scratch + kCtlBytes + kCounterBytes);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // clear what must start at zero: control words (ticket, error code) and the
  // flags word, partial sums, in-degree counters (rebuilt by the analyser)
  if (cudaMemsetAsync(scratch, 0, kCtlBytes, s) != cudaSuccess ||
      cudaMemsetAsync(left_sum, 0, sizeof(double) * (size_t)n, s) != cudaSuccess ||
      cudaMemsetAsync(counters, 0, sizeof(int) * (size_t)n, s) != cudaSuccess) {
    cudaGetLastError();
    return SPTRSV_ERR_CUDA;
  }
  // validation, analyser and executor in one stream: the executor does nothing
  // but record DEV_BAD_INPUT when validation raised a flag, and the analyser
  // skips rows outside [0, n), so malformed input never writes past the array
  SysDesc sd;
  sd.substitution = substitution;
  if (launch_validate_ptr(d_colPtr, n, nnz, flags, s) != cudaSuccess ||
      launch_validate_rows(d_colPtr, d_rowIdx, n, nnz, sd, flags, s) != cudaSuccess ||
      launch_in_degree(d_rowIdx, n, nnz, counters, s, flags) != cudaSuccess ||
      launch_ref_executor<double>(d_colPtr, d_rowIdx, d_val, counters, left_sum, n, substitution, 1,
                                  SPTRSV_OPT_WARP_AUTO, d_b, d_x, ctl, 1000000000ull, s, flags) != cudaSuccess) {
    cudaGetLastError();
    return SPTRSV_ERR_CUDA;
  }
  int code = 0;
  if (cudaMemcpyAsync(&code, &ctl->code, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    return SPTRSV_ERR_CUDA;
  }
  if (code == DEV_OK) return SPTRSV_OK;
  return code == DEV_BAD_INPUT ? SPTRSV_ERR_BAD_STRUCTURE : SPTRSV_ERR_TIMEOUT;
}
