// Mixed-precision support kernels: the FP64 residual r = b - L x (written as
// FP32 for the next FP32 correction solve), FP64/FP32 conversions, and the
// FP64 update x += d with the max-norms the host uses to stop refining.
#include "internal.h"

namespace sptrsv {

namespace {
inline int grid_1d(long long count, int threads = 256) {
  long long g = (count + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > (1 << 20)) g = 1 << 20;
  return static_cast<int>(g);
}
}  // namespace

template <typename TI, typename TO>
__global__ void k_cast(const TI* __restrict__ in, TO* out, long long count) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride)
    out[i] = static_cast<TO>(in[i]);
}

// r[row,k] = b[row,k] - sum over the stored entries of row `row` of L(row,j) x[j,k],
// accumulated in FP64 from FP64 values; G lanes of a group split the right-hand sides.
template <int G>
__global__ void k_residual(int n, int rhs, const int* __restrict__ perm, const int* __restrict__ dep_ptr,
                           const int* __restrict__ dep_col, const double* __restrict__ dep_val,
                           const double* __restrict__ diag, const double* __restrict__ b,
                           const double* __restrict__ x, long long si, long long sk, float* r) {
  const int lane = threadIdx.x % G;
  const long long group = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / G;
  const long long ngroups = ((long long)gridDim.x * blockDim.x) / G;
  for (long long p = group; p < n; p += ngroups) {
    const long long row = perm[p];
    const int e0 = dep_ptr[p], e1 = dep_ptr[p + 1];
    const double d = diag[p];
    for (int k = lane; k < rhs; k += G) {
      const long long o = row * si + (long long)k * sk;
      double acc = fma(-d, x[o], b[o]);
      for (int e = e0; e < e1; ++e) acc = fma(-dep_val[e], x[(long long)dep_col[e] * si + (long long)k * sk], acc);
      r[o] = static_cast<float>(acc);
    }
  }
}

// x += d; stats[0] = max |d|, stats[1] = max |x| (as ordered bit patterns of
// non-negative doubles).
__global__ void k_update(double* x, const float* __restrict__ d, long long count, unsigned long long* stats) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  double dmax = 0.0, xmax = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride) {
    const double di = static_cast<double>(d[i]);
    const double xi = x[i] + di;
    x[i] = xi;
    dmax = fmax(dmax, fabs(di));
    xmax = fmax(xmax, fabs(xi));
  }
  for (int o = 16; o > 0; o >>= 1) {
    dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    xmax = fmax(xmax, __shfl_xor_sync(0xffffffffu, xmax, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&stats[0], static_cast<unsigned long long>(__double_as_longlong(dmax)));
    atomicMax(&stats[1], static_cast<unsigned long long>(__double_as_longlong(xmax)));
  }
}

// stats[1] = max |x| (initial iterate), after x = (double) d.
__global__ void k_init_x(double* x, const float* __restrict__ d, long long count, unsigned long long* stats) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  double xmax = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride) {
    const double xi = static_cast<double>(d[i]);
    x[i] = xi;
    xmax = fmax(xmax, fabs(xi));
  }
  for (int o = 16; o > 0; o >>= 1) xmax = fmax(xmax, __shfl_xor_sync(0xffffffffu, xmax, o));
  if ((threadIdx.x & 31) == 0) atomicMax(&stats[1], static_cast<unsigned long long>(__double_as_longlong(xmax)));
}

// out[c * rows + r] = in[r * cols + c]: a rows x cols row-major matrix to its
// transpose, through 32 x 32 shared-memory tiles (coalesced on both sides);
// one CTA per tile, tiles numbered row-major over the input.
template <typename T>
__global__ void k_transpose(const T* __restrict__ in, T* __restrict__ out, int rows, int cols, long long ctiles) {
  __shared__ T tile[32][33];
  const long long t = blockIdx.x;
  const int r0 = static_cast<int>(t / ctiles) * 32, c0 = static_cast<int>(t % ctiles) * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[i][threadIdx.x] = in[(long long)r * cols + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[(long long)c * rows + r] = tile[threadIdx.x][i];
  }
}

template <typename T>
cudaError_t launch_transpose(const T* in, T* out, int rows, int cols, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  const long long rtiles = (rows + 31) / 32, ctiles = (cols + 31) / 32;
  if (rtiles * ctiles > 0x7fffffffLL) return cudaErrorInvalidValue;
  k_transpose<T><<<static_cast<unsigned>(rtiles * ctiles), dim3(32, 8), 0, s>>>(in, out, rows, cols, ctiles);
  return cudaGetLastError();
}
template cudaError_t launch_transpose<double>(const double*, double*, int, int, cudaStream_t);
template cudaError_t launch_transpose<float>(const float*, float*, int, int, cudaStream_t);

cudaError_t launch_cast_d2f(const double* in, float* out, long long count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_cast<double, float><<<grid_1d(count), 256, 0, s>>>(in, out, count);
  return cudaGetLastError();
}

cudaError_t launch_residual(const Layout& L, const Values<double>& V, int rhs, const double* b, const double* x,
                            long long si, long long sk, float* r, cudaStream_t s) {
  if (L.n == 0) return cudaSuccess;
  if (rhs >= 16) {
    k_residual<16><<<grid_1d((long long)L.n * 16), 256, 0, s>>>(L.n, rhs, L.perm, L.dep_ptr, L.dep_col, V.dep_val,
                                                                V.diag, b, x, si, sk, r);
  } else if (rhs >= 4) {
    k_residual<4><<<grid_1d((long long)L.n * 4), 256, 0, s>>>(L.n, rhs, L.perm, L.dep_ptr, L.dep_col, V.dep_val,
                                                              V.diag, b, x, si, sk, r);
  } else {
    k_residual<1><<<grid_1d(L.n), 256, 0, s>>>(L.n, rhs, L.perm, L.dep_ptr, L.dep_col, V.dep_val, V.diag, b, x, si,
                                               sk, r);
  }
  return cudaGetLastError();
}

cudaError_t launch_update(double* x, const float* d, long long count, unsigned long long* stats, bool first,
                          cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  const int grid = grid_1d(count, 256) > 4096 ? 4096 : grid_1d(count, 256);
  if (first) k_init_x<<<grid, 256, 0, s>>>(x, d, count, stats);
  else k_update<<<grid, 256, 0, s>>>(x, d, count, stats);
  return cudaGetLastError();
}

}  // namespace sptrsv
