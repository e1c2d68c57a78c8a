// Device helpers shared by the executor translation units.
#pragma once
#include "common.cuh"

namespace sptrsv {

// The last CTA to leave resets the chunk ticket so the next launch starts at 0.
__device__ __forceinline__ void leave(DeviceCtl* ctl) {
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned d = atomicAdd(&ctl->done, 1u);
    if (d == gridDim.x - 1) {
      ctl->ticket = 0;
      ctl->done = 0;
      __threadfence();
    }
  }
}

// Wait until the value-as-flag word at p is published; returns EMPTY on
// timeout or when another thread already failed. Global words back off
// between polls (sleep_min..sleep_max ns); shared-memory words do not sleep.
template <typename T, bool SHARED>
__device__ __forceinline__ typename Flag<T>::Bits wait_flag_dev(const T* p, DeviceCtl* ctl, unsigned long long timeout,
                                                                int where, unsigned sleep_min, unsigned sleep_max) {
  using F = Flag<T>;
  typename F::Bits bits = SHARED ? F::load_shared(p) : F::load(p);
  if (bits != F::EMPTY) return bits;
  WaitBudget w(timeout, SHARED ? 0u : sleep_min, SHARED ? 0u : sleep_max);
  do {
    if (!w.poll(ctl, where)) return F::EMPTY;
    bits = SHARED ? F::load_shared(p) : F::load(p);
  } while (bits == F::EMPTY);
  return bits;
}

// The serial executor's arithmetic: partial = partial + x*L (two roundings),
// x = (b - partial) / diag (true division). SpTRSV_cuda/sptrsv_syncfree_serialref.h:59, :68-71.
template <typename T>
__device__ __forceinline__ T exact_mul_add(T acc, T v, T xq);
template <>
__device__ __forceinline__ double exact_mul_add<double>(double acc, double v, double xq) {
  return __dadd_rn(acc, __dmul_rn(xq, v));
}
template <>
__device__ __forceinline__ float exact_mul_add<float>(float acc, float v, float xq) {
  return __fadd_rn(acc, __fmul_rn(xq, v));
}
template <typename T>
__device__ __forceinline__ T exact_finish(T bi, T acc, T diag);
template <>
__device__ __forceinline__ double exact_finish<double>(double bi, double acc, double diag) {
  return __ddiv_rn(__dsub_rn(bi, acc), diag);
}
template <>
__device__ __forceinline__ float exact_finish<float>(float bi, float acc, float diag) {
  return __fdiv_rn(__fsub_rn(bi, acc), diag);
}

}  // namespace sptrsv
