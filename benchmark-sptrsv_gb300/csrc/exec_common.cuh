// Device helpers shared by the executor translation units.
#pragma once
#include "common.cuh"

namespace sptrsv {

// Claim the next chunk for this CTA (uniform across the CTA).
__device__ __forceinline__ unsigned next_chunk(DeviceCtl* ctl, unsigned nchunks, unsigned* s_chunk) {
  if (threadIdx.x == 0) *s_chunk = ctl_failed(ctl) ? nchunks : atomicAdd(&ctl->ticket, 1u);
  __syncthreads();
  const unsigned c = *s_chunk;
  __syncthreads();
  return c;
}

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

// Accumulates the dependencies e = e_first, e_first + STRIDE, ... < e_end of
// one unknown into acc: acc -= w_e * x_q (any order), or with EXACT the serial
// executor's product-then-sum in list order. The index/value loads and the
// flag loads of U dependencies are issued together; every dependency still
// unpublished is re-polled together on each retry, so once the last one is
// published the wait ends within one poll round trip, whatever the list
// length. local_slot(q) gives the shared-memory slot of an in-chunk
// dependency, or -1 for one read from global memory (which backs off between
// polls, sleep_min..sleep_max ns). Returns false on timeout / failure.
template <typename T, bool EXACT, int U, int STRIDE, class LocalSlot>
__device__ __forceinline__ bool gather_deps(const int* __restrict__ pos, const T* __restrict__ val, int e_first,
                                            int e_end, const T* xw, const T* s_x, LocalSlot local_slot,
                                            DeviceCtl* ctl, unsigned long long timeout, int where,
                                            unsigned sleep_min, unsigned sleep_max, T& acc) {
  using F = Flag<T>;
  using Bits = typename F::Bits;
  for (int e = e_first; e < e_end; e += U * STRIDE) {
    int q[U], ls[U];
    T w[U];
    Bits bits[U];
    unsigned todo = 0u;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int ee = e + u * STRIDE;
      q[u] = ee < e_end ? pos[ee] : -1;
      w[u] = ee < e_end ? val[ee] : T(0);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      ls[u] = -1;
      bits[u] = F::EMPTY;
      if (q[u] >= 0) {
        ls[u] = local_slot(q[u]);
        bits[u] = ls[u] >= 0 ? F::load_shared(&s_x[ls[u]]) : F::load(&xw[q[u]]);
        todo |= 1u << u;
      }
    }
    WaitBudget wb(timeout);
    unsigned nap = sleep_min;
    unsigned local_spins = 0u;
    for (;;) {
      bool prefix = true;
      unsigned global_pending = 0u;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (!(todo & (1u << u))) continue;
        if (bits[u] != F::EMPTY && (!EXACT || prefix)) {
          acc = EXACT ? exact_mul_add<T>(acc, w[u], F::value(bits[u])) : fma(-w[u], F::value(bits[u]), acc);
          todo &= ~(1u << u);
        } else {
          prefix = false;
          if (bits[u] == F::EMPTY && ls[u] < 0) global_pending |= 1u << u;
        }
      }
      if (!todo) break;
      if (global_pending && sleep_max) {
        __nanosleep(nap);
        nap = nap * 2u < sleep_max ? nap * 2u : sleep_max;
      }
      // spins on shared memory only skip the (global-memory) status and timer
      // checks most of the time, so an in-chunk hop stays a few dozen cycles
      if ((global_pending || (++local_spins & 255u) == 0u) && !wb.poll(ctl, where)) return false;
#pragma unroll
      for (int u = 0; u < U; ++u)
        if ((todo & (1u << u)) && bits[u] == F::EMPTY)
          bits[u] = ls[u] >= 0 ? F::load_shared(&s_x[ls[u]]) : F::load(&xw[q[u]]);
    }
  }
  return true;
}

}  // namespace sptrsv
