// Device-side building blocks shared by the analysis and solve kernels:
// scoped loads/stores/reductions written as PTX, bounded waits that report a
// timeout instead of spinning forever, and the status words the host reads.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sptrsv {

// Device status word bits (DeviceStatus::code).
constexpr int DEV_OK = 0;
constexpr int DEV_TIMEOUT = 1;         // a bounded wait ran out
constexpr int DEV_BAD_INPUT = 2;       // a kernel met data it cannot process

// Per-handle control block in device memory. Every field self-resets at the
// end of a successful launch, so consecutive solves need no host memset.
struct alignas(64) DeviceCtl {
  unsigned int ticket;      // next chunk to hand out
  unsigned int done;        // CTAs that left the chunk loop
  int code;                 // DEV_* (sticky until the host clears it)
  int where;                // diagnostic: position whose wait ran out
  unsigned int barrier_count;
  unsigned int barrier_gen;
  unsigned int pad[10];
};

// ------------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed_u32(unsigned* p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_release_add_u32(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_relaxed_add_u32(unsigned* p, unsigned v) {
  asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_add_f64(double* p, double v) {
  asm volatile("red.relaxed.gpu.global.add.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ void red_add_f32(float* p, float v) {
  asm volatile("red.relaxed.gpu.global.add.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned ld_shared_acquire_u32(const unsigned* p) {
  unsigned v;
  const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(p));
  asm volatile("ld.acquire.cta.shared.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
  return v;
}

// Value-as-flag words. A slot holding the all-ones pattern has not been
// published yet; a computed result that happens to be that exact NaN is
// replaced by the canonical quiet NaN so it can never be mistaken for "empty".
template <typename T> struct Flag;
template <> struct Flag<double> {
  using Bits = unsigned long long;
  static constexpr Bits EMPTY = 0xFFFFFFFFFFFFFFFFull;
  __device__ static __forceinline__ Bits load(const double* p) {
    return ld_relaxed_u64(reinterpret_cast<const unsigned long long*>(p));
  }
  __device__ static __forceinline__ Bits load_shared(const double* p) {
    return *reinterpret_cast<const volatile unsigned long long*>(p);
  }
  __device__ static __forceinline__ double value(Bits b) { return __longlong_as_double(static_cast<long long>(b)); }
  __device__ static __forceinline__ Bits bits(double v) {
    Bits b = static_cast<Bits>(__double_as_longlong(v));
    return b == EMPTY ? 0x7FF8000000000000ull : b;
  }
  __device__ static __forceinline__ void store(double* p, double v) {
    st_relaxed_u64(reinterpret_cast<unsigned long long*>(p), bits(v));
  }
  __device__ static __forceinline__ void store_shared(double* p, double v) {
    *reinterpret_cast<volatile unsigned long long*>(p) = bits(v);
  }
};
template <> struct Flag<float> {
  using Bits = unsigned;
  static constexpr Bits EMPTY = 0xFFFFFFFFu;
  __device__ static __forceinline__ Bits load(const float* p) {
    return ld_relaxed_u32(reinterpret_cast<const unsigned*>(p));
  }
  __device__ static __forceinline__ Bits load_shared(const float* p) {
    return *reinterpret_cast<const volatile unsigned*>(p);
  }
  __device__ static __forceinline__ float value(Bits b) { return __uint_as_float(b); }
  __device__ static __forceinline__ Bits bits(float v) {
    Bits b = __float_as_uint(v);
    return b == EMPTY ? 0x7FC00000u : b;
  }
  __device__ static __forceinline__ void store(float* p, float v) {
    st_relaxed_u32(reinterpret_cast<unsigned*>(p), bits(v));
  }
  __device__ static __forceinline__ void store_shared(float* p, float v) {
    *reinterpret_cast<volatile unsigned*>(p) = bits(v);
  }
};

// Bounded-wait bookkeeping. `poll` is called once per failed poll. It backs
// off with __nanosleep (doubling from sleep_min up to sleep_max nanoseconds;
// 0 = spin) so that thousands of waiting threads do not flood L2 with polls,
// and every 16 failed polls it reads the global timer and the shared status
// word. It returns false once the wait must be abandoned (timeout here, or an
// error raised elsewhere), after recording DEV_TIMEOUT the first time.
struct WaitBudget {
  unsigned long long start;
  unsigned long long limit_ns;
  unsigned iters;
  unsigned sleep_ns;
  unsigned sleep_max;
  __device__ __forceinline__ explicit WaitBudget(unsigned long long limit, unsigned smin = 0, unsigned smax = 0)
      : start(0), limit_ns(limit), iters(0), sleep_ns(smin), sleep_max(smax) {}
  __device__ __forceinline__ bool poll(DeviceCtl* ctl, int where) {
    ++iters;
    if (sleep_max) {
      __nanosleep(sleep_ns);
      sleep_ns = sleep_ns * 2u < sleep_max ? sleep_ns * 2u : sleep_max;
    }
    if ((iters & 15u) != 0u) return true;
    const unsigned long long now = globaltimer_ns();
    if (start == 0) { start = now; return true; }
    if (*reinterpret_cast<volatile int*>(&ctl->code) != DEV_OK) return false;
    if (now - start > limit_ns) {
      if (atomicCAS(&ctl->code, DEV_OK, DEV_TIMEOUT) == DEV_OK) ctl->where = where;
      return false;
    }
    return true;
  }
};

__device__ __forceinline__ bool ctl_failed(const DeviceCtl* ctl) {
  return *reinterpret_cast<const volatile int*>(&ctl->code) != DEV_OK;
}

// Grid-wide barrier for cooperative launches (all CTAs co-resident). Bounded:
// returns false if the wait runs out or another CTA already failed. Waiting
// CTAs back off from smin to smax nanoseconds between polls.
__device__ __forceinline__ bool grid_barrier(DeviceCtl* ctl, unsigned long long limit_ns, unsigned smin = 32u,
                                             unsigned smax = 256u) {
  __syncthreads();
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
    const unsigned gen = ld_acquire_u32(&ctl->barrier_gen);
    __threadfence();
    const unsigned arrived = atomicAdd(&ctl->barrier_count, 1u) + 1u;
    int ok = 1;
    if (arrived == nblocks) {
      ctl->barrier_count = 0;
      __threadfence();
      red_release_add_u32(&ctl->barrier_gen, 1u);
    } else {
      WaitBudget w(limit_ns, smin, smax);
      while (ld_acquire_u32(&ctl->barrier_gen) == gen) {
        if (!w.poll(ctl, -1)) { ok = 0; break; }
      }
    }
    s_ok = ok && !ctl_failed(ctl);
  }
  __syncthreads();
  return s_ok != 0;
}

}  // namespace sptrsv
