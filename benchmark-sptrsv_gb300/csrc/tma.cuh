// Bulk-copy (1-D TMA) and mbarrier helpers shared by the staged executors:
// streaming slices of the position-space layout into shared memory, with
// completion signalled on an mbarrier, and bounded waits on barrier phases.
#pragma once
#include "common.cuh"

namespace sptrsv {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Copies elements [a, b) of src into dst (16-byte aligned smem) through the
// bulk-copy engine; returns the element offset of `a` inside dst and adds the
// byte count to *tx. The source range is widened to 16-byte boundaries (the
// layout arrays are padded so the widened range stays in bounds).
template <typename E>
__device__ __forceinline__ int stage_slice(E* dst, const E* src, long long a, long long b, unsigned long long* bar,
                                           unsigned* tx) {
  constexpr long long per16 = 16 / sizeof(E);
  const long long a16 = a & ~(per16 - 1);
  const long long b16 = (b + per16 - 1) & ~(per16 - 1);
  const unsigned bytes = static_cast<unsigned>((b16 - a16) * (long long)sizeof(E));
  if (bytes) {
    bulk_g2s(dst, src + a16, bytes, bar);
    *tx += bytes;
  }
  return static_cast<int>(a - a16);
}

// Bounded wait on an mbarrier phase; false once the budget runs out or
// another thread failed.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, DeviceCtl* ctl,
                                          unsigned long long timeout, int where) {
  if (mbar_test(bar, parity)) return true;
  WaitBudget w(timeout);
  while (!mbar_test(bar, parity)) {
    if (!w.poll(ctl, where)) return false;
  }
  return true;
}

constexpr int kMaxStages = 4;

template <typename T>
struct StageBufs {
  int* ptr;
  int* perm;
  T* sc;
  int* pos;
  T* val;
};

// Shared-memory carve-up for one stage (all regions 16-byte aligned).
template <typename T>
__host__ __device__ inline size_t stage_bytes(int cmax, int emax) {
  auto up = [](size_t v) { return (v + 15) & ~(size_t)15; };
  return up(sizeof(int) * (size_t)(cmax + 1 + 8)) + up(sizeof(int) * (size_t)(cmax + 8)) +
         up(sizeof(T) * (size_t)(cmax + 8)) + up(sizeof(int) * (size_t)(emax + 8)) + up(sizeof(T) * (size_t)(emax + 8));
}
template <typename T>
__device__ inline StageBufs<T> carve(unsigned char* base, int cmax, int emax) {
  auto up = [](size_t v) { return (v + 15) & ~(size_t)15; };
  StageBufs<T> s;
  size_t o = 0;
  s.ptr = reinterpret_cast<int*>(base + o);
  o += up(sizeof(int) * (size_t)(cmax + 1 + 8));
  s.perm = reinterpret_cast<int*>(base + o);
  o += up(sizeof(int) * (size_t)(cmax + 8));
  s.sc = reinterpret_cast<T*>(base + o);
  o += up(sizeof(T) * (size_t)(cmax + 8));
  s.pos = reinterpret_cast<int*>(base + o);
  o += up(sizeof(int) * (size_t)(emax + 8));
  s.val = reinterpret_cast<T*>(base + o);
  return s;
}

}  // namespace sptrsv
