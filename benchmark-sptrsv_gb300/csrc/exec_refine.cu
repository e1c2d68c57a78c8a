// Fused first refinement step: one pass over the dependency DAG that solves
// in FP32, forms the FP64 residual and solves the FP32 correction together.
//
// Mixed-precision refinement solves L x0 = b in FP32, forms r = b - L x0 in
// FP64 and solves L d = r in FP32, then x = x0 + d. All three walk the same
// DAG, and at position p everything they need is final as soon as the
// dependencies of p are: x0_j and d_j of every dependency j, and x0_p itself.
// So one sync-free pass does all three. With w = L(p,j)/L(p,p) (FP32 and FP64
// copies, ready order) and rho = r/L(p,p):
//
//   x0_p  = b_p/d_p - sum_j w32_j x0_j                     (FP32)
//   rho_p = b_p/d_p - x0_p - sum_j w64_j x0_j              (FP64, x0_j exact in FP64)
//   d_p   = RN32(rho_p) - sum_j w32_j d_j                  (FP32)
//   x_p   = x0_p + d_p                                     (FP64)
//
// Position p publishes the pair (x0_p, d_p) as one 64-bit value-as-flag word
// (low half x0, high half d; all ones = not yet published), so a dependency
// costs one poll, exactly as in a single solve. The FP32 recurrences are the
// separate passes' arithmetic; the residual is formed in FP64 from the scaled
// FP64 weights the FP64 solve uses (so it is r/L(p,p), with the scaling
// rounded into the weights), which moves it only at the FP64 rounding level,
// far below the FP32 error it corrects.
//
// Lanes and lockstep as in the warp-synchronous many-rhs executor: G lanes per
// unknown (32/G unknowns per warp), each lane covering RPL right-hand sides,
// UD dependencies loaded per batch; a group moves to its next batch once all
// its lanes consumed the current one. In-chunk dependencies resolve through
// shared memory when the chunk's words fit. Every wait is bounded.
//
// stats (non-negative doubles as ordered bit patterns, max over the pass,
// taken in FP32): [0] max |d|, [1] max |x|, [2] max |x0| -- the refinement's
// stopping estimate.
//
// DF variant (the residual in double-float on the FP32 pipe). On this GPU an
// FP64 FMA issues at 1/64 of the FP32 rate and has 64 cycles of latency, so
// the residual's FP64 FMA per dependency sits both on the FP64 pipe and on
// every hop's critical path. The DF variant keeps the FP64 weight as two
// floats, w ~ hi + lo (hi = RN32(w), lo = RN32(w - hi), 48 significant bits),
// and carries S = b/d - sum_j w_j x0_j as an unevaluated float pair (acc, rl):
//   p  = RN(hi * x0_j),  pe = hi * x0_j - p (exact, by FMA),
//   t  = RN(lo * x0_j + pe)                 (the product's low part),
//   acc' = RN(acc - p),  e = (acc - p) - acc' (exact, TwoSum),
//   rl' = RN(rl + (e - t)).
// acc is the FP32 solve's own accumulator, so when the list is done x0 = acc
// and the scaled residual rho = S - x0 is rl itself: d = rl - sum_j hi_j d_j.
// The terms dropped are the product's low part rounding (2^-24 of a 2^-24
// fraction of each term) and the roundings of rl, which stays at the size of
// the residual: rho is exact to about 2^-44 relative to x, far below what the
// FP32 correction resolves. FP64 work is left only once per unknown: b/d at
// the start (product, split into the pair) and x = x0 + d at the end.
#include "exec_common.cuh"
#include "internal.h"

namespace sptrsv {

namespace {

constexpr unsigned long long kPairEmpty = 0xFFFFFFFFFFFFFFFFull;
constexpr unsigned long long kPairNaN = 0x7FC000007FC00000ull;

struct RefineArgs {
  int n, rhs, chunk, nchunks, smem_tier, ctas_per_sm;
  const int* perm;
  const int* dep_ptr;
  const int* dep_pos_f;
  const float* w32;
  const double* w64;
  const float2* wsplit;       // DF: (hi, lo) of every FP64 weight, ready order
  // imported dependencies of a blocked layout (k_pull_refine1_imp): unit c covers
  // positions [im_start[c], im_start[c+1]) and imports im_q[im_ptr[c] ..
  // im_ptr[c+1]); dep_slot[e] is the shared-memory slot of dependency e
  const int* im_start;
  const int* im_ptr;
  const int* im_q;
  const int* dep_slot;
  const float* rcp32;
  const double* rcp64;
  const double* b;
  double* x;
  long long b_si, b_sk, x_si, x_sk;
  unsigned long long* xw;     // [n * rhs] (x0, d) pairs, position-major
  unsigned long long* stats;  // [3]
  DeviceCtl* ctl;
  unsigned long long timeout_ns;
  unsigned sleep_min, sleep_max;  // backoff of global polls (ns)
};

__device__ __forceinline__ unsigned long long pack_pair(float x0, float d) {
  const unsigned long long v = (static_cast<unsigned long long>(__float_as_uint(d)) << 32) |
                               static_cast<unsigned long long>(__float_as_uint(x0));
  return v == kPairEmpty ? kPairNaN : v;
}
__device__ __forceinline__ float pair_x0(unsigned long long v) {
  return __uint_as_float(static_cast<unsigned>(v & 0xFFFFFFFFull));
}
__device__ __forceinline__ float pair_d(unsigned long long v) { return __uint_as_float(static_cast<unsigned>(v >> 32)); }

// Exact FP32 -> FP64 widening from the IEEE 754 bit fields (sign kept,
// exponent re-biased from 127 to 1023, 23-bit fraction shifted into the top of
// the 52-bit one), on the integer pipe: FP64 instructions are scarce on this
// GPU, and the fused pass widens every FP32 value it reads. Subnormal, infinite
// and NaN inputs take the hardware conversion.
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xFFu, man = u & 0x7FFFFFu;
  if (ex == 0xFFu || (ex == 0u && man != 0u)) return static_cast<double>(f);
  const unsigned hi = (u & 0x80000000u) | (ex != 0u ? (ex + 896u) << 20 : 0u) | (man >> 3);
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(man << 29));
}

__device__ __forceinline__ unsigned long long ld_shared_u64(const unsigned long long* p) {
  return *reinterpret_cast<const volatile unsigned long long*>(p);
}
__device__ __forceinline__ void st_shared_u64(unsigned long long* p, unsigned long long v) {
  *reinterpret_cast<volatile unsigned long long*>(p) = v;
}

__device__ __forceinline__ void stats_max(unsigned long long* p, float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0)
    atomicMax(p, static_cast<unsigned long long>(__double_as_longlong(static_cast<double>(v))));
}

// Exact FP32 error-free steps; the intrinsics keep the compiler from fusing
// the product into the subtraction, which would break the exactness.
__device__ __forceinline__ void df_sub_product(float& acc, float& rl, float hi, float lo, float x) {
  const float p = __fmul_rn(hi, x);
  const float pe = __fmaf_rn(hi, x, -p);
  const float t = __fmaf_rn(lo, x, pe);
  const float s = __fsub_rn(acc, p);
  const float bb = __fsub_rn(s, acc);
  const float e = __fadd_rn(__fsub_rn(acc, __fsub_rn(s, bb)), __fsub_rn(-p, bb));
  acc = s;
  rl = __fadd_rn(rl, __fsub_rn(e, t));
}

template <int G, int RPL, int UD, bool DF = false>
__global__ void __launch_bounds__(256) k_pull_refine1(RefineArgs a) {
  using Bits = unsigned long long;
  constexpr int P = 32 / G;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Bits* s_x = reinterpret_cast<Bits*>(smem_raw);
  __shared__ unsigned s_chunk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int gi = lane / G, gl = lane % G;
  const unsigned gmask = G >= 32 ? 0xffffffffu : ((1u << G) - 1u) << (lane & ~(G - 1));
  const int rhs = a.rhs;
  // stopping-estimate maxima, kept in FP32 (the estimate needs no more)
  float mx_d = 0.f, mx_x = 0.f, mx_x0 = 0.f;
  for (;;) {
    const unsigned c = next_chunk(a.ctl, a.nchunks, &s_chunk);
    if (c >= (unsigned)a.nchunks) break;
    const int base = static_cast<int>(c) * a.chunk;
    const int len = min(base + a.chunk, a.n) - base;
    if (a.smem_tier)
      for (long long i = threadIdx.x; i < (long long)len * rhs; i += blockDim.x) s_x[i] = kPairEmpty;
    __syncthreads();
    bool fail = false;
    for (int seg = warp; seg * P < len && !fail; seg += nwarps) {
      const int j = seg * P + gi;
      bool done = j >= len;  // group-uniform
      const int p = base + j;
      int row = 0, e = 0, e1 = 0;
      float acc0[RPL], accd[RPL];
      double res[RPL];   // FP64 residual accumulator (not DF)
      float rlo[RPL];    // DF: low part of S = b/d - sum w x0
#pragma unroll
      for (int r = 0; r < RPL; ++r) {
        acc0[r] = 0.f;
        accd[r] = 0.f;
        res[r] = 0.0;
        rlo[r] = 0.f;
      }
      if (!done) {
        row = a.perm[p];
        e = a.dep_ptr[p];
        e1 = a.dep_ptr[p + 1];
        const float s32 = a.rcp32[p];
        const double s64 = a.rcp64[p];
#pragma unroll
        for (int r = 0; r < RPL; ++r) {
          const int k = gl + r * G;
          if (k < rhs) {
            const double bv = a.b[(long long)row * a.b_si + (long long)k * a.b_sk];
            if (DF) {
              // b/d as a float pair: hi = RN32(b*s), lo = RN32(b*s - hi)
              const double bs = bv * s64;
              const float hi = __double2float_rn(bs);
              acc0[r] = hi;
              rlo[r] = __double2float_rn(__fma_rn(bv, s64, -widen(hi)));
            } else {
              acc0[r] = static_cast<float>(bv) * s32;
              res[r] = bv * s64;
            }
          }
        }
      }
      int q[UD], sl[UD];
      float w32[UD], wlo[UD];
      double w64[UD];
      Bits bits[UD][RPL];
      unsigned todo = 0u;
      auto load_batch = [&]() {
        todo = 0u;
#pragma unroll
        for (int u = 0; u < UD; ++u) {
          const bool in = e + u < e1;
          q[u] = in ? a.dep_pos_f[e + u] : -1;
          if (DF) {
            const float2 ws = in ? a.wsplit[e + u] : make_float2(0.f, 0.f);
            w32[u] = ws.x;
            wlo[u] = ws.y;
          } else {
            w32[u] = in ? a.w32[e + u] : 0.f;
            w64[u] = in ? a.w64[e + u] : 0.0;
          }
          sl[u] = (q[u] >= 0 && a.smem_tier && q[u] >= base) ? q[u] - base : -1;
#pragma unroll
          for (int r = 0; r < RPL; ++r) {
            const int k = gl + r * G;
            bits[u][r] = kPairEmpty;
            if (q[u] >= 0 && k < rhs) {
              bits[u][r] = sl[u] >= 0 ? ld_shared_u64(&s_x[(long long)sl[u] * rhs + k])
                                      : ld_relaxed_u64(&a.xw[(long long)q[u] * rhs + k]);
              todo |= 1u << (u * RPL + r);
            }
          }
        }
      };
      if (!done) load_batch();
      WaitBudget wb(a.timeout_ns);
      unsigned nap = a.sleep_min, idle = 0u;
      for (;;) {
        bool progress = false, global_wait = false;
        if (!done) {
#pragma unroll
          for (int r = 0; r < RPL; ++r)
#pragma unroll
            for (int u = 0; u < UD; ++u) {
              const unsigned bit = 1u << (u * RPL + r);
              if (!(todo & bit)) continue;
              if (bits[u][r] != kPairEmpty) {
                const float xj = pair_x0(bits[u][r]);
                if (DF) {
                  df_sub_product(acc0[r], rlo[r], w32[u], wlo[u], xj);
                } else {
                  acc0[r] = fmaf(-w32[u], xj, acc0[r]);
                  res[r] = fma(-w64[u], widen(xj), res[r]);
                }
                accd[r] = fmaf(-w32[u], pair_d(bits[u][r]), accd[r]);
                todo &= ~bit;
                progress = true;
              } else if (sl[u] < 0) {
                global_wait = true;
              }
            }
        }
        const unsigned clear = __ballot_sync(0xffffffffu, done || todo == 0u);
        const bool group_clear = (clear & gmask) == gmask;
        if (!done) {
          if (group_clear) {
            e += UD;
            if (e < e1) {
              load_batch();
            } else {
#pragma unroll
              for (int r = 0; r < RPL; ++r) {
                const int k = gl + r * G;
                if (k < rhs) {
                  const float x0 = acc0[r];
                  // DF: rho = S - x0 = the pair's low part
                  const float d = DF ? __fadd_rn(rlo[r], accd[r]) : static_cast<float>(res[r] - widen(x0)) + accd[r];
                  const Bits v = pack_pair(x0, d);
                  if (a.smem_tier) st_shared_u64(&s_x[(long long)j * rhs + k], v);
                  st_relaxed_u64(&a.xw[(long long)p * rhs + k], v);
                  accd[r] = d;  // d from here on; x and the maxima follow the lockstep loop
                }
              }
              done = true;
            }
            progress = true;
          } else {
#pragma unroll
            for (int u = 0; u < UD; ++u)
#pragma unroll
              for (int r = 0; r < RPL; ++r) {
                const int k = gl + r * G;
                if ((todo & (1u << (u * RPL + r))) && bits[u][r] == kPairEmpty)
                  bits[u][r] = sl[u] >= 0 ? ld_shared_u64(&s_x[(long long)sl[u] * rhs + k])
                                          : ld_relaxed_u64(&a.xw[(long long)q[u] * rhs + k]);
              }
          }
        }
        // no lane consumed anything: nothing was published, so the completion
        // vote is skipped
        if (__any_sync(0xffffffffu, progress)) {
          if (__all_sync(0xffffffffu, done)) break;
          __syncwarp();
          nap = a.sleep_min;
        } else {
          const bool any_global = __any_sync(0xffffffffu, global_wait);
          __syncwarp();
          if (any_global && a.sleep_max) {
            __nanosleep(nap);
            nap = nap * 2u < a.sleep_max ? nap * 2u : a.sleep_max;
          }
          if ((any_global || (++idle & 255u) == 0u) && !wb.poll(a.ctl, p)) fail = true;
          if (__any_sync(0xffffffffu, fail)) {
            fail = true;
            break;
          }
        }
      }
      // x = x0 + d and the stopping-estimate maxima, once the segment is done:
      // off the lockstep iterations, on which the in-warp hops wait
      if (!fail && j < len) {
#pragma unroll
        for (int r = 0; r < RPL; ++r) {
          const int k = gl + r * G;
          if (k < rhs) {
            a.x[(long long)row * a.x_si + (long long)k * a.x_sk] = widen(acc0[r]) + widen(accd[r]);
            mx_d = fmaxf(mx_d, fabsf(accd[r]));
            mx_x = fmaxf(mx_x, fabsf(acc0[r] + accd[r]));
            mx_x0 = fmaxf(mx_x0, fabsf(acc0[r]));
          }
        }
      }
    }
    if (__syncthreads_or(fail)) break;
  }
  stats_max(&a.stats[0], mx_d);
  stats_max(&a.stats[1], mx_x);
  stats_max(&a.stats[2], mx_x0);
  leave(a.ctl);
}

// ------------------------------------------------------------------ fused step, blocked layouts
// The fused first refinement step (double-float residual, one right-hand side)
// on a blocked layout, with the importer warp of k_pull_wsync_imp: one CTA per
// order block, an extra warp that polls the block's external (x0, d) pairs from
// global memory and copies each into a shared-memory slot as it lands, and
// consumer warps that resolve every dependency in shared memory (slot from
// dep_slot), one lane per unknown in lockstep. Without the importer the
// consumer warps' lockstep iterations would wait on L2 polls of the few
// cross-block dependencies. ONE: every list holds at most U entries, so a lane
// publishes once its first batch is consumed.
template <int U, bool ONE>
__global__ void __launch_bounds__(288) k_pull_refine1_imp(RefineArgs a) {
  using Bits = unsigned long long;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Bits* s_x = reinterpret_cast<Bits*>(smem_raw);
  __shared__ unsigned s_chunk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ncw = (blockDim.x >> 5) - 1;  // consumer warps; warp ncw imports
  float mx_d = 0.f, mx_x = 0.f, mx_x0 = 0.f;
  for (;;) {
    const unsigned c = next_chunk(a.ctl, a.nchunks, &s_chunk);
    if (c >= (unsigned)a.nchunks) break;
    const int base = a.im_start[c];
    const int len = a.im_start[c + 1] - base;  // <= a.chunk (the window)
    const int i0 = a.im_ptr[c], nimp = a.im_ptr[c + 1] - i0;
    for (int i = threadIdx.x; i < len; i += blockDim.x) s_x[i] = kPairEmpty;
    for (int i = threadIdx.x; i < nimp; i += blockDim.x) s_x[a.chunk + i] = kPairEmpty;
    __syncthreads();
    bool fail = false;
    if (warp == ncw) {
      // importer: each lane walks its imports in order, one poll at a time
      WaitBudget wb(a.timeout_ns);
      unsigned idle = 0u;
      int i = lane;
      Bits v = kPairEmpty;
      if (i < nimp) v = ld_relaxed_u64(&a.xw[a.im_q[i0 + i]]);
      for (;;) {
        bool progress = false;
        if (i < nimp) {
          if (v != kPairEmpty) {
            st_shared_u64(&s_x[a.chunk + i], v);
            i += 32;
            v = i < nimp ? ld_relaxed_u64(&a.xw[a.im_q[i0 + i]]) : kPairEmpty;
            progress = true;
          } else {
            v = ld_relaxed_u64(&a.xw[a.im_q[i0 + i]]);
          }
        }
        if (__all_sync(0xffffffffu, i >= nimp)) break;
        if (!__any_sync(0xffffffffu, progress) && ((++idle & 15u) == 0u)) {
          if (__any_sync(0xffffffffu, !wb.poll(a.ctl, base))) {
            fail = true;
            break;
          }
        }
      }
    } else {
      // A warp takes every ncw-th segment; the row and list bounds of its next
      // segment are loaded while it works on the current one.
      int n_row = 0, n_e = 0, n_e1 = 0;
      auto fetch = [&](int sg) {
        const int jj = sg * 32 + lane;
        if (jj < len) {
          n_row = a.perm[base + jj];
          n_e = a.dep_ptr[base + jj];
          n_e1 = a.dep_ptr[base + jj + 1];
        }
      };
      if (warp * 32 < len) fetch(warp);
      for (int seg = warp; seg * 32 < len && !fail; seg += ncw) {
        const int j = seg * 32 + lane;
        bool done = j >= len;
        const int p = base + j;
        const int row = n_row;
        int e = n_e;
        const int e1 = n_e1;
        if ((seg + ncw) * 32 < len) fetch(seg + ncw);
        float acc0 = 0.f, rlo = 0.f, accd = 0.f;
        if (!done) {
          // b/d as a float pair: hi = RN32(b*s), lo = RN32(b*s - hi)
          const double bv = a.b[(long long)row * a.b_si];
          const double s64 = a.rcp64[p];
          const float hi = __double2float_rn(bv * s64);
          acc0 = hi;
          rlo = __double2float_rn(__fma_rn(bv, s64, -widen(hi)));
        }
        int ls[U];
        float wh[U], wl[U];
        Bits bits[U];
        unsigned todo = 0u;
        auto load_batch = [&]() {
          todo = 0u;
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int ee = e + u;
            ls[u] = ee < e1 ? a.dep_slot[ee] : -1;
            const float2 ws = ee < e1 ? a.wsplit[ee] : make_float2(0.f, 0.f);
            wh[u] = ws.x;
            wl[u] = ws.y;
          }
#pragma unroll
          for (int u = 0; u < U; ++u) {
            bits[u] = kPairEmpty;
            if (ls[u] >= 0) {
              bits[u] = ld_shared_u64(&s_x[ls[u]]);
              todo |= 1u << u;
            }
          }
        };
        if (!done) load_batch();
        WaitBudget wb(a.timeout_ns);
        unsigned idle = 0u;
        for (;;) {
          bool progress = false;
          if (!done) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
              if (!(todo & (1u << u))) continue;
              if (bits[u] != kPairEmpty) {
                df_sub_product(acc0, rlo, wh[u], wl[u], pair_x0(bits[u]));
                accd = fmaf(-wh[u], pair_d(bits[u]), accd);
                todo &= ~(1u << u);
                progress = true;
              }
            }
            if (!todo) {
              if (!ONE) e += U;
              if (!ONE && e < e1) {
                load_batch();
              } else {
                // rho = S - x0 is the pair's low part
                accd = __fadd_rn(rlo, accd);  // accd holds d from here on
                const Bits v = pack_pair(acc0, accd);
                st_shared_u64(&s_x[j], v);
                st_relaxed_u64(&a.xw[p], v);
                done = true;
              }
              progress = true;
            } else {
#pragma unroll
              for (int u = 0; u < U; ++u)  // pending entries are unpublished: arrived ones were consumed
                if (todo & (1u << u)) bits[u] = ld_shared_u64(&s_x[ls[u]]);
            }
          }
          // no lane consumed anything: nothing was published, so the
          // completion vote is skipped
          if (__any_sync(0xffffffffu, progress)) {
            if (__all_sync(0xffffffffu, done)) break;
          } else if (((++idle & 255u) == 0u) && __any_sync(0xffffffffu, !wb.poll(a.ctl, p))) {
            fail = true;
            break;
          }
        }
        // x = x0 + d and the stopping-estimate maxima, once the segment is done:
        // off the lockstep iterations, on which the in-warp hops wait
        if (!fail && j < len) {
          a.x[(long long)row * a.x_si] = widen(acc0) + widen(accd);
          mx_d = fmaxf(mx_d, fabsf(accd));
          mx_x = fmaxf(mx_x, fabsf(acc0 + accd));
          mx_x0 = fmaxf(mx_x0, fabsf(acc0));
        }
      }
    }
    if (__syncthreads_or(fail)) break;
  }
  stats_max(&a.stats[0], mx_d);
  stats_max(&a.stats[1], mx_x);
  stats_max(&a.stats[2], mx_x0);
  leave(a.ctl);
}

template <int G, int RPL, int UD, bool DF>
cudaError_t run_refine1(const RefineArgs& a, int block, size_t smem, int num_sms, cudaStream_t s) {
  auto kernel = k_pull_refine1<G, RPL, UD, DF>;
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
  if (per_sm < 1) per_sm = 1;
  if (a.ctas_per_sm > 0 && per_sm > a.ctas_per_sm) per_sm = a.ctas_per_sm;
  long long grid = (long long)num_sms * per_sm;
  if (grid > a.nchunks) grid = a.nchunks;
  if (grid < 1) grid = 1;
  kernel<<<static_cast<int>(grid), block, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_refine_fused(const Layout& L, const Values<float>& v32, const Values<double>& v64, int rhs,
                                const double* b, double* x, long long si, long long sk, unsigned long long* xw,
                                unsigned long long* stats, DeviceCtl* ctl, const ExecConfig& cfg,
                                unsigned long long timeout_ns, int num_sms, cudaStream_t s, const float2* wsplit) {
  if (L.n == 0) return cudaSuccess;
  if (rhs < 1 || rhs > 64) return cudaErrorInvalidValue;
  RefineArgs a{};
  a.n = L.n;
  a.rhs = rhs;
  a.chunk = cfg.chunk > 0 ? cfg.chunk : 256;
  a.nchunks = (L.n + a.chunk - 1) / a.chunk;
  a.ctas_per_sm = cfg.ctas_per_sm;
  a.perm = L.perm;
  a.dep_ptr = L.dep_ptr;
  a.dep_pos_f = L.dep_pos_f;
  a.w32 = v32.dep_w;
  a.w64 = v64.dep_w;
  a.rcp32 = v32.rcp;
  a.rcp64 = v64.rcp;
  a.b = b;
  a.x = x;
  a.b_si = a.x_si = si;
  a.b_sk = a.x_sk = sk;
  a.xw = xw;
  a.stats = stats;
  a.ctl = ctl;
  a.timeout_ns = timeout_ns;
  a.sleep_min = cfg.sleep_max ? 16u : 0u;
  a.sleep_max = cfg.sleep_max;
  size_t smem = 0;
  if (cfg.smem_tier) {
    smem = (size_t)a.chunk * (size_t)rhs * sizeof(unsigned long long);
    if (smem <= 200 * 1024) a.smem_tier = 1;
    else smem = 0;
  }
  const int block = cfg.block;
  const int ud = cfg.wsync_batch == 1 ? 1 : 2;
  a.wsplit = wsplit;
  if (wsplit) {
    if (rhs == 1) return ud == 1 ? run_refine1<1, 1, 1, true>(a, block, smem, num_sms, s)
                                 : run_refine1<1, 1, 2, true>(a, block, smem, num_sms, s);
    if (rhs <= 4) return run_refine1<4, 1, 2, true>(a, block, smem, num_sms, s);
    if (rhs <= 8) return run_refine1<8, 1, 2, true>(a, block, smem, num_sms, s);
    if (rhs <= 16) return run_refine1<16, 1, 2, true>(a, block, smem, num_sms, s);
    if (rhs <= 32) return run_refine1<32, 1, 2, true>(a, block, smem, num_sms, s);
    return run_refine1<32, 2, 2, true>(a, block, smem, num_sms, s);
  }
  if (rhs == 1) return ud == 1 ? run_refine1<1, 1, 1, false>(a, block, smem, num_sms, s)
                               : run_refine1<1, 1, 2, false>(a, block, smem, num_sms, s);
  if (rhs <= 4) return run_refine1<4, 1, 2, false>(a, block, smem, num_sms, s);
  if (rhs <= 8) return run_refine1<8, 1, 2, false>(a, block, smem, num_sms, s);
  if (rhs <= 16) return run_refine1<16, 1, 2, false>(a, block, smem, num_sms, s);
  if (rhs <= 32) return run_refine1<32, 1, 2, false>(a, block, smem, num_sms, s);
  return run_refine1<32, 2, 2, false>(a, block, smem, num_sms, s);
}

cudaError_t launch_refine_fused_imported(const Layout& L, const Values<double>& v64, const float2* wsplit,
                                         const double* b, double* x, unsigned long long* xw,
                                         unsigned long long* stats, DeviceCtl* ctl, const ExecConfig& cfg,
                                         unsigned long long timeout_ns, int num_sms, cudaStream_t s,
                                         const ImportTable& im) {
  if (L.n == 0) return cudaSuccess;
  RefineArgs a{};
  a.n = L.n;
  a.rhs = 1;
  a.chunk = im.width;  // the window: first import slot
  a.nchunks = im.nchunks;
  a.ctas_per_sm = cfg.ctas_per_sm;
  a.perm = L.perm;
  a.dep_ptr = L.dep_ptr;
  a.dep_pos_f = L.dep_pos_f;
  a.rcp64 = v64.rcp;
  a.wsplit = wsplit;
  a.b = b;
  a.x = x;
  a.b_si = a.x_si = 1;
  a.b_sk = a.x_sk = L.n;
  a.xw = xw;
  a.stats = stats;
  a.ctl = ctl;
  a.timeout_ns = timeout_ns;
  a.im_start = im.start;
  a.im_ptr = im.ptr;
  a.im_q = im.q;
  a.dep_slot = im.dep_slot;
  const size_t smem = (size_t)(im.width + im.max_imports) * sizeof(unsigned long long);
  const int block = cfg.block + 32;
  auto launch = [&](auto kernel) -> cudaError_t {
    if (smem > 48 * 1024) {
      const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
    if (per_sm < 1) per_sm = 1;
    if (a.ctas_per_sm > 0 && per_sm > a.ctas_per_sm) per_sm = a.ctas_per_sm;
    long long grid = (long long)num_sms * per_sm;
    if (grid > a.nchunks) grid = a.nchunks;
    if (grid < 1) grid = 1;
    kernel<<<static_cast<int>(grid), block, smem, s>>>(a);
    return cudaGetLastError();
  };
  const bool one = cfg.one_batch != 0;
  switch (cfg.wsync_batch) {
    case 1: return one ? launch(k_pull_refine1_imp<1, true>) : launch(k_pull_refine1_imp<1, false>);
    case 4: return one ? launch(k_pull_refine1_imp<4, true>) : launch(k_pull_refine1_imp<4, false>);
    default: return one ? launch(k_pull_refine1_imp<2, true>) : launch(k_pull_refine1_imp<2, false>);
  }
}

// (hi, lo) float pairs of the FP64 weights for the DF fused pass:
// hi = RN32(w), lo = RN32(w - hi).
__global__ void k_split_weights(const double* __restrict__ w, long long count, float2* out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride) {
    const double v = w[i];
    const float hi = __double2float_rn(v);
    out[i] = make_float2(hi, __double2float_rn(v - static_cast<double>(hi)));
  }
}
cudaError_t launch_split_weights(const double* w, long long count, float2* out, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  long long grid = (count + 255) / 256;
  if (grid > (1 << 20)) grid = 1 << 20;
  k_split_weights<<<static_cast<int>(grid), 256, 0, s>>>(w, count, out);
  return cudaGetLastError();
}

}  // namespace sptrsv
