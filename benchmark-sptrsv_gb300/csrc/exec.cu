// Sync-free triangular-solve executors.
//
// All executors walk "positions": position p is the p-th unknown of the
// schedule built at analysis time (row perm[p]); every dependency of p sits at
// a smaller position, so a CTA that owns position p only ever waits on work
// that was handed out before it (forward progress without co-residency).
// Work is handed out in chunks of consecutive positions through a ticket
// counter; inside a chunk, groups of `G` lanes take positions in order.
//
//  pull   : p gathers x of its dependencies (CSR row, value-as-flag words,
//           relaxed loads), then publishes x_p. Deterministic summation;
//           EXACT reproduces the serial executor's operation order.
//  push   : the reference's scheme (SpTRSV_cuda/sptrsv_syncfree_cuda.h:21-107,
//           :290-407): p waits for its in-degree counter, reads its partial
//           sum, finishes x_p and pushes x_p*L(r,p) into the partial sums of
//           its dependents with atomics, then bumps their counters.
//  levelset: one grid barrier per level (cooperative launch).
//
// Every wait is bounded (DeviceCtl::code = DEV_TIMEOUT on expiry) and a CTA
// that sees a failure drains to its barriers and leaves.
#include <algorithm>

#include "exec_common.cuh"
#include "internal.h"

namespace sptrsv {

namespace {

template <typename T>
struct ExecArgs {
  int n, rhs, chunk, nchunks, smem_tier, ctas_per_sm;
  int opt;  // push, many rhs: lane mode (1 over entries, 2 over rhs, 3 the reference's rule per column)
  // pull walks: chunk c covers walk indices [c*chunk - walk_pad, (c+1)*chunk - walk_pad);
  // the reverse (adjoint) walk is shifted so its chunks line up with order blocks
  int walk_pad;
  const int* perm;
  const int* dep_ptr;
  const int* dep_pos;
  const int* dep_pos_f;  // ready order (pairs with dep_w)
  const T* dep_val;
  const T* dep_w;
  const int* dep_src;
  const int* dep_col;
  const int* diag_src;
  const int* out_ptr;
  const int* out_pos;
  const int* out_pos_f;  // ready order (pairs with out_w)
  const T* out_val;
  const T* out_w;
  T* grad;           // adjoint: gradient w.r.t. the stored values (CSC order), or null
  const T* xf;       // adjoint: forward solution x (row-indexed)
  long long xf_si, xf_sk;
  const T* diag;
  const T* rcp;
  const T* b;
  T* x;
  long long b_si, b_sk, x_si, x_sk;
  T* xw;             // pull / levelset: position-major value flags [n * rhs]
  T* left_sum;       // push: position-major partial sums [n * rhs] (zero between solves)
  unsigned* counters;  // push: arrivals per position (zero between solves)
  DeviceCtl* ctl;
  unsigned long long timeout_ns;
  unsigned sleep_min, sleep_max;  // backoff of global polls (ns)
  const int* level_ptr;
  int nlevels;
  // split-list work units (k_pull_wsync_split): piece i covers entries
  // [pc_lo[i], pc_hi[i]) of walk index pc_walk[i] (-1: padding); 32 pieces per
  // warp segment; chunk c = segments [pc_cseg[c], pc_cseg[c+1]), starting at
  // walk index pc_cbase[c] and spanning at most `chunk` walk indices
  const int* pc_walk;
  const int* pc_row;    // row of the piece's unknown (perm of its position)
  const int* pc_lo;
  const int* pc_hi;
  const int* pc_cseg;
  const int* pc_cbase;
  const unsigned char* pc_split;  // per segment: 1 if an unknown spans several lanes
  // imported dependencies (k_pull_wsync_imp): chunk c needs the positions
  // im_q[im_ptr[c] .. im_ptr[c+1]) from other chunks; dep_slot[e] is the
  // shared-memory slot of dependency e (in-chunk: position - chunk base;
  // imported: chunk + import index)
  const int* im_start;
  const int* im_ptr;
  const int* im_q;
  const int* dep_slot;
};

template <typename T>
__device__ __forceinline__ T mul_add(T acc, T v, T xq, bool exact);
template <>
__device__ __forceinline__ double mul_add<double>(double acc, double v, double xq, bool exact) {
  return exact ? __dadd_rn(acc, __dmul_rn(xq, v)) : fma(v, xq, acc);
}
template <>
__device__ __forceinline__ float mul_add<float>(float acc, float v, float xq, bool exact) {
  return exact ? __fadd_rn(acc, __fmul_rn(xq, v)) : fmaf(v, xq, acc);
}
template <typename T>
__device__ __forceinline__ T finish(T bi, T acc, T d, T r, bool exact);
template <>
__device__ __forceinline__ double finish<double>(double bi, double acc, double d, double r, bool exact) {
  return exact ? __ddiv_rn(__dsub_rn(bi, acc), d) : (bi - acc) * r;
}
template <>
__device__ __forceinline__ float finish<float>(float bi, float acc, float d, float r, bool exact) {
  return exact ? __fdiv_rn(__fsub_rn(bi, acc), d) : (bi - acc) * r;
}

__device__ __forceinline__ unsigned group_mask(int G) {
  if (G >= 32) return 0xffffffffu;
  const int lane32 = threadIdx.x & 31;
  return ((1u << G) - 1u) << (lane32 & ~(G - 1));
}

template <typename T, bool SHARED>
__device__ __forceinline__ typename Flag<T>::Bits wait_flag(const T* p, DeviceCtl* ctl, unsigned long long timeout,
                                                            int where, unsigned sleep_min, unsigned sleep_max) {
  return wait_flag_dev<T, SHARED>(p, ctl, timeout, where, sleep_min, sleep_max);
}

// ------------------------------------------------------------------ pull, one rhs
// x_p = b_p/d_p - sum_j w_j x_j with w = L(p,j)/d_p staged in advance, so each
// dependency costs one fused multiply-add once its value is published
// (EXACT keeps the serial executor's product, sum and true division instead).
// Each lane issues the index, value and flag loads of U dependencies together
// before consuming them in order.
//
// ADJ runs the transposed (adjoint) solve on the same analysis: positions are
// walked in reverse, and the dependencies of p are its dependents in the
// forward solve (the push lists, stored in the order the serial executor
// applied to L^T accumulates them). With a.grad set it also writes the
// gradient of every stored entry of row p, dL(p,j) = -lambda_p * x_j, as soon
// as lambda_p is known (fused adjoint + gradient).
template <typename T, int G, bool EXACT, int U, bool ADJ>
__global__ void __launch_bounds__(256) k_pull_vec(ExecArgs<T> a) {
  using F = Flag<T>;
  using Bits = typename F::Bits;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_x = reinterpret_cast<T*>(smem_raw);
  __shared__ unsigned s_chunk;
  const int NG = blockDim.x / G;
  const int g = threadIdx.x / G, lane = threadIdx.x % G;
  const unsigned gmask = group_mask(G);
  const int* __restrict__ lptr = ADJ ? a.out_ptr : a.dep_ptr;
  const int* __restrict__ lpos = ADJ ? (EXACT ? a.out_pos : a.out_pos_f) : (EXACT ? a.dep_pos : a.dep_pos_f);
  const T* __restrict__ vals = ADJ ? (EXACT ? a.out_val : a.out_w) : (EXACT ? a.dep_val : a.dep_w);
  const int last = a.n - 1;
  for (;;) {
    const unsigned c = next_chunk(a.ctl, a.nchunks, &s_chunk);
    if (c >= (unsigned)a.nchunks) break;
    const int base0 = static_cast<int>(c) * a.chunk - a.walk_pad;
    const int base = max(base0, 0);
    const int cend = min(base0 + a.chunk, a.n);
    if (a.smem_tier)
      for (int i = threadIdx.x; i < cend - base; i += blockDim.x)
        *reinterpret_cast<Bits*>(&s_x[i]) = F::EMPTY;
    __syncthreads();
    bool fail = false;
    for (int pr = base + g; pr < cend; pr += NG) {
      const int p = ADJ ? last - pr : pr;
      const int row = a.perm[p];
      const int e0 = lptr[p], e1 = lptr[p + 1];
      const T bi = a.b[(long long)row * a.b_si];
      T acc = T(0);
      if (!EXACT && lane == 0) acc = bi * a.rcp[p];
      auto slot = [&](int q) {
        const int qr = ADJ ? last - q : q;
        return (a.smem_tier && qr >= base) ? qr - base : -1;
      };
      if (!gather_deps<T, EXACT, U, G>(lpos, vals, e0 + lane, e1, a.xw, s_x, slot, a.ctl, a.timeout_ns, p,
                                       a.sleep_min, a.sleep_max, acc))
        fail = true;
      if (G > 1) {
        fail = __any_sync(gmask, fail);
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(gmask, acc, o);
      }
      if (fail) break;
      const T xi = EXACT ? finish<T>(bi, acc, a.diag[p], T(0), true) : acc;
      if (lane == 0) {
        if (a.smem_tier) F::store_shared(&s_x[pr - base], xi);
        F::store(&a.xw[p], xi);
        a.x[(long long)row * a.x_si] = xi;
      }
      if (ADJ && a.grad) {
        for (int e = a.dep_ptr[p] + lane; e < a.dep_ptr[p + 1]; e += G)
          a.grad[a.dep_src[e]] = -xi * a.xf[(long long)a.dep_col[e] * a.xf_si];
        if (lane == 0) a.grad[a.diag_src[p]] = -xi * a.xf[(long long)row * a.xf_si];
      }
    }
    if (__syncthreads_or(fail)) break;
  }
  leave(a.ctl);
}

// ------------------------------------------------------------------ pull, warp-synchronous
// One lane per unknown; the 32 lanes of a warp take 32 consecutive positions of
// the chunk and advance in lockstep: every iteration each unfinished lane
// consumes the dependencies that have arrived, issues the next loads (or
// re-polls what is still pending), and publishes its x once its list is done;
// __syncwarp() ends the iteration. A lane never spins while a lane of its own
// warp that it depends on waits to run, so a chain inside a warp (common in
// blocked orders of narrow DAGs) costs one short iteration per hop. Global
// waits back off only when no lane of the warp made progress.
//
// U = dependencies a lane loads per lockstep iteration. Small U keeps the
// iteration short, which is what a hop costs once the last dependency lands;
// ready-order lists let the earlier dependencies be consumed before that.
template <typename T, bool EXACT, bool ADJ, int U>
__global__ void __launch_bounds__(256) k_pull_wsync(ExecArgs<T> a) {
  using F = Flag<T>;
  using Bits = typename F::Bits;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_x = reinterpret_cast<T*>(smem_raw);
  __shared__ unsigned s_chunk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int* __restrict__ lptr = ADJ ? a.out_ptr : a.dep_ptr;
  const int* __restrict__ lpos = ADJ ? (EXACT ? a.out_pos : a.out_pos_f) : (EXACT ? a.dep_pos : a.dep_pos_f);
  const T* __restrict__ vals = ADJ ? (EXACT ? a.out_val : a.out_w) : (EXACT ? a.dep_val : a.dep_w);
  const int last = a.n - 1;
  for (;;) {
    const unsigned c = next_chunk(a.ctl, a.nchunks, &s_chunk);
    if (c >= (unsigned)a.nchunks) break;
    const int base0 = static_cast<int>(c) * a.chunk - a.walk_pad;
    const int base = max(base0, 0);
    const int cend = min(base0 + a.chunk, a.n);
    const int len = cend - base;
    if (a.smem_tier)
      for (int i = threadIdx.x; i < len; i += blockDim.x) *reinterpret_cast<Bits*>(&s_x[i]) = F::EMPTY;
    __syncthreads();
    bool fail = false;
    // row and list bounds of this warp's next segment are loaded one segment ahead
    int n_row = 0, n_e = 0, n_e1 = 0;
    auto fetch = [&](int sg) {
      const int jj = sg * 32 + lane;
      if (jj < len) {
        const int pp = ADJ ? last - (base + jj) : base + jj;
        n_row = a.perm[pp];
        n_e = lptr[pp];
        n_e1 = lptr[pp + 1];
      }
    };
    if (warp * 32 < len) fetch(warp);
    for (int seg = warp; seg * 32 < len && !fail; seg += nwarps) {
      const int j = seg * 32 + lane;
      bool done = j >= len;
      const int pr = base + j;
      const int p = ADJ ? last - pr : pr;
      const int row = n_row;
      int e = n_e;
      const int e1 = n_e1;
      if ((seg + nwarps) * 32 < len) fetch(seg + nwarps);
      T bi = T(0), sc = T(0), acc = T(0);
      if (!done) {
        bi = a.b[(long long)row * a.b_si];
        sc = EXACT ? a.diag[p] : a.rcp[p];
        acc = EXACT ? T(0) : bi * sc;
      }
      auto slot = [&](int q) {
        const int qr = ADJ ? last - q : q;
        return (a.smem_tier && qr >= base) ? qr - base : -1;
      };
      int q[U], ls[U];
      T w[U];
      Bits bits[U];
      unsigned todo = 0u;
      auto load_batch = [&]() {
        todo = 0u;
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int ee = e + u;
          q[u] = ee < e1 ? lpos[ee] : -1;
          w[u] = ee < e1 ? vals[ee] : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          ls[u] = -1;
          bits[u] = F::EMPTY;
          if (q[u] >= 0) {
            ls[u] = slot(q[u]);
            bits[u] = ls[u] >= 0 ? F::load_shared(&s_x[ls[u]]) : F::load(&a.xw[q[u]]);
            todo |= 1u << u;
          }
        }
      };
      if (!done) load_batch();
      WaitBudget wb(a.timeout_ns);
      unsigned nap = a.sleep_min, idle = 0u;
      for (;;) {
        bool progress = false, global_wait = false;
        if (!done) {
          bool prefix = true;
#pragma unroll
          for (int u = 0; u < U; ++u) {
            if (!(todo & (1u << u))) continue;
            if (bits[u] != F::EMPTY && (!EXACT || prefix)) {
              acc = EXACT ? exact_mul_add<T>(acc, w[u], F::value(bits[u])) : fma(-w[u], F::value(bits[u]), acc);
              todo &= ~(1u << u);
              progress = true;
            } else {
              prefix = false;
              if (bits[u] == F::EMPTY && ls[u] < 0) global_wait = true;
            }
          }
          if (!todo) {
            e += U;
            if (e < e1) {
              load_batch();
              progress = true;
            } else {
              const T xi = EXACT ? exact_finish<T>(bi, acc, sc) : acc;
              if (a.smem_tier) F::store_shared(&s_x[pr - base], xi);
              F::store(&a.xw[p], xi);
              a.x[(long long)row * a.x_si] = xi;
              if (ADJ && a.grad) {
                for (int ee = a.dep_ptr[p]; ee < a.dep_ptr[p + 1]; ++ee)
                  a.grad[a.dep_src[ee]] = -xi * a.xf[(long long)a.dep_col[ee] * a.xf_si];
                a.grad[a.diag_src[p]] = -xi * a.xf[(long long)row * a.xf_si];
              }
              done = true;
              progress = true;
            }
          } else {
            // every entry still pending is unpublished (arrived ones were consumed
            // above; in exact order a reload of an arrived one reads the same word)
#pragma unroll
            for (int u = 0; u < U; ++u)
              if (todo & (1u << u)) bits[u] = ls[u] >= 0 ? F::load_shared(&s_x[ls[u]]) : F::load(&a.xw[q[u]]);
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
    }
    if (__syncthreads_or(fail)) break;
  }
  leave(a.ctl);
}

// ------------------------------------------------------------------ pull, warp-synchronous, imported dependencies
// Blocked orders put most of a chunk's dependencies inside the chunk; the few
// that come from other chunks would make every lockstep iteration of the
// warps that hold them wait for an L2 round trip. Here one extra warp per CTA
// imports them: it polls the chunk's external positions (sorted, so roughly
// in the order they are published) from global memory and copies each value
// into a shared-memory slot as it lands. The consumer warps then resolve every
// dependency in shared memory (slot from dep_slot), so their iterations stay
// short. Fast arithmetic, one rhs, forward walks. ONE: every list holds at most
// U entries, so a lane publishes once its first batch is consumed.
template <typename T, int U, bool ONE>
__global__ void __launch_bounds__(288) k_pull_wsync_imp(ExecArgs<T> a) {
  using F = Flag<T>;
  using Bits = typename F::Bits;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_x = reinterpret_cast<T*>(smem_raw);
  __shared__ unsigned s_chunk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ncw = (blockDim.x >> 5) - 1;  // consumer warps; warp ncw imports
  const int* __restrict__ lpos = a.dep_pos_f;
  const T* __restrict__ vals = a.dep_w;
  for (;;) {
    const unsigned c = next_chunk(a.ctl, a.nchunks, &s_chunk);
    if (c >= (unsigned)a.nchunks) break;
    const int base = a.im_start[c];
    const int len = a.im_start[c + 1] - base;  // <= a.chunk (the window)
    const int i0 = a.im_ptr[c], nimp = a.im_ptr[c + 1] - i0;
    for (int i = threadIdx.x; i < len; i += blockDim.x) *reinterpret_cast<Bits*>(&s_x[i]) = F::EMPTY;
    for (int i = threadIdx.x; i < nimp; i += blockDim.x) *reinterpret_cast<Bits*>(&s_x[a.chunk + i]) = F::EMPTY;
    __syncthreads();
    bool fail = false;
    if (warp == ncw) {
      // importer: each lane walks its imports in order, one poll at a time
      WaitBudget wb(a.timeout_ns);
      unsigned idle = 0u;
      int i = lane;
      Bits v = F::EMPTY;
      if (i < nimp) v = F::load(&a.xw[a.im_q[i0 + i]]);
      for (;;) {
        bool progress = false;
        if (i < nimp) {
          if (v != F::EMPTY) {
            F::store_shared(&s_x[a.chunk + i], F::value(v));
            i += 32;
            v = i < nimp ? F::load(&a.xw[a.im_q[i0 + i]]) : F::EMPTY;
            progress = true;
          } else {
            v = F::load(&a.xw[a.im_q[i0 + i]]);
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
      // A warp takes every ncw-th segment of the chunk. Its next segment's
      // scaled right-hand side and first U list entries are loaded while it
      // works on the current one, and the row and list bounds they need one
      // segment earlier still, so a segment starts on values that have landed
      // instead of waiting for two dependent global round trips.
      int f_row = 0, f_e = 0, f_e1 = 0;           // bounds, two segments ahead
      auto fetch = [&](int sg) {
        const int jj = sg * 32 + lane;
        if (jj < len) {
          f_row = a.perm[base + jj];
          f_e = a.dep_ptr[base + jj];
          f_e1 = a.dep_ptr[base + jj + 1];
        }
      };
      int s_row = 0, s_e = 0, s_e1 = 0;           // staged, one segment ahead
      T s_acc = T(0);
      int s_ls[U];
      T s_w[U];
      auto stage = [&](int sg) {
        const int jj = sg * 32 + lane;
        s_row = f_row;
        s_e = f_e;
        s_e1 = jj < len ? f_e1 : f_e;
        s_acc = jj < len ? a.b[(long long)f_row * a.b_si] * a.rcp[base + jj] : T(0);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int ee = s_e + u;
          s_ls[u] = ee < s_e1 ? a.dep_slot[ee] : -1;
          s_w[u] = ee < s_e1 ? vals[ee] : T(0);
        }
      };
      if (warp * 32 < len) {
        fetch(warp);
        stage(warp);
        if ((warp + ncw) * 32 < len) fetch(warp + ncw);
      }
      for (int seg = warp; seg * 32 < len && !fail; seg += ncw) {
        const int j = seg * 32 + lane;
        bool done = j >= len;
        const int p = base + j;
        const int row = s_row;
        int e = s_e;
        const int e1 = s_e1;
        T acc = s_acc;
        int ls[U];
        T w[U];
        Bits bits[U];
        unsigned todo = 0u;
#pragma unroll
        for (int u = 0; u < U; ++u) {
          ls[u] = s_ls[u];
          w[u] = s_w[u];
        }
        if ((seg + ncw) * 32 < len) stage(seg + ncw);
        if ((seg + 2 * ncw) * 32 < len) fetch(seg + 2 * ncw);
        auto poll_batch = [&]() {
          todo = 0u;
#pragma unroll
          for (int u = 0; u < U; ++u) {
            bits[u] = F::EMPTY;
            if (ls[u] >= 0) {
              bits[u] = F::load_shared(&s_x[ls[u]]);
              todo |= 1u << u;
            }
          }
        };
        auto load_batch = [&]() {
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int ee = e + u;
            ls[u] = ee < e1 ? a.dep_slot[ee] : -1;
            w[u] = ee < e1 ? vals[ee] : T(0);
          }
          poll_batch();
        };
        if (!done) poll_batch();
        WaitBudget wb(a.timeout_ns);
        unsigned idle = 0u;
        for (;;) {
          bool progress = false;
          if (!done) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
              if (!(todo & (1u << u))) continue;
              if (bits[u] != F::EMPTY) {
                acc = fma(-w[u], F::value(bits[u]), acc);
                todo &= ~(1u << u);
                progress = true;
              }
            }
            if (!todo) {
              if (!ONE) e += U;
              if (!ONE && e < e1) {
                load_batch();
              } else {
                F::store_shared(&s_x[j], acc);
                F::store(&a.xw[p], acc);
                a.x[(long long)row * a.x_si] = acc;
                done = true;
              }
              progress = true;
            } else {
#pragma unroll
              for (int u = 0; u < U; ++u)  // pending entries are unpublished: arrived ones were consumed
                if (todo & (1u << u)) bits[u] = F::load_shared(&s_x[ls[u]]);
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
      }
    }
    if (__syncthreads_or(fail)) break;
  }
  leave(a.ctl);
}

// ------------------------------------------------------------------ pull, warp-synchronous, split lists
// As k_pull_wsync (fast arithmetic), over pieces: a dependency list longer than
// the split length is cut into up to 32 consecutive slices of its ready-ordered
// list, held by adjacent lanes of one warp segment. Every lane accumulates its
// slice in lockstep with the others; once all slices of an unknown are in, a
// segmented suffix sum over its lanes hands the head lane the value to publish.
// A 1000-entry list then takes about as many lockstep iterations as a
// 30-entry one, and only its last slice waits on the latest dependencies.
// Segments without a split list run the one-lane loop (SPLIT = false).
template <typename T, bool ADJ, bool SPLIT, int U>
__device__ __forceinline__ bool wsync_segment(const ExecArgs<T>& a, T* s_x, int cbase, int walk, int row, int e,
                                              const int e1, unsigned at_or_below) {
  using F = Flag<T>;
  using Bits = typename F::Bits;
  constexpr unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int* __restrict__ lpos = ADJ ? a.out_pos_f : a.dep_pos_f;
  const T* __restrict__ vals = ADJ ? a.out_w : a.dep_w;
  const int last = a.n - 1;
  const bool valid = walk >= 0;
  bool head = valid;
  int ge = lane, gs = lane;
  unsigned gmask = 0u;
  int step = 1;  // entries of an unknown split over k lanes interleave: lane j takes j, j+k, j+2k, ...
  unsigned heads = 0u;  // split segments: first lane of every unknown (warp-uniform)
  if (SPLIT) {
    const int prev = __shfl_up_sync(kFull, walk, 1);
    head = valid && (lane == 0 || prev != walk);
    heads = __ballot_sync(kFull, head);
    const unsigned valids = __ballot_sync(kFull, valid);
    // this lane's group: from its head (at or below) to the lane before the next head
    const unsigned above = heads & ~at_or_below;
    ge = above ? __ffs(above) - 2 : 31 - __clz(valids);
    gs = valid ? 31 - __clz(heads & at_or_below) : lane;
    // head lanes: the lanes of their unknown (ge >= lane >= 0 there)
    gmask = head ? (ge >= 31 ? kFull : ((2u << ge) - 1u)) & ~((1u << lane) - 1u) : 0u;
    step = valid ? ge - gs + 1 : 1;
  }
  // the widest unknown of the segment bounds the suffix-sum rounds (most split
  // lists span a few lanes, so usually one or two rounds instead of five)
  const unsigned span = SPLIT ? __reduce_max_sync(kFull, static_cast<unsigned>(step)) : 1u;
  const int p = ADJ ? last - walk : walk;
  T acc = T(0);
  if (head) acc = a.b[(long long)row * a.b_si] * a.rcp[p];
  auto slot = [&](int q) {
    const int qr = ADJ ? last - q : q;
    return (a.smem_tier && qr >= cbase) ? qr - cbase : -1;
  };
  auto publish = [&](T xi) {
    if (a.smem_tier) F::store_shared(&s_x[walk - cbase], xi);
    F::store(&a.xw[p], xi);
    a.x[(long long)row * a.x_si] = xi;
  };
  int q[U], ls[U];
  T w[U];
  Bits bits[U];
  unsigned todo = 0u;
  auto load_batch = [&]() {
    todo = 0u;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int ee = e + u * (SPLIT ? step : 1);
      q[u] = ee < e1 ? lpos[ee] : -1;
      w[u] = ee < e1 ? vals[ee] : T(0);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      ls[u] = -1;
      bits[u] = F::EMPTY;
      if (q[u] >= 0) {
        ls[u] = slot(q[u]);
        bits[u] = ls[u] >= 0 ? F::load_shared(&s_x[ls[u]]) : F::load(&a.xw[q[u]]);
        todo |= 1u << u;
      }
    }
  };
  bool sdone = !valid;  // slice consumed (one-lane unknowns publish at the same moment)
  bool done = !valid;   // unknown published
  unsigned published = 0u;  // split segments: heads of the unknowns published so far (warp-uniform)
  if (__all_sync(kFull, done)) return false;
  if (!sdone) load_batch();
  WaitBudget wb(a.timeout_ns);
  unsigned nap = a.sleep_min, idle = 0u;
  for (;;) {
    bool progress = false, global_wait = false;
    if (!sdone) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (!(todo & (1u << u))) continue;
        if (bits[u] != F::EMPTY) {
          acc = fma(-w[u], F::value(bits[u]), acc);
          todo &= ~(1u << u);
          progress = true;
        } else if (ls[u] < 0) {
          global_wait = true;
        }
      }
      if (!todo) {
        e += U * (SPLIT ? step : 1);
        if (e < e1) {
          load_batch();
        } else {
          sdone = true;
          if (!SPLIT) {
            publish(acc);
            done = true;
          }
        }
        progress = true;
      } else {
        // (the re-poll keeps its empty check here: without it, the same loads
        // measured 12 % slower on the power-law backward walk)
#pragma unroll
        for (int u = 0; u < U; ++u)
          if ((todo & (1u << u)) && bits[u] == F::EMPTY)
            bits[u] = ls[u] >= 0 ? F::load_shared(&s_x[ls[u]]) : F::load(&a.xw[q[u]]);
      }
    }
    // Nothing consumed in the warp means no slice finished and nothing was
    // published, so the completion checks (and their warp votes) are skipped.
    const bool any_progress = __any_sync(kFull, progress);
    if (any_progress) {
      if (SPLIT) {
        // publish every unknown whose slices are all in. Which unknowns are
        // complete follows from one ballot, worked out identically by every
        // lane: a segmented OR from each unknown's last lane down to its head
        // marks the unknowns that still have a lane with its slice pending.
        const unsigned pending = ~__ballot_sync(kFull, sdone);
        unsigned v = pending, f = (heads >> 1) | 0x80000000u;  // f: last lane of an unknown
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const unsigned open = ~f;
          v |= (v >> d) & open;
          f |= (f >> d) & open;
        }
        const unsigned ready = heads & ~v & ~published;
        if (ready) {
          T xi = acc;
#pragma unroll
          for (unsigned off = 1; off < span; off <<= 1) {
            const T t = __shfl_down_sync(kFull, xi, off);
            if (lane + static_cast<int>(off) <= ge) xi += t;
          }
          if ((ready >> lane) & 1u) publish(xi);
          published |= ready;
          if (valid) done = (published >> gs) & 1u;
        }
        if (published == heads) return false;
      } else if (__all_sync(kFull, done)) {
        return false;
      }
      __syncwarp();
      nap = a.sleep_min;
    } else {
      const bool any_global = __any_sync(kFull, global_wait);
      __syncwarp();
      if (any_global && a.sleep_max) {
        __nanosleep(nap);
        nap = nap * 2u < a.sleep_max ? nap * 2u : a.sleep_max;
      }
      bool fail = false;
      if ((any_global || (++idle & 255u) == 0u) && !wb.poll(a.ctl, p)) fail = true;
      if (__any_sync(kFull, fail)) return true;
    }
  }
}

template <typename T, bool ADJ, int U>
__global__ void __launch_bounds__(256) k_pull_wsync_split(ExecArgs<T> a) {
  using F = Flag<T>;
  using Bits = typename F::Bits;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_x = reinterpret_cast<T*>(smem_raw);
  __shared__ unsigned s_chunk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const unsigned at_or_below = (2u << lane) - 1u;  // lanes 0..lane (wraps to all lanes for lane 31)
  for (;;) {
    const unsigned c = next_chunk(a.ctl, a.nchunks, &s_chunk);
    if (c >= (unsigned)a.nchunks) break;
    const int seg0 = a.pc_cseg[c];
    const int seg1 = a.pc_cseg[c + 1];
    const int cbase = a.pc_cbase[c];
    if (a.smem_tier)
      for (int i = threadIdx.x; i < min(a.chunk, a.n - cbase); i += blockDim.x)
        *reinterpret_cast<Bits*>(&s_x[i]) = F::EMPTY;
    __syncthreads();
    bool fail = false;
    // piece data of this warp's next segment is loaded one segment ahead
    int n_walk = -1, n_lo = 0, n_hi = 0, n_row = 0, n_split = 0;
    auto fetch = [&](int sg) {
      const int pi = sg * 32 + lane;
      n_walk = a.pc_walk[pi];
      n_lo = a.pc_lo[pi];
      n_hi = a.pc_hi[pi];
      n_row = a.pc_row[pi];
      n_split = a.pc_split[sg];
    };
    if (seg0 + warp < seg1) fetch(seg0 + warp);
    for (int seg = seg0 + warp; seg < seg1 && !fail; seg += nwarps) {
      const int walk = n_walk, lo = n_lo, hi = n_hi, row = n_row;
      const bool split = n_split != 0;  // some unknown of the segment spans several lanes
      if (seg + nwarps < seg1) fetch(seg + nwarps);
      fail = split ? wsync_segment<T, ADJ, true, U>(a, s_x, cbase, walk, row, lo, hi, at_or_below)
                   : wsync_segment<T, ADJ, false, U>(a, s_x, cbase, walk, row, lo, hi, at_or_below);
    }
    if (__syncthreads_or(fail)) break;
  }
  leave(a.ctl);
}

// ------------------------------------------------------------------ pull, warp-synchronous, many rhs
// As k_pull_wsync, with G lanes per unknown (32/G unknowns per warp), each lane
// covering RPL right-hand sides (rhs <= G*RPL). A group moves to its next
// batch of dependencies once every lane of the group has consumed the batch.
template <typename T, bool EXACT, bool ADJ, int G, int RPL>
__global__ void __launch_bounds__(256) k_pull_wsync_multi(ExecArgs<T> a) {
  using F = Flag<T>;
  using Bits = typename F::Bits;
  constexpr int UD = 2;
  constexpr int P = 32 / G;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_x = reinterpret_cast<T*>(smem_raw);
  __shared__ unsigned s_chunk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int gi = lane / G, gl = lane % G;
  const unsigned gmask = group_mask(G);
  const int rhs = a.rhs;
  const int* __restrict__ lptr = ADJ ? a.out_ptr : a.dep_ptr;
  const int* __restrict__ lpos = ADJ ? (EXACT ? a.out_pos : a.out_pos_f) : (EXACT ? a.dep_pos : a.dep_pos_f);
  const T* __restrict__ vals = ADJ ? (EXACT ? a.out_val : a.out_w) : (EXACT ? a.dep_val : a.dep_w);
  const int last = a.n - 1;
  for (;;) {
    const unsigned c = next_chunk(a.ctl, a.nchunks, &s_chunk);
    if (c >= (unsigned)a.nchunks) break;
    const int base0 = static_cast<int>(c) * a.chunk - a.walk_pad;
    const int base = max(base0, 0);
    const int cend = min(base0 + a.chunk, a.n);
    const int len = cend - base;
    if (a.smem_tier)
      for (long long i = threadIdx.x; i < (long long)len * rhs; i += blockDim.x)
        *reinterpret_cast<Bits*>(&s_x[i]) = F::EMPTY;
    __syncthreads();
    bool fail = false;
    for (int seg = warp; seg * P < len && !fail; seg += nwarps) {
      const int j = seg * P + gi;
      bool done = j >= len;     // group-uniform
      const int pr = base + j;
      const int p = ADJ ? last - pr : pr;
      int row = 0, e = 0, e1 = 0;
      T sc = T(0);
      T acc[RPL];
#pragma unroll
      for (int r = 0; r < RPL; ++r) acc[r] = T(0);
      if (!done) {
        row = a.perm[p];
        e = lptr[p];
        e1 = lptr[p + 1];
        sc = EXACT ? a.diag[p] : a.rcp[p];
        if (!EXACT) {
#pragma unroll
          for (int r = 0; r < RPL; ++r) {
            const int k = gl + r * G;
            if (k < rhs) acc[r] = a.b[(long long)row * a.b_si + (long long)k * a.b_sk] * sc;
          }
        }
      }
      int q[UD], sl[UD];
      T w[UD];
      Bits bits[UD][RPL];
      unsigned todo = 0u;
      auto load_batch = [&]() {
        todo = 0u;
#pragma unroll
        for (int u = 0; u < UD; ++u) {
          q[u] = e + u < e1 ? lpos[e + u] : -1;
          w[u] = e + u < e1 ? vals[e + u] : T(0);
          const int qr = ADJ ? last - q[u] : q[u];
          sl[u] = (q[u] >= 0 && a.smem_tier && qr >= base) ? qr - base : -1;
#pragma unroll
          for (int r = 0; r < RPL; ++r) {
            const int k = gl + r * G;
            bits[u][r] = F::EMPTY;
            if (q[u] >= 0 && k < rhs) {
              bits[u][r] = sl[u] >= 0 ? F::load_shared(&s_x[(long long)sl[u] * rhs + k])
                                      : F::load(&a.xw[(long long)q[u] * rhs + k]);
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
          for (int r = 0; r < RPL; ++r) {
            bool prefix = true;
#pragma unroll
            for (int u = 0; u < UD; ++u) {
              const unsigned bit = 1u << (u * RPL + r);
              if (!(todo & bit)) continue;
              if (bits[u][r] != F::EMPTY && (!EXACT || prefix)) {
                acc[r] = EXACT ? exact_mul_add<T>(acc[r], w[u], F::value(bits[u][r])) : fma(-w[u], F::value(bits[u][r]), acc[r]);
                todo &= ~bit;
                progress = true;
              } else {
                prefix = false;
                if (bits[u][r] == F::EMPTY && sl[u] < 0) global_wait = true;
              }
            }
          }
        }
        // a group advances once all its lanes have consumed the batch
        const unsigned empty_lanes = __ballot_sync(0xffffffffu, done || todo == 0u);
        const bool group_clear = (empty_lanes & gmask) == gmask;
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
                  const T xi = EXACT ? exact_finish<T>(a.b[(long long)row * a.b_si + (long long)k * a.b_sk], acc[r], sc)
                                     : acc[r];
                  acc[r] = xi;
                  if (a.smem_tier) F::store_shared(&s_x[(long long)(pr - base) * rhs + k], xi);
                  F::store(&a.xw[(long long)p * rhs + k], xi);
                  a.x[(long long)row * a.x_si + (long long)k * a.x_sk] = xi;
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
                if ((todo & (1u << (u * RPL + r))) && bits[u][r] == F::EMPTY)
                  bits[u][r] = sl[u] >= 0 ? F::load_shared(&s_x[(long long)sl[u] * rhs + k])
                                          : F::load(&a.xw[(long long)q[u] * rhs + k]);
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
    }
    if (__syncthreads_or(fail)) break;
  }
  leave(a.ctl);
}

// ------------------------------------------------------------------ pull, many rhs
// Lanes of a group cover right-hand sides; dependencies are walked in order.
template <typename T, int G, int RPL, bool EXACT, bool ADJ>
__global__ void __launch_bounds__(256) k_pull_multi(ExecArgs<T> a) {
  using F = Flag<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_x = reinterpret_cast<T*>(smem_raw);
  __shared__ unsigned s_chunk;
  const int NG = blockDim.x / G;
  const int g = threadIdx.x / G, lane = threadIdx.x % G;
  const unsigned gmask = group_mask(G);
  const int rhs = a.rhs;
  const int* __restrict__ lptr = ADJ ? a.out_ptr : a.dep_ptr;
  const int* __restrict__ lpos = ADJ ? (EXACT ? a.out_pos : a.out_pos_f) : (EXACT ? a.dep_pos : a.dep_pos_f);
  const T* __restrict__ vals = ADJ ? (EXACT ? a.out_val : a.out_w) : (EXACT ? a.dep_val : a.dep_w);
  const int last = a.n - 1;
  for (;;) {
    const unsigned c = next_chunk(a.ctl, a.nchunks, &s_chunk);
    if (c >= (unsigned)a.nchunks) break;
    const int base0 = static_cast<int>(c) * a.chunk - a.walk_pad;
    const int base = max(base0, 0);
    const int cend = min(base0 + a.chunk, a.n);
    if (a.smem_tier)
      for (long long i = threadIdx.x; i < (long long)(cend - base) * rhs; i += blockDim.x)
        *reinterpret_cast<typename F::Bits*>(&s_x[i]) = F::EMPTY;
    __syncthreads();
    bool fail = false;
    for (int pr = base + g; pr < cend && !fail; pr += NG) {
      const int p = ADJ ? last - pr : pr;
      const int row = a.perm[p];
      const int e0 = lptr[p], e1 = lptr[p + 1];
      const T dg = EXACT ? a.diag[p] : T(0);
      const T rc = EXACT ? T(0) : a.rcp[p];
      for (int kt = 0; kt < rhs && !fail; kt += G * RPL) {
        T acc[RPL];
#pragma unroll
        for (int j = 0; j < RPL; ++j) {
          const int k = kt + lane + j * G;
          acc[j] = (!EXACT && k < rhs) ? a.b[(long long)row * a.b_si + (long long)k * a.b_sk] * rc : T(0);
        }
        // dependencies in batches of UD: all flag loads of a batch (every dependency x every
        // right-hand side this lane covers) are issued together and re-polled together
        constexpr int UD = 4;
        for (int eb = e0; eb < e1 && !fail; eb += UD) {
          int q[UD], sl[UD];
          T v[UD];
          typename F::Bits bits[UD][RPL];
          unsigned todo = 0u;
#pragma unroll
          for (int u = 0; u < UD; ++u) {
            q[u] = eb + u < e1 ? lpos[eb + u] : -1;
            v[u] = eb + u < e1 ? vals[eb + u] : T(0);
            const int qr = ADJ ? last - q[u] : q[u];
            sl[u] = (q[u] >= 0 && a.smem_tier && qr >= base) ? qr - base : -1;
          }
#pragma unroll
          for (int u = 0; u < UD; ++u)
#pragma unroll
            for (int j = 0; j < RPL; ++j) {
              const int k = kt + lane + j * G;
              bits[u][j] = F::EMPTY;
              if (q[u] >= 0 && k < rhs) {
                bits[u][j] = sl[u] >= 0 ? F::load_shared(&s_x[(long long)sl[u] * rhs + k])
                                        : F::load(&a.xw[(long long)q[u] * rhs + k]);
                todo |= 1u << (u * RPL + j);
              }
            }
          WaitBudget wb(a.timeout_ns);
          unsigned nap = a.sleep_min;
          for (;;) {
            bool global_pending = false;
#pragma unroll
            for (int j = 0; j < RPL; ++j) {
              bool prefix = true;
#pragma unroll
              for (int u = 0; u < UD; ++u) {
                const unsigned bit = 1u << (u * RPL + j);
                if (!(todo & bit)) continue;
                if (bits[u][j] != F::EMPTY && (!EXACT || prefix)) {
                  acc[j] = EXACT ? mul_add<T>(acc[j], v[u], F::value(bits[u][j]), true)
                                 : fma(-v[u], F::value(bits[u][j]), acc[j]);
                  todo &= ~bit;
                } else {
                  prefix = false;
                  if (bits[u][j] == F::EMPTY && sl[u] < 0) global_pending = true;
                }
              }
            }
            if (!todo) break;
            if (global_pending && a.sleep_max) {
              __nanosleep(nap);
              nap = nap * 2u < a.sleep_max ? nap * 2u : a.sleep_max;
            }
            if (!wb.poll(a.ctl, p)) { fail = true; break; }
#pragma unroll
            for (int u = 0; u < UD; ++u)
#pragma unroll
              for (int j = 0; j < RPL; ++j) {
                const int k = kt + lane + j * G;
                if ((todo & (1u << (u * RPL + j))) && bits[u][j] == F::EMPTY)
                  bits[u][j] = sl[u] >= 0 ? F::load_shared(&s_x[(long long)sl[u] * rhs + k])
                                          : F::load(&a.xw[(long long)q[u] * rhs + k]);
              }
          }
        }
        fail = __any_sync(gmask, fail);
        if (fail) break;
#pragma unroll
        for (int j = 0; j < RPL; ++j) {
          const int k = kt + lane + j * G;
          if (k < rhs) {
            const T xi = EXACT ? finish<T>(a.b[(long long)row * a.b_si + (long long)k * a.b_sk], acc[j], dg, rc, true)
                               : acc[j];
            acc[j] = xi;
            if (a.smem_tier) F::store_shared(&s_x[(long long)(pr - base) * rhs + k], xi);
            F::store(&a.xw[(long long)p * rhs + k], xi);
            a.x[(long long)row * a.x_si + (long long)k * a.x_sk] = xi;
          }
        }
        if (ADJ && a.grad) {
          // dL(p,j) = -sum_k lambda_{p,k} x_{j,k}: this tile's share, reduced over the group
          for (int e = a.dep_ptr[p] - 1; e < a.dep_ptr[p + 1]; ++e) {
            const int col = e < a.dep_ptr[p] ? row : a.dep_col[e];
            T part = T(0);
#pragma unroll
            for (int j = 0; j < RPL; ++j) {
              const int k = kt + lane + j * G;
              if (k < rhs) part = fma(acc[j], a.xf[(long long)col * a.xf_si + (long long)k * a.xf_sk], part);
            }
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) part += __shfl_xor_sync(gmask, part, o);
            if (lane == 0) {
              T* dst = &a.grad[e < a.dep_ptr[p] ? a.diag_src[p] : a.dep_src[e]];
              *dst = (kt == 0 ? T(0) : *dst) - part;
            }
          }
        }
      }
    }
    if (__syncthreads_or(fail)) break;
  }
  leave(a.ctl);
}

// ------------------------------------------------------------------ push, one rhs
template <typename T>
__device__ __forceinline__ void smem_atomic_add(T* p, T v) { atomicAdd(p, v); }

template <typename T, int G>
__global__ void __launch_bounds__(256) k_push_vec(ExecArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_sum = reinterpret_cast<T*>(smem_raw);
  unsigned* s_cnt = reinterpret_cast<unsigned*>(s_sum + a.chunk);
  __shared__ unsigned s_chunk;
  const int NG = blockDim.x / G;
  const int g = threadIdx.x / G, lane = threadIdx.x % G;
  const unsigned gmask = group_mask(G);
  const int lane0 = (threadIdx.x & 31) & ~(G - 1);
  for (;;) {
    const unsigned c = next_chunk(a.ctl, a.nchunks, &s_chunk);
    if (c >= (unsigned)a.nchunks) break;
    const int base = static_cast<int>(c) * a.chunk;
    const int cend = min(base + a.chunk, a.n);
    if (a.smem_tier)
      for (int i = threadIdx.x; i < cend - base; i += blockDim.x) { s_sum[i] = T(0); s_cnt[i] = 0u; }
    __syncthreads();
    bool fail = false;
    for (int p = base + g; p < cend; p += NG) {
      const int col = a.perm[p];
      const unsigned target = static_cast<unsigned>(a.dep_ptr[p + 1] - a.dep_ptr[p]);
      const T bi = a.b[(long long)col * a.b_si];
      const T rc = a.rcp[p];
      T sum = T(0);
      if (lane == 0) {
        // Consumer: wait until global + shared arrivals cover the in-degree.
        WaitBudget w(a.timeout_ns, a.sleep_min, a.sleep_max);
        for (;;) {
          unsigned got = target == 0u ? 0u : ld_acquire_u32(&a.counters[p]);
          if (a.smem_tier && target != 0u) got += ld_shared_acquire_u32(&s_cnt[p - base]);
          if (got == target) break;
          if (!w.poll(a.ctl, p)) { fail = true; break; }
        }
        if (!fail) {
          if (target != 0u) {
            sum = Flag<T>::value(Flag<T>::load(&a.left_sum[p]));
            if (a.smem_tier) sum += *reinterpret_cast<volatile T*>(&s_sum[p - base]);
            // Self-clean the global slots for the next solve (all producers are done).
            a.counters[p] = 0u;
            a.left_sum[p] = T(0);
          }
        }
      }
      if (G > 1) {
        fail = __shfl_sync(gmask, fail ? 1 : 0, lane0) != 0;
        sum = __shfl_sync(gmask, sum, lane0);
      }
      if (fail) break;
      const T xi = (bi - sum) * rc;
      // Producer: partial sums first, one fence, then the arrival counters.
      const int o0 = a.out_ptr[p], o1 = a.out_ptr[p + 1];
      for (int e = o0 + lane; e < o1; e += G) {
        const int tp = a.out_pos[e];
        const T contrib = xi * a.out_val[e];
        if (a.smem_tier && tp < cend) smem_atomic_add(&s_sum[tp - base], contrib);
        else if (sizeof(T) == 8) red_add_f64(reinterpret_cast<double*>(&a.left_sum[tp]), (double)contrib);
        else red_add_f32(reinterpret_cast<float*>(&a.left_sum[tp]), (float)contrib);
      }
      __threadfence();
      for (int e = o0 + lane; e < o1; e += G) {
        const int tp = a.out_pos[e];
        if (a.smem_tier && tp < cend) atomicAdd(&s_cnt[tp - base], 1u);
        else red_relaxed_add_u32(&a.counters[tp], 1u);
      }
      if (lane == 0) a.x[(long long)col * a.x_si] = xi;
    }
    if (__syncthreads_or(fail)) break;
  }
  leave(a.ctl);
}

// ------------------------------------------------------------------ push, many rhs
template <typename T, int G, int RPL>
__global__ void __launch_bounds__(256) k_push_multi(ExecArgs<T> a) {
  __shared__ unsigned s_chunk;
  const int NG = blockDim.x / G;
  const int g = threadIdx.x / G, lane = threadIdx.x % G;
  const unsigned gmask = group_mask(G);
  const int lane0 = (threadIdx.x & 31) & ~(G - 1);
  const int rhs = a.rhs;
  for (;;) {
    const unsigned c = next_chunk(a.ctl, a.nchunks, &s_chunk);
    if (c >= (unsigned)a.nchunks) break;
    const int base = static_cast<int>(c) * a.chunk;
    const int cend = min(base + a.chunk, a.n);
    bool fail = false;
    for (int p = base + g; p < cend; p += NG) {
      const int col = a.perm[p];
      const unsigned target = static_cast<unsigned>(a.dep_ptr[p + 1] - a.dep_ptr[p]);
      if (lane == 0 && target != 0u) {
        WaitBudget w(a.timeout_ns, a.sleep_min, a.sleep_max);
        while (ld_acquire_u32(&a.counters[p]) != target) {
          if (!w.poll(a.ctl, p)) { fail = true; break; }
        }
      }
      fail = __shfl_sync(gmask, fail ? 1 : 0, lane0) != 0;
      if (fail) break;
      // Make lane 0's acquire cover the whole group before its loads.
      __syncwarp(gmask);
      const T rc = a.rcp[p];
      const int o0 = a.out_ptr[p], o1 = a.out_ptr[p + 1];
      // Lanes over right-hand sides (the loop below) or over the column's
      // entries (after it); the automatic mode is the reference's rule
      // (SpTRSV_cuda/sptrsv_syncfree_cuda.h:258-262), decided per column.
      const int len = o1 - o0;
      const bool rhs_lanes = a.opt == 2 || (a.opt != 1 && (len <= rhs || rhs > 16) && len < 2048);
      for (int kt = 0; kt < rhs; kt += G * RPL) {
        T xi[RPL];
#pragma unroll
        for (int j = 0; j < RPL; ++j) {
          const int k = kt + lane + j * G;
          xi[j] = T(0);
          if (k < rhs) {
            T s = T(0);
            if (target != 0u) {
              T* slot = &a.left_sum[(long long)p * rhs + k];
              s = Flag<T>::value(Flag<T>::load(slot));
              *slot = T(0);
            }
            xi[j] = (a.b[(long long)col * a.b_si + (long long)k * a.b_sk] - s) * rc;
            a.x[(long long)col * a.x_si + (long long)k * a.x_sk] = xi[j];
          }
        }
        if (!rhs_lanes) continue;
        for (int e = o0; e < o1; ++e) {
          const int tp = a.out_pos[e];
          const T v = a.out_val[e];
#pragma unroll
          for (int j = 0; j < RPL; ++j) {
            const int k = kt + lane + j * G;
            if (k < rhs) {
              T* dst = &a.left_sum[(long long)tp * rhs + k];
              if (sizeof(T) == 8) red_add_f64(reinterpret_cast<double*>(dst), (double)(xi[j] * v));
              else red_add_f32(reinterpret_cast<float*>(dst), (float)(xi[j] * v));
            }
          }
        }
      }
      if (!rhs_lanes) {
        // lanes over entries: each lane pushes x_p * L(r, p) of its dependents for
        // every right-hand side, reading x_p back (written by the group above)
        __syncwarp(gmask);
        for (int e = o0 + lane; e < o1; e += G) {
          const int tp = a.out_pos[e];
          const T v = a.out_val[e];
          for (int k = 0; k < rhs; ++k) {
            T* dst = &a.left_sum[(long long)tp * rhs + k];
            const T xk = a.x[(long long)col * a.x_si + (long long)k * a.x_sk];
            if (sizeof(T) == 8) red_add_f64(reinterpret_cast<double*>(dst), (double)(xk * v));
            else red_add_f32(reinterpret_cast<float*>(dst), (float)(xk * v));
          }
        }
      }
      if (target != 0u && lane == 0) a.counters[p] = 0u;
      // All lanes' partial sums, then one fence, then the counters (one lane).
      __syncwarp(gmask);
      if (lane == 0) {
        __threadfence();
        for (int e = o0; e < o1; ++e) red_relaxed_add_u32(&a.counters[a.out_pos[e]], 1u);
      }
    }
    if (__syncthreads_or(fail)) break;
  }
  leave(a.ctl);
}

// ------------------------------------------------------------------ level sets
template <typename T, int G>
__global__ void __launch_bounds__(256) k_levelset(ExecArgs<T> a) {
  using F = Flag<T>;
  const int NG = blockDim.x / G;
  const long long gstride = (long long)gridDim.x * NG;
  const int g = threadIdx.x / G, lane = threadIdx.x % G;
  const unsigned gmask = group_mask(G);
  const int rhs = a.rhs;
  for (int l = 0; l < a.nlevels; ++l) {
    const int p0 = a.level_ptr[l], p1 = a.level_ptr[l + 1];
    for (long long pp = p0 + (long long)blockIdx.x * NG + g; pp < p1; pp += gstride) {
      const int p = static_cast<int>(pp);
      const int row = a.perm[p];
      const int e0 = a.dep_ptr[p], e1 = a.dep_ptr[p + 1];
      const T rc = a.rcp[p];
      for (int k = 0; k < rhs; ++k) {
        T acc = lane == 0 ? a.b[(long long)row * a.b_si + (long long)k * a.b_sk] * rc : T(0);
        for (int e = e0 + lane; e < e1; e += G)
          acc = fma(-a.dep_w[e], F::value(F::load(&a.xw[(long long)a.dep_pos_f[e] * rhs + k])), acc);
        if (G > 1) {
#pragma unroll
          for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(gmask, acc, o);
        }
        if (lane == 0) {
          const T xi = acc;
          F::store(&a.xw[(long long)p * rhs + k], xi);
          a.x[(long long)row * a.x_si + (long long)k * a.x_sk] = xi;
        }
      }
    }
    if (!grid_barrier(a.ctl, a.timeout_ns)) return;
  }
}

template <typename T>
ExecArgs<T> make_args(const Layout& L, const Values<T>& V, int rhs, const VecView<T>& v, int chunk) {
  ExecArgs<T> a{};
  a.sleep_min = 0;
  a.sleep_max = 0;
  a.n = L.n;
  a.rhs = rhs;
  a.chunk = chunk;
  a.nchunks = (L.n + chunk - 1) / chunk;
  a.perm = L.perm;
  a.dep_ptr = L.dep_ptr;
  a.dep_pos = L.dep_pos;
  a.dep_pos_f = L.dep_pos_f;
  a.dep_val = V.dep_val;
  a.dep_w = V.dep_w;
  a.dep_src = L.dep_src;
  a.dep_col = L.dep_col;
  a.diag_src = L.diag_src;
  a.out_w = V.out_w;
  a.out_ptr = L.out_ptr;
  a.out_pos = L.out_pos;
  a.out_pos_f = L.out_pos_f;
  a.out_val = V.out_val;
  a.diag = V.diag;
  a.rcp = V.rcp;
  a.b = v.b;
  a.x = v.x;
  a.b_si = v.b_si;
  a.b_sk = v.b_sk;
  a.x_si = v.x_si;
  a.x_sk = v.x_sk;
  return a;
}

template <typename K>
int persistent_grid(K kernel, int block, size_t smem, int num_sms, int nchunks, int cap_per_sm) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
  if (per_sm < 1) per_sm = 1;
  if (cap_per_sm > 0 && per_sm > cap_per_sm) per_sm = cap_per_sm;
  long long grid = (long long)num_sms * per_sm;
  if (grid > nchunks) grid = nchunks;
  if (grid < 1) grid = 1;
  return static_cast<int>(grid);
}

template <typename K>
cudaError_t launch_persistent(K kernel, const ExecArgs<int>*, int, size_t, int, cudaStream_t);

template <typename T, typename K>
cudaError_t run(K kernel, const ExecArgs<T>& a, int block, size_t smem, int num_sms, cudaStream_t s) {
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const int grid = persistent_grid(kernel, block, smem, num_sms, a.nchunks, a.ctas_per_sm);
  kernel<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

size_t pull_smem_bytes(int chunk, int rhs, size_t elem) { return (size_t)chunk * (size_t)rhs * elem; }

template <typename T, bool ADJ>
cudaError_t launch_pull_impl(ExecArgs<T>& a, int rhs, const ExecConfig& cfg, size_t smem, int num_sms,
                             cudaStream_t s) {
  const int block = cfg.block;
  if (rhs == 1 && cfg.wsync && !cfg.exact && a.grad == nullptr && a.pc_walk != nullptr)
    switch (cfg.wsync_batch) {
      case 1: return run(k_pull_wsync_split<T, ADJ, 1>, a, block, smem, num_sms, s);
      case 2: return run(k_pull_wsync_split<T, ADJ, 2>, a, block, smem, num_sms, s);
      default: return run(k_pull_wsync_split<T, ADJ, 4>, a, block, smem, num_sms, s);
    }
  if (rhs == 1 && cfg.wsync) {
    if (cfg.exact) return run(k_pull_wsync<T, true, ADJ, 4>, a, block, smem, num_sms, s);
    switch (cfg.wsync_batch) {
      case 1: return run(k_pull_wsync<T, false, ADJ, 1>, a, block, smem, num_sms, s);
      case 2: return run(k_pull_wsync<T, false, ADJ, 2>, a, block, smem, num_sms, s);
      default: return run(k_pull_wsync<T, false, ADJ, 4>, a, block, smem, num_sms, s);
    }
  }
  if (rhs == 1) {
    if (cfg.exact) return run(k_pull_vec<T, 1, true, 4, ADJ>, a, block, smem, num_sms, s);
    switch (cfg.lanes) {
      case 1: return run(k_pull_vec<T, 1, false, 4, ADJ>, a, block, smem, num_sms, s);
      case 2: return run(k_pull_vec<T, 2, false, 2, ADJ>, a, block, smem, num_sms, s);
      case 4: return run(k_pull_vec<T, 4, false, 2, ADJ>, a, block, smem, num_sms, s);
      case 8: return run(k_pull_vec<T, 8, false, 1, ADJ>, a, block, smem, num_sms, s);
      case 16: return run(k_pull_vec<T, 16, false, 1, ADJ>, a, block, smem, num_sms, s);
      default: return run(k_pull_vec<T, 32, false, 1, ADJ>, a, block, smem, num_sms, s);
    }
  }
  // many right-hand sides: lanes over rhs, G lanes per unknown covering RPL
  // right-hand sides each (the right-hand-side tile, multi_group)
  if (cfg.wsync && rhs <= 64 && a.grad == nullptr) {
    if (cfg.exact) {
      if (rhs <= 8) return run(k_pull_wsync_multi<T, true, ADJ, 8, 1>, a, block, smem, num_sms, s);
      return run(k_pull_wsync_multi<T, true, ADJ, 32, 2>, a, block, smem, num_sms, s);
    }
    int rpl = 1;
    const int g = multi_group(rhs, cfg.rhs_tile, &rpl);
    switch (g * 8 + rpl) {
      case 4 * 8 + 1: return run(k_pull_wsync_multi<T, false, ADJ, 4, 1>, a, block, smem, num_sms, s);
      case 8 * 8 + 1: return run(k_pull_wsync_multi<T, false, ADJ, 8, 1>, a, block, smem, num_sms, s);
      case 16 * 8 + 1: return run(k_pull_wsync_multi<T, false, ADJ, 16, 1>, a, block, smem, num_sms, s);
      case 32 * 8 + 1: return run(k_pull_wsync_multi<T, false, ADJ, 32, 1>, a, block, smem, num_sms, s);
      case 4 * 8 + 2: return run(k_pull_wsync_multi<T, false, ADJ, 4, 2>, a, block, smem, num_sms, s);
      case 8 * 8 + 2: return run(k_pull_wsync_multi<T, false, ADJ, 8, 2>, a, block, smem, num_sms, s);
      case 16 * 8 + 2: return run(k_pull_wsync_multi<T, false, ADJ, 16, 2>, a, block, smem, num_sms, s);
      case 32 * 8 + 2: return run(k_pull_wsync_multi<T, false, ADJ, 32, 2>, a, block, smem, num_sms, s);
      case 4 * 8 + 4: return run(k_pull_wsync_multi<T, false, ADJ, 4, 4>, a, block, smem, num_sms, s);
      case 8 * 8 + 4: return run(k_pull_wsync_multi<T, false, ADJ, 8, 4>, a, block, smem, num_sms, s);
      default: return run(k_pull_wsync_multi<T, false, ADJ, 16, 4>, a, block, smem, num_sms, s);
    }
  }
  if (cfg.exact) {
    if (rhs <= 8) return run(k_pull_multi<T, 8, 1, true, ADJ>, a, block, smem, num_sms, s);
    return run(k_pull_multi<T, 32, 2, true, ADJ>, a, block, smem, num_sms, s);
  }
  if (rhs <= 4) return run(k_pull_multi<T, 4, 1, false, ADJ>, a, block, smem, num_sms, s);
  if (rhs <= 8) return run(k_pull_multi<T, 8, 1, false, ADJ>, a, block, smem, num_sms, s);
  if (rhs <= 16) return run(k_pull_multi<T, 16, 1, false, ADJ>, a, block, smem, num_sms, s);
  if (rhs <= 32) return run(k_pull_multi<T, 32, 1, false, ADJ>, a, block, smem, num_sms, s);
  return run(k_pull_multi<T, 32, 2, false, ADJ>, a, block, smem, num_sms, s);
}

template <typename T>
cudaError_t launch_pull_imported(const Layout& L, const Values<T>& V, const VecView<T>& v, T* xw, DeviceCtl* ctl,
                                 const ExecConfig& cfg, unsigned long long timeout_ns, int num_sms, cudaStream_t s,
                                 const ImportTable& im) {
  if (L.n == 0) return cudaSuccess;
  ExecArgs<T> a = make_args<T>(L, V, 1, v, im.width);
  a.xw = xw;
  a.ctl = ctl;
  a.timeout_ns = timeout_ns;
  a.ctas_per_sm = cfg.ctas_per_sm;
  a.im_start = im.start;
  a.im_ptr = im.ptr;
  a.im_q = im.q;
  a.dep_slot = im.dep_slot;
  a.nchunks = im.nchunks;
  const size_t smem = (size_t)(im.width + im.max_imports) * sizeof(T);
  const int block = cfg.block + 32;
  const bool one = cfg.one_batch != 0;
  switch (cfg.wsync_batch) {
    case 1:
      return one ? run(k_pull_wsync_imp<T, 1, true>, a, block, smem, num_sms, s)
                 : run(k_pull_wsync_imp<T, 1, false>, a, block, smem, num_sms, s);
    case 4:
      return one ? run(k_pull_wsync_imp<T, 4, true>, a, block, smem, num_sms, s)
                 : run(k_pull_wsync_imp<T, 4, false>, a, block, smem, num_sms, s);
    default:
      return one ? run(k_pull_wsync_imp<T, 2, true>, a, block, smem, num_sms, s)
                 : run(k_pull_wsync_imp<T, 2, false>, a, block, smem, num_sms, s);
  }
}

size_t imported_smem_bytes(int chunk, int max_imports, size_t elem) {
  return (size_t)(chunk + max_imports) * elem;
}

template <typename T>
cudaError_t launch_pull(const Layout& L, const Values<T>& V, int rhs, const VecView<T>& v, T* xw, DeviceCtl* ctl,
                        const ExecConfig& cfg, unsigned long long timeout_ns, int num_sms, cudaStream_t s,
                        const AdjointArgs<T>* adj, const PieceTable* pc) {
  if (L.n == 0) return cudaSuccess;
  ExecArgs<T> a = make_args<T>(L, V, rhs, v, cfg.chunk);
  const bool use_pc = pc && pc->walk && rhs == 1 && cfg.wsync && !cfg.exact && !(adj && adj->grad);
  if (use_pc) {
    a.pc_walk = pc->walk;
    a.pc_row = pc->row;
    a.pc_lo = pc->lo;
    a.pc_hi = pc->hi;
    a.pc_cseg = pc->cseg;
    a.pc_cbase = pc->cbase;
    a.pc_split = pc->seg_split;
    a.nchunks = pc->nchunks;
  }
  a.xw = xw;
  a.ctl = ctl;
  a.timeout_ns = timeout_ns;
  a.sleep_min = cfg.sleep_max ? 16u : 0u;
  a.sleep_max = cfg.sleep_max;
  a.ctas_per_sm = cfg.ctas_per_sm;
  size_t smem = 0;
  a.smem_tier = 0;
  if (cfg.smem_tier) {
    smem = pull_smem_bytes(cfg.chunk, rhs, sizeof(T));
    if (smem <= 200 * 1024) a.smem_tier = 1;
    else smem = 0;
  }
  if (adj) {
    a.grad = adj->grad;
    a.xf = adj->xf;
    a.xf_si = adj->xf_si;
    a.xf_sk = adj->xf_sk;
    if (!use_pc) {
      a.walk_pad = (a.chunk - a.n % a.chunk) % a.chunk;
      a.nchunks = (a.n + a.walk_pad + a.chunk - 1) / a.chunk;
    }
    return launch_pull_impl<T, true>(a, rhs, cfg, smem, num_sms, s);
  }
  return launch_pull_impl<T, false>(a, rhs, cfg, smem, num_sms, s);
}

template <typename T>
cudaError_t launch_push(const Layout& L, const Values<T>& V, int rhs, const VecView<T>& v, T* left_sum,
                        unsigned* counters, DeviceCtl* ctl, const ExecConfig& cfg, unsigned long long timeout_ns,
                        int num_sms, cudaStream_t s) {
  if (L.n == 0) return cudaSuccess;
  ExecArgs<T> a = make_args<T>(L, V, rhs, v, cfg.chunk);
  a.left_sum = left_sum;
  a.counters = counters;
  a.ctl = ctl;
  a.timeout_ns = timeout_ns;
  a.sleep_min = cfg.sleep_max ? 16u : 0u;
  a.sleep_max = cfg.sleep_max;
  a.ctas_per_sm = cfg.ctas_per_sm;
  const int block = cfg.block;
  if (rhs == 1) {
    size_t smem = 0;
    a.smem_tier = 0;
    if (cfg.smem_tier) {
      smem = (size_t)cfg.chunk * (sizeof(T) + sizeof(unsigned));
      if (smem <= 200 * 1024) a.smem_tier = 1;
      else smem = 0;
    }
    switch (cfg.lanes) {
      case 1: return run(k_push_vec<T, 1>, a, block, smem, num_sms, s);
      case 2: return run(k_push_vec<T, 2>, a, block, smem, num_sms, s);
      case 4: return run(k_push_vec<T, 4>, a, block, smem, num_sms, s);
      case 8: return run(k_push_vec<T, 8>, a, block, smem, num_sms, s);
      case 16: return run(k_push_vec<T, 16>, a, block, smem, num_sms, s);
      default: return run(k_push_vec<T, 32>, a, block, smem, num_sms, s);
    }
  }
  a.smem_tier = 0;
  a.opt = cfg.opt;
  if (rhs <= 4) return run(k_push_multi<T, 4, 1>, a, block, 0, num_sms, s);
  if (rhs <= 8) return run(k_push_multi<T, 8, 1>, a, block, 0, num_sms, s);
  if (rhs <= 16) return run(k_push_multi<T, 16, 1>, a, block, 0, num_sms, s);
  if (rhs <= 32) return run(k_push_multi<T, 32, 1>, a, block, 0, num_sms, s);
  return run(k_push_multi<T, 32, 2>, a, block, 0, num_sms, s);
}

template <typename T>
cudaError_t launch_levelset(const Layout& L, const Values<T>& V, int rhs, const VecView<T>& v, T* xw, DeviceCtl* ctl,
                            const ExecConfig& cfg, unsigned long long timeout_ns, cudaStream_t s) {
  if (L.n == 0) return cudaSuccess;
  ExecArgs<T> a = make_args<T>(L, V, rhs, v, cfg.chunk);
  a.xw = xw;
  a.ctl = ctl;
  a.timeout_ns = timeout_ns;
  a.level_ptr = L.level_ptr;
  a.nlevels = L.nlevels;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int block = 256;
  auto kernel = cfg.lanes >= 8 ? k_levelset<T, 8> : k_levelset<T, 1>;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
  if (per_sm < 1) per_sm = 1;
  const int grid = sms * std::min(per_sm, cfg.ctas_per_sm > 0 ? cfg.ctas_per_sm : 2);
  void* args[] = {(void*)&a};
  return cudaLaunchCooperativeKernel((void*)kernel, dim3(grid), dim3(block), args, 0, s);
}

// ------------------------------------------------------------------ gradient w.r.t. values
// dval[e] = -sum_k lambda[row(e), k] * x[col(e), k] on the stored pattern.
template <typename T>
__global__ void k_grad_values(const int* __restrict__ csc_row, const int* __restrict__ csc_col, int nnz, int rhs,
                              const T* __restrict__ lambda, const T* __restrict__ x, long long si, long long sk,
                              T* dval) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nnz; e += stride) {
    const long long r = csc_row[e], c = csc_col[e];
    T acc = T(0);
    for (int k = 0; k < rhs; ++k) acc = fma(lambda[r * si + k * sk], x[c * si + k * sk], acc);
    dval[e] = -acc;
  }
}

template <typename T>
cudaError_t launch_grad_values(const int* csc_row, const int* csc_col, int nnz, int rhs, const T* lambda, const T* x,
                               long long si, long long sk, T* dval, cudaStream_t s) {
  if (nnz <= 0) return cudaSuccess;
  long long grid = (nnz + 255) / 256;
  if (grid > (1 << 20)) grid = 1 << 20;
  k_grad_values<T><<<(int)grid, 256, 0, s>>>(csc_row, csc_col, nnz, rhs, lambda, x, si, sk, dval);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ reference kernel surface
// Natural column order, one warp per column, a ticket so warps start in
// dependency order (SpTRSV_cuda/sptrsv_syncfree_cuda.h:110-172, :290-407).
// in_degree counts down from the analysed in-degree; a column is ready when
// its count reaches 1. The caller zeroes left_sum and restores in_degree
// between solves, as with the reference. A row index outside [0, m) is never
// written through: the lane that meets it records DEV_BAD_INPUT and skips it,
// and every warp stops at its next ticket or wait. With `gate` set and *gate non-zero (structural
// flags raised earlier in the stream) nothing is solved and DEV_BAD_INPUT is
// recorded.
__device__ __forceinline__ void raise_bad_input(DeviceCtl* ctl, int where) {
  if (atomicCAS(&ctl->code, DEV_OK, DEV_BAD_INPUT) == DEV_OK) ctl->where = where;
}

template <typename T>
__global__ void __launch_bounds__(128) k_ref_exec(const int* __restrict__ col_ptr, const int* __restrict__ row_idx,
                                                  const T* __restrict__ val, int* in_degree, T* left_sum, int m,
                                                  int substitution, int rhs, int opt, const T* __restrict__ b, T* x,
                                                  DeviceCtl* ctl, unsigned long long timeout_ns,
                                                  const int* __restrict__ gate) {
  const int lane = threadIdx.x & 31;
  if (gate && *gate != 0 && blockIdx.x == 0 && threadIdx.x == 0) raise_bad_input(ctl, -1);
  if (gate && *gate != 0) m = 0;   // every warp skips the loop and joins the exit count
  for (;;) {
    int id = 0;
    if (lane == 0) id = ctl_failed(ctl) ? m : static_cast<int>(atomicAdd(&ctl->ticket, 1u));
    id = __shfl_sync(0xffffffffu, id, 0);
    if (id >= m) break;
    const int col = substitution == 0 ? id : m - 1 - id;
    const int beg = col_ptr[col], end = col_ptr[col + 1];
    const int dpos = substitution == 0 ? beg : end - 1;
    const T coef = T(1) / val[dpos];
    int ok = 1;
    if (lane == 0) {
      WaitBudget w(timeout_ns);
      while (ld_acquire_u32(reinterpret_cast<const unsigned*>(&in_degree[col])) != 1u) {
        if (!w.poll(ctl, col)) { ok = 0; break; }
      }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok) break;
    __syncwarp();
    const int s0 = substitution == 0 ? beg + 1 : beg;
    const int s1 = substitution == 0 ? end : end - 1;
    const int len = s1 - s0;
    // Lanes over right-hand sides (RHS mode) or over entries (NNZ mode); AUTO
    // follows the reference's rule (sptrsv_syncfree_cuda.h:262).
    const bool rhs_mode = rhs > 1 && (opt == 2 || (opt == 3 && (len <= rhs || rhs > 16) && len < 2048));
    for (int k = lane; k < rhs; k += 32) {
      const long long p = (long long)col * rhs + k;
      x[p] = (b[p] - Flag<T>::value(Flag<T>::load(&left_sum[p]))) * coef;
    }
    __syncwarp();
    // a row outside [0, m) would write past the counters and partial sums: it is
    // skipped and recorded (the other warps stop at their next ticket or wait)
    const unsigned mm = static_cast<unsigned>(m);
    if (rhs_mode) {
      for (int e = s0; e < s1; ++e) {
        const int r = row_idx[e];
        if (static_cast<unsigned>(r) >= mm) {
          if (lane == 0) raise_bad_input(ctl, col);
          continue;
        }
        const T v = val[e];
        for (int k = lane; k < rhs; k += 32) atomicAdd(&left_sum[(long long)r * rhs + k], x[(long long)col * rhs + k] * v);
      }
      __syncwarp();
      if (lane == 0) {
        __threadfence();
        for (int e = s0; e < s1; ++e) {
          const int r = row_idx[e];
          if (static_cast<unsigned>(r) < mm) atomicSub(&in_degree[r], 1);
        }
      }
    } else {
      for (int e = s0 + lane; e < s1; e += 32) {
        const int r = row_idx[e];
        if (static_cast<unsigned>(r) >= mm) {
          raise_bad_input(ctl, col);
          continue;
        }
        const T v = val[e];
        for (int k = 0; k < rhs; ++k) atomicAdd(&left_sum[(long long)r * rhs + k], x[(long long)col * rhs + k] * v);
      }
      __threadfence();
      for (int e = s0 + lane; e < s1; e += 32) {
        const int r = row_idx[e];
        if (static_cast<unsigned>(r) < mm) atomicSub(&in_degree[r], 1);
      }
    }
  }
  if (lane == 0) {
    __threadfence();
    const unsigned total_warps = gridDim.x * (blockDim.x / 32);
    const unsigned d = atomicAdd(&ctl->done, 1u);
    if (d == total_warps - 1) {
      ctl->ticket = 0;
      ctl->done = 0;
      __threadfence();
    }
  }
}

template <typename T>
cudaError_t launch_ref_executor(const int* col_ptr, const int* row_idx, const T* val, int* in_degree, T* left_sum,
                                int m, int substitution, int rhs, int opt, const T* b, T* x, DeviceCtl* ctl,
                                unsigned long long timeout_ns, cudaStream_t s, const int* gate) {
  if (m == 0) return cudaSuccess;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ref_exec<T>, 128, 0);
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)sms * per_sm;
  const long long need = ((long long)m + 3) / 4;
  if (grid > need) grid = need;
  k_ref_exec<T><<<(int)grid, 128, 0, s>>>(col_ptr, row_idx, val, in_degree, left_sum, m, substitution, rhs, opt, b,
                                          x, ctl, timeout_ns, gate);
  return cudaGetLastError();
}

#define SPTRSV_INSTANTIATE(T)                                                                                    \
  template cudaError_t launch_pull<T>(const Layout&, const Values<T>&, int, const VecView<T>&, T*, DeviceCtl*,   \
                                      const ExecConfig&, unsigned long long, int, cudaStream_t,                  \
                                      const AdjointArgs<T>*, const PieceTable*);                                 \
  template cudaError_t launch_pull_imported<T>(const Layout&, const Values<T>&, const VecView<T>&, T*,           \
                                               DeviceCtl*, const ExecConfig&, unsigned long long, int,           \
                                               cudaStream_t, const ImportTable&);                                \
  template cudaError_t launch_push<T>(const Layout&, const Values<T>&, int, const VecView<T>&, T*, unsigned*,    \
                                      DeviceCtl*, const ExecConfig&, unsigned long long, int, cudaStream_t);     \
  template cudaError_t launch_levelset<T>(const Layout&, const Values<T>&, int, const VecView<T>&, T*,           \
                                          DeviceCtl*, const ExecConfig&, unsigned long long, cudaStream_t);      \
  template cudaError_t launch_grad_values<T>(const int*, const int*, int, int, const T*, const T*, long long,     \
                                             long long, T*, cudaStream_t);                                       \
  template cudaError_t launch_ref_executor<T>(const int*, const int*, const T*, int*, T*, int, int, int, int,    \
                                              const T*, T*, DeviceCtl*, unsigned long long, cudaStream_t,        \
                                              const int*);
SPTRSV_INSTANTIATE(double)
SPTRSV_INSTANTIATE(float)

}  // namespace sptrsv
