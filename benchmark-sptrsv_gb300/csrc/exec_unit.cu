// Pull executor over the units of a blocked order, with a bulk-copy loader
// (one right-hand side, fast arithmetic, forward walk).
//
// A unit is a run of consecutive positions of a blocked order: one natural
// block of the matrix, level order inside the block. Narrow DAGs (meshes and
// banded factors) put almost every dependency of a unit inside it, and the
// chain through a unit is then as long as the unit's level count. One CTA
// takes a whole unit with three warps:
//  * the consumer warp solves the unit's unknowns 32 at a time in position
//    order, its lanes in warp-synchronous lockstep. Every operand it reads
//    sits in shared memory: the stage buffers, values of the unit's recent
//    positions in a ring of `ring` slots, and imported values after the ring.
//    A dependency in an earlier segment is final when a segment starts; one in
//    the same segment costs one lockstep iteration;
//  * the importer warp polls the unit's external dependencies (and in-unit
//    dependencies too far back for the ring) in global memory and copies each
//    value into its shared-memory slot once it is published;
//  * the loader (one lane) streams the unit's stages -- runs of at most pmax
//    positions holding at most emax list entries -- into a ring of stage
//    buffers with bulk copies: list pointers, rows, first terms b/d (folded
//    for every position by k_first_term before the launch), dependency slots
//    and scaled values.
//
// Ring slots. Position p of the unit owns slot (p - base) mod ring. A list
// entry reads the ring only if the dependency is fewer than ring - 32
// positions back (the table builder routes the others through the importer),
// so when a segment starts, every reader of the slot's previous owner has
// finished and the consumer can reset the slot to "empty" for its new owner.
//
// Barriers: full[s] completes when stage buffer s has landed (bulk-copy
// transaction count), empty[s] when the consumer is done with it. Every wait
// is bounded.
#include "exec_common.cuh"
#include "internal.h"
#include "tma.cuh"

namespace sptrsv {

namespace {

template <typename T>
struct UnitArgs {
  int nchunks, ring, pmax, emax, smax, stages;
  const int* ustart;    // [nchunks+1] first position of each unit
  const int* ustage;    // [nchunks+1] first stage of each unit
  const int4* stab;     // per stage {lo, hi, e0, e1}, {g0, g1, -, -}: positions [lo, hi),
                        // list entries [e0, e1), segments [g0, g1)
  const int* segs;      // first position of each segment
  const int* im_ptr;    // [nchunks+1] imports of each unit
  const int* im_q;      // imported positions, ascending within a unit
  const int* perm;
  const int* dep_ptr;
  const int* dep_slot;  // shared-memory slot read by each list entry
  const T* dep_w;
  const T* c0;          // [n] first term b[perm[p]] / d_p of every position
  T* x;
  long long x_si;
  T* xw;
  DeviceCtl* ctl;
  unsigned long long timeout_ns;
};

constexpr unsigned kFull = 0xffffffffu;

// One stage buffer: the layout slices (StageBufs) and the stage's segment starts.
template <typename T>
__host__ __device__ inline size_t unit_stage_bytes(int pmax, int emax, int smax) {
  return stage_bytes<T>(pmax, emax) + ((sizeof(int) * (size_t)(smax + 1 + 8) + 15) & ~(size_t)15);
}

// Shared-memory accesses by 32-bit shared-window address (ld/st.shared), the
// ring words volatile.
__device__ __forceinline__ int lds_s32(unsigned a) {
  int v;
  asm volatile("ld.shared.s32 %0, [%1];" : "=r"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ double lds_val(unsigned a, double) {
  double v;
  asm volatile("ld.shared.f64 %0, [%1];" : "=d"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ float lds_val(unsigned a, float) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ unsigned long long ldsv_bits(unsigned a, unsigned long long) {
  unsigned long long v;
  asm volatile("ld.volatile.shared.u64 %0, [%1];" : "=l"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ldsv_bits(unsigned a, unsigned) {
  unsigned v;
  asm volatile("ld.volatile.shared.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ void stsv_bits(unsigned a, unsigned long long v) {
  asm volatile("st.volatile.shared.u64 [%0], %1;" ::"r"(a), "l"(v) : "memory");
}
__device__ __forceinline__ void stsv_bits(unsigned a, unsigned v) {
  asm volatile("st.volatile.shared.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}

// c0[p] = b[perm[p]] * rcp[p], every position (the first term of each unknown).
template <typename T>
__global__ void k_first_term(const int* __restrict__ perm, const T* __restrict__ b, long long b_si,
                             const T* __restrict__ rcp, T* __restrict__ c0, int n) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    c0[p] = b[(long long)perm[p] * b_si] * rcp[p];
}

template <typename T, int U>
__global__ void __launch_bounds__(96) k_pull_unit(UnitArgs<T> a) {
  using F = Flag<T>;
  using Bits = typename F::Bits;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ unsigned long long s_full[kMaxStages], s_empty[kMaxStages];
  __shared__ int4 s_tab[kMaxStages], s_tab2[kMaxStages];
  __shared__ int s_off[kMaxStages][6];
  __shared__ unsigned s_chunk;
  const int S = a.stages;
  const size_t sbytes = unit_stage_bytes<T>(a.pmax, a.emax, a.smax);
  const size_t lbytes = stage_bytes<T>(a.pmax, a.emax);  // segment starts follow the layout slices
  T* s_x = reinterpret_cast<T*>(smem_raw + (size_t)S * sbytes);
  const unsigned ring_a = smem_u32(s_x);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int rmask = a.ring - 1;
  if (threadIdx.x == 0) {
    for (int i = 0; i < S; ++i) {
      mbar_init(&s_full[i], 1);
      mbar_init(&s_empty[i], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  unsigned rbase = 0;  // stages this CTA streamed before the current unit (barrier phases)
  for (;;) {
    const unsigned c = next_chunk(a.ctl, a.nchunks, &s_chunk);
    if (c >= (unsigned)a.nchunks) break;
    const int base = a.ustart[c], end = a.ustart[c + 1];
    const int len = end - base;
    const int st0 = a.ustage[c], nst = a.ustage[c + 1] - st0;
    const int i0 = a.im_ptr[c], nimp = a.im_ptr[c + 1] - i0;
    const bool wrap = len > a.ring;
    const int nring = wrap ? a.ring : len;
    for (int i = threadIdx.x; i < nring; i += blockDim.x) *reinterpret_cast<Bits*>(&s_x[i]) = F::EMPTY;
    for (int i = threadIdx.x; i < nimp; i += blockDim.x) *reinterpret_cast<Bits*>(&s_x[a.ring + i]) = F::EMPTY;
    __syncthreads();
    auto buf_of = [&](int k) { return static_cast<int>((rbase + static_cast<unsigned>(k)) % static_cast<unsigned>(S)); };
    auto use_of = [&](int k) { return (rbase + static_cast<unsigned>(k)) / static_cast<unsigned>(S); };
    bool fail = false;
    if (warp == 2) {
      // ---------------- loader (lane 0): stage k goes into its buffer once the
      // consumer has released the buffer's previous stage
      if (lane == 0) {
        int issued = 0;
        for (; issued < nst; ++issued) {
          const int k = issued;
          const int bi = buf_of(k);
          const unsigned u = use_of(k);
          if (u > 0 && !mbar_wait(&s_empty[bi], (u - 1u) & 1u, a.ctl, a.timeout_ns, base)) {
            fail = true;
            break;
          }
          const int4 t = a.stab[2 * (st0 + k)];
          const int4 t2 = a.stab[2 * (st0 + k) + 1];
          StageBufs<T> sb = carve<T>(smem_raw + (size_t)bi * sbytes, a.pmax, a.emax);
          int* sg = reinterpret_cast<int*>(smem_raw + (size_t)bi * sbytes + lbytes);
          auto wide = [](long long x0, long long x1, long long per16) {
            return ((x1 + per16 - 1) & ~(per16 - 1)) - (x0 & ~(per16 - 1));
          };
          constexpr long long tper = 16 / sizeof(T);
          const unsigned expect = static_cast<unsigned>(
              wide(t.x, t.y + 1, 4) * 4 + wide(t.x, t.y, 4) * 4 + wide(t.x, t.y, tper) * (long long)sizeof(T) +
              wide(t.z, t.w, 4) * 4 + wide(t.z, t.w, tper) * (long long)sizeof(T) + wide(t2.x, t2.y + 1, 4) * 4);
          s_tab[bi] = t;
          s_tab2[bi] = t2;
          fence_proxy_async_smem();
          mbar_arrive_expect_tx(&s_full[bi], expect);
          unsigned tx = 0;
          s_off[bi][0] = stage_slice<int>(sb.ptr, a.dep_ptr, t.x, t.y + 1, &s_full[bi], &tx);
          s_off[bi][1] = stage_slice<int>(sb.perm, a.perm, t.x, t.y, &s_full[bi], &tx);
          s_off[bi][2] = stage_slice<T>(sb.sc, a.c0, t.x, t.y, &s_full[bi], &tx);
          s_off[bi][3] = stage_slice<int>(sb.pos, a.dep_slot, t.z, t.w, &s_full[bi], &tx);
          s_off[bi][4] = stage_slice<T>(sb.val, a.dep_w, t.z, t.w, &s_full[bi], &tx);
          s_off[bi][5] = stage_slice<int>(sg, a.segs, t2.x, t2.y + 1, &s_full[bi], &tx);
        }
        // copies land before the unit ends (in a normal run the consumer has
        // already waited for them; after a failure they may still be in flight)
        for (int k = issued - S > 0 ? issued - S : 0; k < issued; ++k)
          mbar_wait(&s_full[buf_of(k)], use_of(k) & 1u, a.ctl, a.timeout_ns, base);
      }
    } else if (warp == 1) {
      // ---------------- importer: each lane walks its imports in order
      WaitBudget wb(a.timeout_ns);
      unsigned idle = 0u;
      int i = lane;
      Bits v = F::EMPTY;
      if (i < nimp) v = F::load(&a.xw[a.im_q[i0 + i]]);
      for (;;) {
        bool progress = false;
        if (i < nimp) {
          if (v != F::EMPTY) {
            F::store_shared(&s_x[a.ring + i], F::value(v));
            i += 32;
            v = i < nimp ? F::load(&a.xw[a.im_q[i0 + i]]) : F::EMPTY;
            progress = true;
          } else {
            v = F::load(&a.xw[a.im_q[i0 + i]]);
          }
        }
        if (__all_sync(kFull, i >= nimp)) break;
        if (!__any_sync(kFull, progress) && ((++idle & 15u) == 0u)) {
          if (__any_sync(kFull, !wb.poll(a.ctl, base))) {
            fail = true;
            break;
          }
        }
      }
    } else {
      // ---------------- consumer
      for (int k = 0; k < nst && !fail; ++k) {
        const int bi = buf_of(k);
        if (!__all_sync(kFull, mbar_wait(&s_full[bi], use_of(k) & 1u, a.ctl, a.timeout_ns, base))) {
          fail = true;
          break;
        }
        const int4 t = s_tab[bi];
        const StageBufs<T> sb = carve<T>(smem_raw + (size_t)bi * sbytes, a.pmax, a.emax);
        const unsigned a_ptr = smem_u32(sb.ptr + s_off[bi][0]);
        const unsigned a_perm = smem_u32(sb.perm + s_off[bi][1]);
        const unsigned a_c0 = smem_u32(sb.sc + s_off[bi][2]);
        const unsigned a_slot = smem_u32(sb.pos + s_off[bi][3]);
        const unsigned a_w = smem_u32(sb.val + s_off[bi][4]);
        const unsigned a_seg =
            smem_u32(reinterpret_cast<int*>(smem_raw + (size_t)bi * sbytes + lbytes) + s_off[bi][5]);
        const int nsg = s_tab2[bi].y - s_tab2[bi].x;
        const int lo = t.x, e0 = t.z;
        for (int g = 0; g < nsg && !fail; ++g) {
          const int s0 = lds_s32(a_seg + 4u * g), s1 = lds_s32(a_seg + 4u * g + 4u);
          const int p = s0 + lane;
          bool done = p >= s1;
          const unsigned i = static_cast<unsigned>(p - lo);
          const unsigned my = ring_a + static_cast<unsigned>((p - base) & rmask) * (unsigned)sizeof(T);
          if (wrap) {
            if (!done) stsv_bits(my, F::EMPTY);
            __syncwarp();
          }
          int row = 0, e = 0, e1 = 0;
          T acc = T(0);
          if (!done) {
            row = lds_s32(a_perm + 4u * i);
            acc = lds_val(a_c0 + (unsigned)sizeof(T) * i, T(0));
            e = lds_s32(a_ptr + 4u * i) - e0;
            e1 = lds_s32(a_ptr + 4u * i + 4u) - e0;
          }
          unsigned ls[U];
          T w[U];
          Bits bits[U];
          unsigned todo = 0u;
          auto load_batch = [&]() {
            todo = 0u;
#pragma unroll
            for (int u = 0; u < U; ++u) {
              const int ee = e + u;
              if (ee < e1) {
                ls[u] = ring_a + static_cast<unsigned>(lds_s32(a_slot + 4u * ee)) * (unsigned)sizeof(T);
                w[u] = lds_val(a_w + (unsigned)sizeof(T) * ee, T(0));
                todo |= 1u << u;
              }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) bits[u] = (todo & (1u << u)) ? ldsv_bits(ls[u], Bits(0)) : F::EMPTY;
          };
          if (!done) load_batch();
          WaitBudget wb(a.timeout_ns);
          unsigned idle = 0u;
          for (;;) {
            bool progress = false;
            if (!done) {
#pragma unroll
              for (int u = 0; u < U; ++u) {
                if ((todo & (1u << u)) && bits[u] != F::EMPTY) {
                  acc = fma(-w[u], F::value(bits[u]), acc);
                  todo &= ~(1u << u);
                  progress = true;
                }
              }
              if (!todo) {
                e += U;
                if (e < e1) {
                  load_batch();
                } else {
                  const Bits ob = F::bits(acc);
                  stsv_bits(my, ob);
                  F::store(&a.xw[p], acc);
                  a.x[(long long)row * a.x_si] = acc;
                  done = true;
                }
                progress = true;
              } else {
#pragma unroll
                for (int u = 0; u < U; ++u)
                  if ((todo & (1u << u)) && bits[u] == F::EMPTY) bits[u] = ldsv_bits(ls[u], Bits(0));
              }
            }
            if (__all_sync(kFull, done)) break;
            if (!__any_sync(kFull, progress) && ((++idle & 255u) == 0u)) {
              if (__any_sync(kFull, !wb.poll(a.ctl, p))) {
                fail = true;
                break;
              }
            }
          }
        }
        __syncwarp();
        if (!fail && lane == 0) mbar_arrive(&s_empty[bi]);
      }
    }
    rbase += static_cast<unsigned>(nst);
    if (__syncthreads_or(fail)) break;
  }
  leave(a.ctl);
}

template <typename T, int U>
cudaError_t run_unit(const UnitArgs<T>& a, size_t smem, int num_sms, cudaStream_t s) {
  auto kernel = k_pull_unit<T, U>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 96, smem);
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)num_sms * per_sm;
  if (grid > a.nchunks) grid = a.nchunks;
  if (grid < 1) grid = 1;
  kernel<<<static_cast<int>(grid), 96, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

size_t unit_smem_bytes(int ring, int max_imports, int pmax, int emax, int smax, int stages, size_t elem) {
  const size_t sb = elem == sizeof(double) ? unit_stage_bytes<double>(pmax, emax, smax)
                                           : unit_stage_bytes<float>(pmax, emax, smax);
  return (size_t)stages * sb + (size_t)(ring + max_imports) * elem;
}

template <typename T>
cudaError_t launch_pull_unit(const Layout& L, const Values<T>& V, const VecView<T>& v, T* xw, T* c0, DeviceCtl* ctl,
                             const ExecConfig& cfg, unsigned long long timeout_ns, int num_sms, cudaStream_t s,
                             const ImportTable& im) {
  if (L.n == 0) return cudaSuccess;
  {
    const int threads = 256;
    long long blocks = ((long long)L.n + threads - 1) / threads;
    if (blocks > 8LL * num_sms) blocks = 8LL * num_sms;
    k_first_term<T><<<static_cast<int>(blocks), threads, 0, s>>>(L.perm, v.b, v.b_si, V.rcp, c0, L.n);
  }
  UnitArgs<T> a{};
  a.nchunks = im.nchunks;
  a.ring = im.ring;
  a.pmax = im.pmax;
  a.emax = im.emax;
  a.smax = im.smax;
  a.stages = im.stages;
  a.ustart = im.start;
  a.ustage = im.ustage;
  a.stab = im.stab;
  a.segs = im.segs;
  a.im_ptr = im.ptr;
  a.im_q = im.q;
  a.perm = L.perm;
  a.dep_ptr = L.dep_ptr;
  a.dep_slot = im.dep_slot;
  a.dep_w = V.dep_w;
  a.c0 = c0;
  a.x = v.x;
  a.x_si = v.x_si;
  a.xw = xw;
  a.ctl = ctl;
  a.timeout_ns = timeout_ns;
  const size_t smem = unit_smem_bytes(im.ring, im.max_imports, im.pmax, im.emax, im.smax, im.stages, sizeof(T));
  switch (cfg.wsync_batch) {
    case 1: return run_unit<T, 1>(a, smem, num_sms, s);
    case 4: return run_unit<T, 4>(a, smem, num_sms, s);
    default: return run_unit<T, 2>(a, smem, num_sms, s);
  }
}

template cudaError_t launch_pull_unit<double>(const Layout&, const Values<double>&, const VecView<double>&, double*,
                                              double*, DeviceCtl*, const ExecConfig&, unsigned long long, int,
                                              cudaStream_t, const ImportTable&);
template cudaError_t launch_pull_unit<float>(const Layout&, const Values<float>&, const VecView<float>&, float*,
                                             float*, DeviceCtl*, const ExecConfig&, unsigned long long, int,
                                             cudaStream_t, const ImportTable&);

}  // namespace sptrsv
