// Pull executor with TMA-staged chunks (one right-hand side).
//
// Work unit: a chunk of consecutive positions from a precomputed chunk table
// (bounded position count C and dependency count E, one processing mode per
// chunk). A persistent CTA double-buffers its chunks: while it solves chunk k
// from shared memory, the bulk-copy engine (cp.async.bulk, 1-D TMA, completion
// on an mbarrier) streams chunk k+1's slices of the position-space layout --
// dependency pointers, rows, 1/diag, dependency positions and scaled values --
// into the other buffer. The only global traffic left on the dependency path
// is the gather of published x values (value-as-flag words, relaxed loads)
// and b.
//
// Modes: 0 = one thread per unknown (short dependency lists), 1 = one warp per
// unknown with lanes over its dependencies (long lists), 2 = one warp per
// unknown reading its list straight from global memory (lists longer than a
// stage buffer).
//
// ADJ solves the transposed system on the same analysis: the chunk table is
// built over reversed positions and the dependency lists are the push lists.
#include "exec_common.cuh"
#include "internal.h"
#include "tma.cuh"

namespace sptrsv {

namespace {
template <typename T>
struct StagedArgs {
  int n, nchunks, cmax, emax, smem_tier, stages;
  const int* tab_start;   // [nchunks+1] first original position of each chunk (in walk order)
  const int* tab_mode;    // [nchunks]
  const int* perm;
  const int* lptr;        // dependency pointers (pull lists, or push lists for ADJ)
  const int* lpos;
  const T* lval;          // scaled values (or unscaled with EXACT)
  const T* dscale;        // 1/diag (or diag with EXACT)
  const T* b;
  T* x;
  long long b_si, x_si;
  T* xw;
  DeviceCtl* ctl;
  unsigned long long timeout_ns;
  unsigned sleep_min, sleep_max;
  // fused gradient (ADJ only)
  T* grad;
  const T* xf;
  long long xf_si;
  const int* dep_ptr;
  const int* dep_src;
  const int* dep_col;
  const int* diag_src;
};

struct StageInfo {
  int chunk;    // chunk id (>= nchunks: none)
  int lo, hi;   // original positions [lo, hi)
  int ebase;    // lptr[lo]
  int off_ptr, off_perm, off_sc, off_pos, off_val;  // element offsets inside the staged slices
  int mode;
};

// Producer lane: claim a chunk and start streaming its slices into stage
// buffer `sb`; the copies complete on `bar` (armed with their byte count).
// A chunk id >= nchunks marks the end of the work.
template <typename T, bool ADJ>
__device__ void issue_stage(const StagedArgs<T>& a, StageBufs<T> sb, unsigned long long* bar, StageInfo* info) {
  const unsigned c = ctl_failed(a.ctl) ? (unsigned)a.nchunks : atomicAdd(&a.ctl->ticket, 1u);
  info->chunk = static_cast<int>(c);
  if (c >= (unsigned)a.nchunks) {
    mbar_arrive_expect_tx(bar, 0);
    return;
  }
  const int s0 = a.tab_start[c], s1 = a.tab_start[c + 1];
  // walk order s0..s1-1; in ADJ the walk runs over reversed positions
  const int lo = ADJ ? a.n - s1 : s0;
  const int hi = ADJ ? a.n - s0 : s1;
  const int mode = a.tab_mode[c];
  const int e0 = a.lptr[lo], e1 = a.lptr[hi];
  info->lo = lo;
  info->hi = hi;
  info->ebase = e0;
  info->mode = mode;
  auto wide = [](long long a_, long long b_, long long per16) {
    return ((b_ + per16 - 1) & ~(per16 - 1)) - (a_ & ~(per16 - 1));
  };
  unsigned expect = 0;
  expect += (unsigned)(wide(lo, hi + 1, 4) * 4);
  expect += (unsigned)(wide(lo, hi, 4) * 4);
  expect += (unsigned)(wide(lo, hi, 16 / sizeof(T)) * sizeof(T));
  if (mode != 2) {
    expect += (unsigned)(wide(e0, e1, 4) * 4);
    expect += (unsigned)(wide(e0, e1, 16 / sizeof(T)) * sizeof(T));
  }
  fence_proxy_async_smem();
  mbar_arrive_expect_tx(bar, expect);
  unsigned tx = 0;
  info->off_ptr = stage_slice<int>(sb.ptr, a.lptr, lo, hi + 1, bar, &tx);
  info->off_perm = stage_slice<int>(sb.perm, a.perm, lo, hi, bar, &tx);
  info->off_sc = stage_slice<T>(sb.sc, a.dscale, lo, hi, bar, &tx);
  if (mode != 2) {
    info->off_pos = stage_slice<int>(sb.pos, a.lpos, e0, e1, bar, &tx);
    info->off_val = stage_slice<T>(sb.val, a.lval, e0, e1, bar, &tx);
  } else {
    info->off_pos = info->off_val = 0;
  }
}


// Warp-specialised pipeline. Warp 0 is the producer: it claims chunks and
// streams them into a ring of `a.stages` buffers (full[s] completes when a
// chunk's bytes have landed; empty[s] when every consumer warp is done with
// it). Warps 1.. are consumers: they take the ring in order, solve the chunk's
// unknowns from shared memory, and release the buffer. There is no CTA-wide
// barrier between chunks.
template <typename T, bool EXACT, bool ADJ>
__global__ void __launch_bounds__(256) k_pull_staged(StagedArgs<T> a) {
  using F = Flag<T>;
  using Bits = typename F::Bits;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ unsigned long long s_full[kMaxStages], s_empty[kMaxStages];
  __shared__ StageInfo s_info[kMaxStages];
  const int S = a.stages;
  const size_t sbytes = stage_bytes<T>(a.cmax, a.emax);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nconsumer_warps = (blockDim.x >> 5) - 1;
  const int nconsumers = nconsumer_warps * 32;
  T* s_xbase = reinterpret_cast<T*>(smem_raw + (size_t)S * sbytes);
  if (threadIdx.x == 0) {
    for (int i = 0; i < S; ++i) {
      mbar_init(&s_full[i], 1);
      mbar_init(&s_empty[i], nconsumer_warps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  if (warp == 0) {
    // ---------------- producer
    bool in_flight[kMaxStages] = {false, false, false, false};
    unsigned issued_parity[kMaxStages] = {0u, 0u, 0u, 0u};
    for (int r = 0;; ++r) {
      const int st = r % S;
      const unsigned round = static_cast<unsigned>(r / S);
      // wait until every consumer warp released this buffer (first round: free)
      bool ok = true;
      if (lane == 0) ok = mbar_wait(&s_empty[st], (round & 1u) ^ 1u, a.ctl, a.timeout_ns, -1);
      ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      if (!ok) break;
      in_flight[st] = false;
      if (a.smem_tier) {
        T* sx = s_xbase + (size_t)st * a.cmax;
        for (int i = lane; i < a.cmax; i += 32) *reinterpret_cast<Bits*>(&sx[i]) = F::EMPTY;
      }
      __syncwarp();
      int chunk = 0;
      if (lane == 0) {
        StageBufs<T> sb = carve<T>(smem_raw + (size_t)st * sbytes, a.cmax, a.emax);
        issue_stage<T, ADJ>(a, sb, &s_full[st], &s_info[st]);
        chunk = s_info[st].chunk;
      }
      chunk = __shfl_sync(0xffffffffu, chunk, 0);
      if (chunk >= a.nchunks) break;
      in_flight[st] = true;
      issued_parity[st] = round & 1u;
    }
    if (lane == 0) {
      // copies issued but possibly never consumed (a consumer failed) must land
      // before the CTA leaves; in a normal run these phases are already complete
      for (int i = 0; i < S; ++i) {
        if (!in_flight[i]) continue;
        WaitBudget w(a.timeout_ns);
        while (!mbar_test(&s_full[i], issued_parity[i])) {
          if (!w.poll(a.ctl, -1)) break;
        }
      }
    }
  } else {
    // ---------------- consumers
    const int ct = threadIdx.x - 32;     // consumer thread index
    const int cw = warp - 1;             // consumer warp index
    bool fail = false;
    for (int r = 0;; ++r) {
      const int st = r % S;
      const unsigned round = static_cast<unsigned>(r / S);
      if (!mbar_wait(&s_full[st], round & 1u, a.ctl, a.timeout_ns, -1)) fail = true;
      fail = __any_sync(0xffffffffu, fail);
      if (fail) break;
      const StageInfo info = s_info[st];
      if (info.chunk >= a.nchunks) break;
      const StageBufs<T> sb = carve<T>(smem_raw + (size_t)st * sbytes, a.cmax, a.emax);
      T* s_x = s_xbase + (size_t)st * a.cmax;
      const int* sptr = sb.ptr + info.off_ptr;
      const int* sperm = sb.perm + info.off_perm;
      const T* ssc = sb.sc + info.off_sc;
      const int* spos = sb.pos + info.off_pos;
      const T* sval = sb.val + info.off_val;
      const int lo = info.lo, hi = info.hi;
      const int len = hi - lo;
      auto pos_of = [&](int i) { return ADJ ? hi - 1 - i : lo + i; };
      auto is_local = [&](int q) { return ADJ ? (q < hi) : (q >= lo); };
      const bool tier = a.smem_tier != 0;
      auto slot = [&](int q) { return (tier && (ADJ ? q < hi : q >= lo)) ? q - lo : -1; };
      if (EXACT || info.mode == 0) {
        const bool from_smem = info.mode != 2;
        const int* vpos = from_smem ? spos : a.lpos;
        const T* vval = from_smem ? sval : a.lval;
        for (int i = ct; i < len && !fail; i += nconsumers) {
          const int p = pos_of(i);
          const int li = p - lo;
          const int row = sperm[li];
          const int ea = from_smem ? sptr[li] - info.ebase : sptr[li];
          const int eb = from_smem ? sptr[li + 1] - info.ebase : sptr[li + 1];
          const T bi = a.b[(long long)row * a.b_si];
          const T sc = ssc[li];
          T acc = EXACT ? T(0) : bi * sc;
          if (!gather_deps<T, EXACT, 8, 1>(vpos, vval, ea, eb, a.xw, s_x, slot, a.ctl, a.timeout_ns, p, a.sleep_min,
                                           a.sleep_max, acc)) {
            fail = true;
            break;
          }
          const T xi = EXACT ? exact_finish<T>(bi, acc, sc) : acc;
          if (a.smem_tier) F::store_shared(&s_x[li], xi);
          F::store(&a.xw[p], xi);
          a.x[(long long)row * a.x_si] = xi;
          if (ADJ && a.grad) {
            for (int e = a.dep_ptr[p]; e < a.dep_ptr[p + 1]; ++e)
              a.grad[a.dep_src[e]] = -xi * a.xf[(long long)a.dep_col[e] * a.xf_si];
            a.grad[a.diag_src[p]] = -xi * a.xf[(long long)row * a.xf_si];
          }
        }
      } else {
        // one warp per unknown; lanes over its dependency list
        const bool from_smem = info.mode == 1;
        for (int i = cw; i < len && !fail; i += nconsumer_warps) {
          const int p = pos_of(i);
          const int li = p - lo;
          const int row = sperm[li];
          const int ea = from_smem ? sptr[li] - info.ebase : sptr[li];
          const int eb = from_smem ? sptr[li + 1] - info.ebase : sptr[li + 1];
          const int* vpos = from_smem ? spos : a.lpos;
          const T* vval = from_smem ? sval : a.lval;
          const T bi = a.b[(long long)row * a.b_si];
          const T sc = ssc[li];
          T acc = lane == 0 ? bi * sc : T(0);
          if (!gather_deps<T, false, 2, 32>(vpos, vval, ea + lane, eb, a.xw, s_x, slot, a.ctl, a.timeout_ns, p,
                                            a.sleep_min, a.sleep_max, acc))
            fail = true;
          fail = __any_sync(0xffffffffu, fail);
          if (fail) break;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
          const T xi = acc;
          if (lane == 0) {
            if (a.smem_tier) F::store_shared(&s_x[li], xi);
            F::store(&a.xw[p], xi);
            a.x[(long long)row * a.x_si] = xi;
          }
          if (ADJ && a.grad) {
            for (int e = a.dep_ptr[p] + lane; e < a.dep_ptr[p + 1]; e += 32)
              a.grad[a.dep_src[e]] = -xi * a.xf[(long long)a.dep_col[e] * a.xf_si];
            if (lane == 0) a.grad[a.diag_src[p]] = -xi * a.xf[(long long)row * a.xf_si];
          }
        }
      }
      fail = __any_sync(0xffffffffu, fail);
      if (fail) break;
      // release the buffer (one arrival per consumer warp)
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&s_empty[st])) : "memory");
    }
    if (fail && lane == 0) {
      // make the producer stop: record a failure if none is recorded yet
      atomicCAS(&a.ctl->code, DEV_OK, DEV_TIMEOUT);
    }
  }
  __syncthreads();
  leave(a.ctl);
}

template <typename T, bool EXACT, bool ADJ>
cudaError_t run_staged(const StagedArgs<T>& a, int block, int ctas_per_sm, int num_sms, cudaStream_t s) {
  const size_t smem = (size_t)a.stages * (stage_bytes<T>(a.cmax, a.emax) + (a.smem_tier ? sizeof(T) * (size_t)a.cmax : 0));
  auto kernel = k_pull_staged<T, EXACT, ADJ>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  if (ctas_per_sm > 0 && per_sm > ctas_per_sm) per_sm = ctas_per_sm;
  long long grid = (long long)num_sms * per_sm;
  if (grid > a.nchunks) grid = a.nchunks;
  if (grid < 1) grid = 1;
  kernel<<<(int)grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

size_t staged_smem_bytes(int cmax, int emax, size_t elem, bool smem_tier, int stages) {
  return (size_t)stages * ((elem == 8 ? stage_bytes<double>(cmax, emax) : stage_bytes<float>(cmax, emax)) +
                           (smem_tier ? elem * (size_t)cmax : 0));
}

template <typename T>
cudaError_t launch_pull_staged(const Layout& L, const Values<T>& V, const ChunkTable& tab, const VecView<T>& v, T* xw,
                               DeviceCtl* ctl, const ExecConfig& cfg, unsigned long long timeout_ns, int num_sms,
                               cudaStream_t s, const AdjointArgs<T>* adj) {
  if (L.n == 0) return cudaSuccess;
  StagedArgs<T> a{};
  a.n = L.n;
  a.nchunks = tab.nchunks;
  a.cmax = tab.cmax;
  a.emax = tab.emax;
  a.smem_tier = cfg.smem_tier;
  a.stages = cfg.stages < 2 ? 2 : (cfg.stages > kMaxStages ? kMaxStages : cfg.stages);
  a.tab_start = tab.start;
  a.tab_mode = tab.mode;
  a.perm = L.perm;
  const bool is_adj = adj != nullptr;
  a.lptr = is_adj ? L.out_ptr : L.dep_ptr;
  a.lpos = is_adj ? (cfg.exact ? L.out_pos : L.out_pos_f) : (cfg.exact ? L.dep_pos : L.dep_pos_f);
  a.lval = is_adj ? (cfg.exact ? V.out_val : V.out_w) : (cfg.exact ? V.dep_val : V.dep_w);
  a.dscale = cfg.exact ? V.diag : V.rcp;
  a.b = v.b;
  a.x = v.x;
  a.b_si = v.b_si;
  a.x_si = v.x_si;
  a.xw = xw;
  a.ctl = ctl;
  a.timeout_ns = timeout_ns;
  a.sleep_min = cfg.sleep_max ? 16u : 0u;
  a.sleep_max = cfg.sleep_max;
  if (is_adj) {
    a.grad = adj->grad;
    a.xf = adj->xf;
    a.xf_si = adj->xf_si;
    a.dep_ptr = L.dep_ptr;
    a.dep_src = L.dep_src;
    a.dep_col = L.dep_col;
    a.diag_src = L.diag_src;
  }
  const int block = cfg.block;
  if (cfg.exact) {
    return is_adj ? run_staged<T, true, true>(a, block, cfg.ctas_per_sm, num_sms, s)
                  : run_staged<T, true, false>(a, block, cfg.ctas_per_sm, num_sms, s);
  }
  return is_adj ? run_staged<T, false, true>(a, block, cfg.ctas_per_sm, num_sms, s)
                : run_staged<T, false, false>(a, block, cfg.ctas_per_sm, num_sms, s);
}

template cudaError_t launch_pull_staged<double>(const Layout&, const Values<double>&, const ChunkTable&,
                                                const VecView<double>&, double*, DeviceCtl*, const ExecConfig&,
                                                unsigned long long, int, cudaStream_t, const AdjointArgs<double>*);
template cudaError_t launch_pull_staged<float>(const Layout&, const Values<float>&, const ChunkTable&,
                                               const VecView<float>&, float*, DeviceCtl*, const ExecConfig&,
                                               unsigned long long, int, cudaStream_t, const AdjointArgs<float>*);

}  // namespace sptrsv
