// Machine probe behind the executor design choices (not part of the library):
// FP64/FP32 FMA throughput, dependent DFMA and FP64-division latency, the
// one-way latency of a flag hop between two SMs (relaxed, release/acquire,
// and the push scheme's atomic sum + release counter), a shared-memory hop,
// and atomic throughput. The two ping-pong CTAs are one cooperative launch, so
// they are co-resident; every spin is bounded and reports through `err`.
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o machine_probe machine_probe.cu && ./machine_probe
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { printf("CUDA %s at %d: %s\n", #x, __LINE__, cudaGetErrorString(e_)); exit(1);} } while (0)

__global__ void k_dfma(double* out, int iters) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, 0.999999, 1e-7); a1 = fma(a1, 0.999999, 1e-7); a2 = fma(a2, 0.999999, 1e-7); a3 = fma(a3, 0.999999, 1e-7);
    a4 = fma(a4, 0.999999, 1e-7); a5 = fma(a5, 0.999999, 1e-7); a6 = fma(a6, 0.999999, 1e-7); a7 = fma(a7, 0.999999, 1e-7);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
__global__ void k_sfma(float* out, int iters) {
  float a0 = threadIdx.x * 1e-3f, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < iters; ++i) {
    a0 = fmaf(a0, 0.999999f, 1e-7f); a1 = fmaf(a1, 0.999999f, 1e-7f); a2 = fmaf(a2, 0.999999f, 1e-7f); a3 = fmaf(a3, 0.999999f, 1e-7f);
    a4 = fmaf(a4, 0.999999f, 1e-7f); a5 = fmaf(a5, 0.999999f, 1e-7f); a6 = fmaf(a6, 0.999999f, 1e-7f); a7 = fmaf(a7, 0.999999f, 1e-7f);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
__global__ void k_ddiv(double* out, int iters) {
  double a0 = threadIdx.x + 1.5, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
  for (int i = 0; i < iters; ++i) {
    a0 = 3.0 / a0 + 1.0; a1 = 3.0 / a1 + 1.0; a2 = 3.0 / a2 + 1.0; a3 = 3.0 / a3 + 1.0;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3;
}
// dependent chain latency, one warp
__global__ void k_dlat(double* out, long long* cyc, int iters) {
  double a = threadIdx.x * 1e-3;
  long long t0 = clock64();
  for (int i = 0; i < iters; ++i) a = fma(a, 0.999999, 1e-7);
  long long t1 = clock64();
  out[threadIdx.x] = a;
  if (threadIdx.x == 0) cyc[0] = t1 - t0;
  double d = threadIdx.x + 1.5;
  t0 = clock64();
  for (int i = 0; i < iters; ++i) d = 3.0 / d + 1.0;
  t1 = clock64();
  out[32 + threadIdx.x] = d;
  if (threadIdx.x == 0) cyc[1] = t1 - t0;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v; asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory"); return v;
}
__device__ __forceinline__ unsigned ld_relaxed(const unsigned* p) {
  unsigned v; asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory"); return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(unsigned* p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned smid() { unsigned r; asm volatile("mov.u32 %0, %%smid;" : "=r"(r)); return r; }

constexpr long long SPIN_MAX = 1LL << 24;

// mode 0: relaxed store / relaxed poll; 1: release/acquire; 2: push-style (red f64 + release red counter; acquire poll + load)
__global__ void k_pingpong(unsigned* flags, double* sums, int rounds, int mode, long long* out, int* err) {
  if (threadIdx.x != 0) return;
  const int me = blockIdx.x;           // 0 or 1
  unsigned* mine = flags + me * 64;    // separate 256B lines
  unsigned* theirs = flags + (1 - me) * 64;
  double* my_sum = sums + me * 32;
  double* their_sum = sums + (1 - me) * 32;
  long long t0 = clock64();
  long long g0; asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g0));
  double acc = 0;
  for (int r = 1; r <= rounds; ++r) {
    // CTA 0 sends first, CTA 1 answers
    if (me == 1) {
      long long s = 0;
      if (mode == 0) { while (ld_relaxed(theirs) != (unsigned)r && ++s < SPIN_MAX) {} }
      else { while (ld_acquire(theirs) != (unsigned)r && ++s < SPIN_MAX) {} }
      if (s >= SPIN_MAX) { atomicExch(err, 100 + mode); return; }
      if (mode == 2) acc += *(volatile double*)my_sum;
    }
    if (mode == 0) st_relaxed(mine, r);
    else if (mode == 1) st_release(mine, r);
    else { atomicAdd(their_sum, 1.0); red_release_add(mine, 1u); }
    if (me == 0) {
      long long s = 0;
      if (mode == 0) { while (ld_relaxed(theirs) != (unsigned)r && ++s < SPIN_MAX) {} }
      else { while (ld_acquire(theirs) != (unsigned)r && ++s < SPIN_MAX) {} }
      if (s >= SPIN_MAX) { atomicExch(err, 200 + mode); return; }
      if (mode == 2) acc += *(volatile double*)my_sum;
    }
  }
  long long t1 = clock64();
  long long g1; asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g1));
  out[me * 4 + 0] = t1 - t0;
  out[me * 4 + 1] = g1 - g0;
  out[me * 4 + 2] = smid();
  out[me * 4 + 3] = (long long)acc;
}

// smem ping-pong between warp 0 and warp 1 of one CTA
__global__ void k_smem_pingpong(int rounds, long long* out, int* err) {
  __shared__ volatile unsigned f[64];
  if (threadIdx.x < 64) f[threadIdx.x] = 0;
  __syncthreads();
  const int w = threadIdx.x / 32;
  if ((threadIdx.x & 31) != 0 || w > 1) return;
  long long t0 = clock64();
  for (int r = 1; r <= rounds; ++r) {
    if (w == 1) { long long s = 0; while (f[0] != (unsigned)r && ++s < SPIN_MAX) {} if (s >= SPIN_MAX) { atomicExch(err, 300); return; } f[32] = r; }
    else { f[0] = r; long long s = 0; while (f[32] != (unsigned)r && ++s < SPIN_MAX) {} if (s >= SPIN_MAX) { atomicExch(err, 301); return; } }
  }
  long long t1 = clock64();
  if (w == 0) out[0] = t1 - t0;
}

__global__ void k_atomic_one(unsigned* p, int per_thread) {
  for (int i = 0; i < per_thread; ++i) atomicAdd(p, 1u);
}
__global__ void k_atomic_many(unsigned* p, int per_thread, int nslots) {
  unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
  for (int i = 0; i < per_thread; ++i) atomicAdd(p + ((id * 2654435761u + i * 40503u) % nslots), 1u);
}
__global__ void k_ratomic_f64(double* p, int per_thread, int nslots) {
  unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
  for (int i = 0; i < per_thread; ++i) atomicAdd(p + ((id * 2654435761u + i * 40503u) % nslots), 1.0);
}

int main() {
  cudaDeviceProp prop; CK(cudaGetDeviceProperties(&prop, 0));
  printf("device %s sms=%d l2=%d MB smem/blk optin=%zu clock? \n", prop.name, prop.multiProcessorCount, prop.l2CacheSize >> 20, prop.sharedMemPerBlockOptin);
  const int sms = prop.multiProcessorCount;
  cudaEvent_t e0, e1; CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
  float ms;
  {
    const int blocks = sms * 8, threads = 256, iters = 4096;
    double* d; CK(cudaMalloc(&d, sizeof(double) * blocks * threads));
    k_dfma<<<blocks, threads>>>(d, 16); CK(cudaDeviceSynchronize());
    CK(cudaEventRecord(e0)); k_dfma<<<blocks, threads>>>(d, iters); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(&ms, e0, e1));
    double flops = 2.0 * 8 * iters * (double)blocks * threads;
    printf("DFMA: %.3f ms  %.3f TFLOP/s\n", ms, flops / ms / 1e9);
    float* f; CK(cudaMalloc(&f, sizeof(float) * blocks * threads));
    k_sfma<<<blocks, threads>>>(f, 16); CK(cudaDeviceSynchronize());
    CK(cudaEventRecord(e0)); k_sfma<<<blocks, threads>>>(f, iters * 8); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(&ms, e0, e1));
    flops = 2.0 * 8 * iters * 8 * (double)blocks * threads;
    printf("FFMA: %.3f ms  %.3f TFLOP/s\n", ms, flops / ms / 1e9);
    k_ddiv<<<blocks, threads>>>(d, 16); CK(cudaDeviceSynchronize());
    CK(cudaEventRecord(e0)); k_ddiv<<<blocks, threads>>>(d, iters / 8); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(&ms, e0, e1));
    double divs = 4.0 * (iters / 8) * (double)blocks * threads;
    printf("DDIV: %.3f ms  %.3f Gdiv/s\n", ms, divs / ms / 1e6);
    long long* cyc; CK(cudaMalloc(&cyc, 16));
    k_dlat<<<1, 32>>>(d, cyc, 1024); CK(cudaDeviceSynchronize());
    long long hc[2]; CK(cudaMemcpy(hc, cyc, 16, cudaMemcpyDeviceToHost));
    printf("DFMA dep latency %.1f cyc; DDIV dep latency %.1f cyc\n", hc[0] / 1024.0, hc[1] / 1024.0);
    CK(cudaFree(d)); CK(cudaFree(f)); CK(cudaFree(cyc));
  }
  {
    unsigned* flags; double* sums; long long* out; int* err;
    CK(cudaMalloc(&flags, 4096)); CK(cudaMalloc(&sums, 4096)); CK(cudaMalloc(&out, 64)); CK(cudaMalloc(&err, 4));
    for (int mode = 0; mode < 3; ++mode) {
      CK(cudaMemset(flags, 0, 4096)); CK(cudaMemset(sums, 0, 4096)); CK(cudaMemset(err, 0, 4)); CK(cudaMemset(out, 0, 64));
      int rounds = 20000;
      void* args[] = {&flags, &sums, &rounds, &mode, &out, &err};
      CK(cudaLaunchCooperativeKernel((void*)k_pingpong, dim3(2), dim3(32), args, 0, 0));
      CK(cudaDeviceSynchronize());
      long long h[8]; int herr; CK(cudaMemcpy(h, out, 64, cudaMemcpyDeviceToHost)); CK(cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost));
      printf("pingpong mode %d: err=%d  one-way hop %.1f cyc  %.1f ns  (sm %lld <-> sm %lld)\n", mode, herr,
             h[0] / (2.0 * rounds), h[1] / (2.0 * rounds), h[2], h[6]);
    }
    CK(cudaMemset(err, 0, 4));
    k_smem_pingpong<<<1, 64>>>(20000, out, err); CK(cudaDeviceSynchronize());
    long long h; int herr; CK(cudaMemcpy(&h, out, 8, cudaMemcpyDeviceToHost)); CK(cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost));
    printf("smem pingpong: err=%d one-way %.1f cyc\n", herr, h / 40000.0);
    CK(cudaFree(flags)); CK(cudaFree(sums)); CK(cudaFree(out)); CK(cudaFree(err));
  }
  {
    unsigned* p; CK(cudaMalloc(&p, sizeof(unsigned) * (1 << 22))); CK(cudaMemset(p, 0, 4 << 22));
    k_atomic_one<<<sms, 256>>>(p, 4); CK(cudaDeviceSynchronize());
    CK(cudaEventRecord(e0)); k_atomic_one<<<sms, 256>>>(p, 64); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(&ms, e0, e1));
    printf("single-address atomics: %.3f ms  %.1f M/s\n", ms, sms * 256.0 * 64 / ms / 1e3);
    CK(cudaEventRecord(e0)); k_atomic_many<<<sms * 8, 256>>>(p, 64, 1 << 22); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(&ms, e0, e1));
    printf("scattered int atomics (4M slots): %.3f ms  %.1f G/s\n", ms, sms * 8 * 256.0 * 64 / ms / 1e6);
    double* q; CK(cudaMalloc(&q, sizeof(double) * (1 << 22))); CK(cudaMemset(q, 0, 8 << 22));
    CK(cudaEventRecord(e0)); k_ratomic_f64<<<sms * 8, 256>>>(q, 64, 1 << 22); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(&ms, e0, e1));
    printf("scattered f64 atomics (4M slots): %.3f ms  %.1f G/s\n", ms, sms * 8 * 256.0 * 64 / ms / 1e6);
    CK(cudaFree(p)); CK(cudaFree(q));
  }
  printf("probe done\n");
  return 0;
}
