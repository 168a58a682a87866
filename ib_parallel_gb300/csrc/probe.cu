// Arithmetic throughput probes (register-resident loops of 8 independent chains
// per thread).  probe_fp64 is the FP64 roof the DST kernels are measured against;
// probe_throughput also reports the effect of partially active warps and the FP32
// and INT32 rates for comparison.
#include <cooperative_groups.h>

#include "kernels.cuh"

namespace ib {

template <int ACTIVE>
__global__ void k_dfma_probe(double* out, int iters, double a, double b) {
  IB_GRID_DEP_WAIT();
  if ((int)(threadIdx.x & 31) >= ACTIVE) return;
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_ffma_probe(float* out, int iters, float a, float b) {
  IB_GRID_DEP_WAIT();
  float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_imad_probe(unsigned* out, int iters, unsigned a, unsigned b) {
  IB_GRID_DEP_WAIT();
  unsigned x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// which: 0 FP64 FMA, 1 FP64 FMA with 16 of 32 lanes active (useful rate),
// 2 FP64 FMA with one warp per SM, 3 FP32 FMA, 4 INT32 IMAD.  Units: T(FL)OP/s.
int probe_latency(int which, double* cycles);
int probe_throughput(int which, double* value) {
  if (which >= 5) return probe_latency(which - 5, value);
  int dev = 0, nsm = 0;
  IB_CUDA_CHECK(cudaGetDevice(&dev));
  IB_CUDA_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  int blocks = nsm * 8, threads = 256;
  int iters = which >= 3 ? 32000 : 4000;
  if (which == 2) { blocks = nsm; threads = 32; }
  void* buf = nullptr;
  IB_CUDA_CHECK(cudaMalloc(&buf, sizeof(double) * (size_t)blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto launch = [&](int it) {
    count_launch();
    switch (which) {
      case 1: k_dfma_probe<16><<<blocks, threads>>>((double*)buf, it, 1.0000001, 1e-9); break;
      case 3: k_ffma_probe<<<blocks, threads>>>((float*)buf, it, 1.0000001f, 1e-9f); break;
      case 4: k_imad_probe<<<blocks, threads>>>((unsigned*)buf, it, 1664525u, 1013904223u); break;
      default: k_dfma_probe<32><<<blocks, threads>>>((double*)buf, it, 1.0000001, 1e-9); break;
    }
  };
  launch(200);
  cudaEventRecord(e0);
  launch(iters);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (e != cudaSuccess || ms <= 0.f) return IB_ERR_CUDA;
  double lanes = (double)blocks * threads * (which == 1 ? 0.5 : 1.0);
  double ops = (which == 4 ? 1.0 : 2.0) * 8.0 * iters * lanes;
  *value = ops / (ms * 1e-3) / 1e12;
  return IB_OK;
}

int probe_fp64(double* tflops) { return probe_throughput(0, tflops); }

// Latencies of dependent operations (cycles per operation, clock64 on one SM; CTA 0 of a cluster
// of 8 CTAs of 128 threads): [0] FP64 FMA, [1] sqrt, [2] division, [3] rsqrt, [4] correctly
// rounded reciprocal (each of [1]-[4] less one dependent FP64 add), [5] cluster barrier,
// [6] load from another CTA's shared memory (a dependent chain of index loads, each index
// converted from the loaded double),
// [7] warp shuffle + FP64 add, [8] CTA barrier.
namespace cgp = cooperative_groups;
__global__ void __cluster_dims__(8, 1, 1) k_latency_probe(long long* out, double a, double b, int n) {
  IB_GRID_DEP_WAIT();
  cgp::cluster_group cl = cgp::this_cluster();
  __shared__ double buf[64];
  const int tid = threadIdx.x;
  for (int i = tid; i < 64; i += blockDim.x) buf[i] = (double)((i * 7) & 63);
  cl.sync();
  const bool lead = cl.block_rank() == 0 && tid == 0;
  long long t0, t1;
  double x = a;
  if (lead) {
    double y = a;
    t0 = clock64(); for (int i = 0; i < n; ++i) y = fma(y, a, b); t1 = clock64(); out[0] = t1 - t0; x += y;
    y = a;
    t0 = clock64(); for (int i = 0; i < n; ++i) y = y + b; t1 = clock64(); out[9] = t1 - t0; x += y;
    y = a + 2.0;
    t0 = clock64(); for (int i = 0; i < n; ++i) y = sqrt(y) + 1.5; t1 = clock64(); out[1] = t1 - t0; x += y;
    y = a + 2.0;
    t0 = clock64(); for (int i = 0; i < n; ++i) y = b / y + 1.5; t1 = clock64(); out[2] = t1 - t0; x += y;
    y = a + 2.0;
    t0 = clock64(); for (int i = 0; i < n; ++i) y = rsqrt(y) + 1.5; t1 = clock64(); out[3] = t1 - t0; x += y;
    y = a + 2.0;
    t0 = clock64(); for (int i = 0; i < n; ++i) y = __drcp_rn(y) + 1.5; t1 = clock64(); out[4] = t1 - t0; x += y;
  }
  __syncthreads();
  t0 = clock64();
  for (int i = 0; i < n; ++i) cl.sync();
  t1 = clock64();
  if (lead) out[5] = t1 - t0;
  if (tid == 0) {
    const double* rb = cl.map_shared_rank(buf, (cl.block_rank() + 1) % 8);
    int idx = 0;
    t0 = clock64();
    for (int i = 0; i < n; ++i) idx = (int)rb[idx];
    t1 = clock64();
    if (lead) out[6] = t1 - t0;
    x += idx;
  }
  if (tid < 32) {
    double y = a + tid;
    t0 = clock64();
    for (int i = 0; i < n; ++i) y += __shfl_xor_sync(0xffffffffu, y, 1 << (i & 3));
    t1 = clock64();
    if (lead) out[7] = t1 - t0;
    x += y;
  }
  __syncthreads();
  t0 = clock64();
  for (int i = 0; i < n; ++i) __syncthreads();
  t1 = clock64();
  if (lead) out[8] = t1 - t0;
  cl.sync();   // no CTA exits while another reads its shared memory
  if (x == 12345.678) out[15] = 1;
}

int probe_latency(int which, double* cycles) {
  if (which < 0 || which > 8) return IB_ERR_ARG;
  long long* d = nullptr;
  IB_CUDA_CHECK(cudaMalloc(&d, 16 * sizeof(long long)));
  const int n = 256;
  count_launches(2);
  k_latency_probe<<<8, 128>>>(d, 1.0000001, 1e-9, n);
  k_latency_probe<<<8, 128>>>(d, 1.0000001, 1e-9, n);
  long long h[16] = {};
  cudaError_t e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return IB_ERR_CUDA;
  double v = (double)h[which] / n;
  if (which >= 1 && which <= 4) v -= (double)h[9] / n;   // less the dependent add of the chain
  *cycles = v;
  return IB_OK;
}

}  // namespace ib
