// The FP64 roof the benchmark reports its DST pass against: FP64 FMA throughput of the
// current device, measured with a register-resident loop (8 independent FMA chains per
// thread, 8 CTAs of 256 threads per SM, so every SM sub-partition's FP64 pipe stays busy).
#include "kernels.cuh"

namespace ib {

__global__ void k_dfma_peak(double* out, int iters, double a, double b) {
  IB_GRID_DEP_WAIT();
  double x[8];
  for (int j = 0; j < 8; ++j) x[j] = threadIdx.x + j;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
  double s = 0.0;
  for (int j = 0; j < 8; ++j) s += x[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int probe_fp64(double* tflops) {
  int dev = 0, nsm = 0;
  IB_CUDA_CHECK(cudaGetDevice(&dev));
  IB_CUDA_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = nsm * 8, threads = 256, iters = 4000;
  double* buf = nullptr;
  IB_CUDA_CHECK(cudaMalloc(&buf, sizeof(double) * (size_t)blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  count_launches(2);
  k_dfma_peak<<<blocks, threads>>>(buf, 200, 1.0000001, 1e-9);   // warm-up (clocks, module load)
  cudaEventRecord(e0);
  k_dfma_peak<<<blocks, threads>>>(buf, iters, 1.0000001, 1e-9);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (e != cudaSuccess || ms <= 0.f) return IB_ERR_CUDA;
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  return IB_OK;
}

}  // namespace ib
