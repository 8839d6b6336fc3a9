// osb_probe.cu -- FMA-throughput probe used by bench.py to measure the FP32 and FP64 pipe
// peaks of the GPU it runs on (the compute roof of the reconstruction kernels).  Not part of
// the solver ABI.
#include <cuda_runtime.h>

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)-12345) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" {

// Returns the sustained FMA rate in FLOP/s (2 flops per FMA) for double (fp64 != 0) or float.
int osb_probe_fma(int device, int fp64, double* flops_out) {
  if (cudaSetDevice(device) != cudaSuccess) return -2;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return -2;
  const int threads = 256;
  const int blocks = prop.multiProcessorCount * 8;
  const int iters = fp64 ? 64 : 2048;
  void* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess) return -2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    if (fp64) k_fma<double><<<blocks, threads>>>((double*)buf, iters, 0.999999, 1e-7);
    else k_fma<float><<<blocks, threads>>>((float*)buf, iters, 0.9999f, 1e-5f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (cudaGetLastError() != cudaSuccess) return -2;
  double fmas = (double)blocks * threads * iters * 16 * 8;
  *flops_out = 2.0 * fmas / (best * 1e-3);
  return 0;
}

}  // extern "C"
