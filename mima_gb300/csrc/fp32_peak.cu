// FP32 FMA throughput of the device, measured: the denominator of the compute
// roofline of the FP32-split solvers (non-tensor FP32 pipe).  Built as its own
// small library (libfp32peak.so), used by the benchmark only.
//
// Every thread runs 8 independent FMA chains (enough to cover the FMA latency
// with 2048 threads per SM); the grid is 8 blocks of 256 threads per SM.  The
// result is the FMA count x 2 / CUDA-event time of one launch after a warm-up
// launch.  The chains' values stay finite (x -> 0.999 x + 0.001) and are
// folded into one store per block so that nothing is optimised away.
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;
constexpr int kUnroll = 16;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) ffma_chains(float* out, int iters, float a, float b) {
  float x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) x[k] = (float)(threadIdx.x + k) * 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
#pragma unroll
      for (int k = 0; k < kChains; ++k) x[k] = fmaf(x[k], a, b);
    }
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += x[k];
  __shared__ float red[kThreads];
  red[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int j = 0; j < kThreads; ++j) t += red[j];
    out[blockIdx.x] = t;
  }
}

}  // namespace

// Measures the FP32 FMA rate of `device`: TFLOP/s (FMA = 2) and the timed
// launch's duration in ms.  Returns a cudaError_t value (0 on success).
extern "C" int fp32_peak_measure(int device, double* tflops, double* ms) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return (int)e;
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return (int)e;
  const int blocks = sms * 8;
  float* out = nullptr;
  e = cudaMalloc(&out, sizeof(float) * blocks);
  if (e != cudaSuccess) return (int)e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int iters = 4096;
  ffma_chains<<<blocks, kThreads>>>(out, iters / 8, 0.999f, 0.001f);  // warm-up
  cudaEventRecord(e0);
  ffma_chains<<<blocks, kThreads>>>(out, iters, 0.999f, 0.001f);
  cudaEventRecord(e1);
  e = cudaEventSynchronize(e1);
  float t = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return (int)e;
  const double flops = 2.0 * (double)blocks * kThreads * (double)iters * kUnroll * kChains;
  *ms = t;
  *tflops = flops / (t * 1e-3) / 1e12;
  return 0;
}
