// Arithmetic and copy throughput of the device the handle runs on, measured
// in the run that reports against it: FP64 and FP32 fused multiply-add rates
// (the roofs of the transform kernels, whose FP64 forms are bound by the FP64
// pipe on this part) and a device-to-device copy rate.
//
// FMA loop: every thread carries CHAINS independent dependency chains
// x = x * a + b (a, b known only at run time) through ITERS rounds; the grid
// is 8 blocks of 256 threads per SM.  flops = 2 * CHAINS * ITERS * threads.
// The result is stored only when a run-time flag that the host never sets is
// non-zero, so the compiler keeps every FMA.  Copy: float4 grid-stride copy
// of a buffer larger than L2; bytes = read + write.
#include <cuda_runtime.h>

#include <cstdio>

#include "chgpu.h"

namespace {

template <typename T, int CHAINS>
__global__ void __launch_bounds__(256) k_fma_loop(T a, T b, int iters, int flag, T* __restrict__ sink) {
  T x[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) x[c] = T(threadIdx.x + c) * T(1e-3f);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = fma(x[c], a, b);
  }
  if (flag) {
    T s = T();
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += x[c];
    sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
  }
}

__global__ void __launch_bounds__(256) k_copy(const float4* __restrict__ src, float4* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

template <typename K>
float time_launches(K launch, int reps, cudaStream_t s) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();  // warm-up
  cudaEventRecord(e0, s);
  for (int r = 0; r < reps; ++r) launch();
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / reps;
}

}  // namespace

extern "C" int chgpu_measure_peaks(double* fp64_tflops, double* fp32_tflops, double* copy_gbs, char* err,
                                   size_t errlen) {
  auto fail = [&](cudaError_t e, const char* what) {
    if (err && errlen) snprintf(err, errlen, "%s: %s", what, cudaGetErrorString(e));
    return CHGPU_E_CUDA;
  };
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(e, "cudaGetDevice");
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return fail(e, "cudaDeviceGetAttribute");
  cudaStream_t s;
  if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "cudaStreamCreate");
  const int blocks = sms * 8, threads = 256;
  const double nthreads = (double)blocks * threads;
  if (fp64_tflops) {
    constexpr int CH = 8;
    const int iters = 4096;
    const float ms = time_launches([&] { k_fma_loop<double, CH><<<blocks, threads, 0, s>>>(0.999, 1e-7, iters, 0, nullptr); }, 3, s);
    *fp64_tflops = 2.0 * CH * iters * nthreads / (ms * 1e-3) / 1e12;
  }
  if (fp32_tflops) {
    constexpr int CH = 8;
    const int iters = 65536;
    const float ms = time_launches([&] { k_fma_loop<float, CH><<<blocks, threads, 0, s>>>(0.999f, 1e-7f, iters, 0, nullptr); }, 3, s);
    *fp32_tflops = 2.0 * CH * iters * nthreads / (ms * 1e-3) / 1e12;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) {
    cudaStreamDestroy(s);
    return fail(e, "FMA loop");
  }
  if (copy_gbs) {
    const size_t bytes = (size_t)1 << 30;  // 1 GiB each way: far larger than L2
    void *a = nullptr, *b = nullptr;
    if ((e = cudaMalloc(&a, bytes)) != cudaSuccess) {
      cudaStreamDestroy(s);
      return fail(e, "cudaMalloc");
    }
    if ((e = cudaMalloc(&b, bytes)) != cudaSuccess) {
      cudaFree(a);
      cudaStreamDestroy(s);
      return fail(e, "cudaMalloc");
    }
    cudaMemsetAsync(a, 0, bytes, s);
    const size_t n = bytes / sizeof(float4);
    const float ms = time_launches(
        [&] { k_copy<<<sms * 4, 256, 0, s>>>((const float4*)a, (float4*)b, n); }, 10, s);
    *copy_gbs = 2.0 * bytes / (ms * 1e-3) / 1e9;
    cudaFree(a);
    cudaFree(b);
  }
  e = cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? CHGPU_OK : fail(e, "peak measurement");
}
