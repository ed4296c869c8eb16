// Arithmetic and copy rates of the GPU: the ceilings the plain FP64 form and
// the mixed form are held against (FP64 fused multiply-add, FP32 FMA, FP64
// divide and square root, FP64 -> FP32 conversion, and a device-to-device
// copy).  Built and run by `python -m weldform_gb300.probe_rates`; every loop
// is bounded and every buffer is written in range.
#include <cstdio>
#include <cuda_runtime.h>

#define ITERS 2048

__global__ void k_dfma(double* out, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < ITERS; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_ffma(float* out, float a, float b) {
  float x0 = threadIdx.x * 1e-9f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < ITERS; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_ddiv(double* out, double a) {
  double x0 = threadIdx.x + 1.5, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  for (int i = 0; i < ITERS / 8; ++i) {
    x0 = a / x0 + 1.0; x1 = a / x1 + 1.0; x2 = a / x2 + 1.0; x3 = a / x3 + 1.0;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}
__global__ void k_dsqrt(double* out) {
  double x0 = threadIdx.x + 1.5, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  for (int i = 0; i < ITERS / 8; ++i) {
    x0 = sqrt(x0) + 1.0; x1 = sqrt(x1) + 1.0; x2 = sqrt(x2) + 1.0; x3 = sqrt(x3) + 1.0;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}
__global__ void k_d2f(float* out, double a) {
  double x0 = threadIdx.x * 1e-3;
  float s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  for (int i = 0; i < ITERS; ++i) {
    x0 += a;
    s0 += (float)x0; s1 += (float)(x0 * 2.0); s2 += (float)(x0 * 3.0); s3 += (float)(x0 * 5.0);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = s0 + s1 + s2 + s3;
}
__global__ void k_copy(const double4_32a* __restrict__ a, double4_32a* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) b[i] = a[i];
}

int main() {
  int nsm = 0; cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0);
  int clk = 0; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  int blocks = nsm * 8, threads = 256;
  size_t nthreads = (size_t)blocks * threads;
  double* dout; float* fout;
  cudaMalloc(&dout, nthreads * sizeof(double)); cudaMalloc(&fout, nthreads * sizeof(float));
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  float ms;
  auto timeit = [&](const char* name, double ops_per_thread, auto launch) {
    for (int w = 0; w < 3; ++w) launch();
    cudaEventRecord(e0);
    for (int r = 0; r < 5; ++r) launch();
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    double ops = ops_per_thread * nthreads * 5;
    printf("%-8s %10.3f Gop/s  (%.3f ms/launch)\n", name, ops / (ms * 1e-3) / 1e9, ms / 5);
  };
  timeit("dfma", 8.0 * ITERS, [&] { k_dfma<<<blocks, threads>>>(dout, 0.999999, 1e-7); });
  timeit("ffma", 8.0 * ITERS, [&] { k_ffma<<<blocks, threads>>>(fout, 0.999999f, 1e-7f); });
  timeit("ddiv", 4.0 * ITERS / 8, [&] { k_ddiv<<<blocks, threads>>>(dout, 3.0); });
  timeit("dsqrt", 4.0 * ITERS / 8, [&] { k_dsqrt<<<blocks, threads>>>(dout); });
  timeit("d2f", 4.0 * ITERS, [&] { k_d2f<<<blocks, threads>>>(fout, 1e-3); });
  size_t n4 = (size_t)1 << 27;  // 4 GiB each buffer of double4_32a (32 B) -> 4 GiB
  double4_32a *a, *b;
  if (cudaMalloc(&a, n4 * 32) == cudaSuccess && cudaMalloc(&b, n4 * 32) == cudaSuccess) {
    cudaMemset(a, 0, n4 * 32);
    for (int w = 0; w < 3; ++w) k_copy<<<nsm * 4, 512>>>(a, b, n4);
    cudaEventRecord(e0);
    for (int r = 0; r < 5; ++r) k_copy<<<nsm * 4, 512>>>(a, b, n4);
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    printf("copy     %10.1f GB/s\n", 2.0 * n4 * 32 * 5 / (ms * 1e-3) / 1e9);
  }
  printf("SMs %d clock %d kHz; err=%s\n", nsm, clk, cudaGetErrorString(cudaDeviceSynchronize()));
  return 0;
}
