// Measurement helper (not part of the library): throughput of the arithmetic
// pipes the chain kernel is designed around -- FP64 FMA/add, FP32 FMA, the
// FP64 -> FP32 conversion, FP64 min/max and FP64 division -- each as
// independent chains of one instruction kind over 8 blocks of 256 threads per
// SM, timed with CUDA events after one warm-up pass.  Prints one line per
// kind and exits non-zero on a CUDA error.
#include <cstdio>
#include <cuda_runtime.h>
#define ITERS 4096
__global__ void k_dfma(double* out, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < ITERS; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_dadd(double* out, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < ITERS; ++i) {
    x0 = x0 + a; x1 = x1 + b; x2 = x2 + a; x3 = x3 + b;
    x4 = x4 + a; x5 = x5 + b; x6 = x6 + a; x7 = x7 + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_ffma(float* out, float a, float b) {
  float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < ITERS; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
// f64 -> f32 conversion throughput (each iteration: one F2F plus one FFMA to keep a dependency)
__global__ void k_f2f(float* out, double a) {
  double d0 = a + threadIdx.x, d1 = d0 * 2, d2 = d0 * 3, d3 = d0 * 5;
  float s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  for (int i = 0; i < ITERS; ++i) {
    s0 += __double2float_rn(d0); s1 += __double2float_rn(d1); s2 += __double2float_rn(d2); s3 += __double2float_rn(d3);
    d0 = __longlong_as_double(__double_as_longlong(d0) + 1);
    d1 = __longlong_as_double(__double_as_longlong(d1) + 1);
    d2 = __longlong_as_double(__double_as_longlong(d2) + 1);
    d3 = __longlong_as_double(__double_as_longlong(d3) + 1);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = s0 + s1 + s2 + s3;
}
// f64 compare/select throughput (DSETP + select) as used by a clip
__global__ void k_dmin(double* out, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < ITERS; ++i) {
    x0 = fmin(x0, a); x1 = fmax(x1, b); x2 = fmin(x2, a); x3 = fmax(x3, b);
    x4 = fmin(x4, a); x5 = fmax(x5, b); x6 = fmin(x6, a); x7 = fmax(x7, b);
    a = a + 0.0; // keep values live
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_ddiv(double* out, double a) {
  double x0 = threadIdx.x + 1.5, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  for (int i = 0; i < ITERS / 8; ++i) {
    x0 = a / x0; x1 = a / x1; x2 = a / x2; x3 = a / x3;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}
int main() {
  int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  int clk; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  printf("SMs %d clock %d kHz\n", sms, clk);
  int blocks = sms * 8, threads = 256; size_t nt = (size_t)blocks * threads;
  double* dout; cudaMalloc(&dout, nt * 8);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  float ms;
  for (int rep = 0; rep < 2; ++rep) {
    cudaEventRecord(e0); k_dfma<<<blocks, threads>>>(dout, 0.999, 1e-3); cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1); printf("DFMA: %.3f ms -> %.3f Tinst/s (%.2f /clk/SM at max clock)\n", ms, nt * ITERS * 8 / (ms * 1e9), nt * ITERS * 8 / (ms * 1e-3) / (sms * clk * 1e3));
    cudaEventRecord(e0); k_dadd<<<blocks, threads>>>(dout, 1e-3, 2e-3); cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1); printf("DADD: %.3f ms -> %.3f Tinst/s (%.2f /clk/SM)\n", ms, nt * ITERS * 8 / (ms * 1e9), nt * ITERS * 8 / (ms * 1e-3) / (sms * clk * 1e3));
    cudaEventRecord(e0); k_ffma<<<blocks, threads>>>((float*)dout, 0.999f, 1e-3f); cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1); printf("FFMA: %.3f ms -> %.3f Tinst/s (%.2f /clk/SM)\n", ms, nt * ITERS * 8 / (ms * 1e9), nt * ITERS * 8 / (ms * 1e-3) / (sms * clk * 1e3));
    cudaEventRecord(e0); k_f2f<<<blocks, threads>>>((float*)dout, 1.2345); cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1); printf("F2F64->32: %.3f ms -> %.3f Tinst/s (%.2f /clk/SM)\n", ms, nt * ITERS * 4 / (ms * 1e9), nt * ITERS * 4 / (ms * 1e-3) / (sms * clk * 1e3));
    cudaEventRecord(e0); k_dmin<<<blocks, threads>>>(dout, 0.5, 0.25); cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1); printf("DMNMX: %.3f ms -> %.3f Tinst/s (%.2f /clk/SM)\n", ms, nt * ITERS * 8 / (ms * 1e9), nt * ITERS * 8 / (ms * 1e-3) / (sms * clk * 1e3));
    cudaEventRecord(e0); k_ddiv<<<blocks, threads>>>(dout, 3.0); cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1); printf("DDIV: %.3f ms -> %.3f Tdiv/s (%.3f /clk/SM)\n", ms, nt * (ITERS/8) * 4 / (ms * 1e9), nt * (ITERS/8) * 4 / (ms * 1e-3) / (sms * clk * 1e3));
  }
  cudaError_t err = cudaGetLastError(); printf("status %s\n", cudaGetErrorString(err));
  return err != cudaSuccess;
}
