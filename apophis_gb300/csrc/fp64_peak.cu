// fp64_peak.cu -- throughput of the FP64 instructions this hydro path is made of, on the
// current GPU: add, mul, fma, compare, min, divide, sqrt, rsqrt, reciprocal, with FP32 FMA and
// INT32 for scale.  Eight independent dependency chains per thread over an occupancy-filling
// grid; each line prints operations per second and per clock per SM at the observed clock.
// Built and run by apophis_gb300/fp64_peak.py; the FP64 roofline of bench.py uses its dfma rate.
#include <cstdio>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("CUDA %s @%d\n",cudaGetErrorString(e),__LINE__); return 1;}}while(0)
constexpr int CH = 8;
template <int OP> __global__ void kd(double* out, int iters, double b, double c) {
  double a[CH];
  for (int i = 0; i < CH; ++i) a[i] = 1.0 + 1e-3 * (threadIdx.x + i);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < CH; ++i) {
      if (OP == 0) a[i] = fma(a[i], b, c);
      if (OP == 1) a[i] = a[i] + c;
      if (OP == 2) a[i] = a[i] * b;
      if (OP == 3) a[i] = (a[i] < b) ? a[i] + c : a[i] - c;   // add + setp
      if (OP == 4) a[i] = fmin(a[i], b) + c;                   // add + min
      if (OP == 5) a[i] = b / a[i];
      if (OP == 6) a[i] = sqrt(a[i]) + c;                      // add + sqrt
      if (OP == 7) a[i] = rsqrt(a[i]) + c;
      if (OP == 8) a[i] = __drcp_rn(a[i]) + c;
    }
  }
  double s = 0; for (int i = 0; i < CH; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void kf(float* out, int iters, float b, float c) {
  float a[CH];
  for (int i = 0; i < CH; ++i) a[i] = 1.0f + 1e-3f * (threadIdx.x + i);
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) a[i] = fmaf(a[i], b, c);
  float s = 0; for (int i = 0; i < CH; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void ki(int* out, int iters, int b, int c) {
  unsigned a[CH];
  for (int i = 0; i < CH; ++i) a[i] = threadIdx.x * 7 + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) a[i] = (a[i] ^ b) + c;
  unsigned s = 0; for (int i = 0; i < CH; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
int main() {
  int dev = 0; cudaDeviceProp p; CK(cudaGetDeviceProperties(&p, dev));
  int sms = p.multiProcessorCount;
  printf("device %s sms %d cc %d.%d\n", p.name, sms, p.major, p.minor);
  int blocks = sms * 8, threads = 256, iters = 2048;
  double* d; CK(cudaMalloc(&d, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  const char* names[] = {"dfma", "dadd", "dmul", "dadd+dsetp", "dadd+dmin", "ddiv", "dadd+dsqrt", "dadd+drsqrt", "dadd+drcp"};
  for (int op = 0; op < 9; ++op) {
    for (int rep = 0; rep < 2; ++rep) {
      int it = (op >= 5) ? iters / 8 : iters;
      CK(cudaEventRecord(e0));
      switch (op) {
        case 0: kd<0><<<blocks, threads>>>(d, it, 0.999999, 1e-7); break;
        case 1: kd<1><<<blocks, threads>>>(d, it, 0.999999, 1e-7); break;
        case 2: kd<2><<<blocks, threads>>>(d, it, 0.999999, 1e-7); break;
        case 3: kd<3><<<blocks, threads>>>(d, it, 1.0, 1e-7); break;
        case 4: kd<4><<<blocks, threads>>>(d, it, 1.5, 1e-7); break;
        case 5: kd<5><<<blocks, threads>>>(d, it, 1.0000001, 1e-7); break;
        case 6: kd<6><<<blocks, threads>>>(d, it, 1.0, 1e-7); break;
        case 7: kd<7><<<blocks, threads>>>(d, it, 1.0, 1e-7); break;
        case 8: kd<8><<<blocks, threads>>>(d, it, 1.0, 1e-7); break;
      }
      CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1)); CK(cudaGetLastError());
      float ms; cudaEventElapsedTime(&ms, e0, e1);
      double n = (double)blocks * threads * it * CH;
      if (rep == 1) printf("%-14s %8.3f ms  %10.3f Gop/s  %8.3f op/clk/SM@1.9GHz\n", names[op], ms, n / ms / 1e6, n / (ms * 1e-3) / sms / 1.9e9);
    }
  }
  for (int rep = 0; rep < 2; ++rep) {
    CK(cudaEventRecord(e0)); kf<<<blocks, threads>>>((float*)d, iters, 0.999999f, 1e-7f); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms, e0, e1); double n = (double)blocks * threads * iters * CH;
    if (rep) printf("%-14s %8.3f ms  %10.3f Gop/s  %8.3f op/clk/SM@1.9GHz\n", "ffma", ms, n / ms / 1e6, n / (ms * 1e-3) / sms / 1.9e9);
  }
  for (int rep = 0; rep < 2; ++rep) {
    CK(cudaEventRecord(e0)); ki<<<blocks, threads>>>((int*)d, iters, 12345, 7); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms, e0, e1); double n = (double)blocks * threads * iters * CH * 2;
    if (rep) printf("%-14s %8.3f ms  %10.3f Gop/s  %8.3f op/clk/SM@1.9GHz\n", "int xor+add", ms, n / ms / 1e6, n / (ms * 1e-3) / sms / 1.9e9);
  }
  return 0;
}
