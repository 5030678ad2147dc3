// ffs_measure_fp64_peak: the FP64 arithmetic rate of the current GPU, measured with this
// library's own kernels. It is the denominator of the FP64 plain form's roofline: on
// GB300 the FP64 pipe, not HBM, bounds the FP64 transforms, and no vendor figure is
// measured on the part in use. No counterpart in the reference.
//
// Each thread runs NCH independent dependency chains of fused multiply-adds (or adds) in
// registers; the chains never converge, so the pipe stays full. One FMA counts two
// flops, one add one flop. Grid: every SM x 8 CTAs x 256 threads; timed with CUDA events
// after one warm-up launch.
// On GB300 FP64 adds (and multiplies) issue at about 0.84 of the FMA instruction rate,
// so the transforms, whose butterflies are mostly adds, are bounded by the add rate.
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/ffs.h"

namespace ffsgpu {
void set_global_error(const std::string& msg);
}

namespace {

constexpr int NCH = 8;

template <bool FMA>
__global__ void __launch_bounds__(256) k_fp64_chains(double* out, int iters, double a, double b) {
  double x[NCH];
#pragma unroll
  for (int c = 0; c < NCH; ++c) x[c] = (double)(threadIdx.x + c) * 1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < NCH; ++c) x[c] = FMA ? fma(x[c], a, b) : x[c] + b;
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < NCH; ++c) s += x[c];
  if (s == 1.2345e300) out[0] = s;   // never true for these inputs; keeps the chains live
}

int measure(int device, double* fma_tflops, double* add_tflops) {
  if (!fma_tflops || !add_tflops) return FFS_EINVAL;
  int old = 0;
  if (cudaGetDevice(&old) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) {
    ffsgpu::set_global_error("ffs_measure_fp64_peak: cannot select the device");
    return FFS_ECUDA;
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  double* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(double));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256, iters = 1 << 14;
  double res[2] = {0.0, 0.0};
  for (int v = 0; v < 2 && e == cudaSuccess; ++v) {
    auto k = v == 0 ? k_fp64_chains<true> : k_fp64_chains<false>;
    k<<<blocks, threads>>>(out, iters / 8, 0.999999, 1e-7);   // warm-up
    cudaEventRecord(e0);
    k<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    const double ops = (double)blocks * threads * iters * NCH * (v == 0 ? 2.0 : 1.0);
    res[v] = ms > 0 ? ops / (ms * 1e-3) / 1e12 : 0.0;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  cudaSetDevice(old);
  if (e != cudaSuccess) {
    ffsgpu::set_global_error(std::string("ffs_measure_fp64_peak: ") + cudaGetErrorString(e));
    return FFS_ECUDA;
  }
  *fma_tflops = res[0];
  *add_tflops = res[1];
  return FFS_OK;
}

}  // namespace

extern "C" int ffs_measure_fp64_peak(int32_t device, double* fma_tflops, double* add_tflops) {
  try {
    return measure(device, fma_tflops, add_tflops);
  } catch (...) {
    ffsgpu::set_global_error("ffs_measure_fp64_peak: internal error");
    return FFS_EINVAL;
  }
}
