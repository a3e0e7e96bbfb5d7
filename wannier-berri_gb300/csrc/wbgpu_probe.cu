// FMA-rate probe: the roofline denominator for kernels bound by the FP64 or FP32 pipes,
// which the copy / bf16-GEMM peaks do not cover.  Eight independent FMA chains per thread.
#include "wbgpu_common.cuh"

namespace {
template <typename T>
__global__ void fma_probe(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x * (T)1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  T x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

extern "C" int wbg_probe_fma(int fp64, int blocks, int threads, int iters, void* out, double* flops_per_launch,
                             void* stream) {
  if (blocks < 1 || threads < 32 || threads > 1024 || iters < 1 || !out || !flops_per_launch) return WBG_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (fp64)
    fma_probe<double><<<blocks, threads, 0, s>>>((double*)out, iters, 0.999, 1e-3);
  else
    fma_probe<float><<<blocks, threads, 0, s>>>((float*)out, iters, 0.999f, 1e-3f);
  *flops_per_launch = 2.0 * 8.0 * (double)iters * (double)blocks * (double)threads;
  return wbg_cuda_status(cudaGetLastError());
}
