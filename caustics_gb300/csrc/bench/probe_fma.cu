// Throughput probe for the roofline denominators of the magnification kernels
// (benchmark-only library libcgb_bench.so, not part of the C ABI): FP32 / FP64
// fused multiply-add issue rate of the whole GPU.  The magnification kernels
// are SIMT arithmetic (no dense contraction, negligible HBM traffic), so their
// roofline is the FMA pipe, measured here on the same device and clocks as the
// timed kernels.
//
//   int cgb_probe_fma(int fp64, int iters, int blocks, void *out, void *stream)
// launches `blocks` CTAs of 256 threads, each thread running iters*16*8
// independent fused multiply-adds in FP32 (fp64 = 0) or FP64; flops =
// blocks*256*iters*256.  `out` needs one element per block (never written in
// practice).  Returns 0, or 1 (bad arguments) / 2 (launch error).
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

template <typename T>
__global__ void fma_probe(int iters, T seed, T *out) {
  // 8 independent chains per thread: enough ILP to saturate the pipe
  T a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
    a7 = a0 + 7;
  const T m = (T)0.999999, c = (T)1e-7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll 16
    for (int u = 0; u < 16; ++u) {
      a0 = a0 * m + c;
      a1 = a1 * m + c;
      a2 = a2 * m + c;
      a3 = a3 * m + c;
      a4 = a4 * m + c;
      a5 = a5 * m + c;
      a6 = a6 * m + c;
      a7 = a7 * m + c;
    }
  }
  T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == (T)-1) out[blockIdx.x] = s;  // never true; keeps the chains live
}

}  // namespace

extern "C" int cgb_probe_fma(int32_t fp64, int32_t iters, int32_t blocks, void *out, void *stream) {
  if (iters < 1 || blocks < 1 || !out) return 1;
  cudaStream_t s = (cudaStream_t)stream;
  if (fp64)
    fma_probe<double><<<blocks, 256, 0, s>>>(iters, 1.0, (double *)out);
  else
    fma_probe<float><<<blocks, 256, 0, s>>>(iters, 1.0f, (float *)out);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
