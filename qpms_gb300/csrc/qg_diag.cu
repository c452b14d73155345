// Diagnostics: an FP64 FMA throughput probe used as the FP64-pipe roofline
// denominator (the measured-peaks file covers HBM copy and bf16 GEMM only).
#include "qg_internal.h"

namespace qg {
namespace {
__global__ void __launch_bounds__(256) dfma_probe(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 12345.678) out[blockIdx.x] = s;  // keeps the chain live
}
}  // namespace
}  // namespace qg

extern "C" int qpms_gpu_measure_fp64_peak(double *tflops) {
  using namespace qg;
  clear_error();
  if (!tflops) return QPMS_EINVAL;
  int dev = 0, nsm = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  QG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  double *out = nullptr;
  QG_CUDA_TRY(cudaMalloc(&out, sizeof(double) * nsm * 8));
  cudaEvent_t e0, e1;
  QG_CUDA_TRY(cudaEventCreate(&e0));
  QG_CUDA_TRY(cudaEventCreate(&e1));
  const int iters = 1 << 14, blocks = nsm * 8;
  dfma_probe<<<blocks, 256>>>(out, 64, 0.999999, 1e-7);  // warm-up
  double best = 0;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    dfma_probe<<<blocks, 256>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    QG_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    double fl = 2.0 * 8 * (double)iters * blocks * 256;
    double t = fl / (ms * 1e-3) / 1e12;
    if (t > best) best = t;
  }
  g_launches.fetch_add(4);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  QG_CUDA_TRY(cudaGetLastError());
  *tflops = best;
  return QPMS_SUCCESS;
}
