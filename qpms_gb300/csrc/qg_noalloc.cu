// Allocation-free variant of the host-buffer translation entry point.
//
// Some callers cannot allocate GPU memory while they run: code that sits
// behind a strict device-memory budget or a pool allocator that owns all of
// the device's memory, real-time loops that forbid allocation after start-up,
// and plug-ins that must not change the memory footprint of the process that
// hosts them.  qpms_gpu_trans_AB_arrays_batch_host allocates device staging
// buffers (and pinned host buffers) on first use, so those callers cannot use
// it.  qpms_gpu_trans_AB_arrays_batch_host_noalloc computes the same A/B
// arrays with the same kernel, but stages inputs and outputs in a fixed
// file-scope device array instead.
//
// The array (kNoAllocScratchBytes = 32 MiB) is part of the library's device
// image: every GPU that loads the library holds it until the process exits.
// All calls share it and it keeps the contents of the last call; the kernel
// overwrites every output element, so nothing in it has to start at zero.
// Calls that overlap on the GPU (from several host threads or streams) race on
// the array, so callers must serialise them.
#include <cuda_runtime.h>
#include <string.h>

#include <mutex>

#include "qg_internal.h"

namespace qg {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_trans_scratch[kNoAllocScratchBytes];

std::mutex g_scratch_mutex;
void *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of g_trans_scratch on the current device.  Looked up once per
// device (with that device current); the host-side symbol itself is not a
// device address and must never be passed to a kernel.
int scratch_address(void **out) {
  int dev = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device index %d out of range", dev);
    return QPMS_EINVAL;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    QG_CUDA_TRY(cudaGetSymbolAddress(&p, g_trans_scratch));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return QPMS_SUCCESS;
}

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

}  // namespace
}  // namespace qg

using namespace qg;

extern "C" int qpms_gpu_trans_AB_arrays_batch_host_noalloc(const qpms_trans_calculator *c, size_t n,
                                                           const qpms_complex_t *kr, const double *theta,
                                                           const double *phi, const unsigned char *r_ge_d,
                                                           qpms_bessel_t J, qpms_complex_t *A, qpms_complex_t *B) {
  clear_error();
  if (!c) { set_error("calculator is NULL"); return QPMS_EINVAL; }
  if (J < 1 || J > 4) { set_error("invalid Bessel kind J=%d", J); return QPMS_EINVAL; }
  if (n == 0) return QPMS_SUCCESS;
  if (!kr || !theta || !phi || !A || !B) { set_error("NULL buffer"); return QPMS_EINVAL; }
  int e = check_calc_device(c);
  if (e) return e;
  const TransDevTables &T = priv(c)->dev;
  const size_t ne2 = (size_t)T.ne2;
  // per-translation bytes, padding included, bound n before any product with it can wrap
  const size_t per = 16 + 8 + 8 + (r_ge_d ? 1 : 0) + 2 * ne2 * 16;
  if (n > kNoAllocScratchBytes / per) {
    set_error("batch of %zu translations does not fit the allocation-free entry point's %zu bytes of scratch "
              "(at most about %zu translations at lMax %d)",
              n, kNoAllocScratchBytes, (kNoAllocScratchBytes - 64) / per, T.lMax);
    return QPMS_EINVAL;
  }
  const size_t in_bytes = align16(n * 16) + align16(n * 8) + align16(n * 8) + (r_ge_d ? align16(n) : 0);
  const size_t out_bytes = 2 * n * ne2 * 16;
  if (in_bytes + out_bytes > kNoAllocScratchBytes) {
    set_error("batch of %zu translations needs %zu bytes of scratch; the allocation-free entry point holds "
              "%zu bytes (at most about %zu translations at lMax %d)",
              n, in_bytes + out_bytes, kNoAllocScratchBytes, (kNoAllocScratchBytes - 64) / per, T.lMax);
    return QPMS_EINVAL;
  }
  void *base = nullptr;
  e = scratch_address(&base);
  if (e) return e;
  char *p = (char *)base;
  qg_c *dkr = (qg_c *)p;
  p += align16(n * 16);
  double *dth = (double *)p;
  p += align16(n * 8);
  double *dph = (double *)p;
  p += align16(n * 8);
  unsigned char *drg = nullptr;
  if (r_ge_d) {
    drg = (unsigned char *)p;
    p += align16(n);
  }
  qg_c *dA = (qg_c *)p, *dB = dA + n * ne2;
  // legacy default stream, synchronous copies from the caller's host memory
  QG_CUDA_TRY(cudaMemcpy(dkr, kr, n * 16, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dth, theta, n * 8, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dph, phi, n * 8, cudaMemcpyHostToDevice));
  if (drg) QG_CUDA_TRY(cudaMemcpy(drg, r_ge_d, n, cudaMemcpyHostToDevice));
  if ((e = launch_trans_ab(T, n, dkr, dth, dph, drg, J, dA, dB, 0, 0))) return e;
  QG_CUDA_TRY(cudaMemcpy(A, dA, n * ne2 * 16, cudaMemcpyDeviceToHost));
  QG_CUDA_TRY(cudaMemcpy(B, dB, n * ne2 * 16, cudaMemcpyDeviceToHost));
  return QPMS_SUCCESS;
}
