// Live per-kind kernel timing for measurements: when enabled, launch sites of
// the main kernels record a CUDA event pair on the stream they launch on and
// the work of the launch (flops or bytes); qpms_gpu_kernel_timing_get sums the
// elapsed times.  Off by default (one relaxed atomic load per launch).
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "qg_internal.h"
#include "qg_ktimer.h"

namespace qg {
namespace {

struct Entry {
  int kind;
  cudaEvent_t a, b;
  double work;
};

std::atomic<bool> g_on{false};
std::mutex g_mu;
std::vector<Entry> g_pending;
double g_ms[KT_KINDS], g_work[KT_KINDS];
unsigned long long g_count[KT_KINDS];

void drain_locked() {
  for (Entry &e : g_pending) {
    float ms = 0;
    if (cudaEventSynchronize(e.b) == cudaSuccess && cudaEventElapsedTime(&ms, e.a, e.b) == cudaSuccess) {
      g_ms[e.kind] += ms;
      g_work[e.kind] += e.work;
      g_count[e.kind] += 1;
    }
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  g_pending.clear();
}

}  // namespace

bool kt_on() { return g_on.load(std::memory_order_relaxed); }

KtScope::KtScope(int kind, cudaStream_t st, double work) : kind_(kind), st_(st), work_(work) {
  if (!g_on.load(std::memory_order_relaxed) || kind < 0 || kind >= KT_KINDS) return;
  if (cudaEventCreate(&a_) != cudaSuccess) return;
  if (cudaEventCreate(&b_) != cudaSuccess) {
    cudaEventDestroy(a_);
    return;
  }
  cudaEventRecord(a_, st_);
  active_ = true;
}

KtScope::~KtScope() {
  if (!active_) return;
  cudaEventRecord(b_, st_);
  std::lock_guard<std::mutex> lk(g_mu);
  g_pending.push_back({kind_, a_, b_, work_});
}

}  // namespace qg

using namespace qg;

extern "C" int qpms_gpu_kernel_timing(int enable) {
  std::lock_guard<std::mutex> lk(g_mu);
  drain_locked();
  for (int k = 0; k < KT_KINDS; ++k) g_ms[k] = g_work[k] = 0, g_count[k] = 0;
  g_on.store(enable != 0);
  return QPMS_SUCCESS;
}

extern "C" int qpms_gpu_kernel_timing_get(int kind, double *ms, double *work, unsigned long long *launches) {
  if (kind < 0 || kind >= KT_KINDS) return QPMS_EINVAL;
  std::lock_guard<std::mutex> lk(g_mu);
  drain_locked();
  if (ms) *ms = g_ms[kind];
  if (work) *work = g_work[kind];
  if (launches) *launches = g_count[kind];
  return QPMS_SUCCESS;
}
