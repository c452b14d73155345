// C-ABI of the translation operator: qpms_trans_calculator_* drop-ins and the
// batched qpms_gpu_trans_AB_arrays_batch[_host] entry points.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <thread>

#include "qg_internal.h"

namespace qg {

static thread_local char t_err[512] = "";
std::atomic<unsigned long long> g_launches{0};
std::atomic<unsigned long long> g_graph_replays{0};

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_err, sizeof t_err, fmt, ap);
  va_end(ap);
}
void clear_error() { t_err[0] = 0; }

namespace {

template <typename T>
size_t upload(char *base, size_t off, const std::vector<T> &v, const T **dst) {
  off = (off + 255) & ~size_t(255);
  *dst = reinterpret_cast<const T *>(base + off);
  return off + v.size() * sizeof(T);
}

int upload_tables(TransCalcPriv *p) {
  const TransHostTables &h = p->host;
  size_t total = 0;
  auto add = [&](size_t bytes) { total = ((total + 255) & ~size_t(255)) + bytes; };
  add(h.perm.size() * 4);
  add(h.permB.size() * 4);
  add(h.cntA.size());
  add(h.cntB.size());
  add(h.cntBe.size());
  add(h.coefA.size() * 8);
  add(h.coefB.size() * 8);
  add(h.slotA.size() * 2);
  add(h.slotB.size() * 2);
  void *d = nullptr;
  QG_CUDA_TRY(cudaMalloc(&d, total));
  p->dev_block = d;
  std::vector<char> img(total, 0);
  char *hb = img.data();
  size_t off = 0;
  TransDevTables &T = p->dev;
  T.lMax = h.lMax;
  T.nelem = h.nelem;
  T.ne2 = h.nelem * h.nelem;
  T.tq = h.tq;
  auto put = [&](const void *src, size_t bytes) {
    off = (off + 255) & ~size_t(255);
    memcpy(hb + off, src, bytes);
    size_t o = off;
    off += bytes;
    return (char *)d + o;
  };
  T.perm = (const int32_t *)put(h.perm.data(), h.perm.size() * 4);
  T.permB = (const int32_t *)put(h.permB.data(), h.permB.size() * 4);
  T.cntA = (const uint8_t *)put(h.cntA.data(), h.cntA.size());
  T.cntB = (const uint8_t *)put(h.cntB.data(), h.cntB.size());
  T.cntBe = (const uint8_t *)put(h.cntBe.data(), h.cntBe.size());
  T.coefA = (const double *)put(h.coefA.data(), h.coefA.size() * 8);
  T.coefB = (const double *)put(h.coefB.data(), h.coefB.size() * 8);
  T.slotA = (const uint16_t *)put(h.slotA.data(), h.slotA.size() * 2);
  T.slotB = (const uint16_t *)put(h.slotB.data(), h.slotB.size() * 2);
  QG_CUDA_TRY(cudaMemcpy(d, hb, total, cudaMemcpyHostToDevice));
  return QPMS_SUCCESS;
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

int check_batch_args(const qpms_trans_calculator *c, const void *kr, const void *th, const void *ph, int J,
                     const void *A, const void *B) {
  if (!c) { set_error("calculator is NULL"); return QPMS_EINVAL; }
  if (J < 1 || J > 4) { set_error("invalid Bessel kind J=%d", J); return QPMS_EINVAL; }
  if (!kr || !th || !ph || !A || !B) { set_error("NULL buffer"); return QPMS_EINVAL; }
  if (!aligned16(kr) || !aligned16(A) || !aligned16(B)) {
    set_error("complex buffers must be 16-byte aligned");
    return QPMS_EINVAL;
  }
  return check_calc_device(c);
}

// Host-API staging: chunk of vectors processed per pipeline stage.
int ensure_staging(TransCalcPriv *p, size_t vecs) {
  if (p->stage_vecs >= vecs) return QPMS_SUCCESS;
  const size_t ne2 = (size_t)p->dev.ne2;
  const size_t in_bytes = vecs * (16 + 8 + 8 + 16);  // kr, theta, phi, r_ge_d (padded)
  const size_t out_bytes = vecs * ne2 * 16 * 2;
  if (p->pin_in) cudaFreeHost(p->pin_in);
  if (p->pin_out) cudaFreeHost(p->pin_out);
  if (p->dev_in) cudaFree(p->dev_in);
  if (p->dev_out) cudaFree(p->dev_out);
  p->pin_in = p->pin_out = p->dev_in = p->dev_out = nullptr;
  p->stage_vecs = 0;
  QG_CUDA_TRY(cudaHostAlloc(&p->pin_in, 2 * in_bytes, cudaHostAllocDefault));
  QG_CUDA_TRY(cudaHostAlloc(&p->pin_out, 2 * out_bytes, cudaHostAllocDefault));
  QG_CUDA_TRY(cudaMalloc(&p->dev_in, 2 * in_bytes));
  QG_CUDA_TRY(cudaMalloc(&p->dev_out, 2 * out_bytes));
  for (int s = 0; s < 2; ++s) {
    if (!p->streams[s]) QG_CUDA_TRY(cudaStreamCreateWithFlags(&p->streams[s], cudaStreamNonBlocking));
    if (!p->ev[s]) QG_CUDA_TRY(cudaEventCreateWithFlags(&p->ev[s], cudaEventDisableTiming));
  }
  p->stage_vecs = vecs;
  return QPMS_SUCCESS;
}

bool is_pinned(const void *ptr) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// Parallel memcpy for pageable <-> pinned staging.
void par_memcpy(void *dst, const void *src, size_t bytes) {
  const size_t kMin = size_t(8) << 20;
  unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if (bytes < kMin || nt == 1) {
    memcpy(dst, src, bytes);
    return;
  }
  std::vector<std::thread> th;
  size_t per = (bytes + nt - 1) / nt;
  for (unsigned t = 0; t < nt; ++t) {
    size_t o = t * per;
    if (o >= bytes) break;
    size_t b = std::min(per, bytes - o);
    th.emplace_back([=] { memcpy((char *)dst + o, (const char *)src + o, b); });
  }
  for (auto &x : th) x.join();
}

}  // namespace

int check_calc_device(const qpms_trans_calculator *c) {
  int dev = -1;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != priv(c)->device) {
    set_error("the calculator's tables live on device %d but device %d is current; make device %d current "
              "before calling", priv(c)->device, dev, priv(c)->device);
    return QPMS_EINVAL;
  }
  return QPMS_SUCCESS;
}

}  // namespace qg

using namespace qg;

extern "C" {

const char *qpms_gpu_last_error(void) { return qg::t_err; }
unsigned long long qpms_gpu_kernel_launch_count(void) { return qg::g_launches.load(); }
unsigned long long qpms_gpu_graph_replay_count(void) { return qg::g_graph_replays.load(); }

qpms_trans_calculator *qpms_trans_calculator_init(qpms_l_t lMax, qpms_normalisation_t nt) {
  clear_error();
  TransCalcPriv *p = new (std::nothrow) TransCalcPriv();
  if (!p) { set_error("out of host memory"); return nullptr; }
  if (!build_trans_tables(lMax, nt, &p->host)) {
    set_error("unsupported lMax %d or normalisation %#x", lMax, nt);
    delete p;
    return nullptr;
  }
  if (cudaGetDevice(&p->device) != cudaSuccess || upload_tables(p) != QPMS_SUCCESS) {
    if (!qg::t_err[0]) set_error("no CUDA device");
    if (p->dev_block) cudaFree(p->dev_block);
    delete p;
    return nullptr;
  }
  TransHostTables &h = p->host;
  const size_t ne2 = (size_t)h.nelem * h.nelem;
  p->pub.normalisation = nt;
  p->pub.lMax = lMax;
  p->pub.nelem = h.nelem;
  p->pub.A_multipliers = (qpms_complex_t **)malloc((ne2 + 1) * sizeof(qpms_complex_t *));
  p->pub.B_multipliers = (qpms_complex_t **)malloc((ne2 + 1) * sizeof(qpms_complex_t *));
  for (size_t i = 0; i <= ne2; ++i) {
    p->pub.A_multipliers[i] = (qpms_complex_t *)(h.A_mult.data() + h.A_off[i]);
    p->pub.B_multipliers[i] = (qpms_complex_t *)(h.B_mult.data() + h.B_off[i]);
  }
  p->pub.e3c = nullptr;
  p->pub.legendre0 = nullptr;
  return &p->pub;
}

void qpms_trans_calculator_free(qpms_trans_calculator *c) {
  if (!c) return;
  TransCalcPriv *p = priv(c);
  free(p->pub.A_multipliers);
  free(p->pub.B_multipliers);
  if (p->dev_block) cudaFree(p->dev_block);
  if (p->pin_in) cudaFreeHost(p->pin_in);
  if (p->pin_out) cudaFreeHost(p->pin_out);
  if (p->dev_in) cudaFree(p->dev_in);
  if (p->dev_out) cudaFree(p->dev_out);
  for (int s = 0; s < 2; ++s) {
    if (p->streams[s]) cudaStreamDestroy(p->streams[s]);
    if (p->ev[s]) cudaEventDestroy(p->ev[s]);
  }
  delete p;
}

int qpms_gpu_testing_set_calculator_device(qpms_trans_calculator *c, int device) {
  if (!c) return QPMS_EINVAL;
  priv(c)->device = device;
  return QPMS_SUCCESS;
}

size_t qpms_gpu_trans_calculator_n_multipliers(const qpms_trans_calculator *c, int which_B) {
  const TransCalcPriv *p = priv(c);
  return which_B ? p->host.B_mult.size() : p->host.A_mult.size();
}

int qpms_gpu_trans_AB_arrays_batch(const qpms_trans_calculator *c, size_t n, const qpms_complex_t *kr,
                                   const double *theta, const double *phi, const unsigned char *r_ge_d,
                                   qpms_bessel_t J, qpms_complex_t *A, qpms_complex_t *B, void *stream) {
  clear_error();
  int e = check_batch_args(c, kr, theta, phi, J, A, B);
  if (e) return e;
  const char *v = getenv("QPMS_GB300_TRANS_VARIANT");
  int variant = v ? atoi(v) : 0;
  return launch_trans_ab(priv(c)->dev, n, (const qg_c *)kr, theta, phi, r_ge_d, J, (qg_c *)A, (qg_c *)B,
                         (cudaStream_t)stream, variant);
}

int qpms_gpu_trans_AB_arrays_batch_host(const qpms_trans_calculator *c, size_t n, const qpms_complex_t *kr,
                                        const double *theta, const double *phi, const unsigned char *r_ge_d,
                                        qpms_bessel_t J, qpms_complex_t *A, qpms_complex_t *B) {
  clear_error();
  int e = check_batch_args(c, kr, theta, phi, J, A, B);
  if (e) return e;
  if (n == 0) return QPMS_SUCCESS;
  TransCalcPriv *p = priv(c);
  const size_t ne2 = (size_t)p->dev.ne2;
  // ~64 MiB of output per chunk and stream
  size_t chunk = std::max<size_t>(1, (size_t(64) << 20) / (ne2 * 32));
  chunk = std::min(chunk, n);
  if ((e = ensure_staging(p, chunk))) return e;
  const bool in_pinned = is_pinned(kr) && is_pinned(theta) && is_pinned(phi) && (!r_ge_d || is_pinned(r_ge_d));
  const bool out_pinned = is_pinned(A) && is_pinned(B);
  const size_t in_stride = p->stage_vecs * (16 + 8 + 8 + 16);
  const size_t out_stride = p->stage_vecs * ne2 * 32;
  const size_t nch = (n + chunk - 1) / chunk;
  const char *vv = getenv("QPMS_GB300_TRANS_VARIANT");
  const int variant = vv ? atoi(vv) : 0;
  // pipeline: chunk i on stream i%2; pageable outputs are drained one chunk behind
  for (size_t i = 0; i <= nch; ++i) {
    if (i < nch) {
      const int s = (int)(i & 1);
      cudaStream_t st = p->streams[s];
      QG_CUDA_TRY(cudaEventSynchronize(p->ev[s]));  // buffers of chunk i-2 are free
      if (i >= 2 && !out_pinned) {
        // drain chunk i-2 (same buffers) into the caller's pageable arrays
        const size_t j = i - 2, o = j * chunk, m = std::min(chunk, n - o);
        char *po = (char *)p->pin_out + s * out_stride;
        par_memcpy(A + o * ne2, po, m * ne2 * 16);
        par_memcpy(B + o * ne2, po + m * ne2 * 16, m * ne2 * 16);
      }
      const size_t o = i * chunk, m = std::min(chunk, n - o);
      char *di = (char *)p->dev_in + s * in_stride;
      qg_c *dkr = (qg_c *)di;
      double *dth = (double *)(di + m * 16), *dph = dth + m;
      unsigned char *drg = r_ge_d ? (unsigned char *)(dph + m) : nullptr;
      if (in_pinned) {
        QG_CUDA_TRY(cudaMemcpyAsync(dkr, kr + o, m * 16, cudaMemcpyHostToDevice, st));
        QG_CUDA_TRY(cudaMemcpyAsync(dth, theta + o, m * 8, cudaMemcpyHostToDevice, st));
        QG_CUDA_TRY(cudaMemcpyAsync(dph, phi + o, m * 8, cudaMemcpyHostToDevice, st));
        if (drg) QG_CUDA_TRY(cudaMemcpyAsync(drg, r_ge_d + o, m, cudaMemcpyHostToDevice, st));
      } else {
        char *pi = (char *)p->pin_in + s * in_stride;
        memcpy(pi, kr + o, m * 16);
        memcpy(pi + m * 16, theta + o, m * 8);
        memcpy(pi + m * 24, phi + o, m * 8);
        if (drg) memcpy(pi + m * 32, r_ge_d + o, m);
        QG_CUDA_TRY(cudaMemcpyAsync(di, pi, m * 32 + (drg ? m : 0), cudaMemcpyHostToDevice, st));
      }
      qg_c *dA = (qg_c *)((char *)p->dev_out + s * out_stride), *dB = dA + m * ne2;
      if ((e = launch_trans_ab(p->dev, m, dkr, dth, dph, drg, J, dA, dB, st, variant))) return e;
      if (out_pinned) {
        QG_CUDA_TRY(cudaMemcpyAsync(A + o * ne2, dA, m * ne2 * 16, cudaMemcpyDeviceToHost, st));
        QG_CUDA_TRY(cudaMemcpyAsync(B + o * ne2, dB, m * ne2 * 16, cudaMemcpyDeviceToHost, st));
      } else {
        char *po = (char *)p->pin_out + s * out_stride;
        QG_CUDA_TRY(cudaMemcpyAsync(po, dA, m * ne2 * 32, cudaMemcpyDeviceToHost, st));
      }
      QG_CUDA_TRY(cudaEventRecord(p->ev[s], st));
    }
  }
  // drain the last two chunks
  for (size_t j = (nch >= 2 ? nch - 2 : 0); j < nch; ++j) {
    const int s = (int)(j & 1);
    QG_CUDA_TRY(cudaEventSynchronize(p->ev[s]));
    if (!out_pinned) {
      const size_t o = j * chunk, m = std::min(chunk, n - o);
      char *po = (char *)p->pin_out + s * out_stride;
      par_memcpy(A + o * ne2, po, m * ne2 * 16);
      par_memcpy(B + o * ne2, po + m * ne2 * 16, m * ne2 * 16);
    }
  }
  return QPMS_SUCCESS;
}

int qpms_trans_calculator_get_AB_arrays_ext(const qpms_trans_calculator *c, qpms_complex_t *Adest,
                                            qpms_complex_t *Bdest, size_t deststride, size_t srcstride,
                                            qpms_complex_t kdlj_r, double kdlj_theta, double kdlj_phi, int r_ge_d,
                                            int J) {
  clear_error();
  if (!c || !Adest || !Bdest) { set_error("NULL argument"); return QPMS_EINVAL; }
  const size_t ne = c->nelem, ne2 = ne * ne;
  std::vector<qg_c> buf(2 * ne2);
  alignas(16) qpms_complex_t kr = kdlj_r;
  unsigned char rg = r_ge_d ? 1 : 0;
  int e = qpms_gpu_trans_AB_arrays_batch_host(c, 1, &kr, &kdlj_theta, &kdlj_phi, &rg, J,
                                              (qpms_complex_t *)buf.data(), (qpms_complex_t *)(buf.data() + ne2));
  if (e) return e;
  for (size_t y = 0; y < ne; ++y)
    for (size_t yu = 0; yu < ne; ++yu) {
      ((qg_c *)Adest)[deststride * y + srcstride * yu] = buf[y * ne + yu];
      ((qg_c *)Bdest)[deststride * y + srcstride * yu] = buf[ne2 + y * ne + yu];
    }
  return QPMS_SUCCESS;
}

int qpms_trans_calculator_get_AB_arrays(const qpms_trans_calculator *c, qpms_complex_t *Adest,
                                        qpms_complex_t *Bdest, size_t deststride, size_t srcstride, csph_t kdlj,
                                        bool r_ge_d, qpms_bessel_t J) {
  return qpms_trans_calculator_get_AB_arrays_ext(c, Adest, Bdest, deststride, srcstride, kdlj.r, kdlj.theta,
                                                 kdlj.phi, r_ge_d ? 1 : 0, J);
}

int qpms_trans_calculator_get_trans_array(const qpms_trans_calculator *c, qpms_complex_t *target,
                                          const qpms_vswf_set_spec_t *destspec, size_t deststride,
                                          const qpms_vswf_set_spec_t *srcspec, size_t srcstride, csph_t kdlj,
                                          bool r_ge_d, qpms_bessel_t J) {
  clear_error();
  if (!c || !target || !destspec || !srcspec) {
    set_error("NULL argument");
    return QPMS_EINVAL;
  }
  if (destspec->norm != c->normalisation || srcspec->norm != c->normalisation || destspec->lMax > c->lMax ||
      srcspec->lMax > c->lMax || destspec->lMax_L >= 0 || srcspec->lMax_L >= 0) {
    set_error("VSWF sets must share the calculator's normalisation, lMax <= %d, no longitudinal waves", c->lMax);
    return QPMS_EINVAL;
  }
  const size_t ne = c->nelem;
  std::vector<qpms_complex_t> A(ne * ne), B(ne * ne);
  const int rc = qpms_trans_calculator_get_AB_arrays(c, A.data(), B.data(), ne, 1, kdlj, r_ge_d, J);
  if (rc) return rc;
  // qpms_trans_array_from_AB (translations_inlines.h:8-35); u = 4 (y + 1) + type (indexing.h:83-90)
  for (size_t di = 0; di < destspec->n; ++di) {
    const qpms_uvswfi_t ud = destspec->ilist[di];
    const unsigned td = (unsigned)(ud & 3);
    const long long yd = (long long)(ud / 4) - 1;
    if (td == 0 || td == 3 || yd < 0 || (size_t)yd >= ne) {
      set_error("invalid VSWF index %llx", (unsigned long long)ud);
      return QPMS_EINVAL;
    }
    for (size_t si = 0; si < srcspec->n; ++si) {
      const qpms_uvswfi_t us = srcspec->ilist[si];
      const unsigned ts = (unsigned)(us & 3);
      const long long ys = (long long)(us / 4) - 1;
      if (ts == 0 || ts == 3 || ys < 0 || (size_t)ys >= ne) {
        set_error("invalid VSWF index %llx", (unsigned long long)us);
        return QPMS_EINVAL;
      }
      target[si * srcstride + di * deststride] = (ts == td) ? A[yd * ne + ys] : B[yd * ne + ys];
    }
  }
  return QPMS_SUCCESS;
}

int qpms_trans_calculator_get_trans_array_lc3p(const qpms_trans_calculator *c, qpms_complex_t *target,
                                               const qpms_vswf_set_spec_t *destspec, size_t deststride,
                                               const qpms_vswf_set_spec_t *srcspec, size_t srcstride,
                                               qpms_complex_t k, cart3_t destpos, cart3_t srcpos, qpms_bessel_t J) {
  // cart2csph (vectors.h:359-365) of destpos - srcpos, then r *= k
  const double x = destpos.x - srcpos.x, y = destpos.y - srcpos.y, z = destpos.z - srcpos.z;
  const double r = sqrt(x * x + y * y + z * z);
  csph_t kd;
  kd.r.re = r * k.re;
  kd.r.im = r * k.im;
  kd.theta = r ? acos(z / r) : M_PI_2;
  kd.phi = atan2(y, x);
  return qpms_trans_calculator_get_trans_array(c, target, destspec, deststride, srcspec, srcstride, kd, false, J);
}

}  // extern "C"

extern "C" int qpms_gpu_trans_multipliers_export(qpms_l_t lMax, qpms_normalisation_t nt, qpms_complex_t *A_out,
                                                 size_t *nA, qpms_complex_t *B_out, size_t *nB) {
  clear_error();
  TransHostTables h;
  if (!build_trans_tables(lMax, nt, &h)) {
    set_error("unsupported lMax %d or normalisation %#x", lMax, nt);
    return QPMS_EINVAL;
  }
  if (!nA || !nB) { set_error("NULL size pointer"); return QPMS_EINVAL; }
  const size_t capA = *nA, capB = *nB;
  *nA = h.A_mult.size();
  *nB = h.B_mult.size();
  if (!A_out || !B_out) return QPMS_SUCCESS;
  if (capA < h.A_mult.size() || capB < h.B_mult.size()) { set_error("output too small"); return QPMS_EINVAL; }
  memcpy(A_out, h.A_mult.data(), h.A_mult.size() * 16);
  memcpy(B_out, h.B_mult.data(), h.B_mult.size() * 16);
  return QPMS_SUCCESS;
}
