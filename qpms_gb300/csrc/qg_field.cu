// Scattered-field evaluation of a finite system,
//
//   E(r) = sum_p sum_{l,m} ( f_N[p](l,m) N_lm^{(J)}(k (r - r_p)) + f_M[p](l,m) M_lm^{(J)}(k (r - r_p)) ),
//
// in cartesian components: qpms_scatsys_scattered_E (scatsystem.c:2013-2039),
// i.e. per particle kr = k * cart2sph(where - pos) (vectors.h:134-140), the
// VSWFs of qpms_vswf_fill_csph (vswf.c:230-288) summed with the particle's
// coefficients (qpms_eval_vswf_csph, vswf.c:533-560) and turned to cartesian
// components by csphvec2ccart (vectors.h:272-303).  Default normalisation
// (qpms_types.h:167): Condon-Shortley phase, e^{i m phi}, factors 1.
//
// Layout: one thread per evaluation point, all threads of a block walk the
// same particles, so positions and coefficient vectors are warp-uniform loads
// (L1 broadcasts).  grid.y splits the particle list when the points alone do
// not fill the GPU; the partial sums [split][point][3] are then added in a
// fixed order by a second kernel, so the result does not depend on timing.
//
// Per (point, particle) pair: one complex reciprocal, the Hankel/Bessel
// recurrence (L + 1 orders), the normalised Legendre recurrence in l for all m
// at once (registers), and per (l, |m|) four complex products with the
// coefficients.  The work is FP64 arithmetic on data that stays in L1/L2: the
// kernel is bound by the FP64 pipe, not by HBM.
#include <math.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "qg_internal.h"
#include "qg_specfunc.cuh"

namespace qg {
bool scatsys_is_own(const qpms_scatsys_t *ss);
int scatsys_lmax(const qpms_scatsys_t *ss);

namespace {

constexpr int kFieldLMax = 8;
constexpr int kFieldThreads = 128;
constexpr int kFieldT = (kFieldLMax + 1) * (kFieldLMax + 2) / 2;  // (l, m >= 0) pairs

// Normalised associated Legendre recurrences (GSL_SF_LEGENDRE_SPHARM with the
// Condon-Shortley phase), index t = l (l + 1) / 2 + m:
//   Pbar_m^m     = mm[m] sin(theta) Pbar_{m-1}^{m-1},   mm[m] = -sqrt((2m+1)/(2m))
//   Pbar_{m+1}^m = sub[m] x Pbar_m^m,                   sub[m] = sqrt(2m+3)
//   Pbar_l^m     = a[t] (x Pbar_{l-1}^m - b[t] Pbar_{l-2}^m)
//   (x^2 - 1) dPbar_l^m/dx = l x Pbar_l^m - e[t] Pbar_{l-1}^m,  e = sqrt((2l+1)(l^2-m^2)/(2l-1))
// il[l] = 1/sqrt(l(l+1)) is the power-normalisation factor (legendre.c:65-117).
struct FieldTables {
  double y00;
  double mm[kFieldLMax + 1], sub[kFieldLMax + 1], il[kFieldLMax + 1];
  double a[kFieldT], b[kFieldT], e[kFieldT];
  double pole_leg[kFieldLMax + 1], pole_f[kFieldLMax + 1];
};

struct FieldArgs {
  int npts, np, chunk, J;
  qg_c k;
  const double *where;  // [npts][3]
  const double *pos;    // [np][3]
  const qg_c *cvf;      // [np][2 nelem]: electric block, then magnetic
  qg_c *out;            // [split][npts][3]
  FieldTables tb;
};

const FieldTables &field_tables() {
  static FieldTables t;
  static std::once_flag once;
  std::call_once(once, [] {
    memset(&t, 0, sizeof t);
    typedef long double ld;
    t.y00 = (double)(1.0L / sqrtl(4.0L * 3.14159265358979323846264338327950288L));
    for (int m = 1; m <= kFieldLMax; ++m) t.mm[m] = (double)(-sqrtl((2.0L * m + 1) / (2.0L * m)));
    for (int m = 0; m <= kFieldLMax; ++m) t.sub[m] = (double)sqrtl(2.0L * m + 3);
    for (int l = 1; l <= kFieldLMax; ++l) {
      t.il[l] = (double)(1.0L / sqrtl((ld)l * (l + 1)));
      const ld pi_l = 3.14159265358979323846264338327950288L;
      t.pole_leg[l] = (double)sqrtl((2.0L * l + 1) / (4 * pi_l * l * (l + 1)));
      t.pole_f[l] = (double)(0.25L * sqrtl((2.0L * l + 1) / pi_l));
      for (int m = 0; m <= l; ++m) {
        const int ti = l * (l + 1) / 2 + m;
        const ld L2 = (ld)l * l, M2 = (ld)m * m;
        if (l >= m + 2) {
          t.a[ti] = (double)sqrtl((4 * L2 - 1) / (L2 - M2));
          t.b[ti] = (double)sqrtl((((ld)l - 1) * (l - 1) - M2) / (4 * ((ld)l - 1) * (l - 1) - 1));
        }
        t.e[ti] = (double)sqrtl((2.0L * l + 1) * (L2 - M2) / (2.0L * l - 1));
      }
    }
  });
  return t;
}

__device__ __forceinline__ qg_c ldg_c(const qg_c *p) {
  const double2 v = __ldg(reinterpret_cast<const double2 *>(p));
  return cmk(v.x, v.y);
}

template <int L>
__global__ void __launch_bounds__(kFieldThreads) scattered_field_kernel(const FieldArgs a) {
  constexpr int NE = L * (L + 2);
  const int q = blockIdx.x * kFieldThreads + threadIdx.x;
  if (q >= a.npts) return;
  const double wx = a.where[3 * q], wy = a.where[3 * q + 1], wz = a.where[3 * q + 2];
  const int p0 = blockIdx.y * a.chunk;
  const int p1 = min(a.np, p0 + a.chunk);
  qg_c Ex = cmk(0, 0), Ey = cmk(0, 0), Ez = cmk(0, 0);
  for (int p = p0; p < p1; ++p) {
    const double dx = wx - __ldg(a.pos + 3 * p), dy = wy - __ldg(a.pos + 3 * p + 1),
                 dz = wz - __ldg(a.pos + 3 * p + 2);
    const double rho2 = dx * dx + dy * dy;
    const double r = sqrt(rho2 + dz * dz);
    // cart2sph: theta = pi/2, phi = atan2(0, 0) = 0 at r = 0
    double ct = 0.0, st = 1.0, cf = 1.0, sf = 0.0;
    if (r > 0.0) {
      // true divisions: z / r is exactly +-1 on the polar axis, which selects
      // the |cos theta| = 1 branch as acos/cos do in the reference
      const double rho = sqrt(rho2);
      ct = dz / r;
      st = rho / r;
      if (rho > 0.0) {
        const double ir = 1.0 / rho;
        cf = dx * ir;
        sf = dy * ir;
      }
    }
    const bool pole = (fabs(ct) == 1.0);  // legendre.c:72-86 branch
    const qg_c kr = cscale(a.k, r);
    qg_c z[L + 1];
    if (a.J == 3) {  // h+_l by forward recurrence from h_0, h_1 (real or complex kr)
      const qg_c ri = crecip(kr);
      const qg_c ex = cexpi(kr);
      const qg_c h0 = cmul(cmk(0.0, -1.0), cmul(ex, ri));
      const qg_c h1 = cscale(cmul(cmul(ex, cadd(kr, cmk(0.0, 1.0))), cmul(ri, ri)), -1.0);
      sph_forward<L>(ri, h0, h1, z);
    } else {
      sph_bessel<L>(a.J, kr, z);
    }
    const qg_c rkr = (r > 0.0) ? crecip(kr) : cmk(0, 0);
    // e^{i m phi}, m = 0..L
    qg_c em[L + 1];
    em[0] = cmk(1.0, 0.0);
#pragma unroll
    for (int m = 1; m <= L; ++m) em[m] = cmul(em[m - 1], cmk(cf, sf));
    const double ist = pole ? 0.0 : 1.0 / st;
    const qg_c *cv = a.cvf + (size_t)p * 2 * NE;
    double P1[L + 1], P2[L + 1];  // Pbar_{l-1}^m, Pbar_{l-2}^m
#pragma unroll
    for (int m = 0; m <= L; ++m) P1[m] = P2[m] = 0.0;
    P1[0] = a.tb.y00;
    qg_c sr = cmk(0, 0), sth = cmk(0, 0), sph = cmk(0, 0);
#pragma unroll
    for (int l = 1; l <= L; ++l) {
      qg_c R = cmk(0, 0), T = cmk(0, 0), Pp = cmk(0, 0), TM = cmk(0, 0), PM = cmk(0, 0);
      double Pc[L + 1];
#pragma unroll
      for (int m = 0; m <= l; ++m) {
        const int ti = l * (l + 1) / 2 + m;
        double Pl;
        if (m == l) Pl = a.tb.mm[l] * st * P1[l - 1];
        else if (m == l - 1) Pl = a.tb.sub[m] * ct * P1[m];
        else Pl = a.tb.a[ti] * (ct * P1[m] - a.tb.b[ti] * P2[m]);
        Pc[m] = Pl;
        double leg, pi, tau;
        if (!pole) {
          const double Pm1 = (m <= l - 1) ? P1[m] : 0.0;
          leg = Pl * a.tb.il[l];
          pi = m * leg * ist;
          tau = (l * ct * Pl - a.tb.e[ti] * Pm1) * a.tb.il[l] * ist;
        } else {
          const double lpar = (l & 1) ? -1.0 : 1.0;
          leg = (m == 0) ? ((l & 1) ? ct : 1.0) * a.tb.pole_leg[l] : 0.0;
          pi = (m == 1) ? ((ct > 0) ? -1.0 : lpar) * a.tb.pole_f[l] : 0.0;
          tau = (m == 1) ? -((ct > 0) ? 1.0 : lpar) * a.tb.pole_f[l] : 0.0;
        }
        const int yp = l * (l + 1) + m - 1;
        const qg_c SNp = cmul(ldg_c(cv + yp), em[m]);
        const qg_c SMp = cmul(ldg_c(cv + NE + yp), em[m]);
        if (m == 0) {
          R = cadd(R, cscale(SNp, leg));
          T = cadd(T, cscale(SNp, tau));
          PM = cadd(PM, cscale(SMp, tau));
        } else {
          const int ym = l * (l + 1) - m - 1;
          const double sg = (m & 1) ? -1.0 : 1.0;
          const qg_c SNm = cscale(cmul(ldg_c(cv + ym), cconj(em[m])), sg);
          const qg_c SMm = cscale(cmul(ldg_c(cv + NE + ym), cconj(em[m])), sg);
          // y(l, -m): leg, tau times (-1)^m, pi times -(-1)^m
          const qg_c U = cadd(SNp, SNm), V = csub(SNp, SNm), W = csub(SMp, SMm), X = cadd(SMp, SMm);
          R = cadd(R, cscale(U, leg));
          T = cadd(T, cscale(U, tau));
          Pp = cadd(Pp, cscale(V, pi));
          TM = cadd(TM, cscale(W, pi));
          PM = cadd(PM, cscale(X, tau));
        }
      }
#pragma unroll
      for (int m = 0; m <= L; ++m) {
        P2[m] = P1[m];
        P1[m] = (m <= l) ? Pc[m] : 0.0;
      }
      // qpms_vswf_fill_csph: besfac = z_l / kr (1/3 for l = 1 at r = 0), besderfac = z_{l-1} - l besfac
      const qg_c besfac = (r > 0.0) ? cmul(z[l], rkr) : cmk((l == 1) ? 1.0 / 3.0 : 0.0, 0.0);
      const qg_c besder = csub(z[l - 1], cscale(besfac, (double)l));
      const qg_c iPp = cmk(-Pp.im, Pp.re), iTM = cmk(-TM.im, TM.re);  // the i of d(e^{im phi})/dphi / m
      sr = cadd(sr, cscale(cmul(besfac, R), (double)(l * (l + 1))));
      sth = cadd(sth, cadd(cmul(besder, T), cmul(z[l], iTM)));
      sph = cadd(sph, csub(cmul(besder, iPp), cmul(z[l], PM)));
    }
    // csphvec2ccart
    Ex = cadd(Ex, cadd(cadd(cscale(sr, st * cf), cscale(sth, ct * cf)), cscale(sph, -sf)));
    Ey = cadd(Ey, cadd(cadd(cscale(sr, st * sf), cscale(sth, ct * sf)), cscale(sph, cf)));
    Ez = cadd(Ez, csub(cscale(sr, ct), cscale(sth, st)));
  }
  qg_c *o = a.out + ((size_t)blockIdx.y * a.npts + q) * 3;
  o[0] = Ex;
  o[1] = Ey;
  o[2] = Ez;
}

// out[q][c] = sum over s of part[s][q][c], s in increasing order.
__global__ void field_reduce_kernel(const qg_c *__restrict__ part, int nsplit, size_t n, qg_c *__restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  qg_c s = part[i];
  for (int j = 1; j < nsplit; ++j) s = cadd(s, part[(size_t)j * n + i]);
  out[i] = s;
}

// Resident blocks of the lMax kernel on the whole device (one wave).
template <int L>
long field_wave_L() {
  int dev = 0, nsm = 152, per = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, scattered_field_kernel<L>, kFieldThreads, 0) !=
          cudaSuccess ||
      per < 1) {
    cudaGetLastError();
    per = 1;
  }
  return (long)nsm * per;
}

long field_wave(int lMax) {
  switch (lMax) {
    case 1: return field_wave_L<1>();
    case 2: return field_wave_L<2>();
    case 3: return field_wave_L<3>();
    case 4: return field_wave_L<4>();
    case 5: return field_wave_L<5>();
    case 6: return field_wave_L<6>();
    case 7: return field_wave_L<7>();
    default: return field_wave_L<8>();
  }
}

template <int L>
cudaError_t launch_field_L(const FieldArgs &a, int nsplit, cudaStream_t st) {
  dim3 grid((a.npts + kFieldThreads - 1) / kFieldThreads, nsplit);
  scattered_field_kernel<L><<<grid, kFieldThreads, 0, st>>>(a);
  g_launches.fetch_add(1);
  return cudaGetLastError();
}

cudaError_t launch_field(int lMax, const FieldArgs &a, int nsplit, cudaStream_t st) {
  switch (lMax) {
    case 1: return launch_field_L<1>(a, nsplit, st);
    case 2: return launch_field_L<2>(a, nsplit, st);
    case 3: return launch_field_L<3>(a, nsplit, st);
    case 4: return launch_field_L<4>(a, nsplit, st);
    case 5: return launch_field_L<5>(a, nsplit, st);
    case 6: return launch_field_L<6>(a, nsplit, st);
    case 7: return launch_field_L<7>(a, nsplit, st);
    case 8: return launch_field_L<8>(a, nsplit, st);
    default: return cudaErrorInvalidValue;
  }
}

// Device positions of a system, uploaded once and kept with it.
struct PosCache {
  std::mutex mu;
  std::vector<std::pair<const qpms_scatsys_t *, std::pair<int, double *>>> v;  // ss -> (device, buffer)
};
PosCache &pos_cache() {
  static PosCache *c = new PosCache;
  return *c;
}

}  // namespace

// Forgets the device positions of a freed system.
void field_forget_system(const qpms_scatsys_t *ss) {
  PosCache &c = pos_cache();
  std::lock_guard<std::mutex> g(c.mu);
  for (size_t i = 0; i < c.v.size();) {
    if (c.v[i].first == ss) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaSetDevice(c.v[i].second.first);
      cudaFree(c.v[i].second.second);
      cudaSetDevice(dev);
      c.v.erase(c.v.begin() + i);
    } else {
      ++i;
    }
  }
}

namespace {
int device_positions(const qpms_scatsys_t *ss, const double **out) {
  int dev = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  PosCache &c = pos_cache();
  std::lock_guard<std::mutex> g(c.mu);
  for (auto &e : c.v)
    if (e.first == ss && e.second.first == dev) {
      *out = e.second.second;
      return QPMS_SUCCESS;
    }
  std::vector<double> h(3 * (size_t)ss->p_count);
  for (int i = 0; i < ss->p_count; ++i) {
    h[3 * i] = ss->p[i].pos.x;
    h[3 * i + 1] = ss->p[i].pos.y;
    h[3 * i + 2] = ss->p[i].pos.z;
  }
  double *d = nullptr;
  QG_CUDA_TRY(cudaMalloc(&d, h.size() * 8));
  QG_CUDA_TRY(cudaMemcpy(d, h.data(), h.size() * 8, cudaMemcpyHostToDevice));
  c.v.push_back({ss, {dev, d}});
  *out = d;
  return QPMS_SUCCESS;
}

int field_device(const qpms_scatsys_t *ss, int btyp, qg_c k, const qg_c *d_cvf, size_t npoints,
                 const double *d_where, qg_c *d_E, cudaStream_t st) {
  if (!ss || !d_cvf || !d_where || !d_E) { set_error("NULL argument"); return QPMS_EINVAL; }
  if (!scatsys_is_own(ss)) { set_error("system not created by this library"); return QPMS_EINVAL; }
  if (ss->lattice_dimension != 0) {
    set_error("scattered_E: finite systems only (the periodic field needs the lattice sums)");
    return QPMS_EINVAL;
  }
  if (btyp < 1 || btyp > 4) { set_error("scattered_E: Bessel kind %d", btyp); return QPMS_EINVAL; }
  if (npoints == 0) return QPMS_SUCCESS;
  if (npoints > (size_t)(1u << 30)) { set_error("scattered_E: too many points"); return QPMS_EINVAL; }
  const int lMax = scatsys_lmax(ss);
  if (lMax < 1 || lMax > kFieldLMax) { set_error("scattered_E: lMax %d", lMax); return QPMS_EINVAL; }
  const double *d_pos = nullptr;
  int e;
  if ((e = device_positions(ss, &d_pos))) return e;
  FieldArgs a;
  a.npts = (int)npoints;
  a.np = ss->p_count;
  a.J = btyp;
  a.k = k;
  a.where = d_where;
  a.pos = d_pos;
  a.cvf = d_cvf;
  a.tb = field_tables();
  // Split the particles over grid.y so that the grid fills whole waves of
  // resident blocks (at least two waves), with >= 8 particles per split.
  const long bx = ((long)npoints + kFieldThreads - 1) / kFieldThreads;
  const long wave = field_wave(lMax);
  const long maxsplit = std::max(1, std::min(a.np / 8, 65535));
  long nsplit = 1;
  double best = 2.0;
  for (long sp = 1; sp <= maxsplit; ++sp) {
    const long tot = bx * sp, waves = (tot + wave - 1) / wave;
    if (waves < 2 && sp < maxsplit) continue;
    const double idle = (double)(waves * wave - tot) / (double)(waves * wave);
    if (idle < best - 0.02) {  // a smaller split unless a larger one idles clearly less
      best = idle;
      nsplit = sp;
    }
    if (tot >= 16 * wave) break;
  }
  a.chunk = (int)((a.np + nsplit - 1) / nsplit);
  nsplit = (a.np + a.chunk - 1) / a.chunk;
  if (nsplit == 1) {
    a.out = d_E;
    QG_CUDA_TRY(launch_field(lMax, a, 1, st));
    return QPMS_SUCCESS;
  }
  qg_c *part = nullptr;
  const size_t n = 3 * npoints;
  QG_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&part), (size_t)nsplit * n * sizeof(qg_c), st));
  a.out = part;
  cudaError_t le = launch_field(lMax, a, (int)nsplit, st);
  if (le == cudaSuccess) {
    field_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, (int)nsplit, n, d_E);
    g_launches.fetch_add(1);
    le = cudaGetLastError();
  }
  cudaFreeAsync(part, st);
  QG_CUDA_TRY(le);
  return QPMS_SUCCESS;
}

}  // namespace
}  // namespace qg

using namespace qg;

extern "C" {

int qpms_gpu_scatsys_scattered_E_device(const qpms_scatsys_t *ss, qpms_bessel_t btyp, qpms_complex_t wavenumber,
                                        const qpms_complex_t *d_cvf, size_t npoints, const double *d_where_xyz,
                                        qpms_complex_t *d_E_xyz, void *stream) {
  clear_error();
  qg_c k;
  memcpy(&k, &wavenumber, sizeof k);
  return field_device(ss, btyp, k, reinterpret_cast<const qg_c *>(d_cvf), npoints, d_where_xyz,
                      reinterpret_cast<qg_c *>(d_E_xyz), reinterpret_cast<cudaStream_t>(stream));
}

int qpms_gpu_scatsys_scattered_E(const qpms_scatsys_t *ss, qpms_bessel_t btyp, qpms_complex_t wavenumber,
                                 const qpms_complex_t *cvf, size_t npoints, const double *where_xyz,
                                 qpms_complex_t *E_xyz) {
  clear_error();
  if (!ss || !cvf || !where_xyz || !E_xyz) { set_error("NULL argument"); return QPMS_EINVAL; }
  if (npoints == 0) return QPMS_SUCCESS;
  qg_c k;
  memcpy(&k, &wavenumber, sizeof k);
  const size_t nf = ss->fecv_size;
  cudaStream_t st = nullptr;
  QG_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  char *buf = nullptr;
  const size_t bf = nf * 16, bw = (npoints * 24 + 15) / 16 * 16, be = npoints * 48;
  cudaError_t ce = cudaMallocAsync(reinterpret_cast<void **>(&buf), bf + bw + be, st);
  int e = QPMS_SUCCESS;
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(buf, cvf, bf, cudaMemcpyHostToDevice, st);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(buf + bf, where_xyz, npoints * 24, cudaMemcpyHostToDevice, st);
  if (ce == cudaSuccess) {
    e = field_device(ss, btyp, k, reinterpret_cast<const qg_c *>(buf), npoints,
                     reinterpret_cast<const double *>(buf + bf), reinterpret_cast<qg_c *>(buf + bf + bw), st);
    if (e == QPMS_SUCCESS) ce = cudaMemcpyAsync(E_xyz, buf + bf + bw, be, cudaMemcpyDeviceToHost, st);
  }
  if (buf) cudaFreeAsync(buf, st);
  cudaError_t se = cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  if (e) return e;
  QG_CUDA_TRY(ce);
  QG_CUDA_TRY(se);
  return QPMS_SUCCESS;
}

// Single-point drop-ins (scatsystem.h:715-770).  A failure is reported as a
// NaN field and qpms_gpu_last_error(); the reference aborts instead.
ccart3_t qpms_scatsys_scattered_E(const qpms_scatsys_t *ss, qpms_bessel_t btyp, qpms_complex_t wavenumber,
                                  const qpms_complex_t *cvf, cart3_t where) {
  ccart3_t res;
  const double w[3] = {where.x, where.y, where.z};
  if (qpms_gpu_scatsys_scattered_E(ss, btyp, wavenumber, cvf, 1, w, &res.x)) {
    const double nan = NAN;
    qpms_complex_t c;
    memcpy(&c, &nan, sizeof nan);
    memcpy(reinterpret_cast<char *>(&c) + 8, &nan, sizeof nan);
    res.x = res.y = res.z = c;
  }
  return res;
}

ccart3_t qpms_scatsysw_scattered_E(const qpms_scatsys_at_omega_t *ssw, qpms_bessel_t btyp,
                                   const qpms_complex_t *cvf, cart3_t where) {
  return qpms_scatsys_scattered_E(ssw ? ssw->ss : nullptr, btyp, ssw ? ssw->wavenumber : qpms_complex_t{}, cvf,
                                  where);
}

// The reference's alternative route (translation to electric dipoles at the
// evaluation point, scatsystem.c:2048-2112) evaluates the same field; both
// names run the direct kernel.
ccart3_t qpms_scatsys_scattered_E__alt(const qpms_scatsys_t *ss, qpms_bessel_t btyp, qpms_complex_t wavenumber,
                                       const qpms_complex_t *cvf, cart3_t where) {
  return qpms_scatsys_scattered_E(ss, btyp, wavenumber, cvf, where);
}

ccart3_t qpms_scatsysw_scattered_E__alt(const qpms_scatsys_at_omega_t *ssw, qpms_bessel_t btyp,
                                        const qpms_complex_t *cvf, cart3_t where) {
  return qpms_scatsysw_scattered_E(ssw, btyp, cvf, where);
}

}  // extern "C"
