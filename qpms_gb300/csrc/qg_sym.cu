// Point symmetry of finite systems and the irrep-packed (symmetry-adapted)
// mode problem (scatsystem.c:700-1000 projectors, bases and packing,
// 1361-1471 packed builder, 2202-2273 packed LU / solve).
//
// Groups: the reference's point_group_info entries (symmetries.py:485-700)
// generated by coordinate mirrors and rotations about z: trivial(_g), C2,
// C2v, D2h (x, y, z mirrors), x_and_z_flip, y_and_z_flip, C4 (rotation by
// pi/2), C4v (rotation by pi/2 and the x mirror), D4h (those and the z
// mirror), D3h (rotation by 2pi/3, x and z mirrors), with the reference's
// irrep names, irrep matrices on the generators (E of C4v / D4h: ra =
// ((0,-1),(1,0)), -lam = ((-1,0),(0,1)); E of D3h: alif (rotation by 2pi/3),
// lam = ((1,0),(0,-1)); E'' also -1 on the z mirror) and irrep order (the
// names sorted, qpms_c.pyx:204).
//
// Action on VSWF coefficients (default normalisation, e^{i m phi},
// Condon-Shortley phase), checked against the fields the oracle evaluates:
//   z -> -z:       a_N(l,m) -> (-1)^(l+m) a_N(l,m),  a_M(l,m) -> -(-1)^(l+m) a_M(l,m)
//   y -> -y:       a_N(l,m) -> (-1)^m a_N(l,-m),      a_M(l,m) -> -(-1)^m a_M(l,-m)
//   x -> -x:       a_N(l,m) -> a_N(l,-m),             a_M(l,m) -> -a_M(l,-m)
//   rotation by alpha about z: a(l,m) -> e^{-i m alpha} a(l,m) (both types)
// and the particle at r goes to the particle at g r.  The representation on
// the full coefficient vector is monomial: each index goes to one index with
// a phase.  The projector of irrep i, P_i = (d_i/|G|) sum_g chi_i(g) D(g)
// (the character summed from the diagonal irrep entries, as
// qpms_orbit_irrep_projector_matrix does, scatsystem.c:716-731), maps the span
// of an index orbit (at most |G| indices) into itself; Gram-Schmidt on the
// images P_i e_s of the orbit's indices gives an orthonormal basis of the
// irrep subspace there (the reference takes the SVD of the orbit projector,
// scatsystem.c:758-800): one vector per orbit for a 1D irrep, d x
// multiplicity for a d-dimensional one.  Packed index a is such a basis
// vector b_a, stored as (full index, coefficient) pairs of U = [b_a^H]:
// packed = U full, full = U^H packed.  The packed basis is this library's
// (particle-major order); the reference orders by orbit type and uses its own
// orbit bases, so packed vectors of the two libraries differ by a unitary
// change of basis inside each irrep, while eigenvalues, determinants and
// unpacked solutions agree.
//
// On the GPU: irrep_pack_kernel forms U M U^H from the full matrix (each
// packed element gathers at most |G|^2 products); pack / unpack kernels move
// right-hand sides and solutions between the full and the packed bases
// (unpacking through the transposed table, one thread per full index).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <complex>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "qg_internal.h"

namespace qg {

typedef std::complex<double> cdx;

struct SymDevCopy {
  int dev = -1;
  int *off = nullptr, *idx = nullptr, *toff = nullptr, *tidx = nullptr;
  qg_c *val = nullptr, *tval = nullptr;
};

struct SymData {
  const qpms_scatsys_t *ss = nullptr;
  std::string group;
  int order = 1;
  std::vector<std::string> names;
  std::vector<int> dims;                     // irrep dimensions
  std::vector<size_t> sizes;                 // saecv_sizes
  std::vector<std::vector<int>> off, idx;    // [irrep] CSR of U: packed a -> entries off[a]..off[a+1]
  std::vector<std::vector<cdx>> val;         // U[a][idx]
  std::vector<std::vector<int>> toff, tidx;  // [irrep] CSR of U^H: full s -> (packed a, conj U[a][s])
  std::vector<std::vector<cdx>> tval;
  std::vector<std::vector<SymDevCopy>> dev;  // [irrep] device copies
  std::mutex mu;
  ~SymData() {
    for (auto &v : dev)
      for (auto &d : v) {
        cudaFree(d.off);
        cudaFree(d.idx);
        cudaFree(d.val);
        cudaFree(d.toff);
        cudaFree(d.tidx);
        cudaFree(d.tval);
      }
  }
};

namespace {

std::mutex g_sym_mu;
std::vector<SymData *> &sym_table() {
  static std::vector<SymData *> *t = new std::vector<SymData *>;
  return *t;
}

// generators: 'X', 'Y', 'Z' mirrors (x -> -x etc.), 'R' rotation by +pi/2
// about z, 'T' rotation by +2pi/3 about z, 'C' rotation by pi about z
struct IrrepDef {
  const char *name;
  int dim;
  std::vector<std::vector<cdx>> gen;  // d x d row-major matrix per generator
};
struct GroupDef {
  const char *name;
  std::string gens;
  std::vector<IrrepDef> irreps;
};

std::vector<cdx> sc(double v) { return {cdx(v, 0)}; }

const std::vector<GroupDef> &group_defs() {
  static const double h3 = 0.86602540378443864676;  // sqrt(3) / 2
  static const std::vector<cdx> ra = {0, -1, 1, 0}, mlam = {-1, 0, 0, 1}, eps = {1, 0, 0, 1}, meps = {-1, 0, 0, -1},
                                lam = {1, 0, 0, -1}, alif = {-0.5, -h3, h3, -0.5};
  static const std::vector<GroupDef> defs = {
      {"trivial", "", {{"A", 1, {}}}},
      {"trivial_g", "", {{"A", 1, {}}}},
      {"x_and_z_flip", "XZ",
       {{"P'", 1, {sc(1), sc(1)}}, {"R'", 1, {sc(-1), sc(1)}}, {"P''", 1, {sc(-1), sc(-1)}},
        {"R''", 1, {sc(1), sc(-1)}}}},
      {"y_and_z_flip", "YZ",
       {{"P'", 1, {sc(1), sc(1)}}, {"R'", 1, {sc(-1), sc(1)}}, {"P''", 1, {sc(-1), sc(-1)}},
        {"R''", 1, {sc(1), sc(-1)}}}},
      {"D3h", "TXZ",
       {{"E'", 2, {alif, lam, eps}},
        {"E''", 2, {alif, lam, meps}},
        {"A1'", 1, {sc(1), sc(1), sc(1)}},
        {"A2'", 1, {sc(1), sc(-1), sc(1)}},
        {"A1''", 1, {sc(1), sc(-1), sc(-1)}},
        {"A2''", 1, {sc(1), sc(1), sc(-1)}}}},
      {"C2", "C", {{"A", 1, {sc(1)}}, {"B", 1, {sc(-1)}}}},
      {"C2v", "XY",
       {{"A1", 1, {sc(1), sc(1)}}, {"B2", 1, {sc(-1), sc(1)}}, {"A2", 1, {sc(-1), sc(-1)}},
        {"B1", 1, {sc(1), sc(-1)}}}},
      {"D2h", "XYZ",
       {{"A1'", 1, {sc(1), sc(1), sc(1)}},
        {"B2'", 1, {sc(-1), sc(1), sc(1)}},
        {"A2'", 1, {sc(-1), sc(-1), sc(1)}},
        {"B1'", 1, {sc(1), sc(-1), sc(1)}},
        {"A1''", 1, {sc(-1), sc(-1), sc(-1)}},
        {"B2''", 1, {sc(1), sc(-1), sc(-1)}},
        {"A2''", 1, {sc(1), sc(1), sc(-1)}},
        {"B1''", 1, {sc(-1), sc(1), sc(-1)}}}},
      {"C4", "R",
       {{"A", 1, {sc(1)}}, {"B", 1, {sc(-1)}}, {"1E", 1, {{cdx(0, -1)}}}, {"2E", 1, {{cdx(0, 1)}}}}},
      {"C4v", "RX",
       {{"E", 2, {ra, mlam}},
        {"A1", 1, {sc(1), sc(1)}},
        {"A2", 1, {sc(1), sc(-1)}},
        {"B1", 1, {sc(-1), sc(1)}},
        {"B2", 1, {sc(-1), sc(-1)}}}},
      {"D4h", "RXZ",
       {{"E'", 2, {ra, mlam, eps}},
        {"E''", 2, {ra, mlam, meps}},
        {"A1'", 1, {sc(1), sc(1), sc(1)}},
        {"A2'", 1, {sc(1), sc(-1), sc(1)}},
        {"A1''", 1, {sc(1), sc(-1), sc(-1)}},
        {"A2''", 1, {sc(1), sc(1), sc(-1)}},
        {"B1'", 1, {sc(-1), sc(1), sc(1)}},
        {"B2'", 1, {sc(-1), sc(-1), sc(1)}},
        {"B1''", 1, {sc(-1), sc(-1), sc(-1)}},
        {"B2''", 1, {sc(-1), sc(1), sc(-1)}}}},
  };
  return defs;
}

// Position matrix (3 x 3, row-major) of a generator.
std::array<double, 9> gen_matrix(char g) {
  const double h3 = 0.86602540378443864676;
  switch (g) {
    case 'X': return {-1, 0, 0, 0, 1, 0, 0, 0, 1};
    case 'Y': return {1, 0, 0, 0, -1, 0, 0, 0, 1};
    case 'Z': return {1, 0, 0, 0, 1, 0, 0, 0, -1};
    case 'C': return {-1, 0, 0, 0, -1, 0, 0, 0, 1};
    case 'T': return {-0.5, -h3, 0, h3, -0.5, 0, 0, 0, 1};  // rotation by +2pi/3
    default: return {0, -1, 0, 1, 0, 0, 0, 0, 1};            // 'R': (x, y) -> (-y, x)
  }
}

// Image j' and phase of wave j (bspec order: electric block y = l(l+1)+m-1,
// then magnetic) under one generator.
void gen_wave(int lMax, char g, int j, int *jo, cdx *ph) {
  const int ne = lMax * (lMax + 2);
  const bool mag = j >= ne;
  const int y = mag ? j - ne : j;
  const int l = (int)floor(sqrt((double)y + 1) + 1e-9);
  int m = y - (l * (l + 1) - 1);
  const int tsg = mag ? -1 : 1;
  cdx p = 1.0;
  switch (g) {
    case 'Z': p = (double)((((l + m) & 1) ? -1 : 1) * tsg); break;
    case 'Y':
      p = (double)(((m & 1) ? -1 : 1) * tsg);
      m = -m;
      break;
    case 'X':
      p = (double)tsg;
      m = -m;
      break;
    case 'C': p = (double)((m & 1) ? -1 : 1); break;  // X then Y: (-1)^m
    case 'T': p = std::polar(1.0, -m * 2.0943951023931954923); break;  // e^{-i m 2pi/3}
    default: {                                        // 'R': (-i)^m
      static const cdx mi[4] = {cdx(1, 0), cdx(0, -1), cdx(-1, 0), cdx(0, 1)};
      p = mi[((m % 4) + 4) % 4];
    }
  }
  *jo = (mag ? ne : 0) + l * (l + 1) + m - 1;
  *ph = p;
}

struct Element {
  std::array<double, 9> M;
  std::vector<int> wimg;  // wave image
  std::vector<cdx> wph;   // phase
  std::vector<std::vector<cdx>> rep;  // irrep matrices
};

__global__ void irrep_pack_kernel(const qg_c *__restrict__ M, size_t ldm, int na, const int *__restrict__ off,
                                  const int *__restrict__ idx, const qg_c *__restrict__ val, qg_c *__restrict__ out) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)na * na) return;
  const int a = (int)(t / na), b = (int)(t % na);
  double re = 0, im = 0;
  for (int i = off[a]; i < off[a + 1]; ++i) {
    const qg_c *row = M + (size_t)idx[i] * ldm;
    double rr = 0, ri = 0;  // sum_j M[i][j] conj(U[b][j])
    for (int j = off[b]; j < off[b + 1]; ++j) {
      const qg_c v = row[idx[j]], u = val[j];
      rr = fma(v.re, u.re, fma(v.im, u.im, rr));
      ri = fma(v.im, u.re, fma(-v.re, u.im, ri));
    }
    const qg_c u = val[i];
    re = fma(u.re, rr, fma(-u.im, ri, re));
    im = fma(u.re, ri, fma(u.im, rr, im));
  }
  out[t] = cmk(re, im);
}

// out[a] = sum over the entries of a of U[a][s] v[s]
__global__ void irrep_pack_vec_kernel(const qg_c *__restrict__ v, int na, int nrhs, size_t ldv, size_t ldo,
                                      const int *__restrict__ off, const int *__restrict__ idx,
                                      const qg_c *__restrict__ val, qg_c *__restrict__ out) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)na * nrhs) return;
  const int a = (int)(t % na), r = (int)(t / na);
  qg_c acc = cmk(0, 0);
  for (int i = off[a]; i < off[a + 1]; ++i) acc = cadd(acc, cmul(val[i], v[(size_t)r * ldv + idx[i]]));
  out[(size_t)r * ldo + a] = acc;
}

// full[s] += sum over the packed a of conj(U[a][s]) packed[a] (transposed
// table: one thread per full index, no write conflicts)
__global__ void irrep_unpack_vec_kernel(const qg_c *__restrict__ p, int nfull, int nrhs, size_t ldp, size_t ldf,
                                        const int *__restrict__ toff, const int *__restrict__ tidx,
                                        const qg_c *__restrict__ tval, qg_c *__restrict__ full) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)nfull * nrhs) return;
  const int sidx = (int)(t % nfull), r = (int)(t / nfull);
  if (toff[sidx] == toff[sidx + 1]) return;
  qg_c acc = full[(size_t)r * ldf + sidx];
  for (int i = toff[sidx]; i < toff[sidx + 1]; ++i) acc = cadd(acc, cmul(tval[i], p[(size_t)r * ldp + tidx[i]]));
  full[(size_t)r * ldf + sidx] = acc;
}

}  // namespace

SymData *sym_of(const qpms_scatsys_t *ss) {
  std::lock_guard<std::mutex> g(g_sym_mu);
  for (SymData *d : sym_table())
    if (d->ss == ss) return d;
  return nullptr;
}

void sym_forget_system(const qpms_scatsys_t *ss) {
  std::lock_guard<std::mutex> g(g_sym_mu);
  auto &t = sym_table();
  for (size_t i = 0; i < t.size(); ++i)
    if (t[i]->ss == ss) {
      delete t[i];
      t.erase(t.begin() + i);
      return;
    }
}

// Device tables of irrep iri (uploaded on first use on the current device).
int sym_device(SymData *sd, int iri, SymDevCopy *out) {
  int dev = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> g(sd->mu);
  for (auto &d : sd->dev[iri])
    if (d.dev == dev) {
      *out = d;
      return QPMS_SUCCESS;
    }
  SymDevCopy d;
  d.dev = dev;
  const auto put_i = [](int **p, const std::vector<int> &v) -> int {
    QG_CUDA_TRY(cudaMalloc(p, std::max<size_t>(1, v.size()) * 4));
    QG_CUDA_TRY(cudaMemcpy(*p, v.data(), v.size() * 4, cudaMemcpyHostToDevice));
    return QPMS_SUCCESS;
  };
  const auto put_c = [](qg_c **p, const std::vector<cdx> &v) -> int {
    QG_CUDA_TRY(cudaMalloc(p, std::max<size_t>(1, v.size()) * 16));
    QG_CUDA_TRY(cudaMemcpy(*p, v.data(), v.size() * 16, cudaMemcpyHostToDevice));
    return QPMS_SUCCESS;
  };
  int e;
  if ((e = put_i(&d.off, sd->off[iri])) || (e = put_i(&d.idx, sd->idx[iri])) || (e = put_c(&d.val, sd->val[iri])) ||
      (e = put_i(&d.toff, sd->toff[iri])) || (e = put_i(&d.tidx, sd->tidx[iri])) ||
      (e = put_c(&d.tval, sd->tval[iri])))
    return e;
  sd->dev[iri].push_back(d);
  *out = d;
  return QPMS_SUCCESS;
}

// Device-level helpers for the solver paths.
int sym_pack_matrix_device(const qpms_scatsys_t *ss, int iri, const qg_c *dM, size_t ldm, qg_c *dout,
                           cudaStream_t st) {
  SymData *sd = sym_of(ss);
  if (!sd) { set_error("system has no symmetry"); return QPMS_EINVAL; }
  SymDevCopy Dc;
  const SymDevCopy *D = &Dc;
  int e;
  if ((e = sym_device(sd, iri, &Dc))) return e;
  const size_t na = sd->sizes[iri];
  if (!na) return QPMS_SUCCESS;
  irrep_pack_kernel<<<(unsigned)((na * na + 255) / 256), 256, 0, st>>>(dM, ldm, (int)na, D->off, D->idx, D->val,
                                                                      dout);
  g_launches.fetch_add(1);
  QG_CUDA_TRY(cudaGetLastError());
  return QPMS_SUCCESS;
}

int sym_pack_vectors_device(const qpms_scatsys_t *ss, int iri, const qg_c *dv, int nrhs, size_t ldv, qg_c *dout,
                            size_t ldo, cudaStream_t st) {
  SymData *sd = sym_of(ss);
  if (!sd) { set_error("system has no symmetry"); return QPMS_EINVAL; }
  SymDevCopy Dc;
  const SymDevCopy *D = &Dc;
  int e;
  if ((e = sym_device(sd, iri, &Dc))) return e;
  const size_t na = sd->sizes[iri];
  if (!na) return QPMS_SUCCESS;
  irrep_pack_vec_kernel<<<(unsigned)((na * nrhs + 255) / 256), 256, 0, st>>>(dv, (int)na, nrhs, ldv, ldo, D->off,
                                                                            D->idx, D->val, dout);
  g_launches.fetch_add(1);
  QG_CUDA_TRY(cudaGetLastError());
  return QPMS_SUCCESS;
}

int sym_unpack_add_vectors_device(const qpms_scatsys_t *ss, int iri, const qg_c *dp, int nrhs, size_t ldp,
                                  qg_c *dfull, size_t ldf, cudaStream_t st) {
  SymData *sd = sym_of(ss);
  if (!sd) { set_error("system has no symmetry"); return QPMS_EINVAL; }
  SymDevCopy Dc;
  const SymDevCopy *D = &Dc;
  int e;
  if ((e = sym_device(sd, iri, &Dc))) return e;
  const size_t na = sd->sizes[iri], N = ss->fecv_size;
  if (!na) return QPMS_SUCCESS;
  irrep_unpack_vec_kernel<<<(unsigned)((N * nrhs + 255) / 256), 256, 0, st>>>(dp, (int)N, nrhs, ldp, ldf, D->toff,
                                                                             D->tidx, D->tval, dfull);
  g_launches.fetch_add(1);
  QG_CUDA_TRY(cudaGetLastError());
  return QPMS_SUCCESS;
}

int sym_nirreps(const qpms_scatsys_t *ss) {
  SymData *sd = sym_of(ss);
  return sd ? (int)sd->names.size() : 0;
}

size_t sym_size(const qpms_scatsys_t *ss, int iri) {
  SymData *sd = sym_of(ss);
  return (sd && iri >= 0 && iri < (int)sd->sizes.size()) ? sd->sizes[iri] : 0;
}

int ssw_modeproblem_device(const qpms_scatsys_at_omega_t *ssw, qg_c *dM, cudaStream_t st);  // qg_scatsys.cu
int ss_translation_device(const qpms_scatsys_t *ss, qg_c k, int J, qg_c *dM, cudaStream_t st);

namespace {
struct DBuf {
  void *p = nullptr;
  ~DBuf() {
    if (p) cudaFree(p);
  }
};

// check iri and return the symmetry data
SymData *sym_check(const qpms_scatsys_t *ss, int iri) {
  if (!ss) { set_error("NULL system"); return nullptr; }
  SymData *sd = sym_of(ss);
  if (!sd) { set_error("the system has no point symmetry (qpms_gpu_scatsys_set_symmetry)"); return nullptr; }
  if (iri < 0 || iri >= (int)sd->names.size()) {
    set_error("invalid irrep index %d (of %d irreps)", iri, (int)sd->names.size());
    return nullptr;
  }
  return sd;
}

// target (na x na, host) = U M U^H for the device matrix dM (N x N)
qpms_complex_t *pack_device_to_host(const qpms_scatsys_t *ss, SymData *sd, int iri, const qg_c *dM,
                                    qpms_complex_t *target) {
  const size_t na = sd->sizes[iri], N = ss->fecv_size;
  bool own = false;
  if (!target) {
    target = (qpms_complex_t *)malloc(std::max<size_t>(1, na * na) * 16);
    own = true;
    if (!target) { set_error("out of host memory"); return nullptr; }
  }
  if (!na) return target;
  DBuf dout;
  if (cudaMalloc(&dout.p, na * na * 16) != cudaSuccess) {
    set_error("out of device memory");
    if (own) free(target);
    return nullptr;
  }
  if (sym_pack_matrix_device(ss, iri, dM, N, (qg_c *)dout.p, 0)) {
    if (own) free(target);
    return nullptr;
  }
  if (cudaMemcpy(target, dout.p, na * na * 16, cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("device to host copy failed");
    if (own) free(target);
    return nullptr;
  }
  return target;
}
}  // namespace
}  // namespace qg

using namespace qg;

extern "C" {

// Gives a finite system the point symmetry `group` ("trivial", "C2", "C2v",
// "D2h", "x_and_z_flip", "y_and_z_flip", "C4", "C4v", "D4h", "D3h"; the
// reference's point_group_info entries of these names).  Checks that every operation maps each particle onto a
// particle of the same kind; the particles' T-matrices must be invariant
// (Mie spheres are).
int qpms_gpu_scatsys_set_symmetry(qpms_scatsys_t *ss, const char *group) {
  clear_error();
  if (!ss || !group) { set_error("NULL argument"); return QPMS_EINVAL; }
  if (ss->lattice_dimension != 0) {
    set_error("Irreps decomposition not yet supported for periodic systems");
    return QPMS_EINVAL;
  }
  const GroupDef *gd = nullptr;
  for (const auto &g : group_defs())
    if (!strcmp(g.name, group)) gd = &g;
  if (!gd) {
    set_error("unknown point group %s (trivial, C2, C2v, D2h, x_and_z_flip, y_and_z_flip, C4, C4v, D4h, D3h)", group);
    return QPMS_EINVAL;
  }
  const int np = ss->p_count, n = (int)(ss->fecv_size / np), N = (int)ss->fecv_size;
  const int lMax = (int)lround(sqrt(n / 2.0 + 1) - 1);
  const int ng = (int)gd->gens.size(), nir = (int)gd->irreps.size();
  // ---- the group: closure of the generators (element = g o previous) ----
  std::vector<Element> el(1);
  el[0].M = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  el[0].wimg.resize(n);
  el[0].wph.assign(n, 1.0);
  for (int j = 0; j < n; ++j) el[0].wimg[j] = j;
  el[0].rep.resize(nir);
  for (int i = 0; i < nir; ++i) {
    const int d = gd->irreps[i].dim;
    el[0].rep[i].assign(d * d, 0.0);
    for (int a = 0; a < d; ++a) el[0].rep[i][a * d + a] = 1.0;
  }
  std::vector<std::vector<int>> gimg(ng, std::vector<int>(n));
  std::vector<std::vector<cdx>> gph(ng, std::vector<cdx>(n));
  for (int b = 0; b < ng; ++b)
    for (int j = 0; j < n; ++j) gen_wave(lMax, gd->gens[b], j, &gimg[b][j], &gph[b][j]);
  for (size_t q = 0; q < el.size() && el.size() <= 64; ++q)
    for (int b = 0; b < ng; ++b) {
      const std::array<double, 9> G = gen_matrix(gd->gens[b]);
      Element e;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          double v = 0;
          for (int k = 0; k < 3; ++k) v += G[r * 3 + k] * el[q].M[k * 3 + c];
          e.M[r * 3 + c] = v;
        }
      bool seen = false;
      for (const auto &x : el) {
        double d = 0;
        for (int c = 0; c < 9; ++c) d = std::max(d, fabs(x.M[c] - e.M[c]));
        seen = seen || d < 1e-9;
      }
      if (seen) continue;
      e.wimg.resize(n);
      e.wph.resize(n);
      for (int j = 0; j < n; ++j) {
        const int j1 = el[q].wimg[j];
        e.wimg[j] = gimg[b][j1];
        e.wph[j] = el[q].wph[j] * gph[b][j1];
      }
      e.rep.resize(nir);
      for (int i = 0; i < nir; ++i) {
        const int d = gd->irreps[i].dim;
        const std::vector<cdx> &Gm = gd->irreps[i].gen[b];
        e.rep[i].assign(d * d, 0.0);
        for (int r = 0; r < d; ++r)
          for (int c = 0; c < d; ++c)
            for (int k = 0; k < d; ++k) e.rep[i][r * d + c] += Gm[r * d + k] * el[q].rep[i][k * d + c];
      }
      el.push_back(std::move(e));
    }
  const int order = (int)el.size();
  // ---- particle permutations ----
  double scale = 0;
  for (int p = 0; p < np; ++p)
    scale = std::max(scale, fabs(ss->p[p].pos.x) + fabs(ss->p[p].pos.y) + fabs(ss->p[p].pos.z));
  const double tol = 1e-10 * (scale > 0 ? scale : 1.0);
  std::vector<std::vector<int>> perm(order, std::vector<int>(np, -1));
  for (int e = 0; e < order; ++e)
    for (int p = 0; p < np; ++p) {
      const double r0[3] = {ss->p[p].pos.x, ss->p[p].pos.y, ss->p[p].pos.z};
      double x[3];
      for (int r = 0; r < 3; ++r)
        x[r] = el[e].M[r * 3] * r0[0] + el[e].M[r * 3 + 1] * r0[1] + el[e].M[r * 3 + 2] * r0[2];
      for (int q = 0; q < np; ++q)
        if (fabs(ss->p[q].pos.x - x[0]) <= tol && fabs(ss->p[q].pos.y - x[1]) <= tol &&
            fabs(ss->p[q].pos.z - x[2]) <= tol && ss->p[q].tmatrix_id == ss->p[p].tmatrix_id) {
          perm[e][p] = q;
          break;
        }
      if (perm[e][p] < 0) {
        set_error("the system is not symmetric under %s: particle %d has no image of its kind", group, p);
        return QPMS_EINVAL;
      }
    }
  auto *sd = new SymData();
  sd->ss = ss;
  sd->group = group;
  sd->order = order;
  // irreps in the reference's order: names sorted
  std::vector<int> ord(nir);
  for (int i = 0; i < nir; ++i) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](int a, int b) {
    return std::string(gd->irreps[a].name) < std::string(gd->irreps[b].name);
  });
  sd->names.resize(nir);
  sd->dims.resize(nir);
  sd->sizes.assign(nir, 0);
  sd->off.assign(nir, std::vector<int>(1, 0));
  sd->idx.resize(nir);
  sd->val.resize(nir);
  sd->dev.resize(nir);
  // ---- index orbits ----
  std::vector<int> orbit_of(N, -1);
  std::vector<std::vector<int>> orbits;
  for (int s = 0; s < N; ++s) {
    if (orbit_of[s] >= 0) continue;
    const int p = s / n, j = s % n;
    std::vector<int> o;
    for (int e = 0; e < order; ++e) {
      const int t = perm[e][p] * n + el[e].wimg[j];
      if (std::find(o.begin(), o.end(), t) == o.end()) o.push_back(t);
    }
    std::sort(o.begin(), o.end());
    for (int t : o) orbit_of[t] = (int)orbits.size();
    orbits.push_back(o);
  }
  // ---- bases: Gram-Schmidt on P e_s over each orbit ----
  for (int ii = 0; ii < nir; ++ii) {
    const IrrepDef &ir = gd->irreps[ord[ii]];
    sd->names[ii] = ir.name;
    sd->dims[ii] = ir.dim;
    const int d = ir.dim;
    std::vector<cdx> chi(order);
    for (int e = 0; e < order; ++e) {
      cdx c = 0;
      for (int a = 0; a < d; ++a) c += el[e].rep[ord[ii]][a * d + a];
      chi[e] = c * (double)d / (double)order;
    }
    for (const auto &o : orbits) {
      const int no = (int)o.size();
      std::vector<std::vector<cdx>> basis;
      for (int si = 0; si < no; ++si) {
        const int s = o[si], p = s / n, j = s % n;
        std::vector<cdx> v(no, 0.0);
        for (int e = 0; e < order; ++e) {
          const int t = perm[e][p] * n + el[e].wimg[j];
          const int ti = (int)(std::lower_bound(o.begin(), o.end(), t) - o.begin());
          v[ti] += chi[e] * el[e].wph[j];
        }
        for (int pass = 0; pass < 2; ++pass)  // re-orthogonalised once
          for (const auto &b : basis) {
            cdx dot = 0;
            for (int k = 0; k < no; ++k) dot += std::conj(b[k]) * v[k];
            for (int k = 0; k < no; ++k) v[k] -= dot * b[k];
          }
        double nrm = 0;
        for (int k = 0; k < no; ++k) nrm += std::norm(v[k]);
        if (nrm < 1e-16) continue;
        const double inv = 1.0 / sqrt(nrm);
        for (int k = 0; k < no; ++k) v[k] *= inv;
        basis.push_back(v);
      }
      for (const auto &b : basis) {
        for (int k = 0; k < no; ++k)
          if (std::abs(b[k]) > 1e-15) {
            sd->idx[ii].push_back(o[k]);
            sd->val[ii].push_back(std::conj(b[k]));  // U[a][s] = conj(b_a[s])
          }
        sd->off[ii].push_back((int)sd->idx[ii].size());
        ++sd->sizes[ii];
      }
    }
  }
  size_t tot = 0;
  for (size_t v : sd->sizes) tot += v;
  if (tot != (size_t)N) {
    set_error("internal: irrep bases span %zu of %d dimensions", tot, N);
    delete sd;
    return QPMS_ERROR;
  }
  // transposed tables (U^H: full s -> packed a, conj U[a][s])
  sd->toff.resize(nir);
  sd->tidx.resize(nir);
  sd->tval.resize(nir);
  for (int ii = 0; ii < nir; ++ii) {
    std::vector<std::vector<std::pair<int, cdx>>> rows(N);
    for (size_t a = 0; a < sd->sizes[ii]; ++a)
      for (int i = sd->off[ii][a]; i < sd->off[ii][a + 1]; ++i)
        rows[sd->idx[ii][i]].push_back({(int)a, std::conj(sd->val[ii][i])});
    sd->toff[ii].assign(1, 0);
    for (int t = 0; t < N; ++t) {
      for (const auto &x : rows[t]) {
        sd->tidx[ii].push_back(x.first);
        sd->tval[ii].push_back(x.second);
      }
      sd->toff[ii].push_back((int)sd->tidx[ii].size());
    }
  }
  sym_forget_system(ss);
  {
    std::lock_guard<std::mutex> g(g_sym_mu);
    sym_table().push_back(sd);
  }
  ss->saecv_sizes = sd->sizes.data();
  return QPMS_SUCCESS;
}

int qpms_gpu_scatsys_nirreps(const qpms_scatsys_t *ss) { return sym_nirreps(ss); }

const size_t *qpms_gpu_scatsys_saecv_sizes(const qpms_scatsys_t *ss) {
  SymData *sd = sym_of(ss);
  return sd ? sd->sizes.data() : nullptr;
}

const char *qpms_gpu_scatsys_irrep_name(const qpms_scatsys_t *ss, int iri) {
  SymData *sd = sym_of(ss);
  if (!sd || iri < 0 || iri >= (int)sd->names.size()) return nullptr;
  return sd->names[iri].c_str();
}

// U (saecv_sizes[iri] x fecv_size, row-major): packed = U full (scatsystem.c:800-836).
qpms_complex_t *qpms_scatsys_irrep_transform_matrix(qpms_complex_t *U, const qpms_scatsys_t *ss, int iri) {
  clear_error();
  SymData *sd = sym_check(ss, iri);
  if (!sd) return nullptr;
  const size_t na = sd->sizes[iri], N = ss->fecv_size;
  if (!U) U = (qpms_complex_t *)malloc(std::max<size_t>(1, na * N) * 16);
  if (!U) { set_error("out of host memory"); return nullptr; }
  memset(U, 0, na * N * 16);
  for (size_t a = 0; a < na; ++a)
    for (int i = sd->off[iri][a]; i < sd->off[iri][a + 1]; ++i) {
      U[a * N + sd->idx[iri][i]].re = sd->val[iri][i].real();
      U[a * N + sd->idx[iri][i]].im = sd->val[iri][i].imag();
    }
  return U;
}

qpms_complex_t *qpms_scatsys_irrep_pack_vector(qpms_complex_t *target, const qpms_complex_t *orig,
                                               const qpms_scatsys_t *ss, int iri) {
  clear_error();
  SymData *sd = sym_check(ss, iri);
  if (!sd || !orig) return nullptr;
  const size_t na = sd->sizes[iri];
  if (!target) target = (qpms_complex_t *)malloc(std::max<size_t>(1, na) * 16);
  if (!target) { set_error("out of host memory"); return nullptr; }
  for (size_t a = 0; a < na; ++a) {
    cdx acc = 0;
    for (int i = sd->off[iri][a]; i < sd->off[iri][a + 1]; ++i) {
      const qpms_complex_t &o = orig[sd->idx[iri][i]];
      acc += sd->val[iri][i] * cdx(o.re, o.im);
    }
    target[a].re = acc.real();
    target[a].im = acc.imag();
  }
  return target;
}

qpms_complex_t *qpms_scatsys_irrep_unpack_vector(qpms_complex_t *target, const qpms_complex_t *orig,
                                                 const qpms_scatsys_t *ss, int iri, bool add) {
  clear_error();
  SymData *sd = sym_check(ss, iri);
  if (!sd || !orig) return nullptr;
  const size_t N = ss->fecv_size, na = sd->sizes[iri];
  if (!target) target = (qpms_complex_t *)malloc(N * 16);
  if (!target) { set_error("out of host memory"); return nullptr; }
  if (!add) memset(target, 0, N * 16);
  for (size_t a = 0; a < na; ++a)
    for (int i = sd->off[iri][a]; i < sd->off[iri][a + 1]; ++i) {
      const cdx v = std::conj(sd->val[iri][i]) * cdx(orig[a].re, orig[a].im);
      target[sd->idx[iri][i]].re += v.real();
      target[sd->idx[iri][i]].im += v.imag();
    }
  return target;
}

// U M U^H on the GPU (scatsystem.c:870-930).
qpms_complex_t *qpms_scatsys_irrep_pack_matrix(qpms_complex_t *target, const qpms_complex_t *orig,
                                               const qpms_scatsys_t *ss, int iri) {
  clear_error();
  SymData *sd = sym_check(ss, iri);
  if (!sd || !orig) return nullptr;
  const size_t N = ss->fecv_size;
  DBuf dM;
  if (cudaMalloc(&dM.p, N * N * 16) != cudaSuccess ||
      cudaMemcpy(dM.p, orig, N * N * 16, cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error("device buffer for the full matrix");
    return nullptr;
  }
  return pack_device_to_host(ss, sd, iri, (const qg_c *)dM.p, target);
}

// full (+)= U^H packed U (scatsystem.c:933-1000).
qpms_complex_t *qpms_scatsys_irrep_unpack_matrix(qpms_complex_t *target, const qpms_complex_t *orig,
                                                 const qpms_scatsys_t *ss, int iri, bool add) {
  clear_error();
  SymData *sd = sym_check(ss, iri);
  if (!sd || !orig) return nullptr;
  const size_t N = ss->fecv_size, na = sd->sizes[iri];
  if (!target) target = (qpms_complex_t *)malloc(N * N * 16);
  if (!target) { set_error("out of host memory"); return nullptr; }
  if (!add) memset(target, 0, N * N * 16);
  const auto &off = sd->off[iri];
  const auto &idx = sd->idx[iri];
  const auto &val = sd->val[iri];
  for (size_t a = 0; a < na; ++a)
    for (size_t b = 0; b < na; ++b) {
      const cdx x(orig[a * na + b].re, orig[a * na + b].im);
      for (int i = off[a]; i < off[a + 1]; ++i)
        for (int j = off[b]; j < off[b + 1]; ++j) {
          const cdx v = std::conj(val[i]) * x * val[j];
          qpms_complex_t &o = target[(size_t)idx[i] * N + idx[j]];
          o.re += v.real();
          o.im += v.imag();
        }
    }
  return target;
}

// The reference's slow reference-implementation names (scatsystem.h:318-326)
// and its orbit-ordered / serial builder variants (scatsystem.h:413-430)
// compute the same matrices.
qpms_complex_t *qpms_scatsys_irrep_pack_matrix_stupid(qpms_complex_t *target, const qpms_complex_t *orig,
                                                      const qpms_scatsys_t *ss, int iri) {
  return qpms_scatsys_irrep_pack_matrix(target, orig, ss, iri);
}
qpms_complex_t *qpms_scatsys_irrep_unpack_matrix_stupid(qpms_complex_t *target, const qpms_complex_t *orig,
                                                        const qpms_scatsys_t *ss, int iri, bool add) {
  return qpms_scatsys_irrep_unpack_matrix(target, orig, ss, iri, add);
}

// Symmetry from the reference's group object: its first member is the
// group's name (groups.h:53-54), which selects the same group here.
int qpms_gpu_scatsys_set_symmetry_group(qpms_scatsys_t *ss, const void *finite_group) {
  clear_error();
  if (!finite_group) { set_error("NULL group"); return QPMS_EINVAL; }
  const char *name = *(const char *const *)finite_group;
  if (!name) { set_error("group without a name"); return QPMS_EINVAL; }
  return qpms_gpu_scatsys_set_symmetry(ss, name);
}

// (I - T S) directly in the irrep-packed form (scatsystem.c:1361-1471, 1602-1728):
// the full matrix is assembled on the GPU and packed there.
qpms_complex_t *qpms_scatsysw_build_modeproblem_matrix_irrep_packed(qpms_complex_t *target,
                                                                    const qpms_scatsys_at_omega_t *ssw, int iri) {
  clear_error();
  if (!ssw) { set_error("NULL ssw"); return nullptr; }
  SymData *sd = sym_check(ssw->ss, iri);
  if (!sd) return nullptr;
  const size_t N = ssw->ss->fecv_size;
  DBuf dM;
  if (cudaMalloc(&dM.p, N * N * 16) != cudaSuccess) { set_error("out of device memory"); return nullptr; }
  if (ssw_modeproblem_device(ssw, (qg_c *)dM.p, 0)) return nullptr;
  return pack_device_to_host(ssw->ss, sd, iri, (const qg_c *)dM.p, target);
}

qpms_complex_t *qpms_scatsysw_build_modeproblem_matrix_irrep_packed_orbitorderR(
    qpms_complex_t *target, const qpms_scatsys_at_omega_t *ssw, int iri) {
  return qpms_scatsysw_build_modeproblem_matrix_irrep_packed(target, ssw, iri);
}
qpms_complex_t *qpms_scatsysw_build_modeproblem_matrix_irrep_packed_serial(qpms_complex_t *target,
                                                                          const qpms_scatsys_at_omega_t *ssw, int iri) {
  return qpms_scatsysw_build_modeproblem_matrix_irrep_packed(target, ssw, iri);
}

// The translation matrix S (Bessel kind J) projected on an irrep (scatsystem.c:1132-1178).
qpms_complex_t *qpms_scatsys_build_translation_matrix_e_irrep_packed(qpms_complex_t *target,
                                                                     const qpms_scatsys_t *ss, int iri,
                                                                     qpms_complex_t k, qpms_bessel_t J) {
  clear_error();
  SymData *sd = sym_check(ss, iri);
  if (!sd) return nullptr;
  if (J < 1 || J > 4) { set_error("invalid J"); return nullptr; }
  const size_t N = ss->fecv_size, na = sd->sizes[iri];
  DBuf dM;
  if (cudaMalloc(&dM.p, N * N * 16) != cudaSuccess) { set_error("out of device memory"); return nullptr; }
  if (ss_translation_device(ss, cmk(k.re, k.im), J, (qg_c *)dM.p, 0)) return nullptr;
  qpms_complex_t *r = pack_device_to_host(ss, sd, iri, (const qg_c *)dM.p, target);
  if (r)  // U (I + S) U^H = I + U S U^H
    for (size_t a = 0; a < na; ++a) r[a * na + a].re -= 1.0;
  return r;
}

}  // extern "C"
