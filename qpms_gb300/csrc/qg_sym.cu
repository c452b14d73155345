// Point symmetry of finite systems and the irrep-packed (symmetry-adapted)
// mode problem (scatsystem.c:751-1000 bases and packing, 1361-1471 packed
// builder, 2202-2273 packed LU / solve).
//
// Groups: those the reference's scripts use for rectangular arrays, generated
// by the coordinate mirror operations (symmetries.py point_group_info:
// trivial, C2 = rotation by pi about z, C2v = {x, y flips}, D2h = {x, y, z
// flips}), with the reference's irrep names and its irrep order (the names
// sorted, qpms_c.pyx:204).  Every element is a diagonal sign matrix S, and
// all irreps are one-dimensional (characters +-1 fixed by the signs on the
// generators).
//
// Action on VSWF coefficients (default normalisation, e^{i m phi},
// Condon-Shortley phase), checked against the fields the oracle evaluates:
//   z -> -z:  a_N(l,m) -> (-1)^(l+m) a_N(l,m),    a_M(l,m) -> -(-1)^(l+m) a_M(l,m)
//   y -> -y:  a_N(l,m) -> (-1)^m a_N(l,-m),        a_M(l,m) -> -(-1)^m a_M(l,-m)
//   x -> -x:  a_N(l,m) -> a_N(l,-m),               a_M(l,m) -> -a_M(l,-m)
// and the particle at r goes to the particle at S r.  The representation on
// the full coefficient vector is therefore monomial: each index goes to one
// index with a sign.  The projector of irrep i, P_i = (1/|G|) sum_g chi_i(g) D(g),
// maps a unit vector e_s to at most |G| entries; the normalised non-zero
// P_i e_s of the smallest index s of every index orbit form an orthonormal
// basis of the irrep subspace.  Packed index a is such a basis vector, stored
// as (full index, coefficient) pairs: packed = U full with U[a][s] = c,
// full = U^H packed.  The packed basis is this library's (particle-major
// order); the reference orders by orbit type and uses its own orbit bases, so
// packed vectors of the two libraries differ by a unitary change of basis
// inside each irrep, while eigenvalues, determinants and unpacked solutions
// agree.
//
// On the GPU: irrep_pack_kernel forms U M U^H from the full matrix (each
// packed element gathers at most |G|^2 products); pack / unpack kernels move
// right-hand sides and solutions between the full and the packed bases.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <mutex>
#include <string>
#include <vector>

#include "qg_internal.h"

namespace qg {

struct SymDevCopy {
  int dev = -1;
  int *off = nullptr, *idx = nullptr;
  double *val = nullptr;
};

struct SymData {
  const qpms_scatsys_t *ss = nullptr;
  std::string group;
  int order = 1;
  std::vector<std::string> names;
  std::vector<size_t> sizes;                 // saecv_sizes
  std::vector<std::vector<int>> off, idx;    // [irrep] CSR: packed a -> entries off[a]..off[a+1]
  std::vector<std::vector<double>> val;
  std::vector<std::vector<SymDevCopy>> dev;  // [irrep] device copies
  std::mutex mu;
  ~SymData() {
    for (auto &v : dev)
      for (auto &d : v) {
        cudaFree(d.off);
        cudaFree(d.idx);
        cudaFree(d.val);
      }
  }
};

namespace {

std::mutex g_sym_mu;
std::vector<SymData *> &sym_table() {
  static std::vector<SymData *> *t = new std::vector<SymData *>;
  return *t;
}

struct GroupDef {
  const char *name;
  std::vector<std::array<int, 3>> gens;
  std::vector<std::pair<const char *, std::vector<int>>> irreps;  // name, signs on the generators
};

const std::vector<GroupDef> &group_defs() {
  static const std::vector<GroupDef> defs = {
      {"trivial", {}, {{"A", {}}}},
      {"C2", {{{-1, -1, 1}}}, {{"A", {1}}, {"B", {-1}}}},
      {"C2v", {{{-1, 1, 1}}, {{1, -1, 1}}}, {{"A1", {1, 1}}, {"B2", {-1, 1}}, {"A2", {-1, -1}}, {"B1", {1, -1}}}},
      {"D2h",
       {{{-1, 1, 1}}, {{1, -1, 1}}, {{1, 1, -1}}},
       {{"A1'", {1, 1, 1}},
        {"B2'", {-1, 1, 1}},
        {"A2'", {-1, -1, 1}},
        {"B1'", {1, -1, 1}},
        {"A1''", {-1, -1, -1}},
        {"B2''", {1, -1, -1}},
        {"A2''", {1, 1, -1}},
        {"B1''", {-1, 1, -1}}}},
  };
  return defs;
}

// Wave index j' and sign of the image of wave j (bspec order: electric block
// y = l(l+1)+m-1, then magnetic) under the diagonal sign matrix S.
void wave_image(int lMax, const std::array<int, 3> &S, int j, int *jo, int *sg) {
  const int ne = lMax * (lMax + 2);
  const bool mag = j >= ne;
  const int y = mag ? j - ne : j;
  const int l = (int)floor(sqrt((double)y + 1) + 1e-9);
  int m = y - (l * (l + 1) - 1);
  int s = 1;
  const int tsg = mag ? -1 : 1;
  if (S[2] < 0) s *= (((l + m) & 1) ? -1 : 1) * tsg;
  if (S[1] < 0) {
    s *= ((m & 1) ? -1 : 1) * tsg;
    m = -m;
  }
  if (S[0] < 0) {
    s *= tsg;
    m = -m;
  }
  *jo = (mag ? ne : 0) + l * (l + 1) + m - 1;
  *sg = s;
}

__global__ void irrep_pack_kernel(const qg_c *__restrict__ M, size_t ldm, int na, const int *__restrict__ off,
                                  const int *__restrict__ idx, const double *__restrict__ val, qg_c *__restrict__ out) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)na * na) return;
  const int a = (int)(t / na), b = (int)(t % na);
  double re = 0, im = 0;
  for (int i = off[a]; i < off[a + 1]; ++i) {
    const qg_c *row = M + (size_t)idx[i] * ldm;
    double rr = 0, ri = 0;
    for (int j = off[b]; j < off[b + 1]; ++j) {
      const qg_c v = row[idx[j]];
      rr = fma(val[j], v.re, rr);
      ri = fma(val[j], v.im, ri);
    }
    re = fma(val[i], rr, re);
    im = fma(val[i], ri, im);
  }
  out[t] = cmk(re, im);
}

// out[a] = sum over the entries of a of c * v[s]
__global__ void irrep_pack_vec_kernel(const qg_c *__restrict__ v, int na, int nrhs, size_t ldv, size_t ldo,
                                      const int *__restrict__ off, const int *__restrict__ idx,
                                      const double *__restrict__ val, qg_c *__restrict__ out) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)na * nrhs) return;
  const int a = (int)(t % na), r = (int)(t / na);
  qg_c acc = cmk(0, 0);
  for (int i = off[a]; i < off[a + 1]; ++i) acc = cadd(acc, cscale(v[(size_t)r * ldv + idx[i]], val[i]));
  out[(size_t)r * ldo + a] = acc;
}

// full[s] += c * packed[a] over the entries (each full index appears at most
// once per irrep, so the threads of one irrep never write the same element)
__global__ void irrep_unpack_vec_kernel(const qg_c *__restrict__ p, int na, int nrhs, size_t ldp, size_t ldf,
                                        const int *__restrict__ off, const int *__restrict__ idx,
                                        const double *__restrict__ val, qg_c *__restrict__ full) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)na * nrhs) return;
  const int a = (int)(t % na), r = (int)(t / na);
  const qg_c x = p[(size_t)r * ldp + a];
  for (int i = off[a]; i < off[a + 1]; ++i) {
    qg_c &o = full[(size_t)r * ldf + idx[i]];
    o = cadd(o, cscale(x, val[i]));
  }
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

// Device CSR of irrep iri (uploaded on first use on the current device).
int sym_device(SymData *sd, int iri, const int **off, const int **idx, const double **val) {
  int dev = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> g(sd->mu);
  for (auto &d : sd->dev[iri])
    if (d.dev == dev) {
      *off = d.off;
      *idx = d.idx;
      *val = d.val;
      return QPMS_SUCCESS;
    }
  SymDevCopy d;
  d.dev = dev;
  QG_CUDA_TRY(cudaMalloc(&d.off, sd->off[iri].size() * 4));
  QG_CUDA_TRY(cudaMalloc(&d.idx, std::max<size_t>(1, sd->idx[iri].size()) * 4));
  QG_CUDA_TRY(cudaMalloc(&d.val, std::max<size_t>(1, sd->val[iri].size()) * 8));
  QG_CUDA_TRY(cudaMemcpy(d.off, sd->off[iri].data(), sd->off[iri].size() * 4, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(d.idx, sd->idx[iri].data(), sd->idx[iri].size() * 4, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(d.val, sd->val[iri].data(), sd->val[iri].size() * 8, cudaMemcpyHostToDevice));
  sd->dev[iri].push_back(d);
  *off = d.off;
  *idx = d.idx;
  *val = d.val;
  return QPMS_SUCCESS;
}

// Device-level helpers for the solver paths.
int sym_pack_matrix_device(const qpms_scatsys_t *ss, int iri, const qg_c *dM, size_t ldm, qg_c *dout,
                           cudaStream_t st) {
  SymData *sd = sym_of(ss);
  if (!sd) { set_error("system has no symmetry"); return QPMS_EINVAL; }
  const int *o, *ix;
  const double *v;
  int e;
  if ((e = sym_device(sd, iri, &o, &ix, &v))) return e;
  const size_t na = sd->sizes[iri];
  if (!na) return QPMS_SUCCESS;
  irrep_pack_kernel<<<(unsigned)((na * na + 255) / 256), 256, 0, st>>>(dM, ldm, (int)na, o, ix, v, dout);
  g_launches.fetch_add(1);
  QG_CUDA_TRY(cudaGetLastError());
  return QPMS_SUCCESS;
}

int sym_pack_vectors_device(const qpms_scatsys_t *ss, int iri, const qg_c *dv, int nrhs, size_t ldv, qg_c *dout,
                            size_t ldo, cudaStream_t st) {
  SymData *sd = sym_of(ss);
  if (!sd) { set_error("system has no symmetry"); return QPMS_EINVAL; }
  const int *o, *ix;
  const double *v;
  int e;
  if ((e = sym_device(sd, iri, &o, &ix, &v))) return e;
  const size_t na = sd->sizes[iri];
  if (!na) return QPMS_SUCCESS;
  irrep_pack_vec_kernel<<<(unsigned)((na * nrhs + 255) / 256), 256, 0, st>>>(dv, (int)na, nrhs, ldv, ldo, o, ix,
                                                                            v, dout);
  g_launches.fetch_add(1);
  QG_CUDA_TRY(cudaGetLastError());
  return QPMS_SUCCESS;
}

int sym_unpack_add_vectors_device(const qpms_scatsys_t *ss, int iri, const qg_c *dp, int nrhs, size_t ldp,
                                  qg_c *dfull, size_t ldf, cudaStream_t st) {
  SymData *sd = sym_of(ss);
  if (!sd) { set_error("system has no symmetry"); return QPMS_EINVAL; }
  const int *o, *ix;
  const double *v;
  int e;
  if ((e = sym_device(sd, iri, &o, &ix, &v))) return e;
  const size_t na = sd->sizes[iri];
  if (!na) return QPMS_SUCCESS;
  irrep_unpack_vec_kernel<<<(unsigned)((na * nrhs + 255) / 256), 256, 0, st>>>(dp, (int)na, nrhs, ldp, ldf, o, ix,
                                                                              v, dfull);
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
// "D2h"; the reference's point_group_info entries of these names).  Checks
// that every operation maps each particle onto a particle of the same kind;
// the particles' T-matrices must be invariant (Mie spheres are).
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
  if (!gd) { set_error("unknown point group %s (trivial, C2, C2v, D2h)", group); return QPMS_EINVAL; }
  const int np = ss->p_count, n = (int)(ss->fecv_size / np), N = (int)ss->fecv_size;
  const int lMax = (int)lround(sqrt(n / 2.0 + 1) - 1);
  const int ng = (int)gd->gens.size(), order = 1 << ng;
  // elements: products of generator subsets (bit b <-> generator b)
  std::vector<std::array<int, 3>> el(order);
  for (int e = 0; e < order; ++e) {
    std::array<int, 3> S = {1, 1, 1};
    for (int b = 0; b < ng; ++b)
      if (e >> b & 1)
        for (int c = 0; c < 3; ++c) S[c] *= gd->gens[b][c];
    el[e] = S;
  }
  // particle permutations
  double scale = 0;
  for (int p = 0; p < np; ++p)
    scale = std::max(scale, fabs(ss->p[p].pos.x) + fabs(ss->p[p].pos.y) + fabs(ss->p[p].pos.z));
  const double tol = 1e-10 * (scale > 0 ? scale : 1.0);
  std::vector<std::vector<int>> perm(order, std::vector<int>(np, -1));
  for (int e = 0; e < order; ++e)
    for (int p = 0; p < np; ++p) {
      const double x = el[e][0] * ss->p[p].pos.x, y = el[e][1] * ss->p[p].pos.y, z = el[e][2] * ss->p[p].pos.z;
      for (int q = 0; q < np; ++q)
        if (fabs(ss->p[q].pos.x - x) <= tol && fabs(ss->p[q].pos.y - y) <= tol && fabs(ss->p[q].pos.z - z) <= tol &&
            ss->p[q].tmatrix_id == ss->p[p].tmatrix_id) {
          perm[e][p] = q;
          break;
        }
      if (perm[e][p] < 0) {
        set_error("the system is not symmetric under %s: particle %d has no image of its kind", group, p);
        return QPMS_EINVAL;
      }
    }
  // wave images
  std::vector<std::vector<int>> wimg(order, std::vector<int>(n)), wsg(order, std::vector<int>(n));
  for (int e = 0; e < order; ++e)
    for (int j = 0; j < n; ++j) wave_image(lMax, el[e], j, &wimg[e][j], &wsg[e][j]);
  auto *sd = new SymData();
  sd->ss = ss;
  sd->group = group;
  sd->order = order;
  // irreps in the reference's order: names sorted
  std::vector<int> ord(gd->irreps.size());
  for (size_t i = 0; i < ord.size(); ++i) ord[i] = (int)i;
  std::sort(ord.begin(), ord.end(),
            [&](int a, int b) { return std::string(gd->irreps[a].first) < std::string(gd->irreps[b].first); });
  const int nir = (int)ord.size();
  sd->names.resize(nir);
  sd->sizes.assign(nir, 0);
  sd->off.assign(nir, std::vector<int>(1, 0));
  sd->idx.resize(nir);
  sd->val.resize(nir);
  sd->dev.resize(nir);
  // smallest index of each index orbit
  std::vector<char> isrep(N, 1);
  for (int s = 0; s < N; ++s) {
    const int p = s / n, j = s % n;
    for (int e = 0; e < order; ++e)
      if (perm[e][p] * n + wimg[e][j] < s) isrep[s] = 0;
  }
  std::vector<double> acc(N, 0.0);
  std::vector<int> touched;
  for (int ii = 0; ii < nir; ++ii) {
    const auto &ir = gd->irreps[ord[ii]];
    sd->names[ii] = ir.first;
    std::vector<int> chi(order);
    for (int e = 0; e < order; ++e) {
      int c = 1;
      for (int b = 0; b < ng; ++b)
        if (e >> b & 1) c *= ir.second[b];
      chi[e] = c;
    }
    for (int s = 0; s < N; ++s) {
      if (!isrep[s]) continue;
      const int p = s / n, j = s % n;
      touched.clear();
      for (int e = 0; e < order; ++e) {
        const int t = perm[e][p] * n + wimg[e][j];
        if (std::find(touched.begin(), touched.end(), t) == touched.end()) touched.push_back(t);
        acc[t] += (double)chi[e] * wsg[e][j];
      }
      double nrm = 0;
      for (int t : touched) nrm += acc[t] * acc[t];
      if (nrm > 0.5) {  // entries are integers: non-zero projection
        std::sort(touched.begin(), touched.end());
        const double inv = 1.0 / sqrt(nrm);
        for (int t : touched)
          if (acc[t] != 0) {
            sd->idx[ii].push_back(t);
            sd->val[ii].push_back(acc[t] * inv);
          }
        sd->off[ii].push_back((int)sd->idx[ii].size());
        ++sd->sizes[ii];
      }
      for (int t : touched) acc[t] = 0;
    }
  }
  size_t tot = 0;
  for (size_t v : sd->sizes) tot += v;
  if (tot != (size_t)N) {
    set_error("internal: irrep bases span %zu of %d dimensions", tot, N);
    delete sd;
    return QPMS_ERROR;
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
    for (int i = sd->off[iri][a]; i < sd->off[iri][a + 1]; ++i) U[a * N + sd->idx[iri][i]].re = sd->val[iri][i];
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
    double re = 0, im = 0;
    for (int i = sd->off[iri][a]; i < sd->off[iri][a + 1]; ++i) {
      re += sd->val[iri][i] * orig[sd->idx[iri][i]].re;
      im += sd->val[iri][i] * orig[sd->idx[iri][i]].im;
    }
    target[a].re = re;
    target[a].im = im;
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
      target[sd->idx[iri][i]].re += sd->val[iri][i] * orig[a].re;
      target[sd->idx[iri][i]].im += sd->val[iri][i] * orig[a].im;
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
      const qpms_complex_t x = orig[a * na + b];
      for (int i = off[a]; i < off[a + 1]; ++i)
        for (int j = off[b]; j < off[b + 1]; ++j) {
          qpms_complex_t &o = target[(size_t)idx[i] * N + idx[j]];
          o.re += val[i] * val[j] * x.re;
          o.im += val[i] * val[j] * x.im;
        }
    }
  return target;
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
