// ORACLE — test infrastructure only (see oracle.h). CPU restatement of the reference path.
#include "oracle.h"

#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <map>
#include <limits>
#include <numeric>

#include "fem.hpp"
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace orc;

struct orc_csr {
  long n = 0;
  std::vector<int64_t> rp;
  std::vector<int32_t> col;
  std::vector<double> val;
  // add_to_entry: binary search in the sorted row (restates the LA container's BCRS lookup)
  inline long slot(long i, long j) const {
    const int32_t* b = col.data() + rp[i];
    const int32_t* e = col.data() + rp[i + 1];
    const int32_t* p = std::lower_bound(b, e, int32_t(j));
    if (p == e || *p != j) throw std::runtime_error("entry not in sparsity pattern");
    return long(p - col.data());
  }
};

static int g_threads = 1;

extern "C" void orc_set_threads(int nthreads) { g_threads = nthreads < 1 ? 1 : nthreads; }
extern "C" int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_num_procs();
#else
  return 1;
#endif
}

namespace {

Grid make_grid(const orc_grid* g) {
  Grid out(g->dim, g->n, g->lo, g->hi, g->simplex != 0, g->periodic != 0);
  out.xv = g->vertices;
  return out;
}

// ------------------------------------------------------------------- spaces ---
// Mappers: ContinuousMapper (spaces/mapper/continuous.hh:117-182): DoF = MCMG offset of the
// DoF-carrying entity block (codims in ascending order) + entity index; vertices use the grid
// vertex index, cells the element index, other codims are numbered in order of first appearance
// in the element walk. DiscontinuousMapper (spaces/mapper/discontinuous.hh:92-125):
// offset[e] + i with offsets accumulated in element order. FiniteVolumeMapper
// (spaces/mapper/finite-volume.hh:89-107): e * m + i.
struct Space {
  int kind = ORC_CG, order = 1;
  const Grid* grid = nullptr;
  LagrangeFE fe;
  long size = 0;
  int lsize = 0;
  std::vector<int64_t> gi;  // [nelem * lsize]
  const int64_t* indices(long e) const { return gi.data() + e * lsize; }
};

// local vertex support (subentity closure) of a Lagrange node
int node_support(const Grid& g, const LagrangeFE& fe, int node, int* lv) {
  const Vec3& x = fe.nodes[node];
  int cnt = 0;
  if (!fe.simplex) {
    for (int v = 0; v < (1 << g.dim); ++v) {
      bool ok = true;
      for (int k = 0; k < g.dim; ++k) {
        double c = x[k];
        if (c == 0.0 && ((v >> k) & 1) != 0) ok = false;
        if (c == 1.0 && ((v >> k) & 1) != 1) ok = false;
      }
      if (ok) lv[cnt++] = v;
    }
    return cnt;
  }
  double lam[4];
  lam[0] = 1.0;
  for (int k = 0; k < g.dim; ++k) { lam[k + 1] = x[k]; lam[0] -= x[k]; }
  for (int a = 0; a <= g.dim; ++a)
    if (lam[a] > 1e-12) lv[cnt++] = a;
  return cnt;
}

void build_space(const Grid& g, int kind, int order, Space& s) {
  s.kind = kind;
  s.order = order;
  s.grid = &g;
  bool smplx = g.simplex && g.dim >= 2;
  if (kind == ORC_FV) {
    s.fe = LagrangeFE(smplx, g.dim, 0);
    s.lsize = 1;
    s.size = g.nelem;
    s.gi.resize(g.nelem);
    for (long e = 0; e < g.nelem; ++e) s.gi[e] = e;
    return;
  }
  s.fe = LagrangeFE(smplx, g.dim, order);
  s.lsize = s.fe.size;
  s.gi.resize(size_t(g.nelem) * s.lsize);
  if (kind == ORC_DG) {
    long off = 0;
    for (long e = 0; e < g.nelem; ++e) {
      for (int i = 0; i < s.lsize; ++i) s.gi[e * s.lsize + i] = off + i;
      off += s.lsize;
    }
    s.size = off;
    return;
  }
  // continuous
  if (order == 1) {
    long gv[8];
    Vec3 xs[8];
    for (long e = 0; e < g.nelem; ++e) {
      g.element_vertices(e, gv, xs);
      for (int i = 0; i < s.lsize; ++i) s.gi[e * s.lsize + i] = gv[i];
    }
    s.size = g.nvert;
    return;
  }
  // order >= 2: entity numbering (first appearance) per codim, then MCMG offsets
  std::vector<std::map<std::vector<long>, long>> ent(g.dim + 1);
  std::vector<int> codim_of(s.lsize);
  std::vector<std::vector<int>> support(s.lsize);
  for (int i = 0; i < s.lsize; ++i) {
    int lv[8];
    int c = node_support(g, s.fe, i, lv);
    support[i].assign(lv, lv + c);
    int subdim = smplx ? c - 1 : (c == 1 ? 0 : (c == 2 ? 1 : (c == 4 ? 2 : 3)));
    codim_of[i] = g.dim - subdim;
  }
  std::vector<int> has(g.dim + 1, 0);
  for (int i = 0; i < s.lsize; ++i) has[codim_of[i]] = 1;
  std::vector<std::vector<long>> local_entity(size_t(g.nelem) * s.lsize);
  std::vector<long> tmpidx(size_t(g.nelem) * s.lsize);
  long gv[8];
  Vec3 xs[8];
  for (long e = 0; e < g.nelem; ++e) {
    g.element_vertices(e, gv, xs);
    for (int i = 0; i < s.lsize; ++i) {
      int c = codim_of[i];
      long idx;
      if (c == g.dim) idx = gv[support[i][0]];
      else if (c == 0) idx = e;
      else {
        std::vector<long> key;
        for (int a : support[i]) key.push_back(gv[a]);
        std::sort(key.begin(), key.end());
        auto it = ent[c].find(key);
        if (it == ent[c].end()) {
          idx = long(ent[c].size());
          ent[c][key] = idx;
        } else idx = it->second;
      }
      tmpidx[e * s.lsize + i] = idx;
    }
  }
  std::vector<long> offset(g.dim + 1, 0);
  long run = 0;
  for (int c = 0; c <= g.dim; ++c) {
    offset[c] = run;
    if (!has[c]) continue;
    long cnt = (c == 0) ? g.nelem : (c == g.dim ? g.nvert : long(ent[c].size()));
    run += cnt;
  }
  s.size = run;
  for (long e = 0; e < g.nelem; ++e)
    for (int i = 0; i < s.lsize; ++i) s.gi[e * s.lsize + i] = offset[codim_of[i]] + tmpidx[e * s.lsize + i];
}

// --------------------------------------------------------------- intersections ---
struct Topology {
  // neighbour[e * nf + f] = (element, face) or -1
  std::vector<long> nb;
  std::vector<int> nbf;
  int nf = 0;
};

void build_topology(const Grid& g, Topology& t) {
  t.nf = g.num_faces();
  t.nb.assign(size_t(g.nelem) * t.nf, -1);
  t.nbf.assign(size_t(g.nelem) * t.nf, -1);
  if (!g.simplex || g.dim == 1) {
    for (long e = 0; e < g.nelem; ++e) {
      long ci[3];
      g.cell_multi(e, ci);
      for (int f = 0; f < t.nf; ++f) {
        int k = f / 2, side = f % 2;
        long cj[3] = {ci[0], ci[1], ci[2]};
        cj[k] += side ? 1 : -1;
        if (cj[k] < 0 || cj[k] >= g.n[k]) {
          if (!g.periodic) continue;
          cj[k] = (cj[k] + g.n[k]) % g.n[k];
        }
        t.nb[e * t.nf + f] = g.cell_index(cj);
        t.nbf[e * t.nf + f] = k * 2 + (1 - side);
      }
    }
    return;
  }
  std::map<std::vector<long>, std::pair<long, int>> faces;
  long gv[8];
  Vec3 xs[8];
  for (long e = 0; e < g.nelem; ++e) {
    g.element_vertices(e, gv, xs);
    for (int f = 0; f < t.nf; ++f) {
      int lv[4];
      int c = g.face_local_vertices(f, lv);
      std::vector<long> key;
      for (int i = 0; i < c; ++i) key.push_back(gv[lv[i]]);
      std::sort(key.begin(), key.end());
      auto it = faces.find(key);
      if (it == faces.end()) faces[key] = {e, f};
      else {
        long e2 = it->second.first;
        int f2 = it->second.second;
        t.nb[e * t.nf + f] = e2;
        t.nbf[e * t.nf + f] = f2;
        t.nb[e2 * t.nf + f2] = e;
        t.nbf[e2 * t.nf + f2] = f;
      }
    }
  }
}

Intersection make_intersection(const Grid& g, const Topology& t, long e, int f) {
  Intersection I;
  I.inside = e;
  I.face_in = f;
  I.outside = t.nb[e * t.nf + f];
  I.face_out = t.nbf[e * t.nf + f];
  long gv[8];
  Vec3 xs[8];
  g.element_vertices(e, gv, xs);
  int lv[4];
  I.nv = g.face_local_vertices(f, lv);
  for (int i = 0; i < I.nv; ++i) I.corners[i] = xs[lv[i]];
  bool on_boundary = false;
  if (!g.simplex || g.dim == 1) {
    int k = f / 2, side = f % 2;
    I.normal = {0, 0, 0};
    I.normal[k] = side ? 1.0 : -1.0;
    long ci[3];
    g.cell_multi(e, ci);
    on_boundary = side ? (ci[k] == g.n[k] - 1) : (ci[k] == 0);
    double vol = 1.0;
    for (int j = 0; j < g.dim; ++j)
      if (j != k) vol *= g.h[j];
    I.volume = vol;
  } else {
    int opp = g.dim - f;
    Vec3 c0 = I.corners[0];
    Vec3 nrm{0, 0, 0};
    if (g.dim == 2) {
      Vec3 t0{I.corners[1][0] - c0[0], I.corners[1][1] - c0[1], 0};
      nrm = {t0[1], -t0[0], 0};
      I.volume = std::sqrt(t0[0] * t0[0] + t0[1] * t0[1]);
    } else {
      Vec3 a{I.corners[1][0] - c0[0], I.corners[1][1] - c0[1], I.corners[1][2] - c0[2]};
      Vec3 b{I.corners[2][0] - c0[0], I.corners[2][1] - c0[1], I.corners[2][2] - c0[2]};
      nrm = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
      I.volume = 0.5 * std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    }
    double len = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    for (int r = 0; r < 3; ++r) nrm[r] /= len;
    Vec3 xo = xs[opp];
    double s = 0;
    for (int r = 0; r < g.dim; ++r) s += (xo[r] - c0[r]) * nrm[r];
    if (s > 0)
      for (int r = 0; r < 3; ++r) nrm[r] = -nrm[r];
    I.normal = nrm;
    on_boundary = (I.outside < 0);
  }
  I.boundary = on_boundary;
  I.periodic = on_boundary && I.outside >= 0;
  return I;
}

// physical point of a reference-face point (affine faces; cube faces multilinear over corners)
Vec3 face_global(const Grid& g, const Intersection& I, const Vec3& xf) {
  Vec3 y{0, 0, 0};
  int fd = g.dim - 1;
  if (fd == 0) return I.corners[0];
  if (g.simplex) {
    y = I.corners[0];
    for (int k = 0; k < fd; ++k)
      for (int r = 0; r < 3; ++r) y[r] += (I.corners[k + 1][r] - I.corners[0][r]) * xf[k];
    return y;
  }
  for (int v = 0; v < I.nv; ++v) {
    double N = 1.0;
    for (int k = 0; k < fd; ++k) N *= ((v >> k) & 1) ? xf[k] : (1.0 - xf[k]);
    for (int r = 0; r < 3; ++r) y[r] += N * I.corners[v][r];
  }
  return y;
}

double ref_face_volume(const Grid& g) {
  int fd = g.dim - 1;
  if (fd <= 0 || !g.simplex) return 1.0;
  return fd == 1 ? 1.0 : 0.5;
}

// ------------------------------------------------------------------ pattern ---
orc_csr* build_pattern(const Grid& g, const Space& test, const Space& ansatz, int stencil, const Topology* topo) {
  // make_{element,intersection,element_and_intersection}_sparsity_pattern
  // (tools/sparsity-pattern.hh:33-50, 72-95, 117-144): insert every local index pair, then sort.
  std::vector<std::vector<int32_t>> rows(test.size);
  for (long e = 0; e < g.nelem; ++e) {
    const int64_t* ri = test.indices(e);
    if (stencil != ORC_STENCIL_INTERSECTION) {
      const int64_t* ci = ansatz.indices(e);
      for (int i = 0; i < test.lsize; ++i)
        for (int j = 0; j < ansatz.lsize; ++j) rows[ri[i]].push_back(int32_t(ci[j]));
    }
    if (stencil != ORC_STENCIL_ELEMENT) {
      for (int f = 0; f < topo->nf; ++f) {
        long nb = topo->nb[e * topo->nf + f];
        if (nb < 0) continue;
        const int64_t* ci = ansatz.indices(nb);
        for (int i = 0; i < test.lsize; ++i)
          for (int j = 0; j < ansatz.lsize; ++j) rows[ri[i]].push_back(int32_t(ci[j]));
      }
    }
  }
  orc_csr* m = new orc_csr;
  m->n = test.size;
  m->rp.assign(test.size + 1, 0);
  for (long i = 0; i < test.size; ++i) {
    auto& r = rows[i];
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    m->rp[i + 1] = m->rp[i] + long(r.size());
  }
  m->col.resize(m->rp[test.size]);
  for (long i = 0; i < test.size; ++i) {
    std::copy(rows[i].begin(), rows[i].end(), m->col.begin() + m->rp[i]);
    std::vector<int32_t>().swap(rows[i]);
  }
  m->val.assign(m->col.size(), 0.0);
  return m;
}

// --------------------------------------------------------- data functions ---
constexpr double kHalfPi = 1.5707963267948966;
double esv2007_force(const Vec3& x) {
  // ESV2007 test case 1: f = (pi^2/2) cos(pi x/2) cos(pi y/2) (examples/stationary-heat-equation.cc:68-70)
  return kHalfPi * M_PI * std::cos(kHalfPi * x[0]) * std::cos(kHalfPi * x[1]);
}
void esv2007_grad(const Vec3& x, double* g) {
  g[0] = -kHalfPi * std::sin(kHalfPi * x[0]) * std::cos(kHalfPi * x[1]);
  g[1] = -kHalfPi * std::cos(kHalfPi * x[0]) * std::sin(kHalfPi * x[1]);
}

struct Coeffs {
  const double* kappa = nullptr;
  double kappa_const = 1.0;
  const double* force = nullptr;
  double force_const = 1.0;
  int force_fn = ORC_FORCE_DATA;
  int force_order = 0;
  double k(long e) const { return kappa ? kappa[e] : kappa_const; }
  double f(long e, const Vec3& x) const {
    if (force_fn == ORC_FORCE_ESV2007) return esv2007_force(x);
    return force ? force[e] : force_const;
  }
};

// ------------------------------------------------------------- local forms ---
struct ElementKernel {
  const Grid& g;
  const LagrangeFE& fe;
  std::vector<QPoint> qa, qf;  // stiffness rule (order 2k), functional rule
  std::vector<double> phi_a, dphi_a, phi_f;
  ElementKernel(const Grid& gg, const LagrangeFE& f, int order_a, int order_f) : g(gg), fe(f) {
    bool sm = g.simplex && g.dim >= 2;
    qa = quadrature(sm, g.dim, order_a);
    qf = quadrature(sm, g.dim, order_f);
    int n = fe.size;
    phi_a.resize(qa.size() * n);
    dphi_a.resize(qa.size() * n * 3);
    for (size_t q = 0; q < qa.size(); ++q) {
      fe.eval(qa[q].x, &phi_a[q * n]);
      fe.grad(qa[q].x, reinterpret_cast<double(*)[3]>(&dphi_a[q * n * 3]));
    }
    phi_f.resize(qf.size() * n);
    for (size_t q = 0; q < qf.size(); ++q) fe.eval(qf[q].x, &phi_f[q * n]);
  }
  // LocalElementIntegralBilinearForm::apply2 (local/bilinear-forms/integrals.hh:97-134) with
  // LocalLaplaceIntegrand::evaluate (local/integrands/laplace.hh:81-102), scalar kappa * I.
  void laplace(const Geometry& geo, double kappa, double* A) const {
    int n = fe.size;
    for (int i = 0; i < n * n; ++i) A[i] = 0.0;
    double G[27][3];
    for (size_t q = 0; q < qa.size(); ++q) {
      double Jit[3][3];
      double det = geo.jit(qa[q].x, Jit);
      double factor = det * qa[q].w;
      const double* dp = &dphi_a[q * n * 3];
      for (int i = 0; i < n; ++i)
        for (int r = 0; r < 3; ++r) {
          double s = 0;
          for (int k = 0; k < g.dim; ++k) s += Jit[r][k] * dp[i * 3 + k];
          G[i][r] = s;
        }
      for (int ii = 0; ii < n; ++ii)
        for (int jj = 0; jj < n; ++jj) {
          double v = 0.0;
          for (int rr = 0; rr < g.dim; ++rr) v += (kappa * G[jj][rr]) * G[ii][rr];
          A[ii * n + jj] += v * factor;
        }
    }
  }
  // LocalLaplaceIntegrand::evaluate with a d x d diffusion tensor K (local/integrands/laplace.hh:81-102):
  // (K grad phi_j) . grad psi_i, K row-major
  void laplace_tensor(const Geometry& geo, const double* K, double* A) const {
    int n = fe.size;
    for (int i = 0; i < n * n; ++i) A[i] = 0.0;
    double G[27][3];
    for (size_t q = 0; q < qa.size(); ++q) {
      double Jit[3][3];
      double det = geo.jit(qa[q].x, Jit);
      double factor = det * qa[q].w;
      const double* dp = &dphi_a[q * n * 3];
      for (int i = 0; i < n; ++i)
        for (int r = 0; r < 3; ++r) {
          double s = 0;
          for (int k = 0; k < g.dim; ++k) s += Jit[r][k] * dp[i * 3 + k];
          G[i][r] = s;
        }
      for (int ii = 0; ii < n; ++ii)
        for (int jj = 0; jj < n; ++jj) {
          double v = 0.0;
          for (int rr = 0; rr < g.dim; ++rr) {
            double kg = 0.0;  // (K grad phi_j)_rr
            for (int ss = 0; ss < g.dim; ++ss) kg += K[rr * g.dim + ss] * G[jj][ss];
            v += kg * G[ii][rr];
          }
          A[ii * n + jj] += v * factor;
        }
    }
  }
  // LocalElementProductIntegrand (local/integrands/product.hh:104-130), weight 1
  void mass(const Geometry& geo, double* A) const {
    int n = fe.size;
    for (int i = 0; i < n * n; ++i) A[i] = 0.0;
    for (size_t q = 0; q < qa.size(); ++q) {
      double Jit[3][3];
      double factor = geo.jit(qa[q].x, Jit) * qa[q].w;
      const double* p = &phi_a[q * n];
      for (int ii = 0; ii < n; ++ii)
        for (int jj = 0; jj < n; ++jj) A[ii * n + jj] += ((1.0 * p[ii]) * p[jj]) * factor;
    }
  }
  // LocalElementIntegralFunctional::apply (local/functionals/integrals.hh:72-98) with
  // LocalElementProductIntegrand().with_ansatz(f) (local/integrands/conversion.hh:97-128)
  void rhs(const Geometry& geo, const Coeffs& c, long e, double* b) const {
    int n = fe.size;
    for (int i = 0; i < n; ++i) b[i] = 0.0;
    for (size_t q = 0; q < qf.size(); ++q) {
      double Jit[3][3];
      double ie = geo.jit(qf[q].x, Jit);
      double fv = c.f(e, geo.global(qf[q].x));
      const double* p = &phi_f[q * n];
      for (int ii = 0; ii < n; ++ii) b[ii] += ((1.0 * p[ii]) * fv) * ie * qf[q].w;
    }
  }
};

struct FaceParams {
  double theta = 1.0, sigma_in = 8.0, sigma_bd = 14.0;
  bool weight_is_diffusion = true;
  double beta = 1.0;  // penalty length h = |I|^beta (local/integrands/elliptic-ipdg.hh:677-741; 1: ipdg.hh)
  // Dirichlet data for the right-hand side: ORC_DIRICHLET_CONST (g = gconst) or ORC_DIRICHLET_TEST
  // (g = cos(pi x / 2) cos(pi y / 2) + 0.3 x); rhs_terms bit 0: the unary DirichletCoupling term
  // (local/integrands/laplace-ipdg.hh:292-320), bit 1: the boundary penalty weight times g
  int gfn = 0;
  double gconst = 0.0;
  int rhs_terms = 0;
  double h(double vol) const { return beta == 1.0 ? vol : std::pow(vol, beta); }
  double g(const Vec3& x) const {
    if (gfn == ORC_DIRICHLET_TEST) return std::cos(kHalfPi * x[0]) * std::cos(kHalfPi * x[1]) + 0.3 * x[0];
    return gconst;
  }
};

struct FaceKernel {
  const Grid& g;
  const LagrangeFE& fe;
  std::vector<QPoint> qf;
  double ref_vol;
  FaceKernel(const Grid& gg, const LagrangeFE& f, int order) : g(gg), fe(f) {
    qf = quadrature(g.simplex, g.dim - 1, order);
    ref_vol = ref_face_volume(g);
  }
  void basis_at(const Geometry& geo, const Vec3& x, double* v, double (*G)[3]) const {
    Vec3 xh = geo.local(x);
    fe.eval(xh, v);
    double dref[27][3];
    fe.grad(xh, dref);
    double Jit[3][3];
    geo.jit(xh, Jit);
    for (int i = 0; i < fe.size; ++i)
      for (int r = 0; r < 3; ++r) {
        double s = 0;
        for (int k = 0; k < g.dim; ++k) s += Jit[r][k] * dref[i][k];
        G[i][r] = s;
      }
  }
  // LocalCouplingIntersectionIntegralBilinearForm::apply2 (local/bilinear-forms/integrals.hh:197-267)
  // with LocalLaplaceIPDGIntegrands::InnerCoupling (local/integrands/laplace-ipdg.hh:107-186)
  // + LocalIPDGIntegrands::InnerPenalty (local/integrands/ipdg.hh:113-171).
  void inner(const Intersection& I, const Geometry& gin, const Geometry& gout, double kin, double kout,
             const FaceParams& p, double* Bii, double* Bio, double* Boi, double* Boo) const {
    int n = fe.size;
    for (int i = 0; i < n * n; ++i) Bii[i] = Bio[i] = Boi[i] = Boo[i] = 0.0;
    const Vec3& nrm = I.normal;
    double win = p.weight_is_diffusion ? kin : 1.0, wout = p.weight_is_diffusion ? kout : 1.0;
    double nn = 0;
    for (int r = 0; r < g.dim; ++r) nn += nrm[r] * nrm[r];
    const double delta_plus = wout * nn;
    const double delta_minus = win * nn;
    const double weight_minus = delta_plus / (delta_plus + delta_minus);
    const double weight_plus = delta_minus / (delta_plus + delta_minus);
    const double pen_weight = (delta_plus * delta_minus) / (delta_plus + delta_minus);
    const double penalty = (p.sigma_in * pen_weight) / p.h(I.volume);
    const double th = p.theta;
    double vin[27], vout[27], Gin[27][3], Gout[27][3], dn_in[27], dn_out[27];
    for (const auto& qp : qf) {
      Vec3 x = face_global(g, I, qp.x);
      double factor = (I.volume / ref_vol) * qp.w;
      basis_at(gin, x, vin, Gin);
      basis_at(gout, x, vout, Gout);
      for (int i = 0; i < n; ++i) {
        double a = 0, b = 0;
        for (int r = 0; r < g.dim; ++r) { a += (kin * Gin[i][r]) * nrm[r]; b += (kout * Gout[i][r]) * nrm[r]; }
        dn_in[i] = a;
        dn_out[i] = b;
      }
      for (int ii = 0; ii < n; ++ii) {
        for (int jj = 0; jj < n; ++jj) {
          double v = -1.0 * weight_minus * dn_in[jj] * vin[ii];
          v += -1.0 * th * weight_minus * vin[jj] * dn_in[ii];
          v += penalty * vin[jj] * vin[ii];
          Bii[ii * n + jj] += v * factor;
          double w = -1.0 * weight_plus * dn_out[jj] * vin[ii];
          w += th * weight_minus * vout[jj] * dn_in[ii];
          w += -1.0 * penalty * vout[jj] * vin[ii];
          Bio[ii * n + jj] += w * factor;
        }
      }
      for (int ii = 0; ii < n; ++ii) {
        for (int jj = 0; jj < n; ++jj) {
          double v = weight_minus * dn_in[jj] * vout[ii];
          v += -1.0 * th * weight_plus * vin[jj] * dn_out[ii];
          v += -1.0 * penalty * vin[jj] * vout[ii];
          Boi[ii * n + jj] += v * factor;
          double w = weight_plus * dn_out[jj] * vout[ii];
          w += th * weight_plus * vout[jj] * dn_out[ii];
          w += penalty * vout[jj] * vout[ii];
          Boo[ii * n + jj] += w * factor;
        }
      }
    }
  }
  // LocalIntersectionIntegralBilinearForm::apply2 (integrals.hh:338-369) with
  // DirichletCoupling (laplace-ipdg.hh:331-368) + BoundaryPenalty (ipdg.hh:254-282)
  void boundary(const Intersection& I, const Geometry& gin, double kin, const FaceParams& p, double* B) const {
    int n = fe.size;
    for (int i = 0; i < n * n; ++i) B[i] = 0.0;
    const Vec3& nrm = I.normal;
    double w = p.weight_is_diffusion ? kin : 1.0;
    double nn = 0;
    for (int r = 0; r < g.dim; ++r) nn += nrm[r] * nrm[r];
    const double penalty = (p.sigma_bd * (w * nn)) / p.h(I.volume);
    double v[27], G[27][3], dn[27];
    for (const auto& qp : qf) {
      Vec3 x = face_global(g, I, qp.x);
      double factor = (I.volume / ref_vol) * qp.w;
      basis_at(gin, x, v, G);
      for (int i = 0; i < n; ++i) {
        double a = 0;
        for (int r = 0; r < g.dim; ++r) a += (kin * G[i][r]) * nrm[r];
        dn[i] = a;
      }
      for (int ii = 0; ii < n; ++ii)
        for (int jj = 0; jj < n; ++jj) {
          double val = -1.0 * dn[jj] * v[ii];
          val += -1.0 * p.theta * v[jj] * dn[ii];
          val += penalty * v[jj] * v[ii];
          B[ii * n + jj] += val * factor;
        }
    }
  }
  // right-hand side of a Dirichlet boundary face: LocalIntersectionIntegralFunctional with the unary
  // DirichletCoupling integrand -theta g (kappa grad psi_i . n) (local/integrands/laplace-ipdg.hh:292-320)
  // and, with bit 1, the boundary penalty's weight sigma (n . w n) / h times g psi_i
  void boundary_rhs(const Intersection& I, const Geometry& gin, double kin, const FaceParams& p, double* b) const {
    int n = fe.size;
    for (int i = 0; i < n; ++i) b[i] = 0.0;
    const Vec3& nrm = I.normal;
    double w = p.weight_is_diffusion ? kin : 1.0;
    double nn = 0;
    for (int r = 0; r < g.dim; ++r) nn += nrm[r] * nrm[r];
    const double penalty = (p.sigma_bd * (w * nn)) / p.h(I.volume);
    double v[27], G[27][3];
    for (const auto& qp : qf) {
      Vec3 x = face_global(g, I, qp.x);
      double factor = (I.volume / ref_vol) * qp.w;
      basis_at(gin, x, v, G);
      const double gx = p.g(x);
      for (int ii = 0; ii < n; ++ii) {
        double dn = 0;
        for (int r = 0; r < g.dim; ++r) dn += (kin * G[ii][r]) * nrm[r];
        double val = 0.0;
        if (p.rhs_terms & 1) val += -1.0 * p.theta * gx * dn;
        if (p.rhs_terms & 2) val += penalty * gx * v[ii];
        b[ii] += val * factor;
      }
    }
  }
};

void scatter(orc_csr* m, const int64_t* ri, const int64_t* ci, int n, const double* A) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) m->val[m->slot(ri[i], ci[j])] += A[i * n + j];
}

// element colours for the threaded walks: elements of one colour share no DoF. Cubes of equal index
// parity are two cells apart; the d! simplices of one cube share its vertices, so the simplex type is
// part of the colour.
long colour_of(const Grid& g, long e) {
  long ci[3];
  g.cell_multi(e / g.nsub, ci);
  const long par = (ci[0] & 1) | ((ci[1] & 1) << 1) | ((ci[2] & 1) << 2);
  return par * g.nsub + e % g.nsub;
}
int num_colours(const Grid& g) { return (1 << g.dim) * g.nsub; }

// all-Dirichlet boundary DoFs (DirichletConstraints::apply_local, tools/dirichlet-constraints.hh:85-110):
// the DoFs attached to subentities of boundary faces, i.e. nodes on the domain boundary.
std::vector<int64_t> dirichlet_dofs(const Grid& g, const Space& s) {
  std::vector<char> flag(s.size, 0);
  long gv[8];
  if (g.xv) {  // mapped grid (order-1 continuous spaces): the vertices of the index boundary
    std::vector<int64_t> out;
    for (long v = 0; v < g.nvert; ++v) {
      const long vi[3] = {v % g.vn[0], (v / g.vn[0]) % g.vn[1], v / (g.vn[0] * g.vn[1])};
      bool b = false;
      for (int k = 0; k < g.dim; ++k) b = b || vi[k] == 0 || vi[k] == g.n[k];
      if (b) out.push_back(v);
    }
    return out;
  }
  for (long e = 0; e < g.nelem; ++e) {
    Geometry geo = element_geometry(g, e, gv);
    for (int i = 0; i < s.lsize; ++i) {
      Vec3 x = geo.global(s.fe.nodes[i]);
      bool b = false;
      for (int k = 0; k < g.dim; ++k) {
        double tol = 1e-10 * (g.hi[k] - g.lo[k]);
        if (std::fabs(x[k] - g.lo[k]) < tol || std::fabs(x[k] - g.hi[k]) < tol) b = true;
      }
      if (b) flag[s.gi[e * s.lsize + i]] = 1;
    }
  }
  std::vector<int64_t> out;
  for (long i = 0; i < s.size; ++i)
    if (flag[i]) out.push_back(i);
  return out;
}

// DirichletConstraints::apply(M, V, only_clear=false, ensure_symmetry=true)
// (tools/dirichlet-constraints.hh:153-184): unit_col, unit_row, vector[DoF] = 0.
void apply_dirichlet(orc_csr* m, double* rhs, const std::vector<int64_t>& dofs) {
  for (int64_t D : dofs) {
    // unit_col(D): every row holding column D (pattern is symmetric: rows = columns of row D)
    for (int64_t k = m->rp[D]; k < m->rp[D + 1]; ++k) {
      long r = m->col[k];
      m->val[m->slot(r, D)] = (r == D) ? 1.0 : 0.0;
    }
    // unit_row(D)
    for (int64_t k = m->rp[D]; k < m->rp[D + 1]; ++k) m->val[k] = (m->col[k] == D) ? 1.0 : 0.0;
    if (rhs) rhs[D] = 0.0;
  }
}

void set_threads() {
#ifdef _OPENMP
  omp_set_num_threads(g_threads);
#endif
}

}  // namespace

// ============================================================== C interface ===
extern "C" long orc_num_elements(const orc_grid* gd) { return make_grid(gd).nelem; }

extern "C" long orc_space_size(const orc_grid* gd, int kind, int order) {
  Grid g = make_grid(gd);
  Space s;
  build_space(g, kind, order, s);
  return s.size;
}

extern "C" int orc_local_size(const orc_grid* gd, int kind, int order) {
  Grid g = make_grid(gd);
  if (kind == ORC_FV) return 1;
  return LagrangeFE(g.simplex && g.dim >= 2, g.dim, order).size;
}

extern "C" int orc_global_indices(const orc_grid* gd, int kind, int order, int64_t* out) {
  Grid g = make_grid(gd);
  Space s;
  build_space(g, kind, order, s);
  std::copy(s.gi.begin(), s.gi.end(), out);
  return s.lsize;
}

extern "C" long orc_dirichlet_dofs(const orc_grid* gd, int order, int64_t* out) {
  Grid g = make_grid(gd);
  Space s;
  build_space(g, ORC_CG, order, s);
  auto d = dirichlet_dofs(g, s);
  if (out) std::copy(d.begin(), d.end(), out);
  return long(d.size());
}

extern "C" orc_csr* orc_pattern(const orc_grid* gd, int kind, int order, int stencil) {
  Grid g = make_grid(gd);
  Space s;
  build_space(g, kind, order, s);
  Topology t;
  if (stencil != ORC_STENCIL_ELEMENT) build_topology(g, t);
  return build_pattern(g, s, s, stencil, &t);
}

extern "C" long orc_csr_rows(const orc_csr* m) { return m->n; }
extern "C" long orc_csr_nnz(const orc_csr* m) { return long(m->col.size()); }
extern "C" void orc_csr_export(const orc_csr* m, int64_t* rp, int32_t* col, double* val) {
  if (rp) std::copy(m->rp.begin(), m->rp.end(), rp);
  if (col) std::copy(m->col.begin(), m->col.end(), col);
  if (val) std::copy(m->val.begin(), m->val.end(), val);
}
extern "C" orc_csr* orc_csr_import(long n, const int64_t* rp, const int32_t* col, const double* val) {
  orc_csr* m = new orc_csr;
  m->n = n;
  m->rp.assign(rp, rp + n + 1);
  m->col.assign(col, col + rp[n]);
  m->val.assign(val, val + rp[n]);
  return m;
}
extern "C" void orc_csr_free(orc_csr* m) { delete m; }

extern "C" orc_csr* orc_assemble_cg(const orc_grid* gd, int order, const double* kappa, double kappa_const,
                                    const double* force, double force_const, int force_fn, int force_order,
                                    int dirichlet, double* rhs) {
  Grid g = make_grid(gd);
  Space s;
  build_space(g, ORC_CG, order, s);
  orc_csr* m = build_pattern(g, s, s, ORC_STENCIL_ELEMENT, nullptr);
  Coeffs c{kappa, kappa_const, force, force_const, force_fn, force_order};
  int k = s.fe.basis_order();
  ElementKernel K(g, s.fe, 0 + k + k, force_order + k);
  if (rhs) std::fill(rhs, rhs + s.size, 0.0);
  int n = s.lsize;
  set_threads();
  int ncol = g_threads > 1 ? num_colours(g) : 1;
  // grid walk (MatrixOperator + VectorBasedFunctional as walker functors); with threads the cells
  // are coloured by index parity so that concurrently processed elements share no DoF.
  for (int colour = 0; colour < ncol; ++colour) {
#pragma omp parallel for schedule(static) if (g_threads > 1)
    for (long e = 0; e < g.nelem; ++e) {
      if (ncol > 1 && colour_of(g, e) != colour) continue;
      double A[27 * 27], b[27];
      long gv[8];
      Geometry geo = element_geometry(g, e, gv);
      K.laplace(geo, c.k(e), A);
      const int64_t* gi = s.indices(e);
      scatter(m, gi, gi, n, A);
      if (rhs) {
        K.rhs(geo, c, e, b);
        for (int i = 0; i < n; ++i) rhs[gi[i]] += b[i];
      }
    }
  }
  if (dirichlet) apply_dirichlet(m, rhs, dirichlet_dofs(g, s));
  return m;
}

// the same walk with a d x d diffusion tensor per element (kappa_tensor[e * d * d + r * d + s])
extern "C" orc_csr* orc_assemble_cg_tensor(const orc_grid* gd, int order, const double* kappa_tensor,
                                           const double* force, double force_const, int dirichlet, double* rhs) {
  Grid g = make_grid(gd);
  Space s;
  build_space(g, ORC_CG, order, s);
  orc_csr* m = build_pattern(g, s, s, ORC_STENCIL_ELEMENT, nullptr);
  Coeffs c{nullptr, 1.0, force, force_const, ORC_FORCE_DATA, 0};
  int k = s.fe.basis_order();
  ElementKernel K(g, s.fe, 0 + k + k, k);
  if (rhs) std::fill(rhs, rhs + s.size, 0.0);
  int n = s.lsize;
  set_threads();
  int ncol = g_threads > 1 ? num_colours(g) : 1;
  for (int colour = 0; colour < ncol; ++colour) {
#pragma omp parallel for schedule(static) if (g_threads > 1)
    for (long e = 0; e < g.nelem; ++e) {
      if (ncol > 1 && colour_of(g, e) != colour) continue;
      double A[27 * 27], b[27];
      long gv[8];
      Geometry geo = element_geometry(g, e, gv);
      K.laplace_tensor(geo, kappa_tensor + e * g.dim * g.dim, A);
      const int64_t* gi = s.indices(e);
      scatter(m, gi, gi, n, A);
      if (rhs) {
        K.rhs(geo, c, e, b);
        for (int i = 0; i < n; ++i) rhs[gi[i]] += b[i];
      }
    }
  }
  if (dirichlet) apply_dirichlet(m, rhs, dirichlet_dofs(g, s));
  return m;
}

extern "C" orc_csr* orc_assemble_mass(const orc_grid* gd, int kind, int order) {
  Grid g = make_grid(gd);
  Space s;
  build_space(g, kind, order, s);
  orc_csr* m = build_pattern(g, s, s, ORC_STENCIL_ELEMENT, nullptr);
  int k = s.fe.basis_order();
  ElementKernel K(g, s.fe, k + k, k);
  double A[27 * 27];
  for (long e = 0; e < g.nelem; ++e) {
    Geometry geo = element_geometry(g, e);
    K.mass(geo, A);
    scatter(m, s.indices(e), s.indices(e), s.lsize, A);
  }
  return m;
}

extern "C" orc_csr* orc_assemble_swipdg_data(const orc_grid* gd, int order, const double* kappa,
                                             double kappa_const, const double* force, double force_const,
                                             int force_fn, int force_order, double theta, double sigma_in,
                                             double sigma_bd, int weight_is_diffusion, double beta, int gfn,
                                             double gconst, int rhs_terms, double* rhs);

extern "C" orc_csr* orc_assemble_swipdg(const orc_grid* gd, int order, const double* kappa, double kappa_const,
                                        const double* force, double force_const, int force_fn, int force_order,
                                        double theta, double sigma_in, double sigma_bd, int weight_is_diffusion,
                                        double* rhs) {
  return orc_assemble_swipdg_data(gd, order, kappa, kappa_const, force, force_const, force_fn, force_order, theta,
                                  sigma_in, sigma_bd, weight_is_diffusion, 1.0, ORC_DIRICHLET_CONST, 0.0, 0, rhs);
}

// the same with the penalty length |I|^beta and Dirichlet data on the right-hand side
extern "C" orc_csr* orc_assemble_swipdg_data(const orc_grid* gd, int order, const double* kappa,
                                             double kappa_const, const double* force, double force_const,
                                             int force_fn, int force_order, double theta, double sigma_in,
                                             double sigma_bd, int weight_is_diffusion, double beta, int gfn,
                                             double gconst, int rhs_terms, double* rhs) {
  // test/stationary-eocstudies/diffusion-ipdg.hh:283-326: element Laplace on all elements,
  // coupling terms on InnerIntersectionsOnce, Dirichlet terms on boundary intersections.
  Grid g = make_grid(gd);
  Space s;
  build_space(g, ORC_DG, order, s);
  Topology t;
  build_topology(g, t);
  orc_csr* m = build_pattern(g, s, s, ORC_STENCIL_ELEMENT_AND_INTERSECTION, &t);
  Coeffs c{kappa, kappa_const, force, force_const, force_fn, force_order};
  int k = s.fe.basis_order();
  ElementKernel K(g, s.fe, k + k, force_order + k);
  FaceKernel F(g, s.fe, k + k);
  FaceParams p{theta, sigma_in, sigma_bd, weight_is_diffusion != 0, beta, gfn, gconst, rhs_terms};
  if (rhs) std::fill(rhs, rhs + s.size, 0.0);
  int n = s.lsize;
  double A[27 * 27], B1[27 * 27], B2[27 * 27], B3[27 * 27], B4[27 * 27], b[27];
  for (long e = 0; e < g.nelem; ++e) {
    Geometry geo = element_geometry(g, e);
    K.laplace(geo, c.k(e), A);
    scatter(m, s.indices(e), s.indices(e), n, A);
    if (rhs) {
      K.rhs(geo, c, e, b);
      for (int i = 0; i < n; ++i) rhs[s.indices(e)[i]] += b[i];
    }
    for (int f = 0; f < t.nf; ++f) {
      Intersection I = make_intersection(g, t, e, f);
      if (I.outside >= 0 && !I.boundary) {
        if (!(e < I.outside)) continue;
        Geometry go = element_geometry(g, I.outside);
        F.inner(I, geo, go, c.k(e), c.k(I.outside), p, B1, B2, B3, B4);
        scatter(m, s.indices(e), s.indices(e), n, B1);
        scatter(m, s.indices(e), s.indices(I.outside), n, B2);
        scatter(m, s.indices(I.outside), s.indices(e), n, B3);
        scatter(m, s.indices(I.outside), s.indices(I.outside), n, B4);
      } else if (I.outside < 0) {
        F.boundary(I, geo, c.k(e), p, B1);
        scatter(m, s.indices(e), s.indices(e), n, B1);
        if (rhs && p.rhs_terms) {
          F.boundary_rhs(I, geo, c.k(e), p, b);
          for (int i = 0; i < n; ++i) rhs[s.indices(e)[i]] += b[i];
        }
      }
    }
  }
  return m;
}

namespace {
double swipdg_local_energy(const Grid& g, const Space& s, const Topology& t, const ElementKernel& K,
                           const FaceKernel& F, const FaceParams& p, const double* kappa, long e, double ke,
                           const double* u, const double* lam) {
  // sum over every term of the operator that involves kappa_e: lam^T B u
  int n = s.lsize;
  double A[27 * 27], B1[27 * 27], B2[27 * 27], B3[27 * 27], B4[27 * 27];
  auto quad = [&](const double* M, long r, long c) {
    const int64_t* ri = s.indices(r);
    const int64_t* ci = s.indices(c);
    double acc = 0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) acc += lam[ri[i]] * M[i * n + j] * u[ci[j]];
    return acc;
  };
  Geometry geo = element_geometry(g, e);
  K.laplace(geo, ke, A);
  double acc = quad(A, e, e);
  for (int f = 0; f < t.nf; ++f) {
    Intersection I = make_intersection(g, t, e, f);
    if (I.outside >= 0 && !I.boundary) {
      Geometry go = element_geometry(g, I.outside);
      F.inner(I, geo, go, ke, kappa[I.outside], p, B1, B2, B3, B4);
      acc += quad(B1, e, e) + quad(B2, e, I.outside) + quad(B3, I.outside, e) + quad(B4, I.outside, I.outside);
    } else if (I.outside < 0) {
      F.boundary(I, geo, ke, p, B1);
      acc += quad(B1, e, e);
    }
  }
  return acc;
}
}  // namespace

extern "C" void orc_swipdg_dlogkappa(const orc_grid* gd, int order, const double* kappa, double theta,
                                     double sigma_in, double sigma_bd, const double* u, const double* lam,
                                     double* out) {
  Grid g = make_grid(gd);
  Space s;
  build_space(g, ORC_DG, order, s);
  Topology t;
  build_topology(g, t);
  int k = s.fe.basis_order();
  ElementKernel K(g, s.fe, k + k, k);
  FaceKernel F(g, s.fe, k + k);
  FaceParams p{theta, sigma_in, sigma_bd, true};
  const double eps = 1e-3;
  for (long e = 0; e < g.nelem; ++e) {
    auto D = [&](double h) {
      double kp = kappa[e] * std::exp(h), km = kappa[e] * std::exp(-h);
      return (swipdg_local_energy(g, s, t, K, F, p, kappa, e, kp, u, lam) -
              swipdg_local_energy(g, s, t, K, F, p, kappa, e, km, u, lam)) /
             (2 * h);
    };
    double d1 = D(eps), d2 = D(eps / 2);
    out[e] = -((4.0 * d2 - d1) / 3.0);
  }
}

extern "C" void orc_cg_dlogkappa(const orc_grid* gd, int order, const double* kappa, const double* u,
                                 const double* lam, double* out) {
  Grid g = make_grid(gd);
  Space s;
  build_space(g, ORC_CG, order, s);
  int k = s.fe.basis_order();
  ElementKernel K(g, s.fe, k + k, k);
  int n = s.lsize;
  double A[27 * 27];
  for (long e = 0; e < g.nelem; ++e) {
    Geometry geo = element_geometry(g, e);
    K.laplace(geo, kappa[e], A);  // d A_e / d log kappa_e = A_e
    const int64_t* gi = s.indices(e);
    double acc = 0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) acc += lam[gi[i]] * A[i * n + j] * u[gi[j]];
    out[e] = -acc;
  }
}

// ================================================================= solvers ===
// The reference hands the solve to dune-xt-la / dune-istl (operators/matrix-based.hh:131-159),
// which are not part of the reference tree. Restated here from the published algorithms:
// preconditioned CG (Hestenes-Stiefel), BiCGStab (van der Vorst 1992), Jacobi, ILU(0).
namespace {
double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0;
  long n = long(a.size());
#pragma omp parallel for reduction(+ : s) schedule(static) if (g_threads > 1)
  for (long i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}
void spmv(const orc_csr* m, const double* x, double* y) {
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (long i = 0; i < m->n; ++i) {
    double s = 0;
    for (int64_t k = m->rp[i]; k < m->rp[i + 1]; ++k) s += m->val[k] * x[m->col[k]];
    y[i] = s;
  }
}
struct Precond {
  int kind;
  const orc_csr* A;
  std::vector<double> dinv;
  std::vector<double> lu;      // ILU(0) factors on A's pattern
  std::vector<int64_t> diag;   // position of the diagonal in each row
  Precond(const orc_csr* a, int k) : kind(k), A(a) {
    long n = a->n;
    diag.assign(n, -1);
    for (long i = 0; i < n; ++i)
      for (int64_t p = a->rp[i]; p < a->rp[i + 1]; ++p)
        if (a->col[p] == i) diag[i] = p;
    if (kind == ORC_PREC_JACOBI) {
      dinv.resize(n);
      for (long i = 0; i < n; ++i) dinv[i] = 1.0 / a->val[diag[i]];
    } else if (kind == ORC_PREC_ILU0) {
      lu = a->val;
      // IKJ ILU(0): for each row i, eliminate with rows k < i present in the pattern
      for (long i = 0; i < n; ++i) {
        for (int64_t pk = a->rp[i]; pk < a->rp[i + 1]; ++pk) {
          long k = a->col[pk];
          if (k >= i) break;
          lu[pk] /= lu[diag[k]];
          double lik = lu[pk];
          // row_i -= lik * row_k (restricted to pattern of row i, columns > k)
          int64_t pi = pk + 1;
          for (int64_t pj = diag[k] + 1; pj < a->rp[k + 1]; ++pj) {
            long j = a->col[pj];
            while (pi < a->rp[i + 1] && a->col[pi] < j) ++pi;
            if (pi < a->rp[i + 1] && a->col[pi] == j) lu[pi] -= lik * lu[pj];
          }
        }
      }
    }
  }
  void apply(const std::vector<double>& r, std::vector<double>& z) const {
    long n = A->n;
    if (kind == ORC_PREC_NONE) { z = r; return; }
    if (kind == ORC_PREC_JACOBI) {
#pragma omp parallel for schedule(static) if (g_threads > 1)
      for (long i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
      return;
    }
    // L y = r (unit lower), U z = y
    for (long i = 0; i < n; ++i) {
      double s = r[i];
      for (int64_t p = A->rp[i]; p < diag[i]; ++p) s -= lu[p] * z[A->col[p]];
      z[i] = s;
    }
    for (long i = n - 1; i >= 0; --i) {
      double s = z[i];
      for (int64_t p = diag[i] + 1; p < A->rp[i + 1]; ++p) s -= lu[p] * z[A->col[p]];
      z[i] = s / lu[diag[i]];
    }
  }
};
}  // namespace

extern "C" void orc_spmv(const orc_csr* m, const double* x, double* y) {
  set_threads();
  spmv(m, x, y);
}

extern "C" int orc_solve(const orc_csr* m, const double* b, double* x, int solver, int prec, double tol,
                         int max_iter, int* iterations, double* rel_residual) {
  set_threads();
  long n = m->n;
  Precond P(m, prec);
  std::vector<double> r(n), z(n), p(n), q(n), xv(x, x + n);
  spmv(m, xv.data(), q.data());
  for (long i = 0; i < n; ++i) r[i] = b[i] - q[i];
  double def0 = std::sqrt(dot(r, r));
  int it = 0;
  double def = def0;
  if (def0 == 0.0) {
    if (iterations) *iterations = 0;
    if (rel_residual) *rel_residual = 0.0;
    return 0;
  }
  if (solver == ORC_SOLVER_CG) {
    P.apply(r, z);
    p = z;
    double rho = dot(r, z);
    for (it = 1; it <= max_iter; ++it) {
      spmv(m, p.data(), q.data());
      double alpha = rho / dot(p, q);
#pragma omp parallel for schedule(static) if (g_threads > 1)
      for (long i = 0; i < n; ++i) { xv[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
      def = std::sqrt(dot(r, r));
      if (def / def0 <= tol) break;
      P.apply(r, z);
      double rho_new = dot(r, z);
      double beta = rho_new / rho;
      rho = rho_new;
#pragma omp parallel for schedule(static) if (g_threads > 1)
      for (long i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
  } else {
    std::vector<double> rt = r, v(n, 0.0), s(n), t(n), y(n);
    double rho = 1, alpha = 1, omega = 1;
    std::fill(p.begin(), p.end(), 0.0);
    for (it = 1; it <= max_iter; ++it) {
      double rho_new = dot(rt, r);
      double beta = (rho_new / rho) * (alpha / omega);
#pragma omp parallel for schedule(static) if (g_threads > 1)
      for (long i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
      P.apply(p, y);
      spmv(m, y.data(), v.data());
      alpha = rho_new / dot(rt, v);
#pragma omp parallel for schedule(static) if (g_threads > 1)
      for (long i = 0; i < n; ++i) { xv[i] += alpha * y[i]; s[i] = r[i] - alpha * v[i]; }
      def = std::sqrt(dot(s, s));
      if (def / def0 <= tol) { r = s; break; }
      P.apply(s, z);
      spmv(m, z.data(), t.data());
      omega = dot(t, s) / dot(t, t);
#pragma omp parallel for schedule(static) if (g_threads > 1)
      for (long i = 0; i < n; ++i) { xv[i] += omega * z[i]; r[i] = s[i] - omega * t[i]; }
      rho = rho_new;
      def = std::sqrt(dot(r, r));
      if (def / def0 <= tol) break;
    }
  }
  std::copy(xv.begin(), xv.end(), x);
  if (iterations) *iterations = it > max_iter ? max_iter : it;
  if (rel_residual) *rel_residual = def / def0;
  return (def / def0 <= tol) ? 0 : 1;
}

extern "C" double orc_h1_semi_error_esv2007(const orc_grid* gd, int kind, int order, const double* u) {
  Grid g = make_grid(gd);
  Space s;
  build_space(g, kind, order, s);
  bool sm = g.simplex && g.dim >= 2;
  auto q = quadrature(sm, g.dim, 12);
  double acc = 0;
  double dref[27][3], gex[3];
  for (long e = 0; e < g.nelem; ++e) {
    Geometry geo = element_geometry(g, e);
    const int64_t* gi = s.indices(e);
    for (const auto& qp : q) {
      double Jit[3][3];
      double det = geo.jit(qp.x, Jit);
      s.fe.grad(qp.x, dref);
      double gh[3] = {0, 0, 0};
      for (int i = 0; i < s.lsize; ++i)
        for (int r = 0; r < g.dim; ++r) {
          double v = 0;
          for (int k = 0; k < g.dim; ++k) v += Jit[r][k] * dref[i][k];
          gh[r] += u[gi[i]] * v;
        }
      esv2007_grad(geo.global(qp.x), gex);
      double d2 = 0;
      for (int r = 0; r < g.dim; ++r) d2 += (gex[r] - gh[r]) * (gex[r] - gh[r]);
      acc += d2 * det * qp.w;
    }
  }
  return std::sqrt(acc);
}

extern "C" double orc_l2_norm(const orc_grid* gd, int kind, int order, const double* u) {
  Grid g = make_grid(gd);
  Space s;
  build_space(g, kind, order, s);
  auto q = quadrature(g.simplex && g.dim >= 2, g.dim, 2 * s.fe.order + 2);
  double acc = 0, phi[27];
  for (long e = 0; e < g.nelem; ++e) {
    Geometry geo = element_geometry(g, e);
    const int64_t* gi = s.indices(e);
    for (const auto& qp : q) {
      double Jit[3][3];
      double det = geo.jit(qp.x, Jit);
      s.fe.eval(qp.x, phi);
      double v = 0;
      for (int i = 0; i < s.lsize; ++i) v += u[gi[i]] * phi[i];
      acc += v * v * det * qp.w;
    }
  }
  return std::sqrt(acc);
}

// ========================================================== finite volumes ===
namespace {
inline double flux_f(int flux, const double* vel, double u, int d) {
  return flux == ORC_FLUX_BURGERS ? 0.5 * u * u : vel[d] * u;
}
inline double flux_df(int flux, const double* vel, double u, int d) { return flux == ORC_FLUX_BURGERS ? u : vel[d]; }

// NumericalLaxFriedrichsFlux::apply (local/numerical-fluxes/lax-friedrichs.hh:61-87),
// NumericalUpwindFlux::apply (local/numerical-fluxes/upwind.hh:61-73) and
// NumericalEngquistOsherFlux::apply (local/numerical-fluxes/engquist-osher.hh:72-103), m = 1
double numerical_flux(int flux, const double* vel, int numflux, double lf_lambda, int dim, double u, double v,
                      const double* n) {
  if (numflux == ORC_NUMFLUX_LAX_FRIEDRICHS) {
    double lambda = lf_lambda;
    if (std::fabs(lambda) < 1e-15) {
      for (int dd = 0; dd < dim; ++dd) {
        lambda = std::max(lambda, std::fabs(flux_df(flux, vel, u, dd)));
        lambda = std::max(lambda, std::fabs(flux_df(flux, vel, v, dd)));
      }
      lambda = 1. / lambda;
    }
    double ret = 0.0;
    for (int dd = 0; dd < dim; ++dd) ret += (flux_f(flux, vel, u, dd) + flux_f(flux, vel, v, dd)) * (n[dd] * 0.5);
    ret += (u - v) * (0.5 / lambda);
    return ret;
  }
  if (numflux == ORC_NUMFLUX_ENGQUIST_OSHER) {
    // NumericalEngquistOsherFlux::apply (local/numerical-fluxes/engquist-osher.hh:72-103): f(0).n plus
    // int_0^u max(n.f'(s), 0) ds and int_0^v min(n.f'(s), 0) ds, each by a Gauss rule of the flux
    // order on [0, state] and only for a positive state (the reference builds the interval [0, state]
    // only then and returns 0 otherwise)
    double ret = 0.0;
    for (int dd = 0; dd < dim; ++dd) ret += flux_f(flux, vel, 0.0, dd) * n[dd];
    const int order = flux == ORC_FLUX_BURGERS ? 2 : 1;
    std::vector<double> xq, wq;
    gauss_legendre01(order / 2 + 1, xq, wq);
    auto integral = [&](double state, bool take_max) {
      if (!(state > 0.)) return 0.0;
      double acc = 0.0;
      for (size_t q = 0; q < xq.size(); ++q) {
        const double uu = state * xq[q];
        double ndf = 0.0;
        for (int dd = 0; dd < dim; ++dd) ndf += n[dd] * flux_df(flux, vel, uu, dd);
        acc += state * wq[q] * (take_max ? std::max(ndf, 0.0) : std::min(ndf, 0.0));
      }
      return acc;
    };
    return ret + integral(u, true) + integral(v, false);
  }
  double w = (u + v) / 2.;
  double nd = 0;
  for (int dd = 0; dd < dim; ++dd) nd += n[dd] * flux_df(flux, vel, w, dd);
  double s = nd > 0 ? u : v;
  double ret = 0;
  for (int dd = 0; dd < dim; ++dd) ret += flux_f(flux, vel, s, dd) * n[dd];
  return ret;
}

// LocalizableOperator::apply with LocalAdvectionFvCouplingOperator on inner and periodic
// intersections, each once (operators/advection-fv.hh:77-82, local/operators/advection-fv.hh:127-153),
// and the boundary treatments appended for the other boundary intersections
// (operators/advection-fv.hh:95-115): by extrapolation, g = numerical flux(u, v, n) with the ghost
// state v = u or v = value (LocalAdvectionFvBoundaryTreatmentByCustomExtrapolationOperator::apply,
// local/operators/advection-fv.hh:411-436), or by a boundary flux g = value
// (...ByCustomNumericalFluxOperator::apply, :279-297); range[inside] += g |I| / |E|. bkind / bval per
// side (-x, +x, -y, +y, -z, +z), null: none. A treated direction of a periodic grid is not periodic
// (the reference's periodicity restriction).
void fv_apply(const Grid& g, int flux, const double* vel, int numflux, double lf_lambda, const double* u,
              double* out, const int* bkind, const double* bval) {
  std::fill(out, out + g.nelem, 0.0);
  const double vol = g.element_volume();
  const double hinv = 1. / vol;
  for (long e = 0; e < g.nelem; ++e) {
    long ci[3];
    g.cell_multi(e, ci);
    for (int f = 0; f < 2 * g.dim; ++f) {
      int k = f / 2, side = f % 2;
      long cj[3] = {ci[0], ci[1], ci[2]};
      cj[k] += side ? 1 : -1;
      if (cj[k] < 0 || cj[k] >= g.n[k]) {
        const int kind = bkind ? bkind[f] : ORC_FV_BOUNDARY_NONE;
        const bool treated = bkind && (bkind[2 * k] != ORC_FV_BOUNDARY_NONE || bkind[2 * k + 1] != ORC_FV_BOUNDARY_NONE);
        if (g.periodic && !treated) {
          cj[k] = (cj[k] + g.n[k]) % g.n[k];
        } else {
          if (kind == ORC_FV_BOUNDARY_NONE) continue;  // no operator on this boundary
          double n[3] = {0, 0, 0};
          n[k] = side ? 1.0 : -1.0;
          double gb;
          if (kind == ORC_FV_BOUNDARY_FLUX) {
            gb = bval[f];
          } else {
            const double v = kind == ORC_FV_BOUNDARY_EXTRAPOLATE ? u[e] : bval[f];
            gb = numerical_flux(flux, vel, numflux, lf_lambda, g.dim, u[e], v, n);
          }
          double h_int = 1.0;
          for (int j = 0; j < g.dim; ++j)
            if (j != k) h_int *= g.h[j];
          out[e] += gb * (h_int / vol);
          continue;
        }
      }
      long nb = g.cell_index(cj);
      if (!(e < nb)) continue;
      double n[3] = {0, 0, 0};
      n[k] = side ? 1.0 : -1.0;
      double gval = numerical_flux(flux, vel, numflux, lf_lambda, g.dim, u[e], u[nb], n);
      double h_int = 1.0;
      for (int j = 0; j < g.dim; ++j)
        if (j != k) h_int *= g.h[j];
      const double g_ii = gval * h_int;
      out[e] += g_ii * hinv;
      out[nb] += -g_ii * hinv;
    }
  }
}
}  // namespace

extern "C" double orc_fv_estimate_dt(const orc_grid* gd, int flux, const double* vel, const double* u0) {
  // estimate_dt_for_hyperbolic_system (tools/hyperbolic.hh:38-86), m = 1, state of order 0
  Grid g = make_grid(gd);
  double data_minimum = std::numeric_limits<double>::max();
  double data_maximum = std::numeric_limits<double>::min();
  for (long e = 0; e < g.nelem; ++e) {
    data_minimum = std::min(data_minimum, u0[e]);
    data_maximum = std::max(data_maximum, u0[e]);
  }
  if (!(data_minimum < data_maximum)) data_maximum = data_minimum + 1e-6 * data_minimum;
  double max_flux_derivative = std::numeric_limits<double>::min();
  int flux_order = flux == ORC_FLUX_BURGERS ? 2 : 1;
  std::vector<double> xq, wq;
  gauss_legendre01(flux_order / 2 + 1, xq, wq);
  for (double xi : xq) {
    double uq = data_minimum + (data_maximum - data_minimum) * xi;
    for (int ss = 0; ss < g.dim; ++ss) max_flux_derivative = std::max(max_flux_derivative, std::fabs(flux_df(flux, vel, uq, ss)));
  }
  double perimeter = 0;
  for (int k = 0; k < g.dim; ++k) {
    double a = 1.0;
    for (int j = 0; j < g.dim; ++j)
      if (j != k) a *= g.h[j];
    perimeter += 2 * a;
  }
  double perimeter_over_volume = std::max(std::numeric_limits<double>::min(), perimeter / g.element_volume());
  return 1. / (perimeter_over_volume * max_flux_derivative);
}

extern "C" void orc_fv_apply(const orc_grid* gd, int flux, const double* vel, int numflux, double lf_lambda,
                             const double* u, double* out, const int* bkind, const double* bval) {
  Grid g = make_grid(gd);
  fv_apply(g, flux, vel, numflux, lf_lambda, u, out, bkind, bval);
}

extern "C" void orc_fv_explicit_euler(const orc_grid* gd, int flux, const double* vel, int numflux,
                                      double lf_lambda, double* u, double dt, long steps, const int* bkind,
                                      const double* bval) {
  // solve_instationary_system_explicit_euler (test/instationary-eocstudies/base.hh:428-447):
  // u_{n+1} = u_n - op.apply(u_n) * dt
  Grid g = make_grid(gd);
  std::vector<double> L(g.nelem);
  for (long s = 0; s < steps; ++s) {
    fv_apply(g, flux, vel, numflux, lf_lambda, u, L.data(), bkind, bval);
    for (long i = 0; i < g.nelem; ++i) u[i] = u[i] - L[i] * dt;
  }
}

extern "C" void orc_fv_ssprk2(const orc_grid* gd, int flux, const double* vel, int numflux, double lf_lambda,
                              double* u, double dt, long steps, const int* bkind, const double* bval) {
  // ExplicitRungeKuttaTimeStepper::step (tools/timestepper/explicit-rungekutta.hh:237-270) with the
  // second-order SSP tableau A = {{0,0},{1,0}}, b = {1/2,1/2} (:82-97) and r = -1.
  Grid g = make_grid(gd);
  const double r = -1.0;
  long N = g.nelem;
  std::vector<double> k0(N), k1(N), ui(N);
  for (long s = 0; s < steps; ++s) {
    fv_apply(g, flux, vel, numflux, lf_lambda, u, k0.data(), bkind, bval);
    const double a10 = dt * r * 1.0;
    for (long i = 0; i < N; ++i) ui[i] = u[i] + k0[i] * a10;
    fv_apply(g, flux, vel, numflux, lf_lambda, ui.data(), k1.data(), bkind, bval);
    const double bb = r * dt * 0.5;
    for (long i = 0; i < N; ++i) u[i] += k0[i] * bb;
    for (long i = 0; i < N; ++i) u[i] += k1[i] * bb;
  }
}

// -------------------------------------------------------------- unstructured simplex meshes ---
// A simplex grid given by its index sets (vertex coordinates, element vertex lists in index-set
// order), as the leaf view of an ALUGrid/UGGrid: the continuous P1 element loop of
// MatrixOperator::assemble (operators/matrix-based.hh:496-500) with LocalLaplaceIntegrand and the
// product right-hand side, the element pattern of make_element_sparsity_pattern
// (tools/sparsity-pattern.hh:33-50) and DirichletConstraints on the boundary vertices.
namespace {

struct Mesh {
  int dim;
  long nv, ne;
  const double* x;
  const int64_t* c;
};

// boundary vertices: the vertices of faces (an element's vertices without one of them) that belong to
// one element only, i.e. of the boundary intersections (Intersection::boundary()), ascending
std::vector<int64_t> mesh_boundary(const Mesh& M) {
  std::map<std::array<int64_t, 3>, int> faces;
  for (long e = 0; e < M.ne; ++e)
    for (int skip = 0; skip <= M.dim; ++skip) {
      std::array<int64_t, 3> f = {-1, -1, -1};
      int k = 0;
      for (int j = 0; j <= M.dim; ++j)
        if (j != skip) f[k++] = M.c[e * (M.dim + 1) + j];
      std::sort(f.begin(), f.begin() + M.dim);
      ++faces[f];
    }
  std::vector<char> flag(M.nv, 0);
  for (const auto& kv : faces)
    if (kv.second == 1)
      for (int a = 0; a < M.dim; ++a) flag[kv.first[a]] = 1;
  std::vector<int64_t> out;
  for (long v = 0; v < M.nv; ++v)
    if (flag[v]) out.push_back(v);
  return out;
}

// P1 on element e: physical gradients of the barycentric basis (the reference gradients mapped by
// J^{-T}, J = [x_1 - x_0, ..., x_d - x_0]) and the volume |det J| / d!
double mesh_gradients(const Mesh& M, long e, int64_t* w, double G[4][3]) {
  const int d = M.dim;
  double X[4][3] = {};
  for (int j = 0; j <= d; ++j) {
    w[j] = M.c[e * (d + 1) + j];
    for (int a = 0; a < d; ++a) X[j][a] = M.x[w[j] * d + a];
  }
  double J[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int k = 0; k < d; ++k)
    for (int a = 0; a < d; ++a) J[a][k] = X[k + 1][a] - X[0][a];
  // inverse by cofactors (the 2D case is the 3D one with J[2][2] = 1)
  double cof[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
      cof[r][c] = J[r1][c1] * J[r2][c2] - J[r1][c2] * J[r2][c1];
    }
  const double det = J[0][0] * cof[0][0] + J[0][1] * cof[0][1] + J[0][2] * cof[0][2];
  // (J^{-1})[k][a] = cof[a][k] / det; grad phi_j = J^{-T} e_{j-1}: component a = (J^{-1})[j-1][a]
  for (int a = 0; a < d; ++a) {
    double s0 = 0.0;
    for (int j = 1; j <= d; ++j) {
      G[j][a] = cof[a][j - 1] / det;
      s0 += G[j][a];
    }
    G[0][a] = -s0;
  }
  return std::fabs(det) / (d == 2 ? 2.0 : 6.0);
}

}  // namespace

extern "C" long orc_mesh_boundary(int dim, long nv, long ne, const int64_t* cells, int64_t* out) {
  Mesh M{dim, nv, ne, nullptr, cells};
  std::vector<int64_t> b = mesh_boundary(M);
  if (out) std::copy(b.begin(), b.end(), out);
  return long(b.size());
}

extern "C" orc_csr* orc_mesh_assemble(int dim, long nv, const double* x, long ne, const int64_t* cells,
                                      const double* kappa, double kappa_const, const double* force,
                                      double force_const, int dirichlet, double* rhs) {
  Mesh M{dim, nv, ne, x, cells};
  const int n = dim + 1;
  // element pattern: row i holds the vertices of every element that contains vertex i
  std::vector<std::vector<int32_t>> rows(nv);
  for (long e = 0; e < ne; ++e)
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) rows[cells[e * n + i]].push_back(int32_t(cells[e * n + j]));
  orc_csr* m = new orc_csr;
  m->n = nv;
  m->rp.assign(nv + 1, 0);
  for (long r = 0; r < nv; ++r) {
    std::sort(rows[r].begin(), rows[r].end());
    rows[r].erase(std::unique(rows[r].begin(), rows[r].end()), rows[r].end());
    m->rp[r + 1] = m->rp[r] + int64_t(rows[r].size());
    m->col.insert(m->col.end(), rows[r].begin(), rows[r].end());
  }
  m->val.assign(m->col.size(), 0.0);
  if (rhs) std::fill(rhs, rhs + nv, 0.0);
  for (long e = 0; e < ne; ++e) {
    int64_t w[4];
    double G[4][3] = {};
    const double vol = mesh_gradients(M, e, w, G);
    const double kv = (kappa ? kappa[e] : kappa_const) * vol;
    double A[16];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double s = 0.0;
        for (int a = 0; a < dim; ++a) s += G[i][a] * G[j][a];
        A[i * n + j] = kv * s;
      }
    scatter(m, w, w, n, A);
    if (rhs)
      for (int i = 0; i < n; ++i) rhs[w[i]] += (force ? force[e] : force_const) * vol / double(n);
  }
  if (dirichlet) apply_dirichlet(m, rhs, mesh_boundary(M));
  return m;
}

// SWIPDG with DG P1 on a triangle mesh: the element Laplace on every element, the coupling terms on
// every inner intersection once (four blocks), the Dirichlet terms on boundary intersections
// (test/stationary-eocstudies/diffusion-ipdg.hh:283-326), with the same element and face kernels as the
// structured restatement. DoF 3 e + i; face k of an element is the edge opposite its local vertex k.
extern "C" orc_csr* orc_mesh_assemble_swipdg(long nv, const double* x, long ne, const int64_t* cells,
                                             const double* kappa, double kappa_const, const double* force,
                                             double force_const, double theta, double sigma_in, double sigma_bd,
                                             int weight_is_diffusion, double beta, int gfn, double gconst,
                                             int rhs_terms, double* rhs) {
  (void)nv;
  Grid g;
  g.dim = 2;
  g.simplex = true;
  g.nelem = ne;
  LagrangeFE fe(true, 2, 1);
  Coeffs c{kappa, kappa_const, force, force_const, ORC_FORCE_DATA, 0};
  ElementKernel K(g, fe, 2, 1);
  FaceKernel F(g, fe, 2);
  FaceParams p{theta, sigma_in, sigma_bd, weight_is_diffusion != 0, beta, gfn, gconst, rhs_terms};
  // neighbours across the faces (the intersections of the grid view)
  std::vector<long> nb(size_t(ne) * 3, -1);
  std::map<std::pair<int64_t, int64_t>, std::pair<long, int>> edges;
  for (long e = 0; e < ne; ++e)
    for (int k = 0; k < 3; ++k) {
      const int a = k == 0 ? 1 : 0, b = k == 2 ? 1 : 2;
      int64_t u = cells[e * 3 + a], v = cells[e * 3 + b];
      if (u > v) std::swap(u, v);
      auto it = edges.find({u, v});
      if (it == edges.end()) {
        edges[{u, v}] = {e, k};
      } else {
        nb[size_t(e) * 3 + k] = it->second.first;
        nb[size_t(it->second.first) * 3 + it->second.second] = e;
      }
    }
  auto geometry = [&](long e) {
    Geometry geo;
    geo.dim = 2;
    geo.simplex = true;
    geo.nv = 3;
    for (int j = 0; j < 3; ++j) geo.x[j] = {x[cells[e * 3 + j] * 2], x[cells[e * 3 + j] * 2 + 1], 0.0};
    return geo;
  };
  auto intersection = [&](long e, const Geometry& geo, int k) {
    Intersection I;
    I.inside = e;
    I.face_in = k;
    I.outside = nb[size_t(e) * 3 + k];
    I.boundary = I.outside < 0;
    I.nv = 2;
    const int a = k == 0 ? 1 : 0, b = k == 2 ? 1 : 2;
    I.corners[0] = geo.x[a];
    I.corners[1] = geo.x[b];
    const double tx = geo.x[b][0] - geo.x[a][0], ty = geo.x[b][1] - geo.x[a][1];
    I.volume = std::sqrt(tx * tx + ty * ty);
    Vec3 n{ty / I.volume, -tx / I.volume, 0.0};
    if ((geo.x[k][0] - geo.x[a][0]) * n[0] + (geo.x[k][1] - geo.x[a][1]) * n[1] > 0) n = {-n[0], -n[1], 0.0};
    I.normal = n;
    return I;
  };
  // element and intersection pattern
  orc_csr* m = new orc_csr;
  m->n = 3 * ne;
  m->rp.assign(size_t(m->n) + 1, 0);
  for (long e = 0; e < ne; ++e) {
    std::vector<long> blocks = {e};
    for (int k = 0; k < 3; ++k)
      if (nb[size_t(e) * 3 + k] >= 0) blocks.push_back(nb[size_t(e) * 3 + k]);
    std::sort(blocks.begin(), blocks.end());
    for (int i = 0; i < 3; ++i) {
      for (long o : blocks)
        for (int j = 0; j < 3; ++j) m->col.push_back(int32_t(3 * o + j));
      m->rp[size_t(3 * e + i) + 1] = int64_t(m->col.size());
    }
  }
  m->val.assign(m->col.size(), 0.0);
  if (rhs) std::fill(rhs, rhs + 3 * ne, 0.0);
  double A[9], B1[9], B2[9], B3[9], B4[9], bl[3];
  auto idx = [](long e, int64_t* out) {
    for (int i = 0; i < 3; ++i) out[i] = 3 * e + i;
  };
  for (long e = 0; e < ne; ++e) {
    Geometry geo = geometry(e);
    int64_t ie[3];
    idx(e, ie);
    K.laplace(geo, c.k(e), A);
    scatter(m, ie, ie, 3, A);
    if (rhs) {
      K.rhs(geo, c, e, bl);
      for (int i = 0; i < 3; ++i) rhs[ie[i]] += bl[i];
    }
    for (int k = 0; k < 3; ++k) {
      Intersection I = intersection(e, geo, k);
      if (I.outside >= 0) {
        if (!(e < I.outside)) continue;
        Geometry go = geometry(I.outside);
        int64_t io[3];
        idx(I.outside, io);
        F.inner(I, geo, go, c.k(e), c.k(I.outside), p, B1, B2, B3, B4);
        scatter(m, ie, ie, 3, B1);
        scatter(m, ie, io, 3, B2);
        scatter(m, io, ie, 3, B3);
        scatter(m, io, io, 3, B4);
      } else {
        F.boundary(I, geo, c.k(e), p, B1);
        scatter(m, ie, ie, 3, B1);
        if (rhs && p.rhs_terms) {
          F.boundary_rhs(I, geo, c.k(e), p, bl);
          for (int i = 0; i < 3; ++i) rhs[ie[i]] += bl[i];
        }
      }
    }
  }
  return m;
}
