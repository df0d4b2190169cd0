// Continuous Lagrange spaces of order 2 (Q2 on cube grids, P2 on their Kuhn simplex split) and the
// element-batched assembly path shared by every order:
//
// * ContinuousMapper (spaces/mapper/continuous.hh:117-182) for order 2: DoFs are numbered per
//   DoF-carrying entity codim in ascending order (MCMG layout), cells by element index, vertices
//   by grid vertex index and the other codims (edges, faces) in order of first appearance in the
//   element walk. The walk is computed on the device: every (element, local node) on an edge or face
//   offers its walk position to the entity (atomicMin), entities are sorted by first position and
//   ranked.
// * Sparsity pattern (tools/sparsity-pattern.hh:33-50): the (row, column) pairs of every element's
//   DoFs, sorted and made unique on the device.
// * Local matrices (local/bilinear-forms/integrals.hh:97-134, LocalLaplaceIntegrand /
//   LocalElementProductIntegrand): for an element, A_ij = sum_q M[ij][q] c_e(q) with the contraction
//   matrix M[ij][q] = w_q |det J| (J^-T grad phi_i).(J^-T grad phi_j) (stiffness) or
//   w_q |det J| phi_i phi_j (product form), identical for all elements of one type on a structured
//   grid, and c_e(q) the coefficient at the quadrature points. A batch of elements is one small
//   GEMM, K(pairs x elements) = M(pairs x q) C(q x elements), run on the FP64 tensor cores
//   (mma.sync m8n8k4 f64), symmetric pairs i <= j only.
// * Global assembly (local/assembler/bilinear-form-assemblers.hh:110-128): coloured scatter into the
//   precomputed CSR pattern. Elements of one colour share no DoF (cube parity classes, times the
//   simplex type on simplex grids), so every colour adds without atomics and the result is
//   deterministic; positions come from a per-matrix map built once with the pattern.
//
// Reference elements (my own restatement of the Lagrange finite elements of dune-localfunctions used
// through local/finite-elements/lagrange.hh:92-143): nodes at the equidistant points (a, b, c) / k,
// lexicographic with the first coordinate fastest (a + b + c <= k on simplices); nodal basis from the
// monomials x^a y^b z^c by inverting the Vandermonde matrix. Quadrature: Gauss-Legendre tensor rules
// on cubes and Duffy-collapsed Gauss rules on simplices, of order 2k + 2 (every integrand of the path
// is a polynomial of lower degree on these affine elements, so the rule is exact).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_reduce.cuh>
#include <cub/device/device_run_length_encode.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>

#include <array>
#include <cmath>
#include <cstring>
#include <vector>

#include "highorder.cuh"
#include "linalg.cuh"
#include "structured.cuh"

namespace gdt {
namespace ho {

// ------------------------------------------------------------------ host: reference tables ---
namespace {

struct V3 {
  double x[3] = {0, 0, 0};
};

// Gauss-Legendre points and weights on [0, 1] (Newton on the Legendre polynomial), ascending
void gauss01(int m, std::vector<double>& x, std::vector<double>& w) {
  x.assign(m, 0.0);
  w.assign(m, 0.0);
  for (int i = 0; i < m; ++i) {
    const double pi = 3.14159265358979323846;
    double z = std::cos(pi * (i + 0.75) / (m + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= m; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (m == 1) p1 = z, p0 = 1.0;
      dp = m * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[m - 1 - i] = 0.5 * (1.0 + z);
    w[m - 1 - i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
}

struct QRule {
  std::vector<V3> x;
  std::vector<double> w;
};

QRule quadrature(int dim, bool simplex, int order) {
  QRule q;
  std::vector<double> a, wa, b, wb, c, wc;
  if (!simplex || dim == 1) {
    gauss01(order / 2 + 1, a, wa);
    const int m = int(a.size()), m2 = dim >= 2 ? m : 1, m3 = dim >= 3 ? m : 1;
    for (int k = 0; k < m3; ++k)
      for (int j = 0; j < m2; ++j)
        for (int i = 0; i < m; ++i) {
          V3 p;
          p.x[0] = a[i];
          if (dim >= 2) p.x[1] = a[j];
          if (dim >= 3) p.x[2] = a[k];
          q.x.push_back(p);
          q.w.push_back(wa[i] * (dim >= 2 ? wa[j] : 1.0) * (dim >= 3 ? wa[k] : 1.0));
        }
    return q;
  }
  if (dim == 2) {
    gauss01((order + 1) / 2 + 1, a, wa);
    gauss01(order / 2 + 1, b, wb);
    for (size_t i = 0; i < a.size(); ++i)
      for (size_t j = 0; j < b.size(); ++j) {
        V3 p;
        p.x[0] = a[i];
        p.x[1] = b[j] * (1.0 - a[i]);
        q.x.push_back(p);
        q.w.push_back(wa[i] * wb[j] * (1.0 - a[i]));
      }
    return q;
  }
  gauss01((order + 2) / 2 + 1, a, wa);
  gauss01((order + 1) / 2 + 1, b, wb);
  gauss01(order / 2 + 1, c, wc);
  for (size_t i = 0; i < a.size(); ++i)
    for (size_t j = 0; j < b.size(); ++j)
      for (size_t k = 0; k < c.size(); ++k) {
        V3 p;
        p.x[0] = a[i];
        p.x[1] = b[j] * (1.0 - a[i]);
        p.x[2] = c[k] * (1.0 - a[i]) * (1.0 - b[j]);
        q.x.push_back(p);
        q.w.push_back(wa[i] * wb[j] * wc[k] * (1.0 - a[i]) * (1.0 - a[i]) * (1.0 - b[j]));
      }
  return q;
}

// nodal Lagrange basis of P_k (simplex) / Q_k (cube)
struct Nodal {
  int dim = 0, order = 0, size = 0;
  bool simplex = false;
  std::vector<V3> nodes;
  std::vector<std::array<int, 3>> mono;
  std::vector<double> coef;  // coef[m * size + i]: coefficient of monomial m in phi_i

  Nodal(int d, bool s, int k) : dim(d), order(k), simplex(s) {
    const int n2 = d >= 2 ? k : 0, n3 = d >= 3 ? k : 0;
    for (int c = 0; c <= n3; ++c)
      for (int b = 0; b <= n2; ++b)
        for (int a = 0; a <= k; ++a) {
          if (s && a + b + c > k) continue;
          V3 p;
          p.x[0] = double(a) / k;
          p.x[1] = double(b) / k;
          p.x[2] = double(c) / k;
          nodes.push_back(p);
          mono.push_back({a, b, c});
        }
    size = int(nodes.size());
    const int n = size;
    std::vector<double> V(n * n), C(n * n, 0.0);
    for (int i = 0; i < n; ++i)
      for (int m = 0; m < n; ++m) V[i * n + m] = monomial(m, nodes[i]);
    for (int i = 0; i < n; ++i) C[i * n + i] = 1.0;
    for (int col = 0; col < n; ++col) {  // Gauss-Jordan with partial pivoting: C = V^-1
      int piv = col;
      for (int r = col + 1; r < n; ++r)
        if (std::fabs(V[r * n + col]) > std::fabs(V[piv * n + col])) piv = r;
      for (int j = 0; j < n; ++j) {
        std::swap(V[col * n + j], V[piv * n + j]);
        std::swap(C[col * n + j], C[piv * n + j]);
      }
      const double pv = V[col * n + col];
      for (int j = 0; j < n; ++j) {
        V[col * n + j] /= pv;
        C[col * n + j] /= pv;
      }
      for (int r = 0; r < n; ++r) {
        if (r == col || V[r * n + col] == 0.0) continue;
        const double f = V[r * n + col];
        for (int j = 0; j < n; ++j) {
          V[r * n + j] -= f * V[col * n + j];
          C[r * n + j] -= f * C[col * n + j];
        }
      }
    }
    coef = C;
  }
  static double ipow(double x, int e) {
    double r = 1.0;
    for (int i = 0; i < e; ++i) r *= x;
    return r;
  }
  double monomial(int m, const V3& x) const {
    return ipow(x.x[0], mono[m][0]) * ipow(x.x[1], mono[m][1]) * ipow(x.x[2], mono[m][2]);
  }
  void values(const V3& x, double* phi) const {
    for (int i = 0; i < size; ++i) phi[i] = 0.0;
    for (int m = 0; m < size; ++m) {
      const double v = monomial(m, x);
      for (int i = 0; i < size; ++i) phi[i] += coef[m * size + i] * v;
    }
  }
  void gradients(const V3& x, double (*g)[3]) const {
    for (int i = 0; i < size; ++i) g[i][0] = g[i][1] = g[i][2] = 0.0;
    for (int m = 0; m < size; ++m)
      for (int r = 0; r < dim; ++r) {
        const int e = mono[m][r];
        if (e == 0) continue;
        double v = e;
        for (int s = 0; s < 3; ++s) v *= ipow(x.x[s], s == r ? e - 1 : mono[m][s]);
        for (int i = 0; i < size; ++i) g[i][r] += coef[m * size + i] * v;
      }
  }
};

}  // namespace

HoSpaceInfo space_info(const GridDesc& g, int order) {
  HoSpaceInfo s;
  const bool simplex = g.simplex != 0 && g.dim >= 2;
  const Nodal fe(g.dim, simplex, order);
  s.lsize = fe.size;
  // support entity of each node: cube nodes by their half-integer coordinates, simplex nodes by
  // their nonzero barycentric coordinates
  for (int i = 0; i < fe.size; ++i) {
    int subdim = 0;
    if (!simplex) {
      for (int a = 0; a < g.dim; ++a)
        if (fe.nodes[i].x[a] != 0.0 && fe.nodes[i].x[a] != 1.0) ++subdim;
    } else {
      double l0 = 1.0;
      int nz = 0;
      for (int a = 0; a < g.dim; ++a) {
        l0 -= fe.nodes[i].x[a];
        if (fe.nodes[i].x[a] > 1e-12) ++nz;
      }
      if (l0 > 1e-12) ++nz;
      subdim = nz - 1;
    }
    s.codim[i] = g.dim - subdim;
    s.has[s.codim[i]] = 1;
  }
  // entity counts: vertices, cells, and s-faces by their corner pattern p in {0,1}^d
  // (cubes: |p| = s; simplex edges: every p != 0, the comparable corner pairs of Kuhn's split)
  for (int c = 0; c <= g.dim; ++c) {
    if (!s.has[c]) continue;
    if (c == g.dim) s.count[c] = g.nvert;
    else if (c == 0) s.count[c] = g.nelem;
    else {
      const int sub = g.dim - c;
      long long cnt = 0;
      for (int p = 1; p < (1 << g.dim); ++p) {
        const int bits = __builtin_popcount(p);
        if (simplex ? (sub != 1) : (bits != sub)) continue;
        long long k = 1;
        for (int a = 0; a < g.dim; ++a) k *= ((p >> a) & 1) ? g.n[a] : g.vn[a];
        cnt += k;
      }
      s.count[c] = cnt;
    }
  }
  long long run = 0;
  for (int c = 0; c <= g.dim; ++c) {
    s.offset[c] = run;
    if (s.has[c]) run += s.count[c];
  }
  s.size = run;
  // support corners (cube corner bit patterns) per element type
  const int ntypes = simplex ? num_sub(g.dim, true) : 1;
  s.ntypes = ntypes;
  for (int t = 0; t < ntypes; ++t)
    for (int i = 0; i < fe.size; ++i) {
      int cnt = 0;
      if (!simplex) {
        for (int v = 0; v < (1 << g.dim); ++v) {
          bool ok = true;
          for (int a = 0; a < g.dim; ++a) {
            const double x = fe.nodes[i].x[a];
            if (x == 0.0 && ((v >> a) & 1)) ok = false;
            if (x == 1.0 && !((v >> a) & 1)) ok = false;
          }
          if (ok) s.sup[t][i][cnt++] = v;
        }
      } else {
        double lam[4];
        lam[0] = 1.0;
        for (int a = 0; a < g.dim; ++a) {
          lam[a + 1] = fe.nodes[i].x[a];
          lam[0] -= fe.nodes[i].x[a];
        }
        for (int a = 0; a <= g.dim; ++a)
          if (lam[a] > 1e-12) s.sup[t][i][cnt++] = local_corner(g.dim, true, t, a);
      }
      s.nsup[t][i] = cnt;
    }
  return s;
}

QuadratureInfo quadrature_info(const GridDesc& g, int order) {
  const QRule q = quadrature(g.dim, g.simplex != 0 && g.dim >= 2, 2 * order + 2);
  QuadratureInfo r;
  r.nq = int(q.w.size());
  for (int k = 0; k < r.nq; ++k) {
    for (int a = 0; a < 3; ++a) r.x.push_back(q.x[k].x[a]);
    r.w.push_back(q.w[k]);
  }
  return r;
}

// affine map of element type t: J[:, m] = X_{m+1} - X_0 (cube: diag(h)); returns |det J|, Ji = J^-1
static double type_jacobian(const GridDesc& g, bool simplex, int t, double (&Ji)[3][3]) {
  double J[3][3] = {{0}};
  if (!simplex) {
    for (int a = 0; a < g.dim; ++a) J[a][a] = g.h[a];
  } else {
    for (int m = 0; m < g.dim; ++m) {
      const int c = local_corner(g.dim, true, t, m + 1);
      for (int a = 0; a < g.dim; ++a) J[a][m] = ((c >> a) & 1) ? g.h[a] : 0.0;
    }
  }
  for (auto& r : Ji)
    for (double& v : r) v = 0.0;
  double det = 1.0;
  if (g.dim == 1) {
    det = J[0][0];
    Ji[0][0] = 1.0 / det;
  } else if (g.dim == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    Ji[0][0] = J[1][1] / det;
    Ji[0][1] = -J[0][1] / det;
    Ji[1][0] = -J[1][0] / det;
    Ji[1][1] = J[0][0] / det;
  } else {
    det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        const int r1 = (c + 1) % 3, r2 = (c + 2) % 3, c1 = (r + 1) % 3, c2 = (r + 2) % 3;
        Ji[r][c] = (J[r1][c1] * J[r2][c2] - J[r1][c2] * J[r2][c1]) / det;
      }
  }
  return std::fabs(det);
}

BasisTables basis_tables(const GridDesc& g, int order, int quad_order) {
  BasisTables B;
  const bool simplex = g.simplex != 0 && g.dim >= 2;
  const Nodal fe(g.dim, simplex, order);
  const QRule q = quadrature(g.dim, simplex, quad_order);
  B.lsize = fe.size;
  B.nq = int(q.w.size());
  B.ntypes = simplex ? num_sub(g.dim, true) : 1;
  B.phi.assign(size_t(B.ntypes) * B.nq * B.lsize, 0.0);
  B.grad.assign(size_t(B.ntypes) * B.nq * B.lsize * 3, 0.0);
  B.wdet.assign(size_t(B.ntypes) * B.nq, 0.0);
  std::vector<double> phi(fe.size), grbuf(3 * fe.size);
  double(*gr)[3] = reinterpret_cast<double(*)[3]>(grbuf.data());
  for (int t = 0; t < B.ntypes; ++t) {
    double Ji[3][3];
    const double adet = type_jacobian(g, simplex, t, Ji);
    for (int k = 0; k < B.nq; ++k) {
      fe.values(q.x[k], phi.data());
      fe.gradients(q.x[k], gr);
      B.wdet[size_t(t) * B.nq + k] = q.w[k] * adet;
      for (int i = 0; i < fe.size; ++i) {
        B.phi[(size_t(t) * B.nq + k) * B.lsize + i] = phi[i];
        for (int a = 0; a < g.dim; ++a) {
          double v = 0.0;
          for (int r = 0; r < g.dim; ++r) v += Ji[r][a] * gr[i][r];
          B.grad[((size_t(t) * B.nq + k) * B.lsize + i) * 3 + a] = v;
        }
      }
    }
  }
  return B;
}

QuadratureInfo quadrature_info_order(const GridDesc& g, int quad_order) {
  const QRule q = quadrature(g.dim, g.simplex != 0 && g.dim >= 2, quad_order);
  QuadratureInfo r;
  r.nq = int(q.w.size());
  for (int k = 0; k < r.nq; ++k) {
    for (int a = 0; a < 3; ++a) r.x.push_back(q.x[k].x[a]);
    r.w.push_back(q.w[k]);
  }
  return r;
}

ContractionTables contraction_tables(const GridDesc& g, int order) {
  ContractionTables T;
  const bool simplex = g.simplex != 0 && g.dim >= 2;
  const Nodal fe(g.dim, simplex, order);
  const QRule q = quadrature(g.dim, simplex, 2 * order + 2);
  T.lsize = fe.size;
  T.nq = int(q.w.size());
  T.nq_pad = (T.nq + 3) / 4 * 4;
  for (int i = 0; i < T.lsize; ++i)
    for (int j = i; j < T.lsize; ++j) {
      T.pi.push_back(i);
      T.pj.push_back(j);
    }
  T.npair = int(T.pi.size());
  T.npair_pad = (T.npair + 7) / 8 * 8;
  T.ntypes = simplex ? num_sub(g.dim, true) : 1;
  const size_t msize = size_t(T.npair_pad) * T.nq_pad;
  T.stiff.assign(msize * T.ntypes, 0.0);
  T.mass.assign(msize * T.ntypes, 0.0);
  T.load.assign(size_t(T.lsize) * T.nq * T.ntypes, 0.0);
  T.ncomp = g.dim * (g.dim + 1) / 2;
  T.nqt = T.nq * T.ncomp;
  T.nqt_pad = (T.nqt + 3) / 4 * 4;
  const size_t tsize = size_t(T.npair_pad) * T.nqt_pad;
  T.stiff_t.assign(tsize * T.ntypes, 0.0);
  std::vector<double> phi(fe.size), grbuf(3 * fe.size);
  double(*gr)[3] = reinterpret_cast<double(*)[3]>(grbuf.data());
  for (int t = 0; t < T.ntypes; ++t) {
    double Ji[3][3];
    const double adet = type_jacobian(g, simplex, t, Ji);
    for (int k = 0; k < T.nq; ++k) {
      fe.values(q.x[k], phi.data());
      fe.gradients(q.x[k], gr);
      // physical gradients J^-T g
      std::vector<std::array<double, 3>> pg(fe.size);
      for (int i = 0; i < fe.size; ++i)
        for (int a = 0; a < 3; ++a) {
          double v = 0.0;
          for (int r = 0; r < g.dim; ++r) v += Ji[r][a] * gr[i][r];
          pg[i][a] = a < g.dim ? v : 0.0;
        }
      const double wq = q.w[k] * adet;
      for (int p = 0; p < T.npair; ++p) {
        const int i = T.pi[p], j = T.pj[p];
        double dot = 0.0;
        for (int a = 0; a < g.dim; ++a) dot += pg[i][a] * pg[j][a];
        T.stiff[msize * t + size_t(p) * T.nq_pad + k] = wq * dot;
        T.mass[msize * t + size_t(p) * T.nq_pad + k] = wq * phi[i] * phi[j];
        int c = 0;
        for (int a = 0; a < g.dim; ++a)
          for (int b = a; b < g.dim; ++b, ++c) {
            const double v = a == b ? pg[i][a] * pg[j][a] : pg[i][a] * pg[j][b] + pg[i][b] * pg[j][a];
            T.stiff_t[tsize * t + size_t(p) * T.nqt_pad + size_t(k) * T.ncomp + c] = wq * v;
          }
      }
      for (int i = 0; i < fe.size; ++i) T.load[(size_t(t) * T.lsize + i) * T.nq + k] = wq * phi[i];
    }
  }
  return T;
}

}  // namespace ho
}  // namespace gdt

// ---------------------------------------------------------------------- device: mapper ---
namespace gdt {
namespace {

struct HoNodes {  // node tables of HoSpaceInfo, copied to the device
  int lsize, ntypes;
  int codim[ho::kMaxL];
  int nsup[ho::kMaxTypes][ho::kMaxL];
  int sup[ho::kMaxTypes][ho::kMaxL][8];
};

constexpr unsigned long long kNone = ~0ull;

// the entity supporting node i of element e: its lowest corner vertex and its corner pattern (the
// axes along which it extends); for cube sub-faces and Kuhn sub-simplices these identify it
__device__ __forceinline__ long long entity_key(const GridDesc& g, const HoNodes& nd, long long e, int i,
                                                long long* vertex) {
  const long long cube = e / g.nsub;
  const int t = int(e % g.nsub);
  long long ci[3];
  cell_multi(g, cube, ci);
  int lo = (1 << g.dim) - 1, hi = 0;
  for (int k = 0; k < nd.nsup[t][i]; ++k) {
    lo &= nd.sup[t][i][k];
    hi |= nd.sup[t][i][k];
  }
  long long vi[3] = {ci[0] + (lo & 1), ci[1] + ((lo >> 1) & 1), ci[2] + ((lo >> 2) & 1)};
  const long long v = vi[0] + g.vn[0] * (vi[1] + g.vn[1] * vi[2]);
  if (vertex) *vertex = v;
  return v * (1LL << g.dim) + (hi & ~lo);
}

__global__ void k_entity_first(GridDesc g, HoNodes nd, int cmin, int cmax, unsigned long long* __restrict__ first,
                               long long keys_per_codim) {
  const long long n = g.nelem * nd.lsize;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < n; w += (long long)gridDim.x * blockDim.x) {
    const long long e = w / nd.lsize;
    const int i = int(w % nd.lsize);
    const int c = nd.codim[i];
    if (c < cmin || c > cmax) continue;
    const long long key = entity_key(g, nd, e, i, nullptr);
    atomicMin(first + (c - cmin) * keys_per_codim + key, (unsigned long long)w);
  }
}

__global__ void k_flag_used(long long n, const unsigned long long* __restrict__ first, unsigned char* __restrict__ flag) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    flag[k] = first[k] != kNone;
}

__global__ void k_iota(long long n, long long* __restrict__ out) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    out[k] = k;
}

__global__ void k_gather_first(long long n, const long long* __restrict__ keys, const unsigned long long* __restrict__ first,
                               unsigned long long* __restrict__ out) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    out[k] = first[keys[k]];
}

__global__ void k_rank(long long n, const long long* __restrict__ keys_sorted, int* __restrict__ num) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    num[keys_sorted[k]] = int(k);
}

__global__ void k_ho_indices(GridDesc g, HoNodes nd, int cmin, const long long* __restrict__ offset,
                             const int* __restrict__ num, long long keys_per_codim, long long* __restrict__ out64,
                             int* __restrict__ out32) {
  const long long n = g.nelem * nd.lsize;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < n; w += (long long)gridDim.x * blockDim.x) {
    const long long e = w / nd.lsize;
    const int i = int(w % nd.lsize);
    const int c = nd.codim[i];
    long long v = 0, dof;
    const long long key = entity_key(g, nd, e, i, &v);
    if (c == g.dim) dof = offset[c] + v;
    else if (c == 0) dof = offset[0] + e;
    else dof = offset[c] + num[(c - cmin) * keys_per_codim + key];
    if (out64) out64[w] = dof;
    if (out32) out32[w] = int(dof);
  }
}

HoNodes make_nodes(const ho::HoSpaceInfo& info) {
  HoNodes nd{};
  nd.lsize = info.lsize;
  nd.ntypes = info.ntypes;
  std::memcpy(nd.codim, info.codim, sizeof(nd.codim));
  std::memcpy(nd.nsup, info.nsup, sizeof(nd.nsup));
  std::memcpy(nd.sup, info.sup, sizeof(nd.sup));
  return nd;
}

int vec_grid(long long n, int num_sms) { return int(std::max(1LL, std::min<long long>((n + 255) / 256, num_sms * 8LL))); }

}  // namespace

gdt_status ho_global_indices(gdt_context ctx, const gdt_space_s& s, int64_t* out64, int32_t* out32) {
  const GridDesc& g = s.g;
  cudaStream_t st = ctx->stream;
  const ho::HoSpaceInfo info = ho::space_info(g, s.order);
  const HoNodes nd = make_nodes(info);
  // codims numbered by first appearance: 1 .. dim - 1
  int cmin = g.dim, cmax = 0;
  for (int c = 1; c < g.dim; ++c)
    if (info.has[c]) cmin = std::min(cmin, c), cmax = std::max(cmax, c);
  const long long keys = g.nvert * (1LL << g.dim);
  const int ncod = cmax >= cmin ? cmax - cmin + 1 : 0;
  std::vector<void*> allocs;
  struct Freer {
    std::vector<void*>* a;
    cudaStream_t s;
    ~Freer() {
      for (void* p : *a) cudaFreeAsync(p, s);
    }
  } freer{&allocs, st};
  auto alloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMallocAsync(&p, std::max<size_t>(bytes, 16), st) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return p;
  };
  int* num = nullptr;
  if (ncod > 0) {
    auto* first = (unsigned long long*)alloc(sizeof(unsigned long long) * keys * ncod);
    num = (int*)alloc(sizeof(int) * keys * ncod);
    auto* flag = (unsigned char*)alloc(keys);
    auto* sel = (long long*)alloc(sizeof(long long) * keys * 2);
    auto* fk = (unsigned long long*)alloc(sizeof(unsigned long long) * keys * 2);
    auto* nsel = (int*)alloc(sizeof(int));
    if (!first || !num || !flag || !sel || !fk || !nsel) return fail(ctx, GDT_ENOMEM, "order-2 mapper scratch");
    GDT_TRY_CUDA(ctx, cudaMemsetAsync(first, 0xff, sizeof(unsigned long long) * keys * ncod, st));
    k_entity_first<<<vec_grid(g.nelem * info.lsize, ctx->num_sms), 256, 0, st>>>(g, nd, cmin, cmax, first, keys);
    ctx->launches++;
    for (int c = cmin; c <= cmax; ++c) {
      if (!info.has[c]) continue;
      unsigned long long* fc = first + (c - cmin) * keys;
      k_flag_used<<<vec_grid(keys, ctx->num_sms), 256, 0, st>>>(keys, fc, flag);
      k_iota<<<vec_grid(keys, ctx->num_sms), 256, 0, st>>>(keys, sel + keys);
      // selected keys (ascending), their first positions, then sort the keys by first position
      size_t tb = 0;
      cub::DeviceSelect::Flagged(nullptr, tb, sel + keys, flag, sel, nsel, keys, st);
      size_t tb2 = 0;
      cub::DeviceRadixSort::SortPairs(nullptr, tb2, fk, fk + keys, sel, sel + keys, int(std::min<long long>(keys, INT32_MAX)), 0, 64, st);
      void* tmp = alloc(std::max(tb, tb2));
      if (!tmp) return fail(ctx, GDT_ENOMEM, "order-2 mapper scratch");
      cub::DeviceSelect::Flagged(tmp, tb, sel + keys, flag, sel, nsel, keys, st);
      int hsel = 0;
      GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&hsel, nsel, sizeof(int), cudaMemcpyDeviceToHost, st));
      GDT_TRY_CUDA(ctx, cudaStreamSynchronize(st));
      if (hsel != info.count[c]) return fail(ctx, GDT_ECUDA, "order-2 mapper: entity count mismatch");
      k_gather_first<<<vec_grid(hsel, ctx->num_sms), 256, 0, st>>>(hsel, sel, fc, fk);
      cub::DeviceRadixSort::SortPairs(tmp, tb2, fk, fk + keys, sel, sel + keys, hsel, 0, 64, st);
      k_rank<<<vec_grid(hsel, ctx->num_sms), 256, 0, st>>>(hsel, sel + keys, num + (c - cmin) * keys);
      ctx->launches += 7;
    }
  }
  long long* doff = (long long*)alloc(sizeof(long long) * 4);
  if (!doff) return fail(ctx, GDT_ENOMEM, "order-2 mapper scratch");
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(doff, info.offset, sizeof(long long) * 4, cudaMemcpyHostToDevice, st));
  k_ho_indices<<<vec_grid(g.nelem * info.lsize, ctx->num_sms), 256, 0, st>>>(g, nd, cmin, doff, num, keys,
                                                                           reinterpret_cast<long long*>(out64), out32);
  ctx->launches++;
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(st));  // the scratch (and the host offsets) outlive the kernels
  return check_launch(ctx, "order-2 global indices");
}

}  // namespace gdt

// ------------------------------------------------- device: pattern and element-batched assembly ---
namespace gdt {

// per-matrix data of the element-batched path (owned by the matrix)
struct HoMatrix {
  ho::HoSpaceInfo info;
  ho::ContractionTables tab;
  int* gi = nullptr;      // [nelem][lsize] DoF indices
  int* smap = nullptr;    // [nelem][lsize][lsize] CSR positions
  double* stiff = nullptr, *mass = nullptr, *load = nullptr;  // contraction tables (device)
  double* stiff_t = nullptr;  // tensor-diffusion table, uploaded at its first use
  int* pi = nullptr, *pj = nullptr;
};

void ho_matrix_free(HoMatrix* h) {
  if (!h) return;
  for (void* p : {(void*)h->gi, (void*)h->smap, (void*)h->stiff, (void*)h->mass, (void*)h->load, (void*)h->pi,
                  (void*)h->pj, (void*)h->stiff_t})
    if (p) cudaFree(p);
  delete h;
}

namespace {

__global__ void k_pairs(long long ne, int L, const int* __restrict__ gi, unsigned long long size,
                        unsigned long long* __restrict__ keys) {
  const long long n = ne * L * L;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < n; w += (long long)gridDim.x * blockDim.x) {
    const long long e = w / (L * L);
    const int r = int(w % (L * L)), i = r / L, j = r % L;
    keys[w] = (unsigned long long)gi[e * L + i] * size + (unsigned long long)gi[e * L + j];
  }
}

__global__ void k_split_pairs(long long nnz, const unsigned long long* __restrict__ keys, unsigned long long size,
                              int* __restrict__ row_cnt, int* __restrict__ col) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nnz; k += (long long)gridDim.x * blockDim.x) {
    const unsigned long long r = keys[k] / size;
    col[k] = int(keys[k] - r * size);
    atomicAdd(row_cnt + r, 1);
  }
}

__global__ void k_scatter_map(long long ne, int L, const int* __restrict__ gi, const int* __restrict__ rp,
                              const int* __restrict__ col, int* __restrict__ smap) {
  const long long n = ne * L * L;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < n; w += (long long)gridDim.x * blockDim.x) {
    const long long e = w / (L * L);
    const int r = int(w % (L * L)), i = r / L, j = r % L;
    const int row = gi[e * L + i], c = gi[e * L + j];
    int lo = rp[row], hi = rp[row + 1] - 1;
    while (lo < hi) {  // the pattern holds every (row, c) pair of the element
      const int mid = (lo + hi) >> 1;
      if (col[mid] < c) lo = mid + 1;
      else hi = mid;
    }
    smap[w] = lo;
  }
}

// elements of one colour: cubes whose index has parity `par` (bit a: axis a) and simplex type t
struct Colour {
  int par, t;
  long long m[3], total;
};

Colour colour_of(const GridDesc& g, int k) {
  Colour c{};
  c.t = k % g.nsub;
  c.par = k / g.nsub;
  c.total = 1;
  for (int a = 0; a < 3; ++a) {
    const long long n = a < g.dim ? g.n[a] : 1;
    const int p = a < g.dim ? (c.par >> a) & 1 : 0;
    c.m[a] = (n - p + 1) / 2;
    c.total *= c.m[a];
  }
  return c;
}

__device__ __forceinline__ long long colour_element(const GridDesc& g, const Colour& c, long long l) {
  const long long jx = l % c.m[0], jy = (l / c.m[0]) % c.m[1], jz = l / (c.m[0] * c.m[1]);
  const long long cube = (2 * jx + (c.par & 1)) + g.n[0] * ((2 * jy + ((c.par >> 1) & 1)) + g.n[1] * (2 * jz + ((c.par >> 2) & 1)));
  return cube * g.nsub + c.t;
}

// D = A B + D on the FP64 tensor cores, m8n8k4: lane l holds A[l/4][l%4], B[l%4][l/4],
// D[l/4][2 (l%4)] and D[l/4][2 (l%4) + 1]
__device__ __forceinline__ void dmma_8x8x4(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

// warp task: 8 elements of colour c and a group of kTileGroup row tiles (8 pairs each) of
// K(pairs x 8) = M(pairs x q) C(q x 8), four tiles at a time (independent accumulator chains), each
// tile scattered into val once complete
constexpr int kTileGroup = 8;

__global__ void __launch_bounds__(256) k_ho_contract(GridDesc g, Colour c, const double* __restrict__ M, int npair,
                                                     int npair_pad, int nq, int nq_pad, const int* __restrict__ pi,
                                                     const int* __restrict__ pj, const double* __restrict__ coef,
                                                     double coef_const, const double* __restrict__ coef_qp,
                                                     const int* __restrict__ smap, int L, double* __restrict__ val) {
  const int lane = threadIdx.x & 31;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const int ntile = npair_pad / 8, ngroup = (ntile + kTileGroup - 1) / kTileGroup;
  const long long ntask = (c.total + 7) / 8 * ngroup;
  for (long long task = warp; task < ntask; task += nwarps) {
    const long long base = task / ngroup * 8;
    const int t0 = int(task % ngroup) * kTileGroup, t1 = min(ntile, t0 + kTileGroup);
    const long long lb = base + (lane >> 2);
    const bool vb = lb < c.total;
    const long long eb = vb ? colour_element(g, c, lb) : 0;
    const double cb = vb ? (coef ? coef[eb] : coef_const) : 0.0;
    long long ec[2];
    bool vc[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long lc = base + 2 * (lane & 3) + h;
      vc[h] = lc < c.total;
      ec[h] = vc[h] ? colour_element(g, c, lc) : 0;
    }
    auto scatter = [&](int rt, double d0, double d1) {
      const int p = rt * 8 + (lane >> 2);
      if (p >= npair) return;
      const int i = pi[p], j = pj[p];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (!vc[h]) continue;
        const double v = h ? d1 : d0;
        const int* sm = smap + ec[h] * L * L;
        val[sm[i * L + j]] += v;
        if (i != j) val[sm[j * L + i]] += v;
      }
    };
    for (int rt = t0; rt < t1; rt += 4) {
      const int nt = min(4, t1 - rt);  // warp-uniform: up to four independent accumulator chains
      double d[4][2] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
      const double* Ma = M + size_t(rt * 8 + (lane >> 2)) * nq_pad + (lane & 3);
      for (int kt = 0; kt < nq_pad / 4; ++kt) {
        double b = cb;
        if (coef_qp) {
          const int q = kt * 4 + (lane & 3);
          b = (vb && q < nq) ? coef_qp[eb * nq + q] : 0.0;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (k < nt) dmma_8x8x4(d[k][0], d[k][1], __ldg(Ma + size_t(k) * 8 * nq_pad + kt * 4), b);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (k < nt) scatter(rt + k, d[k][0], d[k][1]);
    }
  }
}

// rhs[gi] += f_e sum_q w_q |J| phi_i(x_q), colour by colour
__global__ void k_ho_rhs(GridDesc g, Colour c, const double* __restrict__ load, int L, int nq,
                         const double* __restrict__ force, double force_const, const int* __restrict__ gi,
                         double* __restrict__ rhs) {
  const long long n = c.total * L;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < n; w += (long long)gridDim.x * blockDim.x) {
    const long long e = colour_element(g, c, w / L);
    const int i = int(w % L);
    double acc = 0.0;
    for (int q = 0; q < nq; ++q) acc += load[i * nq + q];
    rhs[gi[e * L + i]] += (force ? force[e] : force_const) * acc;
  }
}

// rhs[gi] += sum_q w_q |J| phi_i(x_q) f_e(x_q), f given at the points of a rule ([element][q]), colour by colour
__global__ void k_ho_rhs_qp(GridDesc g, Colour c, const double* __restrict__ phi, const double* __restrict__ wdet,
                            int L, int nq, const double* __restrict__ fqp, const int* __restrict__ gi,
                            double* __restrict__ rhs) {
  const long long n = c.total * L;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < n; w += (long long)gridDim.x * blockDim.x) {
    const long long e = colour_element(g, c, w / L);
    const int i = int(w % L);
    const double* fe = fqp + e * nq;
    double acc = 0.0;
    for (int q = 0; q < nq; ++q) acc = fma(wdet[q] * phi[q * L + i], fe[q], acc);
    rhs[gi[e * L + i]] += acc;
  }
}

__global__ void k_ho_boundary(GridDesc g, HoNodes nd, const int* __restrict__ gi, unsigned char* __restrict__ flag) {
  const long long n = g.nelem * nd.lsize;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < n; w += (long long)gridDim.x * blockDim.x) {
    const long long e = w / nd.lsize;
    const int i = int(w % nd.lsize), t = int(e % g.nsub);
    long long ci[3];
    cell_multi(g, e / g.nsub, ci);
    bool on = false;
    for (int a = 0; a < g.dim && !on; ++a) {
      bool lo = true, hi = true;
      for (int k = 0; k < nd.nsup[t][i]; ++k) {
        const long long x = ci[a] + ((nd.sup[t][i][k] >> a) & 1);
        lo = lo && x == 0;
        hi = hi && x == g.n[a];
      }
      on = lo || hi;
    }
    if (on) flag[gi[w]] = 1;
  }
}

__global__ void k_ho_dirichlet_rows(long long rows, const int* __restrict__ rp, const int* __restrict__ col,
                                    double* __restrict__ val, const unsigned char* __restrict__ flag,
                                    double* __restrict__ rhs) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows; r += (long long)gridDim.x * blockDim.x) {
    if (flag[r]) {
      for (int k = rp[r]; k < rp[r + 1]; ++k) val[k] = col[k] == r ? 1.0 : 0.0;
      if (rhs) rhs[r] = 0.0;
    } else {
      for (int k = rp[r]; k < rp[r + 1]; ++k)
        if (flag[col[k]]) val[k] = 0.0;
    }
  }
}

__global__ void k_ho_zero_flagged(long long n, const unsigned char* __restrict__ flag, double* __restrict__ v) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x)
    if (flag[r]) v[r] = 0.0;
}

template <class T>
T* dalloc(gdt_context ctx, size_t n, gdt_status& st) {
  T* p = nullptr;
  if (st == GDT_OK && cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) {
    st = fail(ctx, GDT_ENOMEM, "order-2 matrix data");
    p = nullptr;
  }
  return p;
}

}  // namespace

// tables, DoF map and device copies of the contraction tables of matrix m (no pattern)
static gdt_status ho_setup(gdt_context ctx, gdt_matrix m, HoMatrix** out) {
  const GridDesc& g = m->test.g;
  cudaStream_t st = ctx->stream;
  HoMatrix* h = new (std::nothrow) HoMatrix;
  if (!h) return fail(ctx, GDT_ENOMEM, "element assembly data");
  m->ho = h;
  *out = h;
  h->info = ho::space_info(g, m->test.order);
  h->tab = ho::contraction_tables(g, m->test.order);
  const int L = h->info.lsize;
  const long long ne = g.nelem;
  gdt_status s = GDT_OK;
  h->gi = dalloc<int>(ctx, size_t(ne) * L, s);
  h->smap = dalloc<int>(ctx, size_t(ne) * L * L, s);
  const ho::ContractionTables& T = h->tab;
  h->stiff = dalloc<double>(ctx, T.stiff.size(), s);
  h->mass = dalloc<double>(ctx, T.mass.size(), s);
  h->load = dalloc<double>(ctx, T.load.size(), s);
  h->pi = dalloc<int>(ctx, T.pi.size(), s);
  h->pj = dalloc<int>(ctx, T.pj.size(), s);
  if (s != GDT_OK) return s;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(h->stiff, T.stiff.data(), sizeof(double) * T.stiff.size(), cudaMemcpyHostToDevice, st));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(h->mass, T.mass.data(), sizeof(double) * T.mass.size(), cudaMemcpyHostToDevice, st));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(h->load, T.load.data(), sizeof(double) * T.load.size(), cudaMemcpyHostToDevice, st));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(h->pi, T.pi.data(), sizeof(int) * T.pi.size(), cudaMemcpyHostToDevice, st));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(h->pj, T.pj.data(), sizeof(int) * T.pj.size(), cudaMemcpyHostToDevice, st));
  return ho_global_indices(ctx, m->test, nullptr, h->gi);
}

// element-batched data for a matrix whose pattern exists already (continuous P1/Q1)
gdt_status ho_prepare(gdt_context ctx, gdt_matrix m) {
  if (m->ho) return GDT_OK;
  HoMatrix* h = nullptr;
  GDT_CHECK(ctx, ho_setup(ctx, m, &h));
  const long long ne = m->test.g.nelem;
  const int L = h->info.lsize;
  k_scatter_map<<<vec_grid(ne * L * L, ctx->num_sms), 256, 0, ctx->stream>>>(ne, L, h->gi, m->rp, m->col, h->smap);
  ctx->launches++;
  return check_launch(ctx, "element scatter map");
}

gdt_status ho_build_pattern(gdt_context ctx, gdt_matrix m) {
  const GridDesc& g = m->test.g;
  cudaStream_t st = ctx->stream;
  HoMatrix* h = nullptr;
  GDT_CHECK(ctx, ho_setup(ctx, m, &h));
  const int L = h->info.lsize;
  const long long ne = g.nelem, size = h->info.size, npairs = ne * L * L;
  // pattern: every (row, column) pair of every element, sorted, unique
  unsigned long long *keys = nullptr, *sorted = nullptr;
  int* nuniq = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&keys, sizeof(unsigned long long) * npairs));
  GDT_TRY_CUDA(ctx, cudaMalloc(&sorted, sizeof(unsigned long long) * npairs));
  GDT_TRY_CUDA(ctx, cudaMalloc(&nuniq, sizeof(int)));
  struct Freer {
    void* p[3];
    ~Freer() {
      for (void* q : p)
        if (q) cudaFree(q);
    }
  } freer{{keys, sorted, nuniq}};
  k_pairs<<<vec_grid(npairs, ctx->num_sms), 256, 0, st>>>(ne, L, h->gi, (unsigned long long)size, keys);
  int end_bit = 1;
  while (end_bit < 64 && (1ull << end_bit) < (unsigned long long)size * (unsigned long long)size) ++end_bit;
  size_t tb1 = 0, tb2 = 0;
  cub::DeviceRadixSort::SortKeys(nullptr, tb1, keys, sorted, npairs, 0, end_bit, st);
  cub::DeviceSelect::Unique(nullptr, tb2, sorted, keys, nuniq, npairs, st);
  void* tmp = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&tmp, std::max(tb1, tb2)));
  cub::DeviceRadixSort::SortKeys(tmp, tb1, keys, sorted, npairs, 0, end_bit, st);
  cub::DeviceSelect::Unique(tmp, tb2, sorted, keys, nuniq, npairs, st);
  int nnz = 0;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&nnz, nuniq, sizeof(int), cudaMemcpyDeviceToHost, st));
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(st));
  cudaFree(tmp);
  const long long rows = m->rows;
  int* row_cnt = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&m->rp, sizeof(int) * (rows + 1)));
  GDT_TRY_CUDA(ctx, cudaMalloc(&row_cnt, sizeof(int) * (rows + 1)));
  GDT_TRY_CUDA(ctx, cudaMalloc(&m->col, sizeof(int) * (nnz + 8)));
  GDT_TRY_CUDA(ctx, cudaMalloc(&m->val, sizeof(double) * (nnz + 8)));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(row_cnt, 0, sizeof(int) * (rows + 1), st));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(m->col, 0, sizeof(int) * (nnz + 8), st));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(m->val, 0, sizeof(double) * (nnz + 8), st));
  k_split_pairs<<<vec_grid(nnz, ctx->num_sms), 256, 0, st>>>(nnz, keys, (unsigned long long)size, row_cnt, m->col);
  size_t ts = 0, tm = 0;
  int* dmax = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&dmax, sizeof(int)));
  cub::DeviceScan::ExclusiveSum(nullptr, ts, row_cnt, m->rp, rows + 1, st);
  cub::DeviceReduce::Max(nullptr, tm, row_cnt, dmax, int(rows), st);
  GDT_TRY_CUDA(ctx, cudaMalloc(&tmp, std::max(ts, tm)));
  cub::DeviceScan::ExclusiveSum(tmp, ts, row_cnt, m->rp, rows + 1, st);
  cub::DeviceReduce::Max(tmp, tm, row_cnt, dmax, int(rows), st);
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&m->max_row, dmax, sizeof(int), cudaMemcpyDeviceToHost, st));
  k_scatter_map<<<vec_grid(npairs, ctx->num_sms), 256, 0, st>>>(ne, L, h->gi, m->rp, m->col, h->smap);
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(st));
  cudaFree(tmp);
  cudaFree(dmax);
  cudaFree(row_cnt);
  ctx->launches += 5;
  m->nnz = nnz;
  const double mean = rows ? double(nnz) / double(rows) : 1.0;
  m->spmv_sched = mean <= 16 ? 0 : mean <= 32 ? 1 : mean <= 64 ? 2 : 3;
  m->tuned = 0;
  return check_launch(ctx, "order-2 pattern");
}

gdt_status ho_dirichlet(gdt_context ctx, gdt_matrix m, double* rhs) {
  HoMatrix* h = static_cast<HoMatrix*>(m->ho);
  cudaStream_t st = ctx->stream;
  unsigned char* flag = nullptr;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&flag, size_t(m->rows), st));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(flag, 0, size_t(m->rows), st));
  const HoNodes nd = make_nodes(h->info);
  const GridDesc& g = m->test.g;
  k_ho_boundary<<<vec_grid(g.nelem * h->info.lsize, ctx->num_sms), 256, 0, st>>>(g, nd, h->gi, flag);
  k_ho_dirichlet_rows<<<vec_grid(m->rows, ctx->num_sms), 256, 0, st>>>(m->rows, m->rp, m->col, m->val, flag, rhs);
  GDT_TRY_CUDA(ctx, cudaFreeAsync(flag, st));
  ctx->launches += 2;
  return check_launch(ctx, "order-2 Dirichlet constraints");
}

gdt_status ho_assemble(gdt_context ctx, gdt_matrix m, int form, const double* coef, double coef_const,
                       const double* coef_qp, const double* force, double force_const, double* rhs, int dirichlet) {
  HoMatrix* h = static_cast<HoMatrix*>(m->ho);
  if (!h) return fail(ctx, GDT_EUNSUPPORTED, "matrix has no element-batched assembly data");
  cudaStream_t st = ctx->stream;
  const GridDesc& g = m->test.g;
  const ho::ContractionTables& T = h->tab;
  const int ncolours = (1 << g.dim) * g.nsub;
  const size_t msize = size_t(T.npair_pad) * T.nq_pad;
  if (m->val) GDT_TRY_CUDA(ctx, cudaMemsetAsync(m->val, 0, sizeof(double) * (m->nnz + 8), st));
  if (rhs) GDT_TRY_CUDA(ctx, cudaMemsetAsync(rhs, 0, sizeof(double) * m->rows, st));
  for (int k = 0; k < ncolours; ++k) {
    const Colour c = colour_of(g, k);
    if (c.total == 0) continue;
    const double* M = (form == 0 ? h->stiff : h->mass) + msize * c.t;
    const long long tasks = (c.total + 7) / 8 * ((T.npair_pad / 8 + kTileGroup - 1) / kTileGroup);
    const int blocks = int(std::max(1LL, std::min<long long>((tasks + 7) / 8, ctx->num_sms * 8LL)));
    k_ho_contract<<<blocks, 256, 0, st>>>(g, c, M, T.npair, T.npair_pad, T.nq, T.nq_pad, h->pi, h->pj, coef,
                                          coef_const, coef_qp, h->smap, T.lsize, m->val);
    if (rhs)
      k_ho_rhs<<<vec_grid(c.total * T.lsize, ctx->num_sms), 256, 0, st>>>(
          g, c, h->load + size_t(c.t) * T.lsize * T.nq, T.lsize, T.nq, force, force_const, h->gi, rhs);
    ctx->launches += rhs ? 2 : 1;
  }
  GDT_CHECK(ctx, check_launch(ctx, "order-2 assembly"));
  if (dirichlet) GDT_CHECK(ctx, ho_dirichlet(ctx, m, rhs));
  return GDT_OK;
}

namespace {
// the components (a <= b) of a symmetric d x d tensor per element or per quadrature point, as the
// coefficient columns (q, c) of the tensor contraction: out[e][q * ncomp + c] = kappa(e, q)[a][b]
__global__ void k_tensor_columns(long long ne, int dim, int nq, int ncomp, const double* __restrict__ kt,
                                 const double* __restrict__ kt_qp, double* __restrict__ out) {
  const long long n = ne * nq * ncomp;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < n; w += (long long)gridDim.x * blockDim.x) {
    const long long e = w / (nq * ncomp);
    const int r = int(w % (nq * ncomp)), q = r / ncomp, c = r % ncomp;
    int a = 0, b = 0, k = 0;
    for (int aa = 0; aa < dim; ++aa)
      for (int bb = aa; bb < dim; ++bb, ++k)
        if (k == c) {
          a = aa;
          b = bb;
        }
    const double* K = kt_qp ? kt_qp + ((size_t)e * nq + q) * dim * dim : kt + (size_t)e * dim * dim;
    out[w] = K[a * dim + b];
  }
}
}  // namespace

gdt_status ho_assemble_tensor(gdt_context ctx, gdt_matrix m, const double* kt, const double* kt_qp,
                              const double* force, double force_const, double* rhs, int dirichlet) {
  HoMatrix* h = static_cast<HoMatrix*>(m->ho);
  if (!h) return fail(ctx, GDT_EUNSUPPORTED, "matrix has no element-batched assembly data");
  cudaStream_t st = ctx->stream;
  const GridDesc& g = m->test.g;
  const ho::ContractionTables& T = h->tab;
  if (!h->stiff_t) {
    gdt_status s = GDT_OK;
    h->stiff_t = dalloc<double>(ctx, T.stiff_t.size(), s);
    if (s != GDT_OK) return s;
    GDT_TRY_CUDA(ctx, cudaMemcpyAsync(h->stiff_t, T.stiff_t.data(), sizeof(double) * T.stiff_t.size(),
                                      cudaMemcpyHostToDevice, st));
  }
  double* cols = nullptr;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&cols, sizeof(double) * size_t(g.nelem) * T.nqt, st));
  k_tensor_columns<<<vec_grid(g.nelem * T.nqt, ctx->num_sms), 256, 0, st>>>(g.nelem, g.dim, T.nq, T.ncomp, kt, kt_qp,
                                                                         cols);
  ctx->launches++;
  const int ncolours = (1 << g.dim) * g.nsub;
  const size_t tsize = size_t(T.npair_pad) * T.nqt_pad;
  if (m->val) GDT_TRY_CUDA(ctx, cudaMemsetAsync(m->val, 0, sizeof(double) * (m->nnz + 8), st));
  if (rhs) GDT_TRY_CUDA(ctx, cudaMemsetAsync(rhs, 0, sizeof(double) * m->rows, st));
  for (int k = 0; k < ncolours; ++k) {
    const Colour c = colour_of(g, k);
    if (c.total == 0) continue;
    const long long tasks = (c.total + 7) / 8 * ((T.npair_pad / 8 + kTileGroup - 1) / kTileGroup);
    const int blocks = int(std::max(1LL, std::min<long long>((tasks + 7) / 8, ctx->num_sms * 8LL)));
    k_ho_contract<<<blocks, 256, 0, st>>>(g, c, h->stiff_t + tsize * c.t, T.npair, T.npair_pad, T.nqt, T.nqt_pad,
                                          h->pi, h->pj, nullptr, 0.0, cols, h->smap, T.lsize, m->val);
    if (rhs)
      k_ho_rhs<<<vec_grid(c.total * T.lsize, ctx->num_sms), 256, 0, st>>>(
          g, c, h->load + size_t(c.t) * T.lsize * T.nq, T.lsize, T.nq, force, force_const, h->gi, rhs);
    ctx->launches += rhs ? 2 : 1;
  }
  GDT_TRY_CUDA(ctx, cudaFreeAsync(cols, st));
  GDT_CHECK(ctx, check_launch(ctx, "tensor diffusion assembly"));
  if (dirichlet) GDT_CHECK(ctx, ho_dirichlet(ctx, m, rhs));
  return GDT_OK;
}

gdt_status ho_assemble_rhs(gdt_context ctx, const gdt_space_s& sp, const double* force, double force_const,
                           int dirichlet, double* rhs) {
  const GridDesc& g = sp.g;
  cudaStream_t st = ctx->stream;
  const ho::HoSpaceInfo info = ho::space_info(g, sp.order);
  const ho::ContractionTables T = ho::contraction_tables(g, sp.order);
  const int L = info.lsize;
  int* gi = nullptr;
  double* load = nullptr;
  unsigned char* flag = nullptr;
  struct Freer {
    void* p[3];
    cudaStream_t s;
    ~Freer() {
      for (void* q : p)
        if (q) cudaFreeAsync(q, s);
    }
  } freer{{nullptr, nullptr, nullptr}, st};
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&gi, sizeof(int) * g.nelem * L, st));
  freer.p[0] = gi;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&load, sizeof(double) * T.load.size(), st));
  freer.p[1] = load;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(load, T.load.data(), sizeof(double) * T.load.size(), cudaMemcpyHostToDevice, st));
  GDT_CHECK(ctx, ho_global_indices(ctx, sp, nullptr, gi));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(rhs, 0, sizeof(double) * info.size, st));
  for (int k = 0; k < (1 << g.dim) * g.nsub; ++k) {
    const Colour c = colour_of(g, k);
    if (c.total == 0) continue;
    k_ho_rhs<<<vec_grid(c.total * L, ctx->num_sms), 256, 0, st>>>(g, c, load + size_t(c.t) * L * T.nq, L, T.nq, force,
                                                                  force_const, gi, rhs);
    ctx->launches++;
  }
  if (dirichlet) {
    GDT_TRY_CUDA(ctx, cudaMallocAsync(&flag, size_t(info.size), st));
    freer.p[2] = flag;
    GDT_TRY_CUDA(ctx, cudaMemsetAsync(flag, 0, size_t(info.size), st));
    k_ho_boundary<<<vec_grid(g.nelem * L, ctx->num_sms), 256, 0, st>>>(g, make_nodes(info), gi, flag);
    k_ho_zero_flagged<<<vec_grid(info.size, ctx->num_sms), 256, 0, st>>>(info.size, flag, rhs);
    ctx->launches += 2;
  }
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(st));  // the host tables outlive the copies
  return check_launch(ctx, "order-2 load vector");
}

gdt_status ho_rhs_qp(gdt_context ctx, const gdt_space_s& sp, const double* fqp, int quad_order, int dirichlet,
                     double* rhs) {
  const GridDesc& g = sp.g;
  cudaStream_t st = ctx->stream;
  const ho::HoSpaceInfo info = ho::space_info(g, sp.order);
  const ho::BasisTables B = ho::basis_tables(g, sp.order, quad_order);
  const int L = info.lsize, nq = B.nq;
  int* gi = nullptr;
  double* phi = nullptr;
  double* wdet = nullptr;
  unsigned char* flag = nullptr;
  struct Freer {
    void* p[4];
    cudaStream_t s;
    ~Freer() {
      for (void* q : p)
        if (q) cudaFreeAsync(q, s);
    }
  } freer{{nullptr, nullptr, nullptr, nullptr}, st};
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&gi, sizeof(int) * g.nelem * L, st));
  freer.p[0] = gi;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&phi, sizeof(double) * B.phi.size(), st));
  freer.p[1] = phi;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&wdet, sizeof(double) * B.wdet.size(), st));
  freer.p[2] = wdet;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(phi, B.phi.data(), sizeof(double) * B.phi.size(), cudaMemcpyHostToDevice, st));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(wdet, B.wdet.data(), sizeof(double) * B.wdet.size(), cudaMemcpyHostToDevice, st));
  GDT_CHECK(ctx, ho_global_indices(ctx, sp, nullptr, gi));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(rhs, 0, sizeof(double) * info.size, st));
  for (int k = 0; k < (1 << g.dim) * g.nsub; ++k) {
    const Colour c = colour_of(g, k);
    if (c.total == 0) continue;
    k_ho_rhs_qp<<<vec_grid(c.total * L, ctx->num_sms), 256, 0, st>>>(
        g, c, phi + size_t(c.t) * nq * L, wdet + size_t(c.t) * nq, L, nq, fqp, gi, rhs);
    ctx->launches++;
  }
  if (dirichlet) {
    GDT_TRY_CUDA(ctx, cudaMallocAsync(&flag, size_t(info.size), st));
    freer.p[3] = flag;
    GDT_TRY_CUDA(ctx, cudaMemsetAsync(flag, 0, size_t(info.size), st));
    k_ho_boundary<<<vec_grid(g.nelem * L, ctx->num_sms), 256, 0, st>>>(g, make_nodes(info), gi, flag);
    k_ho_zero_flagged<<<vec_grid(info.size, ctx->num_sms), 256, 0, st>>>(info.size, flag, rhs);
    ctx->launches += 2;
  }
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(st));  // the host tables outlive the copies
  return check_launch(ctx, "load vector at quadrature points");
}

int ho_quadrature(const gdt_space_s& sp, double* x_ref, double* w_ref) {
  const ho::QuadratureInfo q = ho::quadrature_info(sp.g, sp.order);
  for (int k = 0; k < q.nq; ++k) {
    if (x_ref)
      for (int a = 0; a < 3; ++a) x_ref[3 * k + a] = q.x[3 * k + a];
    if (w_ref) w_ref[k] = q.w[k];
  }
  return q.nq;
}

namespace {

// eta_e^2 = sum_q w_q |J| |grad u_h(x_q) - g(x_q)|^2 (norm 0) or (u_h(x_q) - v(x_q))^2 (norm 1)
__global__ void k_element_error(GridDesc g, int L, int nq, int norm, const double* __restrict__ phi,
                                const double* __restrict__ grad, const double* __restrict__ wdet,
                                const int* __restrict__ gi, const double* __restrict__ u,
                                const double* __restrict__ ref, double* __restrict__ eta2) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < g.nelem; e += (long long)gridDim.x * blockDim.x) {
    const int t = int(e % g.nsub);
    double ue[ho::kMaxL];
    for (int i = 0; i < L; ++i) ue[i] = u[gi ? gi[e * L + i] : e * L + i];
    double acc = 0.0;
    for (int q = 0; q < nq; ++q) {
      const size_t tq = size_t(t) * nq + q;
      if (norm == 0) {
        double d2 = 0.0;
        for (int a = 0; a < g.dim; ++a) {
          double v = 0.0;
          for (int i = 0; i < L; ++i) v = fma(ue[i], grad[(tq * L + i) * 3 + a], v);
          const double d = v - ref[(e * nq + q) * g.dim + a];
          d2 = fma(d, d, d2);
        }
        acc = fma(wdet[tq], d2, acc);
      } else {
        double v = 0.0;
        for (int i = 0; i < L; ++i) v = fma(ue[i], phi[tq * L + i], v);
        const double d = v - ref[e * nq + q];
        acc = fma(wdet[tq], d * d, acc);
      }
    }
    eta2[e] = acc;
  }
}

}  // namespace

gdt_status element_error(gdt_context ctx, const gdt_space_s& sp, int norm, int quad_order, const double* u,
                         const double* ref, double* eta2, double* total) {
  const GridDesc& g = sp.g;
  cudaStream_t st = ctx->stream;
  const ho::BasisTables B = ho::basis_tables(g, sp.order, quad_order);
  if (B.lsize != sp.lsize) return fail(ctx, GDT_EUNSUPPORTED, "element error: unsupported space");
  double *phi = nullptr, *grad = nullptr, *wdet = nullptr, *sum = nullptr;
  int* gi = nullptr;
  void* tmp = nullptr;
  struct Freer {
    void* p[6];
    cudaStream_t s;
    ~Freer() {
      for (void* q : p)
        if (q) cudaFreeAsync(q, s);
    }
  } freer{{}, st};
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&phi, sizeof(double) * B.phi.size(), st));
  freer.p[0] = phi;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&grad, sizeof(double) * B.grad.size(), st));
  freer.p[1] = grad;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&wdet, sizeof(double) * B.wdet.size(), st));
  freer.p[2] = wdet;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(phi, B.phi.data(), sizeof(double) * B.phi.size(), cudaMemcpyHostToDevice, st));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(grad, B.grad.data(), sizeof(double) * B.grad.size(), cudaMemcpyHostToDevice, st));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(wdet, B.wdet.data(), sizeof(double) * B.wdet.size(), cudaMemcpyHostToDevice, st));
  if (sp.kind == GDT_SPACE_CG) {
    GDT_TRY_CUDA(ctx, cudaMallocAsync(&gi, sizeof(int) * g.nelem * B.lsize, st));
    freer.p[3] = gi;
    GDT_CHECK(ctx, ho_global_indices(ctx, sp, nullptr, gi));
  }
  k_element_error<<<vec_grid(g.nelem, ctx->num_sms), 256, 0, st>>>(g, B.lsize, B.nq, norm, phi, grad, wdet, gi, u, ref,
                                                                   eta2);
  ctx->launches++;
  if (total) {
    GDT_TRY_CUDA(ctx, cudaMallocAsync(&sum, sizeof(double), st));
    freer.p[4] = sum;
    size_t tb = 0;
    cub::DeviceReduce::Sum(nullptr, tb, eta2, sum, int(g.nelem), st);
    GDT_TRY_CUDA(ctx, cudaMallocAsync(&tmp, std::max<size_t>(tb, 16), st));
    freer.p[5] = tmp;
    cub::DeviceReduce::Sum(tmp, tb, eta2, sum, int(g.nelem), st);
    double h = 0.0;
    GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&h, sum, sizeof(double), cudaMemcpyDeviceToHost, st));
    GDT_TRY_CUDA(ctx, cudaStreamSynchronize(st));
    *total = std::sqrt(h);
  }
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(st));  // the host tables outlive the copies
  return check_launch(ctx, "element error");
}

int quadrature_order(const gdt_space_s& sp, int quad_order, double* x_ref, double* w_ref) {
  const ho::QuadratureInfo q = ho::quadrature_info_order(sp.g, quad_order);
  for (int k = 0; k < q.nq; ++k) {
    if (x_ref)
      for (int a = 0; a < 3; ++a) x_ref[3 * k + a] = q.x[3 * k + a];
    if (w_ref) w_ref[k] = q.w[k];
  }
  return q.nq;
}

}  // namespace gdt
