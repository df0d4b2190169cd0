// ORACLE — test infrastructure only. CPU restatement of the reference's finite-element
// building blocks (quadrature, Lagrange finite elements, structured grids). Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may use it; the product path never does.
//
// Conventions restated from the reference and the DUNE modules it builds on:
//  * Cube grids follow YaspGrid: elements and vertices numbered lexicographically, x fastest
//    (make_cube_grid, used e.g. by examples/stationary-heat-equation.cc:87).
//  * Simplex grids follow the structured simplex factory of dune-grid: every cube is split into
//    d! simplices, one per permutation pi of the axes in std::next_permutation order, with
//    corners base, base+e_pi0, base+e_pi0+e_pi1, ... (element index = cube index * d! + perm).
//  * Reference elements: cube vertex i has coordinates (bit0, bit1, bit2) of i; cube face 2k is
//    x_k = 0 and face 2k+1 is x_k = 1; simplex vertices are 0, e_0, e_1, (e_2).
//  * Lagrange nodes are equidistant (LagrangeLocalFiniteElement<EquidistantPointSet>,
//    local/finite-elements/lagrange.hh:140-142), listed lexicographically with x fastest.
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <stdexcept>
#include <vector>

namespace orc {

using Vec3 = std::array<double, 3>;

// ------------------------------------------------------------------ quadrature ---
struct QPoint {
  Vec3 x;
  double w;
};

// Gauss-Legendre nodes/weights on [0,1] (Newton iteration on P_m; Golub-Welsch-free classic method).
inline void gauss_legendre01(int m, std::vector<double>& x, std::vector<double>& w) {
  x.assign(m, 0.0);
  w.assign(m, 0.0);
  for (int i = 0; i < m; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (m + 0.5));
    double p1 = 0, p0 = 0, dp = 1;
    for (int it = 0; it < 200; ++it) {
      p0 = 1.0;
      p1 = z;
      for (int k = 2; k <= m; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (m == 1) { p1 = z; p0 = 1.0; }
      dp = (m == 1) ? 1.0 : m * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    // recompute derivative at the converged root
    p0 = 1.0;
    p1 = z;
    for (int k = 2; k <= m; ++k) {
      double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = (m == 1) ? 1.0 : m * (z * p1 - p0) / (z * z - 1.0);
    x[i] = 0.5 * (1.0 - z);
    w[i] = 1.0 / ((1.0 - z * z) * dp * dp);  // 2/((1-z^2)P'^2) on [-1,1], halved for [0,1]
  }
  std::vector<int> idx(m);
  for (int i = 0; i < m; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return x[a] < x[b]; });
  std::vector<double> xs(m), ws(m);
  for (int i = 0; i < m; ++i) { xs[i] = x[idx[i]]; ws[i] = w[idx[i]]; }
  x = xs;
  w = ws;
}

// Rule exact for polynomials of the given (total / per-direction) order on the reference
// element of dimension dim (cube: tensor Gauss with order/2+1 points per axis; simplex: Duffy
// collapsed tensor Gauss, one extra point per collapsed axis).
inline std::vector<QPoint> quadrature(bool simplex, int dim, int order) {
  std::vector<QPoint> q;
  if (order < 0) order = 0;
  if (dim == 0) {
    q.push_back({{0, 0, 0}, 1.0});
    return q;
  }
  if (!simplex) {
    int m = order / 2 + 1;
    std::vector<double> x, w;
    gauss_legendre01(m, x, w);
    int n1 = m, n2 = dim >= 2 ? m : 1, n3 = dim >= 3 ? m : 1;
    for (int k = 0; k < n3; ++k)
      for (int j = 0; j < n2; ++j)
        for (int i = 0; i < n1; ++i) {
          QPoint p;
          p.x = {x[i], dim >= 2 ? x[j] : 0.0, dim >= 3 ? x[k] : 0.0};
          p.w = w[i] * (dim >= 2 ? w[j] : 1.0) * (dim >= 3 ? w[k] : 1.0);
          q.push_back(p);
        }
    return q;
  }
  if (dim == 1) return quadrature(false, 1, order);
  if (dim == 2) {
    std::vector<double> xs, ws, xt, wt;
    gauss_legendre01((order + 1) / 2 + 1, xs, ws);
    gauss_legendre01(order / 2 + 1, xt, wt);
    for (size_t i = 0; i < xs.size(); ++i)
      for (size_t j = 0; j < xt.size(); ++j) {
        double s = xs[i], t = xt[j];
        q.push_back({{s, t * (1.0 - s), 0.0}, ws[i] * wt[j] * (1.0 - s)});
      }
    return q;
  }
  std::vector<double> xs, ws, xt, wt, xr, wr;
  gauss_legendre01((order + 2) / 2 + 1, xs, ws);
  gauss_legendre01((order + 1) / 2 + 1, xt, wt);
  gauss_legendre01(order / 2 + 1, xr, wr);
  for (size_t i = 0; i < xs.size(); ++i)
    for (size_t j = 0; j < xt.size(); ++j)
      for (size_t k = 0; k < xr.size(); ++k) {
        double s = xs[i], t = xt[j], r = xr[k];
        q.push_back({{s, t * (1.0 - s), r * (1.0 - s) * (1.0 - t)},
                     ws[i] * wt[j] * wr[k] * (1.0 - s) * (1.0 - s) * (1.0 - t)});
      }
  return q;
}

// ------------------------------------------------------------ Lagrange elements ---
// Generic Lagrange element: nodal basis of P_k (simplex) or Q_k (cube) obtained by inverting
// the monomial Vandermonde matrix at the equidistant nodes.
struct LagrangeFE {
  bool simplex = false;
  int dim = 0, order = 0, size = 0;
  std::vector<Vec3> nodes;
  std::vector<std::array<int, 3>> monos;  // exponents
  std::vector<double> coef;               // coef[m*size + i]: coefficient of mono m in phi_i

  LagrangeFE() = default;
  LagrangeFE(bool smplx, int d, int k) : simplex(smplx), dim(d), order(k) {
    if (k == 0) {
      // P0: single node at the barycentre
      Vec3 c{0, 0, 0};
      for (int i = 0; i < d; ++i) c[i] = simplex ? 1.0 / (d + 1) : 0.5;
      nodes.push_back(c);
      monos.push_back({0, 0, 0});
      coef = {1.0};
      size = 1;
      return;
    }
    int n2 = d >= 2 ? k : 0, n3 = d >= 3 ? k : 0;
    for (int c = 0; c <= n3; ++c)
      for (int b = 0; b <= n2; ++b)
        for (int a = 0; a <= k; ++a) {
          if (simplex && a + b + c > k) continue;
          nodes.push_back({double(a) / k, double(b) / k, double(c) / k});
          monos.push_back({a, b, c});
        }
    size = int(nodes.size());
    // Vandermonde V[i][m] = mono_m(node_i); solve V * C = I  -> C[m][i]
    int n = size;
    std::vector<double> V(n * n), C(n * n, 0.0);
    for (int i = 0; i < n; ++i)
      for (int m = 0; m < n; ++m) V[i * n + m] = mono(m, nodes[i]);
    for (int i = 0; i < n; ++i) C[i * n + i] = 1.0;
    // Gauss-Jordan with partial pivoting on [V | I]
    for (int col = 0; col < n; ++col) {
      int piv = col;
      for (int r = col + 1; r < n; ++r)
        if (std::fabs(V[r * n + col]) > std::fabs(V[piv * n + col])) piv = r;
      for (int j = 0; j < n; ++j) {
        std::swap(V[col * n + j], V[piv * n + j]);
        std::swap(C[col * n + j], C[piv * n + j]);
      }
      double p = V[col * n + col];
      for (int j = 0; j < n; ++j) { V[col * n + j] /= p; C[col * n + j] /= p; }
      for (int r = 0; r < n; ++r) {
        if (r == col) continue;
        double f = V[r * n + col];
        if (f == 0.0) continue;
        for (int j = 0; j < n; ++j) { V[r * n + j] -= f * V[col * n + j]; C[r * n + j] -= f * C[col * n + j]; }
      }
    }
    // C is now V^{-1}: phi_i(x) = sum_m (V^{-1})[m][i] mono_m(x)
    coef = C;
  }
  double mono(int m, const Vec3& x) const {
    const auto& e = monos[m];
    return std::pow(x[0], e[0]) * std::pow(x[1], e[1]) * std::pow(x[2], e[2]);
  }
  void eval(const Vec3& x, double* phi) const {
    for (int i = 0; i < size; ++i) phi[i] = 0.0;
    for (int m = 0; m < size; ++m) {
      double v = mono(m, x);
      for (int i = 0; i < size; ++i) phi[i] += coef[m * size + i] * v;
    }
  }
  // reference gradients g[i][r]
  void grad(const Vec3& x, double (*g)[3]) const {
    for (int i = 0; i < size; ++i) g[i][0] = g[i][1] = g[i][2] = 0.0;
    for (int m = 0; m < size; ++m) {
      const auto& e = monos[m];
      double dv[3];
      for (int r = 0; r < 3; ++r) {
        if (e[r] == 0) { dv[r] = 0.0; continue; }
        double v = e[r];
        for (int s = 0; s < 3; ++s) v *= std::pow(x[s], s == r ? e[s] - 1 : e[s]);
        dv[r] = v;
      }
      for (int i = 0; i < size; ++i)
        for (int r = 0; r < dim; ++r) g[i][r] += coef[m * size + i] * dv[r];
    }
  }
  // polynomial order reported to quadrature-order computations (basis.order()).
  int basis_order() const { return order; }
};

// ------------------------------------------------------------------------- grid ---
struct Intersection {
  long inside = -1, outside = -1;
  int face_in = -1, face_out = -1;
  bool boundary = false;  // domain boundary (a periodic face has boundary == true and outside >= 0)
  bool periodic = false;
  Vec3 normal{0, 0, 0};   // unit outer normal of inside
  double volume = 0.0;
  int nv = 0;
  Vec3 corners[4];        // physical corners of the face (seen from inside)
};

struct Grid {
  int dim = 2;
  long n[3] = {1, 1, 1};
  double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1}, h[3] = {1, 1, 1};
  bool simplex = false, periodic = false;
  int nsub = 1;
  long ncells = 1, nelem = 1, nvert = 1;
  long vn[3] = {1, 1, 1};
  std::vector<std::array<int, 3>> perms;  // simplex permutations
  // vertex coordinates of a mapped grid ([vertex][dim], lexicographic, x fastest), or null for the
  // equidistant grid of lo, hi and n
  const double* xv = nullptr;

  Grid() = default;
  Grid(int d, const long* nn, const double* l, const double* u, bool smplx, bool per)
      : dim(d), simplex(smplx), periodic(per) {
    ncells = 1;
    nvert = 1;
    for (int i = 0; i < 3; ++i) {
      n[i] = i < d ? nn[i] : 1;
      lo[i] = i < d ? l[i] : 0.0;
      hi[i] = i < d ? u[i] : 1.0;
      h[i] = (hi[i] - lo[i]) / n[i];
      vn[i] = i < d ? n[i] + 1 : 1;
      ncells *= n[i];
      nvert *= vn[i];
    }
    nsub = 1;
    if (simplex && d >= 2) {
      std::array<int, 3> p{0, 1, 2};
      std::vector<int> q(d);
      for (int i = 0; i < d; ++i) q[i] = i;
      do {
        std::array<int, 3> a{0, 0, 0};
        for (int i = 0; i < d; ++i) a[i] = q[i];
        perms.push_back(a);
      } while (std::next_permutation(q.begin(), q.end()));
      nsub = int(perms.size());
      (void)p;
    }
    nelem = ncells * nsub;
  }
  void cell_multi(long c, long* ci) const {
    ci[0] = c % n[0];
    ci[1] = (c / n[0]) % n[1];
    ci[2] = c / (n[0] * n[1]);
  }
  long cell_index(const long* ci) const { return ci[0] + n[0] * (ci[1] + n[1] * ci[2]); }
  long vertex_index(const long* vi) const { return vi[0] + vn[0] * (vi[1] + vn[1] * vi[2]); }
  Vec3 vertex_coord(const long* vi) const {
    Vec3 x{0, 0, 0};
    if (xv) {
      const long v = vertex_index(vi);
      for (int i = 0; i < dim; ++i) x[i] = xv[v * dim + i];
      return x;
    }
    for (int i = 0; i < dim; ++i) x[i] = lo[i] + vi[i] * h[i];
    return x;
  }
  int element_nvertices() const { return simplex ? dim + 1 : (1 << dim); }
  // element vertices in reference-local order (global index + physical coordinate)
  int element_vertices(long e, long* gv, Vec3* x) const {
    long c = e / nsub;
    int s = int(e % nsub);
    long ci[3];
    cell_multi(c, ci);
    if (!simplex || dim == 1) {
      int nv = 1 << dim;
      for (int v = 0; v < nv; ++v) {
        long vi[3] = {ci[0] + (v & 1), ci[1] + (dim >= 2 ? ((v >> 1) & 1) : 0), ci[2] + (dim >= 3 ? ((v >> 2) & 1) : 0)};
        gv[v] = vertex_index(vi);
        x[v] = vertex_coord(vi);
      }
      return nv;
    }
    long vi[3] = {ci[0], ci[1], ci[2]};
    gv[0] = vertex_index(vi);
    x[0] = vertex_coord(vi);
    for (int k = 0; k < dim; ++k) {
      vi[perms[s][k]] += 1;
      gv[k + 1] = vertex_index(vi);
      x[k + 1] = vertex_coord(vi);
    }
    return dim + 1;
  }
  double element_volume() const {
    double v = 1.0;
    for (int i = 0; i < dim; ++i) v *= h[i];
    if (simplex) {
      double f = 1.0;
      for (int i = 2; i <= dim; ++i) f *= i;
      v /= f;
    }
    return v;
  }
  int num_faces() const { return simplex ? dim + 1 : 2 * dim; }
  // local vertex indices of reference face f
  int face_local_vertices(int f, int* lv) const {
    if (!simplex || dim == 1) {
      int k = f / 2, side = f % 2, cnt = 0;
      for (int v = 0; v < (1 << dim); ++v)
        if (((v >> k) & 1) == side) lv[cnt++] = v;
      return cnt;
    }
    // simplex face f is opposite vertex dim - f
    int opp = dim - f, cnt = 0;
    for (int v = 0; v <= dim; ++v)
      if (v != opp) lv[cnt++] = v;
    return cnt;
  }
};

// Affine (simplex) or multilinear (cube) geometry of one element.
struct Geometry {
  int dim;
  bool simplex;
  int nv;
  Vec3 x[8];
  Vec3 global(const Vec3& xh) const {
    Vec3 y{0, 0, 0};
    if (simplex) {
      for (int r = 0; r < dim; ++r) y[r] = x[0][r];
      for (int k = 0; k < dim; ++k)
        for (int r = 0; r < dim; ++r) y[r] += (x[k + 1][r] - x[0][r]) * xh[k];
      return y;
    }
    for (int v = 0; v < nv; ++v) {
      double N = 1.0;
      for (int k = 0; k < dim; ++k) N *= ((v >> k) & 1) ? xh[k] : (1.0 - xh[k]);
      for (int r = 0; r < dim; ++r) y[r] += N * x[v][r];
    }
    return y;
  }
  // J[r][k] = d x_r / d xh_k
  void jacobian(const Vec3& xh, double J[3][3]) const {
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 3; ++k) J[r][k] = (r == k && r >= dim) ? 1.0 : 0.0;
    if (simplex) {
      for (int k = 0; k < dim; ++k)
        for (int r = 0; r < dim; ++r) J[r][k] = x[k + 1][r] - x[0][r];
      return;
    }
    for (int v = 0; v < nv; ++v)
      for (int k = 0; k < dim; ++k) {
        double dN = ((v >> k) & 1) ? 1.0 : -1.0;
        for (int s = 0; s < dim; ++s)
          if (s != k) dN *= ((v >> s) & 1) ? xh[s] : (1.0 - xh[s]);
        for (int r = 0; r < dim; ++r) J[r][k] += dN * x[v][r];
      }
  }
  static double det3(const double J[3][3]) {
    return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  }
  // returns |det J| and fills Jit = J^{-T}
  double jit(const Vec3& xh, double Jit[3][3]) const {
    double J[3][3];
    jacobian(xh, J);
    double det = det3(J);
    double inv[3][3];
    inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
    inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
    inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 3; ++k) Jit[r][k] = inv[k][r];
    return std::fabs(det);
  }
  // inverse map for affine geometries (simplices, parallelepipeds)
  Vec3 local(const Vec3& y) const {
    Vec3 xh{0.5, 0.5, 0.5};
    if (simplex) xh = {0, 0, 0};
    for (int it = 0; it < 4; ++it) {
      Vec3 g = global(xh);
      double Jit[3][3];
      jit(xh, Jit);
      // xh += J^{-1} (y - g) ; J^{-1}[k][r] = Jit[r][k]
      Vec3 d{0, 0, 0};
      for (int k = 0; k < dim; ++k)
        for (int r = 0; r < dim; ++r) d[k] += Jit[r][k] * (y[r] - g[r]);
      for (int k = 0; k < dim; ++k) xh[k] += d[k];
    }
    for (int k = dim; k < 3; ++k) xh[k] = 0.0;
    return xh;
  }
};

inline Geometry element_geometry(const Grid& g, long e, long* gv = nullptr) {
  Geometry geo;
  geo.dim = g.dim;
  geo.simplex = g.simplex && g.dim >= 2;
  long tmp[8];
  geo.nv = g.element_vertices(e, gv ? gv : tmp, geo.x);
  return geo;
}

}  // namespace orc
