// Continuous P1/Q1 assembly on structured grids: stiffness of LocalLaplaceIntegrand(kappa)
// (local/integrands/laplace.hh:81-102 under LocalElementIntegralBilinearForm,
// local/bilinear-forms/integrals.hh:97-134), load vector of LocalElementProductIntegrand().with_ansatz(f)
// (local/functionals/integrals.hh:72-98) and DirichletConstraints::apply (tools/dirichlet-constraints.hh:153-184).
//
// Design: output-stationary. One thread owns one matrix row (one vertex); it visits the <= 2^d cells
// around its vertex, adds kappa_e * K_t[li][lj] of every element containing it into a register
// accumulator laid out over the 3^d vertex stencil, applies the Dirichlet unit row/column rule and
// writes its CSR row exactly once. No atomics and no colouring passes: each value is produced by
// exactly one thread, so the result is deterministic and the HBM traffic is one write per nonzero.
// Elements of one type t share their geometry on an equidistant grid, so the per-type local matrices
// K_t (exact integrals, equal to the reference's exact quadrature up to rounding) are kernel parameters.
#include <cmath>

#include "structured.cuh"

namespace gdt {
namespace {

constexpr int kMaxSub = 6, kMaxLoc = 8;
// per-type local matrices, passed by value (kernel parameter space) so that contexts on
// different grids never share mutable device state
struct LocalTables {
  double K[kMaxSub * kMaxLoc * kMaxLoc];
  double B[kMaxSub * kMaxLoc];
};

// host: exact local stiffness / load of element type t (P1 simplex or Q1 cube) on cells of size h
void local_matrices(const GridDesc& g, double* K, double* B) {
  const int d = g.dim, ns = g.nsub, nl = g.simplex ? d + 1 : (1 << d);
  for (int t = 0; t < ns; ++t) {
    double* Kt = K + t * kMaxLoc * kMaxLoc;
    double* Bt = B + t * kMaxLoc;
    if (g.simplex) {
      // vertices X_j = h * corner(t, j); J = [X_1 - X_0, ..., X_d - X_0]
      double X[4][3] = {};
      for (int j = 0; j < nl; ++j) {
        int c = local_corner(d, true, t, j);
        for (int a = 0; a < d; ++a) X[j][a] = ((c >> a) & 1) * g.h[a];
      }
      double J[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
      for (int k = 0; k < d; ++k)
        for (int a = 0; a < d; ++a) J[a][k] = X[k + 1][a] - X[0][a];
      double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                   J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
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
      // reference gradients: phi_0 = 1 - sum x, phi_j = x_{j-1}; physical = J^{-T} grad_ref
      double G[4][3] = {};
      for (int j = 0; j < nl; ++j)
        for (int a = 0; a < d; ++a) {
          double s = 0;
          for (int k = 0; k < d; ++k) {
            double gr = (j == 0) ? -1.0 : (k == j - 1 ? 1.0 : 0.0);
            s += inv[k][a] * gr;
          }
          G[j][a] = s;
        }
      double fact = 1;
      for (int i = 2; i <= d; ++i) fact *= i;
      double vol = std::fabs(det) / fact;
      for (int i = 0; i < nl; ++i) {
        for (int j = 0; j < nl; ++j) {
          double s = 0;
          for (int a = 0; a < d; ++a) s += G[i][a] * G[j][a];
          Kt[i * kMaxLoc + j] = vol * s;
        }
        Bt[i] = vol / (d + 1);
      }
    } else {
      // Q1 tensor product: int dpsi_p dpsi_q = +-1/h, int psi_p psi_q = h/3 or h/6
      double vol = 1;
      for (int a = 0; a < d; ++a) vol *= g.h[a];
      for (int i = 0; i < nl; ++i) {
        for (int j = 0; j < nl; ++j) {
          double s = 0;
          for (int a = 0; a < d; ++a) {
            int pa = (i >> a) & 1, qa = (j >> a) & 1;
            double term = (pa == qa ? 1.0 : -1.0) / g.h[a];
            for (int b = 0; b < d; ++b) {
              if (b == a) continue;
              int pb = (i >> b) & 1, qb = (j >> b) & 1;
              term *= g.h[b] * (pb == qb ? 1.0 / 3.0 : 1.0 / 6.0);
            }
            s += term;
          }
          Kt[i * kMaxLoc + j] = s;
        }
        Bt[i] = vol / nl;
      }
    }
  }
}

__device__ __forceinline__ bool on_boundary(const GridDesc& g, const long long* vi, int dim) {
  bool b = false;
  for (int a = 0; a < dim; ++a) b = b || vi[a] == 0 || vi[a] == g.n[a];
  return b;
}

// Row v of the assembled operator from its gathered stencil acc (slots of the 3^d neighbourhood) and
// load b: Dirichlet unit row / zero columns with the lifting of given boundary values, then the
// right-hand side entry and the CSR row (slots in ascending column order)
template <int DIM, bool SIMPLEX>
__device__ __forceinline__ void finish_row(const GridDesc& g, long long v, const long long (&vi)[3],
                                           const double (&acc)[pow3(DIM)], double b, const int* __restrict__ rp,
                                           double* __restrict__ val, double* __restrict__ rhs, int dirichlet,
                                           const double* __restrict__ gD, double gD_const) {
  constexpr int NS = pow3(DIM);
  const bool bnd = dirichlet && on_boundary(g, vi, DIM);
  // Dirichlet values g: b_v = g_v on a boundary row; elsewhere the zeroed columns move to the right-hand
  // side, b_v -= sum over boundary neighbours w of A_vw g_w (all zero for homogeneous data)
  const bool lift = dirichlet && rhs && (gD || gD_const != 0.0);
  if (lift && !bnd) {
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      if (!slot_in_stencil(DIM, SIMPLEX, k)) continue;
      long long w[3] = {0, 0, 0};
      bool ok = true;
#pragma unroll
      for (int a = 0; a < DIM; ++a) {
        w[a] = vi[a] + slot_offset(k, a);
        ok = ok && w[a] >= 0 && w[a] <= g.n[a];
      }
      if (ok && on_boundary(g, w, DIM)) b -= acc[k] * (gD ? gD[w[0] + g.vn[0] * (w[1] + g.vn[1] * w[2])] : gD_const);
    }
  }
  if (rhs) rhs[v] = bnd ? (lift ? (gD ? gD[v] : gD_const) : 0.0) : b;
  if (!val) return;
  long long pos = rp[v];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    if (!slot_in_stencil(DIM, SIMPLEX, k)) continue;
    long long w[3] = {0, 0, 0};
    bool ok = true;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      w[a] = vi[a] + slot_offset(k, a);
      ok = ok && w[a] >= 0 && w[a] <= g.n[a];
    }
    if (!ok) continue;
    double value = acc[k];
    if (dirichlet) {
      if (bnd) value = (k == center_slot(DIM)) ? 1.0 : 0.0;  // unit_row
      else if (on_boundary(g, w, DIM)) value = 0.0;          // unit_col
    }
    val[pos++] = value;
  }
}

template <int DIM, bool SIMPLEX>
__global__ void __launch_bounds__(256) assemble_cg_rows(GridDesc g, const int* __restrict__ rp, double* __restrict__ val,
                                                        double* __restrict__ rhs, const LocalTables tab,
                                                        const double* __restrict__ kappa,
                                                        double kappa_const, const double* __restrict__ force,
                                                        double force_const, int dirichlet,
                                                        const double* __restrict__ gD, double gD_const) {
  constexpr int NS = pow3(DIM), NSUB = num_sub(DIM, SIMPLEX), NLOC = num_local(DIM, SIMPLEX);
  const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (v >= g.nvert) return;
  long long vi[3];
  vertex_multi(g, v, vi);
  double acc[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) acc[k] = 0.0;
  double b = 0.0;
#pragma unroll
  for (int cv = 0; cv < (1 << DIM); ++cv) {
    // v is corner cv of cell vi - bits(cv)
    long long ci[3] = {0, 0, 0};
    bool inside = true;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      ci[a] = vi[a] - ((cv >> a) & 1);
      inside = inside && ci[a] >= 0 && ci[a] < g.n[a];
    }
    if (!inside) continue;
    const long long cell = cell_index(g, ci);
#pragma unroll
    for (int t = 0; t < NSUB; ++t) {
#pragma unroll
      for (int li = 0; li < NLOC; ++li) {
        if (local_corner(DIM, SIMPLEX, t, li) != cv) continue;
        const long long e = cell * NSUB + t;
        const double kap = kappa ? kappa[e] : kappa_const;
#pragma unroll
        for (int lj = 0; lj < NLOC; ++lj)
          acc[slot_between(DIM, cv, local_corner(DIM, SIMPLEX, t, lj))] += kap * tab.K[(t * kMaxLoc + li) * kMaxLoc + lj];
        if (rhs) b += (force ? force[e] : force_const) * tab.B[t * kMaxLoc + li];
      }
    }
  }
  finish_row<DIM, SIMPLEX>(g, v, vi, acc, b, rp, val, rhs, dirichlet, gD, gD_const);
}

// Mapped grids (vertex coordinates g.xv) in two passes, so that each element's geometry is formed once:
// 1. mapped_cell_tables: one thread per cube forms J, J^{-1} and |det J| of its elements from its own
//    corners, as DefaultGlobalBasis::jacobians does from the element geometry
//    (spaces/basis/default.hh:152-175), with the quadrature of LocalElementIntegralBilinearForm at the
//    integrand's order (local/bilinear-forms/integrals.hh:97-134), and writes the cube's local stiffness
//    (kappa included; entries (i, j), i <= j, of its 2^d corners, entry-major so that a warp's stores are
//    contiguous) and its load per corner:
//    - simplices (P1, affine): grad phi_j = J^{-T} grad phi_hat_j is constant; the stiffness
//      kappa |det J| / d! grad phi_i . grad phi_j and the load f |det J| / (d! (d + 1)) are exact, and
//      the d! simplices of a cube are summed into its corner pairs (only corners whose bit sets are
//      nested share a simplex);
//    - cubes (Q1, multilinear map): the stiffness at the 2^d Gauss points of order 2 (two per axis, J,
//      J^{-1} and |det J| at each point), the load of a source per element at the one-point rule of
//      order 1 (the element centre: phi_i = 2^{-d} there), the same for every corner.
// 2. assemble_cg_rows_tabled: the output-stationary row gather of the equidistant kernel, reading the
//    tables of the <= 2^d cubes around the row's vertex instead of per-type constants.
template <int DIM>
__device__ __forceinline__ double inv_det(const double (&J)[DIM][DIM], double (&Ji)[DIM][DIM]) {
  if constexpr (DIM == 1) {
    Ji[0][0] = 1.0 / J[0][0];
    return J[0][0];
  } else if constexpr (DIM == 2) {
    const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double r = 1.0 / det;
    Ji[0][0] = J[1][1] * r;
    Ji[0][1] = -J[0][1] * r;
    Ji[1][0] = -J[1][0] * r;
    Ji[1][1] = J[0][0] * r;
    return det;
  } else {
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1], c01 = J[0][2] * J[2][1] - J[0][1] * J[2][2],
                 c02 = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    const double det = J[0][0] * c00 + J[1][0] * c01 + J[2][0] * c02;
    const double r = 1.0 / det;
    Ji[0][0] = c00 * r;
    Ji[0][1] = c01 * r;
    Ji[0][2] = c02 * r;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * r;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * r;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
    return det;
  }
}

// entry of corner pair (i, j) in the cube table: the upper triangle, row by row
__host__ __device__ constexpr int pair_entry(int nc, int i, int j) {
  return i <= j ? i * nc - i * (i - 1) / 2 + (j - i) : j * nc - j * (j - 1) / 2 + (i - j);
}
// do cube corners i and j share an element? (all pairs of a cube; nested bit sets for the Kuhn split)
__host__ __device__ constexpr bool pair_shared(bool simplex, int i, int j) {
  return !simplex || (i & j) == i || (i & j) == j;
}

// 1D factors of the trilinear shape functions at the two Gauss points g_0, g_1 of order 2 on [0, 1]
// ((3 -+ sqrt 3) / 6): ell_x(g_q) = 1 - g_q for x = 0, g_q for x = 1; q1_pair(e, q) the product of two
// of them by pair class e = 0: (0, 0), 1: (0, 1) or (1, 0), 2: (1, 1)
constexpr double kGauss0 = 0.21132486540518711775, kGauss1 = 0.78867513459481288225;
__host__ __device__ constexpr double q1_ell(int x, int q) {
  return x == 0 ? 1.0 - (q == 0 ? kGauss0 : kGauss1) : (q == 0 ? kGauss0 : kGauss1);
}
__host__ __device__ constexpr double q1_pair(int e, int q) {
  return e == 0 ? q1_ell(0, q) * q1_ell(0, q) : e == 1 ? q1_ell(0, q) * q1_ell(1, q) : q1_ell(1, q) * q1_ell(1, q);
}
__host__ __device__ constexpr int q1_class(int x, int y) { return x + y; }
__host__ __device__ constexpr double q1_sign(int x) { return x ? 1.0 : -1.0; }
// the other two axes of axis k, ascending
__host__ __device__ constexpr int q1_other(int k, int m) { return k == 0 ? 1 + m : (k == 1 ? 2 * m : m); }

// Local Q1 stiffness of a trilinear hexahedron (corners X, coefficient kap) in sum-factorised form,
// written as the upper triangle of its corner pairs to tm (entry-major, stride nc). The same integral
// as the direct 8-point loop (2 x 2 x 2 Gauss points, J, J^{-1} and |det J| at each) in about half the
// FP64 operations:
//   M_q = kap w |det J| J^{-1} J^{-T} = kap w adj(J) adj(J)^T / |det J| (w = 1/8) at every point q;
//   A_ij = sum_q sum_ab M_q[a][b] d_a phi_i(q) d_b phi_j(q), with d_a phi_i = s(i_a) prod_{k != a}
//   ell_{i_k}: the diagonal terms a = b need sum over q_a of M_q[a][a] against the pair classes of the
//   two other axes (T_a, 3 x 3 values), the mixed terms a < b the sums W_ab[x][y][e] of M_q[a][b]
//   ell_x(q_a) ell_y(q_b) pair_e(q_c) (2 x 2 x 3 values, contracted one axis at a time), and
//   A_ij = sum_a s(i_a) s(j_a) T_a[e_b][e_c] + sum_{a<b} (s(i_a) s(j_b) W_ab[j_a][i_b][e_c] +
//   s(i_b) s(j_a) W_ab[i_a][j_b][e_c]).
// Column k of J at a Gauss point depends only on the other two coordinates, so the 12 distinct
// columns are formed once from the 12 edge vectors.
__device__ __forceinline__ void q1_hex_stiffness(const double (&X)[8][3], double kap, double* __restrict__ tm,
                                                 long long nc, long long cell) {
  double Jc[3][2][2][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int o1 = q1_other(k, 0), o2 = q1_other(k, 1);
#pragma unroll
    for (int q1 = 0; q1 < 2; ++q1)
#pragma unroll
      for (int q2 = 0; q2 < 2; ++q2)
#pragma unroll
        for (int a = 0; a < 3; ++a) Jc[k][q1][q2][a] = 0.0;
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const int c0 = (u << o1) | (v << o2), c1 = c0 | (1 << k);
        double E[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) E[a] = X[c1][a] - X[c0][a];
#pragma unroll
        for (int q1 = 0; q1 < 2; ++q1)
#pragma unroll
          for (int q2 = 0; q2 < 2; ++q2) {
            const double wgt = q1_ell(u, q1) * q1_ell(v, q2);
#pragma unroll
            for (int a = 0; a < 3; ++a) Jc[k][q1][q2][a] = fma(wgt, E[a], Jc[k][q1][q2][a]);
          }
      }
  }
  // M_q: components 00, 11, 22, 01, 02, 12 at point q = q0 | q1 << 1 | q2 << 2
  double Mq[6][8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int qb[3] = {q & 1, (q >> 1) & 1, (q >> 2) & 1};
    double J[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int a = 0; a < 3; ++a) J[a][k] = Jc[k][qb[q1_other(k, 0)]][qb[q1_other(k, 1)]][a];
    double ad[3][3];  // adj(J) = det J * J^{-1}
    ad[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    ad[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    ad[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    ad[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    ad[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    ad[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    ad[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    ad[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    ad[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double det = J[0][0] * ad[0][0] + J[0][1] * ad[1][0] + J[0][2] * ad[2][0];
    const double f = (0.125 * kap) / fabs(det);
    constexpr int ka[6] = {0, 1, 2, 0, 0, 1}, kb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int m = 0; m < 6; ++m)
      Mq[m][q] = f * fma(ad[ka[m]][0], ad[kb[m]][0], fma(ad[ka[m]][1], ad[kb[m]][1], ad[ka[m]][2] * ad[kb[m]][2]));
  }
  // T_a[e_b][e_c] (a = b terms)
  double T[3][3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int b = q1_other(a, 0), c = q1_other(a, 1);
    double mm[2][2];
#pragma unroll
    for (int qb = 0; qb < 2; ++qb)
#pragma unroll
      for (int qc = 0; qc < 2; ++qc) mm[qb][qc] = Mq[a][(qb << b) | (qc << c)] + Mq[a][(1 << a) | (qb << b) | (qc << c)];
#pragma unroll
    for (int eb = 0; eb < 3; ++eb) {
      double u[2];
#pragma unroll
      for (int qc = 0; qc < 2; ++qc) u[qc] = fma(mm[0][qc], q1_pair(eb, 0), mm[1][qc] * q1_pair(eb, 1));
#pragma unroll
      for (int ec = 0; ec < 3; ++ec) T[a][eb][ec] = fma(u[0], q1_pair(ec, 0), u[1] * q1_pair(ec, 1));
    }
  }
  // W_ab[x][y][e_c] (a < b terms), one axis at a time: pair m = 3 (01), 4 (02), 5 (12)
  double W[3][2][2][3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const int a = m == 2 ? 1 : 0, b = m == 0 ? 1 : 2, c = 3 - a - b;
    double Y[2][2][2];  // [x][q_b][q_c]
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
      for (int qb = 0; qb < 2; ++qb)
#pragma unroll
        for (int qc = 0; qc < 2; ++qc)
          Y[x][qb][qc] = fma(Mq[3 + m][(qb << b) | (qc << c)], q1_ell(x, 0),
                             Mq[3 + m][(1 << a) | (qb << b) | (qc << c)] * q1_ell(x, 1));
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
      for (int y = 0; y < 2; ++y) {
        double Z[2];
#pragma unroll
        for (int qc = 0; qc < 2; ++qc) Z[qc] = fma(Y[x][0][qc], q1_ell(y, 0), Y[x][1][qc] * q1_ell(y, 1));
#pragma unroll
        for (int e = 0; e < 3; ++e) W[m][x][y][e] = fma(Z[0], q1_pair(e, 0), Z[1] * q1_pair(e, 1));
      }
  }
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = i; j < 8; ++j) {
      const int bi[3] = {i & 1, (i >> 1) & 1, (i >> 2) & 1}, bj[3] = {j & 1, (j >> 1) & 1, (j >> 2) & 1};
      double v = 0.0;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const int b = q1_other(a, 0), c = q1_other(a, 1);
        v += q1_sign(bi[a]) * q1_sign(bj[a]) * T[a][q1_class(bi[b], bj[b])][q1_class(bi[c], bj[c])];
      }
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const int a = m == 2 ? 1 : 0, b = m == 0 ? 1 : 2, c = 3 - a - b;
        const int e = q1_class(bi[c], bj[c]);
        v += q1_sign(bi[a]) * q1_sign(bj[b]) * W[m][bj[a]][bi[b]][e];
        v += q1_sign(bi[b]) * q1_sign(bj[a]) * W[m][bi[a]][bj[b]][e];
      }
      tm[pair_entry(8, i, j) * nc + cell] = v;
    }
}

template <int DIM, bool SIMPLEX>
__global__ void __launch_bounds__(128) mapped_cell_tables(GridDesc g, double* __restrict__ tm, double* __restrict__ tb,
                                                          const double* __restrict__ kappa, double kappa_const,
                                                          const double* __restrict__ force, double force_const) {
  constexpr int NC = 1 << DIM, NP = NC * (NC + 1) / 2, NSUB = num_sub(DIM, SIMPLEX), NLOC = num_local(DIM, SIMPLEX);
  const long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (cell >= g.ncells) return;
  const long long nc = g.ncells;
  long long ci[3] = {0, 0, 0};
  cell_multi(g, cell, ci);
  // the cube's corner coordinates, corner c at bits c
  double X[NC][DIM];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    long long w[3] = {ci[0], ci[1], ci[2]};
#pragma unroll
    for (int a = 0; a < DIM; ++a) w[a] += (c >> a) & 1;
    const long long wv = w[0] + g.vn[0] * (w[1] + g.vn[1] * w[2]);
#pragma unroll
    for (int a = 0; a < DIM; ++a) X[c][a] = g.xv[wv * DIM + a];
  }
  if constexpr (SIMPLEX) {
    double fact = 1.0;  // d!
#pragma unroll
    for (int a = 2; a <= DIM; ++a) fact *= a;
    double A[NP], B[NC];
#pragma unroll
    for (int k = 0; k < NP; ++k) A[k] = 0.0;
#pragma unroll
    for (int c = 0; c < NC; ++c) B[c] = 0.0;
#pragma unroll
    for (int t = 0; t < NSUB; ++t) {
      const long long e = cell * NSUB + t;
      // J[a][k] = x_{k+1} - x_0 (local vertices in Kuhn order)
      double J[DIM][DIM], Ji[DIM][DIM];
      const int c0 = local_corner(DIM, true, t, 0);
#pragma unroll
      for (int k = 0; k < DIM; ++k)
#pragma unroll
        for (int a = 0; a < DIM; ++a) J[a][k] = X[local_corner(DIM, true, t, k + 1)][a] - X[c0][a];
      const double vol = fabs(inv_det<DIM>(J, Ji)) / fact;
      if (tm) {
        // grad phi_j = row j-1 of J^{-1} (j >= 1); grad phi_0 = minus the sum of the others
        double G[NLOC][DIM];
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
          double s0 = 0.0;
#pragma unroll
          for (int j = 1; j < NLOC; ++j) {
            G[j][a] = Ji[j - 1][a];
            s0 += Ji[j - 1][a];
          }
          G[0][a] = -s0;
        }
        const double kv = (kappa ? kappa[e] : kappa_const) * vol;
#pragma unroll
        for (int li = 0; li < NLOC; ++li)
#pragma unroll
          for (int lj = li; lj < NLOC; ++lj) {
            double d = 0.0;
#pragma unroll
            for (int a = 0; a < DIM; ++a) d += G[li][a] * G[lj][a];
            A[pair_entry(NC, local_corner(DIM, true, t, li), local_corner(DIM, true, t, lj))] += kv * d;
          }
      }
      if (tb) {
        const double bl = (force ? force[e] : force_const) * vol / double(DIM + 1);
#pragma unroll
        for (int li = 0; li < NLOC; ++li) B[local_corner(DIM, true, t, li)] += bl;
      }
    }
    if (tm) {
#pragma unroll
      for (int i = 0; i < NC; ++i)
#pragma unroll
        for (int j = i; j < NC; ++j)
          if (pair_shared(true, i, j)) tm[pair_entry(NC, i, j) * nc + cell] = A[pair_entry(NC, i, j)];
    }
    if (tb) {
#pragma unroll
      for (int c = 0; c < NC; ++c) tb[c * nc + cell] = B[c];
    }
  } else {
    if constexpr (DIM == 3) {
      if (tm) q1_hex_stiffness(X, kappa ? kappa[cell] : kappa_const, tm, nc, cell);
    } else if (tm) {
      const double kap = kappa ? kappa[cell] : kappa_const;
      // Gauss points of order 2 on [0, 1]: (3 -+ sqrt 3) / 6, weights 1/2 per axis
      constexpr double gp0 = 0.21132486540518711775, gp1 = 0.78867513459481288225;
      double A[NP];
#pragma unroll
      for (int k = 0; k < NP; ++k) A[k] = 0.0;
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        double xh[DIM];
#pragma unroll
        for (int a = 0; a < DIM; ++a) xh[a] = ((q >> a) & 1) ? gp1 : gp0;
        // reference gradients of the multilinear shape functions at xh (constants after unrolling)
        double gr[NC][DIM];
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
          for (int k = 0; k < DIM; ++k) {
            double d = ((c >> k) & 1) ? 1.0 : -1.0;
#pragma unroll
            for (int s2 = 0; s2 < DIM; ++s2)
              if (s2 != k) d *= ((c >> s2) & 1) ? xh[s2] : 1.0 - xh[s2];
            gr[c][k] = d;
          }
        double J[DIM][DIM], Ji[DIM][DIM];
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
          for (int k = 0; k < DIM; ++k) {
            double sj = 0.0;
#pragma unroll
            for (int c = 0; c < NC; ++c) sj += gr[c][k] * X[c][a];
            J[a][k] = sj;
          }
        const double factor = kap * fabs(inv_det<DIM>(J, Ji)) / double(NC);
        // grad phi_i . grad phi_j = gr_i^T (J^{-1} J^{-T}) gr_j: M = factor J^{-1} J^{-T} (symmetric)
        double M[DIM][DIM];
#pragma unroll
        for (int k = 0; k < DIM; ++k)
#pragma unroll
          for (int l = k; l < DIM; ++l) {
            double s = 0.0;
#pragma unroll
            for (int a = 0; a < DIM; ++a) s += Ji[k][a] * Ji[l][a];
            M[k][l] = s * factor;
            M[l][k] = M[k][l];
          }
#pragma unroll
        for (int i = 0; i < NC; ++i) {
          double hi[DIM];
#pragma unroll
          for (int k = 0; k < DIM; ++k) {
            double s = 0.0;
#pragma unroll
            for (int l = 0; l < DIM; ++l) s += M[k][l] * gr[i][l];
            hi[k] = s;
          }
#pragma unroll
          for (int j = i; j < NC; ++j) {
            double d = 0.0;
#pragma unroll
            for (int k = 0; k < DIM; ++k) d += gr[j][k] * hi[k];
            A[pair_entry(NC, i, j)] += d;
          }
        }
      }
#pragma unroll
      for (int k = 0; k < NP; ++k) tm[k * nc + cell] = A[k];
    }
    if (tb) {
      // one-point rule at the centre: |det J(1/2, ...)| f, phi = 2^{-d}, weight 1
      double J[DIM][DIM], Ji[DIM][DIM];
#pragma unroll
      for (int a = 0; a < DIM; ++a)
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
          double sj = 0.0;
#pragma unroll
          for (int c = 0; c < NC; ++c) sj += (((c >> k) & 1) ? 1.0 : -1.0) * X[c][a];
          J[a][k] = sj / double(NC / 2);
        }
      tb[cell] = (force ? force[cell] : force_const) * fabs(inv_det<DIM>(J, Ji)) / double(NC);
    }
  }
}

template <int DIM, bool SIMPLEX>
__global__ void __launch_bounds__(256) assemble_cg_rows_tabled(GridDesc g, const int* __restrict__ rp,
                                                               double* __restrict__ val, double* __restrict__ rhs,
                                                               const double* __restrict__ tm,
                                                               const double* __restrict__ tb, int dirichlet,
                                                               const double* __restrict__ gD, double gD_const) {
  constexpr int NS = pow3(DIM), NC = 1 << DIM;
  const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (v >= g.nvert) return;
  const long long nc = g.ncells;
  long long vi[3];
  vertex_multi(g, v, vi);
  double acc[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) acc[k] = 0.0;
  double b = 0.0;
#pragma unroll
  for (int cv = 0; cv < NC; ++cv) {
    // v is corner cv of cell vi - bits(cv)
    long long ci[3] = {0, 0, 0};
    bool inside = true;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      ci[a] = vi[a] - ((cv >> a) & 1);
      inside = inside && ci[a] >= 0 && ci[a] < g.n[a];
    }
    if (!inside) continue;
    const long long cell = cell_index(g, ci);
    if (val) {
#pragma unroll
      for (int lj = 0; lj < NC; ++lj)
        if (pair_shared(SIMPLEX, cv, lj)) acc[slot_between(DIM, cv, lj)] += tm[pair_entry(NC, cv, lj) * nc + cell];
    }
    if (rhs) b += tb[(SIMPLEX ? cv : 0) * nc + cell];
  }
  finish_row<DIM, SIMPLEX>(g, v, vi, acc, b, rp, val, rhs, dirichlet, gD, gD_const);
}

// DirichletConstraints::apply(M, V) as a separate pass over an assembled matrix: unit rows for
// boundary DoFs, zero boundary columns elsewhere (pattern is symmetric), rhs[D] = 0.
template <int DIM>
__global__ void dirichlet_rows(GridDesc g, const int* __restrict__ rp, const int* __restrict__ col,
                               double* __restrict__ val, double* __restrict__ rhs, const double* __restrict__ gD,
                               double gD_const) {
  const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (v >= g.nvert) return;
  long long vi[3];
  vertex_multi(g, v, vi);
  const bool bnd = on_boundary(g, vi, DIM);
  const bool lift = rhs && (gD || gD_const != 0.0);
  double b = (lift && !bnd) ? rhs[v] : 0.0;
  for (int k = rp[v]; k < rp[v + 1]; ++k) {
    const long long w = col[k];
    if (bnd) {
      val[k] = (w == v) ? 1.0 : 0.0;
    } else {
      long long wi[3];
      vertex_multi(g, w, wi);
      if (on_boundary(g, wi, DIM)) {
        if (lift) b -= val[k] * (gD ? gD[w] : gD_const);
        val[k] = 0.0;
      }
    }
  }
  if (rhs && bnd) rhs[v] = lift ? (gD ? gD[v] : gD_const) : 0.0;
  else if (lift) rhs[v] = b;
}

// -lam_e^T (dA_e / dlog kappa_e) u_e = -kappa_e lam_e^T K_t u_e, Dirichlet rows and columns excluded
template <int DIM, bool SIMPLEX>
__global__ void cg_dlogkappa_kernel(GridDesc g, const LocalTables tab, const double* __restrict__ kappa, const double* __restrict__ u,
                                    const double* __restrict__ lam, double* __restrict__ out) {
  constexpr int NSUB = num_sub(DIM, SIMPLEX), NLOC = num_local(DIM, SIMPLEX);
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= g.nelem) return;
  const long long cell = e / NSUB;
  const int t = int(e % NSUB);
  long long ci[3];
  cell_multi(g, cell, ci);
  double ul[NLOC], ll[NLOC];
#pragma unroll
  for (int j = 0; j < NLOC; ++j) {
    int c = 0;
#pragma unroll
    for (int tt = 0; tt < NSUB; ++tt)
      if (tt == t) c = local_corner(DIM, SIMPLEX, tt, j);
    long long vi[3] = {0, 0, 0}, vidx = 0, stride = 1;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      vi[a] = ci[a] + ((c >> a) & 1);
      vidx += vi[a] * stride;
      stride *= g.vn[a];
    }
    const bool bnd = on_boundary(g, vi, DIM);
    ul[j] = bnd ? 0.0 : u[vidx];
    ll[j] = bnd ? 0.0 : lam[vidx];
  }
  double acc = 0.0;
#pragma unroll
  for (int i = 0; i < NLOC; ++i) {
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < NLOC; ++j) s += tab.K[(t * kMaxLoc + i) * kMaxLoc + j] * ul[j];
    acc += ll[i] * s;
  }
  out[e] = -kappa[e] * acc;
}

LocalTables make_tables(const GridDesc& g) {
  LocalTables tab = {};
  local_matrices(g, tab.K, tab.B);
  return tab;
}

}  // namespace

__global__ void k_mf_kappa(long long n, const double* __restrict__ kappa, double kc, float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = float(kappa ? kappa[i] : kc);
}

gdt_status mf_capture(gdt_context ctx, gdt_matrix m, const gdt_diffusion_desc* d) {
  const GridDesc& g = m->test.g;
  m->mf_valid = 0;
  if (g.dim != 3 || g.simplex || m->test.order != 1 || m->test.kind != GDT_SPACE_CG) return GDT_OK;
  if (!m->mf_kappa) GDT_TRY_CUDA(ctx, cudaMalloc(&m->mf_kappa, sizeof(float) * g.nelem));
  const int bl = std::max(1, std::min(grid_blocks(g.nelem, 256), ctx->num_sms * 8));
  k_mf_kappa<<<bl, 256, 0, ctx->stream>>>(g.nelem, d->kappa, d->kappa_const, m->mf_kappa);
  const LocalTables tab = make_tables(g);
  for (int li = 0; li < 8; ++li)
    for (int lj = 0; lj < 8; ++lj)
      m->mf_K[local_corner(3, false, 0, li) * 8 + local_corner(3, false, 0, lj)] = float(tab.K[li * kMaxLoc + lj]);
  m->mf_dirichlet = d->dirichlet ? 1 : 0;
  m->mf_valid = 1;
  return check_launch(ctx, "mf_capture");
}

// mapped grids: the cube tables (stiffness and/or load), then the row gather over them
gdt_status assemble_cg_mapped(gdt_context ctx, const GridDesc& g, const int* rp, double* val,
                              const gdt_diffusion_desc* d, double* rhs, const double* gD, double gD_const) {
  const int nc = 1 << g.dim, np = nc * (nc + 1) / 2, nb = g.simplex ? nc : 1;
  cudaStream_t s = ctx->stream;
  double* tm = nullptr;
  double* tb = nullptr;
  if ((val && cudaMallocAsync(&tm, sizeof(double) * size_t(np) * g.ncells, s) != cudaSuccess) ||
      (rhs && cudaMallocAsync(&tb, sizeof(double) * size_t(nb) * g.ncells, s) != cudaSuccess)) {
    cudaGetLastError();
    if (tm) cudaFreeAsync(tm, s);
    return fail(ctx, GDT_ENOMEM, "mapped assembly tables");
  }
  const int bl1 = grid_blocks(g.ncells, 128), bl2 = grid_blocks(g.nvert, 256);
#define GDT_LAUNCH_MAPPED(D, S)                                                                                \
  do {                                                                                                          \
    mapped_cell_tables<D, S><<<bl1, 128, 0, s>>>(g, tm, tb, d->kappa, d->kappa_const, d->force, d->force_const); \
    assemble_cg_rows_tabled<D, S><<<bl2, 256, 0, s>>>(g, rp, val, rhs, tm, tb, d->dirichlet, gD, gD_const);      \
  } while (0)
  if (g.dim == 1) GDT_LAUNCH_MAPPED(1, false);
  else if (g.dim == 2 && !g.simplex) GDT_LAUNCH_MAPPED(2, false);
  else if (g.dim == 2) GDT_LAUNCH_MAPPED(2, true);
  else if (!g.simplex) GDT_LAUNCH_MAPPED(3, false);
  else GDT_LAUNCH_MAPPED(3, true);
#undef GDT_LAUNCH_MAPPED
  ctx->launches++;  // the second of the two launches; check_launch counts the other
  const gdt_status st = check_launch(ctx, "assemble_cg mapped");
  if (tm) cudaFreeAsync(tm, s);
  if (tb) cudaFreeAsync(tb, s);
  return st;
}

gdt_status assemble_cg(gdt_context ctx, gdt_matrix m, const gdt_diffusion_desc* d, double* rhs) {
  const GridDesc& g = m->test.g;
  if (g.xv) {
    m->mf_valid = 0;  // the matrix-free mixed operator assumes one geometry for all elements
    return assemble_cg_mapped(ctx, g, m->rp, m->val, d, rhs, d->dirichlet_values, d->dirichlet_value_const);
  }
  const LocalTables tab = make_tables(g);
  const int th = 256;
  const int bl = grid_blocks(g.nvert, th);
  cudaStream_t s = ctx->stream;
#define GDT_LAUNCH_ASM(D, S)                                                                                   \
  assemble_cg_rows<D, S><<<bl, th, 0, s>>>(g, m->rp, m->val, rhs, tab, d->kappa, d->kappa_const, d->force, d->force_const, \
                                           d->dirichlet, d->dirichlet_values, d->dirichlet_value_const)
  if (g.dim == 1) GDT_LAUNCH_ASM(1, false);
  else if (g.dim == 2 && !g.simplex) GDT_LAUNCH_ASM(2, false);
  else if (g.dim == 2) GDT_LAUNCH_ASM(2, true);
  else if (!g.simplex) GDT_LAUNCH_ASM(3, false);
  else GDT_LAUNCH_ASM(3, true);
#undef GDT_LAUNCH_ASM
  GDT_CHECK(ctx, check_launch(ctx, "assemble_cg_rows"));
  return mf_capture(ctx, m, d);
}

gdt_status assemble_cg_rhs(gdt_context ctx, const gdt_space_s& sp, const gdt_diffusion_desc* d, double* rhs) {
  const GridDesc& g = sp.g;
  if (g.xv) return assemble_cg_mapped(ctx, g, nullptr, nullptr, d, rhs, nullptr, 0.0);
  const LocalTables tab = make_tables(g);
  const int th = 256;
  const int bl = grid_blocks(g.nvert, th);
  cudaStream_t s = ctx->stream;
#define GDT_LAUNCH_RHS(D, S)                                                                                  \
  assemble_cg_rows<D, S><<<bl, th, 0, s>>>(g, nullptr, nullptr, rhs, tab, d->kappa, d->kappa_const, d->force, \
                                           d->force_const, d->dirichlet, nullptr, 0.0)
  if (g.dim == 1) GDT_LAUNCH_RHS(1, false);
  else if (g.dim == 2 && !g.simplex) GDT_LAUNCH_RHS(2, false);
  else if (g.dim == 2) GDT_LAUNCH_RHS(2, true);
  else if (!g.simplex) GDT_LAUNCH_RHS(3, false);
  else GDT_LAUNCH_RHS(3, true);
#undef GDT_LAUNCH_RHS
  return check_launch(ctx, "assemble_cg_rhs");
}

gdt_status dirichlet_apply(gdt_context ctx, gdt_matrix m, double* rhs, const double* values, double value_const) {
  const GridDesc& g = m->test.g;
  const int th = 256;
  const int bl = grid_blocks(g.nvert, th);
  cudaStream_t s = ctx->stream;
  if (g.dim == 1) dirichlet_rows<1><<<bl, th, 0, s>>>(g, m->rp, m->col, m->val, rhs, values, value_const);
  else if (g.dim == 2) dirichlet_rows<2><<<bl, th, 0, s>>>(g, m->rp, m->col, m->val, rhs, values, value_const);
  else dirichlet_rows<3><<<bl, th, 0, s>>>(g, m->rp, m->col, m->val, rhs, values, value_const);
  return check_launch(ctx, "dirichlet_rows");
}

gdt_status cg_dlogkappa(gdt_context ctx, const gdt_space_s& sp, const double* kappa, const double* u,
                        const double* lam, double* out) {
  const GridDesc& g = sp.g;
  const LocalTables tab = make_tables(g);
  const int th = 256;
  const int bl = grid_blocks(g.nelem, th);
  cudaStream_t s = ctx->stream;
  if (g.dim == 1) cg_dlogkappa_kernel<1, false><<<bl, th, 0, s>>>(g, tab, kappa, u, lam, out);
  else if (g.dim == 2 && !g.simplex) cg_dlogkappa_kernel<2, false><<<bl, th, 0, s>>>(g, tab, kappa, u, lam, out);
  else if (g.dim == 2) cg_dlogkappa_kernel<2, true><<<bl, th, 0, s>>>(g, tab, kappa, u, lam, out);
  else if (!g.simplex) cg_dlogkappa_kernel<3, false><<<bl, th, 0, s>>>(g, tab, kappa, u, lam, out);
  else cg_dlogkappa_kernel<3, true><<<bl, th, 0, s>>>(g, tab, kappa, u, lam, out);
  return check_launch(ctx, "cg_dlogkappa");
}

}  // namespace gdt
