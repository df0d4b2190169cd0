// SWIPDG / IPDG assembly for DG P1 on structured triangle grids (Kuhn split of 2D cube grids):
// element LocalLaplaceIntegrand (local/integrands/laplace.hh:81-102), InnerCoupling + InnerPenalty on
// inner intersections (local/integrands/laplace-ipdg.hh:107-186, local/integrands/ipdg.hh:113-171) and
// DirichletCoupling + BoundaryPenalty on the (homogeneous Dirichlet) boundary (laplace-ipdg.hh:331-368,
// ipdg.hh:254-282), penalty length h = |I| (test/stationary-heat-equation/ESV2007.hh:112), and the
// product RHS. The reference visits each inner intersection once and scatters four blocks
// (local/assembler/bilinear-form-assemblers.hh:238-278).
//
// GB300 design: output-stationary. One thread owns the 3 rows of one element: its diagonal block is
// the element term plus the in/in term of each of its faces, and its off-diagonal block to a
// neighbour is the in/out term of the shared face, all evaluated from the element's own side (the
// out/out and out/in blocks of the reference are exactly the in/in and in/out blocks seen from the
// neighbour, with the normal flipped). Rows are written once, no atomics, no face colouring.
// Geometry is identical for all elements of one of the two triangle types, so basis values at the
// face quadrature points, gradients, normals and local matrices are precomputed per type on the host
// (kernel parameters). The adjoint kernel uses that every SWIPDG face term scales with
// H = k_in k_out / (k_in + k_out), so dH/dlog k_in = H k_out / (k_in + k_out).
#include <cmath>

#include "structured.cuh"

namespace gdt {
namespace {

struct TriFace {
  double n[2];
  double vol;
  double hb;          // vol^beta: the penalty's length scale
  double xq[2][2];    // the two Gauss points, relative to the element's cell corner
  double w[2];        // quadrature weight * integration element
  double vin[2][3];   // own basis at the face points
  double vout[2][3];  // neighbour basis at the same points
  int dcx, dcy, tnb;  // neighbour cell offset and type
};

struct TriTables {
  double K[2][3][3];
  double B[2][3];
  double G[2][3][2];
  TriFace F[2][3];
};

void tri_vertices(int t, const double* h, double X[3][2]) {
  // A (t = 0): (0,0), (h0,0), (h0,h1); B (t = 1): (0,0), (0,h1), (h0,h1)
  X[0][0] = 0;
  X[0][1] = 0;
  X[2][0] = h[0];
  X[2][1] = h[1];
  if (t == 0) {
    X[1][0] = h[0];
    X[1][1] = 0;
  } else {
    X[1][0] = 0;
    X[1][1] = h[1];
  }
}

// barycentric coordinates of x in the triangle X
void bary(const double X[3][2], const double* x, double* lam) {
  const double a = X[1][0] - X[0][0], b = X[2][0] - X[0][0], c = X[1][1] - X[0][1], d = X[2][1] - X[0][1];
  const double det = a * d - b * c;
  const double rx = x[0] - X[0][0], ry = x[1] - X[0][1];
  const double l1 = (d * rx - b * ry) / det, l2 = (-c * rx + a * ry) / det;
  lam[0] = 1.0 - l1 - l2;
  lam[1] = l1;
  lam[2] = l2;
}

void grads(const double X[3][2], double G[3][2]) {
  const double a = X[1][0] - X[0][0], b = X[2][0] - X[0][0], c = X[1][1] - X[0][1], d = X[2][1] - X[0][1];
  const double det = a * d - b * c;
  // rows of J^{-1}: grad l1 = (d, -b)/det, grad l2 = (-c, a)/det
  G[1][0] = d / det;
  G[1][1] = -b / det;
  G[2][0] = -c / det;
  G[2][1] = a / det;
  G[0][0] = -G[1][0] - G[2][0];
  G[0][1] = -G[1][1] - G[2][1];
}

TriTables make_tables(const GridDesc& g, double beta = 1.0) {
  TriTables T = {};
  const double h[2] = {g.h[0], g.h[1]};
  const double gq = 0.5 / std::sqrt(3.0);
  const double xi[2] = {0.5 - gq, 0.5 + gq};
  // neighbour across face f of type t: A: f0 bottom -> B below, f1 diagonal -> B, f2 right -> B right;
  // B: f0 left -> A left, f1 diagonal -> A, f2 top -> A above
  const int dcx[2][3] = {{0, 0, 1}, {-1, 0, 0}}, dcy[2][3] = {{-1, 0, 0}, {0, 0, 1}};
  for (int t = 0; t < 2; ++t) {
    double X[3][2];
    tri_vertices(t, h, X);
    double G[3][2];
    grads(X, G);
    const double area = 0.5 * h[0] * h[1];
    for (int i = 0; i < 3; ++i) {
      T.G[t][i][0] = G[i][0];
      T.G[t][i][1] = G[i][1];
      T.B[t][i] = area / 3.0;
      for (int j = 0; j < 3; ++j) T.K[t][i][j] = area * (G[i][0] * G[j][0] + G[i][1] * G[j][1]);
    }
    for (int f = 0; f < 3; ++f) {
      TriFace& F = T.F[t][f];
      // face f is opposite local vertex 2 - f
      const int opp = 2 - f;
      int a = -1, b = -1;
      for (int v = 0; v < 3; ++v)
        if (v != opp) (a < 0 ? a : b) = v;
      const double ex = X[b][0] - X[a][0], ey = X[b][1] - X[a][1];
      F.vol = std::sqrt(ex * ex + ey * ey);
      F.hb = beta == 1.0 ? F.vol : std::pow(F.vol, beta);
      double nx = ey / F.vol, ny = -ex / F.vol;
      if ((X[opp][0] - X[a][0]) * nx + (X[opp][1] - X[a][1]) * ny > 0) {
        nx = -nx;
        ny = -ny;
      }
      F.n[0] = nx;
      F.n[1] = ny;
      F.dcx = dcx[t][f];
      F.dcy = dcy[t][f];
      F.tnb = 1 - t;
      double Y[3][2];
      tri_vertices(1 - t, h, Y);
      for (int v = 0; v < 3; ++v) {
        Y[v][0] += F.dcx * h[0];
        Y[v][1] += F.dcy * h[1];
      }
      for (int q = 0; q < 2; ++q) {
        const double x[2] = {X[a][0] + xi[q] * ex, X[a][1] + xi[q] * ey};
        F.xq[q][0] = x[0];
        F.xq[q][1] = x[1];
        F.w[q] = 0.5 * F.vol;
        bary(X, x, F.vin[q]);
        bary(Y, x, F.vout[q]);
      }
    }
  }
  return T;
}

struct IpdgParams {
  double theta, sigma_in, sigma_bd;
  int weight_is_diffusion;
  // Dirichlet data on the boundary faces for the right-hand side: g at the two Gauss points of each
  // face ([element][face][point]) or the constant g_const; rhs_terms bit 0: the unary DirichletCoupling
  // term, bit 1: the boundary penalty's counterpart
  const double* g_face;
  double g_const;
  int rhs_terms;
};

// right-hand side of boundary face f: sum_q w_q g_q (-theta (kappa grad psi_i . n) [bit 0]
// + sigma (n . w n) / h^beta psi_i(x_q) [bit 1]) (local/integrands/laplace-ipdg.hh:292-320 and the
// product of the boundary penalty's weight with g)
__device__ __forceinline__ void boundary_rhs(const TriTables& T, int t, int f, long long e, double kin,
                                             const IpdgParams& p, double b[3]) {
  const TriFace& F = T.F[t][f];
  const double w = p.weight_is_diffusion ? kin : 1.0;
  const double penalty = (p.sigma_bd * w) / F.hb;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const double gq = p.g_face ? p.g_face[(e * 3 + f) * 2 + q] : p.g_const;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double v = 0.0;
      if (p.rhs_terms & 1) {
        const double dn = (kin * T.G[t][i][0]) * F.n[0] + (kin * T.G[t][i][1]) * F.n[1];
        v += -1.0 * p.theta * gq * dn;
      }
      if (p.rhs_terms & 2) v += penalty * gq * F.vin[q][i];
      b[i] += v * F.w[q];
    }
  }
}

// in/in (Bii) and in/out (Bio) blocks of an inner face seen from the element of type t
__device__ __forceinline__ void inner_blocks(const TriTables& T, int t, int f, double kin, double kout,
                                             const IpdgParams& p, double Bii[3][3], double Bio[3][3]) {
  const TriFace& F = T.F[t][f];
  const double win = p.weight_is_diffusion ? kin : 1.0, wout = p.weight_is_diffusion ? kout : 1.0;
  const double delta_plus = wout, delta_minus = win;  // n.(w n) with |n| = 1
  const double weight_minus = delta_plus / (delta_plus + delta_minus);
  const double weight_plus = delta_minus / (delta_plus + delta_minus);
  const double penalty = (p.sigma_in * ((delta_plus * delta_minus) / (delta_plus + delta_minus))) / F.hb;
  double dn_in[3], dn_out[3];
  const int tn = F.tnb;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    dn_in[i] = (kin * T.G[t][i][0]) * F.n[0] + (kin * T.G[t][i][1]) * F.n[1];
    dn_out[i] = (kout * T.G[tn][i][0]) * F.n[0] + (kout * T.G[tn][i][1]) * F.n[1];
  }
#pragma unroll
  for (int ii = 0; ii < 3; ++ii)
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) {
      Bii[ii][jj] = 0.0;
      Bio[ii][jj] = 0.0;
    }
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const double fac = F.w[q];
#pragma unroll
    for (int ii = 0; ii < 3; ++ii)
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) {
        double v = -1.0 * weight_minus * dn_in[jj] * F.vin[q][ii];
        v += -1.0 * p.theta * weight_minus * F.vin[q][jj] * dn_in[ii];
        v += penalty * F.vin[q][jj] * F.vin[q][ii];
        Bii[ii][jj] += v * fac;
        double w = -1.0 * weight_plus * dn_out[jj] * F.vin[q][ii];
        w += p.theta * weight_minus * F.vout[q][jj] * dn_in[ii];
        w += -1.0 * penalty * F.vout[q][jj] * F.vin[q][ii];
        Bio[ii][jj] += w * fac;
      }
  }
}

__device__ __forceinline__ void boundary_block(const TriTables& T, int t, int f, double kin, const IpdgParams& p,
                                               double Bb[3][3]) {
  const TriFace& F = T.F[t][f];
  const double w = p.weight_is_diffusion ? kin : 1.0;
  const double penalty = (p.sigma_bd * w) / F.hb;
  double dn[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) dn[i] = (kin * T.G[t][i][0]) * F.n[0] + (kin * T.G[t][i][1]) * F.n[1];
#pragma unroll
  for (int ii = 0; ii < 3; ++ii)
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) Bb[ii][jj] = 0.0;
#pragma unroll
  for (int q = 0; q < 2; ++q)
#pragma unroll
    for (int ii = 0; ii < 3; ++ii)
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) {
        double v = -1.0 * dn[jj] * F.vin[q][ii];
        v += -1.0 * p.theta * F.vin[q][jj] * dn[ii];
        v += penalty * F.vin[q][jj] * F.vin[q][ii];
        Bb[ii][jj] += v * F.w[q];
      }
}

// neighbour element across face f, or -1 on the domain boundary
__device__ __forceinline__ long long neighbour(const GridDesc& g, const TriTables& T, int t, int f, long long cx,
                                               long long cy) {
  const long long nx = cx + T.F[t][f].dcx, ny = cy + T.F[t][f].dcy;
  if (nx < 0 || nx >= g.n[0] || ny < 0 || ny >= g.n[1]) return -1;
  return 2 * (nx + g.n[0] * ny) + T.F[t][f].tnb;
}

__global__ void __launch_bounds__(128) swipdg_rows(GridDesc g, TriTables T, IpdgParams p, const int* __restrict__ rp,
                                                   double* __restrict__ val, double* __restrict__ rhs,
                                                   const double* __restrict__ kappa, double kappa_const,
                                                   const double* __restrict__ force, double force_const) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= g.nelem) return;
  const int t = int(e & 1);
  const long long c = e >> 1, cx = c % g.n[0], cy = c / g.n[0];
  const double kin = kappa ? kappa[e] : kappa_const;
  double D[3][3], O[3][3][3];
  long long nb[3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) D[i][j] = kin * T.K[t][i][j];
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    nb[f] = neighbour(g, T, t, f, cx, cy);
    double Bii[3][3];
    if (nb[f] >= 0) {
      const double kout = kappa ? kappa[nb[f]] : kappa_const;
      inner_blocks(T, t, f, kin, kout, p, Bii, O[f]);
    } else {
      boundary_block(T, t, f, kin, p, Bii);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) D[i][j] += Bii[i][j];
  }
  if (rhs) {
    const double fe = force ? force[e] : force_const;
    double b[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) b[i] = fe * T.B[t][i];
    if (p.rhs_terms)
#pragma unroll
      for (int f = 0; f < 3; ++f)
        if (nb[f] < 0) boundary_rhs(T, t, f, e, kin, p, b);
#pragma unroll
    for (int i = 0; i < 3; ++i) rhs[3 * e + i] = b[i];
  }
  // block order by element index: A: f0, self, f1, f2; B: f0, f1, self, f2
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    long long pos = rp[3 * e + i];
#pragma unroll
    for (int slot = 0; slot < 4; ++slot) {
      const int f = (t == 0) ? (slot == 0 ? 0 : slot == 1 ? -1 : slot - 1) : (slot == 2 ? -1 : slot < 2 ? slot : 2);
      if (f >= 0 && nb[f] < 0) continue;
#pragma unroll
      for (int j = 0; j < 3; ++j) val[pos + j] = (f < 0) ? D[i][j] : O[f][i][j];
      pos += 3;
    }
  }
}

__device__ __forceinline__ double bilin(const double M[3][3], const double* l, const double* u) {
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) s += l[i] * (M[i][0] * u[0] + M[i][1] * u[1] + M[i][2] * u[2]);
  return s;
}

// out[e] = -d/dlog(kappa_e) [lam^T A(kappa) u] for SWIPDG (weight = kappa)
__global__ void __launch_bounds__(128) swipdg_dlogkappa_kernel(GridDesc g, TriTables T, IpdgParams p,
                                                               const double* __restrict__ kappa,
                                                               const double* __restrict__ u,
                                                               const double* __restrict__ lam,
                                                               double* __restrict__ out) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= g.nelem) return;
  const int t = int(e & 1);
  const long long c = e >> 1, cx = c % g.n[0], cy = c / g.n[0];
  const double ke = kappa[e];
  double ue[3], le[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    ue[i] = u[3 * e + i];
    le[i] = lam[3 * e + i];
  }
  double K[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) K[i][j] = ke * T.K[t][i][j];
  double acc = bilin(K, le, ue);
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    const long long n = neighbour(g, T, t, f, cx, cy);
    double B1[3][3], B2[3][3];
    if (n < 0) {
      boundary_block(T, t, f, ke, p, B1);
      acc += bilin(B1, le, ue);
      continue;
    }
    const double kn = kappa[n];
    double un[3], ln[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      un[i] = u[3 * n + i];
      ln[i] = lam[3 * n + i];
    }
    // the whole face term lam^T B_face u: own half (rows of e) + neighbour half (rows of n)
    inner_blocks(T, t, f, ke, kn, p, B1, B2);
    double tf = bilin(B1, le, ue) + bilin(B2, le, un);
    const int tn = 1 - t, fn = 2 - f;
    inner_blocks(T, tn, fn, kn, ke, p, B1, B2);
    tf += bilin(B1, ln, un) + bilin(B2, ln, ue);
    acc += tf * (kn / (ke + kn));
  }
  out[e] = -acc;
}

bool supported(const GridDesc& g) { return g.dim == 2 && g.simplex; }

}  // namespace

gdt_status assemble_swipdg(gdt_context ctx, gdt_matrix m, const gdt_ipdg_desc* d, double* rhs) {
  const GridDesc& g = m->test.g;
  if (!supported(g)) return fail(ctx, GDT_EUNSUPPORTED, "SWIPDG assembly is provided for 2D simplex grids");
  if (d->penalty_beta < 0.0 || (d->dirichlet_rhs & ~3)) return fail(ctx, GDT_EINVAL, "SWIPDG descriptor");
  const TriTables T = make_tables(g, d->penalty_beta > 0.0 ? d->penalty_beta : 1.0);
  const IpdgParams p{d->symmetry_prefactor, d->sigma_inner, d->sigma_boundary, d->weight_is_diffusion,
                     d->dirichlet_face, d->dirichlet_const, d->dirichlet_rhs};
  swipdg_rows<<<grid_blocks(g.nelem, 128), 128, 0, ctx->stream>>>(g, T, p, m->rp, m->val, rhs, d->kappa,
                                                                  d->kappa_const, d->force, d->force_const);
  return check_launch(ctx, "swipdg_rows");
}

gdt_status dg_face_points(const gdt_space_s& sp, double* xy) {
  const GridDesc& g = sp.g;
  if (!supported(g)) return GDT_EUNSUPPORTED;
  const TriTables T = make_tables(g);
  for (long long e = 0; e < g.nelem; ++e) {
    const int t = int(e & 1);
    const long long c = e >> 1, cx = c % g.n[0], cy = c / g.n[0];
    for (int f = 0; f < 3; ++f)
      for (int q = 0; q < 2; ++q) {
        double* out = xy + ((e * 3 + f) * 2 + q) * 2;
        out[0] = g.lo[0] + double(cx) * g.h[0] + T.F[t][f].xq[q][0];
        out[1] = g.lo[1] + double(cy) * g.h[1] + T.F[t][f].xq[q][1];
      }
  }
  return GDT_OK;
}

gdt_status swipdg_dlogkappa(gdt_context ctx, const gdt_space_s& sp, const gdt_ipdg_desc* d, const double* u,
                            const double* lam, double* out) {
  const GridDesc& g = sp.g;
  if (!supported(g)) return fail(ctx, GDT_EUNSUPPORTED, "SWIPDG adjoint is provided for 2D simplex grids");
  if (!d->weight_is_diffusion) return fail(ctx, GDT_EUNSUPPORTED, "adjoint needs the SWIPDG weight (kappa)");
  const TriTables T = make_tables(g, d->penalty_beta > 0.0 ? d->penalty_beta : 1.0);
  const IpdgParams p{d->symmetry_prefactor, d->sigma_inner, d->sigma_boundary, 1, nullptr, 0.0, 0};
  swipdg_dlogkappa_kernel<<<grid_blocks(g.nelem, 128), 128, 0, ctx->stream>>>(g, T, p, d->kappa, u, lam, out);
  return check_launch(ctx, "swipdg_dlogkappa");
}

}  // namespace gdt
