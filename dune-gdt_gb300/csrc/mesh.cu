// Unstructured simplex meshes: the leaf view of a DUNE simplex grid (ALUGrid, UGGrid, a gmsh import),
// exported as vertex coordinates and element vertex lists in the grid's index-set order. Continuous
// P1 on it: DoF = vertex index (ContinuousMapper, spaces/mapper/continuous.hh:139-150), the element
// sparsity pattern (tools/sparsity-pattern.hh:33-50), the Laplace stiffness and load vector of
// LocalLaplaceIntegrand / LocalElementProductIntegrand with kappa and source per element
// (local/integrands/laplace.hh:81-102, local/integrands/product.hh:104-130), DirichletConstraints on the
// boundary vertices (tools/dirichlet-constraints.hh:153-184) and the adjoint log-kappa gradient.
//
// Setup (once per mesh, on the host like the grid construction of the reference): the element
// lists are checked, the boundary vertices are the vertices of faces that belong to one element, and
// the vertex -> element adjacency is built as CSR. Device side, every kernel is output-stationary:
// one thread owns one row (one vertex), walks the elements around its vertex, forms each element's
// affine geometry (J, J^{-1}, |det J|) from its own vertices and adds into its own row, so each
// value has one writer (no atomics, no colouring, deterministic). The pattern is built the same way:
// a row's columns are the vertices of its elements, sorted, without repeats.
#include <cub/cub.cuh>

#include <algorithm>
#include <array>
#include <cmath>
#include <new>
#include <vector>

#include "highorder.cuh"
#include "internal.cuh"

namespace gdt {
namespace {

// the device arrays of a mesh (owned by the grid and every space made from it)
struct MeshData {
  double* xv = nullptr;
  int* cells = nullptr;
  int* v2e_ptr = nullptr;
  int* v2e = nullptr;
  unsigned char* bnd = nullptr;
  int* nbr = nullptr;
  std::vector<double> hx;   // host copies of the coordinates and element lists (face points)
  std::vector<int> hcells;
  ~MeshData() {
    cudaFree(xv);
    cudaFree(cells);
    cudaFree(v2e_ptr);
    cudaFree(v2e);
    cudaFree(bnd);
    cudaFree(nbr);
  }
};

constexpr int kMeshMaxRow = 128;  // longest row of a mesh pattern (the vertex and its neighbours)

// affine geometry of element e: its vertices w, the gradients G of its barycentric basis and its volume
template <int DIM>
__device__ __forceinline__ double mesh_element(const GridDesc& g, int e, int (&w)[DIM + 1],
                                               double (&G)[DIM + 1][DIM]) {
  double X[DIM + 1][DIM];
#pragma unroll
  for (int j = 0; j <= DIM; ++j) {
    w[j] = g.mcells[e * (DIM + 1) + j];
#pragma unroll
    for (int a = 0; a < DIM; ++a) X[j][a] = g.xv[(long long)w[j] * DIM + a];
  }
  // J[a][k] = X_{k+1} - X_0; grad phi_j = row j - 1 of J^{-1} (j >= 1), grad phi_0 = minus their sum
  double J[DIM][DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k)
#pragma unroll
    for (int a = 0; a < DIM; ++a) J[a][k] = X[k + 1][a] - X[0][a];
  double det, Ji[DIM][DIM];
  if constexpr (DIM == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double r = 1.0 / det;
    Ji[0][0] = J[1][1] * r;
    Ji[0][1] = -J[0][1] * r;
    Ji[1][0] = -J[1][0] * r;
    Ji[1][1] = J[0][0] * r;
  } else {
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1], c01 = J[0][2] * J[2][1] - J[0][1] * J[2][2],
                 c02 = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    det = J[0][0] * c00 + J[1][0] * c01 + J[2][0] * c02;
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
  }
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    double s0 = 0.0;
#pragma unroll
    for (int j = 1; j <= DIM; ++j) {
      G[j][a] = Ji[j - 1][a];
      s0 += Ji[j - 1][a];
    }
    G[0][a] = -s0;
  }
  return fabs(det) / (DIM == 2 ? 2.0 : 6.0);
}

// columns of row v: the vertices of the elements around v, ascending, without repeats
template <int DIM>
__device__ int mesh_row_columns(const GridDesc& g, int v, int (&c)[kMeshMaxRow], bool& overflow) {
  int n = 0;
  for (int k = g.v2e_ptr[v]; k < g.v2e_ptr[v + 1]; ++k) {
    const int e = g.v2e[k];
    for (int j = 0; j <= DIM; ++j) {
      const int w = g.mcells[e * (DIM + 1) + j];
      int pos = n;
      while (pos > 0 && c[pos - 1] > w) --pos;
      if (pos > 0 && c[pos - 1] == w) continue;
      if (n == kMeshMaxRow) {
        overflow = true;
        continue;
      }
      for (int t = n; t > pos; --t) c[t] = c[t - 1];
      c[pos] = w;
      ++n;
    }
  }
  return n;
}

// count pass (count != null) or fill pass (col != null, rows starting at rp)
template <int DIM>
__global__ void k_mesh_pattern(GridDesc g, int* __restrict__ count, const int* __restrict__ rp, int* __restrict__ col,
                               int* __restrict__ err) {
  const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (v >= g.nvert) return;
  int c[kMeshMaxRow];
  bool over = false;
  const int n = mesh_row_columns<DIM>(g, int(v), c, over);
  if (over) atomicExch(err, 1);
  if (count) count[v] = n;
  if (col) {
    const int p = rp[v];
    for (int k = 0; k < n; ++k) col[p + k] = c[k];
  }
}

__device__ __forceinline__ int find_column(const int* __restrict__ col, int lo, int hi, int w) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (col[mid] < w) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Row v of the stiffness (val != null) and/or the load vector (rhs != null), then the Dirichlet rule:
// a unit row on a boundary vertex (b_v = g_v, or 0), elsewhere zero boundary columns whose given values
// move to the right-hand side (b_v -= A_vw g_w)
template <int DIM>
__global__ void __launch_bounds__(128) k_mesh_rows(GridDesc g, const int* __restrict__ rp, const int* __restrict__ col,
                                                   double* __restrict__ val, double* __restrict__ rhs,
                                                   const double* __restrict__ kappa, double kappa_const,
                                                   const double* __restrict__ force, double force_const, int dirichlet,
                                                   const double* __restrict__ gD, double gD_const) {
  const long long vl = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (vl >= g.nvert) return;
  const int v = int(vl);
  const int r0 = val ? rp[v] : 0, r1 = val ? rp[v + 1] : 0;
  for (int k = r0; k < r1; ++k) val[k] = 0.0;
  double b = 0.0;
  for (int k = g.v2e_ptr[v]; k < g.v2e_ptr[v + 1]; ++k) {
    const int e = g.v2e[k];
    int w[DIM + 1];
    double G[DIM + 1][DIM];
    const double vol = mesh_element<DIM>(g, e, w, G);
    int li = 0;
#pragma unroll
    for (int j = 0; j <= DIM; ++j)
      if (w[j] == v) li = j;
    if (val) {
      const double kv = (kappa ? kappa[e] : kappa_const) * vol;
#pragma unroll
      for (int lj = 0; lj <= DIM; ++lj) {
        double d = 0.0;
#pragma unroll
        for (int a = 0; a < DIM; ++a) d += G[li][a] * G[lj][a];
        val[find_column(col, r0, r1, w[lj])] += kv * d;
      }
    }
    if (rhs) b += (force ? force[e] : force_const) * vol / double(DIM + 1);
  }
  const bool bnd = dirichlet && g.mbnd[v];
  const bool lift = dirichlet && rhs && val && (gD || gD_const != 0.0);
  if (dirichlet && val) {
    for (int k = r0; k < r1; ++k) {
      const int w = col[k];
      if (bnd) {
        val[k] = (w == v) ? 1.0 : 0.0;
      } else if (g.mbnd[w]) {
        if (lift) b -= val[k] * (gD ? gD[w] : gD_const);
        val[k] = 0.0;
      }
    }
  }
  if (rhs) rhs[v] = bnd ? (lift ? (gD ? gD[v] : gD_const) : 0.0) : b;
}

// DirichletConstraints::apply on an assembled mesh matrix (separate pass), with optional values
__global__ void k_mesh_dirichlet(GridDesc g, const int* __restrict__ rp, const int* __restrict__ col,
                                 double* __restrict__ val, double* __restrict__ rhs, const double* __restrict__ gD,
                                 double gD_const) {
  const long long vl = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (vl >= g.nvert) return;
  const int v = int(vl);
  const bool bnd = g.mbnd[v];
  const bool lift = rhs && (gD || gD_const != 0.0);
  double b = (lift && !bnd) ? rhs[v] : 0.0;
  for (int k = rp[v]; k < rp[v + 1]; ++k) {
    const int w = col[k];
    if (bnd) {
      val[k] = (w == v) ? 1.0 : 0.0;
    } else if (g.mbnd[w]) {
      if (lift) b -= val[k] * (gD ? gD[w] : gD_const);
      val[k] = 0.0;
    }
  }
  if (rhs && bnd) rhs[v] = lift ? (gD ? gD[v] : gD_const) : 0.0;
  else if (lift) rhs[v] = b;
}

// -lam_e^T (dA_e / dlog kappa_e) u_e = -kappa_e lam_e^T K_e u_e, boundary rows and columns excluded
template <int DIM>
__global__ void k_mesh_dlogkappa(GridDesc g, const double* __restrict__ kappa, const double* __restrict__ u,
                                 const double* __restrict__ lam, double* __restrict__ out) {
  const long long el = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (el >= g.nelem) return;
  const int e = int(el);
  int w[DIM + 1];
  double G[DIM + 1][DIM];
  const double vol = mesh_element<DIM>(g, e, w, G);
  double ul[DIM + 1], ll[DIM + 1];
#pragma unroll
  for (int j = 0; j <= DIM; ++j) {
    const bool bnd = g.mbnd[w[j]];
    ul[j] = bnd ? 0.0 : u[w[j]];
    ll[j] = bnd ? 0.0 : lam[w[j]];
  }
  double acc = 0.0;
#pragma unroll
  for (int i = 0; i <= DIM; ++i) {
    double s = 0.0;
#pragma unroll
    for (int j = 0; j <= DIM; ++j) {
      double d = 0.0;
#pragma unroll
      for (int a = 0; a < DIM; ++a) d += G[i][a] * G[j][a];
      s += vol * d * ul[j];
    }
    acc += ll[i] * s;
  }
  out[e] = -kappa[e] * acc;
}

__global__ void k_mesh_indices(long long n, const int* __restrict__ cells, long long* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = cells[i];
}

// --------------------------------------------------------------------- DG P1 / SWIPDG on meshes ---
// DoF 3 e + i (DiscontinuousMapper, spaces/mapper/discontinuous.hh:102-125); the element-and-intersection
// pattern couples an element's rows with its own columns and those of its face neighbours, blocks in
// ascending element order.
__global__ void k_mesh_dg_pattern(GridDesc g, int* __restrict__ count, const int* __restrict__ rp,
                                  int* __restrict__ col) {
  const long long el = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (el >= g.nelem) return;
  const int e = int(el);
  int blk[4] = {e, -1, -1, -1};
  int nb = 1;
  for (int k = 0; k < 3; ++k) {
    const int o = g.mnbr[e * 3 + k];
    if (o < 0) continue;
    int pos = nb;
    while (pos > 0 && blk[pos - 1] > o) {
      blk[pos] = blk[pos - 1];
      --pos;
    }
    blk[pos] = o;
    ++nb;
  }
  for (int i = 0; i < 3; ++i) {
    const long long row = 3LL * e + i;
    if (count) count[row] = 3 * nb;
    if (col) {
      int p = rp[row];
      for (int b = 0; b < nb; ++b)
        for (int j = 0; j < 3; ++j) col[p++] = 3 * blk[b] + j;
    }
  }
}

struct MeshIpdg {
  double theta, sigma_in, sigma_bd, beta;
  int weight_is_diffusion;
  const double* g_face;  // Dirichlet data at the two Gauss points of every face ([element][face][point])
  double g_const;
  int rhs_terms;
};

// a triangle's vertices, coordinates, basis gradients and area
__device__ __forceinline__ double mesh_tri(const GridDesc& g, int e, int (&w)[3], double (&X)[3][2],
                                           double (&G)[3][2]) {
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    w[j] = g.mcells[e * 3 + j];
    X[j][0] = g.xv[2LL * w[j]];
    X[j][1] = g.xv[2LL * w[j] + 1];
  }
  const double a = X[1][0] - X[0][0], b = X[2][0] - X[0][0], c = X[1][1] - X[0][1], d = X[2][1] - X[0][1];
  const double det = a * d - b * c;
  G[1][0] = d / det;
  G[1][1] = -b / det;
  G[2][0] = -c / det;
  G[2][1] = a / det;
  G[0][0] = -G[1][0] - G[2][0];
  G[0][1] = -G[1][1] - G[2][1];
  return 0.5 * fabs(det);
}

// face k of a triangle: the other two local vertices (ascending), the unit outer normal and the length
__device__ __forceinline__ double mesh_tri_face(const double (&X)[3][2], int k, int& a, int& b, double (&n)[2]) {
  a = k == 0 ? 1 : 0;
  b = k == 2 ? 1 : 2;
  const double ex = X[b][0] - X[a][0], ey = X[b][1] - X[a][1];
  const double len = sqrt(ex * ex + ey * ey);
  n[0] = ey / len;
  n[1] = -ex / len;
  if ((X[k][0] - X[a][0]) * n[0] + (X[k][1] - X[a][1]) * n[1] > 0) {
    n[0] = -n[0];
    n[1] = -n[1];
  }
  return len;
}

// SWIPDG on a triangle mesh, output-stationary as on the Kuhn grid: one thread owns the 3 rows of one
// element; its diagonal block is the element Laplace plus the in/in term of each face, its block to
// a neighbour the in/out term of the shared face, both from the element's own side with the terms of
// LocalLaplaceIPDGIntegrands::InnerCoupling + LocalIPDGIntegrands::InnerPenalty
// (local/integrands/laplace-ipdg.hh:107-186, local/integrands/ipdg.hh:113-171), DirichletCoupling +
// BoundaryPenalty on boundary faces (laplace-ipdg.hh:331-368, ipdg.hh:254-282), h = |I|^beta, the
// 2-point Gauss rule on every face. On a face the basis of either element is linear along the shared
// edge, so its values at the face points are the edge parameters of the shared vertices.
__global__ void __launch_bounds__(128) k_mesh_swipdg_rows(GridDesc g, MeshIpdg p, const int* __restrict__ rp,
                                                          double* __restrict__ val, double* __restrict__ rhs,
                                                          const double* __restrict__ kappa, double kappa_const,
                                                          const double* __restrict__ force, double force_const) {
  const long long el = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (el >= g.nelem) return;
  const int e = int(el);
  int w[3];
  double X[3][2], G[3][2];
  const double area = mesh_tri(g, e, w, X, G);
  const double kin = kappa ? kappa[e] : kappa_const;
  const double gq = 0.5 / sqrt(3.0);
  const double xi[2] = {0.5 - gq, 0.5 + gq};
  double D[3][3], O[3][3][3], b[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    b[i] = (force ? force[e] : force_const) * area / 3.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) D[i][j] = kin * area * (G[i][0] * G[j][0] + G[i][1] * G[j][1]);
  }
  int nb[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    int a, bb;
    double n[2];
    const double len = mesh_tri_face(X, k, a, bb, n);
    const double hb = p.beta == 1.0 ? len : pow(len, p.beta);
    double vin[2][3];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
#pragma unroll
      for (int i = 0; i < 3; ++i) vin[q][i] = 0.0;
      vin[q][a] = 1.0 - xi[q];
      vin[q][bb] = xi[q];
    }
    double dn_in[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) dn_in[i] = (kin * G[i][0]) * n[0] + (kin * G[i][1]) * n[1];
    nb[k] = g.mnbr[e * 3 + k];
    if (nb[k] >= 0) {
      int wn[3];
      double Xn[3][2], Gn[3][2];
      mesh_tri(g, nb[k], wn, Xn, Gn);
      const double kout = kappa ? kappa[nb[k]] : kappa_const;
      double vout[2][3];
#pragma unroll
      for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int j = 0; j < 3; ++j) vout[q][j] = wn[j] == w[a] ? 1.0 - xi[q] : (wn[j] == w[bb] ? xi[q] : 0.0);
      double dn_out[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) dn_out[j] = (kout * Gn[j][0]) * n[0] + (kout * Gn[j][1]) * n[1];
      const double win = p.weight_is_diffusion ? kin : 1.0, wout = p.weight_is_diffusion ? kout : 1.0;
      const double delta_plus = wout, delta_minus = win;
      const double weight_minus = delta_plus / (delta_plus + delta_minus);
      const double weight_plus = delta_minus / (delta_plus + delta_minus);
      const double penalty = (p.sigma_in * ((delta_plus * delta_minus) / (delta_plus + delta_minus))) / hb;
#pragma unroll
      for (int ii = 0; ii < 3; ++ii)
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) O[k][ii][jj] = 0.0;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const double fac = 0.5 * len;
#pragma unroll
        for (int ii = 0; ii < 3; ++ii)
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) {
            double v = -1.0 * weight_minus * dn_in[jj] * vin[q][ii];
            v += -1.0 * p.theta * weight_minus * vin[q][jj] * dn_in[ii];
            v += penalty * vin[q][jj] * vin[q][ii];
            D[ii][jj] += v * fac;
            double u = -1.0 * weight_plus * dn_out[jj] * vin[q][ii];
            u += p.theta * weight_minus * vout[q][jj] * dn_in[ii];
            u += -1.0 * penalty * vout[q][jj] * vin[q][ii];
            O[k][ii][jj] += u * fac;
          }
      }
    } else {
      const double wb = p.weight_is_diffusion ? kin : 1.0;
      const double penalty = (p.sigma_bd * wb) / hb;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const double fac = 0.5 * len;
#pragma unroll
        for (int ii = 0; ii < 3; ++ii)
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) {
            double v = -1.0 * dn_in[jj] * vin[q][ii];
            v += -1.0 * p.theta * vin[q][jj] * dn_in[ii];
            v += penalty * vin[q][jj] * vin[q][ii];
            D[ii][jj] += v * fac;
          }
        if (rhs && p.rhs_terms) {
          const double gv = p.g_face ? p.g_face[(3LL * e + k) * 2 + q] : p.g_const;
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            double v = 0.0;
            if (p.rhs_terms & 1) v += -1.0 * p.theta * gv * dn_in[i];
            if (p.rhs_terms & 2) v += penalty * gv * vin[q][i];
            b[i] += v * fac;
          }
        }
      }
    }
  }
  if (rhs)
#pragma unroll
    for (int i = 0; i < 3; ++i) rhs[3LL * e + i] = b[i];
  if (!val) return;
  // blocks in ascending element order: the element itself and its neighbours
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    int pos = rp[3LL * e + i];
    int last = -1;
    for (int s = 0; s < 4; ++s) {
      // the next block: the smallest element id above `last` among e and the neighbours
      int nxt = 0x7fffffff, kk = -2;
      if (e > last && e < nxt) {
        nxt = e;
        kk = -1;
      }
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (nb[k] > last && nb[k] < nxt) {
          nxt = nb[k];
          kk = k;
        }
      if (kk == -2) break;
      last = nxt;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        double v = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k)
          if (kk == k) v = O[k][i][j];
        val[pos++] = kk == -1 ? D[i][j] : v;
      }
    }
  }
}

}  // namespace

gdt_status mesh_dg_pattern(gdt_context ctx, gdt_matrix m) {
  const GridDesc& g = m->test.g;
  if (g.dim != 2 || m->stencil != GDT_STENCIL_ELEMENT_AND_INTERSECTION)
    return fail(ctx, GDT_EUNSUPPORTED, "DG on meshes: 2D with the element_and_intersection stencil");
  cudaStream_t s = ctx->stream;
  const long long rows = m->rows;
  int* count = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&m->rp, sizeof(int) * (rows + 1)));
  GDT_TRY_CUDA(ctx, cudaMalloc(&count, sizeof(int) * (rows + 1)));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(count + rows, 0, sizeof(int), s));
  const int bl = grid_blocks(g.nelem, 128);
  k_mesh_dg_pattern<<<bl, 128, 0, s>>>(g, count, nullptr, nullptr);
  GDT_CHECK(ctx, check_launch(ctx, "mesh DG pattern count"));
  size_t tb = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb, count, m->rp, rows + 1, s);
  void* tmp = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&tmp, tb));
  cub::DeviceScan::ExclusiveSum(tmp, tb, count, m->rp, rows + 1, s);
  int nnz = 0;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&nnz, m->rp + rows, sizeof(int), cudaMemcpyDeviceToHost, s));
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
  cudaFree(tmp);
  cudaFree(count);
  m->nnz = nnz;
  m->max_row = 12;
  GDT_TRY_CUDA(ctx, cudaMalloc(&m->col, sizeof(int) * (nnz + 8)));
  GDT_TRY_CUDA(ctx, cudaMalloc(&m->val, sizeof(double) * (nnz + 8)));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(m->val, 0, sizeof(double) * (nnz + 8), s));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(m->col, 0, sizeof(int) * (nnz + 8), s));
  k_mesh_dg_pattern<<<bl, 128, 0, s>>>(g, nullptr, m->rp, m->col);
  GDT_CHECK(ctx, check_launch(ctx, "mesh DG pattern fill"));
  m->spmv_sched = 0;
  m->tuned = 0;
  return GDT_OK;
}

gdt_status mesh_swipdg(gdt_context ctx, gdt_matrix m, const gdt_ipdg_desc* d, double* rhs) {
  const GridDesc& g = m->test.g;
  if (d->penalty_beta < 0.0 || (d->dirichlet_rhs & ~3)) return fail(ctx, GDT_EINVAL, "SWIPDG descriptor");
  const MeshIpdg p{d->symmetry_prefactor, d->sigma_inner, d->sigma_boundary,
                   d->penalty_beta > 0.0 ? d->penalty_beta : 1.0, d->weight_is_diffusion, d->dirichlet_face,
                   d->dirichlet_const, d->dirichlet_rhs};
  k_mesh_swipdg_rows<<<grid_blocks(g.nelem, 128), 128, 0, ctx->stream>>>(g, p, m->rp, m->val, rhs, d->kappa,
                                                                          d->kappa_const, d->force, d->force_const);
  return check_launch(ctx, "mesh SWIPDG assembly");
}

gdt_status mesh_dg_face_points(const gdt_space_s& sp, double* xy) {
  const auto* md = static_cast<const MeshData*>(sp.mesh_owner.get());
  if (!md || sp.g.dim != 2) return GDT_EUNSUPPORTED;
  const double gq = 0.5 / std::sqrt(3.0);
  const double xi[2] = {0.5 - gq, 0.5 + gq};
  for (long long e = 0; e < sp.g.nelem; ++e)
    for (int k = 0; k < 3; ++k) {
      const int a = k == 0 ? 1 : 0, b = k == 2 ? 1 : 2;
      const double* xa = &md->hx[2 * size_t(md->hcells[size_t(e) * 3 + a])];
      const double* xb = &md->hx[2 * size_t(md->hcells[size_t(e) * 3 + b])];
      for (int q = 0; q < 2; ++q) {
        double* out = xy + ((e * 3 + k) * 2 + q) * 2;
        out[0] = xa[0] + xi[q] * (xb[0] - xa[0]);
        out[1] = xa[1] + xi[q] * (xb[1] - xa[1]);
      }
    }
  return GDT_OK;
}

namespace {

// Element indicators of the EOC studies (test/stationary-eocstudies/base.hh:259-269) on a mesh:
// eta_e^2 = sum_q w_q |det J_e| |grad u_h - g(x_q)|^2 (norm 0) or (u_h(x_q) - v(x_q))^2 (norm 1), the
// reference values given at the points of the reference rule mapped by each element's affine map;
// u_h from the P1 vertex DoFs (continuous) or the element's own DoFs (DG)
template <int DIM>
__global__ void k_mesh_element_error(GridDesc g, int dg, int nq, int norm, const double* __restrict__ phi,
                                     const double* __restrict__ wq, const double* __restrict__ u,
                                     const double* __restrict__ ref, double* __restrict__ eta2) {
  for (long long el = blockIdx.x * (long long)blockDim.x + threadIdx.x; el < g.nelem;
       el += (long long)gridDim.x * blockDim.x) {
    const int e = int(el);
    int w[DIM + 1];
    double G[DIM + 1][DIM];
    const double adet = mesh_element<DIM>(g, e, w, G) * (DIM == 2 ? 2.0 : 6.0);
    double ue[DIM + 1], gu[DIM];
#pragma unroll
    for (int i = 0; i <= DIM; ++i) ue[i] = u[dg ? (DIM + 1) * el + i : w[i]];
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i <= DIM; ++i) s = fma(ue[i], G[i][a], s);
      gu[a] = s;
    }
    double acc = 0.0;
    for (int q = 0; q < nq; ++q) {
      double d2 = 0.0;
      if (norm == 0) {
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
          const double d = gu[a] - ref[(el * nq + q) * DIM + a];
          d2 = fma(d, d, d2);
        }
      } else {
        double v = 0.0;
#pragma unroll
        for (int i = 0; i <= DIM; ++i) v = fma(ue[i], phi[q * (DIM + 1) + i], v);
        const double d = v - ref[el * nq + q];
        d2 = d * d;
      }
      acc = fma(wq[q] * adet, d2, acc);
    }
    eta2[el] = acc;
  }
}

}  // namespace

gdt_status mesh_element_error(gdt_context ctx, const gdt_space_s& sp, int norm, int quad_order, const double* u,
                              const double* ref, double* eta2, double* total) {
  const GridDesc& g = sp.g;
  if (sp.order != 1 || !(sp.kind == GDT_SPACE_CG || (sp.kind == GDT_SPACE_DG && g.dim == 2)))
    return fail(ctx, GDT_EUNSUPPORTED, "element error on meshes: order-1 continuous and DG spaces");
  cudaStream_t st = ctx->stream;
  const ho::QuadratureInfo Q = ho::quadrature_info_order(g, quad_order);
  const int nl = g.dim + 1;
  // P1 on the reference simplex: phi_0 = 1 - sum xi, phi_k = xi_{k-1}
  std::vector<double> phi(size_t(Q.nq) * nl);
  for (int q = 0; q < Q.nq; ++q) {
    double s = 0.0;
    for (int k = 0; k < g.dim; ++k) {
      phi[size_t(q) * nl + k + 1] = Q.x[3 * size_t(q) + k];
      s += Q.x[3 * size_t(q) + k];
    }
    phi[size_t(q) * nl] = 1.0 - s;
  }
  double *dphi = nullptr, *dw = nullptr, *sum = nullptr;
  void* tmp = nullptr;
  struct Freer {
    void* p[4];
    cudaStream_t s;
    ~Freer() {
      for (void* q : p)
        if (q) cudaFreeAsync(q, s);
    }
  } freer{{}, st};
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&dphi, sizeof(double) * phi.size(), st));
  freer.p[0] = dphi;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&dw, sizeof(double) * Q.w.size(), st));
  freer.p[1] = dw;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(dphi, phi.data(), sizeof(double) * phi.size(), cudaMemcpyHostToDevice, st));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(dw, Q.w.data(), sizeof(double) * Q.w.size(), cudaMemcpyHostToDevice, st));
  const int bl = std::max(1, std::min(grid_blocks(g.nelem, 128), ctx->num_sms * 8));
  const int dg = sp.kind == GDT_SPACE_DG ? 1 : 0;
  if (g.dim == 2) k_mesh_element_error<2><<<bl, 128, 0, st>>>(g, dg, Q.nq, norm, dphi, dw, u, ref, eta2);
  else k_mesh_element_error<3><<<bl, 128, 0, st>>>(g, dg, Q.nq, norm, dphi, dw, u, ref, eta2);
  GDT_CHECK(ctx, check_launch(ctx, "mesh element error"));
  if (total) {
    GDT_TRY_CUDA(ctx, cudaMallocAsync(&sum, sizeof(double), st));
    freer.p[2] = sum;
    size_t tb = 0;
    cub::DeviceReduce::Sum(nullptr, tb, eta2, sum, int(g.nelem), st);
    GDT_TRY_CUDA(ctx, cudaMallocAsync(&tmp, std::max<size_t>(tb, 16), st));
    freer.p[3] = tmp;
    cub::DeviceReduce::Sum(tmp, tb, eta2, sum, int(g.nelem), st);
    double h = 0.0;
    GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&h, sum, sizeof(double), cudaMemcpyDeviceToHost, st));
    GDT_TRY_CUDA(ctx, cudaStreamSynchronize(st));
    *total = std::sqrt(h);
  }
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(st));  // the host tables outlive the copies
  return GDT_OK;
}

namespace {

template <typename T>
bool upload(T** dst, const std::vector<T>& src) {
  if (cudaMalloc(dst, sizeof(T) * std::max<size_t>(src.size(), 1)) != cudaSuccess) return false;
  return cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice) == cudaSuccess;
}

}  // namespace

gdt_status mesh_pattern(gdt_context ctx, gdt_matrix m) {
  const GridDesc& g = m->test.g;
  cudaStream_t s = ctx->stream;
  const long long rows = m->rows;
  int* count = nullptr;
  int* err = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&m->rp, sizeof(int) * (rows + 1)));
  GDT_TRY_CUDA(ctx, cudaMalloc(&count, sizeof(int) * (rows + 1)));
  GDT_TRY_CUDA(ctx, cudaMalloc(&err, sizeof(int)));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(count + rows, 0, sizeof(int), s));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(err, 0, sizeof(int), s));
  const int bl = grid_blocks(rows, 128);
  if (g.dim == 2) k_mesh_pattern<2><<<bl, 128, 0, s>>>(g, count, nullptr, nullptr, err);
  else k_mesh_pattern<3><<<bl, 128, 0, s>>>(g, count, nullptr, nullptr, err);
  GDT_CHECK(ctx, check_launch(ctx, "mesh pattern count"));
  size_t tb = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb, count, m->rp, rows + 1, s);
  void* tmp = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&tmp, tb));
  cub::DeviceScan::ExclusiveSum(tmp, tb, count, m->rp, rows + 1, s);
  size_t tbm = 0;
  int* dmax = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&dmax, sizeof(int)));
  cub::DeviceReduce::Max(nullptr, tbm, count, dmax, int(rows), s);
  void* tmpm = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&tmpm, tbm));
  cub::DeviceReduce::Max(tmpm, tbm, count, dmax, int(rows), s);
  int nnz = 0, herr = 0;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&nnz, m->rp + rows, sizeof(int), cudaMemcpyDeviceToHost, s));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&m->max_row, dmax, sizeof(int), cudaMemcpyDeviceToHost, s));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
  cudaFree(tmp);
  cudaFree(tmpm);
  cudaFree(dmax);
  cudaFree(count);
  cudaFree(err);
  if (herr) return fail(ctx, GDT_EUNSUPPORTED, "mesh pattern: a vertex with more than 127 neighbours");
  m->nnz = nnz;
  GDT_TRY_CUDA(ctx, cudaMalloc(&m->col, sizeof(int) * (nnz + 8)));
  GDT_TRY_CUDA(ctx, cudaMalloc(&m->val, sizeof(double) * (nnz + 8)));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(m->val, 0, sizeof(double) * (nnz + 8), s));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(m->col, 0, sizeof(int) * (nnz + 8), s));
  if (g.dim == 2) k_mesh_pattern<2><<<bl, 128, 0, s>>>(g, nullptr, m->rp, m->col, nullptr);
  else k_mesh_pattern<3><<<bl, 128, 0, s>>>(g, nullptr, m->rp, m->col, nullptr);
  GDT_CHECK(ctx, check_launch(ctx, "mesh pattern fill"));
  const double mean = rows ? double(nnz) / double(rows) : 1.0;
  m->spmv_sched = mean <= 16 ? 0 : mean <= 32 ? 1 : mean <= 64 ? 2 : 3;
  m->tuned = 0;
  return GDT_OK;
}

gdt_status mesh_assemble(gdt_context ctx, const GridDesc& g, const int* rp, const int* col, double* val,
                         const gdt_diffusion_desc* d, double* rhs, const double* gD, double gD_const) {
  const int bl = grid_blocks(g.nvert, 128);
  cudaStream_t s = ctx->stream;
  if (g.dim == 2)
    k_mesh_rows<2><<<bl, 128, 0, s>>>(g, rp, col, val, rhs, d->kappa, d->kappa_const, d->force, d->force_const,
                                       d->dirichlet, gD, gD_const);
  else
    k_mesh_rows<3><<<bl, 128, 0, s>>>(g, rp, col, val, rhs, d->kappa, d->kappa_const, d->force, d->force_const,
                                       d->dirichlet, gD, gD_const);
  return check_launch(ctx, "mesh assembly");
}

gdt_status mesh_dirichlet(gdt_context ctx, gdt_matrix m, double* rhs, const double* values, double value_const) {
  const GridDesc& g = m->test.g;
  k_mesh_dirichlet<<<grid_blocks(g.nvert, 256), 256, 0, ctx->stream>>>(g, m->rp, m->col, m->val, rhs, values,
                                                                        value_const);
  return check_launch(ctx, "mesh Dirichlet constraints");
}

gdt_status mesh_dlogkappa(gdt_context ctx, const GridDesc& g, const double* kappa, const double* u, const double* lam,
                          double* out) {
  const int bl = grid_blocks(g.nelem, 128);
  if (g.dim == 2) k_mesh_dlogkappa<2><<<bl, 128, 0, ctx->stream>>>(g, kappa, u, lam, out);
  else k_mesh_dlogkappa<3><<<bl, 128, 0, ctx->stream>>>(g, kappa, u, lam, out);
  return check_launch(ctx, "mesh log-kappa gradient");
}

gdt_status mesh_global_indices(gdt_context ctx, const GridDesc& g, int64_t* out) {
  const long long n = g.nelem * (g.dim + 1);
  k_mesh_indices<<<std::max(1, std::min(grid_blocks(n, 256), ctx->num_sms * 8)), 256, 0, ctx->stream>>>(
      n, g.mcells, reinterpret_cast<long long*>(out));
  return check_launch(ctx, "mesh global indices");
}

}  // namespace gdt

extern "C" gdt_status gdt_grid_create_simplex_mesh(int dim, int64_t nvert, const double* coords, int64_t nelem,
                                                   const int64_t* cells, gdt_grid* out) {
  using namespace gdt;
  if (!out || !coords || !cells) return GDT_EINVAL;
  *out = nullptr;
  if (dim != 2 && dim != 3) return GDT_EUNSUPPORTED;
  if (nvert < dim + 1 || nelem < 1) return GDT_EINVAL;
  const int nl = dim + 1;
  if (nvert >= (1LL << 31) || nelem * nl >= (1LL << 31)) return GDT_EUNSUPPORTED;
  // host copies (the pointers may be host or device memory: unified addressing)
  std::vector<double> X(size_t(nvert) * dim);
  std::vector<int64_t> C(size_t(nelem) * nl);
  if (cudaMemcpy(X.data(), coords, sizeof(double) * X.size(), cudaMemcpyDefault) != cudaSuccess ||
      cudaMemcpy(C.data(), cells, sizeof(int64_t) * C.size(), cudaMemcpyDefault) != cudaSuccess) {
    cudaGetLastError();
    return GDT_EINVAL;
  }
  // elements: vertex indices in range and distinct, positive volume
  std::vector<int> cells32(C.size());
  for (int64_t e = 0; e < nelem; ++e) {
    const int64_t* c = &C[size_t(e) * nl];
    for (int j = 0; j < nl; ++j) {
      if (c[j] < 0 || c[j] >= nvert) return GDT_EINVAL;
      for (int i = 0; i < j; ++i)
        if (c[i] == c[j]) return GDT_EINVAL;
      cells32[size_t(e) * nl + j] = int(c[j]);
    }
    double J[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int k = 0; k < dim; ++k)
      for (int a = 0; a < dim; ++a) J[a][k] = X[size_t(c[k + 1]) * dim + a] - X[size_t(c[0]) * dim + a];
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                       J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                       J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    // positive volume beyond rounding: |det J| against the product of the edge lengths
    double scale = 1.0;
    for (int k = 0; k < dim; ++k) {
      double l2 = 0.0;
      for (int a = 0; a < dim; ++a) l2 += J[a][k] * J[a][k];
      scale *= std::sqrt(l2);
    }
    if (!std::isfinite(det) || !(std::fabs(det) > 1e-12 * scale)) return GDT_EINVAL;
  }
  // faces (an element's vertices without the one at local index k: face k): the boundary vertices are
  // those of faces that belong to one element, the neighbour across face k the other element of it
  struct Face {
    std::array<int, 3> key;
    int e, k;
  };
  std::vector<Face> faces;
  faces.reserve(size_t(nelem) * nl);
  for (int64_t e = 0; e < nelem; ++e)
    for (int skip = 0; skip < nl; ++skip) {
      Face f{{-1, -1, -1}, int(e), skip};
      int k = 0;
      for (int j = 0; j < nl; ++j)
        if (j != skip) f.key[k++] = cells32[size_t(e) * nl + j];
      std::sort(f.key.begin(), f.key.begin() + dim);
      faces.push_back(f);
    }
  std::sort(faces.begin(), faces.end(), [](const Face& a, const Face& b) {
    return a.key != b.key ? a.key < b.key : (a.e != b.e ? a.e < b.e : a.k < b.k);
  });
  std::vector<unsigned char> bnd(size_t(nvert), 0);
  std::vector<int> nbr(cells32.size(), -1);
  for (size_t i = 0; i < faces.size();) {
    size_t j = i + 1;
    while (j < faces.size() && faces[j].key == faces[i].key) ++j;
    if (j - i > 2) return GDT_EINVAL;  // a face shared by three elements: not a manifold mesh
    if (j - i == 1) {
      for (int a = 0; a < dim; ++a) bnd[size_t(faces[i].key[a])] = 1;
    } else {
      nbr[size_t(faces[i].e) * nl + faces[i].k] = faces[i + 1].e;
      nbr[size_t(faces[i + 1].e) * nl + faces[i + 1].k] = faces[i].e;
    }
    i = j;
  }
  // vertex -> element adjacency, elements ascending
  std::vector<int> ptr(size_t(nvert) + 1, 0), adj(cells32.size());
  for (int c : cells32) ++ptr[size_t(c) + 1];
  // every vertex belongs to an element (a vertex of no element would give an empty, singular row)
  for (int64_t v = 0; v < nvert; ++v)
    if (ptr[size_t(v) + 1] == 0) return GDT_EINVAL;
  for (int64_t v = 0; v < nvert; ++v) ptr[size_t(v) + 1] += ptr[size_t(v)];
  std::vector<int> fillpos(ptr.begin(), ptr.end() - 1);
  for (int64_t e = 0; e < nelem; ++e)
    for (int j = 0; j < nl; ++j) adj[size_t(fillpos[size_t(cells32[size_t(e) * nl + j])]++)] = int(e);
  auto* md = new (std::nothrow) MeshData;
  if (!md) return GDT_ENOMEM;
  std::shared_ptr<void> owner(md, [](void* p) { delete static_cast<MeshData*>(p); });
  if (!upload(&md->xv, X) || !upload(&md->cells, cells32) || !upload(&md->v2e_ptr, ptr) || !upload(&md->v2e, adj) ||
      !upload(&md->bnd, bnd) || !upload(&md->nbr, nbr)) {
    cudaGetLastError();
    return GDT_ENOMEM;
  }
  gdt_grid g = new (std::nothrow) gdt_grid_s;
  if (!g) return GDT_ENOMEM;
  GridDesc& d = g->d;
  d.dim = dim;
  d.simplex = 1;
  d.mesh = 1;
  d.nsub = 1;
  d.n[0] = nelem;
  d.vn[0] = nvert;
  d.ncells = nelem;
  d.nelem = nelem;
  d.nvert = nvert;
  d.xv = md->xv;
  d.mcells = md->cells;
  d.v2e_ptr = md->v2e_ptr;
  d.v2e = md->v2e;
  d.mbnd = md->bnd;
  d.mnbr = md->nbr;
  md->hx = std::move(X);
  md->hcells = std::move(cells32);
  g->mesh_owner = owner;
  *out = g;
  return GDT_OK;
}
