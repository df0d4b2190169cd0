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
  ~MeshData() {
    cudaFree(xv);
    cudaFree(cells);
    cudaFree(v2e_ptr);
    cudaFree(v2e);
    cudaFree(bnd);
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
  // boundary vertices: those of faces (vertex subsets without one vertex) that belong to one element
  std::vector<std::array<int, 3>> faces;
  faces.reserve(size_t(nelem) * nl);
  for (int64_t e = 0; e < nelem; ++e)
    for (int skip = 0; skip < nl; ++skip) {
      std::array<int, 3> f = {-1, -1, -1};
      int k = 0;
      for (int j = 0; j < nl; ++j)
        if (j != skip) f[k++] = cells32[size_t(e) * nl + j];
      std::sort(f.begin(), f.begin() + dim);
      faces.push_back(f);
    }
  std::sort(faces.begin(), faces.end());
  std::vector<unsigned char> bnd(size_t(nvert), 0);
  for (size_t i = 0; i < faces.size();) {
    size_t j = i + 1;
    while (j < faces.size() && faces[j] == faces[i]) ++j;
    if (j - i > 2) return GDT_EINVAL;  // a face shared by three elements: not a manifold mesh
    if (j - i == 1)
      for (int a = 0; a < dim; ++a) bnd[size_t(faces[i][a])] = 1;
    i = j;
  }
  // vertex -> element adjacency, elements ascending
  std::vector<int> ptr(size_t(nvert) + 1, 0), adj(cells32.size());
  for (int c : cells32) ++ptr[size_t(c) + 1];
  for (int64_t v = 0; v < nvert; ++v) ptr[size_t(v) + 1] += ptr[size_t(v)];
  std::vector<int> fillpos(ptr.begin(), ptr.end() - 1);
  for (int64_t e = 0; e < nelem; ++e)
    for (int j = 0; j < nl; ++j) adj[size_t(fillpos[size_t(cells32[size_t(e) * nl + j])]++)] = int(e);
  auto* md = new (std::nothrow) MeshData;
  if (!md) return GDT_ENOMEM;
  std::shared_ptr<void> owner(md, [](void* p) { delete static_cast<MeshData*>(p); });
  if (!upload(&md->xv, X) || !upload(&md->cells, cells32) || !upload(&md->v2e_ptr, ptr) || !upload(&md->v2e, adj) ||
      !upload(&md->bnd, bnd)) {
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
  g->mesh_owner = owner;
  *out = g;
  return GDT_OK;
}
