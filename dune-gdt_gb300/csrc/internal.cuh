// Internal declarations of the GB300 discretize-and-solve library (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "gdt_gb300.h"

namespace gdt {

constexpr int kMaxDim = 3;

// Structured grid descriptor, passed by value to kernels. Elements: cube index * nsub + sub,
// cube index and vertex index lexicographic with x fastest (YaspGrid convention).
struct GridDesc {
  int dim = 2;
  int simplex = 0;
  int periodic = 0;
  int nsub = 1;  // simplices per cube (d!), 1 for cube grids
  long long n[3] = {1, 1, 1};
  long long vn[3] = {1, 1, 1};
  double lo[3] = {0, 0, 0};
  double hi[3] = {1, 1, 1};
  double h[3] = {1, 1, 1};
  long long ncells = 1, nelem = 1, nvert = 1;
  // vertex coordinates of a mapped grid (device, [vertex][dim], vertices lexicographic with x fastest);
  // null for the equidistant grid of lo, hi and n. Also the coordinates of a simplex mesh.
  const double* xv = nullptr;
  // Unstructured simplex mesh (mesh = 1; the fields above other than dim, simplex, nelem, nvert and
  // xv are unused): element vertex lists [element][dim + 1], vertex -> element adjacency (CSR over the
  // vertices, elements ascending) and boundary-vertex flags (vertices of faces of one element), all
  // on the device
  int mesh = 0;
  const int* mcells = nullptr;
  const int* v2e_ptr = nullptr;
  const int* v2e = nullptr;
  const unsigned char* mbnd = nullptr;
  const int* mnbr = nullptr;  // element across face k (opposite local vertex k) of element e at e * (dim + 1) + k, or -1
};

}  // namespace gdt

struct gdt_context_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  long long launches = 0;
  // small device scratch for reductions and solver scalars
  double* scratch = nullptr;       // kScratchDoubles doubles
  unsigned int* counters = nullptr; // kCounters uints (last-block tickets)
  double* host_pinned = nullptr;   // pinned host mirror for convergence checks
  int num_sms = 152;
  // kernel timing: when on, solver iterations run without graph capture and the launches of each
  // kernel class (GDT_TIMING_*) are bracketed by CUDA events on the launching stream; durations
  // accumulate per class
  int timing = 0;
  int solver_launch = 0;       // GDT_SOLVER_LAUNCH_* requested for FP64 CG
  int persistent_blocks = 0;   // grid size cap of the persistent solver launches (0: one block per SM)
  long long persistent_wait_ns = 0;  // longest grid-barrier wait of the persistent solvers (0: 1 s)
  int last_solver_launch = 0;  // the form the last FP64 CG solve ran in
  std::vector<cudaEvent_t> events;  // pairs (start, stop)
  std::vector<int> event_kind;      // GDT_TIMING_* class of each pair
  size_t events_used = 0;
  double kind_ms[GDT_TIMING_KINDS] = {};
  long long kind_launches[GDT_TIMING_KINDS] = {};
};

struct gdt_grid_s {
  gdt::GridDesc d;
  std::shared_ptr<double> xv_owner;  // the device coordinates of a mapped grid (d.xv)
  std::shared_ptr<void> mesh_owner;  // the device arrays of a simplex mesh
};

struct gdt_space_s {
  gdt::GridDesc g;
  int kind = GDT_SPACE_CG;
  int order = 1;
  int lsize = 1;
  long long size = 0;
  std::shared_ptr<double> xv_owner;  // keeps g.xv alive with every copy of the space
  std::shared_ptr<void> mesh_owner;  // and the mesh arrays
};

struct gdt_matrix_s {
  gdt_context ctx = nullptr;
  gdt_space_s test, ansatz;
  int stencil = GDT_STENCIL_ELEMENT;
  long long rows = 0, cols = 0, nnz = 0;
  int* rp = nullptr;
  int* col = nullptr;
  double* val = nullptr;
  int max_row = 0;     // longest row
  int spmv_sched = 1;  // SpMV schedule (see linalg.cuh), picked by tune_spmv on first use
  int tuned = 0;
  int pinned = 0;      // schedule set by gdt_matrix_set_schedule: no autotuning
  int cg_sched = -1;   // schedule of the fused FP64 CG iteration, timed inside that iteration (krylov.cu)
  int mx_tiled = -1;   // mixed solver, 3D grids: plane-tiled (1) or linear (0) FP32 stencil SpMV, timed on first use
  void* ho = nullptr;  // element-batched assembly data (order-2 spaces), owned (highorder.cu)
  // 3D Q1 Laplace assemblies: the element coefficients in FP32 and the reference element stiffness
  // (corner-bit indexing), for the matrix-free inner operator of the mixed-precision solver
  float* mf_kappa = nullptr;
  // SELL-32 copy (linalg.cuh SellView): slices of 32 rows stored column-major, padded to the slice's
  // longest row; (offset, width) per slice (from the pattern, built once), values and columns copied
  // from the CSR arrays when the values changed (val_version) and at every solve
  int* sell_meta = nullptr;
  int* sell_col = nullptr;
  double* sell_val = nullptr;
  long long sell_len = 0;
  long long val_version = 0;    // bumped by every entry point that may change the values
  long long sell_version = -1;  // val_version the SELL copy was filled at
  int use_sell = 0;             // plain SpMV and the graph-form CG SpMV read the SELL copy (tuned or pinned)
  float mf_K[64] = {};
  int mf_valid = 0;      // the values are exactly that assembly (cleared by any other value change)
  int mf_dirichlet = 0;  // with Dirichlet unit rows and columns
  int mx_operator = -1;  // inner operator of the last mixed-precision solve (GDT_MIXED_OPERATOR_*)
};

namespace gdt {

constexpr int kScratchDoubles = 1 << 16;
constexpr int kCounters = 64;

gdt_status fail(gdt_context ctx, gdt_status s, const std::string& msg);
// keeps the element coefficients of a 3D Q1 Laplace assembly for the matrix-free FP32 operator
gdt_status mf_capture(gdt_context ctx, gdt_matrix m, const gdt_diffusion_desc* d);
gdt_status check_launch(gdt_context ctx, const char* what);

#define GDT_TRY_CUDA(ctx, call)                                                                   \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) return ::gdt::fail((ctx), GDT_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define GDT_CHECK(ctx, st)            \
  do {                                \
    gdt_status s_ = (st);             \
    if (s_ != GDT_OK) return s_;      \
  } while (0)

inline int grid_blocks(long long n, int threads) { return int((n + threads - 1) / threads); }

// kernel timing helpers (capi.cu): bracket one launch; harvest after a stream synchronisation
void timing_begin(gdt_context ctx, cudaStream_t s, int kind);
void timing_end(gdt_context ctx, cudaStream_t s);
void timing_harvest(gdt_context ctx);

// ---------------------------------------------------------------- kernels (host launchers) ---
// pattern.cu
gdt_status build_pattern(gdt_context ctx, gdt_matrix m);
// unstructured simplex meshes (mesh.cu)
gdt_status mesh_pattern(gdt_context ctx, gdt_matrix m);
gdt_status mesh_assemble(gdt_context ctx, const GridDesc& g, const int* rp, const int* col, double* val,
                         const gdt_diffusion_desc* d, double* rhs, const double* gD, double gD_const);
gdt_status mesh_dirichlet(gdt_context ctx, gdt_matrix m, double* rhs, const double* values, double value_const);
gdt_status mesh_dlogkappa(gdt_context ctx, const GridDesc& g, const double* kappa, const double* u, const double* lam,
                          double* out);
gdt_status mesh_global_indices(gdt_context ctx, const GridDesc& g, int64_t* out);
gdt_status mesh_dg_pattern(gdt_context ctx, gdt_matrix m);
gdt_status mesh_swipdg(gdt_context ctx, gdt_matrix m, const gdt_ipdg_desc* d, double* rhs);
gdt_status mesh_dg_face_points(const gdt_space_s& s, double* xy);
gdt_status mesh_element_error(gdt_context ctx, const gdt_space_s& s, int norm, int quad_order, const double* u,
                              const double* ref, double* eta2, double* total);
// assemble_cg.cu
gdt_status assemble_cg(gdt_context ctx, gdt_matrix m, const gdt_diffusion_desc* d, double* rhs);
gdt_status assemble_cg_rhs(gdt_context ctx, const gdt_space_s& s, const gdt_diffusion_desc* d, double* rhs);
gdt_status dirichlet_apply(gdt_context ctx, gdt_matrix m, double* rhs, const double* values = nullptr,
                           double value_const = 0.0);
gdt_status cg_dlogkappa(gdt_context ctx, const gdt_space_s& s, const double* kappa, const double* u,
                        const double* lam, double* out);
// assemble_ipdg.cu
gdt_status assemble_swipdg(gdt_context ctx, gdt_matrix m, const gdt_ipdg_desc* d, double* rhs);
gdt_status dg_face_points(const gdt_space_s& sp, double* xy);
gdt_status swipdg_dlogkappa(gdt_context ctx, const gdt_space_s& s, const gdt_ipdg_desc* d, const double* u,
                            const double* lam, double* out);
// spmv.cu
gdt_status spmv(gdt_context ctx, gdt_matrix m, const double* x, double* y);
gdt_status tune_spmv(gdt_context ctx, gdt_matrix m, double* times_ms = nullptr);
// SELL-32 copy of m: slice table built once per pattern (GDT_EUNSUPPORTED when there is no room or the
// offsets do not fit 32 bits), values and columns copied when the values changed or `refill` is set
gdt_status sell_prepare(gdt_context ctx, gdt_matrix m, cudaStream_t s, bool refill);
void sell_free(gdt_matrix m);
// index of the SELL-32 schedule in gdt_matrix_tune / gdt_matrix_set_schedule
constexpr int kSellSchedule = 8;
// krylov.cu
gdt_status solve(gdt_context ctx, gdt_matrix m, const double* b, double* x, const gdt_solver_opts* o,
                 gdt_solve_info* info);
// newton.cu
gdt_status newton_solve(gdt_context ctx, gdt_matrix m, const double* range, double* x, const gdt_newton_opts* o,
                        gdt_newton_info* info);
// mixed.cu: FP32 symmetric-stencil CG with FP64 reliable updates (structured continuous spaces)
bool mixed_stencil_supported(gdt_matrix m);
gdt_status solve_mixed_stencil(gdt_context ctx, gdt_matrix m, const double* b, double* x, const gdt_solver_opts* o,
                               gdt_solve_info* info, cudaStream_t s);
// mixed_mf.cu: matrix-free FP32 CG (3D Q1 Laplace, element coefficients kept at assembly) in persistent
// launches with FP64 reliable updates; GDT_EUNSUPPORTED (before touching x) where it does not apply
bool mixed_mf_applies(gdt_matrix m);
gdt_status solve_mixed_mf(gdt_context ctx, gdt_matrix m, const double* b, double* x, const gdt_solver_opts* o,
                          gdt_solve_info* info, cudaStream_t s);
// fv.cu
gdt_status fv_apply(gdt_context ctx, const gdt_space_s& s, const gdt_fv_desc* d, const double* u, double* out);
gdt_status fv_estimate_dt(gdt_context ctx, const gdt_space_s& s, const gdt_fv_desc* d, const double* u0,
                          double* dt);
gdt_status fv_timestep(gdt_context ctx, const gdt_space_s& s, const gdt_fv_desc* d, int stepper, double dt,
                       long long steps, long long nbatch, double* u, double* work);

// ------------------------------------------------------------------ device helpers ---
__host__ __device__ inline void vertex_multi(const GridDesc& g, long long v, long long* vi) {
  vi[0] = v % g.vn[0];
  vi[1] = (v / g.vn[0]) % g.vn[1];
  vi[2] = v / (g.vn[0] * g.vn[1]);
}
__host__ __device__ inline void cell_multi(const GridDesc& g, long long c, long long* ci) {
  ci[0] = c % g.n[0];
  ci[1] = (c / g.n[0]) % g.n[1];
  ci[2] = c / (g.n[0] * g.n[1]);
}
__host__ __device__ inline long long cell_index(const GridDesc& g, const long long* ci) {
  return ci[0] + g.n[0] * (ci[1] + g.n[1] * ci[2]);
}

// Deterministic block reduction of NV doubles; result valid in thread 0.
template <int NV>
__device__ inline void block_reduce(double (&v)[NV], double* smem /* >= NV * 32 */) {
#pragma unroll
  for (int k = 0; k < NV; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) smem[k * 32 + warp] = v[k];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = lane < nw ? smem[k * 32 + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      v[k] = s;
    }
  }
  __syncthreads();
}

}  // namespace gdt
