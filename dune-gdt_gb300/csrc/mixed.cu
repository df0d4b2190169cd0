// Mixed-precision CG for the structured continuous P1/Q1 matrices: FP32 inner iterations with
// reliable updates (residual replacement) in FP64.
//
// The FP32 operator is the assembled FP64 CSR matrix rounded to FP32 and stored as a symmetric
// stencil: one array per stencil slot with a non-negative linear offset (the diagonal and the
// "upper" neighbours), D_o[i] = A[i][i + o]; the lower entries are read back from the neighbour as
// A[i][i - o] = D_o[i - o]. Arrays and the iterated vector carry a zero halo of the largest offset,
// so the SpMV needs no bounds checks: y_i = D_0[i] x_i + sum_o (D_o[i] x_{i+o} + D_o[i-o] x_{i-o}).
// Per row it streams (1 + upper slots) * 4 bytes instead of the 12 bytes per nonzero of FP64 CSR.
//
// Reliable updates (one Krylov sequence, no restarts): x32 accumulates the FP32 correction; whenever
// the iterated residual has dropped by 10x since the last update (or reached the tolerance), the
// correction is added to the FP64 solution, the true residual r = b - A x is recomputed from the FP64
// CSR matrix and replaces the FP32 residual, and beta is recomputed from it. Convergence is decided
// only on the true FP64 residual.
#include <cmath>
#include <vector>

#include "linalg.cuh"
#include "structured.cuh"

namespace gdt {

namespace {

constexpr int TH = 256;
constexpr int MAXU = 13;  // upper slots of the 27-point stencil

struct MState {
  double rho, rho_prev, alpha, beta, rr, rr0, rr_ref, tol2;
  int iter, max_iter, converged, flag, breakdown, updates;
};

__device__ __forceinline__ bool mstopped(const MState* st) { return *((volatile const int*)&st->converged) != 0; }

struct Stencil {
  int nu;               // upper slots
  long long off[MAXU];  // their linear offsets (> 0)
  long long pad;        // halo = largest offset
};

// D_o arrays: diag at D, upper slot u at D + (u + 1) * ld (each with `pad` leading zeros before index 0)
template <int DIM>
__global__ void k_build_stencil(GridDesc g, int n, const int* __restrict__ rp, const int* __restrict__ col,
                                const double* __restrict__ val, Stencil S, float* __restrict__ D, long long ld,
                                int* __restrict__ bad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      const long long o = (long long)col[k] - i;
      if (o < 0) continue;
      int slot = -1;
      if (o == 0) slot = 0;
      for (int u = 0; u < S.nu; ++u)
        if (S.off[u] == o) slot = u + 1;
      if (slot < 0) {
        atomicExch(bad, 1);
        continue;
      }
      D[slot * ld + S.pad + i] = float(val[k]);
    }
  }
}

// q = A32 p ; p.q -> alpha. NU (upper slots) is a template parameter so the slot loop unrolls and the
// offsets stay in the kernel-parameter bank.
template <int NU>
__global__ void __launch_bounds__(TH) k_mx_spmv(int n, Stencil S, const float* __restrict__ D, long long ld,
                                               const float* __restrict__ p, float* __restrict__ q, MState* st,
                                               double* partials, unsigned int* ticket) {
  if (mstopped(st)) return;
  float acc = 0.f;
  const float* D0 = D + S.pad;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float pi = p[i];
    float s = D0[i] * pi;
#pragma unroll
    for (int u = 0; u < NU; ++u) {
      const float* Du = D + (u + 1) * ld + S.pad;
      const long long o = S.off[u];
      s = fmaf(Du[i], p[i + o], s);
      s = fmaf(Du[i - o], p[i - o], s);
    }
    q[i] = s;
    acc = fmaf(pi, s, acc);
  }
  double v[1] = {double(acc)};
  if (grid_reduce<1>(v, partials, ticket) && threadIdx.x == 0) {
    if (!(v[0] > 0.0) || !isfinite(v[0])) {
      st->breakdown = 1;
      st->converged = 1;
    }
    st->alpha = st->rho / v[0];
  }
}

// x32 += alpha p ; r32 -= alpha q ; rz, rr ; reliable-update trigger
__global__ void __launch_bounds__(TH) k_mx_update(int n, float* __restrict__ x32, const float* __restrict__ p,
                                                 float* __restrict__ r, const float* __restrict__ q,
                                                 const float* __restrict__ dinv, MState* st, double* partials,
                                                 unsigned int* ticket) {
  if (mstopped(st)) return;
  const float alpha = float(st->alpha);
  float a0 = 0.f, a1 = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x32[i] = fmaf(alpha, p[i], x32[i]);
    const float ri = fmaf(-alpha, q[i], r[i]);
    r[i] = ri;
    a0 = fmaf(ri, dinv[i] * ri, a0);
    a1 = fmaf(ri, ri, a1);
  }
  double v[2] = {double(a0), double(a1)};
  if (grid_reduce<2>(v, partials, ticket) && threadIdx.x == 0) {
    st->rho_prev = st->rho;
    st->beta = v[0] / st->rho;
    st->rho = v[0];
    st->rr = v[1];
    st->iter += 1;
    st->flag = (v[1] <= 0.01 * st->rr_ref || v[1] <= st->tol2 * st->rr0 || st->iter >= st->max_iter) ? 1 : 0;
    if (!isfinite(v[1])) {
      st->breakdown = 1;
      st->converged = 1;
    }
  }
}

// reliable update, part 1: x64 += x32, x32 = 0
__global__ void __launch_bounds__(TH) k_mx_accumulate(int n, double* __restrict__ x, float* __restrict__ x32,
                                                     const MState* st) {
  if (mstopped(st) || !*((volatile const int*)&st->flag)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] += double(x32[i]);
    x32[i] = 0.f;
  }
}

// reliable update, part 2: r64 = b - A64 x (FP64 CSR), r32 = r64, beta from the replaced residual
template <int G, int PL>
__global__ void __launch_bounds__(TH) k_mx_true_residual(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                        const double* __restrict__ val, const double* __restrict__ x,
                                                        const double* __restrict__ b, float* __restrict__ r32,
                                                        const float* __restrict__ dinv, MState* st, double* partials,
                                                        unsigned int* ticket) {
  if (mstopped(st) || !*((volatile const int*)&st->flag)) return;
  double a0 = 0.0, a1 = 0.0;
  for_rows_csr<G, PL, double>(n, rp, col, val, x, [&](int row, bool leader, double s) {
    if (leader) {
      const double ri = b[row] - s;
      const float rf = float(ri);
      r32[row] = rf;
      a0 = fma(double(rf), double(dinv[row] * rf), a0);
      a1 = fma(ri, ri, a1);
    }
  });
  double v[2] = {a0, a1};
  if (grid_reduce<2>(v, partials, ticket) && threadIdx.x == 0) {
    st->rr_ref = v[1];
    st->rr = v[1];
    st->beta = v[0] / st->rho_prev;
    st->rho = v[0];
    st->flag = 0;
    st->updates += 1;
    if (v[1] <= st->tol2 * st->rr0 || st->iter >= st->max_iter) st->converged = 1;
    if (!isfinite(v[1])) {
      st->breakdown = 1;
      st->converged = 1;
    }
  }
}

__global__ void __launch_bounds__(TH) k_mx_p(int n, float* __restrict__ p, const float* __restrict__ r,
                                            const float* __restrict__ dinv, const MState* st) {
  if (mstopped(st)) return;
  const float beta = float(st->beta);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = fmaf(beta, p[i], dinv[i] * r[i]);
}

// start: r64 = b - A x (FP64), r32 = r64, p = dinv r32, rho, rr0
template <int G, int PL>
__global__ void __launch_bounds__(TH) k_mx_init(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                               const double* __restrict__ val, const double* __restrict__ x,
                                               const double* __restrict__ b, float* __restrict__ r32,
                                               const float* __restrict__ dinv, float* __restrict__ p, MState* st,
                                               double* partials, unsigned int* ticket) {
  double a0 = 0.0, a1 = 0.0;
  for_rows_csr<G, PL, double>(n, rp, col, val, x, [&](int row, bool leader, double s) {
    if (leader) {
      const double ri = b[row] - s;
      const float rf = float(ri);
      r32[row] = rf;
      const float zi = dinv[row] * rf;
      p[row] = zi;
      a0 = fma(double(rf), double(zi), a0);
      a1 = fma(ri, ri, a1);
    }
  });
  double v[2] = {a0, a1};
  if (grid_reduce<2>(v, partials, ticket) && threadIdx.x == 0) {
    st->rho = v[0];
    st->rho_prev = v[0];
    st->rr = st->rr0 = st->rr_ref = v[1];
    st->iter = 0;
    st->flag = 0;
    st->updates = 0;
    st->breakdown = 0;
    st->converged = (v[1] == 0.0) ? 1 : 0;
  }
}

template <class TD>
__global__ void k_diag_inv(int n, const int* __restrict__ rp, const int* __restrict__ col,
                           const double* __restrict__ val, TD* __restrict__ dinv, int jacobi) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double d = 1.0;
    if (jacobi)
      for (int k = rp[i]; k < rp[i + 1]; ++k)
        if (col[k] == i) d = val[k];
    dinv[i] = TD(1.0 / d);
  }
}

}  // namespace

bool mixed_stencil_supported(gdt_matrix m) {
  return m->test.kind == GDT_SPACE_CG && m->rows == m->test.g.nvert && m->max_row > 0 && m->max_row <= 32;
}

// the stencil slots with a positive linear offset of the P1/Q1 vertex stencil of grid g
static Stencil make_stencil(const GridDesc& g) {
  Stencil S{};
  const int ns = pow3(g.dim);
  for (int k = 0; k < ns; ++k) {
    if (!slot_in_stencil(g.dim, g.simplex != 0, k)) continue;
    long long o = 0, stride = 1;
    for (int a = 0; a < g.dim; ++a) {
      o += slot_offset(k, a) * stride;
      stride *= g.vn[a];
    }
    if (o > 0) S.off[S.nu++] = o;
    if (o > S.pad) S.pad = o;
  }
  return S;
}

gdt_status solve_mixed_stencil(gdt_context ctx, gdt_matrix m, const double* b, double* x, const gdt_solver_opts* o,
                               gdt_solve_info* info, cudaStream_t s) {
  const int n = int(m->rows);
  const GridDesc& g = m->test.g;
  const Stencil S = make_stencil(g);
  const long long ld = n + 2 * S.pad;  // per-slot array with halos
  const int vec_blocks = std::max(1, std::min(grid_blocks(n, TH), ctx->num_sms * 8));
  double* partials = ctx->scratch;
  unsigned int* ticket = ctx->counters;
  std::vector<void*> allocs;
  struct Freer {
    std::vector<void*>* a;
    cudaStream_t s;
    ~Freer() {
      for (void* p : *a) cudaFreeAsync(p, s);
    }
  } freer{&allocs, s};
  auto alloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMallocAsync(&p, bytes, s) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return p;
  };
  float* D = (float*)alloc(sizeof(float) * ld * (S.nu + 1));
  float* pfull = (float*)alloc(sizeof(float) * ld);  // p with zero halos
  float* r32 = (float*)alloc(sizeof(float) * n);
  float* q32 = (float*)alloc(sizeof(float) * n);
  float* x32 = (float*)alloc(sizeof(float) * n);
  float* dinv = (float*)alloc(sizeof(float) * n);
  MState* st = (MState*)alloc(sizeof(MState));
  int* bad = (int*)alloc(sizeof(int));
  if (!D || !pfull || !r32 || !q32 || !x32 || !dinv || !st || !bad) return fail(ctx, GDT_ENOMEM, "mixed solver vectors");
  float* p = pfull + S.pad;
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(D, 0, sizeof(float) * ld * (S.nu + 1), s));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(pfull, 0, sizeof(float) * ld, s));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(x32, 0, sizeof(float) * n, s));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(bad, 0, sizeof(int), s));
  MState init{};
  init.tol2 = o->tol * o->tol;
  init.max_iter = o->max_iter;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(st, &init, sizeof(MState), cudaMemcpyHostToDevice, s));
  if (g.dim == 1) k_build_stencil<1><<<vec_blocks, TH, 0, s>>>(g, n, m->rp, m->col, m->val, S, D, ld, bad);
  else if (g.dim == 2) k_build_stencil<2><<<vec_blocks, TH, 0, s>>>(g, n, m->rp, m->col, m->val, S, D, ld, bad);
  else k_build_stencil<3><<<vec_blocks, TH, 0, s>>>(g, n, m->rp, m->col, m->val, S, D, ld, bad);
  k_diag_inv<float><<<vec_blocks, TH, 0, s>>>(n, m->rp, m->col, m->val, dinv, o->precond == GDT_PREC_JACOBI);
  ctx->launches += 2;
  GDT_CHECK(ctx, tune_spmv(ctx, m));
  const LaunchShape sh = schedule_shape<double>(m->spmv_sched, n, ctx->num_sms);
#define GDT_MX_INIT(GG, PP)                                                                                    \
  k_mx_init<GG, PP><<<sh.blocks, sh.threads, sh.smem, s>>>(n, m->rp, m->col, m->val, x, b, r32, dinv, p, st, partials, \
                                                           ticket)
#define GDT_MX_TRUE_RESIDUAL(GG, PP)                                                                          \
  k_mx_true_residual<GG, PP><<<sh.blocks, sh.threads, sh.smem, s>>>(n, m->rp, m->col, m->val, x, b, r32, dinv, st, \
                                                                    partials, ticket)
  GDT_SCHEDULE_SWITCH(m->spmv_sched, GDT_MX_INIT)
  ctx->launches++;
  const int chunk = o->check_every > 0 ? o->check_every : 32;
  GDT_CHECK(ctx, iterate_chunks(ctx, s, &st->converged, chunk, o->max_iter / chunk + 2, [&] {
    timing_begin(ctx, s, 1);
    switch (S.nu) {
      case 1: k_mx_spmv<1><<<vec_blocks, TH, 0, s>>>(n, S, D, ld, p, q32, st, partials, ticket); break;
      case 3: k_mx_spmv<3><<<vec_blocks, TH, 0, s>>>(n, S, D, ld, p, q32, st, partials, ticket); break;
      case 4: k_mx_spmv<4><<<vec_blocks, TH, 0, s>>>(n, S, D, ld, p, q32, st, partials, ticket); break;
      case 7: k_mx_spmv<7><<<vec_blocks, TH, 0, s>>>(n, S, D, ld, p, q32, st, partials, ticket); break;
      default: k_mx_spmv<13><<<vec_blocks, TH, 0, s>>>(n, S, D, ld, p, q32, st, partials, ticket); break;
    }
    timing_end(ctx, s);
    k_mx_update<<<vec_blocks, TH, 0, s>>>(n, x32, p, r32, q32, dinv, st, partials, ticket);
    k_mx_accumulate<<<vec_blocks, TH, 0, s>>>(n, x, x32, st);
    GDT_SCHEDULE_SWITCH(m->spmv_sched, GDT_MX_TRUE_RESIDUAL)
    k_mx_p<<<vec_blocks, TH, 0, s>>>(n, p, r32, dinv, st);
    ctx->launches += 5;
  }));
#undef GDT_MX_INIT
#undef GDT_MX_TRUE_RESIDUAL
  MState fin;
  int hbad = 0;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&fin, st, sizeof(MState), cudaMemcpyDeviceToHost, s));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
  {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, GDT_ECUDA, std::string("mixed stencil CG: ") + cudaGetErrorString(e));
  }
  if (hbad) return fail(ctx, GDT_EUNSUPPORTED, "matrix entry outside the vertex stencil");
  gdt_solve_info res{};
  res.iterations = fin.iter;
  res.refinements = fin.updates;
  res.rel_residual = fin.rr0 > 0 ? std::sqrt(fin.rr / fin.rr0) : 0.0;
  res.converged = (!fin.breakdown && (fin.rr0 == 0 || fin.rr <= fin.tol2 * fin.rr0)) ? 1 : 0;
  if (info) *info = res;
  if (!res.converged) return fail(ctx, GDT_ENOCONV, "linear solver did not converge");
  return GDT_OK;
}

}  // namespace gdt
