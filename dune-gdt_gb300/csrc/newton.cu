// Damped Newton of OperatorInterface::apply_inverse, type "newton" (operators/interfaces.hh:490-599),
// for the affine residual operator x -> A x - range that the EOC studies invert
// (`op->apply_inverse(zero)` on `lhs - rhs`, test/stationary-eocstudies/base.hh:186-191).
//
// Per Newton step l: residual = A x - range and res = ||residual||_2; stop when res < precision,
// fail after max_iter steps. The Jacobian of the affine operator is A itself; the defect system
// A update = -residual is solved by the library's Krylov solver with the initial guess update = x
// (the reference seeds the linear solver with the current iterate) and the relative tolerance
// 0.1 * precision. Automatic damping [DF2015, Sec. 8.4.4.1]: lambda = 1, 1/2, 1/4, ... until the
// candidate x + lambda update has a smaller residual norm than x, at most max_dampening_iter tries.
// Every vector operation runs on the device; the host reads one residual norm per evaluation.
#include <cmath>
#include <string>

#include "linalg.cuh"

namespace gdt {
namespace {

constexpr int TH = 256;

// r = b - A x (so r = -residual), rr = ||r||^2
template <int G, int PL>
__global__ void __launch_bounds__(TH) k_newton_defect(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                      const double* __restrict__ val, const double* __restrict__ x,
                                                      const double* __restrict__ b, double* __restrict__ r,
                                                      double* rr, double* partials, unsigned int* ticket) {
  double a0 = 0.0;
  for_rows_csr<G, PL, double>(n, rp, col, val, x, [&](int row, bool leader, double s) {
    if (leader) {
      const double ri = b[row] - s;
      r[row] = ri;
      a0 = fma(ri, ri, a0);
    }
  });
  double v[1] = {a0};
  if (grid_reduce<1>(v, partials, ticket) && threadIdx.x == 0) *rr = v[0];
}

// y = x + lambda u
__global__ void k_newton_candidate(int n, const double* __restrict__ x, const double* __restrict__ u, double lambda,
                                   double* __restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = fma(lambda, u[i], x[i]);
}

}  // namespace

gdt_status newton_solve(gdt_context ctx, gdt_matrix m, const double* range, double* x, const gdt_newton_opts* o,
                        gdt_newton_info* info) {
  const int n = int(m->rows);
  cudaStream_t s = ctx->stream;
  GDT_CHECK(ctx, tune_spmv(ctx, m));
  const LaunchShape sh = schedule_shape<double>(m->spmv_sched, n, ctx->num_sms);
  const int vec_blocks = std::max(1, std::min(grid_blocks(n, TH), ctx->num_sms * 8));
  double *r = nullptr, *u = nullptr, *cand = nullptr, *rr = nullptr;
  const size_t vb = sizeof(double) * std::max(n, 1);
  struct Freer {
    double** p[4];
    cudaStream_t s;
    ~Freer() {
      for (double** q : p)
        if (*q) cudaFreeAsync(*q, s);
    }
  } freer{{&r, &u, &cand, &rr}, s};
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&r, vb, s));
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&u, vb, s));
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&cand, vb, s));
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&rr, sizeof(double), s));
  // ||range - A y||_2, with r = range - A y left on the device
  auto defect = [&](const double* y, double& norm) -> gdt_status {
#define GDT_NEWTON_DEFECT(GG, PP)                                                                             \
  k_newton_defect<GG, PP><<<sh.blocks, sh.threads, sh.smem, s>>>(n, m->rp, m->col, m->val, y, range, r, rr, \
                                                                 ctx->scratch, ctx->counters)
    GDT_SCHEDULE_SWITCH(m->spmv_sched, GDT_NEWTON_DEFECT)
#undef GDT_NEWTON_DEFECT
    ctx->launches++;
    double h = 0.0;
    GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&h, rr, sizeof(double), cudaMemcpyDeviceToHost, s));
    GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, GDT_ECUDA, std::string("newton residual: ") + cudaGetErrorString(e));
    norm = std::sqrt(h);
    return GDT_OK;
  };
  gdt_newton_info res{};
  gdt_solver_opts lin = o->jacobian_solver;
  lin.tol = 0.1 * o->precision;
  int l = 0;
  while (true) {
    double nrm = 0.0;
    GDT_CHECK(ctx, defect(x, nrm));
    res.residual = nrm;
    res.iterations = l;
    if (info) *info = res;
    if (nrm < o->precision) return GDT_OK;
    if (l >= o->max_iter) return fail(ctx, GDT_ENOCONV, "newton: max iterations reached");
    // A u = -residual = r, initial guess u = x
    GDT_TRY_CUDA(ctx, cudaMemcpyAsync(u, x, vb, cudaMemcpyDeviceToDevice, s));
    gdt_solve_info si{};
    const gdt_status ls = solve(ctx, m, r, u, &lin, &si);
    res.linear_iterations += si.iterations;
    if (info) *info = res;
    if (ls != GDT_OK) return fail(ctx, ls, "newton: could not solve the linear system for the defect");
    double lambda = 1.0, cnrm = 2.0 * nrm;
    int k = 0;
    while (!(cnrm / nrm < 1.0)) {
      if (k >= o->max_dampening_iter) return fail(ctx, GDT_ENOCONV, "newton: max iterations reached when dampening");
      k_newton_candidate<<<vec_blocks, TH, 0, s>>>(n, x, u, lambda, cand);
      ctx->launches++;
      GDT_CHECK(ctx, defect(cand, cnrm));
      lambda /= 2;
      k += 1;
    }
    res.dampening_steps += k - 1;
    GDT_TRY_CUDA(ctx, cudaMemcpyAsync(x, cand, vb, cudaMemcpyDeviceToDevice, s));
    l += 1;
  }
}

}  // namespace gdt

extern "C" gdt_status gdt_newton_solve(gdt_context ctx, gdt_matrix m, const double* range, double* x,
                                       const gdt_newton_opts* opts, gdt_newton_info* info) {
  if (!ctx || !m || !range || !x) return GDT_EINVAL;
  if (m->rows != m->cols) return gdt::fail(ctx, GDT_ESHAPE, "matrix is not square");
  gdt_newton_opts o = opts ? *opts : gdt_newton_default_opts();
  if (!(o.precision > 0.0) || o.max_iter < 0 || o.max_dampening_iter < 1)
    return gdt::fail(ctx, GDT_EINVAL, "newton: precision must be > 0, max_iter >= 0, max_dampening_iter >= 1");
  const gdt_solver_opts& j = o.jacobian_solver;
  if ((j.solver != GDT_SOLVER_CG && j.solver != GDT_SOLVER_BICGSTAB) || j.precond < GDT_PREC_NONE ||
      j.precond > GDT_PREC_ILU0 || (j.precision != GDT_PRECISION_FP64 && j.precision != GDT_PRECISION_MIXED) ||
      j.max_iter < 1)
    return gdt::fail(ctx, GDT_EINVAL, "newton: invalid jacobian_solver options");
  return gdt::newton_solve(ctx, m, range, x, &o, info);
}

extern "C" gdt_newton_opts gdt_newton_default_opts(void) {
  gdt_newton_opts o{};
  o.precision = 1e-7;
  o.max_iter = 100;
  o.max_dampening_iter = 100;
  o.jacobian_solver = gdt_solver_opts{GDT_SOLVER_CG, GDT_PREC_JACOBI, GDT_PRECISION_FP64, 1e-8, 100000, 0, 0.0};
  return o;
}
