// CSR SpMV y = A x (ConstMatrixOperator::apply, operators/matrix-based.hh:121-129) and the SpMV
// schedule autotuner.
//
// Schedules (linalg.cuh): vector-CSR with G in {4, 8, 16, 32} lanes per row, register-pipelined
// warp staging with PL in {8, 16, 32} entries per lane, or cp.async double-buffered warp staging for
// rows of at most 28 entries. The first SpMV-type call on a matrix times every schedule valid for its
// longest row with CUDA events (FP64, on a non-trivial probe vector, three launches each, after one
// warm-up) and keeps the fastest; all SpMV-type kernels of that matrix (plain, fused dot, residual,
// mixed-precision residual) then use it.
#include <cfloat>

#include "linalg.cuh"

namespace gdt {

template <int G, int PL, class T>
__global__ void __launch_bounds__(256) spmv_kernel(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                   const T* __restrict__ val, const T* __restrict__ x,
                                                   T* __restrict__ y) {
  for_rows_csr<G, PL, T>(n, rp, col, val, x, [&](int row, bool leader, T s) {
    if (leader) y[row] = s;
  });
}

template <class T>
void launch_spmv(int sched, int n, const int* rp, const int* col, const T* val, const T* x, T* y, int num_sms,
                 cudaStream_t s) {
  const LaunchShape sh = schedule_shape<T>(sched, n, num_sms);
#define GDT_SPMV_LAUNCH(GG, PP) spmv_kernel<GG, PP, T><<<sh.blocks, sh.threads, sh.smem, s>>>(n, rp, col, val, x, y)
  GDT_SCHEDULE_SWITCH(sched, GDT_SPMV_LAUNCH)
#undef GDT_SPMV_LAUNCH
}

template void launch_spmv<double>(int, int, const int*, const int*, const double*, const double*, double*, int,
                                  cudaStream_t);
template void launch_spmv<float>(int, int, const int*, const int*, const float*, const float*, float*, int,
                                 cudaStream_t);

// probe vector of the autotuner: non-trivial values (an all-zero x would time the FMAs on zero operands)
__global__ void k_probe_vector(int n, double* __restrict__ x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] = 1.0 + 0.001 * double(i % 997);
}

gdt_status tune_spmv(gdt_context ctx, gdt_matrix m, double* times_ms) {
  if (m->tuned && !times_ms) return GDT_OK;
  if (times_ms)
    for (int k = 0; k < kSchedules; ++k) times_ms[k] = -1.0;
  const int n = int(m->rows);
  cudaStream_t s = ctx->stream;
  double *x = nullptr, *y = nullptr;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&x, sizeof(double) * std::max(n, 1), s));
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&y, sizeof(double) * std::max(n, 1), s));
  k_probe_vector<<<std::max(1, std::min(grid_blocks(n, 256), ctx->num_sms * 8)), 256, 0, s>>>(n, x);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = FLT_MAX;
  int best_sched = m->spmv_sched;
  for (int sched = 0; sched < kSchedules; ++sched) {
    if (!schedule_valid(sched, m->max_row)) continue;
    launch_spmv<double>(sched, n, m->rp, m->col, m->val, x, y, ctx->num_sms, s);
    cudaEventRecord(e0, s);
    for (int r = 0; r < 3; ++r) launch_spmv<double>(sched, n, m->rp, m->col, m->val, x, y, ctx->num_sms, s);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    const bool ok = cudaGetLastError() == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
    if (ok && times_ms) times_ms[sched] = ms / 3.0;
    if (ok && ms < best) {
      best = ms;
      best_sched = sched;
    }
    ctx->launches += 4;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(x, s);
  cudaFreeAsync(y, s);
  m->spmv_sched = best_sched;
  m->tuned = 1;
  return GDT_OK;
}

gdt_status spmv(gdt_context ctx, gdt_matrix m, const double* x, double* y) {
  GDT_CHECK(ctx, tune_spmv(ctx, m));
  timing_begin(ctx, ctx->stream, GDT_TIMING_SPMV_FP64);
  launch_spmv<double>(m->spmv_sched, int(m->rows), m->rp, m->col, m->val, x, y, ctx->num_sms, ctx->stream);
  timing_end(ctx, ctx->stream);
  return check_launch(ctx, "spmv");
}

}  // namespace gdt

extern "C" gdt_status gdt_matrix_tune(gdt_context ctx, gdt_matrix m, int* schedule, double* times_ms) {
  if (!ctx || !m) return GDT_EINVAL;
  m->tuned = 0;
  m->pinned = 0;
  m->cg_sched = -1;
  GDT_CHECK(ctx, gdt::tune_spmv(ctx, m, times_ms));
  if (schedule) *schedule = m->spmv_sched;
  return GDT_OK;
}

extern "C" gdt_status gdt_matrix_set_schedule(gdt_matrix m, int schedule) {
  static_assert(gdt::kSchedules == GDT_SPMV_SCHEDULES, "schedule table and header disagree");
  if (!m || schedule < 0 || schedule >= gdt::kSchedules || !gdt::schedule_valid(schedule, m->max_row))
    return GDT_EINVAL;
  m->spmv_sched = schedule;
  m->tuned = 1;
  m->pinned = 1;
  m->cg_sched = schedule;
  return GDT_OK;
}

extern "C" int gdt_matrix_mixed_operator(gdt_matrix m) { return m ? m->mx_operator : -1; }
