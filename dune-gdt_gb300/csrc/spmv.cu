// CSR SpMV y = A x (ConstMatrixOperator::apply, operators/matrix-based.hh:121-129), its SELL-32
// form, and the SpMV schedule autotuner.
//
// Schedules (linalg.cuh): vector-CSR with G in {4, 8, 16, 32} lanes per row, register-pipelined
// warp staging with PL in {8, 16, 32} entries per lane, cp.async double-buffered warp staging for
// rows of at most 28 entries, and (index 8) the SELL-32 copy of the matrix read one lane per row.
// The first SpMV-type call on a matrix times every schedule valid for its longest row with CUDA
// events (FP64, on a non-trivial probe vector, three launches each, after one warm-up) and keeps the
// fastest CSR schedule for all CSR kernels of that matrix (plain, fused dot, residual,
// mixed-precision residual); when the SELL-32 schedule is faster still, the plain SpMV and the
// graph-form CG SpMV read the SELL copy instead.
#include <cfloat>
#include <mutex>
#include <vector>

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

// ------------------------------------------------------------------------------ SELL-32 ---
// widths: one warp per slice, the longest row of its 32
__global__ void k_sell_width(int n, int nslices, const int* __restrict__ rp, int* __restrict__ width) {
  const int slice = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (slice >= nslices) return;
  const int row = slice * 32 + (threadIdx.x & 31);
  const int len = row < n ? rp[row + 1] - rp[row] : 0;
  const int w = __reduce_max_sync(0xffffffffu, len);
  if ((threadIdx.x & 31) == 0) width[slice] = w;
}

// values and columns from the CSR arrays; padding entries are 0 * x[row] (row 0 past the end)
__global__ void k_sell_fill(int n, int nslices, const int* __restrict__ rp, const int* __restrict__ col,
                            const double* __restrict__ val, const int2* __restrict__ meta, int* __restrict__ scol,
                            double* __restrict__ sval) {
  const int slice = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (slice >= nslices) return;
  const int lane = threadIdx.x & 31;
  const int row = slice * 32 + lane;
  const int2 md = meta[slice];
  const int beg = row < n ? rp[row] : 0, len = row < n ? rp[row + 1] - beg : 0;
  for (int t = 0; t < md.y; ++t) {
    const long long k = md.x + (long long)t * 32 + lane;
    scol[k] = t < len ? col[beg + t] : (row < n ? row : 0);
    sval[k] = t < len ? val[beg + t] : 0.0;
  }
}

void sell_free(gdt_matrix m) {
  if (m->sell_meta) cudaFree(m->sell_meta);
  if (m->sell_col) cudaFree(m->sell_col);
  if (m->sell_val) cudaFree(m->sell_val);
  m->sell_meta = m->sell_col = nullptr;
  m->sell_val = nullptr;
  m->sell_len = 0;
  m->sell_version = -1;
}

gdt_status sell_prepare(gdt_context ctx, gdt_matrix m, cudaStream_t s, bool refill) {
  const int n = int(m->rows);
  const int nslices = (n + 31) / 32;
  const int blocks = (nslices * 32 + 255) / 256;
  if (!m->sell_meta) {
    int* width = nullptr;
    if (cudaMalloc(&width, sizeof(int) * nslices) != cudaSuccess) {
      cudaGetLastError();
      return GDT_EUNSUPPORTED;
    }
    k_sell_width<<<blocks, 256, 0, s>>>(n, nslices, m->rp, width);
    ctx->launches++;
    std::vector<int> w(nslices);
    cudaError_t e = cudaMemcpyAsync(w.data(), width, sizeof(int) * nslices, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(width);
    if (e != cudaSuccess) return fail(ctx, GDT_ECUDA, std::string("sell widths: ") + cudaGetErrorString(e));
    std::vector<int> meta(2 * size_t(nslices));
    long long off = 0;
    for (int i = 0; i < nslices; ++i) {
      meta[2 * i] = int(off);
      meta[2 * i + 1] = w[i];
      off += 32LL * w[i];
    }
    if (off >= (1LL << 31)) return GDT_EUNSUPPORTED;  // offsets are 32-bit
    int* dmeta = nullptr;
    int* dcol = nullptr;
    double* dval = nullptr;
    e = cudaMalloc(&dmeta, sizeof(int) * meta.size());
    if (e == cudaSuccess) e = cudaMalloc(&dcol, sizeof(int) * std::max(off, 1LL));
    if (e == cudaSuccess) e = cudaMalloc(&dval, sizeof(double) * std::max(off, 1LL));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dmeta, meta.data(), sizeof(int) * meta.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      cudaFree(dmeta);
      cudaFree(dcol);
      cudaFree(dval);
      cudaGetLastError();
      return GDT_EUNSUPPORTED;  // no room for the copy
    }
    m->sell_meta = dmeta;
    m->sell_col = dcol;
    m->sell_val = dval;
    m->sell_len = off;
    m->sell_version = -1;
  }
  if (refill || m->sell_version != m->val_version) {
    k_sell_fill<<<blocks, 256, 0, s>>>(n, nslices, m->rp, m->col, m->val, reinterpret_cast<const int2*>(m->sell_meta),
                                       m->sell_col, m->sell_val);
    m->sell_version = m->val_version;
    return check_launch(ctx, "sell fill");
  }
  return GDT_OK;
}

SellView sell_view(gdt_matrix m) {
  return SellView{int(m->rows), int((m->rows + 31) / 32), reinterpret_cast<const int2*>(m->sell_meta), m->sell_col,
                  m->sell_val};
}

__global__ void __launch_bounds__(256) sell_spmv_kernel(SellView A, const double* __restrict__ x, double* __restrict__ y) {
  for_slices(A, x, [&](int row, bool active, double s, double) {
    if (active) y[row] = s;
  });
}

// one warp per slice in blocks of 8 warps (256 threads), no more blocks than `kernel` keeps resident at
// once (its own occupancy: the fused solver kernels hold more registers than the plain SpMV, and a
// grid sized for the plain one would run a second, partial wave)
int sell_blocks(long long nslices, int num_sms, const void* kernel) {
  static std::mutex lock;
  static std::vector<std::pair<const void*, int>> known;  // (kernel, resident 256-thread blocks per SM)
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> g(lock);
    for (const auto& k : known)
      if (k.first == kernel) per_sm = k.second;
    if (per_sm == 0) {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
      cudaGetLastError();
      known.emplace_back(kernel, per_sm);
    }
  }
  const long long want = (nslices + 7) / 8;
  return int(std::max(1LL, std::min<long long>(want, (long long)num_sms * per_sm)));
}

void launch_sell_spmv(gdt_matrix m, const double* x, double* y, int num_sms, cudaStream_t s) {
  const SellView A = sell_view(m);
  sell_spmv_kernel<<<sell_blocks(A.nslices, num_sms, reinterpret_cast<const void*>(&sell_spmv_kernel)), 256, 0, s>>>(
      A, x, y);
}

// probe vector of the autotuner: non-trivial values (an all-zero x would time the FMAs on zero operands)
__global__ void k_probe_vector(int n, double* __restrict__ x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] = 1.0 + 0.001 * double(i % 997);
}

gdt_status tune_spmv(gdt_context ctx, gdt_matrix m, double* times_ms) {
  if (m->tuned && !times_ms) return GDT_OK;
  if (times_ms)
    for (int k = 0; k < GDT_SPMV_SCHEDULES; ++k) times_ms[k] = -1.0;
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
  auto time3 = [&](auto launch, float& ms) {
    launch();
    cudaEventRecord(e0, s);
    for (int r = 0; r < 3; ++r) launch();
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    ms = 0.f;
    ctx->launches += 4;
    return cudaGetLastError() == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
  };
  for (int sched = 0; sched < kSchedules; ++sched) {
    if (!schedule_valid(sched, m->max_row)) continue;
    float ms = 0.f;
    const bool ok = time3([&] { launch_spmv<double>(sched, n, m->rp, m->col, m->val, x, y, ctx->num_sms, s); }, ms);
    if (ok && times_ms) times_ms[sched] = ms / 3.0;
    if (ok && ms < best) {
      best = ms;
      best_sched = sched;
    }
  }
  // the SELL-32 copy, when there is room for it
  bool sell_best = false;
  if (sell_prepare(ctx, m, s, false) == GDT_OK) {
    float ms = 0.f;
    const bool ok = time3([&] { launch_sell_spmv(m, x, y, ctx->num_sms, s); }, ms);
    if (ok && times_ms) times_ms[kSellSchedule] = ms / 3.0;
    sell_best = ok && ms < best;
  }
  cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(x, s);
  cudaFreeAsync(y, s);
  m->spmv_sched = best_sched;
  m->use_sell = sell_best ? 1 : 0;
  // keep the copy only where a solver or the SpMV reads it (the persistent CG takes rows of <= 32)
  if (!sell_best && m->max_row > 32) sell_free(m);
  m->tuned = 1;
  return GDT_OK;
}

gdt_status spmv(gdt_context ctx, gdt_matrix m, const double* x, double* y) {
  GDT_CHECK(ctx, tune_spmv(ctx, m));
  if (m->use_sell && sell_prepare(ctx, m, ctx->stream, false) != GDT_OK) m->use_sell = 0;
  timing_begin(ctx, ctx->stream, GDT_TIMING_SPMV_FP64);
  if (m->use_sell) launch_sell_spmv(m, x, y, ctx->num_sms, ctx->stream);
  else launch_spmv<double>(m->spmv_sched, int(m->rows), m->rp, m->col, m->val, x, y, ctx->num_sms, ctx->stream);
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
  if (schedule) *schedule = m->use_sell ? gdt::kSellSchedule : m->spmv_sched;
  return GDT_OK;
}

extern "C" gdt_status gdt_matrix_set_schedule(gdt_matrix m, int schedule) {
  static_assert(gdt::kSchedules + 1 == GDT_SPMV_SCHEDULES, "schedule table and header disagree");
  static_assert(gdt::kSellSchedule == gdt::kSchedules, "the SELL-32 schedule follows the CSR ones");
  if (!m || schedule < 0 || schedule >= GDT_SPMV_SCHEDULES) return GDT_EINVAL;
  if (schedule == gdt::kSellSchedule) {
    // the CSR kernels (residuals, mixed-precision checks) keep their schedule
    m->use_sell = 1;
  } else {
    if (!gdt::schedule_valid(schedule, m->max_row)) return GDT_EINVAL;
    m->spmv_sched = schedule;
    m->use_sell = 0;
  }
  m->tuned = 1;
  m->pinned = 1;
  m->cg_sched = schedule;
  return GDT_OK;
}

extern "C" gdt_status gdt_matrix_values_changed(gdt_matrix m) {
  if (!m) return GDT_EINVAL;
  m->val_version++;
  m->mf_valid = 0;
  return GDT_OK;
}

extern "C" int gdt_matrix_mixed_operator(gdt_matrix m) { return m ? m->mx_operator : -1; }
