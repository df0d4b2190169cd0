// FP64 throughput and L2 bandwidth of the GPU at hand, measured with CUDA events (no reference
// counterpart: the denominators of the FP64-bound and the L2-resident kernels' rooflines). GB300 runs FP64 at a small fraction of its
// FP32 rate, so the FV stage kernel, the FP64 CSR SpMV and the element assembly are measured against
// these numbers rather than against a nominal figure.
//
// FMA: every thread runs 8 independent chains of dependent FMAs; DMMA: every warp runs 4 independent
// chains of m8n8k4 FP64 tensor-core products. One resident wave of blocks on every SM; the results
// feed a store that never happens for these inputs, so the compiler keeps the arithmetic.
#include "internal.cuh"

namespace gdt {
namespace {

constexpr int kPeakThreads = 256;

__global__ void __launch_bounds__(kPeakThreads) k_peak_dfma(int iters, double seed, double* sink) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + 1e-9 * double(threadIdx.x + 32 * k);
  const double m = 1.0 - 1e-12, c = 1e-13;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == -1.0) sink[blockIdx.x] = s;  // never true for these inputs
}

__device__ __forceinline__ void peak_dmma(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(kPeakThreads) k_peak_dmma(int iters, double seed, double* sink) {
  double d[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) d[k] = 0.0;
  const double a = seed * 1e-3, b = 1e-3 + 1e-12 * double(threadIdx.x);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k) peak_dmma(d[2 * k], d[2 * k + 1], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += d[k];
  if (s == -1.0) sink[blockIdx.x] = s;
}

// L2 bandwidth: float4 copies between two 24 MB buffers (together well inside the 129 MB L2),
// `reps` passes in one launch; the empty asm statement between passes keeps the compiler from
// hoisting the loads out of the pass loop
__global__ void __launch_bounds__(kPeakThreads) k_l2_copy(const float4* __restrict__ a, float4* __restrict__ b,
                                                          long long n4, int reps) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (int r = 0; r < reps; ++r) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += stride) b[i] = a[i];
    asm volatile("" ::: "memory");
  }
}

}  // namespace
}  // namespace gdt

extern "C" gdt_status gdt_measure_l2_bandwidth(gdt_context ctx, double* gbs) {
  using namespace gdt;
  if (!ctx || !gbs) return GDT_EINVAL;
  cudaStream_t s = ctx->stream;
  const long long n4 = (24ll << 20) / 16;  // 24 MB per buffer
  const int reps = 64;
  float4* buf = nullptr;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&buf, sizeof(float4) * 2 * n4, s));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(buf, 0, sizeof(float4) * 2 * n4, s));
  int per_sm = 0;
  GDT_TRY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_l2_copy, kPeakThreads, 0));
  const int blocks = ctx->num_sms * std::max(per_sm, 1);
  cudaEvent_t e0, e1;
  GDT_TRY_CUDA(ctx, cudaEventCreate(&e0));
  GDT_TRY_CUDA(ctx, cudaEventCreate(&e1));
  float best = 1e30f;
  k_l2_copy<<<blocks, kPeakThreads, 0, s>>>(buf, buf + n4, n4, reps);  // warm-up: the buffers into L2
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0, s);
    k_l2_copy<<<blocks, kPeakThreads, 0, s>>>(buf, buf + n4, n4, reps);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.f && ms < best) best = ms;
  }
  ctx->launches += 4;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(buf, s);
  // read + write bytes
  *gbs = 2.0 * 16.0 * double(n4) * reps / (double(best) * 1e-3) / 1e9;
  return check_launch(ctx, "l2 bandwidth");
}

extern "C" gdt_status gdt_measure_fp64_peak(gdt_context ctx, double* fma_tflops, double* dmma_tflops) {
  using namespace gdt;
  if (!ctx || (!fma_tflops && !dmma_tflops)) return GDT_EINVAL;
  cudaStream_t s = ctx->stream;
  int per_sm_f = 0, per_sm_d = 0;
  GDT_TRY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_f, k_peak_dfma, kPeakThreads, 0));
  GDT_TRY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_d, k_peak_dmma, kPeakThreads, 0));
  const int bf = ctx->num_sms * std::max(per_sm_f, 1), bd = ctx->num_sms * std::max(per_sm_d, 1);
  const int iters_f = 1 << 13, iters_d = 1 << 12;
  cudaEvent_t e0, e1;
  GDT_TRY_CUDA(ctx, cudaEventCreate(&e0));
  GDT_TRY_CUDA(ctx, cudaEventCreate(&e1));
  double* sink = ctx->scratch;  // never written for these inputs
  auto best_ms = [&](auto launch) {
    float best = 1e30f;
    launch();  // warm-up
    for (int r = 0; r < 3; ++r) {
      cudaEventRecord(e0, s);
      launch();
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.f && ms < best) best = ms;
    }
    return double(best);
  };
  if (fma_tflops) {
    const double ms = best_ms([&] { k_peak_dfma<<<bf, kPeakThreads, 0, s>>>(iters_f, 1.0, sink); });
    ctx->launches += 4;
    // 8 chains x 2 flops per FMA
    *fma_tflops = 16.0 * double(iters_f) * bf * kPeakThreads / (ms * 1e-3) / 1e12;
  }
  if (dmma_tflops) {
    const double ms = best_ms([&] { k_peak_dmma<<<bd, kPeakThreads, 0, s>>>(iters_d, 1.0, sink); });
    ctx->launches += 4;
    // 4 chains x m8n8k4 (512 flops) per warp and iteration
    *dmma_tflops = 4.0 * 512.0 * double(iters_d) * bd * (kPeakThreads / 32) / (ms * 1e-3) / 1e12;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return check_launch(ctx, "fp64 peak");
}
