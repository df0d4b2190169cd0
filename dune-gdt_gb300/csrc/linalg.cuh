// Device building blocks for CSR SpMV and the device-resident Krylov solvers.
#pragma once
#include "internal.cuh"

namespace gdt {

// Streaming loads for matrix values/indices (read once per SpMV, kept out of L2's way) and normal
// cached loads for the gathered vector (reused across rows, L2 resident).
template <class T>
__device__ __forceinline__ T ld_stream(const T* p) {
  return __ldcs(p);
}

// y_row = sum_k val[k] x[col[k]] over one CSR row, computed by G cooperating lanes; the result is
// valid in every lane of the group. Accumulation in T (FP64 path: double, inner mixed path: float).
// Every lane of the warp must call this (the group reduction shuffles over the full warp): lanes
// without a row pass beg == end.
template <int G, class T>
__device__ __forceinline__ T csr_row(int beg, int end, int lane, const int* __restrict__ col,
                                     const T* __restrict__ val, const T* __restrict__ x) {
  T s = T(0);
#pragma unroll 4
  for (int k = beg + lane; k < end; k += G) s = fma(ld_stream(val + k), x[ld_stream(col + k)], s);
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
  return s;
}

// Warp-uniform loop over the rows of a CSR matrix, G lanes per row: the loop bound depends only on
// the block, so whole warps iterate together and every lane reaches the shuffles of csr_row.
// body(row, active, s) runs in every lane; `active` is false for lanes past the last row.
template <int G, class T, class Body>
__device__ __forceinline__ void for_rows(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                         const T* __restrict__ val, const T* __restrict__ x, Body body) {
  const int lane = threadIdx.x & (G - 1);
  const int rpb = blockDim.x / G;
  for (int row0 = blockIdx.x * rpb; row0 < n; row0 += gridDim.x * rpb) {
    const int row = row0 + threadIdx.x / G;
    const bool active = row < n;
    const int beg = active ? rp[row] : 0, end = active ? rp[row + 1] : 0;
    const T s = csr_row<G, T>(beg, end, lane, col, val, x);
    body(row, active && lane == 0, s);
  }
}

extern __shared__ __align__(16) unsigned char gdt_dyn_smem[];

// Register-pipelined warp staging: a warp owns 32 consecutive rows; every lane first issues all PL of
// its loads of the warp's contiguous CSR slice (values and indices, coalesced, streaming) into
// registers, then stores them to the warp's shared-memory window, so a lane has up to 2 PL loads in
// flight. Lane i then reduces row r0 + i from the window, unrolled over PL with two accumulators so
// the x gathers are independent. PL >= longest row. body(row, active, s) runs in every lane.
template <class T, int PL, class Body>
__device__ __forceinline__ void for_rows_pipelined(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                   const T* __restrict__ val, const T* __restrict__ x, Body body) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  constexpr int cap = 32 * PL;
  T* wv = reinterpret_cast<T*>(gdt_dyn_smem) + warp * cap;
  int* wc = reinterpret_cast<int*>(reinterpret_cast<T*>(gdt_dyn_smem) + wpb * cap) + warp * cap;
  for (int r0 = (blockIdx.x * wpb + warp) * 32; r0 < n; r0 += gridDim.x * wpb * 32) {
    const int row = r0 + lane;
    const bool active = row < n;
    const int rbeg = active ? rp[row] : 0;
    const int rend = active ? rp[row + 1] : 0;
    const int last = (n - 1 - r0) < 31 ? (n - 1 - r0) : 31;
    const int beg = __shfl_sync(0xffffffffu, rbeg, 0);
    const int end = __shfl_sync(0xffffffffu, rend, last);
    const int cnt = end - beg;
    T v[PL];
    int c[PL];
#pragma unroll
    for (int j = 0; j < PL; ++j) {
      const int k = lane + 32 * j;
      if (k < cnt) {
        v[j] = ld_stream(val + beg + k);
        c[j] = ld_stream(col + beg + k);
      }
    }
#pragma unroll
    for (int j = 0; j < PL; ++j) {
      const int k = lane + 32 * j;
      if (k < cnt) {
        wv[k] = v[j];
        wc[k] = c[j];
      }
    }
    __syncwarp();
    T s0 = T(0), s1 = T(0);
    const int a = rbeg - beg, len = rend - rbeg;
#pragma unroll
    for (int j = 0; j < PL; j += 2) {
      if (j < len) s0 = fma(wv[a + j], x[wc[a + j]], s0);
      if (j + 1 < len) s1 = fma(wv[a + j + 1], x[wc[a + j + 1]], s1);
    }
    body(row, active, s0 + s1);
    __syncwarp();
  }
}

// SpMV schedules: PL == 0 -> vector-CSR with G lanes per row; PL > 0 -> pipelined warp staging with
// PL entries per lane (rows of at most PL entries). Chosen per matrix by the autotuner.
template <int G, int PL, class T, class Body>
__device__ __forceinline__ void for_rows_csr(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                             const T* __restrict__ val, const T* __restrict__ x, Body body) {
  if constexpr (PL > 0) for_rows_pipelined<T, PL>(n, rp, col, val, x, body);
  else for_rows<G, T>(n, rp, col, val, x, body);
}

// the schedule table: index -> (G, PL)
constexpr int kSchedules = 7;
__host__ __device__ constexpr int sched_G(int s) { return s == 0 ? 4 : s == 1 ? 8 : s == 2 ? 16 : s == 3 ? 32 : 0; }
__host__ __device__ constexpr int sched_PL(int s) { return s == 4 ? 8 : s == 5 ? 16 : s == 6 ? 32 : 0; }

// expands F<G, PL> for a runtime schedule index
#define GDT_SCHEDULE_SWITCH(sched, F)  \
  switch (sched) {                     \
    case 0: F(4, 0); break;            \
    case 1: F(8, 0); break;            \
    case 2: F(16, 0); break;           \
    case 3: F(32, 0); break;           \
    case 4: F(0, 8); break;            \
    case 5: F(0, 16); break;           \
    default: F(0, 32); break;          \
  }

struct LaunchShape {
  int blocks, threads;
  size_t smem;
};

template <class T>
inline LaunchShape schedule_shape(int sched, long long n, int num_sms) {
  LaunchShape s;
  const int PL = sched_PL(sched);
  if (PL > 0) {
    const size_t per_warp = size_t(32) * PL * (sizeof(T) + sizeof(int));
    int warps = int((48 * 1024) / per_warp);  // within the default 48 KB of dynamic shared memory
    warps = warps > 4 ? 4 : (warps < 1 ? 1 : warps);
    s.threads = 32 * warps;
    s.smem = size_t(warps) * per_warp;
    const long long b = (n + s.threads - 1) / s.threads;
    s.blocks = int(b < num_sms * 16 ? b : num_sms * 16);
  } else {
    const int G = sched_G(sched);
    s.threads = 256;
    s.smem = 0;
    const long long rpb = 256 / G;
    const long long b = (n + rpb - 1) / rpb;
    s.blocks = int(b < num_sms * 8 ? b : num_sms * 8);
  }
  if (s.blocks < 1) s.blocks = 1;
  return s;
}

// schedules usable for a matrix whose longest row has max_row entries
inline bool schedule_valid(int sched, int max_row) {
  const int PL = sched_PL(sched);
  return PL == 0 || (max_row > 0 && max_row <= PL);
}

// Two-level deterministic reduction of NV partial sums over the whole grid: every block writes its
// partials, the last block to arrive (ticket) sums them in block order. Returns true in the last block;
// the totals are then in v[] of thread 0. partials needs NV * gridDim.x doubles.
template <int NV>
__device__ bool grid_reduce(double (&v)[NV], double* __restrict__ partials, unsigned int* __restrict__ ticket) {
  __shared__ double red[NV * 32];
  __shared__ bool last;
  block_reduce<NV>(v, red);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = 0.0;
    for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x) s += __ldcg(partials + k * gridDim.x + b);
    v[k] = s;
  }
  block_reduce<NV>(v, red);
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}

// Runs `body` (one iteration's launches) in graph-captured chunks until the device flag `converged`
// says stop; the host reads the flag once per chunk. In timing mode the body is launched directly.
template <class Body>
inline gdt_status iterate_chunks(gdt_context ctx, cudaStream_t s, const int* converged, int chunk, int max_chunks,
                          Body body) {
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  bool use_graph = true;
  // launches recorded while capturing run once per graph launch: count them there
  const long long before = ctx->launches;
  if (ctx->timing) {
    use_graph = false;  // per-launch events need plain launches
  } else if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    for (int k = 0; k < chunk; ++k) body();
    if (cudaStreamEndCapture(s, &graph) != cudaSuccess ||
        cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
      use_graph = false;
  } else {
    use_graph = false;
  }
  const long long per_chunk = ctx->launches - before;
  ctx->launches = before;
  cudaGetLastError();
  int* flag = reinterpret_cast<int*>(ctx->host_pinned);
  for (int c = 0; c < max_chunks; ++c) {
    if (use_graph) {
      GDT_TRY_CUDA(ctx, cudaGraphLaunch(exec, s));
      ctx->launches += per_chunk;
    } else {
      for (int k = 0; k < chunk; ++k) body();
    }
    GDT_TRY_CUDA(ctx, cudaMemcpyAsync(flag, converged, sizeof(int), cudaMemcpyDeviceToHost, s));
    GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
    if (ctx->timing) timing_harvest(ctx);
    if (*flag) break;
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  return GDT_OK;
}

}  // namespace gdt
