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

// calls body(row, active, s) or, with a prefetched per-row value, body(row, active, s, w[row])
template <bool HASW, class T, class Body>
__device__ __forceinline__ void row_body(Body& body, int row, bool active, T s, T wr) {
  if constexpr (HASW) body(row, active, s, wr);
  else body(row, active, s);
}

// Warp-uniform loop over the rows of a CSR matrix, G lanes per row: the loop bound depends only on
// the block, so whole warps iterate together and every lane reaches the shuffles of csr_row.
// body(row, active, s) runs in every lane; `active` is false for lanes past the last row. With HASW
// the value w[row] (a vector the body combines with the row result, e.g. for a fused dot product) is
// loaded together with the row bounds, before the row's gathers, and passed as a fourth argument:
// loading it after the row reduction would add one dependent memory latency to every row.
template <int G, class T, bool HASW = false, class Body>
__device__ __forceinline__ void for_rows(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                         const T* __restrict__ val, const T* __restrict__ x, Body body,
                                         const T* __restrict__ w = nullptr) {
  const int lane = threadIdx.x & (G - 1);
  const int rpb = blockDim.x / G;
  for (int row0 = blockIdx.x * rpb; row0 < n; row0 += gridDim.x * rpb) {
    const int row = row0 + threadIdx.x / G;
    const bool active = row < n;
    const int beg = active ? rp[row] : 0, end = active ? rp[row + 1] : 0;
    const T wr = (HASW && active && lane == 0) ? w[row] : T(0);
    const T s = csr_row<G, T>(beg, end, lane, col, val, x);
    row_body<HASW>(body, row, active && lane == 0, s, wr);
  }
}

extern __shared__ __align__(16) unsigned char gdt_dyn_smem[];

// Register-pipelined warp staging: a warp owns 32 consecutive rows; every lane first issues all PL of
// its loads of the warp's contiguous CSR slice (values and indices, coalesced, streaming) into
// registers, then stores them to the warp's shared-memory window, so a lane has up to 2 PL loads in
// flight. Lane i then reduces row r0 + i from the window, unrolled over PL with two accumulators so
// the x gathers are independent. PL >= longest row. body(row, active, s) runs in every lane.
template <class T, int PL, bool HASW = false, class Body>
__device__ __forceinline__ void for_rows_pipelined(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                   const T* __restrict__ val, const T* __restrict__ x, Body body,
                                                   const T* __restrict__ w = nullptr) {
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
    const T wr = (HASW && active) ? w[row] : T(0);
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
    row_body<HASW>(body, row, active, s0 + s1, wr);
    __syncwarp();
  }
}

// 16-byte asynchronous global -> shared copies (LDGSTS, L2 only) and their group waits
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
// 4-byte asynchronous copy; when `valid` is false nothing is read and the word is zero-filled
__device__ __forceinline__ void cp_async4_zfill(void* smem, const void* gmem, bool valid) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  const int bytes = valid ? 4 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Asynchronous double-buffered warp staging: each warp owns 32 consecutive rows per step. While it
// reduces the current slice from one shared-memory buffer, the next slice (values and indices,
// rounded out to 16-byte boundaries; the CSR arrays carry padding) is already being copied into the
// other buffer with cp.async. Lane i reduces row r0 + i: one lane per row, so the FP64 instructions
// per row are the row's FMAs only (no shuffle reductions). Rows of at most CAP entries.
template <class T, int CAP>
struct AsyncWindow {
  static constexpr int VE = 16 / sizeof(T);            // values per 16-byte chunk
  static constexpr int VCAP = 32 * CAP + 2 * VE;       // values per buffer (slack for alignment)
  static constexpr int CCAP = 32 * CAP + 8;            // indices per buffer
  static constexpr size_t bytes_per_warp = 2 * (VCAP * sizeof(T) + CCAP * sizeof(int));
};

template <class T, int CAP, bool HASW = false, class Body>
__device__ __forceinline__ void for_rows_async(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                               const T* __restrict__ val, const T* __restrict__ x, Body body,
                                               const T* __restrict__ w = nullptr) {
  using W = AsyncWindow<T, CAP>;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  unsigned char* const base = gdt_dyn_smem + warp * W::bytes_per_warp;
  auto vbuf = [&](int b) { return reinterpret_cast<T*>(base + b * (W::VCAP * sizeof(T))); };
  auto cbuf = [&](int b) {
    return reinterpret_cast<int*>(base + 2 * W::VCAP * sizeof(T) + b * (W::CCAP * sizeof(int)));
  };
  const int step = gridDim.x * wpb * 32;
  // stage the slice of rows [r, r+32) into buffer b; returns this lane's row bounds and the slice's
  // aligned (value, index) start offsets. Warp-uniform: every lane calls it.
  auto stage = [&](int r, int b, int& rbeg, int& rend, int& vb, int& cb) {
    const int row = r + lane;
    rbeg = row < n ? rp[row] : 0;
    rend = row < n ? rp[row + 1] : 0;
    const int last = (n - 1 - r) < 31 ? (n - 1 - r) : 31;
    const int beg = __shfl_sync(0xffffffffu, rbeg, 0);
    const int end = __shfl_sync(0xffffffffu, rend, last);
    vb = beg & ~(W::VE - 1);
    cb = beg & ~3;
    const int nv = (end - vb + W::VE - 1) / W::VE, nc = (end - cb + 3) / 4;
    T* dv = vbuf(b);
    int* dc = cbuf(b);
    for (int k = lane; k < nv; k += 32) cp_async16(dv + k * W::VE, val + vb + k * W::VE);
    for (int k = lane; k < nc; k += 32) cp_async16(dc + k * 4, col + cb + k * 4);
    cp_async_commit();
  };
  int r0 = (blockIdx.x * wpb + warp) * 32;
  int rb = 0, re = 0, vb = 0, cb = 0, cur = 0;
  if (r0 < n) stage(r0, 0, rb, re, vb, cb);
  for (; r0 < n; r0 += step, cur ^= 1) {
    const bool more = r0 + step < n;
    int rb2 = 0, re2 = 0, vb2 = 0, cb2 = 0;
    if (more) {
      stage(r0 + step, cur ^ 1, rb2, re2, vb2, cb2);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    const int row = r0 + lane;
    const bool active = row < n;
    const T wr = (HASW && active) ? w[row] : T(0);
    __syncwarp();
    const T* wv = vbuf(cur) + (rb - vb);
    const int* wc = cbuf(cur) + (rb - cb);
    const int len = re - rb;
    T s0 = T(0), s1 = T(0);
#pragma unroll
    for (int j = 0; j < CAP; j += 2) {
      if (j < len) s0 = fma(wv[j], __ldg(x + wc[j]), s0);
      if (j + 1 < len) s1 = fma(wv[j + 1], __ldg(x + wc[j + 1]), s1);
    }
    row_body<HASW>(body, row, active, s0 + s1, wr);
    __syncwarp();  // the buffer just read is refilled by the next stage
    rb = rb2, re = re2, vb = vb2, cb = cb2;
  }
}

// SELL-32 copy of a CSR matrix: slices of 32 consecutive rows, each stored column-major and padded
// to the slice's longest row: entry t of row 32 s + l sits at meta[s].x + 32 t + l (meta[s].y = the
// slice's width); padding entries hold 0 and the row's own index as column. One warp owns a slice
// and a lane owns a row, so every load instruction of the warp reads 32 consecutive values
// (256 bytes) or columns (128 bytes), and the FP64 instructions of a row are its FMAs only (no
// shuffle reductions as in vector CSR).
struct SellView {
  int n, nslices;
  const int2* meta;
  const int* col;
  const double* val;
};

// Warp-uniform loop over the slices, one warp per slice (grid-stride): body(row, active, s, wr) runs
// in every lane with s = (A x)[row]; with HASW, wr = w[row] is loaded before the row's gathers (the
// dot partner of a fused reduction), else 0. Entries are consumed 9 at a time (the 27 of a 3D Q1
// row are three full groups), all 9 value/column loads issued before the first FMA, then one at a
// time for the rest of the slice's width.
template <bool HASW = false, class Body>
__device__ __forceinline__ void for_slices(const SellView& A, const double* __restrict__ x, Body body,
                                           const double* __restrict__ w = nullptr) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int slice = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); slice < A.nslices; slice += warps) {
    const int2 md = __ldg(A.meta + slice);
    const int row = slice * 32 + lane;
    const bool active = row < A.n;
    const double wr = (HASW && active) ? w[row] : 0.0;
    const double* v = A.val + md.x + lane;
    const int* c = A.col + md.x + lane;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    int t = 0;
    for (; t + 9 <= md.y; t += 9) {
      double vv[9];
      int cc[9];
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        vv[j] = ld_stream(v + (t + j) * 32);
        cc[j] = ld_stream(c + (t + j) * 32);
      }
#pragma unroll
      for (int j = 0; j < 9; j += 3) {
        s0 = fma(vv[j], __ldg(x + cc[j]), s0);
        s1 = fma(vv[j + 1], __ldg(x + cc[j + 1]), s1);
        s2 = fma(vv[j + 2], __ldg(x + cc[j + 2]), s2);
      }
    }
    for (; t < md.y; ++t) s0 = fma(ld_stream(v + t * 32), __ldg(x + ld_stream(c + t * 32)), s0);
    body(row, active, (s0 + s1) + s2, wr);
  }
}

// the SELL-32 copy of m (spmv.cu; sell_prepare must have succeeded) and the grid of a SELL kernel
// (blocks of 256 threads, one resident wave of that kernel)
SellView sell_view(gdt_matrix m);
int sell_blocks(long long nslices, int num_sms, const void* kernel);

// SpMV schedules: PL == 0 -> vector-CSR with G lanes per row; PL > 0 -> pipelined warp staging with
// PL entries per lane; PL < 0 -> asynchronous double-buffered staging for rows of at most -PL
// entries. Chosen per matrix by the autotuner.
template <int G, int PL, class T, class Body>
__device__ __forceinline__ void for_rows_csr(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                             const T* __restrict__ val, const T* __restrict__ x, Body body) {
  if constexpr (PL > 0) for_rows_pipelined<T, PL>(n, rp, col, val, x, body);
  else if constexpr (PL < 0) for_rows_async<T, -PL>(n, rp, col, val, x, body);
  else for_rows<G, T>(n, rp, col, val, x, body);
}

// the same with w[row] prefetched and passed to body(row, active, s, w[row])
template <int G, int PL, class T, class Body>
__device__ __forceinline__ void for_rows_csr_w(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                               const T* __restrict__ val, const T* __restrict__ x,
                                               const T* __restrict__ w, Body body) {
  if constexpr (PL > 0) for_rows_pipelined<T, PL, true>(n, rp, col, val, x, body, w);
  else if constexpr (PL < 0) for_rows_async<T, -PL, true>(n, rp, col, val, x, body, w);
  else for_rows<G, T, true>(n, rp, col, val, x, body, w);
}

// the schedule table: index -> (G, PL)
constexpr int kSchedules = 8;
__host__ __device__ constexpr int sched_G(int s) { return s == 0 ? 4 : s == 1 ? 8 : s == 2 ? 16 : s == 3 ? 32 : 0; }
__host__ __device__ constexpr int sched_PL(int s) {
  return s == 4 ? 8 : s == 5 ? 16 : s == 6 ? 32 : s == 7 ? -28 : 0;
}

// expands F<G, PL> for a runtime schedule index
#define GDT_SCHEDULE_SWITCH(sched, F)  \
  switch (sched) {                     \
    case 0: F(4, 0); break;            \
    case 1: F(8, 0); break;            \
    case 2: F(16, 0); break;           \
    case 3: F(32, 0); break;           \
    case 4: F(0, 8); break;            \
    case 5: F(0, 16); break;           \
    case 6: F(0, 32); break;           \
    default: F(0, -28); break;         \
  }

struct LaunchShape {
  int blocks, threads;
  size_t smem;
};

template <class T>
inline LaunchShape schedule_shape(int sched, long long n, int num_sms) {
  LaunchShape s;
  const int PL = sched_PL(sched);
  if (PL != 0) {
    const size_t per_warp = PL > 0 ? size_t(32) * PL * (sizeof(T) + sizeof(int))
                                   : AsyncWindow<T, -sched_PL(7)>::bytes_per_warp;
    // the default limit is 48 KB of shared memory per block, static included: the solver kernels
    // that fuse a grid reduction into the SpMV hold up to 1 KB of static reduction buffers
    int warps = int((47 * 1024) / per_warp);
    warps = warps > 4 ? 4 : (warps < 1 ? 1 : warps);
    s.threads = 32 * warps;
    s.smem = size_t(warps) * per_warp;
    const long long b = (n + s.threads - 1) / s.threads;
    // the asynchronous schedule streams its rows per warp, so no more blocks than fit at once
    const int resident = PL > 0 ? 16 : int((220 * 1024) / (s.smem + 1024));
    const long long cap = (long long)num_sms * (resident > 16 ? 16 : (resident < 1 ? 1 : resident));
    s.blocks = int(b < cap ? b : cap);
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
  if (PL < 0) return max_row > 0 && max_row <= -PL;
  return PL == 0 || (max_row > 0 && max_row <= PL);
}

// Solver flags (converged, replacement due, iteration numbers) are written by the last block of an
// earlier kernel and read at the entry of later ones. A weak load cached in L1 sees them, because kernel
// boundaries order memory; a volatile load would send one L2 request per warp to the same address and
// serialise on that L2 slice (tens of thousands of requests per launch of a large grid).
__device__ __forceinline__ int entry_flag(const int* p) { return __ldca(p); }

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

// Conditional section of a captured iteration. Kernels launched between begin() and end() become the
// body of a graph IF node: they run only when a kernel earlier in the same iteration (given the
// handle from next_handle()) set the condition with cudaGraphSetConditional; otherwise the graph
// skips them without a launch. Outside capture (timing mode, or when capture is unavailable) handles
// are 0 and begin() returns the main stream: the kernels are launched every iteration and must
// check the same device-side flag themselves.
struct CondSection {
  cudaStream_t main = nullptr, side = nullptr;
  bool capturing = false;
  cudaError_t err = cudaSuccess;
  cudaGraphConditionalHandle next_handle() {
    if (!capturing) return 0;
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    cudaGraphConditionalHandle h = 0;
    if (err == cudaSuccess) err = cudaStreamGetCaptureInfo(main, &st, nullptr, &g, nullptr, nullptr, nullptr);
    if (err == cudaSuccess) err = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    return h;
  }
  cudaStream_t begin(cudaGraphConditionalHandle h) {
    if (!capturing) return main;
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if (err == cudaSuccess) err = cudaStreamGetCaptureInfo(main, &st, nullptr, &g, &deps, nullptr, &nd);
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    if (err == cudaSuccess) err = cudaGraphAddNode(&node, g, deps, nullptr, nd, &p);
    if (err == cudaSuccess)
      err = cudaStreamUpdateCaptureDependencies(main, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (err == cudaSuccess)
      err = cudaStreamBeginCaptureToGraph(side, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
    side_active = err == cudaSuccess;
    // after a failure the kernels go into the main capture, which is then discarded
    return side_active ? side : main;
  }
  void end() {
    if (!side_active) return;
    side_active = false;
    cudaGraph_t body = nullptr;
    const cudaError_t e = cudaStreamEndCapture(side, &body);
    if (err == cudaSuccess) err = e;
  }
  bool side_active = false;
};

// iterate_chunks for a body(CondSection&) with a conditional section; *graphed tells whether the
// iterations ran as graphs (conditional kernels then launched only when their condition was set)
template <class Body>
inline gdt_status iterate_chunks_cond(gdt_context ctx, cudaStream_t s, const int* converged, int chunk,
                                      int max_chunks, bool* graphed, Body body) {
  CondSection cs;
  cs.main = s;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  bool use_graph = !ctx->timing && cudaStreamCreateWithFlags(&cs.side, cudaStreamNonBlocking) == cudaSuccess;
  const long long before = ctx->launches;
  if (use_graph && cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    cs.capturing = true;
    for (int k = 0; k < chunk; ++k) body(cs);
    const cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (e != cudaSuccess || cs.err != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
      use_graph = false;
  } else {
    use_graph = false;
  }
  cs.capturing = false;
  const long long per_chunk = ctx->launches - before;
  ctx->launches = before;
  cudaGetLastError();
  if (graphed) *graphed = use_graph;
  int* flag = reinterpret_cast<int*>(ctx->host_pinned);
  gdt_status status = GDT_OK;
  for (int c = 0; c < max_chunks; ++c) {
    cudaError_t e = cudaSuccess;
    if (use_graph) {
      e = cudaGraphLaunch(exec, s);
      ctx->launches += per_chunk;
    } else {
      for (int k = 0; k < chunk; ++k) body(cs);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(flag, converged, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      status = fail(ctx, GDT_ECUDA, std::string("solver iterations: ") + cudaGetErrorString(e));
      break;
    }
    if (ctx->timing) timing_harvest(ctx);
    if (*flag) break;
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cs.side) cudaStreamDestroy(cs.side);
  return status;
}

// ------------------------------------------------------------- persistent (cooperative) kernels ---
// Barrier words of a persistent launch (in the context scratch): the 64-bit arrival count at bar[0],
// the generation the waiting blocks poll at bar[kBarGen] and the fault flag at bar[kBarFault], 4 KB
// apart so the polls and the arrivals do not queue at the same L2 slice. All three start at zero.
constexpr int kBarGen = 1024, kBarFault = 2048;
constexpr unsigned long long kBarrierNs = 1000000000ull;  // default longest wait at a grid barrier (1 s)

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// Grid barrier (all blocks are co-resident: cooperative launch). Barrier number `epoch` (counted by
// thread 0 of every block) is complete when the 64-bit arrival count reaches epoch * blocks; the last
// block to arrive publishes the epoch as the generation the others poll (no reset of the count, so
// the release is one store after the arrival). The waits are bounded by time (wait_ns, checked at the
// first poll and every 256 polls) and by count, after which the fault flag is set and every block
// returns false from then on. Data written before the barrier by any block is read after it with
// plain (coherent) loads, not through the non-coherent read-only path.
// Ordering: the block's writes are gathered by __syncthreads, released by thread 0 with
// fence.acq_rel.gpu before its relaxed arrival (the last arrival acquires the others' releases through
// the arrival count and releases the generation behind a second fence), and acquired by the waiters
// with fence.acq_rel.gpu after they observe the generation; the closing __syncthreads passes that on
// to the block (a sequentially consistent fence is not needed). The poll does not sleep: one thread
// per SM polls one L2 line.
__device__ inline bool grid_barrier(unsigned int* bar, unsigned int& epoch, unsigned long long wait_ns) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ++epoch;
    volatile unsigned int* vgen = bar + kBarGen;
    volatile unsigned int* vfault = bar + kBarFault;
    fence_acq_rel_gpu();
    int good = *vfault == 0u;
    if (good) {
      const unsigned long long target = (unsigned long long)epoch * gridDim.x;
      if (atomicAdd(reinterpret_cast<unsigned long long*>(bar), 1ull) == target - 1) {
        fence_acq_rel_gpu();
        atomicExch(bar + kBarGen, epoch);
      } else {
        const unsigned long long t0 = global_ns();
        unsigned int spins = 0;
        while (*vgen != epoch) {
          ++spins;
          if ((spins & 255u) == 1u) {
            if (*vfault) {
              good = 0;
              break;
            }
            if (spins > (1u << 26) || global_ns() - t0 > wait_ns) {
              atomicExch(bar + kBarFault, 1u);
              good = 0;
              break;
            }
          }
        }
      }
    }
    fence_acq_rel_gpu();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Sum of the per-block partials part[k * gridDim.x + b], the same bits in every block (a fixed order:
// per lane the partials b = lane + 32 u in order of u, then a shuffle tree); result in every thread.
// Warp k sums component k: its lanes issue all their loads before the first add (a loop that adds
// each partial as it arrives waits one L2 latency per partial, several microseconds per iteration of
// a persistent solver), and only these NV warps issue FP64 adds (this part runs one FP64 warp
// instruction per 16 SM cycles). Needs blockDim.x >= 32 NV. bc: NV doubles of shared memory.
template <int NV>
__device__ __forceinline__ void grid_allreduce(const double* part, double (&v)[NV], double* bc) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp < NV) {
    const double* pk = part + (long long)warp * gridDim.x;
    constexpr int U = 8;
    double s = 0.0;
    int b = lane;
    for (; b + 32 * (U - 1) < (int)gridDim.x; b += 32 * U) {
      double t[U];
#pragma unroll
      for (int u = 0; u < U; ++u) t[u] = pk[b + 32 * u];
#pragma unroll
      for (int u = 0; u < U; ++u) s += t[u];
    }
    double t[U];
#pragma unroll
    for (int u = 0; u < U; ++u) t[u] = b + 32 * u < (int)gridDim.x ? pk[b + 32 * u] : 0.0;
#pragma unroll
    for (int u = 0; u < U; ++u) s += t[u];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) bc[warp] = s;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = bc[k];
}

// Block reduction of NV per-thread FP32 sums: FP32 shuffles inside each warp, the warps' sums added in
// FP64 by warp 0 (the FP64 tree of block_reduce costs 16 SM cycles per warp instruction here). The
// warp stage adds 32 FP32 values, a relative error of a few 1e-7, the precision of the FP32 vectors the
// sums come from. Result valid in thread 0. smem: NV * 32 doubles.
template <int NV>
__device__ inline void block_reduce_f32(float (&v)[NV], double (&out)[NV], double* smem) {
#pragma unroll
  for (int k = 0; k < NV; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) smem[k * 32 + warp] = double(v[k]);
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = lane < nw ? smem[k * 32 + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      out[k] = s;
    }
  }
  __syncthreads();
}

}  // namespace gdt
