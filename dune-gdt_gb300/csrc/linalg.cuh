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

}  // namespace gdt
