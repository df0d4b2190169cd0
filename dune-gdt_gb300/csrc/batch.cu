// Batched parametric diffusion: many stationary problems -div(kappa_mu grad u) = f on the unit square,
// each on its own structured P1 triangle mesh (n_i x n_i squares, Kuhn split, sizes uneven),
// kappa_mu = mu_q on quadrant q of the 2 x 2 split, homogeneous Dirichlet; every problem is assembled
// (FP64, the same local forms as the single-problem path) and solved with CG + Jacobi inside ONE
// persistent kernel launch (captured in a CUDA graph and replayed).
//
// GB300 design: a thread-block cluster of 8 CTAs owns one problem at a time and pulls problems from a
// largest-first queue (one atomic per problem). Inside the cluster every CG reduction finishes with a
// hardware cluster barrier and a read of the 8 CTA partials through distributed shared memory, summed
// in rank order by every CTA (deterministic, no extra barrier); an iteration needs three cluster
// barriers and no grid-wide synchronisation or software spin-wait. Matrix rows live in a 7-point
// stencil layout (the CSR row order of the P1 triangle pattern) in per-cluster scratch sized for the
// largest problem. Mixed precision: one FP32 CG sequence (FP32 stencil and vectors) with reliable
// updates: whenever the iterated residual has dropped 10x since the last update, the FP32 correction is
// added to the FP64 solution and the FP32 residual is replaced by the true residual b - A x from the
// FP64 stencil (no restarts, so the Krylov sequence keeps its convergence rate). A problem whose
// true residual stops following (the FP32 operator too inaccurate for its condition number) falls
// back to restarted FP64 iterative refinement.
#include <cooperative_groups.h>

#include <cmath>
#include <numeric>
#include <vector>

#include "structured.cuh"

namespace cg = cooperative_groups;

struct gdt_batch_s {
  long long nprob = 0, total = 0, max_dofs = 0;
  std::vector<long long> cells, offsets;
  int* d_order = nullptr;       // problems, largest first
  long long* d_off = nullptr;   // DoF offsets
  int* d_cells = nullptr;
  int* d_queue = nullptr;
  int nclusters = 0;
  double* scratch64 = nullptr;  // [ncl][stride * 12]
  float* scratch32 = nullptr;   // [ncl][stride * 12]
  int* d_iters = nullptr;
  double* d_relres = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  unsigned long long key = 0;
};

namespace gdt {
namespace {

constexpr int CL = 8;    // CTAs per cluster
constexpr int BT = 256;  // threads per CTA
constexpr int NS = 7;    // stencil width

struct BatchArgs {
  int nprob;
  const int* order;
  const long long* off;
  const int* cells;
  const double* mu;
  double force;
  int mixed;
  double tol2;
  int max_iter;
  double* x;
  double* stencil_out;
  int* iters;
  double* relres;
  int* queue;
  long long stride;
  double* s64;
  float* s32;
  double K[2][3][3];
};

// neighbour offsets of the 7 stencil slots (CSR order): (-1,-1),(0,-1),(-1,0),(0,0),(1,0),(0,1),(1,1)
__device__ __forceinline__ int slot_dx(int k) { return k == 0 ? -1 : k == 1 ? 0 : k == 2 ? -1 : k == 3 ? 0 : k == 4 ? 1 : k == 5 ? 0 : 1; }
__device__ __forceinline__ int slot_dy(int k) { return k < 2 ? -1 : k < 5 ? 0 : 1; }

template <int NV>
__device__ __forceinline__ void cluster_reduce(double (&v)[NV], double* slot, cg::cluster_group& cl) {
  __shared__ double red[NV * 32];
  block_reduce<NV>(v, red);
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) slot[k] = v[k];
  cl.sync();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = 0.0;
    for (int r = 0; r < CL; ++r) s += cl.map_shared_rank(slot, r)[k];
    v[k] = s;
  }
}

// y = A x over rows [lo, hi) of an nv x nv vertex grid; boundary rows are unit rows. Neighbour values
// may have been written by another CTA of the cluster: read them from L2 (ld.global.cg), not L1.
template <class T>
__device__ __forceinline__ T stencil_row(const T* __restrict__ S, const T* __restrict__ x, long long i, int nv,
                                         bool bnd) {
  if (bnd) return S[NS * i + 3] * __ldcg(x + i);
  const long long o[NS] = {-nv - 1, -nv, -1, 0, 1, nv, nv + 1};
  T s = T(0);
#pragma unroll
  for (int k = 0; k < NS; ++k) s = fma(S[NS * i + k], __ldcg(x + i + o[k]), s);
  return s;
}

__device__ __forceinline__ bool vbnd(long long ix, long long iy, int n) { return ix == 0 || iy == 0 || ix == n || iy == n; }

template <class T>
__device__ void cg_solve(const BatchArgs& a, cg::cluster_group& cl, double* slots, int n, long long lo, long long hi,
                         const T* __restrict__ S, const T* __restrict__ dinv, T* __restrict__ d, T* __restrict__ r,
                         T* __restrict__ p, T* __restrict__ q, double tol2, int max_iter, int& iters, int& conv) {
  // d = 0 on entry; r = rhs; p = dinv r
  const int nv = n + 1;
  double v2[2] = {0.0, 0.0};
  for (long long i = lo + threadIdx.x; i < hi; i += BT) {
    const T ri = r[i], zi = dinv[i] * ri;
    p[i] = zi;
    v2[0] += double(ri) * double(zi);
    v2[1] += double(ri) * double(ri);
  }
  cluster_reduce<2>(v2, slots, cl);
  double rho = v2[0];
  const double rr0 = v2[1];
  conv = (rr0 == 0.0) ? 1 : 0;
  iters = 0;
  cl.sync();  // p complete before the first SpMV
  while (!conv && iters < max_iter) {
    // q = A p, p.q
    double v1[1] = {0.0};
    for (long long i = lo + threadIdx.x; i < hi; i += BT) {
      const long long ix = i % nv, iy = i / nv;
      const T qi = stencil_row<T>(S, p, i, nv, vbnd(ix, iy, n));
      q[i] = qi;
      v1[0] += double(p[i]) * double(qi);
    }
    cluster_reduce<1>(v1, slots + 2, cl);
    if (!(v1[0] > 0.0)) {  // breakdown: not SPD or exact solution reached
      conv = (v1[0] == 0.0) ? 1 : 0;
      break;
    }
    const T alpha = T(rho / v1[0]);
    double w2[2] = {0.0, 0.0};
    for (long long i = lo + threadIdx.x; i < hi; i += BT) {
      d[i] = fma(alpha, p[i], d[i]);
      const T ri = fma(-alpha, q[i], r[i]);
      r[i] = ri;
      w2[0] += double(ri) * double(dinv[i] * ri);
      w2[1] += double(ri) * double(ri);
    }
    cluster_reduce<2>(w2, slots + 4, cl);
    const T beta = T(w2[0] / rho);
    rho = w2[0];
    ++iters;
    if (w2[1] <= tol2 * rr0) {
      conv = 1;
      break;
    }
    for (long long i = lo + threadIdx.x; i < hi; i += BT) p[i] = fma(beta, p[i], dinv[i] * r[i]);
    cl.sync();
  }
}

// Mixed-precision CG with reliable updates for one problem: x (FP64) = 0 on entry, b the FP64 load;
// the FP32 sequence iterates d32 (correction), r32, p32, q32. Convergence is decided on the true FP64
// residual only; relres = ||b - A x|| / ||b|| of the returned x.
__device__ void cg_reliable(const BatchArgs& a, cg::cluster_group& cl, double* slots, int n, long long lo, long long hi,
                            const double* __restrict__ S, const double* __restrict__ b, double* __restrict__ x,
                            const float* __restrict__ S32, const float* __restrict__ dinv, float* __restrict__ d,
                            float* __restrict__ r, float* __restrict__ p, float* __restrict__ q, int& iters, int& conv,
                            double& relres) {
  const int nv = n + 1;
  double v2[2] = {0.0, 0.0};
  for (long long i = lo + threadIdx.x; i < hi; i += BT) {
    const float ri = float(b[i]), zi = dinv[i] * ri;
    r[i] = ri;
    p[i] = zi;
    d[i] = 0.0f;
    v2[0] += double(ri) * double(zi);
    v2[1] += b[i] * b[i];
  }
  cluster_reduce<2>(v2, slots, cl);
  double rho = v2[0], rho_prev = rho;
  const double rr0 = v2[1];
  double rr_ref = rr0;       // true residual at the last replacement
  double drop = 0.01;        // replace when the iterated residual has dropped by this factor (squared)
  bool restarting = false;   // the FP32 operator is too far from the FP64 one to continue the sequence
  conv = (rr0 == 0.0) ? 1 : 0;
  relres = 0.0;
  iters = 0;
  cl.sync();  // p complete before the first SpMV
  while (!conv && iters < a.max_iter) {
    double v1[1] = {0.0};
    for (long long i = lo + threadIdx.x; i < hi; i += BT) {
      const long long ix = i % nv, iy = i / nv;
      const float qi = stencil_row<float>(S32, p, i, nv, vbnd(ix, iy, n));
      q[i] = qi;
      v1[0] += double(p[i]) * double(qi);
    }
    cluster_reduce<1>(v1, slots + 2, cl);
    if (!(v1[0] > 0.0)) break;  // breakdown: not SPD in FP32; the true residual below decides
    const float alpha = float(rho / v1[0]);
    double w2[2] = {0.0, 0.0};
    for (long long i = lo + threadIdx.x; i < hi; i += BT) {
      d[i] = fmaf(alpha, p[i], d[i]);
      const float ri = fmaf(-alpha, q[i], r[i]);
      r[i] = ri;
      w2[0] += double(ri) * double(dinv[i] * ri);
      w2[1] += double(ri) * double(ri);
    }
    cluster_reduce<2>(w2, slots + 4, cl);
    ++iters;
    double beta = w2[0] / rho;
    rho_prev = rho;
    rho = w2[0];
    if (w2[1] <= drop * rr_ref || w2[1] <= a.tol2 * rr0 || iters >= a.max_iter) {
      // reliable update: x += d, d = 0; r = b - A x (FP64), r32 = r; beta from the replaced residual
      for (long long i = lo + threadIdx.x; i < hi; i += BT) {
        x[i] += double(d[i]);
        d[i] = 0.0f;
      }
      cl.sync();  // x complete before the FP64 residual reads the neighbours' rows
      double t2[2] = {0.0, 0.0};
      for (long long i = lo + threadIdx.x; i < hi; i += BT) {
        const long long ix = i % nv, iy = i / nv;
        const double ri = b[i] - stencil_row<double>(S, x, i, nv, vbnd(ix, iy, n));
        const float rf = float(ri);
        r[i] = rf;
        t2[0] += double(rf) * double(dinv[i] * rf);
        t2[1] += ri * ri;
      }
      cluster_reduce<2>(t2, slots + 6, cl);
      // Stagnation guard: when a whole cycle gained less than 2x on the true residual, the gap between
      // the FP32 and FP64 operators dominates (cond(A) times the FP32 rounding of A near 1). From then
      // on every replacement restarts the direction (beta = 0) and waits for a 1000x drop: FP64
      // iterative refinement around FP32 CG, which converges while the Krylov continuation stalls.
      if (!restarting && t2[1] > 0.25 * rr_ref) {
        restarting = true;
        drop = 1e-6;
      }
      rr_ref = t2[1];
      relres = rr0 > 0.0 ? sqrt(t2[1] / rr0) : 0.0;
      beta = restarting ? 0.0 : t2[0] / rho_prev;
      rho = t2[0];
      if (t2[1] <= a.tol2 * rr0) {
        conv = 1;
        break;
      }
    }
    const float bf = float(beta);
    for (long long i = lo + threadIdx.x; i < hi; i += BT) p[i] = fmaf(bf, p[i], dinv[i] * r[i]);
    cl.sync();
  }
  if (!conv) {  // stopped by breakdown or the iteration limit: fold in the correction, report the true residual
    cl.sync();
    for (long long i = lo + threadIdx.x; i < hi; i += BT) {
      x[i] += double(d[i]);
      d[i] = 0.0f;
    }
    cl.sync();
    double t1[1] = {0.0};
    for (long long i = lo + threadIdx.x; i < hi; i += BT) {
      const long long ix = i % nv, iy = i / nv;
      const double ri = b[i] - stencil_row<double>(S, x, i, nv, vbnd(ix, iy, n));
      t1[0] += ri * ri;
    }
    cluster_reduce<1>(t1, slots + 6, cl);
    relres = rr0 > 0.0 ? sqrt(t1[0] / rr0) : 0.0;
    if (t1[0] <= a.tol2 * rr0) conv = 1;
  }
}

// at most 64 registers: four CTAs per SM, so twice as many clusters (problems in flight) as at the
// 128 registers the compiler would otherwise use; the iterations are latency-bound at low occupancy
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(BT, 4) batch_kernel(BatchArgs a) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = int(cl.block_rank());
  const long long cid = blockIdx.x / CL;
  __shared__ int s_prob;
  __shared__ double slots[8];
  double* s64 = a.s64 + cid * a.stride * 12;
  float* s32 = a.s32 + cid * a.stride * 12;
  for (;;) {
    if (rank == 0 && threadIdx.x == 0) s_prob = atomicAdd(a.queue, 1);
    cl.sync();
    const int pi = *cl.map_shared_rank(&s_prob, 0);
    cl.sync();
    if (pi >= a.nprob) break;
    const int prob = a.order[pi];
    const int n = a.cells[prob];
    const int nv = n + 1;
    const long long N = (long long)nv * nv;
    const long long off = a.off[prob];
    const long long chunk = (N + CL - 1) / CL;
    const long long lo = rank * chunk, hi = lo + chunk < N ? lo + chunk : N;
    // FP64 scratch: S (7 N), b, r, p, q, dinv ; FP32 scratch: S32 (7 N), r, p, q, d, dinv
    double *S = s64, *b = s64 + NS * a.stride, *r = b + a.stride, *p = r + a.stride, *q = p + a.stride,
           *dinv = q + a.stride;
    float *S32 = s32, *r32 = s32 + NS * a.stride, *p32 = r32 + a.stride, *q32 = p32 + a.stride, *d32 = q32 + a.stride,
          *dinv32 = d32 + a.stride;
    double* x = a.x + off;
    const double h = 1.0 / n;
    const double* mu = a.mu + 4LL * prob;
    // ---- assembly (output-stationary, as the single-problem P1 kernel): row, load, Dirichlet
    for (long long i = lo + threadIdx.x; i < hi; i += BT) {
      const long long ix = i % nv, iy = i / nv;
      double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      int ntri = 0;
#pragma unroll
      for (int cv = 0; cv < 4; ++cv) {
        const long long cx = ix - (cv & 1), cy = iy - ((cv >> 1) & 1);
        if (cx < 0 || cy < 0 || cx >= n || cy >= n) continue;
        const double kap = mu[(cx >= n / 2 ? 1 : 0) + (cy >= n / 2 ? 2 : 0)];
#pragma unroll
        for (int t = 0; t < 2; ++t)
#pragma unroll
          for (int li = 0; li < 3; ++li) {
            if (local_corner(2, true, t, li) != cv) continue;
            ++ntri;
#pragma unroll
            for (int lj = 0; lj < 3; ++lj) acc[slot_between(2, cv, local_corner(2, true, t, lj))] += kap * a.K[t][li][lj];
          }
      }
      const bool bnd = vbnd(ix, iy, n);
      const int k9[NS] = {0, 1, 3, 4, 5, 7, 8};
      double* Si = S + NS * i;
#pragma unroll
      for (int k = 0; k < NS; ++k) {
        double v = acc[k9[k]];
        if (bnd) v = (k == 3) ? 1.0 : 0.0;
        else if (vbnd(ix + slot_dx(k), iy + slot_dy(k), n)) v = 0.0;
        Si[k] = v;
        if (a.mixed) S32[NS * i + k] = float(v);
        if (a.stencil_out) a.stencil_out[NS * (off + i) + k] = v;
      }
      const double bi = bnd ? 0.0 : a.force * (0.5 * h * h / 3.0) * ntri;
      b[i] = bi;
      const double di = 1.0 / Si[3];
      dinv[i] = di;
      x[i] = 0.0;
      if (a.mixed) dinv32[i] = float(di);
      else r[i] = bi;
    }
    cl.sync();
    int iters = 0, conv = 0;
    double relres = 0.0;
    if (!a.mixed) {
      cg_solve<double>(a, cl, slots, n, lo, hi, S, dinv, x, r, p, q, a.tol2, a.max_iter, iters, conv);
      // true relative residual of the returned iterate
      double v2[2] = {0.0, 0.0};
      cl.sync();
      for (long long i = lo + threadIdx.x; i < hi; i += BT) {
        const long long ix = i % nv, iy = i / nv;
        const double ri = b[i] - stencil_row<double>(S, x, i, nv, vbnd(ix, iy, n));
        v2[0] += ri * ri;
        v2[1] += b[i] * b[i];
      }
      cluster_reduce<2>(v2, slots, cl);
      relres = v2[1] > 0 ? sqrt(v2[0] / v2[1]) : 0.0;
    } else {
      cg_reliable(a, cl, slots, n, lo, hi, S, b, x, S32, dinv32, d32, r32, p32, q32, iters, conv, relres);
    }
    if (rank == 0 && threadIdx.x == 0) {
      a.iters[prob] = conv ? iters : -iters - 1;
      a.relres[prob] = relres;
    }
    cl.sync();
  }
}

}  // namespace
}  // namespace gdt

using namespace gdt;

extern "C" {

gdt_status gdt_batch_create(gdt_context ctx, int64_t nproblems, const int64_t* cells, gdt_batch* out) {
  if (!ctx || !cells || !out || nproblems < 1) return GDT_EINVAL;
  *out = nullptr;
  gdt_batch b = new (std::nothrow) gdt_batch_s;
  if (!b) return GDT_ENOMEM;
  b->nprob = nproblems;
  b->cells.assign(cells, cells + nproblems);
  b->offsets.assign(nproblems + 1, 0);
  for (long long i = 0; i < nproblems; ++i) {
    if (cells[i] < 2 || cells[i] % 2 != 0 || cells[i] > 16384) {
      delete b;
      return fail(ctx, GDT_EINVAL, "cells per side must be even and in [2, 16384]");
    }
    const long long nd = (cells[i] + 1) * (cells[i] + 1);
    b->offsets[i + 1] = b->offsets[i] + nd;
    b->max_dofs = std::max(b->max_dofs, nd);
  }
  b->total = b->offsets[nproblems];
  std::vector<int> order(nproblems);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cells[x] > cells[y]; });
  std::vector<int> c32(b->cells.begin(), b->cells.end());
  int max_clusters = 0;
  {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CL * 64);
    cfg.blockDim = dim3(BT);
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = CL;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    if (cudaOccupancyMaxActiveClusters(&max_clusters, batch_kernel, &cfg) != cudaSuccess || max_clusters < 1)
      max_clusters = std::max(1, ctx->num_sms / CL);
    cudaGetLastError();
  }
  b->nclusters = int(std::min<long long>(max_clusters, nproblems));
  const long long stride = b->max_dofs;
  cudaError_t e = cudaMalloc(&b->d_order, sizeof(int) * nproblems);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_off, sizeof(long long) * (nproblems + 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_cells, sizeof(int) * nproblems);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_queue, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_iters, sizeof(int) * nproblems);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_relres, sizeof(double) * nproblems);
  if (e == cudaSuccess) e = cudaMalloc(&b->scratch64, sizeof(double) * stride * 12 * b->nclusters);
  if (e == cudaSuccess) e = cudaMalloc(&b->scratch32, sizeof(float) * stride * 12 * b->nclusters);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_order, order.data(), sizeof(int) * nproblems, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_off, b->offsets.data(), sizeof(long long) * (nproblems + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_cells, c32.data(), sizeof(int) * nproblems, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    gdt_batch_destroy(b);
    return fail(ctx, e == cudaErrorMemoryAllocation ? GDT_ENOMEM : GDT_ECUDA, cudaGetErrorString(e));
  }
  *out = b;
  return GDT_OK;
}

gdt_status gdt_batch_destroy(gdt_batch b) {
  if (!b) return GDT_EINVAL;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  cudaFree(b->d_order);
  cudaFree(b->d_off);
  cudaFree(b->d_cells);
  cudaFree(b->d_queue);
  cudaFree(b->d_iters);
  cudaFree(b->d_relres);
  cudaFree(b->scratch64);
  cudaFree(b->scratch32);
  delete b;
  return GDT_OK;
}

int64_t gdt_batch_total_dofs(gdt_batch b) { return b ? b->total : -1; }

gdt_status gdt_batch_dof_offsets(gdt_batch b, int64_t* offsets) {
  if (!b || !offsets) return GDT_EINVAL;
  for (long long i = 0; i <= b->nprob; ++i) offsets[i] = b->offsets[i];
  return GDT_OK;
}

gdt_status gdt_batch_solve(gdt_context ctx, gdt_batch b, const double* mu, double force, int precision, double tol,
                           int max_iter, double* x, double* stencil_out, gdt_batch_info* info) {
  if (!ctx || !b || !mu || !x || !(tol > 0) || max_iter < 1) return GDT_EINVAL;
  if (precision != GDT_PRECISION_FP64 && precision != GDT_PRECISION_MIXED) return GDT_EINVAL;
  BatchArgs a;
  a.nprob = int(b->nprob);
  a.order = b->d_order;
  a.off = b->d_off;
  a.cells = b->d_cells;
  a.mu = mu;
  a.force = force;
  a.mixed = precision == GDT_PRECISION_MIXED;
  a.tol2 = tol * tol;
  a.max_iter = max_iter;
  a.x = x;
  a.stencil_out = stencil_out;
  a.iters = b->d_iters;
  a.relres = b->d_relres;
  a.queue = b->d_queue;
  a.stride = b->max_dofs;
  a.s64 = b->scratch64;
  a.s32 = b->scratch32;
  // P1 stiffness of the two triangle types of a square cell (scale invariant in 2D)
  GridDesc g1;
  g1.dim = 2;
  g1.simplex = 1;
  g1.nsub = 2;
  g1.h[0] = g1.h[1] = 1.0;
  for (int t = 0; t < 2; ++t) {
    double X[3][2];
    for (int j = 0; j < 3; ++j) {
      const int c = local_corner(2, true, t, j);
      X[j][0] = c & 1;
      X[j][1] = (c >> 1) & 1;
    }
    const double ax = X[1][0] - X[0][0], bx = X[2][0] - X[0][0], ay = X[1][1] - X[0][1], by = X[2][1] - X[0][1];
    const double det = ax * by - bx * ay;
    double G[3][2];
    G[1][0] = by / det;
    G[1][1] = -bx / det;
    G[2][0] = -ay / det;
    G[2][1] = ax / det;
    G[0][0] = -G[1][0] - G[2][0];
    G[0][1] = -G[1][1] - G[2][1];
    const double area = 0.5 * std::fabs(det);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) a.K[t][i][j] = area * (G[i][0] * G[j][0] + G[i][1] * G[j][1]);
  }
  cudaStream_t s = ctx->stream;
  cudaStream_t own = nullptr;
  if (!s) {
    GDT_TRY_CUDA(ctx, cudaStreamCreate(&own));
    s = own;
  }
  // one graph per argument set: queue reset + the persistent kernel
  unsigned long long key = reinterpret_cast<unsigned long long>(mu) ^ (reinterpret_cast<unsigned long long>(x) << 1) ^
                           (reinterpret_cast<unsigned long long>(stencil_out) << 2) ^ (unsigned long long)(a.mixed << 3) ^
                           std::hash<double>()(force) ^ (std::hash<double>()(tol) << 4) ^ ((unsigned long long)max_iter << 20);
  gdt_status st = GDT_OK;
  if (!b->exec || b->key != key) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      cudaMemsetAsync(b->d_queue, 0, sizeof(int), s);
      batch_kernel<<<b->nclusters * CL, BT, 0, s>>>(a);
      if (cudaStreamEndCapture(s, &b->graph) != cudaSuccess || cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess)
        b->exec = nullptr;
    }
    cudaGetLastError();
    b->key = key;
  }
  if (b->exec) {
    if (cudaGraphLaunch(b->exec, s) != cudaSuccess) st = fail(ctx, GDT_ECUDA, "batch graph launch");
  } else {
    cudaMemsetAsync(b->d_queue, 0, sizeof(int), s);
    batch_kernel<<<b->nclusters * CL, BT, 0, s>>>(a);
  }
  ctx->launches++;
  if (st == GDT_OK) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = fail(ctx, GDT_ECUDA, std::string("batch_kernel: ") + cudaGetErrorString(e));
  }
  if (st == GDT_OK && info) {
    std::vector<int> it(b->nprob);
    std::vector<double> rr(b->nprob);
    cudaMemcpyAsync(it.data(), b->d_iters, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(rr.data(), b->d_relres, sizeof(double) * b->nprob, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) st = fail(ctx, GDT_ECUDA, "batch synchronize");
    info->problems = b->nprob;
    info->total_dofs = b->total;
    info->max_iterations = 0;
    info->min_iterations = 1 << 30;
    info->all_converged = 1;
    info->max_rel_residual = 0.0;
    for (long long i = 0; i < b->nprob; ++i) {
      const int v = it[i] >= 0 ? it[i] : -it[i] - 1;
      if (it[i] < 0) info->all_converged = 0;
      info->max_iterations = std::max(info->max_iterations, v);
      info->min_iterations = std::min(info->min_iterations, v);
      info->max_rel_residual = std::max(info->max_rel_residual, rr[i]);
    }
    if (st == GDT_OK && !info->all_converged) st = fail(ctx, GDT_ENOCONV, "a batched problem did not converge");
  }
  if (own) {
    cudaStreamSynchronize(own);
    cudaStreamDestroy(own);
    // the cached graph stays valid: it is launched on whatever stream the next call uses
  }
  return st;
}

gdt_status gdt_batch_iterations(gdt_context ctx, gdt_batch b, int* iterations, double* rel_residuals) {
  if (!ctx || !b) return GDT_EINVAL;
  if (iterations) GDT_TRY_CUDA(ctx, cudaMemcpy(iterations, b->d_iters, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost));
  if (rel_residuals)
    GDT_TRY_CUDA(ctx, cudaMemcpy(rel_residuals, b->d_relres, sizeof(double) * b->nprob, cudaMemcpyDeviceToHost));
  return GDT_OK;
}

}  // extern "C"
