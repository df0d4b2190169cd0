// Batched parametric diffusion: many stationary problems -div(kappa grad u) = f on the unit square,
// each on its own structured mesh of n_i x n_i squares (sizes uneven): continuous P1 on the Kuhn split
// (two triangles per square) or continuous Q1 on the squares; kappa per quadrant of the 2 x 2 split
// (kappa_mu = mu_q, the affine parameter sweep of python/dune/gdt/gamm-2019-talk-on-conservative-rb.cc:74-95)
// or per element; homogeneous Dirichlet. Every problem is assembled (FP64, the same local forms as the
// single-problem path) and solved with CG + Jacobi inside ONE persistent launch (captured in a CUDA
// graph and replayed).
//
// GB300 design. The grid is a set of 8-CTA thread-block clusters that pull work items from a queue,
// largest problems first (one atomic per item). An item is solved by teams of one of three sizes:
//   cluster: the 8 CTAs of the cluster share one problem (rows split into 8 chunks); reductions end
//            with a hardware cluster barrier and a read of the 8 CTA partials through distributed
//            shared memory, summed in rank order by every CTA (deterministic);
//   CTA:     each CTA of the cluster solves a problem of its own (up to 8 per item), reductions with
//            block barriers;
//   warp:    each warp solves a problem of its own (up to 64 per item), reductions with shuffles and
//            no barrier at all.
// No team waits on another one (no software spin-wait anywhere). Which team size a problem gets is
// decided per size class by the autotuner (gdt_batch_tune: every allowed team size timed on the
// problems of that size, the fastest kept) or set by the caller; a new batch uses cluster teams.
// Matrix rows live in a stencil layout (the CSR row order of the pattern: 7 entries for P1, 9 for Q1)
// in per-team scratch. Mixed precision: one FP32 CG sequence (FP32 stencil and vectors) with reliable
// updates: whenever the iterated residual has dropped 10x since the last update, the FP32 correction
// is added to the FP64 solution and the FP32 residual is replaced by the true residual b - A x from the
// FP64 stencil (no restarts, so the Krylov sequence keeps its convergence rate). A problem whose true
// residual stops following falls back to restarted FP64 iterative refinement.
//
// Failure handling (per problem, the others are unaffected): non-finite data (kappa or the load) is
// detected after assembly by a team reduction, the problem is skipped with x = 0 and reported as
// GDT_ENAN; a problem that reaches max_iter is reported as GDT_ENOCONV. The iteration count is the
// only budget: the kernel has no wait that could run out.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <functional>
#include <map>
#include <numeric>
#include <vector>

#include "structured.cuh"

namespace cg = cooperative_groups;

namespace gdt {
// one queue entry: `count` problems probs[first ..) solved by teams of kind `team`, each with
// `stride` (>= its DoF count, a multiple of 32) words per scratch array
struct BatchItem {
  int team;
  int first;
  int count;
  int pad;
  long long stride;
};
}  // namespace gdt

struct gdt_batch_s {
  long long nprob = 0, total = 0, total_elems = 0, max_dofs = 0;
  int element = GDT_BATCH_P1_SIMPLEX;
  std::vector<long long> cells, offsets, eoffsets;
  std::vector<int> teams;                // per problem: GDT_BATCH_TEAM_*
  std::vector<gdt::BatchItem> items;     // the queue of the current team assignment
  std::vector<int> probs;
  long long* d_off = nullptr;
  long long* d_eoff = nullptr;
  int* d_cells = nullptr;
  gdt::BatchItem* d_items = nullptr;     // room for nprob items
  int* d_probs = nullptr;
  int* d_queue = nullptr;
  int* d_iters = nullptr;
  double* d_relres = nullptr;
  int* d_status = nullptr;
  int nclusters = 0;                     // clusters resident at once (the larger of the two kernels')
  int nclusters_prec[2] = {0, 0};        // per precision: FP64, mixed
  double* scratch64 = nullptr;           // [nclusters][scratch_words]
  float* scratch32 = nullptr;
  long long scratch_words = 0;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  unsigned long long key = 0;
  unsigned long long generation = 1;     // bumped when the queue changes
};

namespace gdt {
namespace {

constexpr int CL = 8;    // CTAs per cluster
constexpr int BT = 256;  // threads per CTA
constexpr int WPC = BT / 32;
constexpr long long kWarpMaxDofs = 20000;  // the tuner does not try warp teams on larger problems

struct BatchArgs {
  int nitems;
  const BatchItem* items;
  const int* probs;
  const long long* off;
  const long long* eoff;
  const int* cells;
  const double* kappa;
  int kappa_elems;  // 0: kappa[4 i + q] per quadrant; 1: per element from eoff[i]
  double force;
  int mixed;
  double tol2;
  int max_iter;
  double* x;
  double* stencil_out;
  int* iters;
  double* relres;
  int* status;
  int* queue;
  long long cwords;  // scratch words per cluster
  double* s64;
  float* s32;
  double K[2][4][4];  // local stiffness: P1 triangle types t (3 x 3), or Q1 (K[0], 4 x 4)
};

// ----------------------------------------------------------------------------------- teams ---
struct ClusterTeam {
  cg::cluster_group& cl;
  int rank;
  double* slots;  // shared, 10 doubles
  __device__ int tid() const { return threadIdx.x; }
  __device__ int stride() const { return BT; }
  __device__ void range(int N, int& lo, int& hi) const {
    const int chunk = (N + CL - 1) / CL;
    lo = min(rank * chunk, N);
    hi = min(lo + chunk, N);
  }
  __device__ void sync() { cl.sync(); }
  __device__ bool leader() const { return rank == 0 && threadIdx.x == 0; }
  // neighbour rows may have been written by another CTA (another SM): read through L2
  template <class T>
  __device__ T ld(const T* p) const {
    return __ldcg(p);
  }
  template <int NV>
  __device__ void reduce(double (&v)[NV], int slot) {
    __shared__ double red[NV * 32];
    block_reduce<NV>(v, red);
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) slots[slot + k] = v[k];
    cl.sync();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int r = 0; r < CL; ++r) s += cl.map_shared_rank(slots + slot, r)[k];
      v[k] = s;
    }
  }
};

struct CtaTeam {
  double* bc;  // shared, 10 doubles
  __device__ int tid() const { return threadIdx.x; }
  __device__ int stride() const { return BT; }
  __device__ void range(int N, int& lo, int& hi) const {
    lo = 0;
    hi = N;
  }
  __device__ void sync() { __syncthreads(); }
  __device__ bool leader() const { return threadIdx.x == 0; }
  template <class T>
  __device__ T ld(const T* p) const {
    return __ldca(p);
  }
  template <int NV>
  __device__ void reduce(double (&v)[NV], int slot) {
    __shared__ double red[NV * 32];
    block_reduce<NV>(v, red);
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) bc[slot + k] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = bc[slot + k];
  }
};

struct WarpTeam {
  __device__ int tid() const { return threadIdx.x & 31; }
  __device__ int stride() const { return 32; }
  __device__ void range(int N, int& lo, int& hi) const {
    lo = 0;
    hi = N;
  }
  __device__ void sync() { __syncwarp(); }
  __device__ bool leader() const { return (threadIdx.x & 31) == 0; }
  template <class T>
  __device__ T ld(const T* p) const {
    return __ldca(p);
  }
  // butterfly: every lane adds the same pairs (commutative), so every lane holds the same bits
  template <int NV>
  __device__ void reduce(double (&v)[NV], int) {
#pragma unroll
    for (int k = 0; k < NV; ++k)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  }
};

// ----------------------------------------------------------------------------- stencil rows ---
// stencil entry k of a row -> slot of the 3 x 3 vertex neighbourhood (offset (s % 3 - 1, s / 3 - 1)):
// P1 keeps the 7 slots of the Kuhn pattern, Q1 all 9, both in ascending column order
template <int NS>
__device__ __forceinline__ int slot9(int k) {
  if constexpr (NS == 9) return k;
  return k < 2 ? k : (k < 5 ? k + 1 : k + 2);  // 0 1 3 4 5 7 8
}
template <int NS>
__host__ __device__ constexpr int center_entry() {
  return NS == 9 ? 4 : 3;
}

__device__ __forceinline__ bool vbnd(int ix, int iy, int n) { return ix == 0 || iy == 0 || ix == n || iy == n; }

// S: rows written earlier in this launch by the same thread (scratch is reused from problem to problem,
// so no read-only / non-coherent load path for it). Row indices of one problem fit 32 bits (at most
// 16385^2 rows): 32-bit offsets and divisions keep the nine neighbour offsets in nine registers.
template <int NS, class T, class Team>
__device__ __forceinline__ T stencil_row(const Team& t, const T* S, const T* x, int i, int nv, bool bnd) {
  const T* Si = S + (long long)NS * i;
  if (bnd) return Si[center_entry<NS>()] * t.ld(x + i);
  T s = T(0);
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    const int sl = slot9<NS>(k);
    const int o = (sl % 3 - 1) + (sl / 3 - 1) * nv;
    s = fma(Si[k], t.ld(x + (i + o)), s);
  }
  return s;
}

// per-problem scratch: FP64 S (NS stride), b, r, p, q, dinv; FP32 S32 (NS stride), r, p, q, d, dinv.
// The arrays are computed from the two bases on use (one multiply-add): twelve pointers held for the
// whole solve would cost 24 registers of the 64 this kernel runs with.
template <int NS>
struct Scratch {
  double* s64;
  float* s32;
  long long st;
  __device__ double* S() const { return s64; }
  __device__ double* b() const { return s64 + (NS + 0) * st; }
  __device__ double* r() const { return s64 + (NS + 1) * st; }
  __device__ double* p() const { return s64 + (NS + 2) * st; }
  __device__ double* q() const { return s64 + (NS + 3) * st; }
  __device__ double* dinv() const { return s64 + (NS + 4) * st; }
  __device__ float* S32() const { return s32; }
  __device__ float* r32() const { return s32 + (NS + 0) * st; }
  __device__ float* p32() const { return s32 + (NS + 1) * st; }
  __device__ float* q32() const { return s32 + (NS + 2) * st; }
  __device__ float* d32() const { return s32 + (NS + 3) * st; }
  __device__ float* dinv32() const { return s32 + (NS + 4) * st; }
};

// ---------------------------------------------------------------------------------- assembly ---
// Output-stationary, as the single-problem kernels: every row gathers the local matrices of the
// elements around its vertex, then Dirichlet rows become unit rows and columns of Dirichlet vertices
// are dropped (their values are zero). Returns the count of non-finite kappa values and loads seen.
template <int NS, class Team>
__device__ double assemble_rows(const BatchArgs& a, const Team& t, int prob, int n, int lo, int hi,
                                const Scratch<NS>& w, double* x) {
  const int nv = n + 1;
  const double h = 1.0 / n;
  const long long off = a.off[prob];
  const double* kq = a.kappa + 4LL * prob;
  const double* ke = a.kappa + (a.kappa_elems ? a.eoff[prob] : 0);
  double bad = 0.0;
  for (int i = lo + t.tid(); i < hi; i += t.stride()) {
    const int ix = i % nv, iy = i / nv;
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    int nel = 0;
#pragma unroll
    for (int cv = 0; cv < 4; ++cv) {
      const int cx = ix - (cv & 1), cy = iy - ((cv >> 1) & 1);
      if (cx < 0 || cy < 0 || cx >= n || cy >= n) continue;
      const long long cell = cx + (long long)n * cy;
      if constexpr (NS == 7) {
#pragma unroll
        for (int tt = 0; tt < 2; ++tt)
#pragma unroll
          for (int li = 0; li < 3; ++li) {
            if (local_corner(2, true, tt, li) != cv) continue;
            const double kap = a.kappa_elems ? ke[2 * cell + tt] : kq[(cx >= n / 2 ? 1 : 0) + (cy >= n / 2 ? 2 : 0)];
            if (!isfinite(kap)) bad += 1.0;
            ++nel;
#pragma unroll
            for (int lj = 0; lj < 3; ++lj) acc[slot_between(2, cv, local_corner(2, true, tt, lj))] += kap * a.K[tt][li][lj];
          }
      } else {
        const double kap = a.kappa_elems ? ke[cell] : kq[(cx >= n / 2 ? 1 : 0) + (cy >= n / 2 ? 2 : 0)];
        if (!isfinite(kap)) bad += 1.0;
        ++nel;
#pragma unroll
        for (int lj = 0; lj < 4; ++lj) acc[slot_between(2, cv, lj)] += kap * a.K[0][cv][lj];
      }
    }
    const bool bnd = vbnd(ix, iy, n);
    double* Si = w.S() + (long long)NS * i;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int sl = slot9<NS>(k);
      double v = acc[sl];
      if (bnd) v = (k == center_entry<NS>()) ? 1.0 : 0.0;
      else if (vbnd(ix + sl % 3 - 1, iy + sl / 3 - 1, n)) v = 0.0;
      Si[k] = v;
      if (a.mixed) w.S32()[(long long)NS * i + k] = float(v);
      if (a.stencil_out) a.stencil_out[NS * (off + i) + k] = v;
    }
    // load: f times the integral of the hat function, per element: area / 3 (triangle, area h^2 / 2)
    // or h^2 / 4 (bilinear on a square)
    const double per_el = NS == 7 ? 0.5 * h * h / 3.0 : 0.25 * h * h;
    const double bi = bnd ? 0.0 : a.force * per_el * nel;
    if (!isfinite(bi)) bad += 1.0;
    w.b()[i] = bi;
    const double di = 1.0 / Si[center_entry<NS>()];
    w.dinv()[i] = di;
    x[i] = 0.0;
    if (a.mixed) w.dinv32()[i] = float(di);
    else w.r()[i] = bi;
  }
  return bad;
}

// ------------------------------------------------------------------------------ FP64 CG solve ---
template <int NS, class Team>
__device__ bool cg_fp64(const BatchArgs& a, Team& t, int n, int lo, int hi, const Scratch<NS>& w, double* x,
                        double bad, int& iters, int& conv) {
  // x = 0 and r = b on entry; p = dinv r. The first reduction also sums the assembly's count of
  // non-finite values (false: the problem is skipped) and, with its barrier, orders the assembly
  // before the first SpMV reads neighbour rows.
  const int nv = n + 1;
  double v3[3] = {0.0, 0.0, bad};
  for (int i = lo + t.tid(); i < hi; i += t.stride()) {
    const double ri = w.r()[i], zi = w.dinv()[i] * ri;
    w.p()[i] = zi;
    v3[0] += ri * zi;
    v3[1] += ri * ri;
  }
  t.reduce(v3, 0);
  iters = 0;
  conv = 0;
  if (v3[2] > 0.0) return false;
  double rho = v3[0];
  const double rr0 = v3[1];
  conv = (rr0 == 0.0) ? 1 : 0;
  t.sync();  // p complete before the first SpMV
  while (!conv && iters < a.max_iter) {
    double v1[1] = {0.0};
    for (int i = lo + t.tid(); i < hi; i += t.stride()) {
      const int ix = i % nv, iy = i / nv;
      const double qi = stencil_row<NS, double>(t, w.S(), w.p(), i, nv, vbnd(ix, iy, n));
      w.q()[i] = qi;
      v1[0] += w.p()[i] * qi;
    }
    t.reduce(v1, 3);
    if (!(v1[0] > 0.0)) {  // breakdown: not SPD, or the exact solution reached
      conv = (v1[0] == 0.0) ? 1 : 0;
      break;
    }
    const double alpha = rho / v1[0];
    double w2[2] = {0.0, 0.0};
    for (int i = lo + t.tid(); i < hi; i += t.stride()) {
      x[i] = fma(alpha, w.p()[i], x[i]);
      const double ri = fma(-alpha, w.q()[i], w.r()[i]);
      w.r()[i] = ri;
      w2[0] += ri * (w.dinv()[i] * ri);
      w2[1] += ri * ri;
    }
    t.reduce(w2, 4);
    const double beta = w2[0] / rho;
    rho = w2[0];
    ++iters;
    if (w2[1] <= a.tol2 * rr0) {
      conv = 1;
      break;
    }
    for (int i = lo + t.tid(); i < hi; i += t.stride()) w.p()[i] = fma(beta, w.p()[i], w.dinv()[i] * w.r()[i]);
    t.sync();
  }
  return true;
}

// Sum of FP32 products: FP32 over chunks of 16 rows, each chunk added to an FP64 total. This part
// issues one FP64 warp instruction per 16 SM cycles, and an FP64 conversion and add per row for three
// dot products would cost the mixed iteration more than its FP32 arithmetic. The chunk sum of 16
// FP32 products has a relative error of a few 1e-7, the precision of the FP32 vectors themselves.
struct ChunkSum {
  double total = 0.0;
  float part = 0.f;
  int k = 0;
  __device__ __forceinline__ void add(float v) {
    part += v;
    if (++k == 16) {
      total += double(part);
      part = 0.f;
      k = 0;
    }
  }
  __device__ __forceinline__ double sum() const { return total + double(part); }
};

// Reliable update of the mixed sequence: x += d32, d32 = 0, then r32 = b - A x from the FP64 stencil;
// t2 = (r32 . D r32, |r|^2) reduced over the team. Not inlined: its FP64 pointers and temporaries stay
// out of the register allocation of the FP32 iteration (which runs hundreds of times per call of this).
template <int NS, class Team>
__device__ __noinline__ void replace_residual(Team& t, int n, int lo, int hi, const Scratch<NS>& w, double* x,
                                              double* t2) {
  const int nv = n + 1;
  for (int i = lo + t.tid(); i < hi; i += t.stride()) {
    x[i] += double(w.d32()[i]);
    w.d32()[i] = 0.0f;
  }
  t.sync();  // x complete before the FP64 residual reads the neighbours' rows
  double v[2] = {0.0, 0.0};
  for (int i = lo + t.tid(); i < hi; i += t.stride()) {
    const int ix = i % nv, iy = i / nv;
    const double ri = w.b()[i] - stencil_row<NS, double>(t, w.S(), x, i, nv, vbnd(ix, iy, n));
    const float rf = float(ri);
    w.r32()[i] = rf;
    v[0] += double(rf) * double(w.dinv32()[i] * rf);
    v[1] += ri * ri;
  }
  t.reduce(v, 6);
  t2[0] = v[0];
  t2[1] = v[1];
}

// Mixed-precision CG with reliable updates: x (FP64) = 0 on entry, b the FP64 load; the FP32 sequence
// iterates d32 (correction), r32, p32, q32. Convergence is decided on the true FP64 residual only;
// relres = ||b - A x|| / ||b|| of the returned x.
template <int NS, class Team>
__device__ bool cg_reliable(const BatchArgs& a, Team& t, int n, int lo, int hi, const Scratch<NS>& w,
                            double* x, double bad, int& iters, int& conv, double& relres) {
  const int nv = n + 1;
  double v3[3] = {0.0, 0.0, bad};  // (the non-finite count as in cg_fp64)
  for (int i = lo + t.tid(); i < hi; i += t.stride()) {
    const float ri = float(w.b()[i]), zi = w.dinv32()[i] * ri;
    w.r32()[i] = ri;
    w.p32()[i] = zi;
    w.d32()[i] = 0.0f;
    v3[0] += double(ri) * double(zi);
    v3[1] += w.b()[i] * w.b()[i];
  }
  t.reduce(v3, 0);
  iters = 0;
  conv = 0;
  relres = 0.0;
  if (v3[2] > 0.0) return false;
  double rho = v3[0], rho_prev = rho;
  const double rr0 = v3[1];
  double rr_ref = rr0;      // true residual at the last replacement
  double drop = 0.01;       // replace when the iterated residual has dropped by this factor (squared)
  bool restarting = false;  // the FP32 operator is too far from the FP64 one to continue the sequence
  conv = (rr0 == 0.0) ? 1 : 0;
  relres = 0.0;
  iters = 0;
  t.sync();
  while (!conv && iters < a.max_iter) {
    ChunkSum pq;
    for (int i = lo + t.tid(); i < hi; i += t.stride()) {
      const int ix = i % nv, iy = i / nv;
      const float qi = stencil_row<NS, float>(t, w.S32(), w.p32(), i, nv, vbnd(ix, iy, n));
      w.q32()[i] = qi;
      pq.add(w.p32()[i] * qi);
    }
    double v1[1] = {pq.sum()};
    t.reduce(v1, 3);
    if (!(v1[0] > 0.0)) break;  // breakdown in FP32: the true residual below decides
    const float alpha = float(rho / v1[0]);
    ChunkSum rz, rr;
    for (int i = lo + t.tid(); i < hi; i += t.stride()) {
      w.d32()[i] = fmaf(alpha, w.p32()[i], w.d32()[i]);
      const float ri = fmaf(-alpha, w.q32()[i], w.r32()[i]);
      w.r32()[i] = ri;
      rz.add(ri * (w.dinv32()[i] * ri));
      rr.add(ri * ri);
    }
    double w2[2] = {rz.sum(), rr.sum()};
    t.reduce(w2, 4);
    ++iters;
    double beta = w2[0] / rho;
    rho_prev = rho;
    rho = w2[0];
    if (w2[1] <= drop * rr_ref || w2[1] <= a.tol2 * rr0 || iters >= a.max_iter) {
      // reliable update: x += d, d = 0; r = b - A x (FP64), r32 = r; beta from the replaced residual
      double t2[2];
      replace_residual<NS>(t, n, lo, hi, w, x, t2);
      // Stagnation guard: when a whole cycle gained less than 2x on the true residual, the gap between
      // the FP32 and FP64 operators dominates. From then on every replacement restarts the direction
      // (beta = 0) and waits for a 1000x drop: FP64 iterative refinement around FP32 CG.
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
    for (int i = lo + t.tid(); i < hi; i += t.stride()) w.p32()[i] = fmaf(bf, w.p32()[i], w.dinv32()[i] * w.r32()[i]);
    t.sync();
  }
  if (!conv) {  // stopped by breakdown or the iteration limit: fold in the correction, report the true residual
    t.sync();
    double t2[2];
    replace_residual<NS>(t, n, lo, hi, w, x, t2);
    relres = rr0 > 0.0 ? sqrt(t2[1] / rr0) : 0.0;
    if (t2[1] <= a.tol2 * rr0) conv = 1;
  }
  return true;
}

// one problem, start to finish, by one team
template <int NS, bool MIXED, class Team>
__device__ void solve_problem(const BatchArgs& a, Team& t, int prob, double* s64, float* s32, long long stride) {
  const int n = a.cells[prob];
  const int nv = n + 1;
  const int N = nv * nv;
  int lo, hi;
  t.range(N, lo, hi);
  const Scratch<NS> w{s64, s32, stride};
  double* x = a.x + a.off[prob];
  const double bad = assemble_rows<NS>(a, t, prob, n, lo, hi, w, x);
  int iters = 0, conv = 0, st = GDT_OK;
  double relres = 0.0;
  if constexpr (!MIXED) {
    if (cg_fp64<NS>(a, t, n, lo, hi, w, x, bad, iters, conv)) {
      // true relative residual of the returned iterate
      t.sync();
      double v2[2] = {0.0, 0.0};
      for (int i = lo + t.tid(); i < hi; i += t.stride()) {
        const int ix = i % nv, iy = i / nv;
        const double ri = w.b()[i] - stencil_row<NS, double>(t, w.S(), x, i, nv, vbnd(ix, iy, n));
        v2[0] += ri * ri;
        v2[1] += w.b()[i] * w.b()[i];
      }
      t.reduce(v2, 0);
      relres = v2[1] > 0 ? sqrt(v2[0] / v2[1]) : 0.0;
      st = conv ? GDT_OK : GDT_ENOCONV;
    } else {
      st = GDT_ENAN;  // skipped: x stays 0
    }
  } else {
    if (cg_reliable<NS>(a, t, n, lo, hi, w, x, bad, iters, conv, relres)) st = conv ? GDT_OK : GDT_ENOCONV;
    else st = GDT_ENAN;
  }
  if (t.leader()) {
    a.iters[prob] = conv ? iters : -iters - 1;
    a.relres[prob] = relres;
    a.status[prob] = st;
  }
}

// At most 64 registers: four CTAs per SM, so twice as many clusters (problems in flight) as at the
// 128 registers the compiler would otherwise use. One instantiation per precision: the FP64 one then
// needs no spills. The mixed one (the FP32 sequence next to the FP64 residual replacement) spills some
// 300 bytes per thread, and still runs the 512-problem bench 1.4x faster than at three CTAs per SM
// and 80 registers (the large problems want the loads of more CTAs in flight).
template <int NS, bool MIXED>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(BT, 4)
    batch_kernel(const __grid_constant__ BatchArgs a) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = int(cl.block_rank());
  const long long cid = blockIdx.x / CL;
  __shared__ int s_item;
  __shared__ double slots[10];
  double* s64 = a.s64 + cid * a.cwords;
  float* s32 = a.s32 + cid * a.cwords;
  constexpr long long kWords = NS + 5;
  for (;;) {
    if (rank == 0 && threadIdx.x == 0) s_item = atomicAdd(a.queue, 1);
    cl.sync();
    const int it = *cl.map_shared_rank(&s_item, 0);
    cl.sync();
    if (it >= a.nitems) break;
    const BatchItem item = a.items[it];
    if (item.team == GDT_BATCH_TEAM_CLUSTER) {
      ClusterTeam t{cl, rank, slots};
      solve_problem<NS, MIXED>(a, t, a.probs[item.first], s64, s32, item.stride);
    } else if (item.team == GDT_BATCH_TEAM_CTA) {
      if (rank < item.count) {
        CtaTeam t{slots};
        const long long base = rank * kWords * item.stride;
        solve_problem<NS, MIXED>(a, t, a.probs[item.first + rank], s64 + base, s32 + base, item.stride);
      }
    } else {
      const int k = rank * WPC + int(threadIdx.x >> 5);
      if (k < item.count) {
        WarpTeam t;
        const long long base = k * kWords * item.stride;
        solve_problem<NS, MIXED>(a, t, a.probs[item.first + k], s64 + base, s32 + base, item.stride);
      }
    }
    cl.sync();  // the item's teams are done before the scratch is reused
  }
}

const void* kernel_of(int element, bool mixed) {
  if (element == GDT_BATCH_Q1_CUBE)
    return mixed ? reinterpret_cast<const void*>(&batch_kernel<9, true>)
                 : reinterpret_cast<const void*>(&batch_kernel<9, false>);
  return mixed ? reinterpret_cast<const void*>(&batch_kernel<7, true>)
               : reinterpret_cast<const void*>(&batch_kernel<7, false>);
}
int stencil_of(int element) { return element == GDT_BATCH_Q1_CUBE ? 9 : 7; }

// ------------------------------------------------------------------------------------ host ---
// The queue for the problems `subset` under the batch's team assignment: largest first; cluster items
// hold one problem, CTA items up to 8, warp items up to 64 (problems of one team kind, consecutive in
// size order). Returns the scratch words one cluster needs.
long long build_items(const gdt_batch_s& b, std::vector<int> subset, std::vector<BatchItem>& items,
                      std::vector<int>& probs) {
  std::stable_sort(subset.begin(), subset.end(), [&](int x, int y) { return b.cells[x] > b.cells[y]; });
  items.clear();
  probs.clear();
  const long long words = stencil_of(b.element) + 5;
  long long need = 0;
  int cap[3] = {1, CL, CL * WPC};
  std::vector<int> pending[3];
  auto flush = [&](int team) {
    auto& P = pending[team];
    if (P.empty()) return;
    BatchItem it;
    it.team = team;
    it.first = int(probs.size());
    it.count = int(P.size());
    it.pad = 0;
    const long long nd = (b.cells[P[0]] + 1) * (b.cells[P[0]] + 1);
    it.stride = (nd + 31) / 32 * 32;
    for (int p : P) probs.push_back(p);
    items.push_back(it);
    need = std::max(need, it.count * words * it.stride);
    P.clear();
  };
  for (int p : subset) {
    const int team = b.teams[p];
    pending[team].push_back(p);
    if ((int)pending[team].size() == cap[team]) flush(team);
  }
  for (int team = 0; team < 3; ++team) flush(team);
  std::stable_sort(items.begin(), items.end(), [](const BatchItem& x, const BatchItem& y) { return x.stride > y.stride; });
  return need;
}

gdt_status ensure_scratch(gdt_context ctx, gdt_batch b, long long words) {
  if (words <= b->scratch_words) return GDT_OK;
  cudaFree(b->scratch64);
  cudaFree(b->scratch32);
  b->scratch64 = nullptr;
  b->scratch32 = nullptr;
  b->scratch_words = 0;
  cudaError_t e = cudaMalloc(&b->scratch64, sizeof(double) * words * b->nclusters);
  if (e == cudaSuccess) e = cudaMalloc(&b->scratch32, sizeof(float) * words * b->nclusters);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, e == cudaErrorMemoryAllocation ? GDT_ENOMEM : GDT_ECUDA, "batch scratch");
  }
  b->scratch_words = words;
  return GDT_OK;
}

// the queue of the whole batch under the current team assignment, on the device
gdt_status upload_queue(gdt_context ctx, gdt_batch b) {
  // a launch in flight on the context stream may still read the old queue and scratch
  if (ctx->stream) GDT_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<int> all(b->nprob);
  std::iota(all.begin(), all.end(), 0);
  const long long need = build_items(*b, all, b->items, b->probs);
  GDT_TRY_CUDA(ctx, cudaMemcpy(b->d_items, b->items.data(), sizeof(BatchItem) * b->items.size(), cudaMemcpyHostToDevice));
  GDT_TRY_CUDA(ctx, cudaMemcpy(b->d_probs, b->probs.data(), sizeof(int) * b->probs.size(), cudaMemcpyHostToDevice));
  b->generation++;
  return ensure_scratch(ctx, b, need);
}

// P1 stiffness of the two triangle types of a square cell and Q1 stiffness of a square (both scale
// invariant in 2D), from the gradients of the reference shape functions
void local_stiffness(int element, double (&K)[2][4][4]) {
  for (int t = 0; t < 2; ++t)
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) K[t][i][j] = 0.0;
  if (element == GDT_BATCH_Q1_CUBE) {
    // bilinear shape function of corner c (bits x, y) on [0, 1]^2; 2 x 2 Gauss points (exact here)
    const double g = 0.5 / std::sqrt(3.0);
    const double pts[2] = {0.5 - g, 0.5 + g};
    for (int qx = 0; qx < 2; ++qx)
      for (int qy = 0; qy < 2; ++qy) {
        const double X = pts[qx], Y = pts[qy];
        double G[4][2];
        for (int c = 0; c < 4; ++c) {
          const double fx = (c & 1) ? X : 1.0 - X, fy = (c & 2) ? Y : 1.0 - Y;
          const double dx = (c & 1) ? 1.0 : -1.0, dy = (c & 2) ? 1.0 : -1.0;
          G[c][0] = dx * fy;
          G[c][1] = fx * dy;
        }
        for (int i = 0; i < 4; ++i)
          for (int j = 0; j < 4; ++j) K[0][i][j] += 0.25 * (G[i][0] * G[j][0] + G[i][1] * G[j][1]);
      }
    return;
  }
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
      for (int j = 0; j < 3; ++j) K[t][i][j] = area * (G[i][0] * G[j][0] + G[i][1] * G[j][1]);
  }
}

struct SolveArgs {
  const double* kappa;
  int kappa_kind;
  double force;
  int precision;
  double tol;
  int max_iter;
  double* x;
  double* stencil_out;
};

gdt_status check_solve_args(gdt_context ctx, gdt_batch b, const SolveArgs& s) {
  if (!s.kappa || !s.x || !(s.tol > 0) || s.max_iter < 1) return GDT_EINVAL;
  if (s.precision != GDT_PRECISION_FP64 && s.precision != GDT_PRECISION_MIXED) return GDT_EINVAL;
  if (s.kappa_kind != GDT_BATCH_KAPPA_QUADRANTS && s.kappa_kind != GDT_BATCH_KAPPA_ELEMENTS) return GDT_EINVAL;
  if (s.kappa_kind == GDT_BATCH_KAPPA_QUADRANTS)
    for (long long c : b->cells)
      if (c % 2 != 0) return fail(ctx, GDT_EINVAL, "kappa per quadrant needs an even number of cells per side");
  return GDT_OK;
}

BatchArgs make_args(gdt_batch b, const SolveArgs& s) {
  BatchArgs a;
  a.nitems = int(b->items.size());
  a.items = b->d_items;
  a.probs = b->d_probs;
  a.off = b->d_off;
  a.eoff = b->d_eoff;
  a.cells = b->d_cells;
  a.kappa = s.kappa;
  a.kappa_elems = s.kappa_kind == GDT_BATCH_KAPPA_ELEMENTS;
  a.force = s.force;
  a.mixed = s.precision == GDT_PRECISION_MIXED;
  a.tol2 = s.tol * s.tol;
  a.max_iter = s.max_iter;
  a.x = s.x;
  a.stencil_out = s.stencil_out;
  a.iters = b->d_iters;
  a.relres = b->d_relres;
  a.status = b->d_status;
  a.queue = b->d_queue;
  a.cwords = b->scratch_words;
  a.s64 = b->scratch64;
  a.s32 = b->scratch32;
  local_stiffness(b->element, a.K);
  return a;
}

void launch(gdt_batch b, const BatchArgs& a, cudaStream_t s) {
  cudaMemsetAsync(b->d_queue, 0, sizeof(int), s);
  const dim3 grid(b->nclusters_prec[a.mixed ? 1 : 0] * CL);
  if (b->element == GDT_BATCH_Q1_CUBE) {
    if (a.mixed) batch_kernel<9, true><<<grid, BT, 0, s>>>(a);
    else batch_kernel<9, false><<<grid, BT, 0, s>>>(a);
  } else {
    if (a.mixed) batch_kernel<7, true><<<grid, BT, 0, s>>>(a);
    else batch_kernel<7, false><<<grid, BT, 0, s>>>(a);
  }
}

// per-problem results of the last launch over `subset` into info; the status of the call
gdt_status collect(gdt_context ctx, gdt_batch b, const std::vector<int>& subset, cudaStream_t s, gdt_batch_info* info) {
  std::vector<int> it(b->nprob), stv(b->nprob);
  std::vector<double> rr(b->nprob);
  cudaMemcpyAsync(it.data(), b->d_iters, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(rr.data(), b->d_relres, sizeof(double) * b->nprob, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(stv.data(), b->d_status, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail(ctx, GDT_ECUDA, "batch synchronize");
  gdt_batch_info loc;
  gdt_batch_info& I = info ? *info : loc;
  I.problems = (int64_t)subset.size();
  I.total_dofs = 0;
  I.max_iterations = 0;
  I.min_iterations = 1 << 30;
  I.all_converged = 1;
  I.max_rel_residual = 0.0;
  I.nonfinite_problems = 0;
  for (int i : subset) {
    I.total_dofs += b->offsets[i + 1] - b->offsets[i];
    const int v = it[i] >= 0 ? it[i] : -it[i] - 1;
    if (stv[i] != GDT_OK) I.all_converged = 0;
    if (stv[i] == GDT_ENAN) {
      I.nonfinite_problems++;
      continue;
    }
    I.max_iterations = std::max(I.max_iterations, v);
    I.min_iterations = std::min(I.min_iterations, v);
    I.max_rel_residual = std::max(I.max_rel_residual, rr[i]);
  }
  if (I.nonfinite_problems) return fail(ctx, GDT_ENAN, "a batched problem has non-finite data (skipped, x = 0)");
  if (!I.all_converged) return fail(ctx, GDT_ENOCONV, "a batched problem did not converge");
  return GDT_OK;
}

gdt_status solve_impl(gdt_context ctx, gdt_batch b, const SolveArgs& sa, gdt_batch_info* info) {
  gdt_status st = check_solve_args(ctx, b, sa);
  if (st != GDT_OK) return st;
  const BatchArgs a = make_args(b, sa);
  cudaStream_t s = ctx->stream;
  cudaStream_t own = nullptr;
  if (!s) {
    GDT_TRY_CUDA(ctx, cudaStreamCreate(&own));
    s = own;
  }
  // one graph per argument set and queue: queue reset + the persistent kernel
  auto mix = [](unsigned long long h, unsigned long long v) { return (h ^ v) * 0x100000001b3ULL; };
  unsigned long long key = 0xcbf29ce484222325ULL;
  key = mix(key, reinterpret_cast<unsigned long long>(sa.kappa));
  key = mix(key, reinterpret_cast<unsigned long long>(sa.x));
  key = mix(key, reinterpret_cast<unsigned long long>(sa.stencil_out));
  key = mix(key, (unsigned long long)sa.kappa_kind * 7 + (unsigned long long)a.mixed);
  key = mix(key, std::hash<double>()(sa.force));
  key = mix(key, std::hash<double>()(sa.tol));
  key = mix(key, (unsigned long long)sa.max_iter);
  key = mix(key, b->generation);
  key = mix(key, reinterpret_cast<unsigned long long>(b->scratch64));
  if (!b->exec || b->key != key) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      launch(b, a, s);
      if (cudaStreamEndCapture(s, &b->graph) != cudaSuccess || cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess)
        b->exec = nullptr;
    }
    cudaGetLastError();
    b->key = key;
  }
  if (b->exec) {
    if (cudaGraphLaunch(b->exec, s) != cudaSuccess) st = fail(ctx, GDT_ECUDA, "batch graph launch");
  } else {
    launch(b, a, s);
  }
  ctx->launches++;
  if (st == GDT_OK) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = fail(ctx, GDT_ECUDA, std::string("batch_kernel: ") + cudaGetErrorString(e));
  }
  if (st == GDT_OK && info) {
    std::vector<int> all(b->nprob);
    std::iota(all.begin(), all.end(), 0);
    st = collect(ctx, b, all, s, info);
  }
  if (own) {
    cudaStreamSynchronize(own);
    cudaStreamDestroy(own);
    // the cached graph stays valid: it is launched on whatever stream the next call uses
  }
  return st;
}

}  // namespace
}  // namespace gdt

using namespace gdt;

extern "C" {

gdt_status gdt_batch_create_ex(gdt_context ctx, int64_t nproblems, const int64_t* cells, int element, gdt_batch* out) {
  if (!ctx || !cells || !out || nproblems < 1 || nproblems > (1LL << 30)) return GDT_EINVAL;
  if (element != GDT_BATCH_P1_SIMPLEX && element != GDT_BATCH_Q1_CUBE) return GDT_EINVAL;
  *out = nullptr;
  gdt_batch b = new (std::nothrow) gdt_batch_s;
  if (!b) return GDT_ENOMEM;
  b->nprob = nproblems;
  b->element = element;
  b->cells.assign(cells, cells + nproblems);
  b->offsets.assign(nproblems + 1, 0);
  b->eoffsets.assign(nproblems + 1, 0);
  const long long per_cell = element == GDT_BATCH_P1_SIMPLEX ? 2 : 1;
  for (long long i = 0; i < nproblems; ++i) {
    if (cells[i] < 1 || cells[i] > 16384) {
      delete b;
      return fail(ctx, GDT_EINVAL, "cells per side must be in [1, 16384]");
    }
    const long long nd = (cells[i] + 1) * (cells[i] + 1);
    b->offsets[i + 1] = b->offsets[i] + nd;
    b->eoffsets[i + 1] = b->eoffsets[i] + per_cell * cells[i] * cells[i];
    b->max_dofs = std::max(b->max_dofs, nd);
  }
  b->total = b->offsets[nproblems];
  b->total_elems = b->eoffsets[nproblems];
  b->teams.assign(nproblems, GDT_BATCH_TEAM_CLUSTER);
  for (int mixed = 0; mixed < 2; ++mixed) {
    int max_clusters = 0;
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
    if (cudaOccupancyMaxActiveClusters(&max_clusters, kernel_of(element, mixed), &cfg) != cudaSuccess ||
        max_clusters < 1)
      max_clusters = std::max(1, ctx->num_sms / CL);
    cudaGetLastError();
    b->nclusters_prec[mixed] = int(std::min<long long>(max_clusters, nproblems));
  }
  b->nclusters = std::max(b->nclusters_prec[0], b->nclusters_prec[1]);
  std::vector<int> c32(b->cells.begin(), b->cells.end());
  cudaError_t e = cudaMalloc(&b->d_items, sizeof(BatchItem) * nproblems);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_probs, sizeof(int) * nproblems);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_off, sizeof(long long) * (nproblems + 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_eoff, sizeof(long long) * (nproblems + 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_cells, sizeof(int) * nproblems);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_queue, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_iters, sizeof(int) * nproblems);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_relres, sizeof(double) * nproblems);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_status, sizeof(int) * nproblems);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_off, b->offsets.data(), sizeof(long long) * (nproblems + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_eoff, b->eoffsets.data(), sizeof(long long) * (nproblems + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_cells, c32.data(), sizeof(int) * nproblems, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaGetLastError();
    gdt_batch_destroy(b);
    return fail(ctx, e == cudaErrorMemoryAllocation ? GDT_ENOMEM : GDT_ECUDA, cudaGetErrorString(e));
  }
  const gdt_status st = upload_queue(ctx, b);
  if (st != GDT_OK) {
    gdt_batch_destroy(b);
    return st;
  }
  *out = b;
  return GDT_OK;
}

gdt_status gdt_batch_create(gdt_context ctx, int64_t nproblems, const int64_t* cells, gdt_batch* out) {
  return gdt_batch_create_ex(ctx, nproblems, cells, GDT_BATCH_P1_SIMPLEX, out);
}

gdt_status gdt_batch_destroy(gdt_batch b) {
  if (!b) return GDT_EINVAL;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  cudaFree(b->d_items);
  cudaFree(b->d_probs);
  cudaFree(b->d_off);
  cudaFree(b->d_eoff);
  cudaFree(b->d_cells);
  cudaFree(b->d_queue);
  cudaFree(b->d_iters);
  cudaFree(b->d_relres);
  cudaFree(b->d_status);
  cudaFree(b->scratch64);
  cudaFree(b->scratch32);
  delete b;
  return GDT_OK;
}

int64_t gdt_batch_total_dofs(gdt_batch b) { return b ? b->total : -1; }
int64_t gdt_batch_total_elements(gdt_batch b) { return b ? b->total_elems : -1; }

gdt_status gdt_batch_dof_offsets(gdt_batch b, int64_t* offsets) {
  if (!b || !offsets) return GDT_EINVAL;
  for (long long i = 0; i <= b->nprob; ++i) offsets[i] = b->offsets[i];
  return GDT_OK;
}

gdt_status gdt_batch_element_offsets(gdt_batch b, int64_t* offsets) {
  if (!b || !offsets) return GDT_EINVAL;
  for (long long i = 0; i <= b->nprob; ++i) offsets[i] = b->eoffsets[i];
  return GDT_OK;
}

gdt_status gdt_batch_set_teams(gdt_context ctx, gdt_batch b, const int* teams) {
  if (!ctx || !b || !teams) return GDT_EINVAL;
  for (long long i = 0; i < b->nprob; ++i)
    if (teams[i] != GDT_BATCH_TEAM_CLUSTER && teams[i] != GDT_BATCH_TEAM_CTA && teams[i] != GDT_BATCH_TEAM_WARP)
      return fail(ctx, GDT_EINVAL, "team must be GDT_BATCH_TEAM_CLUSTER, _CTA or _WARP");
  b->teams.assign(teams, teams + b->nprob);
  return upload_queue(ctx, b);
}

gdt_status gdt_batch_teams(gdt_batch b, int* teams) {
  if (!b || !teams) return GDT_EINVAL;
  for (long long i = 0; i < b->nprob; ++i) teams[i] = b->teams[i];
  return GDT_OK;
}

gdt_status gdt_batch_solve_ex(gdt_context ctx, gdt_batch b, const double* kappa, int kappa_kind, double force,
                              int precision, double tol, int max_iter, double* x, double* stencil_out,
                              gdt_batch_info* info) {
  if (!ctx || !b) return GDT_EINVAL;
  return solve_impl(ctx, b, SolveArgs{kappa, kappa_kind, force, precision, tol, max_iter, x, stencil_out}, info);
}

gdt_status gdt_batch_solve(gdt_context ctx, gdt_batch b, const double* mu, double force, int precision, double tol,
                           int max_iter, double* x, double* stencil_out, gdt_batch_info* info) {
  if (!ctx || !b) return GDT_EINVAL;
  return solve_impl(ctx, b,
                    SolveArgs{mu, GDT_BATCH_KAPPA_QUADRANTS, force, precision, tol, max_iter, x, stencil_out}, info);
}

gdt_status gdt_batch_tune(gdt_context ctx, gdt_batch b, const double* kappa, int kappa_kind, double force,
                          int precision, double tol, int max_iter, double* x, int64_t* nsizes, int64_t* sizes,
                          double* ms) {
  if (!ctx || !b) return GDT_EINVAL;
  const SolveArgs sa{kappa, kappa_kind, force, precision, tol, max_iter, x, nullptr};
  gdt_status st = check_solve_args(ctx, b, sa);
  if (st != GDT_OK) return st;
  // size classes, largest first
  std::map<long long, std::vector<int>, std::greater<long long>> classes;
  for (long long i = 0; i < b->nprob; ++i) classes[b->cells[i]].push_back(int(i));
  cudaStream_t s = ctx->stream;
  cudaEvent_t e0, e1;
  GDT_TRY_CUDA(ctx, cudaEventCreate(&e0));
  GDT_TRY_CUDA(ctx, cudaEventCreate(&e1));
  std::vector<int> chosen = b->teams;
  const std::vector<int> saved = b->teams;
  long long k = 0;
  for (const auto& cls : classes) {
    const long long n = cls.first;
    const long long nd = (n + 1) * (n + 1);
    double best = -1.0;
    int best_team = GDT_BATCH_TEAM_CLUSTER;
    for (int team = 0; team < 3; ++team) {
      double t_ms = -1.0;
      if (team != GDT_BATCH_TEAM_WARP || nd <= kWarpMaxDofs) {
        for (int i : cls.second) b->teams[i] = team;
        std::vector<BatchItem> items;
        std::vector<int> probs;
        const long long need = build_items(*b, cls.second, items, probs);
        st = ensure_scratch(ctx, b, need);
        if (st != GDT_OK) break;
        if (cudaMemcpyAsync(b->d_items, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice, s) !=
                cudaSuccess ||
            cudaMemcpyAsync(b->d_probs, probs.data(), sizeof(int) * probs.size(), cudaMemcpyHostToDevice, s) !=
                cudaSuccess) {
          st = fail(ctx, GDT_ECUDA, "batch tune upload");
          break;
        }
        BatchArgs a = make_args(b, sa);
        a.nitems = int(items.size());
        launch(b, a, s);  // warm-up (first use of the scratch, caches)
        cudaEventRecord(e0, s);
        launch(b, a, s);
        cudaEventRecord(e1, s);
        ctx->launches += 2;
        gdt_batch_info info;
        st = collect(ctx, b, cls.second, s, &info);
        float f = 0.f;
        cudaEventElapsedTime(&f, e0, e1);
        if (st != GDT_OK) break;  // the data itself fails (non-finite, no convergence): report it
        t_ms = f;
        if (best < 0.0 || t_ms < best) {
          best = t_ms;
          best_team = team;
        }
      }
      if (ms) ms[3 * k + team] = t_ms;
    }
    if (st != GDT_OK) break;
    for (int i : cls.second) chosen[i] = best_team;
    if (sizes) sizes[k] = n;
    ++k;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (nsizes) *nsizes = k;
  b->teams = st == GDT_OK ? chosen : saved;
  const gdt_status up = upload_queue(ctx, b);
  return st != GDT_OK ? st : up;
}

gdt_status gdt_batch_iterations(gdt_context ctx, gdt_batch b, int* iterations, double* rel_residuals) {
  if (!ctx || !b) return GDT_EINVAL;
  if (iterations) GDT_TRY_CUDA(ctx, cudaMemcpy(iterations, b->d_iters, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost));
  if (rel_residuals)
    GDT_TRY_CUDA(ctx, cudaMemcpy(rel_residuals, b->d_relres, sizeof(double) * b->nprob, cudaMemcpyDeviceToHost));
  return GDT_OK;
}

gdt_status gdt_batch_status(gdt_context ctx, gdt_batch b, int* status) {
  if (!ctx || !b || !status) return GDT_EINVAL;
  GDT_TRY_CUDA(ctx, cudaMemcpy(status, b->d_status, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost));
  return GDT_OK;
}

}  // extern "C"
