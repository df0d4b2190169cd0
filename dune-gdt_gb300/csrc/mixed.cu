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
// FP32 layout: vertex rows (x lines) are stored with a pitch, a multiple of 4 on 3D grids (zero
// padding past the last vertex of a line) so that every line starts on a 16-byte boundary, as the
// bulk-tensor (TMA) tile loads of the 3D SpMV require; vertex v = x + nx * r of the FP64 vectors is
// element x + pitch * r of the FP32 ones. The padding stays zero in every FP32 vector.
//
// Reliable updates (one Krylov sequence, no restarts): x32 accumulates the FP32 correction; whenever
// the iterated residual has dropped by 10x since the last update (or reached the tolerance), the
// correction is added to the FP64 solution, the true residual r = b - A x is recomputed from the FP64
// CSR matrix and replaces the FP32 residual, and beta is recomputed from it. Convergence is decided
// only on the true FP64 residual. A solve whose true residual stops following (less than 2x gained over
// a cycle) falls back to restarted iterative refinement: direction reset at every replacement, which
// then waits for a 1000x drop.
#include <cudaTypedefs.h>

#include <cmath>
#include <cstring>
#include <cstdint>
#include <mutex>
#include <vector>

#include "linalg.cuh"
#include "structured.cuh"
#include "tma.cuh"

namespace gdt {

namespace {

constexpr int TH = 256;
constexpr int MAXU = 13;  // upper slots of the 27-point stencil

struct MState {
  double rho, rho_prev, alpha, beta, rr, rr0, rr_ref, tol2;
  double drop;  // replacement when the iterated residual (squared) has dropped by this factor
  int iter, max_iter, converged, flag, breakdown, updates;
  int restarting;  // stagnation guard tripped: every replacement restarts the direction
  // Chronopoulos-Gear recurrences (matrix-free path): gamma = r.z, its previous value, previous alpha
  double gamma, gamma_prev, alpha_prev;
  int replaced_iter;  // iteration of the last residual replacement (gates the operator that follows it)
  int fault;  // a bounded device wait ran out (tile loads of the 3D SpMV)
};

__device__ __forceinline__ bool mstopped(const MState* st) { return entry_flag(&st->converged) != 0; }

struct Stencil {
  int nu;               // upper slots
  long long off[MAXU];  // their linear offsets (> 0) in FP32 (pitched) elements
  long long coff[MAXU]; // the same offsets in vertices (CSR columns)
  long long pad;        // halo >= largest offset, a multiple of 4
};

// FP32 element of vertex v (x lines of nx vertices stored with `pitch`)
struct Pitch {
  int nx;
  int extra;  // pitch - nx
  __device__ __forceinline__ long long of(long long v) const { return extra ? v + extra * (v / nx) : v; }
};

// D_o arrays: diag at D, upper slot u at D + (u + 1) * ld (each with `pad` leading zeros before element 0)
__global__ void k_build_stencil(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                const double* __restrict__ val, Stencil S, Pitch pt, float* __restrict__ D,
                                long long ld, int* __restrict__ bad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const long long ip = pt.of(i);
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      const long long o = (long long)col[k] - i;
      if (o < 0) continue;
      int slot = -1;
      if (o == 0) slot = 0;
      for (int u = 0; u < S.nu; ++u)
        if (S.coff[u] == o) slot = u + 1;
      if (slot < 0) {
        atomicExch(bad, 1);
        continue;
      }
      D[slot * ld + S.pad + ip] = float(val[k]);
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

// 3D form of the same product, tiled for GB300's shared memory and fed by TMA (vertex grids with
// nx, ny >= 3, where every stencil slot has its own linear offset). A CTA owns a 32 x 8 tile of an
// x-y plane and walks a chunk of z planes. One thread issues bulk-tensor loads of 40 x 10-element
// boxes (the tile with a one-vertex halo, x rounded out to 16-byte boundaries; the hardware
// zero-fills outside the grid) LA planes ahead, each plane's boxes completing on its own mbarrier:
// the in-plane upper slots (dz = 0) and out-of-plane upper slots (dz = +1) of the plane and p of the
// plane after it. Row (x, y, z) is
//   D_0 p + sum_in [D_o(i) p(i + o) + D_o(i - o) p(i - o)] + sum_up D_o(i) p(i + o) + L(x, y, z),
// where the in-plane lower terms and the out-of-plane upper terms use plane z's boxes, and
// L(x, y, z) = sum_up D_o(i - o) p(i - o) only needs plane z - 1: each thread computes it for its
// own column while plane z - 1 is resident and carries it in a register to the next plane. So per
// plane the CTA holds the slot boxes of one plane (plus those in flight) and p of two. Per row the
// kernel streams (1 + upper slots) * 4 bytes from HBM and issues no per-element staging
// instructions. A wait that runs out sets MState::fault and the kernel stops computing.
constexpr int S3X = 32, S3Y = 8;
constexpr int TW = 40, TR = 10;  // box: x0 - 4 .. x0 + 35, y0 - 1 .. y0 + 8
constexpr int TS = 416;          // box stride in shared memory, floats (1600 bytes rounded up to 128)
constexpr uint32_t kBoxBytes = TW * TR * 4;
constexpr int LA = 2;            // planes in flight ahead of the one computed

struct Stencil3 {
  int nin, nup;
  int in_slot[4], up_slot[9];  // indices into the upper slots of Stencil
  int in_o[4], up_o[9];        // in-box offsets dy * TW + dx
};

// rings: p of LA + 2 planes, slot boxes of LA + 1 planes, LA + 1 barriers
template <int NIN, int NUP>
constexpr size_t spmv3d_smem_bytes() {
  return 128 + sizeof(float) * TS * ((LA + 2) + (LA + 1) * (NUP + NIN)) + (LA + 1) * sizeof(uint64_t);
}

// 1D grid (the grid reduction counts blocks along x): block b = (bz * tiles_y + by) * tiles_x + bx.
// tmD: slot arrays, 4D (x, y, z, slot); tmP: p, 3D; both with the FP32 pitch.
template <int NIN, int NUP>
__global__ void __launch_bounds__(S3X* S3Y) k_mx_spmv3d(int nx, int ny, int nz, int zlen, long long pitch,
                                                        Stencil3 T3, const __grid_constant__ CUtensorMap tmD,
                                                        const __grid_constant__ CUtensorMap tmP,
                                                        const float* __restrict__ D0, float* __restrict__ q,
                                                        MState* st, double* partials, unsigned int* ticket) {
  if (mstopped(st)) return;
  float* const P = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(gdt_dyn_smem) + 127) & ~uintptr_t(127));
  float* const U = P + (LA + 2) * TS;
  float* const I = U + (LA + 1) * NUP * TS;
  uint64_t* const bar = reinterpret_cast<uint64_t*>(I + (LA + 1) * NIN * TS);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int tiles_x = (nx + S3X - 1) / S3X, tiles_y = (ny + S3Y - 1) / S3Y;
  const int bx = blockIdx.x % tiles_x, by = (blockIdx.x / tiles_x) % tiles_y, bz = blockIdx.x / (tiles_x * tiles_y);
  const int x0 = bx * S3X, y0 = by * S3Y, xs = x0 - 4, ys = y0 - 1;
  const int zb = bz * zlen, ze = min(nz, zb + zlen);
  // ring slots by plane (planes >= zb - 1)
  auto Pz = [&](int z) { return P + ((z - zb + 1) % (LA + 2)) * TS; };
  auto Uz = [&](int z) { return U + ((z - zb + 1) % (LA + 1)) * (NUP * TS); };
  auto Iz = [&](int z) { return I + ((z - zb + 1) % (LA + 1)) * (NIN * TS); };
  // stage k: 0 = out-of-plane slots and p of plane zb - 1, p of plane zb; k >= 1 = slots of plane
  // zb + k - 1 and p of plane zb + k; barrier k % (LA + 1), phase parity (k / (LA + 1)) & 1
  auto issue = [&](int k) {
    uint64_t* b = &bar[k % (LA + 1)];
    if (k == 0) {
      mbar_arrive_expect_tx(b, kBoxBytes * (NUP + 2));
      tma_load_3d(Pz(zb - 1), &tmP, xs, ys, zb - 1, b);
      tma_load_3d(Pz(zb), &tmP, xs, ys, zb, b);
#pragma unroll
      for (int u = 0; u < NUP; ++u) tma_load_4d(Uz(zb - 1) + u * TS, &tmD, xs, ys, zb - 1, T3.up_slot[u] + 1, b);
    } else {
      const int z = zb + k - 1;
      mbar_arrive_expect_tx(b, kBoxBytes * (NIN + NUP + 1));
#pragma unroll
      for (int u = 0; u < NIN; ++u) tma_load_4d(Iz(z) + u * TS, &tmD, xs, ys, z, T3.in_slot[u] + 1, b);
#pragma unroll
      for (int u = 0; u < NUP; ++u) tma_load_4d(Uz(z) + u * TS, &tmD, xs, ys, z, T3.up_slot[u] + 1, b);
      tma_load_3d(Pz(z + 1), &tmP, xs, ys, z + 1, b);
    }
  };
  auto wait = [&](int k) { return mbar_wait(&bar[k % (LA + 1)], (k / (LA + 1)) & 1); };
  const int kmax = ze - zb;  // stages 0 .. kmax
  if (threadIdx.x == 0) {
#pragma unroll
    for (int b = 0; b <= LA; ++b) mbar_init(&bar[b], 1);
    mbar_init_fence();
  }
  __syncthreads();  // every thread sees initialised barriers before its first wait
  if (threadIdx.x == 0)
    for (int k = 0; k <= LA && k <= kmax; ++k) issue(k);
  const int gx = x0 + tx, gy = y0 + ty;
  const bool own = gx < nx && gy < ny;
  const int c = (ty + 1) * TW + tx + 4;
  float acc = 0.f, lower = 0.f;
  int failed_at = -1;
  // L(x, y, zb) from plane zb - 1
  if (!__syncthreads_and(wait(0))) {
    failed_at = 0;
  } else {
    const float* Pm = Pz(zb - 1);
    const float* Um = Uz(zb - 1);
#pragma unroll
    for (int u = 0; u < NUP; ++u) lower = fmaf(Um[u * TS + c - T3.up_o[u]], Pm[c - T3.up_o[u]], lower);
    __syncthreads();  // stage LA + 1 reuses the slots of plane zb - 1
  }
  for (int z = zb, k = 1; failed_at < 0 && z < ze; ++z, ++k) {
    if (threadIdx.x == 0 && k + LA <= kmax) {
      fence_proxy_async_smem();
      issue(k + LA);
    }
    const long long ip = gx + pitch * (gy + (long long)ny * z);
    const float d0 = own ? __ldcs(D0 + ip) : 0.f;
    if (!__syncthreads_and(wait(k))) {
      failed_at = k;
      break;
    }
    const float* Pc = Pz(z);
    const float* Pn = Pz(z + 1);
    const float* Ic = Iz(z);
    const float* Uc = Uz(z);
    float s = fmaf(d0, Pc[c], lower);
    float next = 0.f;
#pragma unroll
    for (int u = 0; u < NIN; ++u) {
      const int o = T3.in_o[u];
      s = fmaf(Ic[u * TS + c], Pc[c + o], s);
      s = fmaf(Ic[u * TS + c - o], Pc[c - o], s);
    }
#pragma unroll
    for (int u = 0; u < NUP; ++u) {
      const int o = T3.up_o[u];
      s = fmaf(Uc[u * TS + c], Pn[c + o], s);
      next = fmaf(Uc[u * TS + c - o], Pc[c - o], next);
    }
    if (own) {
      q[ip] = s;
      acc = fmaf(Pc[c], s, acc);
    }
    lower = next;
    __syncthreads();  // stage k + LA + 1 reuses the slots of plane z and the box of p(z)
  }
  if (failed_at >= 0) {
    // report, then give the copies in flight a bounded chance to land before the CTA's shared
    // memory is released
    if (threadIdx.x == 0) {
      st->fault = 1;
      st->breakdown = 1;
      st->converged = 1;
      for (int k = failed_at; k <= kmax && k <= failed_at + LA; ++k) wait(k);
    }
    acc = 0.f;
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

// x32 += alpha p ; r32 -= alpha q ; rz, rr ; reliable-update trigger. Quads of rows per thread
// (16-byte accesses; every vector starts on a 16-byte boundary), the rows past the last quad scalar.
__device__ __forceinline__ void mx_update_row(float alpha, float& x, float p, float& r, float q, float d, float& a0,
                                              float& a1) {
  x = fmaf(alpha, p, x);
  r = fmaf(-alpha, q, r);
  a0 = fmaf(r, d * r, a0);
  a1 = fmaf(r, r, a1);
}

// cond (0 outside graph capture): the IF node of this iteration's reliable update, set to the flag
__global__ void __launch_bounds__(TH) k_mx_update(int n, float* __restrict__ x32, const float* __restrict__ p,
                                                 float* __restrict__ r, const float* __restrict__ q,
                                                 const float* __restrict__ dinv, MState* st, double* partials,
                                                 unsigned int* ticket, cudaGraphConditionalHandle cond) {
  if (mstopped(st)) return;
  const float alpha = float(st->alpha);
  float a0 = 0.f, a1 = 0.f;
  const int n4 = n >> 2, stride = gridDim.x * blockDim.x;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += stride) {
    float4 xv = reinterpret_cast<const float4*>(x32)[k];
    float4 rv = reinterpret_cast<const float4*>(r)[k];
    const float4 pv = reinterpret_cast<const float4*>(p)[k];
    const float4 qv = reinterpret_cast<const float4*>(q)[k];
    const float4 dv = reinterpret_cast<const float4*>(dinv)[k];
    mx_update_row(alpha, xv.x, pv.x, rv.x, qv.x, dv.x, a0, a1);
    mx_update_row(alpha, xv.y, pv.y, rv.y, qv.y, dv.y, a0, a1);
    mx_update_row(alpha, xv.z, pv.z, rv.z, qv.z, dv.z, a0, a1);
    mx_update_row(alpha, xv.w, pv.w, rv.w, qv.w, dv.w, a0, a1);
    reinterpret_cast<float4*>(x32)[k] = xv;
    reinterpret_cast<float4*>(r)[k] = rv;
  }
  for (int i = 4 * n4 + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    mx_update_row(alpha, x32[i], p[i], r[i], q[i], dinv[i], a0, a1);
  double v[2] = {double(a0), double(a1)};
  if (grid_reduce<2>(v, partials, ticket) && threadIdx.x == 0) {
    st->rho_prev = st->rho;
    st->beta = v[0] / st->rho;
    st->rho = v[0];
    st->rr = v[1];
    st->iter += 1;
    st->flag = (v[1] <= st->drop * st->rr_ref || v[1] <= st->tol2 * st->rr0 || st->iter >= st->max_iter) ? 1 : 0;
    if (!isfinite(v[1])) {
      st->breakdown = 1;
      st->converged = 1;
    }
    if (cond) cudaGraphSetConditional(cond, (st->flag && !st->converged) ? 1u : 0u);
  }
}

// ---------------------------------------------------------------- matrix-free inner operator ---
// 3D Q1 Laplace with element coefficients: q_v = sum over the (up to) 8 cells c around vertex v of
// kappa_c sum_j K[l_v][j] p(corner j of c), the same operator as the assembled matrix (which the
// assembly forms from the same element matrices), in FP32. It streams the coefficients (4 bytes per
// cell) and p instead of 14 stencil values per row; the p and kappa gathers hit L1/L2. With DIR the
// Dirichlet unit rows and zero columns of the assembled matrix are reproduced.
struct MfOp {
  int nx, ny, nz;       // vertices per axis
  long long py, pz;     // FP32 element offsets of +y, +z (pitched lines)
  float K[64];          // reference element stiffness, K[corner i * 8 + corner j], corner bits (x, y, z)
};

constexpr int MFX = 32, MFY = 8;  // vertex tile of the matrix-free kernel (x, y)

// Vertex columns in registers: a thread owns column (x, y) of a 32 x 8 tile and a chunk of z planes;
// it keeps the 3 x 3 neighbourhood of p in the planes z - 1, z, z + 1 and the 2 x 2 coefficients of
// the cell layers z - 1 and z in registers, so each step loads 9 values of p and 4 coefficients
// (neighbouring threads share them through L1) instead of 27 and 8, with no shared memory and no
// barriers. Values outside the grid (and, with DIR, on the boundary) are 0. A per-row variant (27 + 8
// loads per row) took 35 us at 128^3 and a shared-memory plane-ring variant 40 us (instruction
// bound); this one 30 us (37 us with the Chronopoulos-Gear dots). Unpredicated loads with 0/1 weights
// plus the coefficient-sum form of the product (K[i][j] = f[i ^ j], 35 instead of 72 FP operations)
// measured 38 us and was dropped, and so was a form that keeps only two planes and carries the lower
// layer's contribution (64 registers, four blocks per SM: 38 us; with the next plane's loads issued
// one step ahead, 80 registers: 40 us).
// MODE (what the last block does with the reductions):
//   MF_CG: q = A p with p.q -> alpha (standard CG; the probe check)
//   MF_CGCG_INIT / MF_CGCG / MF_CGCG_REPLACE: w = A z with gamma = r.z, delta = z.w and r.r (the
//   Chronopoulos-Gear form of CG: one reduction phase per iteration), p = the z argument, q = w
enum { MF_CG = 0, MF_CGCG = 1, MF_CGCG_REPLACE = 2, MF_CGCG_INIT = 3 };

template <bool DIR, int MODE>
__global__ void __launch_bounds__(MFX* MFY) k_mf_column(MfOp op, int tiles_x, int tiles_y, int zlen,
                                                       const float* __restrict__ kappa, const float* __restrict__ p,
                                                       float* __restrict__ q, const float* __restrict__ r, MState* st,
                                                       double* partials, unsigned int* ticket,
                                                       cudaGraphConditionalHandle cond) {
  if (mstopped(st)) return;
  // after a residual replacement only (outside graphs the reliable-update kernels run every iteration
  // and exit early when there is nothing to do)
  if (MODE == MF_CGCG_REPLACE && entry_flag(&st->replaced_iter) != entry_flag(&st->iter))
    return;
  const int tx = threadIdx.x % MFX, ty = threadIdx.x / MFX;
  const int bt = blockIdx.x % (tiles_x * tiles_y), bz = blockIdx.x / (tiles_x * tiles_y);
  const int x = (bt % tiles_x) * MFX + tx, y = (bt / tiles_x) * MFY + ty;
  const int zb = bz * zlen, ze = min(op.nz, zb + zlen);
  const int ncx = op.nx - 1, ncy = op.ny - 1, ncz = op.nz - 1;
  const bool active = x < op.nx && y < op.ny;
  // which of the 3 x 3 columns around (x, y) hold values: inside the grid, and with DIR not on the
  // x or y boundary; which of the 2 x 2 cell columns exist
  unsigned colmask = 0u, cellmask = 0u;
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
    for (int dx = -1; dx <= 1; ++dx) {
      const int xx = x + dx, yy = y + dy;
      bool ok = xx >= 0 && yy >= 0 && xx < op.nx && yy < op.ny;
      if (DIR) ok = ok && xx != 0 && yy != 0 && xx != op.nx - 1 && yy != op.ny - 1;
      if (ok) colmask |= 1u << ((dy + 1) * 3 + (dx + 1));
    }
#pragma unroll
  for (int b = 0; b < 2; ++b)
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      const int cx = x - 1 + a, cy = y - 1 + b;
      if (cx >= 0 && cy >= 0 && cx < ncx && cy < ncy) cellmask |= 1u << (b * 2 + a);
    }
  const long long ecol = x + op.py * y;  // element of (x, y, 0)
  const long long kcol = (x - 1) + (long long)ncx * (y - 1);  // cell (x - 1, y - 1, 0)
  auto load_plane = [&](int z, float (&v)[9]) {
    const bool zok = z >= 0 && z < op.nz && !(DIR && (z == 0 || z == op.nz - 1));
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const int dx = k % 3 - 1, dy = k / 3 - 1;
      v[k] = (zok && ((colmask >> k) & 1u)) ? __ldg(p + ecol + dx + op.py * dy + op.pz * z) : 0.f;
    }
  };
  auto load_layer = [&](int c, float (&v)[4]) {
    const bool cok = c >= 0 && c < ncz;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int a = k & 1, b = k >> 1;
      v[k] = (cok && ((cellmask >> k) & 1u)) ? __ldg(kappa + kcol + a + ncx * b + (long long)ncx * ncy * c) : 0.f;
    }
  };
  float pm[9], pc[9], pn[9], km[4], kc[4];
  load_plane(zb - 1, pm);
  load_plane(zb, pc);
  load_layer(zb - 1, km);
  float acc = 0.f, acc1 = 0.f, acc2 = 0.f;
  for (int z = zb; z < ze; ++z) {
    load_plane(z + 1, pn);
    load_layer(z, kc);
    if (active) {
      const long long e = ecol + op.pz * z;
      const bool bnd = x == 0 || y == 0 || z == 0 || x == op.nx - 1 || y == op.ny - 1 || z == op.nz - 1;
      float s, pe;
      if (DIR && bnd) {
        pe = __ldg(p + e);
        s = pe;  // unit row
      } else {
        pe = pc[4];
        s = 0.f;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const int a = c & 1, b = (c >> 1) & 1, cc = c >> 2;
          const float kap = cc ? kc[b * 2 + a] : km[b * 2 + a];
          const int lv = (1 - a) | ((1 - b) << 1) | ((1 - cc) << 2);
          float t = 0.f;
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int jx = j & 1, jy = (j >> 1) & 1, jz = j >> 2;
            const int k = (b + jy) * 3 + (a + jx);
            const float pv = (cc + jz) == 0 ? pm[k] : ((cc + jz) == 1 ? pc[k] : pn[k]);
            t = fmaf(op.K[lv * 8 + j], pv, t);
          }
          s = fmaf(kap, t, s);
        }
      }
      q[e] = s;
      if (MODE == MF_CG) {
        acc = fmaf(pe, s, acc);
      } else {
        const float re = __ldg(r + e);
        acc = fmaf(re, pe, acc);   // gamma = r.z
        acc1 = fmaf(pe, s, acc1);  // delta = z.w
        acc2 = fmaf(re, re, acc2); // r.r
      }
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      pm[k] = pc[k];
      pc[k] = pn[k];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) km[k] = kc[k];
  }
  if constexpr (MODE == MF_CG) {
    double vv[1] = {double(acc)};
    if (grid_reduce<1>(vv, partials, ticket) && threadIdx.x == 0) {
      if (!(vv[0] > 0.0) || !isfinite(vv[0])) {
        st->breakdown = 1;
        st->converged = 1;
      }
      st->alpha = st->rho / vv[0];
    }
  } else {
    double vv[3] = {double(acc), double(acc1), double(acc2)};
    if (grid_reduce<3>(vv, partials, ticket) && threadIdx.x == 0) {
      const double gamma = vv[0], delta = vv[1], rr = vv[2];
      double beta = 0.0, alpha;
      if (MODE == MF_CGCG_INIT) {
        st->gamma_prev = gamma;
        alpha = gamma / delta;
        st->alpha_prev = alpha;
      } else {
        if (MODE == MF_CGCG) {
          st->gamma_prev = st->gamma;
          st->alpha_prev = st->alpha;
        }
        beta = (MODE == MF_CGCG_REPLACE && st->restarting) ? 0.0 : gamma / st->gamma_prev;
        alpha = gamma / (delta - beta * gamma / st->alpha_prev);
      }
      st->gamma = gamma;
      st->beta = beta;
      st->alpha = alpha;
      if (MODE == MF_CGCG) {
        st->iter += 1;
        st->rr = rr;
        st->flag = (rr <= st->drop * st->rr_ref || rr <= st->tol2 * st->rr0 || st->iter >= st->max_iter) ? 1 : 0;
      }
      if (!(delta > 0.0) || !isfinite(alpha) || !isfinite(rr)) {
        st->breakdown = 1;
        st->converged = 1;
      }
      if (MODE == MF_CGCG && cond) cudaGraphSetConditional(cond, (st->flag && !st->converged) ? 1u : 0u);
    }
  }
}

// Chronopoulos-Gear vector update (no reduction): p = z + beta p, s = w + beta s (s = A p),
// x32 += alpha p, r32 -= alpha s, z = dinv r32. Quads of rows; every vector 16-byte aligned.
__global__ void __launch_bounds__(TH) k_cgcg_update(int n4, float4* __restrict__ p, float4* __restrict__ s4,
                                                   float4* __restrict__ x32, float4* __restrict__ r,
                                                   float4* __restrict__ z, const float4* __restrict__ w,
                                                   const float4* __restrict__ dinv, const MState* st) {
  if (mstopped(st)) return;
  const float a = float(st->alpha), b = float(st->beta);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += gridDim.x * blockDim.x) {
    float4 pv = p[k], sv = s4[k], xv = x32[k], rv = r[k];
    const float4 zv = z[k], wv = w[k], dv = dinv[k];
    pv.x = fmaf(b, pv.x, zv.x);
    pv.y = fmaf(b, pv.y, zv.y);
    pv.z = fmaf(b, pv.z, zv.z);
    pv.w = fmaf(b, pv.w, zv.w);
    sv.x = fmaf(b, sv.x, wv.x);
    sv.y = fmaf(b, sv.y, wv.y);
    sv.z = fmaf(b, sv.z, wv.z);
    sv.w = fmaf(b, sv.w, wv.w);
    xv.x = fmaf(a, pv.x, xv.x);
    xv.y = fmaf(a, pv.y, xv.y);
    xv.z = fmaf(a, pv.z, xv.z);
    xv.w = fmaf(a, pv.w, xv.w);
    rv.x = fmaf(-a, sv.x, rv.x);
    rv.y = fmaf(-a, sv.y, rv.y);
    rv.z = fmaf(-a, sv.z, rv.z);
    rv.w = fmaf(-a, sv.w, rv.w);
    p[k] = pv;
    s4[k] = sv;
    x32[k] = xv;
    r[k] = rv;
    z[k] = make_float4(dv.x * rv.x, dv.y * rv.y, dv.z * rv.z, dv.w * rv.w);
  }
}

// probe of the matrix-free operator against the assembled FP64 matrix: v(i) pseudo-random in [-1, 1]
__device__ __forceinline__ double mf_probe(long long i) {
  unsigned long long h = (unsigned long long)i * 0x9E3779B97F4A7C15ull;
  h ^= h >> 29;
  h *= 0xBF58476D1CE4E5B9ull;
  h ^= h >> 32;
  return double(h & 0xFFFFFF) / double(0x800000) - 1.0;
}

__global__ void k_mf_probe(int n, Pitch pt, double* __restrict__ v64, float* __restrict__ v32) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = mf_probe(i);
    v64[i] = v;
    v32[pt.of(i)] = float(v);
  }
}

// err[0] = max |A64 v - q|, err[1] = max |A64 v| (non-negative floats compare as their bit patterns)
template <int G, int PL>
__global__ void __launch_bounds__(TH) k_mf_compare(int n, Pitch pt, const int* __restrict__ rp,
                                                  const int* __restrict__ col, const double* __restrict__ val,
                                                  const double* __restrict__ v64, const float* __restrict__ q,
                                                  unsigned int* err) {
  float md = 0.f, my = 0.f;
  for_rows_csr<G, PL, double>(n, rp, col, val, v64, [&](int row, bool leader, double y) {
    if (leader) {
      md = fmaxf(md, float(fabs(y - double(q[pt.of(row)]))));
      my = fmaxf(my, float(fabs(y)));
    }
  });
  for (int o = 16; o > 0; o >>= 1) {
    md = fmaxf(md, __shfl_xor_sync(0xffffffffu, md, o));
    my = fmaxf(my, __shfl_xor_sync(0xffffffffu, my, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(err, __float_as_uint(md));
    atomicMax(err + 1, __float_as_uint(my));
  }
}

// reliable update, part 1: x64 += x32, x32 = 0
__global__ void __launch_bounds__(TH) k_mx_accumulate(int n, Pitch pt, double* __restrict__ x, float* __restrict__ x32,
                                                     const MState* st) {
  if (mstopped(st) || !entry_flag(&st->flag)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const long long ip = pt.of(i);
    x[i] += double(x32[ip]);
    x32[ip] = 0.f;
  }
}

// reliable update, part 2: r64 = b - A64 x (FP64 CSR), r32 = r64, beta from the replaced residual
template <int G, int PL>
__global__ void __launch_bounds__(TH) k_mx_true_residual(int n, Pitch pt, const int* __restrict__ rp,
                                                        const int* __restrict__ col, const double* __restrict__ val,
                                                        const double* __restrict__ x, const double* __restrict__ b,
                                                        float* __restrict__ r32, const float* __restrict__ dinv,
                                                        MState* st, double* partials, unsigned int* ticket,
                                                        float* __restrict__ z32) {
  if (mstopped(st) || !entry_flag(&st->flag)) return;
  double a0 = 0.0, a1 = 0.0;
  for_rows_csr<G, PL, double>(n, rp, col, val, x, [&](int row, bool leader, double s) {
    if (leader) {
      const double ri = b[row] - s;
      const float rf = float(ri);
      const long long ip = pt.of(row);
      r32[ip] = rf;
      if (z32) z32[ip] = dinv[ip] * rf;  // z = M r for the Chronopoulos-Gear recurrences
      a0 = fma(double(rf), double(dinv[ip] * rf), a0);
      a1 = fma(ri, ri, a1);
    }
  });
  double v[2] = {a0, a1};
  if (grid_reduce<2>(v, partials, ticket) && threadIdx.x == 0) {
    // stagnation guard: a cycle that gained less than 2x on the true residual means the FP32 operator
    // is too far from the FP64 one (cond(A) times its rounding near 1) for the sequence to continue;
    // from then on each replacement restarts the direction and waits for a 1000x drop (restarted
    // FP64 iterative refinement around FP32 CG)
    if (!st->restarting && v[1] > 0.25 * st->rr_ref) {
      st->restarting = 1;
      st->drop = 1e-6;
    }
    st->rr_ref = v[1];
    st->rr = v[1];
    st->beta = st->restarting ? 0.0 : v[0] / st->rho_prev;
    st->rho = v[0];
    st->flag = 0;
    st->updates += 1;
    st->replaced_iter = st->iter;
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
  const int n4 = n >> 2, stride = gridDim.x * blockDim.x;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += stride) {
    float4 pv = reinterpret_cast<const float4*>(p)[k];
    const float4 rv = reinterpret_cast<const float4*>(r)[k];
    const float4 dv = reinterpret_cast<const float4*>(dinv)[k];
    pv.x = fmaf(beta, pv.x, dv.x * rv.x);
    pv.y = fmaf(beta, pv.y, dv.y * rv.y);
    pv.z = fmaf(beta, pv.z, dv.z * rv.z);
    pv.w = fmaf(beta, pv.w, dv.w * rv.w);
    reinterpret_cast<float4*>(p)[k] = pv;
  }
  for (int i = 4 * n4 + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) p[i] = fmaf(beta, p[i], dinv[i] * r[i]);
}

// start: r64 = b - A x (FP64), r32 = r64, p = dinv r32, rho, rr0
template <int G, int PL>
__global__ void __launch_bounds__(TH) k_mx_init(int n, Pitch pt, const int* __restrict__ rp, const int* __restrict__ col,
                                               const double* __restrict__ val, const double* __restrict__ x,
                                               const double* __restrict__ b, float* __restrict__ r32,
                                               const float* __restrict__ dinv, float* __restrict__ p, MState* st,
                                               double* partials, unsigned int* ticket) {
  double a0 = 0.0, a1 = 0.0;
  for_rows_csr<G, PL, double>(n, rp, col, val, x, [&](int row, bool leader, double s) {
    if (leader) {
      const double ri = b[row] - s;
      const float rf = float(ri);
      const long long ip = pt.of(row);
      r32[ip] = rf;
      const float zi = dinv[ip] * rf;
      p[ip] = zi;
      a0 = fma(double(rf), double(zi), a0);
      a1 = fma(ri, ri, a1);
    }
  });
  double v[2] = {a0, a1};
  if (grid_reduce<2>(v, partials, ticket) && threadIdx.x == 0) {
    st->rho = v[0];
    st->rho_prev = v[0];
    st->rr = st->rr0 = st->rr_ref = v[1];
    st->drop = 0.01;
    st->restarting = 0;
    st->replaced_iter = -1;
    st->iter = 0;
    st->flag = 0;
    st->updates = 0;
    st->breakdown = 0;
    st->fault = 0;
    st->converged = (v[1] == 0.0) ? 1 : 0;
  }
}

__global__ void k_diag_inv32(int n, Pitch pt, const int* __restrict__ rp, const int* __restrict__ col,
                             const double* __restrict__ val, float* __restrict__ dinv, int jacobi) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double d = 1.0;
    if (jacobi)
      for (int k = rp[i]; k < rp[i + 1]; ++k)
        if (col[k] == i) d = val[k];
    dinv[pt.of(i)] = float(1.0 / d);
  }
}

// the stencil slots with a positive linear offset of the P1/Q1 vertex stencil of grid g, in vertices
// (coff) and in FP32 elements of lines stored with `pitch` (off)
Stencil make_stencil(const GridDesc& g, long long pitch) {
  Stencil S{};
  const int ns = pow3(g.dim);
  for (int k = 0; k < ns; ++k) {
    if (!slot_in_stencil(g.dim, g.simplex != 0, k)) continue;
    long long o = 0, op = 0, stride = 1, pstride = 1;
    for (int a = 0; a < g.dim; ++a) {
      o += slot_offset(k, a) * stride;
      op += slot_offset(k, a) * pstride;
      stride *= g.vn[a];
      pstride *= a == 0 ? pitch : g.vn[a];
    }
    if (o > 0) {
      S.coff[S.nu] = o;
      S.off[S.nu++] = op;
    }
    if (op > S.pad) S.pad = op;
  }
  S.pad = (S.pad + 3) / 4 * 4;
  return S;
}

// the upper slots of make_stencil (same order) split into in-plane (dz = 0) and out-of-plane
// (dz = +1) lists for k_mx_spmv3d; false where that kernel does not apply
bool make_stencil3(const GridDesc& g, Stencil3& T) {
  T = Stencil3{};
  if (g.dim != 3 || g.vn[0] < 3 || g.vn[1] < 3) return false;  // distinct linear offsets per slot
  if (g.vn[0] > (1LL << 30) || g.vn[1] > (1LL << 30) || g.vn[2] > (1LL << 30)) return false;
  int u = 0;
  for (int k = 0; k < pow3(3); ++k) {
    if (!slot_in_stencil(3, g.simplex != 0, k)) continue;
    const int dx = slot_offset(k, 0), dy = slot_offset(k, 1), dz = slot_offset(k, 2);
    const long long o = dx + g.vn[0] * (dy + g.vn[1] * dz);
    if (o <= 0) continue;
    const int to = dy * TW + dx;
    if (dz == 0) {
      if (T.nin == 4) return false;
      T.in_slot[T.nin] = u;
      T.in_o[T.nin++] = to;
    } else {
      if (T.nup == 9) return false;
      T.up_slot[T.nup] = u;
      T.up_o[T.nup++] = to;
    }
    ++u;
  }
  return (T.nin == 4 && T.nup == 9) || (T.nin == 3 && T.nup == 4);
}

}  // namespace

bool encode_tensor_map_f32(CUtensorMap* map, int rank, void* base, const uint64_t* dims, const uint64_t* strides,
                           const uint32_t* box) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  if (!encode || rank < 1 || rank > 5) return false;
  cuuint64_t gdim[5], gstride[4];
  cuuint32_t bdim[5], estride[5];
  for (int a = 0; a < rank; ++a) {
    gdim[a] = dims[a];
    bdim[a] = box[a];
    estride[a] = 1;
    if (a + 1 < rank) gstride[a] = strides[a];
  }
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, cuuint32_t(rank), base, gdim, gstride, bdim, estride,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool mixed_stencil_supported(gdt_matrix m) {
  return m->test.kind == GDT_SPACE_CG && !m->test.g.mesh && m->rows == m->test.g.nvert && m->max_row > 0 &&
         m->max_row <= 32;
}

gdt_status solve_mixed_stencil(gdt_context ctx, gdt_matrix m, const double* b, double* x, const gdt_solver_opts* o,
                               gdt_solve_info* info, cudaStream_t s) {
  const int n = int(m->rows);
  const GridDesc& g = m->test.g;
  // 3D vertex grids: the TMA-fed plane-tiled SpMV (lines padded to a multiple of 4 elements)
  Stencil3 T3;
  const bool tiled3 = make_stencil3(g, T3);
  const int nx = int(g.vn[0]);
  const long long pitch = tiled3 ? (nx + 3) / 4 * 4 : nx;
  const Pitch pt{nx, int(pitch - nx)};
  const long long np = pitch * (n / nx);  // FP32 elements (vertices + line padding)
  const Stencil S = make_stencil(g, pitch);
  const long long ld = np + 2 * S.pad;  // per-slot array with halos
  const int vec_blocks = std::max(1, std::min(grid_blocks(n, TH), ctx->num_sms * 8));
  const int pvec_blocks = std::max(1, std::min(grid_blocks(np, TH), ctx->num_sms * 8));
  const int quad_blocks = std::max(1, std::min(grid_blocks((np + 3) / 4, TH), ctx->num_sms * 4));
  if (np > INT32_MAX - 4) return fail(ctx, GDT_EUNSUPPORTED, "mixed stencil CG: too many vertices");
  const int npi = int(np);
  int grid3 = 1, zlen = 1;
  size_t smem3 = 0;
  if (tiled3) {
    const int ny = int(g.vn[1]), nz = int(g.vn[2]);
    const size_t smem = T3.nup == 9 ? spmv3d_smem_bytes<4, 9>() : spmv3d_smem_bytes<3, 4>();
    int per_sm = 0;
    cudaError_t oe;
    if (T3.nup == 9) {
      oe = cudaFuncSetAttribute(k_mx_spmv3d<4, 9>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
      if (oe == cudaSuccess)
        oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mx_spmv3d<4, 9>, S3X * S3Y, smem);
    } else {
      oe = cudaFuncSetAttribute(k_mx_spmv3d<3, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
      if (oe == cudaSuccess)
        oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mx_spmv3d<3, 4>, S3X * S3Y, smem);
    }
    if (oe != cudaSuccess) return fail(ctx, GDT_ECUDA, std::string("tiled stencil SpMV: ") + cudaGetErrorString(oe));
    if (per_sm < 1) per_sm = 1;
    // one wave: at most as many (tile, z chunk) blocks as fit on the GPU at once
    const long long tiles = (long long)((nx + S3X - 1) / S3X) * ((ny + S3Y - 1) / S3Y);
    long long zc = std::max(1LL, std::min<long long>(nz, (ctx->num_sms * (long long)per_sm) / tiles));
    zlen = int((nz + zc - 1) / zc);
    zc = (nz + zlen - 1) / zlen;
    if (tiles * zc > kScratchDoubles) return fail(ctx, GDT_EUNSUPPORTED, "grid too large for the tiled stencil SpMV");
    grid3 = int(tiles * zc);
    smem3 = smem;
  }
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
  // every array starts on a 256-byte boundary (16-byte vector accesses, TMA base addresses)
  auto alloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMallocAsync(&p, bytes + 256, s) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return reinterpret_cast<void*>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255));
  };
  // p with zero halos of at least `pad` on both sides; the front halo is a multiple of 64 floats so
  // that p itself starts on a 256-byte boundary
  const long long pfront = (S.pad + 63) / 64 * 64, plen = pfront + np + S.pad;
  float* pfull = (float*)alloc(sizeof(float) * plen);
  float* r32 = (float*)alloc(sizeof(float) * np);
  float* q32 = (float*)alloc(sizeof(float) * np);
  float* x32 = (float*)alloc(sizeof(float) * np);
  float* dinv = (float*)alloc(sizeof(float) * np);
  MState* st = (MState*)alloc(sizeof(MState));
  int* bad = (int*)alloc(sizeof(int));
  if (!pfull || !r32 || !q32 || !x32 || !dinv || !st || !bad) return fail(ctx, GDT_ENOMEM, "mixed solver vectors");
  float* p = pfull + pfront;
  // zero: p (halos and line padding), every FP32 vector (line padding)
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(pfull, 0, sizeof(float) * plen, s));
  for (float* v : {r32, q32, x32, dinv}) GDT_TRY_CUDA(ctx, cudaMemsetAsync(v, 0, sizeof(float) * np, s));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(bad, 0, sizeof(int), s));
  MState init{};
  init.tol2 = o->tol * o->tol;
  init.max_iter = o->max_iter;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(st, &init, sizeof(MState), cudaMemcpyHostToDevice, s));
  // Matrix-free inner operator for 3D Q1 Laplace matrices whose values are exactly their assembly
  // (element coefficients kept at assembly). Every solve checks it against the assembled FP64 matrix
  // with one probe product (relative difference below 1e-4, FP32 rounding is ~1e-6); otherwise the
  // stencil kernels below are used.
  MfOp mfop{};
  bool mf = false;
  int mf_tx = 0, mf_ty = 0, mf_zlen = 0, mf_grid = 0;
  // the operator applied to the halo buffer `p` (which holds z in the Chronopoulos-Gear iteration)
  auto launch_mf = [&](cudaStream_t st_, int mode, cudaGraphConditionalHandle c) {
#define GDT_MF_LAUNCH(D, M)                                                                                 \
  k_mf_column<D, M><<<mf_grid, MFX * MFY, 0, st_>>>(mfop, mf_tx, mf_ty, mf_zlen, m->mf_kappa, p, q32, r32, st, \
                                                    partials, ticket, c)
    if (m->mf_dirichlet) {
      if (mode == MF_CG) GDT_MF_LAUNCH(true, MF_CG);
      else if (mode == MF_CGCG) GDT_MF_LAUNCH(true, MF_CGCG);
      else if (mode == MF_CGCG_REPLACE) GDT_MF_LAUNCH(true, MF_CGCG_REPLACE);
      else GDT_MF_LAUNCH(true, MF_CGCG_INIT);
    } else {
      if (mode == MF_CG) GDT_MF_LAUNCH(false, MF_CG);
      else if (mode == MF_CGCG) GDT_MF_LAUNCH(false, MF_CGCG);
      else if (mode == MF_CGCG_REPLACE) GDT_MF_LAUNCH(false, MF_CGCG_REPLACE);
      else GDT_MF_LAUNCH(false, MF_CGCG_INIT);
    }
#undef GDT_MF_LAUNCH
  };
  if (tiled3 && g.dim == 3 && !g.simplex && m->mf_valid && m->mf_kappa) {
    mfop.nx = nx;
    mfop.ny = int(g.vn[1]);
    mfop.nz = int(g.vn[2]);
    mfop.py = pitch;
    mfop.pz = pitch * g.vn[1];
    for (int k = 0; k < 64; ++k) mfop.K[k] = m->mf_K[k];
    double* v64 = (double*)alloc(sizeof(double) * n);
    unsigned int* err = (unsigned int*)alloc(2 * sizeof(unsigned int));
    if (!v64 || !err) return fail(ctx, GDT_ENOMEM, "mixed solver vectors");
    GDT_TRY_CUDA(ctx, cudaMemsetAsync(err, 0, 2 * sizeof(unsigned int), s));
    GDT_CHECK(ctx, tune_spmv(ctx, m));
    const LaunchShape shc = schedule_shape<double>(m->spmv_sched, n, ctx->num_sms);
    // z sweep shape: (x, y) tiles times z chunks, about one resident wave
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mf_column<true, MF_CGCG>, MFX * MFY, 0) !=
            cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
    cudaGetLastError();
    mf_tx = (mfop.nx + MFX - 1) / MFX;
    mf_ty = (mfop.ny + MFY - 1) / MFY;
    // one resident wave (3 blocks of 256 threads per SM at 73 registers; forcing 4 blocks spilled and
    // was slower, and so were two waves of shorter chunks)
    const long long chunks = std::max(1LL, std::min<long long>(mfop.nz, (long long)ctx->num_sms * per_sm /
                                                                             ((long long)mf_tx * mf_ty)));
    mf_zlen = int((mfop.nz + chunks - 1) / chunks);
    mf_grid = mf_tx * mf_ty * ((mfop.nz + mf_zlen - 1) / mf_zlen);
    if (mf_grid > kScratchDoubles) mf_grid = 0;  // the grid reduction's partials must fit the scratch
    k_mf_probe<<<vec_blocks, TH, 0, s>>>(n, pt, v64, p);
    if (mf_grid > 0) launch_mf(s, MF_CG, 0);
#define GDT_MF_COMPARE(GG, PP) \
  k_mf_compare<GG, PP><<<shc.blocks, shc.threads, shc.smem, s>>>(n, pt, m->rp, m->col, m->val, v64, q32, err)
    GDT_SCHEDULE_SWITCH(m->spmv_sched, GDT_MF_COMPARE)
#undef GDT_MF_COMPARE
    unsigned int herr[2] = {0u, 0u};
    GDT_TRY_CUDA(ctx, cudaMemcpyAsync(herr, err, sizeof(herr), cudaMemcpyDeviceToHost, s));
    GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
    ctx->launches += 3;
    float ed, ey;
    std::memcpy(&ed, &herr[0], sizeof(float));
    std::memcpy(&ey, &herr[1], sizeof(float));
    mf = mf_grid > 0 && ey > 0.f && std::isfinite(ed) && ed <= 1e-4f * ey;
    // restore: p (only the real rows were written), q32 and the solver state
    GDT_TRY_CUDA(ctx, cudaMemsetAsync(pfull, 0, sizeof(float) * plen, s));
    GDT_TRY_CUDA(ctx, cudaMemcpyAsync(st, &init, sizeof(MState), cudaMemcpyHostToDevice, s));
  }
  float* D = nullptr;
  if (!mf) {
    D = (float*)alloc(sizeof(float) * ld * (S.nu + 1));
    if (!D) return fail(ctx, GDT_ENOMEM, "mixed solver vectors");
    GDT_TRY_CUDA(ctx, cudaMemsetAsync(D, 0, sizeof(float) * ld * (S.nu + 1), s));
    k_build_stencil<<<vec_blocks, TH, 0, s>>>(n, m->rp, m->col, m->val, S, pt, D, ld, bad);
    ctx->launches++;
  }
  k_diag_inv32<<<vec_blocks, TH, 0, s>>>(n, pt, m->rp, m->col, m->val, dinv, o->precond == GDT_PREC_JACOBI);
  ctx->launches++;
  // tensor maps of the tiled SpMV: slot arrays (x, y, z, slot) and p (x, y, z), boxes of 40 x 10 x 1 (x 1)
  CUtensorMap tmD{}, tmP{};
  if (tiled3 && !mf) {
    const uint64_t ny = uint64_t(g.vn[1]), nz = uint64_t(g.vn[2]);
    const uint64_t dimsD[4] = {uint64_t(nx), ny, nz, uint64_t(S.nu + 1)};
    const uint64_t strD[3] = {4ull * pitch, 4ull * pitch * ny, 4ull * ld};
    const uint32_t boxD[4] = {TW, TR, 1, 1};
    const uint64_t dimsP[3] = {uint64_t(nx), ny, nz};
    const uint64_t strP[2] = {4ull * pitch, 4ull * pitch * ny};
    const uint32_t boxP[3] = {TW, TR, 1};
    if (!encode_tensor_map_f32(&tmD, 4, D + S.pad, dimsD, strD, boxD) ||
        !encode_tensor_map_f32(&tmP, 3, p, dimsP, strP, boxP))
      return fail(ctx, GDT_ECUDA, "tiled stencil SpMV: tensor map encoding failed");
  }
  GDT_CHECK(ctx, tune_spmv(ctx, m));
  const LaunchShape sh = schedule_shape<double>(m->spmv_sched, n, ctx->num_sms);
#define GDT_MX_INIT(GG, PP)                                                                                  \
  k_mx_init<GG, PP><<<sh.blocks, sh.threads, sh.smem, s>>>(n, pt, m->rp, m->col, m->val, x, b, r32, dinv, p, st, \
                                                           partials, ticket)
#define GDT_MX_TRUE_RESIDUAL(GG, PP)                                                                             \
  k_mx_true_residual<GG, PP><<<sh.blocks, sh.threads, sh.smem, cstream>>>(n, pt, m->rp, m->col, m->val, x, b, r32, \
                                                                          dinv, st, partials, ticket, mf ? p : nullptr)
  GDT_SCHEDULE_SWITCH(m->spmv_sched, GDT_MX_INIT)
  ctx->launches++;
  // Chronopoulos-Gear form on the matrix-free path (one reduction phase per iteration): the halo
  // buffer p holds z = M r (written by the init kernel), pd the search direction, s32 = A pd, q32 = A z
  float* pd = nullptr;
  float* s32 = nullptr;
  if (mf) {
    pd = (float*)alloc(sizeof(float) * np);
    s32 = (float*)alloc(sizeof(float) * np);
    if (!pd || !s32) return fail(ctx, GDT_ENOMEM, "mixed solver vectors");
    GDT_TRY_CUDA(ctx, cudaMemsetAsync(pd, 0, sizeof(float) * np, s));
    GDT_TRY_CUDA(ctx, cudaMemsetAsync(s32, 0, sizeof(float) * np, s));
    launch_mf(s, MF_CGCG_INIT, 0);
    ctx->launches++;
  }
  // FP32 stencil SpMV of this matrix: on 3D grids the TMA-tiled and the linear kernel are timed
  // once (CUDA events, one warm-up and three launches each; they only rewrite q32 and alpha, which
  // the first iteration recomputes) and the faster is kept for the matrix
  auto launch_linear = [&](cudaStream_t st_) {
    switch (S.nu) {
      case 1: k_mx_spmv<1><<<pvec_blocks, TH, 0, st_>>>(npi, S, D, ld, p, q32, st, partials, ticket); break;
      case 3: k_mx_spmv<3><<<pvec_blocks, TH, 0, st_>>>(npi, S, D, ld, p, q32, st, partials, ticket); break;
      case 4: k_mx_spmv<4><<<pvec_blocks, TH, 0, st_>>>(npi, S, D, ld, p, q32, st, partials, ticket); break;
      case 7: k_mx_spmv<7><<<pvec_blocks, TH, 0, st_>>>(npi, S, D, ld, p, q32, st, partials, ticket); break;
      default: k_mx_spmv<13><<<pvec_blocks, TH, 0, st_>>>(npi, S, D, ld, p, q32, st, partials, ticket); break;
    }
  };
  auto launch_tiled = [&](cudaStream_t st_) {
    const int ny = int(g.vn[1]), nz = int(g.vn[2]);
    if (T3.nup == 9)
      k_mx_spmv3d<4, 9><<<grid3, S3X * S3Y, smem3, st_>>>(nx, ny, nz, zlen, pitch, T3, tmD, tmP, D + S.pad, q32, st,
                                                          partials, ticket);
    else
      k_mx_spmv3d<3, 4><<<grid3, S3X * S3Y, smem3, st_>>>(nx, ny, nz, zlen, pitch, T3, tmD, tmP, D + S.pad, q32, st,
                                                          partials, ticket);
  };
  if (tiled3 && !mf && m->mx_tiled < 0) {
    cudaEvent_t e0, e1, e2;
    float t_lin = 0.f, t_til = 0.f;
    bool ok = cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess &&
              cudaEventCreate(&e2) == cudaSuccess;
    if (ok) {
      launch_linear(s);
      launch_tiled(s);
      cudaEventRecord(e0, s);
      for (int k = 0; k < 3; ++k) launch_linear(s);
      cudaEventRecord(e1, s);
      for (int k = 0; k < 3; ++k) launch_tiled(s);
      cudaEventRecord(e2, s);
      ok = cudaEventSynchronize(e2) == cudaSuccess && cudaEventElapsedTime(&t_lin, e0, e1) == cudaSuccess &&
           cudaEventElapsedTime(&t_til, e1, e2) == cudaSuccess;
      ctx->launches += 8;
      MState chk;
      if (ok && cudaMemcpy(&chk, st, sizeof(MState), cudaMemcpyDeviceToHost) == cudaSuccess) {
        if (chk.fault) return fail(ctx, GDT_ETIMEOUT, "tiled stencil SpMV: a tile-load wait ran out");
        if (!chk.converged) m->mx_tiled = t_til < t_lin ? 1 : 0;  // a converged start times early exits
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, GDT_ECUDA, std::string("stencil SpMV timing: ") + cudaGetErrorString(e));
  }
  const bool use_tiled = tiled3 && m->mx_tiled == 1;
  m->mx_operator = mf ? GDT_MIXED_OPERATOR_MATRIX_FREE
                      : (use_tiled ? GDT_MIXED_OPERATOR_STENCIL_TILED : GDT_MIXED_OPERATOR_STENCIL);
  const int chunk = o->check_every > 0 ? o->check_every : 32;
  // per iteration: SpMV, update, [reliable update: accumulate + true residual], direction. In graphs
  // the reliable update is the body of an IF node set by the update kernel, so the ~97 % of
  // iterations without one launch three kernels.
  bool graphed = false;
  cudaStream_t cstream = s;
  GDT_CHECK(ctx, iterate_chunks_cond(ctx, s, &st->converged, chunk, o->max_iter / chunk + 2, &graphed,
                                     [&](CondSection& cs) {
    const cudaGraphConditionalHandle cond = cs.next_handle();
    if (mf) {
      // update (no reduction), operator + the three dots (alpha, beta, replacement test), [reliable
      // update: accumulate, true residual and z, operator again for the replaced residual]
      timing_begin(ctx, s, GDT_TIMING_CG_UPDATE);
      k_cgcg_update<<<quad_blocks, TH, 0, s>>>(npi / 4, reinterpret_cast<float4*>(pd), reinterpret_cast<float4*>(s32),
                                               reinterpret_cast<float4*>(x32), reinterpret_cast<float4*>(r32),
                                               reinterpret_cast<float4*>(p), reinterpret_cast<const float4*>(q32),
                                               reinterpret_cast<const float4*>(dinv), st);
      timing_end(ctx, s);
      timing_begin(ctx, s, GDT_TIMING_SPMV_FP32);
      launch_mf(s, MF_CGCG, cond);
      timing_end(ctx, s);
      timing_begin(ctx, s, GDT_TIMING_RELIABLE_UPDATE);
      cstream = cs.begin(cond);
      k_mx_accumulate<<<vec_blocks, TH, 0, cstream>>>(n, pt, x, x32, st);
      GDT_SCHEDULE_SWITCH(m->spmv_sched, GDT_MX_TRUE_RESIDUAL)
      launch_mf(cstream, MF_CGCG_REPLACE, 0);
      cs.end();
      timing_end(ctx, s);
      ctx->launches += cs.capturing ? 2 : 5;  // captured IF bodies are counted when they ran (below)
      return;
    }
    timing_begin(ctx, s, GDT_TIMING_SPMV_FP32);
    if (use_tiled) launch_tiled(s);
    else launch_linear(s);
    timing_end(ctx, s);
    timing_begin(ctx, s, GDT_TIMING_CG_UPDATE);
    k_mx_update<<<quad_blocks, TH, 0, s>>>(npi, x32, p, r32, q32, dinv, st, partials, ticket, cond);
    timing_end(ctx, s);
    timing_begin(ctx, s, GDT_TIMING_RELIABLE_UPDATE);
    cstream = cs.begin(cond);
    k_mx_accumulate<<<vec_blocks, TH, 0, cstream>>>(n, pt, x, x32, st);
    GDT_SCHEDULE_SWITCH(m->spmv_sched, GDT_MX_TRUE_RESIDUAL)
    cs.end();
    timing_end(ctx, s);
    timing_begin(ctx, s, GDT_TIMING_CG_DIRECTION);
    k_mx_p<<<quad_blocks, TH, 0, s>>>(npi, p, r32, dinv, st);
    timing_end(ctx, s);
    ctx->launches += cs.capturing ? 3 : 5;  // captured IF bodies are counted when they ran (below)
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
  if (fin.fault) return fail(ctx, GDT_ETIMEOUT, "tiled stencil SpMV: a tile-load wait ran out");
  if (graphed) ctx->launches += (mf ? 3LL : 2LL) * fin.updates;
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
