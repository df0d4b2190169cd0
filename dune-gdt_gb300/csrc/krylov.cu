// Device-resident Krylov solvers behind ConstMatrixOperator::apply_inverse
// (operators/matrix-based.hh:131-159). The reference hands this to dune-istl through dune-xt-la
// (third-party, absent from the reference tree); the algorithms restated here are the published
// ones: preconditioned CG (Hestenes-Stiefel), BiCGStab (van der Vorst 1992), Jacobi and ILU(0).
//
// GB300 design: all scalars (rho, alpha, beta, omega, residual norms, iteration count, converged
// flag) live in device memory; every reduction finishes in the last block of its kernel (ticketed,
// fixed summation order: deterministic), so an iteration issues no host synchronisation. Iterations
// are captured into a CUDA graph in chunks of `check_every`; the host reads the converged flag once
// per chunk, and kernels of iterations past convergence return immediately. FP64 CG with Jacobi or
// no preconditioner on rows of at most 32 entries instead runs all its iterations in one persistent
// cooperative launch (k_pcg_persistent below).
// Mixed precision: FP32 inner CG (FP32 CSR values, FP32 vectors, FP32 Jacobi) inside FP64
// iterative refinement with an FP64 residual r = b - A x from the FP64 matrix.
#include <cfloat>
#include <cmath>
#include <vector>

#include "linalg.cuh"

namespace gdt {

namespace {

constexpr int TH = 256;

struct KState {
  double rho, alpha, beta, omega, rr, rr0, tol2, hden;
  int iter, max_iter, converged, breakdown;
};

__device__ __forceinline__ bool stopped(const KState* st) { return entry_flag(&st->converged) != 0; }

// ---------------------------------------------------------------- generic pieces ---
// y = A x; optional dot(w, y) -> st->hden / alpha (mode 1: CG alpha = rho / (p.Ap); mode 2: BiCGStab
// alpha = rho / (rt.v); mode 3: two dots (t.s, t.t) -> omega)
template <int G, int PL, class T, int MODE>
__global__ void __launch_bounds__(TH) k_spmv(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                            const T* __restrict__ val, const T* __restrict__ x, T* __restrict__ y,
                                            const T* __restrict__ w, KState* st, double* partials,
                                            unsigned int* ticket) {
  if (stopped(st)) return;
  T a0 = T(0), a1 = T(0);
  if constexpr (MODE == 0) {
    for_rows_csr<G, PL, T>(n, rp, col, val, x, [&](int row, bool leader, T s) {
      if (leader) y[row] = s;
    });
    return;
  } else {
    // the dot partner of row `row` (x for CG's p.Ap, w otherwise) is prefetched with the row bounds
    for_rows_csr_w<G, PL, T>(n, rp, col, val, x, MODE == 1 ? x : w, [&](int row, bool leader, T s, T wr) {
      if (leader) {
        y[row] = s;
        if (MODE == 1 || MODE == 2) a0 = fma(wr, s, a0);
        if (MODE == 3) {
          a0 = fma(s, wr, a0);
          a1 = fma(s, s, a1);
        }
      }
    });
  }
  double v[2] = {double(a0), double(a1)};
  if (grid_reduce<2>(v, partials, ticket) && threadIdx.x == 0) {
    if (MODE == 1) {
      if (!(v[0] > 0.0) || !isfinite(v[0])) {
        st->breakdown = 1;
        st->converged = 1;
      }
      st->alpha = st->rho / v[0];
    } else if (MODE == 2) {
      if (v[0] == 0.0 || !isfinite(v[0])) {
        st->breakdown = 1;
        st->converged = 1;
      }
      st->alpha = st->rho / v[0];
    } else {
      if (v[1] == 0.0 || !isfinite(v[1])) {
        st->breakdown = 1;
        st->converged = 1;
      }
      st->omega = v[0] / v[1];
    }
  }
}

// q = A p on the SELL-32 copy with p.q -> alpha: the graph-form CG SpMV where the SELL schedule
// was tuned fastest inside the iteration (or pinned)
__global__ void __launch_bounds__(256) k_sell_spmv_cg(SellView A, const double* __restrict__ p,
                                                      double* __restrict__ q, KState* st, double* partials,
                                                      unsigned int* ticket) {
  if (stopped(st)) return;
  double a0 = 0.0;
  for_slices<true>(
      A, p,
      [&](int row, bool active, double s, double pr) {
        if (active) {
          q[row] = s;
          a0 = fma(pr, s, a0);
        }
      },
      p);
  double v[1] = {a0};
  if (grid_reduce<1>(v, partials, ticket) && threadIdx.x == 0) {
    if (!(v[0] > 0.0) || !isfinite(v[0])) {
      st->breakdown = 1;
      st->converged = 1;
    }
    st->alpha = st->rho / v[0];
  }
}

// r = b - A x, z = M^{-1} r (Jacobi if dinv, else z = r), p = z (CG start); rho = r.z, rr0 = r.r
template <int G, int PL, class T>
__global__ void __launch_bounds__(TH) k_residual_init(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                     const T* __restrict__ val, const T* __restrict__ x,
                                                     const T* __restrict__ b, T* __restrict__ r,
                                                     const T* __restrict__ dinv, T* __restrict__ p,
                                                     KState* st, double* partials, unsigned int* ticket) {
  T a0 = T(0), a1 = T(0);
  for_rows_csr<G, PL, T>(n, rp, col, val, x, [&](int row, bool leader, T s) {
    if (leader) {
      T ri = b[row] - s;
      r[row] = ri;
      T zi = dinv ? dinv[row] * ri : ri;
      if (p) p[row] = zi;
      a0 = fma(ri, zi, a0);
      a1 = fma(ri, ri, a1);
    }
  });
  double v[2] = {double(a0), double(a1)};
  if (grid_reduce<2>(v, partials, ticket) && threadIdx.x == 0) {
    st->rho = v[0];
    st->rr = v[1];
    st->rr0 = v[1];
    st->iter = 0;
    st->breakdown = 0;
    st->alpha = st->beta = st->omega = 1.0;
    st->converged = (v[1] == 0.0 || v[1] <= st->tol2 * v[1]) ? 1 : 0;
    if (!isfinite(v[1])) {
      st->breakdown = 1;
      st->converged = 1;
    }
  }
}

// x0 = 0 start of the inner FP32 solve: r holds b already; p = dinv r; rho = r.p, rr0 = r.r
template <class T>
__global__ void __launch_bounds__(TH) k_init_from_rhs(int n, const T* __restrict__ r, const T* __restrict__ dinv,
                                                     T* __restrict__ p, KState* st, double* partials,
                                                     unsigned int* ticket) {
  T a0 = T(0), a1 = T(0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    T ri = r[i];
    T zi = dinv[i] * ri;
    p[i] = zi;
    a0 = fma(ri, zi, a0);
    a1 = fma(ri, ri, a1);
  }
  double v[2] = {double(a0), double(a1)};
  if (grid_reduce<2>(v, partials, ticket) && threadIdx.x == 0) {
    st->rho = v[0];
    st->rr = v[1];
    st->rr0 = v[1];
    st->iter = 0;
    st->breakdown = 0;
    st->alpha = st->beta = st->omega = 1.0;
    st->converged = (v[1] == 0.0) ? 1 : 0;
  }
}

// CG with Jacobi, fused: x += alpha p; r -= alpha q; z = dinv r (not stored); rho' = r.z, rr = r.r
template <class TX, class T>
__global__ void __launch_bounds__(TH) k_cg_update_jacobi(int n, TX* __restrict__ x, const T* __restrict__ p,
                                                        T* __restrict__ r, const T* __restrict__ q,
                                                        const T* __restrict__ dinv, KState* st, double* partials,
                                                        unsigned int* ticket) {
  if (stopped(st)) return;
  const T alpha = T(st->alpha);
  T a0 = T(0), a1 = T(0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = TX(fma(alpha, p[i], T(x[i])));
    T ri = fma(-alpha, q[i], r[i]);
    r[i] = ri;
    a0 = fma(ri, dinv[i] * ri, a0);
    a1 = fma(ri, ri, a1);
  }
  double v[2] = {double(a0), double(a1)};
  if (grid_reduce<2>(v, partials, ticket) && threadIdx.x == 0) {
    st->beta = v[0] / st->rho;
    st->rho = v[0];
    st->rr = v[1];
    st->iter += 1;
    if (v[1] <= st->tol2 * st->rr0 || st->iter >= st->max_iter) st->converged = 1;
    if (!isfinite(v[1])) {
      st->breakdown = 1;
      st->converged = 1;
    }
  }
}

// The same two FP64 kernels on pairs of rows (16-byte loads and stores, twice the bytes in flight
// per instruction); for vectors that all start on a 16-byte boundary. The odd last row, if any, is
// done by the first thread of the grid.
__global__ void __launch_bounds__(TH) k_cg_update_jacobi2(int n, double* __restrict__ x, const double* __restrict__ p,
                                                         double* __restrict__ r, const double* __restrict__ q,
                                                         const double* __restrict__ dinv, KState* st,
                                                         double* partials, unsigned int* ticket) {
  if (stopped(st)) return;
  const double alpha = st->alpha;
  double a0 = 0.0, a1 = 0.0;
  const int n2 = n >> 1;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n2; k += gridDim.x * blockDim.x) {
    double2 xv = reinterpret_cast<const double2*>(x)[k], rv = reinterpret_cast<const double2*>(r)[k];
    const double2 pv = reinterpret_cast<const double2*>(p)[k], qv = reinterpret_cast<const double2*>(q)[k],
                  dv = reinterpret_cast<const double2*>(dinv)[k];
    xv.x = fma(alpha, pv.x, xv.x);
    xv.y = fma(alpha, pv.y, xv.y);
    rv.x = fma(-alpha, qv.x, rv.x);
    rv.y = fma(-alpha, qv.y, rv.y);
    a0 = fma(rv.x, dv.x * rv.x, a0);
    a1 = fma(rv.x, rv.x, a1);
    a0 = fma(rv.y, dv.y * rv.y, a0);
    a1 = fma(rv.y, rv.y, a1);
    reinterpret_cast<double2*>(x)[k] = xv;
    reinterpret_cast<double2*>(r)[k] = rv;
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const int i = n - 1;
    x[i] = fma(alpha, p[i], x[i]);
    const double ri = fma(-alpha, q[i], r[i]);
    r[i] = ri;
    a0 = fma(ri, dinv[i] * ri, a0);
    a1 = fma(ri, ri, a1);
  }
  double v[2] = {a0, a1};
  if (grid_reduce<2>(v, partials, ticket) && threadIdx.x == 0) {
    st->beta = v[0] / st->rho;
    st->rho = v[0];
    st->rr = v[1];
    st->iter += 1;
    if (v[1] <= st->tol2 * st->rr0 || st->iter >= st->max_iter) st->converged = 1;
    if (!isfinite(v[1])) {
      st->breakdown = 1;
      st->converged = 1;
    }
  }
}

__global__ void __launch_bounds__(TH) k_cg_p_jacobi2(int n, double* __restrict__ p, const double* __restrict__ r,
                                                    const double* __restrict__ dinv, const KState* st) {
  if (stopped(st)) return;
  const double beta = st->beta;
  const int n2 = n >> 1;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n2; k += gridDim.x * blockDim.x) {
    double2 pv = reinterpret_cast<const double2*>(p)[k];
    const double2 rv = reinterpret_cast<const double2*>(r)[k], dv = reinterpret_cast<const double2*>(dinv)[k];
    pv.x = fma(beta, pv.x, dv.x * rv.x);
    pv.y = fma(beta, pv.y, dv.y * rv.y);
    reinterpret_cast<double2*>(p)[k] = pv;
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) p[n - 1] = fma(beta, p[n - 1], dinv[n - 1] * r[n - 1]);
}

template <class T>
__global__ void __launch_bounds__(TH) k_cg_p_jacobi(int n, T* __restrict__ p, const T* __restrict__ r,
                                                   const T* __restrict__ dinv, const KState* st) {
  if (stopped(st)) return;
  const T beta = T(st->beta);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = fma(beta, p[i], dinv[i] * r[i]);
}

// generic CG (any preconditioner): x += alpha p; r -= alpha q; rr = r.r
__global__ void __launch_bounds__(TH) k_cg_update(int n, double* __restrict__ x, const double* __restrict__ p,
                                                 double* __restrict__ r, const double* __restrict__ q, KState* st,
                                                 double* partials, unsigned int* ticket) {
  if (stopped(st)) return;
  const double alpha = st->alpha;
  double a0 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    double ri = fma(-alpha, q[i], r[i]);
    r[i] = ri;
    a0 = fma(ri, ri, a0);
  }
  double v[1] = {a0};
  if (grid_reduce<1>(v, partials, ticket) && threadIdx.x == 0) {
    st->rr = v[0];
    st->iter += 1;
    if (v[0] <= st->tol2 * st->rr0 || st->iter >= st->max_iter) st->converged = 1;
    if (!isfinite(v[0])) {
      st->breakdown = 1;
      st->converged = 1;
    }
  }
}

// rho' = r.z, beta = rho'/rho (CG)
__global__ void __launch_bounds__(TH) k_cg_beta(int n, const double* __restrict__ r, const double* __restrict__ z,
                                               KState* st, double* partials, unsigned int* ticket) {
  if (stopped(st)) return;
  double a0 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a0 = fma(r[i], z[i], a0);
  double v[1] = {a0};
  if (grid_reduce<1>(v, partials, ticket) && threadIdx.x == 0) {
    st->beta = v[0] / st->rho;
    st->rho = v[0];
  }
}

__global__ void __launch_bounds__(TH) k_cg_p(int n, double* __restrict__ p, const double* __restrict__ z,
                                            const KState* st) {
  if (stopped(st)) return;
  const double beta = st->beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = fma(beta, p[i], z[i]);
}

// ---------------------------------------------------------------- BiCGStab pieces ---
// rho' = rt.r ; beta = (rho'/rho)(alpha/omega) ; p = r + beta (p - omega v) (first iteration: p = r)
__global__ void __launch_bounds__(TH) k_bicg_rho(int n, const double* __restrict__ rt, const double* __restrict__ r,
                                                KState* st, double* partials, unsigned int* ticket) {
  if (stopped(st)) return;
  double a0 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a0 = fma(rt[i], r[i], a0);
  double v[1] = {a0};
  if (grid_reduce<1>(v, partials, ticket) && threadIdx.x == 0) {
    if (v[0] == 0.0 || !isfinite(v[0])) {
      st->breakdown = 1;
      st->converged = 1;
    }
    st->beta = (st->iter == 0) ? 0.0 : (v[0] / st->rho) * (st->alpha / st->omega);
    st->rho = v[0];
  }
}

__global__ void __launch_bounds__(TH) k_bicg_p(int n, double* __restrict__ p, const double* __restrict__ r,
                                              const double* __restrict__ v, const KState* st) {
  if (stopped(st)) return;
  const double beta = st->beta, omega = st->omega;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = fma(beta, fma(-omega, v[i], p[i]), r[i]);
}

// x += alpha y ; s = r - alpha v ; check ||s|| (if converged: r = s)
__global__ void __launch_bounds__(TH) k_bicg_s(int n, double* __restrict__ x, const double* __restrict__ y,
                                              double* __restrict__ r, const double* __restrict__ v, KState* st,
                                              double* partials, unsigned int* ticket) {
  if (stopped(st)) return;
  const double alpha = st->alpha;
  double a0 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = fma(alpha, y[i], x[i]);
    double si = fma(-alpha, v[i], r[i]);
    r[i] = si;  // r now holds s
    a0 = fma(si, si, a0);
  }
  double w[1] = {a0};
  if (grid_reduce<1>(w, partials, ticket) && threadIdx.x == 0) {
    st->rr = w[0];
    if (w[0] <= st->tol2 * st->rr0) {
      st->iter += 1;
      st->converged = 1;
    }
  }
}

// x += omega z ; r = s - omega t ; rr
__global__ void __launch_bounds__(TH) k_bicg_r(int n, double* __restrict__ x, const double* __restrict__ z,
                                              double* __restrict__ r, const double* __restrict__ t, KState* st,
                                              double* partials, unsigned int* ticket) {
  if (stopped(st)) return;
  const double omega = st->omega;
  double a0 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = fma(omega, z[i], x[i]);
    double ri = fma(-omega, t[i], r[i]);
    r[i] = ri;
    a0 = fma(ri, ri, a0);
  }
  double w[1] = {a0};
  if (grid_reduce<1>(w, partials, ticket) && threadIdx.x == 0) {
    st->rr = w[0];
    st->iter += 1;
    if (w[0] <= st->tol2 * st->rr0 || st->iter >= st->max_iter) st->converged = 1;
    if (!isfinite(w[0])) {
      st->breakdown = 1;
      st->converged = 1;
    }
  }
}

// ------------------------------------------------------------------- preconditioners ---
template <class TD, class TS>
__global__ void k_jacobi_diag(int n, const int* __restrict__ rp, const int* __restrict__ col,
                              const TS* __restrict__ val, TD* __restrict__ dinv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    TS d = TS(0);
    for (int k = rp[i]; k < rp[i + 1]; ++k)
      if (col[k] == i) d = val[k];
    dinv[i] = TD(1.0 / double(d));
  }
}

template <class T>
__global__ void k_scale(int n, T* __restrict__ z, const T* __restrict__ d, const T* __restrict__ r, const KState* st) {
  if (stopped(st)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) z[i] = d ? d[i] * r[i] : r[i];
}

// ILU(0), level scheduled: rows of one level depend only on rows of earlier levels.
__global__ void k_ilu_factor_level(const int* __restrict__ rows, int count, const int* __restrict__ rp,
                                   const int* __restrict__ col, const int* __restrict__ diag, double* __restrict__ lu) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = rows[t];
  const int end_i = rp[i + 1];
  for (int pk = rp[i]; pk < end_i; ++pk) {
    const int k = col[pk];
    if (k >= i) break;
    const double lik = lu[pk] / lu[diag[k]];
    lu[pk] = lik;
    int pi = pk + 1;
    for (int pj = diag[k] + 1; pj < rp[k + 1]; ++pj) {
      const int j = col[pj];
      while (pi < end_i && col[pi] < j) ++pi;
      if (pi < end_i && col[pi] == j) lu[pi] -= lik * lu[pj];
    }
  }
}

__global__ void k_ilu_lower_level(const int* __restrict__ rows, int count, const int* __restrict__ rp,
                                  const int* __restrict__ col, const int* __restrict__ diag,
                                  const double* __restrict__ lu, const double* __restrict__ r, double* __restrict__ z,
                                  const KState* st) {
  if (stopped(st)) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = rows[t];
  double s = r[i];
  for (int p = rp[i]; p < diag[i]; ++p) s -= lu[p] * z[col[p]];
  z[i] = s;
}

__global__ void k_ilu_upper_level(const int* __restrict__ rows, int count, const int* __restrict__ rp,
                                  const int* __restrict__ col, const int* __restrict__ diag,
                                  const double* __restrict__ lu, double* __restrict__ z, const KState* st) {
  if (stopped(st)) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = rows[t];
  double s = z[i];
  for (int p = diag[i] + 1; p < rp[i + 1]; ++p) s -= lu[p] * z[col[p]];
  z[i] = s / lu[diag[i]];
}

__global__ void k_find_diag(int n, const int* __restrict__ rp, const int* __restrict__ col, int* __restrict__ diag) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int d = -1;
    for (int k = rp[i]; k < rp[i + 1]; ++k)
      if (col[k] == i) d = k;
    diag[i] = d;
  }
}

// -------------------------------------------------------------- mixed precision helpers ---
__global__ void k_to_float(long long n, const double* __restrict__ a, float* __restrict__ b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = float(a[i]);
}

// r64 = b - A x (FP64) ; rr = r.r ; r32 = r64 * inv_scale where inv_scale = 1/||r|| is applied on the host side
template <int G, int PL>
__global__ void __launch_bounds__(TH) k_residual64(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                  const double* __restrict__ val, const double* __restrict__ x,
                                                  const double* __restrict__ b, double* __restrict__ r,
                                                  double* out_rr, double* partials, unsigned int* ticket) {
  double a0 = 0.0;
  for_rows_csr<G, PL, double>(n, rp, col, val, x, [&](int row, bool leader, double s) {
    if (leader) {
      double ri = b[row] - s;
      r[row] = ri;
      a0 = fma(ri, ri, a0);
    }
  });
  double v[1] = {a0};
  if (grid_reduce<1>(v, partials, ticket) && threadIdx.x == 0) *out_rr = v[0];
}

__global__ void k_scale_to_float(int n, const double* __restrict__ r, const double* __restrict__ rr,
                                 float* __restrict__ r32) {
  const double inv = 1.0 / sqrt(*rr);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) r32[i] = float(r[i] * inv);
}

__global__ void k_correct(int n, double* __restrict__ x, const float* __restrict__ d, const double* __restrict__ rr) {
  const double scale = sqrt(*rr);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] = fma(scale, double(d[i]), x[i]);
}

// ---------------------------------------------------------------------------- host ---
struct Launch {
  gdt_context ctx;
  int n;
  int sched;
  int vec_blocks;
  cudaStream_t s;
  double* partials;
  unsigned int* ticket;
  template <class T>
  LaunchShape shape() const {
    return schedule_shape<T>(sched, n, ctx->num_sms);
  }
};

// the graph-form CG SpMV (q = A p, alpha) on the SELL-32 copy
void spmv_cg_sell(const Launch& L, gdt_matrix m, const double* p, double* q, KState* st) {
  const SellView A = sell_view(m);
  timing_begin(L.ctx, L.s, GDT_TIMING_SPMV_FP64);
  k_sell_spmv_cg<<<sell_blocks(A.nslices, L.ctx->num_sms, reinterpret_cast<const void*>(&k_sell_spmv_cg)), 256, 0,
                   L.s>>>(A, p, q, st, L.partials, L.ticket);
  timing_end(L.ctx, L.s);
  L.ctx->launches++;
}

template <class T, int MODE>
void spmv_mode(const Launch& L, const int* rp, const int* col, const T* val, const T* x, T* y, const T* w,
               KState* st) {
  const LaunchShape sh = L.shape<T>();
  timing_begin(L.ctx, L.s, sizeof(T) == 8 ? GDT_TIMING_SPMV_FP64 : GDT_TIMING_SPMV_FP32);
#define GDT_K_SPMV(GG, PP) \
  k_spmv<GG, PP, T, MODE><<<sh.blocks, sh.threads, sh.smem, L.s>>>(L.n, rp, col, val, x, y, w, st, L.partials, L.ticket)
  GDT_SCHEDULE_SWITCH(L.sched, GDT_K_SPMV)
#undef GDT_K_SPMV
  timing_end(L.ctx, L.s);
  L.ctx->launches++;
}

template <class T>
void residual_init(const Launch& L, const int* rp, const int* col, const T* val, const T* x, const T* b, T* r,
                   const T* dinv, T* p, KState* st) {
  const LaunchShape sh = L.shape<T>();
#define GDT_K_RESINIT(GG, PP)                                                                                    \
  k_residual_init<GG, PP, T><<<sh.blocks, sh.threads, sh.smem, L.s>>>(L.n, rp, col, val, x, b, r, dinv, p, st, \
                                                                      L.partials, L.ticket)
  GDT_SCHEDULE_SWITCH(L.sched, GDT_K_RESINIT)
#undef GDT_K_RESINIT
  L.ctx->launches++;
}

void residual64(const Launch& L, gdt_matrix m, const double* x, const double* b, double* r, double* rr) {
  const LaunchShape sh = L.shape<double>();
#define GDT_K_RES64(GG, PP)                                                                                      \
  k_residual64<GG, PP><<<sh.blocks, sh.threads, sh.smem, L.s>>>(L.n, m->rp, m->col, m->val, x, b, r, rr, L.partials, \
                                                                L.ticket)
  GDT_SCHEDULE_SWITCH(L.sched, GDT_K_RES64)
#undef GDT_K_RES64
  L.ctx->launches++;
}

// level sets of the lower (U = false) or upper (U = true) triangle, computed on the host from the pattern
void level_sets(int n, const std::vector<int>& rp, const std::vector<int>& col, bool upper, std::vector<int>& order,
                std::vector<int>& offsets) {
  std::vector<int> lev(n, 0);
  int maxl = 0;
  if (!upper) {
    for (int i = 0; i < n; ++i) {
      int l = 0;
      for (int k = rp[i]; k < rp[i + 1] && col[k] < i; ++k) l = std::max(l, lev[col[k]] + 1);
      lev[i] = l;
      maxl = std::max(maxl, l);
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      int l = 0;
      for (int k = rp[i + 1] - 1; k >= rp[i] && col[k] > i; --k) l = std::max(l, lev[col[k]] + 1);
      lev[i] = l;
      maxl = std::max(maxl, l);
    }
  }
  offsets.assign(maxl + 2, 0);
  for (int i = 0; i < n; ++i) offsets[lev[i] + 1]++;
  for (int l = 0; l <= maxl; ++l) offsets[l + 1] += offsets[l];
  order.resize(n);
  std::vector<int> fill(offsets.begin(), offsets.end() - 1);
  for (int i = 0; i < n; ++i) order[fill[lev[i]]++] = i;
}

struct Ilu {
  double* lu = nullptr;
  int* diag = nullptr;
  int* lorder = nullptr;
  int* uorder = nullptr;
  std::vector<int> loff, uoff;
};

gdt_status ilu_setup(gdt_context ctx, gdt_matrix m, Ilu& f, cudaStream_t s) {
  const int n = int(m->rows);
  std::vector<int> rp(n + 1), col(m->nnz);
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(rp.data(), m->rp, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(col.data(), m->col, sizeof(int) * m->nnz, cudaMemcpyDeviceToHost, s));
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
  std::vector<int> lo, uo;
  level_sets(n, rp, col, false, lo, f.loff);
  level_sets(n, rp, col, true, uo, f.uoff);
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&f.lu, sizeof(double) * m->nnz, s));
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&f.diag, sizeof(int) * n, s));
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&f.lorder, sizeof(int) * n, s));
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&f.uorder, sizeof(int) * n, s));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(f.lorder, lo.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(f.uorder, uo.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(f.lu, m->val, sizeof(double) * m->nnz, cudaMemcpyDeviceToDevice, s));
  k_find_diag<<<grid_blocks(n, TH), TH, 0, s>>>(n, m->rp, m->col, f.diag);
  GDT_CHECK(ctx, check_launch(ctx, "ilu diag"));
  for (size_t l = 0; l + 1 < f.loff.size(); ++l) {
    int cnt = f.loff[l + 1] - f.loff[l];
    k_ilu_factor_level<<<grid_blocks(cnt, 128), 128, 0, s>>>(f.lorder + f.loff[l], cnt, m->rp, m->col, f.diag, f.lu);
    GDT_CHECK(ctx, check_launch(ctx, "ilu factor"));
  }
  // keep the host copies alive until the asynchronous uploads have completed
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
  return GDT_OK;
}

void ilu_apply(gdt_context ctx, gdt_matrix m, const Ilu& f, const double* r, double* z, const KState* st,
               cudaStream_t s) {
  for (size_t l = 0; l + 1 < f.loff.size(); ++l) {
    int cnt = f.loff[l + 1] - f.loff[l];
    k_ilu_lower_level<<<grid_blocks(cnt, 128), 128, 0, s>>>(f.lorder + f.loff[l], cnt, m->rp, m->col, f.diag, f.lu, r,
                                                            z, st);
    ctx->launches++;
  }
  for (size_t l = 0; l + 1 < f.uoff.size(); ++l) {
    int cnt = f.uoff[l + 1] - f.uoff[l];
    k_ilu_upper_level<<<grid_blocks(cnt, 128), 128, 0, s>>>(f.uorder + f.uoff[l], cnt, m->rp, m->col, f.diag, f.lu, z,
                                                            st);
    ctx->launches++;
  }
}


// ------------------------------------------------------------------------- persistent CG ---
// One cooperative launch runs every iteration of Jacobi-preconditioned (or plain) CG. The kernel
// boundaries of the graph form become grid barriers, three per iteration: after q = A p, after the
// x/r update, after the direction update. Every block reduces the per-block partial sums itself, in
// block order, so all blocks hold bit-identical alpha, beta and convergence decisions without a
// broadcast step. This pays most where an iteration is bound by launch, ramp-up and tail latency
// rather than bandwidth (matrices and vectors that stay in the 129 MB L2), and also where the SpMV
// streams the matrix from HBM (no kernel boundaries, no row-pointer indirection). The Chronopoulos-Gear form (one
// reduction and two barriers per iteration) measured slower here (277 against 250 ms for the SWIPDG
// system of 256^2 squares) and needed up to 65 % more iterations on badly conditioned 1D and 2D
// systems, so the iteration stays the standard one of the graph form. The SpMV reads a SELL-32 copy
// of the matrix (slices of 32 rows stored column-major, padded to the slice's longest row): a lane
// owns one row and reads its entries with loads that are coalesced across the warp, so a pass over
// 32 rows costs two dependent memory latencies (entries, gathers) and no shared memory. (Staging each
// warp's CSR slice in shared memory instead cost three latencies per pass and 8-way bank conflicts
// when the lanes read their rows: 17.6 us of a 43 us iteration on that SWIPDG system.) The matrix
// and the Jacobi diagonal are read-only in the kernel (non-coherent loads); the vectors are written
// by other blocks between barriers and read with plain loads, which the barrier's fences order.
constexpr int PT = 1024;  // threads per block (one block per SM)

struct PcgArgs {
  int n;
  int nslices;
  const int2* meta;   // SELL-32 (offset, width) per slice
  const int* col;     // SELL-32 columns
  const double* val;  // SELL-32 values
  const double* dinv;
  double* x;
  double* r;
  double* p;
  double* q;
  double* z;  // dinv r, kept by the update for the direction step
  KState* st;
  double* part;       // 3 * gridDim.x doubles: p.q | r.z, r.r per block
  unsigned int* bar;  // 64-bit arrival count at bar[0], generation at bar[kBarGen], fault at bar[kBarFault]
  unsigned long long wait_ns;  // longest wait at a grid barrier
};
// q = A p over the warp's slices (rows of at most 32 entries); returns this thread's share of p.q.
// The slices of a warp are the same in every iteration: lane m holds the (offset, width) of the
// warp's m-th slice, so a pass gets them by a shuffle instead of a load.
__device__ __forceinline__ double pcg_spmv(const PcgArgs& a, int2 mymeta) {
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (PT / 32);
  double pq = 0.0;
  int m = 0;
  for (int slice = blockIdx.x * (PT / 32) + (threadIdx.x >> 5); slice < a.nslices; slice += nw, ++m) {
    int2 md;
    if (m < 32) {
      md.x = __shfl_sync(0xffffffffu, mymeta.x, m);
      md.y = __shfl_sync(0xffffffffu, mymeta.y, m);
    } else {
      md = __ldg(a.meta + slice);
    }
    const int row = slice * 32 + lane;
    const bool act = row < a.n;
    const double pr = act ? a.p[row] : 0.0;
    const double* v = a.val + md.x + lane;
    const int* c = a.col + md.x + lane;
    double s0 = 0.0, s1 = 0.0;
#pragma unroll
    for (int t0 = 0; t0 < 32; t0 += 12) {
      if (t0 < md.y) {  // warp-uniform
        double vv[12];
        int cc[12];
#pragma unroll
        for (int j = 0; j < 12; ++j) {
          const bool in = t0 + j < md.y;
          vv[j] = in ? __ldg(v + (t0 + j) * 32) : 0.0;
          cc[j] = in ? __ldg(c + (t0 + j) * 32) : 0;
        }
#pragma unroll
        for (int j = 0; j < 12; j += 2) {
          if (t0 + j < md.y) s0 = fma(vv[j], a.p[cc[j]], s0);
          if (t0 + j + 1 < md.y) s1 = fma(vv[j + 1], a.p[cc[j + 1]], s1);
        }
      }
    }
    const double s = s0 + s1;
    if (act) {
      a.q[row] = s;
      pq = fma(pr, s, pq);
    }
  }
  return pq;
}

__global__ void __launch_bounds__(PT, 1) k_pcg_persistent(PcgArgs a) {
  __shared__ double red[2 * 32];
  __shared__ double bc[2];
  int2 mymeta = make_int2(0, 0);
  {
    const int slice = blockIdx.x * (PT / 32) + (threadIdx.x >> 5) + (threadIdx.x & 31) * gridDim.x * (PT / 32);
    if (slice < a.nslices) mymeta = __ldg(a.meta + slice);
  }
  KState* st = a.st;
  if (entry_flag(&st->converged)) return;
  double rho = st->rho, alpha = st->alpha, beta = st->beta, rr = st->rr;
  const double stop = st->tol2 * st->rr0;
  const int max_iter = st->max_iter;
  int iter = st->iter, conv = 0, brk = 0;
  const int nb = gridDim.x;
  const int stride = nb * PT;
  unsigned int epoch = 0;
  while (true) {
    // q = A p, p.q -> alpha
    double v1[1] = {pcg_spmv(a, mymeta)};
    block_reduce<1>(v1, red);
    if (threadIdx.x == 0) a.part[blockIdx.x] = v1[0];
    if (!grid_barrier(a.bar, epoch, a.wait_ns)) break;
    grid_allreduce<1>(a.part, v1, bc);
    alpha = rho / v1[0];
    if (!(v1[0] > 0.0) || !isfinite(v1[0])) {
      brk = conv = 1;
      break;
    }
    // x += alpha p, r -= alpha q; r.z (z = dinv r) and r.r
    // (two elements per thread and pass, all their loads issued before the first store)
    double v2[2] = {0.0, 0.0};
    for (int i0 = blockIdx.x * PT + threadIdx.x; i0 < a.n; i0 += 2 * stride) {
      double pv[2], qv[2], xv[2], rv[2], dv[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int i = i0 + u * stride;
        const bool in = i < a.n;
        pv[u] = in ? a.p[i] : 0.0;
        qv[u] = in ? a.q[i] : 0.0;
        xv[u] = in ? a.x[i] : 0.0;
        rv[u] = in ? a.r[i] : 0.0;
        dv[u] = in ? __ldg(a.dinv + i) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int i = i0 + u * stride;
        if (i < a.n) {
          a.x[i] = fma(alpha, pv[u], xv[u]);
          const double ri = fma(-alpha, qv[u], rv[u]);
          const double zi = dv[u] * ri;
          a.r[i] = ri;
          a.z[i] = zi;
          v2[0] = fma(ri, zi, v2[0]);
          v2[1] = fma(ri, ri, v2[1]);
        }
      }
    }
    block_reduce<2>(v2, red);
    if (threadIdx.x == 0) {
      a.part[nb + blockIdx.x] = v2[0];
      a.part[2 * nb + blockIdx.x] = v2[1];
    }
    if (!grid_barrier(a.bar, epoch, a.wait_ns)) break;
    grid_allreduce<2>(a.part + nb, v2, bc);
    beta = v2[0] / rho;
    rho = v2[0];
    rr = v2[1];
    iter += 1;
    if (rr <= stop || iter >= max_iter) conv = 1;
    if (!isfinite(rr)) brk = conv = 1;
    if (conv) break;
    // p = dinv r + beta p
    for (int i0 = blockIdx.x * PT + threadIdx.x; i0 < a.n; i0 += 3 * stride) {
      double pv[3], zv[3];
#pragma unroll
      for (int u = 0; u < 3; ++u) {
        const int i = i0 + u * stride;
        const bool in = i < a.n;
        pv[u] = in ? a.p[i] : 0.0;
        zv[u] = in ? a.z[i] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 3; ++u) {
        const int i = i0 + u * stride;
        if (i < a.n) a.p[i] = fma(beta, pv[u], zv[u]);
      }
    }
    if (!grid_barrier(a.bar, epoch, a.wait_ns)) break;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->rho = rho;
    st->alpha = alpha;
    st->beta = beta;
    st->rr = rr;
    st->iter = iter;
    st->breakdown = brk;
    st->converged = 1;
  }
}

// Rows of at most 32 entries (the SELL-32 SpMV's limit). Measured against the graph form: 40.6 against
// 51.7 us per iteration for the L2-resident SWIPDG system of 256^2 squares, and 209 against 264 us
// for the 128^3 Q1 system (727.7 MB streamed from HBM per SpMV), same iteration counts: AUTO takes it
// wherever it applies.
bool persistent_applies(gdt_context ctx, gdt_matrix m) {
  if (ctx->timing || ctx->solver_launch == GDT_SOLVER_LAUNCH_GRAPH) return false;
  return m->max_row >= 1 && m->max_row <= 32 && m->rows >= 1;
}

// Runs the iterations after residual_init; the caller reads the final state from st. Returns
// GDT_EUNSUPPORTED, before anything ran, where no cooperative launch of the kernel can be made
// (the caller then runs the graph form).
gdt_status pcg_persistent(gdt_context ctx, gdt_matrix m, double* x, double* r, double* p, double* q, double* z,
                          const double* dinv, KState* st, cudaStream_t s) {
  const void* fn = reinterpret_cast<const void*>(&k_pcg_persistent);
  int dev = 0, coop = 0, per_sm = 0;
  GDT_TRY_CUDA(ctx, cudaGetDevice(&dev));
  GDT_TRY_CUDA(ctx, cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop) return GDT_EUNSUPPORTED;  // the caller runs the graph form
  GDT_TRY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, PT, 0));
  if (per_sm < 1) return GDT_EUNSUPPORTED;
  int blocks = ctx->num_sms;  // one block per SM
  if (ctx->persistent_blocks > 0) blocks = std::min(blocks, ctx->persistent_blocks);
  // no more blocks than warps have slices
  const int nslices = int((m->rows + 31) / 32);
  const int needed = (nslices + PT / 32 - 1) / (PT / 32);
  if (needed < blocks) blocks = std::max(1, needed);
  {
    // the values are copied at every solve: the caller may have written them through the CSR pointer
    const gdt_status ss = sell_prepare(ctx, m, s, true);
    if (ss != GDT_OK) return ss;
  }
  PcgArgs a;
  a.n = int(m->rows);
  a.nslices = nslices;
  a.meta = reinterpret_cast<const int2*>(m->sell_meta);
  a.col = m->sell_col;
  a.val = m->sell_val;
  a.dinv = dinv;
  a.x = x;
  a.r = r;
  a.p = p;
  a.q = q;
  a.z = z;
  a.st = st;
  a.part = ctx->scratch;
  // the barrier words live in the upper half of the scratch (the partials use its start)
  a.bar = reinterpret_cast<unsigned int*>(ctx->scratch + kScratchDoubles / 2);
  a.wait_ns = ctx->persistent_wait_ns > 0 ? (unsigned long long)ctx->persistent_wait_ns : kBarrierNs;
  if (3 * blocks > kScratchDoubles / 2) return fail(ctx, GDT_EUNSUPPORTED, "persistent solver: grid too large");
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(a.bar, 0, sizeof(unsigned long long), s));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(a.bar + kBarGen, 0, sizeof(unsigned int), s));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(a.bar + kBarFault, 0, sizeof(unsigned int), s));
  void* args[] = {&a};
  const cudaError_t le = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(PT), args, 0, s);
  if (le == cudaErrorCooperativeLaunchTooLarge) {  // fewer SMs available than the device has
    cudaGetLastError();
    return GDT_EUNSUPPORTED;
  }
  GDT_TRY_CUDA(ctx, le);
  ctx->launches++;
  unsigned int fault = 0;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&fault, a.bar + kBarFault, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
  if (fault) return fail(ctx, GDT_ECUDA, "persistent solver: a grid barrier wait ran out");
  return GDT_OK;
}

}  // namespace

__global__ void k_fill(int n, double* __restrict__ v, double value) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = value;
}
__global__ void k_probe(int n, double* __restrict__ a, double* __restrict__ b) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    a[i] = b[i] = 1.0 + 0.001 * double(i % 997);
}

// Picks the SpMV schedule of the fused FP64 CG iteration by timing each valid schedule inside that
// iteration (SpMV + update + direction on scratch vectors, a few real CG steps on A x = probe), not
// back to back: inside the loop the SpMV starts with the vectors the other two kernels just wrote
// dirty in L2, and the schedules rank differently there (128^3 Q1: the staged cp.async schedule
// wins in the loop while 4-lane vector CSR wins back to back). Once per matrix; temporary memory of
// 5 n doubles.
gdt_status tune_cg(gdt_context ctx, gdt_matrix m, const Launch& L0, cudaStream_t s) {
  if (m->cg_sched >= 0) return GDT_OK;
  if (m->pinned) {
    m->cg_sched = m->use_sell ? kSellSchedule : m->spmv_sched;
    return GDT_OK;
  }
  const int n = int(m->rows);
  const size_t vb = sizeof(double) * std::max(n, 1);
  double *x = nullptr, *r = nullptr, *p = nullptr, *q = nullptr, *d = nullptr;
  KState* st = nullptr;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&x, vb, s));
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&r, vb, s));
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&p, vb, s));
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&q, vb, s));
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&d, vb, s));
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&st, sizeof(KState), s));
  const int pair_blocks = std::max(1, std::min(grid_blocks((n + 1) / 2, TH), ctx->num_sms * 8));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int timing = ctx->timing;
  ctx->timing = 0;
  float best = FLT_MAX;
  int best_sched = m->spmv_sched;
  const bool sell = sell_prepare(ctx, m, s, true) == GDT_OK;
  for (int sched = 0; sched <= kSellSchedule; ++sched) {
    if (sched < kSchedules ? !schedule_valid(sched, m->max_row) : !sell) continue;
    Launch L = L0;
    L.sched = sched < kSchedules ? sched : L0.sched;
    KState init{};
    init.rho = 1.0;
    init.rr0 = 1.0;
    init.max_iter = 1 << 30;
    cudaMemcpyAsync(st, &init, sizeof(KState), cudaMemcpyHostToDevice, s);
    k_fill<<<L.vec_blocks, TH, 0, s>>>(n, x, 0.0);
    k_fill<<<L.vec_blocks, TH, 0, s>>>(n, d, 1.0);
    k_probe<<<L.vec_blocks, TH, 0, s>>>(n, r, p);
    float total = 0.f;
    bool ok = true;
    for (int it = 0; it < 5; ++it) {
      cudaEventRecord(e0, s);
      if (sched == kSellSchedule) spmv_cg_sell(L, m, p, q, st);
      else spmv_mode<double, 1>(L, m->rp, m->col, m->val, p, q, nullptr, st);
      cudaEventRecord(e1, s);
      k_cg_update_jacobi2<<<pair_blocks, TH, 0, s>>>(n, x, p, r, q, d, st, L.partials, L.ticket);
      k_cg_p_jacobi2<<<pair_blocks, TH, 0, s>>>(n, p, r, d, st);
      if (it >= 2) {
        float ms = 0.f;
        ok = ok && cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
        total += ms;
      }
    }
    ok = ok && cudaGetLastError() == cudaSuccess;
    ctx->launches += 18;
    if (ok && total < best) {
      best = total;
      best_sched = sched;
    }
  }
  ctx->timing = timing;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(x, s);
  cudaFreeAsync(r, s);
  cudaFreeAsync(p, s);
  cudaFreeAsync(q, s);
  cudaFreeAsync(d, s);
  cudaFreeAsync(st, s);
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
  m->cg_sched = best_sched;
  return GDT_OK;
}

gdt_status solve(gdt_context ctx, gdt_matrix m, const double* b, double* x, const gdt_solver_opts* o,
                 gdt_solve_info* info) {
  cudaStream_t s = ctx->stream;
  cudaStream_t own = nullptr;
  if (s == nullptr) {  // the legacy stream cannot be captured; use a blocking stream ordered with it
    GDT_TRY_CUDA(ctx, cudaStreamCreate(&own));
    s = own;
  }
  struct Cleanup {
    cudaStream_t st;
    ~Cleanup() {
      if (st) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
      }
    }
  } cleanup{own};
  const int n = int(m->rows);
  ctx->last_solver_launch = 0;
  Launch L;
  L.ctx = ctx;
  L.n = n;
  GDT_CHECK(ctx, tune_spmv(ctx, m));
  L.sched = m->spmv_sched;
  L.s = s;
  L.vec_blocks = std::max(1, std::min(grid_blocks(n, TH), ctx->num_sms * 8));
  L.partials = ctx->scratch;
  L.ticket = ctx->counters;
  const int chunk = o->check_every > 0 ? o->check_every : 32;
  const bool mixed = o->precision == GDT_PRECISION_MIXED;
  if (mixed && (o->solver != GDT_SOLVER_CG || o->precond == GDT_PREC_ILU0))
    return fail(ctx, GDT_EUNSUPPORTED, "mixed precision is provided for CG with Jacobi or no preconditioner");
  if (mixed && ctx->solver_launch != GDT_SOLVER_LAUNCH_GRAPH && mixed_mf_applies(m)) {
    // 3D Q1 Laplace matrices: the matrix-free operator, all inner iterations in persistent launches
    const gdt_status ms = solve_mixed_mf(ctx, m, b, x, o, info, s);
    if (ms != GDT_EUNSUPPORTED) {
      ctx->last_solver_launch = GDT_SOLVER_LAUNCH_PERSISTENT;
      return ms;
    }
  }
  if (mixed && mixed_stencil_supported(m)) {
    ctx->last_solver_launch = GDT_SOLVER_LAUNCH_GRAPH;
    return solve_mixed_stencil(ctx, m, b, x, o, info, s);
  }
  KState* st = nullptr;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&st, sizeof(KState), s));
  KState init{};
  init.tol2 = o->tol * o->tol;
  init.max_iter = o->max_iter;
  std::vector<void*> allocs;
  allocs.push_back(st);
  auto alloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMallocAsync(&p, bytes, s) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return p;
  };
  struct Freer {
    std::vector<void*>* a;
    cudaStream_t s;
    ~Freer() {
      for (void* p : *a) cudaFreeAsync(p, s);
    }
  } freer{&allocs, s};
  gdt_solve_info res{};
  if (!mixed) {
    GDT_TRY_CUDA(ctx, cudaMemcpyAsync(st, &init, sizeof(KState), cudaMemcpyHostToDevice, s));
    const size_t vb = sizeof(double) * std::max(n, 1);
    double* r = (double*)alloc(vb);
    double* p = (double*)alloc(vb);
    double* q = (double*)alloc(vb);
    double* dinv = nullptr;
    if (!r || !p || !q) return fail(ctx, GDT_ENOMEM, "solver vectors");
    if (o->precond == GDT_PREC_JACOBI) {
      dinv = (double*)alloc(vb);
      if (!dinv) return fail(ctx, GDT_ENOMEM, "solver vectors");
      k_jacobi_diag<double, double><<<L.vec_blocks, TH, 0, s>>>(n, m->rp, m->col, m->val, dinv);
      GDT_CHECK(ctx, check_launch(ctx, "jacobi"));
    }
    Ilu ilu;
    if (o->precond == GDT_PREC_ILU0) {
      GDT_CHECK(ctx, ilu_setup(ctx, m, ilu, s));
      allocs.push_back(ilu.lu);
      allocs.push_back(ilu.diag);
      allocs.push_back(ilu.lorder);
      allocs.push_back(ilu.uorder);
    }
    const int chunk_used = (o->precond == GDT_PREC_ILU0) ? std::min(chunk, 2) : chunk;
    const int max_chunks = o->max_iter / chunk_used + 2;
    if (o->solver == GDT_SOLVER_CG) {
      if (o->precond != GDT_PREC_ILU0) {
        // fused Jacobi (or identity) path
        double* one = dinv;
        if (!one) {
          one = (double*)alloc(vb);
          if (!one) return fail(ctx, GDT_ENOMEM, "solver vectors");
          std::vector<double> ones(n, 1.0);
          GDT_TRY_CUDA(ctx, cudaMemcpyAsync(one, ones.data(), vb, cudaMemcpyHostToDevice, s));
          GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
        }
        bool persistent = persistent_applies(ctx, m);
        if (persistent) {
          residual_init<double>(L, m->rp, m->col, m->val, x, b, r, one, p, st);
          double* z = (double*)alloc(vb);
          if (!z) return fail(ctx, GDT_ENOMEM, "solver vectors");
          const gdt_status ps = pcg_persistent(ctx, m, x, r, p, q, z, one, st, s);
          if (ps == GDT_EUNSUPPORTED) persistent = false;  // x untouched: the graph form starts afresh
          else if (ps != GDT_OK) return ps;
          else ctx->last_solver_launch = GDT_SOLVER_LAUNCH_PERSISTENT;
        }
        if (!persistent) {
          ctx->last_solver_launch = GDT_SOLVER_LAUNCH_GRAPH;
          GDT_CHECK(ctx, tune_cg(ctx, m, L, s));
          // the SELL copy is refreshed at every solve (the caller may have written the CSR values)
          const bool cg_sell = m->cg_sched == kSellSchedule && sell_prepare(ctx, m, s, true) == GDT_OK;
          L.sched = m->cg_sched == kSellSchedule ? m->spmv_sched : m->cg_sched;
          residual_init<double>(L, m->rp, m->col, m->val, x, b, r, one, p, st);
          // pairs of rows per thread when every vector is 16-byte aligned (the solver's own are; x is
          // the caller's)
          const bool pairs = (reinterpret_cast<uintptr_t>(x) & 15u) == 0;
          const int pair_blocks = std::max(1, std::min(grid_blocks((n + 1) / 2, TH), ctx->num_sms * 8));
          GDT_CHECK(ctx, iterate_chunks(ctx, s, &st->converged, chunk_used, max_chunks, [&] {
            if (cg_sell) spmv_cg_sell(L, m, p, q, st);
            else spmv_mode<double, 1>(L, m->rp, m->col, m->val, p, q, nullptr, st);
            timing_begin(ctx, s, GDT_TIMING_CG_UPDATE);
            if (pairs)
              k_cg_update_jacobi2<<<pair_blocks, TH, 0, s>>>(n, x, p, r, q, one, st, L.partials, L.ticket);
            else
              k_cg_update_jacobi<double, double><<<L.vec_blocks, TH, 0, s>>>(n, x, p, r, q, one, st, L.partials,
                                                                             L.ticket);
            timing_end(ctx, s);
            timing_begin(ctx, s, GDT_TIMING_CG_DIRECTION);
            if (pairs)
              k_cg_p_jacobi2<<<pair_blocks, TH, 0, s>>>(n, p, r, one, st);
            else
              k_cg_p_jacobi<double><<<L.vec_blocks, TH, 0, s>>>(n, p, r, one, st);
            timing_end(ctx, s);
            ctx->launches += 2;
          }));
        }
      } else {
        double* z = (double*)alloc(vb);
        if (!z) return fail(ctx, GDT_ENOMEM, "solver vectors");
        residual_init<double>(L, m->rp, m->col, m->val, x, b, r, nullptr, nullptr, st);
        ilu_apply(ctx, m, ilu, r, z, st, s);
        // rho = r.z, p = z
        k_cg_beta<<<L.vec_blocks, TH, 0, s>>>(n, r, z, st, L.partials, L.ticket);
        GDT_TRY_CUDA(ctx, cudaMemcpyAsync(p, z, vb, cudaMemcpyDeviceToDevice, s));
        ctx->launches++;
        GDT_CHECK(ctx, iterate_chunks(ctx, s, &st->converged, chunk_used, max_chunks, [&] {
          spmv_mode<double, 1>(L, m->rp, m->col, m->val, p, q, nullptr, st);
          k_cg_update<<<L.vec_blocks, TH, 0, s>>>(n, x, p, r, q, st, L.partials, L.ticket);
          ilu_apply(ctx, m, ilu, r, z, st, s);
          k_cg_beta<<<L.vec_blocks, TH, 0, s>>>(n, r, z, st, L.partials, L.ticket);
          k_cg_p<<<L.vec_blocks, TH, 0, s>>>(n, p, z, st);
          ctx->launches += 3;
        }));
      }
    } else {
      // BiCGStab with M = Jacobi / ILU0 / identity
      double* rt = (double*)alloc(vb);
      double* v = (double*)alloc(vb);
      double* y = (double*)alloc(vb);
      double* t = (double*)alloc(vb);
      if (!rt || !v || !y || !t) return fail(ctx, GDT_ENOMEM, "solver vectors");
      GDT_TRY_CUDA(ctx, cudaMemsetAsync(v, 0, vb, s));
      GDT_TRY_CUDA(ctx, cudaMemsetAsync(p, 0, vb, s));
      residual_init<double>(L, m->rp, m->col, m->val, x, b, r, nullptr, nullptr, st);
      GDT_TRY_CUDA(ctx, cudaMemcpyAsync(rt, r, vb, cudaMemcpyDeviceToDevice, s));
      auto prec = [&](const double* in, double* out) {
        if (o->precond == GDT_PREC_ILU0) ilu_apply(ctx, m, ilu, in, out, st, s);
        else {
          k_scale<double><<<L.vec_blocks, TH, 0, s>>>(n, out, dinv, in, st);
          ctx->launches++;
        }
      };
      GDT_CHECK(ctx, iterate_chunks(ctx, s, &st->converged, chunk_used, max_chunks, [&] {
        k_bicg_rho<<<L.vec_blocks, TH, 0, s>>>(n, rt, r, st, L.partials, L.ticket);
        k_bicg_p<<<L.vec_blocks, TH, 0, s>>>(n, p, r, v, st);
        prec(p, y);
        spmv_mode<double, 2>(L, m->rp, m->col, m->val, y, v, rt, st);
        k_bicg_s<<<L.vec_blocks, TH, 0, s>>>(n, x, y, r, v, st, L.partials, L.ticket);
        prec(r, q);  // q = M^{-1} s
        spmv_mode<double, 3>(L, m->rp, m->col, m->val, q, t, r, st);
        k_bicg_r<<<L.vec_blocks, TH, 0, s>>>(n, x, q, r, t, st, L.partials, L.ticket);
        ctx->launches += 4;
      }));
    }
    KState fin;
    GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&fin, st, sizeof(KState), cudaMemcpyDeviceToHost, s));
    GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
    {
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return fail(ctx, GDT_ECUDA, std::string("krylov: ") + cudaGetErrorString(e));
    }
    // report the true FP64 residual of the returned iterate
    residual64(L, m, x, b, r, L.partials + kScratchDoubles - 1);
    double rr_true = 0;
    GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&rr_true, L.partials + kScratchDoubles - 1, sizeof(double),
                                      cudaMemcpyDeviceToHost, s));
    GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
    res.iterations = fin.iter;
    res.refinements = 0;
    res.rel_residual = fin.rr0 > 0 ? std::sqrt(rr_true / fin.rr0) : 0.0;
    res.converged = (fin.breakdown == 0) && (fin.rr0 == 0 || fin.rr <= fin.tol2 * fin.rr0);
  } else {
    // ---------------------------------------------------- FP64 iterative refinement, FP32 inner CG
    const size_t vb = sizeof(double) * std::max(n, 1), fb = sizeof(float) * std::max(n, 1);
    double* r = (double*)alloc(vb);
    float* val32 = (float*)alloc(sizeof(float) * (m->nnz + 8));
    float* r32 = (float*)alloc(fb);
    float* d32 = (float*)alloc(fb);
    float* p32 = (float*)alloc(fb);
    float* q32 = (float*)alloc(fb);
    float* dinv32 = (float*)alloc(fb);
    double* scal = (double*)alloc(sizeof(double) * 4);
    if (!r || !val32 || !r32 || !d32 || !p32 || !q32 || !dinv32 || !scal) return fail(ctx, GDT_ENOMEM, "solver vectors");
    k_to_float<<<ctx->num_sms * 8, TH, 0, s>>>(m->nnz, m->val, val32);
    ctx->launches++;
    if (o->precond == GDT_PREC_JACOBI)
      k_jacobi_diag<float, double><<<L.vec_blocks, TH, 0, s>>>(n, m->rp, m->col, m->val, dinv32);
    else {
      std::vector<float> ones(n, 1.0f);
      GDT_TRY_CUDA(ctx, cudaMemcpyAsync(dinv32, ones.data(), fb, cudaMemcpyHostToDevice, s));
      GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
    }
    ctx->launches++;
    const double inner_tol = o->inner_tol > 0 ? o->inner_tol : 1e-3;
    double rr0 = -1.0, rr = 0.0;
    int total_iter = 0, refinements = 0;
    bool ok = false;
    double* rr_dev = scal;
    for (int outer = 0; outer < 200; ++outer) {
      residual64(L, m, x, b, r, rr_dev);
      GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&rr, rr_dev, sizeof(double), cudaMemcpyDeviceToHost, s));
      GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
      if (rr0 < 0) rr0 = rr;
      if (!std::isfinite(rr)) break;
      if (rr <= o->tol * o->tol * rr0 || rr == 0.0) {
        ok = true;
        break;
      }
      if (total_iter >= o->max_iter) break;
      // inner: A d = r / ||r|| in FP32, d0 = 0
      k_scale_to_float<<<L.vec_blocks, TH, 0, s>>>(n, r, rr_dev, r32);
      GDT_TRY_CUDA(ctx, cudaMemsetAsync(d32, 0, fb, s));
      KState in = init;
      in.tol2 = inner_tol * inner_tol;
      in.max_iter = std::max(1, o->max_iter - total_iter);
      GDT_TRY_CUDA(ctx, cudaMemcpyAsync(st, &in, sizeof(KState), cudaMemcpyHostToDevice, s));
      k_init_from_rhs<float><<<L.vec_blocks, TH, 0, s>>>(n, r32, dinv32, p32, st, L.partials, L.ticket);
      ctx->launches += 2;
      GDT_CHECK(ctx, iterate_chunks(ctx, s, &st->converged, chunk, in.max_iter / chunk + 2, [&] {
        spmv_mode<float, 1>(L, m->rp, m->col, val32, p32, q32, nullptr, st);
        k_cg_update_jacobi<float, float><<<L.vec_blocks, TH, 0, s>>>(n, d32, p32, r32, q32, dinv32, st, L.partials,
                                                                     L.ticket);
        k_cg_p_jacobi<float><<<L.vec_blocks, TH, 0, s>>>(n, p32, r32, dinv32, st);
        ctx->launches += 2;
      }));
      KState fin;
      GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&fin, st, sizeof(KState), cudaMemcpyDeviceToHost, s));
      GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
      total_iter += fin.iter;
      k_correct<<<L.vec_blocks, TH, 0, s>>>(n, x, d32, rr_dev);
      ctx->launches++;
      refinements++;
      if (fin.breakdown) break;
    }
    {
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return fail(ctx, GDT_ECUDA, std::string("mixed krylov: ") + cudaGetErrorString(e));
    }
    res.iterations = total_iter;
    res.refinements = refinements;
    res.rel_residual = rr0 > 0 ? std::sqrt(rr / rr0) : 0.0;
    res.converged = ok ? 1 : 0;
  }
  if (info) *info = res;
  if (!res.converged) return fail(ctx, GDT_ENOCONV, "linear solver did not converge");
  return GDT_OK;
}

}  // namespace gdt
