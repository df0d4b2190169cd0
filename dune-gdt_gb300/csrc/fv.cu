// Finite volumes on structured cube grids (m = 1):
//   AdvectionFvOperator::apply (operators/advection-fv.hh:66-115) = LocalAdvectionFvCouplingOperator on
//   every inner/periodic intersection once (local/operators/advection-fv.hh:127-153), the boundary
//   treatments by extrapolation or by a boundary flux on the non-periodic sides (:187-457), with
//   NumericalLaxFriedrichsFlux (local/numerical-fluxes/lax-friedrichs.hh:61-87), NumericalUpwindFlux
//   (upwind.hh:61-73) or NumericalEngquistOsherFlux (engquist-osher.hh:72-103);
//   estimate_dt_for_hyperbolic_system (tools/hyperbolic.hh:38-86); explicit Euler
//   (test/instationary-eocstudies/base.hh:428-447) and ExplicitRungeKuttaTimeStepper with the SSP2
//   tableau (tools/timestepper/explicit-rungekutta.hh:82-97, 237-270), r = -1.
//
// GB300 design: GB300's FP64 pipe (~0.6e12 instructions/s), not HBM, bounds this update, so the 2D
// stepper computes every face flux exactly once per stage inside a shared-memory tile (tile + periodic
// halo staged from global memory), and the second SSP stage fuses u1 = u - dt k0, k1 = L(u1) and
// u_new = u + (k0 + k1)(-dt/2) into one pass: per step it reads u (twice) and k0 and writes k0 and
// u_new (40 bytes per cell). LF uses the local speed max(|f'(u)|, |f'(v)|) multiplied in directly
// (the reference forms 0.5 / (1 / lambda); both agree to rounding). FP64 instructions per cell and
// stage (Burgers LF): the squares once per staged cell, three per face (u - v, u^2 + v^2 and one FMA,
// with 2 max(|u|, |v|) on the integer pipe), three for the update K and at most two for the stage's
// output: about 10 (first stage) and 13.5 (second) where the per-face form took 25.
#include <cmath>
#include <limits>

#include <cub/device/device_reduce.cuh>

#include "internal.cuh"

namespace gdt {
namespace {

struct FvParams {
  int flux;       // GDT_FLUX_*
  int numflux;    // GDT_NUMFLUX_*
  double vel[3];
  double lf_inv_lambda;  // 0: local LF; else the reference's fixed lambda_ (coefficient 0.5 / lambda_)
  int bkind[6];          // per side (-x, +x, -y, +y, -z, +z): GDT_FV_BOUNDARY_*, or -1 for a periodic side
  double bval[6];
  // the tiled kernels' form of the flux, 4 g (see face_flux4)
  int form4;             // FORM4_*
  double lam2;           // Burgers LF: 2 lambda_ for a fixed lambda_, 0 for the local one
  double tu[3], tv[3];   // linear transport: 4 g = tu u + tv v (EO: each term only for a positive state)
};

enum { FORM4_GENERIC = 0, FORM4_BURGERS_LF = 1, FORM4_TRANSPORT_LINEAR = 2, FORM4_BURGERS_EO = 3,
       FORM4_TRANSPORT_EO = 4, FORM4_BURGERS_UPWIND = 5, FORM4_BURGERS_LF_FIXED = 6 };

__device__ __forceinline__ double f_of(const FvParams& p, double u, int d) {
  return p.flux == GDT_FLUX_BURGERS ? 0.5 * u * u : p.vel[d] * u;
}
__device__ __forceinline__ double df_of(const FvParams& p, double u, int d) {
  return p.flux == GDT_FLUX_BURGERS ? u : p.vel[d];
}

// numerical flux g(u, v, n) for the unit normal n = sgn e_k (sgn = +-1), u the state on the side n
// points away from
__device__ __forceinline__ double normal_flux(const FvParams& p, int dim, int k, double sgn, double u, double v) {
  if (p.numflux == GDT_NUMFLUX_LAX_FRIEDRICHS) {
    double lam;
    if (p.lf_inv_lambda != 0.0) {
      lam = 1.0 / p.lf_inv_lambda;  // coefficient (u - v) * 0.5 / lambda_
    } else if (p.flux == GDT_FLUX_BURGERS) {
      lam = fmax(fabs(u), fabs(v));
    } else {
      lam = 0.0;
      for (int d = 0; d < dim; ++d) lam = fmax(lam, fabs(p.vel[d]));
    }
    const double fsum = sgn * (f_of(p, u, k) + f_of(p, v, k));
    return 0.5 * fma(u - v, lam, fsum);
  }
  if (p.numflux == GDT_NUMFLUX_ENGQUIST_OSHER) {
    // f(0).n + int_0^u max(n.f'(s), 0) ds + int_0^v min(n.f'(s), 0) ds, each integral only for a
    // positive state (the reference integrates over [0, state] only then); in closed form for both
    // fluxes, f(0) = 0: Burgers n.f'(s) = sgn s, transport n.f'(s) = sgn v_k
    if (p.flux == GDT_FLUX_BURGERS) {
      if (sgn > 0.0) return u > 0.0 ? 0.5 * u * u : 0.0;
      return v > 0.0 ? -0.5 * v * v : 0.0;
    }
    const double a = sgn * p.vel[k];
    return (u > 0.0 ? u * fmax(a, 0.0) : 0.0) + (v > 0.0 ? v * fmin(a, 0.0) : 0.0);
  }
  const double w = (u + v) * 0.5;
  return sgn * df_of(p, w, k) > 0.0 ? sgn * f_of(p, u, k) : sgn * f_of(p, v, k);
}

// numerical flux across a face with unit normal +e_k, seen from the lower cell (value u) to the upper (v)
__device__ __forceinline__ double face_flux(const FvParams& p, int dim, int k, double u, double v) {
  return normal_flux(p, dim, k, 1.0, u, v);
}

// flux through the boundary face on `side` (2k: -e_k, 2k+1: +e_k) of a cell with value u, in the
// direction of the outer normal (what the boundary operator adds as g |I| / |E|)
__device__ __forceinline__ double boundary_flux(const FvParams& p, int dim, int side, double u) {
  const int kind = p.bkind[side];
  const int k = side >> 1;
  const double sgn = (side & 1) ? 1.0 : -1.0;
  if (kind == GDT_FV_BOUNDARY_EXTRAPOLATE) return normal_flux(p, dim, k, sgn, u, u);
  if (kind == GDT_FV_BOUNDARY_DIRICHLET) return normal_flux(p, dim, k, sgn, u, p.bval[side]);
  if (kind == GDT_FV_BOUNDARY_FLUX) return p.bval[side];
  return 0.0;  // GDT_FV_BOUNDARY_NONE on a non-periodic grid: no operator on this side
}

// flux in +e_k direction through the lower (upper = false) or upper boundary face of a cell
__device__ __forceinline__ double boundary_face_flux(const FvParams& p, int dim, int k, bool upper, double u) {
  const double g = boundary_flux(p, dim, 2 * k + (upper ? 1 : 0), u);
  return upper ? g : -g;
}

// 4 g(u, v, +e_k), the numerical flux in a form with fewer FP64 instructions (GB300's FP64 pipe
// bounds the FV update): the factors 1/2 of the flux formulas move into the 1/4 of the update
// coefficients (scaling by powers of two is exact), the transport fluxes collapse to precomputed
// linear combinations, and max(|u|, |v|) and the sign tests run on the integer bit patterns (for
// non-negative doubles the integer order is the floating-point order). Equal to 4 face_flux() up
// to the rounding of the rearranged sums.
__device__ __forceinline__ bool positive(double u) { return __double_as_longlong(u) > 0; }
// max(|u|, |v|) on the bit patterns, with `add` added to the result's pattern (1 << 52 doubles a
// normal number). In inline PTX: written in C++, the mask / integer max / exponent add is recognised
// as fabs, fmax and a doubling and moved onto the FP64 pipe (two more FP64 instructions per face in
// the instruction counts), which this part issues at one warp instruction per 16 SM cycles.
__device__ __forceinline__ double abs_max_bits(double u, double v, long long add) {
  long long r;
  asm("{\n\t"
      ".reg .b64 a, b;\n\t"
      "and.b64 a, %1, 0x7fffffffffffffff;\n\t"
      "and.b64 b, %2, 0x7fffffffffffffff;\n\t"
      "max.s64 a, a, b;\n\t"
      "add.s64 %0, a, %3;\n\t"
      "}"
      : "=l"(r)
      : "l"(__double_as_longlong(u)), "l"(__double_as_longlong(v)), "l"(add));
  return __longlong_as_double(r);
}
__device__ __forceinline__ double abs_max(double u, double v) { return abs_max_bits(u, v, 0); }

template <int FORM>
__device__ __forceinline__ double face_flux4(const FvParams& p, int k, double u, double v) {
  if constexpr (FORM == FORM4_BURGERS_LF) {  // 2 (f(u) + f(v)) + 2 lambda (u - v), f(u) = u^2 / 2
    const double lam = abs_max(u, v);
    return fma(lam + lam, u - v, fma(u, u, v * v));
  } else if constexpr (FORM == FORM4_BURGERS_LF_FIXED) {
    return fma(p.lam2, u - v, fma(u, u, v * v));
  } else if constexpr (FORM == FORM4_TRANSPORT_LINEAR) {
    return fma(p.tu[k], u, p.tv[k] * v);
  } else if constexpr (FORM == FORM4_BURGERS_EO) {  // 4 * (u > 0 ? u^2 / 2 : 0)
    return positive(u) ? (u + u) * u : 0.0;
  } else if constexpr (FORM == FORM4_TRANSPORT_EO) {
    return (positive(u) ? p.tu[k] * u : 0.0) + (positive(v) ? p.tv[k] * v : 0.0);
  } else if constexpr (FORM == FORM4_BURGERS_UPWIND) {  // f'((u + v) / 2) > 0 ? 4 f(u) : 4 f(v)
    const double w = (u + v) * 0.5;
    const double sel = positive(w) ? u : v;
    return (sel + sel) * sel;
  } else {
    return 4.0 * face_flux(p, 2, k, u, v);
  }
}

// ------------------------------------------------------------------------- generic (any dim) ---
// range[c] = sum over the 2d faces of c of +-flux * |I| / |E| (periodic neighbours, or the boundary
// treatment of the side)
__global__ void fv_apply_kernel(GridDesc g, FvParams p, long long nbatch, const double* __restrict__ u,
                                double* __restrict__ out, const double* __restrict__ ubase, double a_u1,
                                int mode, double* __restrict__ u_next, double dt_coef) {
  // mode 0: out = L(u); mode 1 (Euler): u_next = u - dt L(u); mode 2 (SSP stage 2, u1 = ubase + a_u1 * out):
  //   u_next = ubase + dt_coef * (k0 + L(u1)) with k0 = out
  const long long N = g.nelem;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= N * nbatch) return;
  const long long b = idx / N, c = idx % N;
  const long long off = b * N;
  long long ci[3];
  cell_multi(g, c, ci);
  auto val = [&](long long cell) -> double {
    if (mode == 2) return fma(out[off + cell], a_u1, ubase[off + cell]);
    return u[off + cell];
  };
  const double uc = val(c);
  double acc = 0.0;
  for (int k = 0; k < g.dim; ++k) {
    double area = 1.0;
    for (int j = 0; j < g.dim; ++j)
      if (j != k) area *= g.h[j];
    double vol = 1.0;
    for (int j = 0; j < g.dim; ++j) vol *= g.h[j];
    const double coef = area / vol;
    if (p.bkind[2 * k] >= 0) {  // boundary treatments on both sides of direction k
      const double fl = ci[k] == 0 ? boundary_face_flux(p, g.dim, k, false, uc) : 0.0;
      const double fu = ci[k] == g.n[k] - 1 ? boundary_face_flux(p, g.dim, k, true, uc) : 0.0;
      long long cm[3] = {ci[0], ci[1], ci[2]}, cp[3] = {ci[0], ci[1], ci[2]};
      double lo = fl, hi = fu;
      if (ci[k] > 0) {
        cm[k] = ci[k] - 1;
        lo = face_flux(p, g.dim, k, val(cell_index(g, cm)), uc);
      }
      if (ci[k] < g.n[k] - 1) {
        cp[k] = ci[k] + 1;
        hi = face_flux(p, g.dim, k, uc, val(cell_index(g, cp)));
      }
      acc += coef * (hi - lo);
      continue;
    }
    long long cm[3] = {ci[0], ci[1], ci[2]}, cp[3] = {ci[0], ci[1], ci[2]};
    cm[k] = (ci[k] + g.n[k] - 1) % g.n[k];
    cp[k] = (ci[k] + 1) % g.n[k];
    const double um = val(cell_index(g, cm)), up = val(cell_index(g, cp));
    if (g.n[k] == 1) continue;  // a cell neighbouring itself has no flux
    acc += coef * (face_flux(p, g.dim, k, uc, up) - face_flux(p, g.dim, k, um, uc));
  }
  if (mode == 0) out[off + c] = acc;
  else if (mode == 1) u_next[off + c] = fma(-dt_coef, acc, u[off + c]);
  else u_next[off + c] = fma(dt_coef, out[off + c] + acc, ubase[off + c]);
}

// ------------------------------------------------------------------------------- 2D tiled ---
constexpr int TX = 32, TY = 32, BY = 8;  // tile TX x TY cells, block TX x BY threads

// 2 max(|u|, |v|) for the local LF speed, on the integer pipe: the larger magnitude's bit pattern with
// the exponent raised by one (exact for normal numbers; for zero and subnormal speeds the product with
// u - v, at most twice their size, underflows to zero either way)
__device__ __forceinline__ double twice_abs_max(double u, double v) { return abs_max_bits(u, v, 1LL << 52); }
// the Burgers LF forms use the squares of the states, computed once per cell when the tile is staged
__host__ __device__ constexpr bool uses_squares(int form) {
  return form == FORM4_BURGERS_LF || form == FORM4_BURGERS_LF_FIXED;
}
// 4 g(u, v, +e_k) with the squares qu = u^2, qv = v^2 at hand: three FP64 instructions for Burgers LF
template <int FORM>
__device__ __forceinline__ double face4s(const FvParams& p, int k, double u, double v, double qu, double qv) {
  if constexpr (FORM == FORM4_BURGERS_LF) return fma(twice_abs_max(u, v), u - v, qu + qv);
  else if constexpr (FORM == FORM4_BURGERS_LF_FIXED) return fma(p.lam2, u - v, qu + qv);
  else return face_flux4<FORM>(p, k, u, v);
}

// One stage over a tile of TX x TY cells of state b (blockIdx.z). The fluxes are kept as 4 g, and the
// update as K = (gx_right - gx_left) + rho (gy_top - gy_bottom), rho = h_x / h_y, so that
// L(u) = (1 / (4 h_x)) K:
//   STAGE 0: out = c_out K (fv_apply: c_out = 1 / (4 h_x), giving L(u))
//   STAGE 3: out = K (the first SSP-RK2 stage keeps K itself: no multiply by one per cell)
//   STAGE 1 (Euler): out = u + c_out K, c_out = -dt / (4 h_x)
//   STAGE 2 (SSP-RK2): u1 = u + c1 k0 on the tile + halo (k0 = K(u), c1 = -dt / (4 h_x)),
//            out = u + c_out (k0 + K(u1)), c_out = -dt / (8 h_x)
// Every FP64 pass runs whole warps over 32 values: the tile interior column by column, the two halo
// columns and the 33rd x face of every row in passes of their own (a pass with one active lane costs
// the FP64 pipe as much as a full one). BND: some side has a boundary treatment; the faces on those
// sides are then replaced by it. FORM: the numerical flux (FORM4_*), compiled as straight-line code.
template <int STAGE, bool BND, int FORM>
__global__ void __launch_bounds__(TX* BY) fv2d_tile(GridDesc g, FvParams p, const double* __restrict__ u,
                                                    const double* __restrict__ k0, double* __restrict__ out,
                                                    double c1, double c_out, double rho) {
  constexpr bool SQ = uses_squares(FORM);
  __shared__ double s[TY + 2][TX + 2];             // staged state: s[j + 1][i + 1] = cell (x0 + i, y0 + j)
  __shared__ double q[SQ ? TY + 2 : 1][TX + 2];    // its squares
  __shared__ double gx[TY][TX + 1];                // gx[j][i]: x face between tile columns i - 1 and i
  __shared__ double gy[TY + 1][TX];                // gy[j][i]: y face between tile rows j - 1 and j
  const long long nx = g.n[0], ny = g.n[1];
  const long long off = (long long)blockIdx.z * nx * ny;
  const long long x0 = (long long)blockIdx.x * TX, y0 = (long long)blockIdx.y * TY;
  const int tx = threadIdx.x, ty = threadIdx.y;
  // periodic wrap by compare and select (a 64-bit modulo would cost more than the flux arithmetic);
  // beyond a partial tile: clamped, unused
  auto wrap = [](long long c, long long n) { return c < 0 ? n - 1 : (c == n ? 0 : (c > n ? n - 1 : c)); };
  auto stage = [&](int j, int i) {
    const long long cidx = off + wrap(y0 + j - 1, ny) * nx + wrap(x0 + i - 1, nx);
    double v = u[cidx];
    if (STAGE == 2) v = fma(k0[cidx], c1, v);
    s[j][i] = v;
    if constexpr (SQ) q[j][i] = v * v;
  };
  for (int j = ty; j < TY + 2; j += BY) stage(j, tx + 1);  // interior columns
  {
    // the two halo columns, 2 (TY + 2) values, in the block's first warps
    const int e = ty * TX + tx;
    if (e < 2 * (TY + 2)) stage(e % (TY + 2), e < TY + 2 ? 0 : TX + 1);
  }
  __syncthreads();
  auto xface = [&](int j, int i) {  // 4 g through the x face between tile columns i - 1 and i of row j
    if (BND && p.bkind[0] >= 0 && x0 + i == 0) return 4.0 * boundary_face_flux(p, 2, 0, false, s[j + 1][i + 1]);
    if (BND && p.bkind[0] >= 0 && x0 + i == nx) return 4.0 * boundary_face_flux(p, 2, 0, true, s[j + 1][i]);
    if constexpr (SQ) return face4s<FORM>(p, 0, s[j + 1][i], s[j + 1][i + 1], q[j + 1][i], q[j + 1][i + 1]);
    else return face4s<FORM>(p, 0, s[j + 1][i], s[j + 1][i + 1], 0.0, 0.0);
  };
  for (int j = ty; j < TY; j += BY) gx[j][tx] = xface(j, tx);
  if (ty == 0) gx[tx][TX] = xface(tx, TX);  // the right face of every row: one pass of the first warp
  for (int j = ty; j <= TY; j += BY) {
    double f;
    if (BND && p.bkind[2] >= 0 && y0 + j == 0) f = 4.0 * boundary_face_flux(p, 2, 1, false, s[j + 1][tx + 1]);
    else if (BND && p.bkind[2] >= 0 && y0 + j == ny) f = 4.0 * boundary_face_flux(p, 2, 1, true, s[j][tx + 1]);
    else if constexpr (SQ) f = face4s<FORM>(p, 1, s[j][tx + 1], s[j + 1][tx + 1], q[j][tx + 1], q[j + 1][tx + 1]);
    else f = face4s<FORM>(p, 1, s[j][tx + 1], s[j + 1][tx + 1], 0.0, 0.0);
    gy[j][tx] = f;
  }
  __syncthreads();
  const long long gxi = x0 + tx;
  if (gxi >= nx) return;
  for (int j = ty; j < TY; j += BY) {
    const long long gyj = y0 + j;
    if (gyj >= ny) break;
    const double K = fma(rho, gy[j + 1][tx] - gy[j][tx], gx[j][tx + 1] - gx[j][tx]);
    const long long cidx = off + gyj * nx + gxi;
    if (STAGE == 3) out[cidx] = K;
    else if (STAGE == 0) out[cidx] = c_out * K;
    else if (STAGE == 1) out[cidx] = fma(c_out, K, u[cidx]);
    else out[cidx] = fma(c_out, k0[cidx] + K, u[cidx]);
  }
}

FvParams make_params(const GridDesc& g, const gdt_fv_desc* d) {
  FvParams p;
  p.flux = d->flux;
  p.numflux = d->numflux;
  for (int i = 0; i < 3; ++i) p.vel[i] = d->velocity[i];
  p.lf_inv_lambda = d->lf_lambda;
  p.form4 = FORM4_GENERIC;
  p.lam2 = 0.0;
  for (int k = 0; k < 3; ++k) p.tu[k] = p.tv[k] = 0.0;
  if (d->flux == GDT_FLUX_BURGERS) {
    if (d->numflux == GDT_NUMFLUX_LAX_FRIEDRICHS) {
      p.form4 = d->lf_lambda != 0.0 ? FORM4_BURGERS_LF_FIXED : FORM4_BURGERS_LF;
      p.lam2 = d->lf_lambda != 0.0 ? 2.0 / d->lf_lambda : 0.0;
    } else if (d->numflux == GDT_NUMFLUX_ENGQUIST_OSHER) {
      p.form4 = FORM4_BURGERS_EO;
    } else {
      p.form4 = FORM4_BURGERS_UPWIND;
    }
  } else {
    double lam = 0.0;
    for (int k = 0; k < g.dim; ++k) lam = std::max(lam, std::fabs(d->velocity[k]));
    if (d->lf_lambda != 0.0) lam = 1.0 / d->lf_lambda;
    p.form4 = d->numflux == GDT_NUMFLUX_ENGQUIST_OSHER ? FORM4_TRANSPORT_EO : FORM4_TRANSPORT_LINEAR;
    for (int k = 0; k < 3; ++k) {
      const double a = d->velocity[k];
      if (d->numflux == GDT_NUMFLUX_LAX_FRIEDRICHS) {  // 2 (a (u + v) + lambda (u - v))
        p.tu[k] = 2.0 * (a + lam);
        p.tv[k] = 2.0 * (a - lam);
      } else if (d->numflux == GDT_NUMFLUX_UPWIND) {  // 4 a u if a > 0 else 4 a v
        p.tu[k] = a > 0.0 ? 4.0 * a : 0.0;
        p.tv[k] = a > 0.0 ? 0.0 : 4.0 * a;
      } else {  // EO: 4 (u max(a, 0) + v min(a, 0)), each for a positive state
        p.tu[k] = 4.0 * std::max(a, 0.0);
        p.tv[k] = 4.0 * std::min(a, 0.0);
      }
    }
  }
  for (int side = 0; side < 6; ++side) {
    // a side is periodic when the grid is and no treatment is given; otherwise the treatment (or none)
    const bool periodic = g.periodic && d->boundary[side] == GDT_FV_BOUNDARY_NONE;
    p.bkind[side] = periodic ? -1 : d->boundary[side];
    p.bval[side] = d->boundary_value[side];
  }
  return p;
}

bool has_boundary(const FvParams& p, int dim) {
  for (int side = 0; side < 2 * dim; ++side)
    if (p.bkind[side] >= 0) return true;
  return false;
}

template <int STAGE, bool BND>
void launch_tile_b(dim3 grid, cudaStream_t s, const GridDesc& g, const FvParams& p, const double* u, const double* k0,
                   double* out, double c1, double c_out, double rho) {
  const dim3 block(TX, BY);
  switch (p.form4) {
    case FORM4_BURGERS_LF: fv2d_tile<STAGE, BND, FORM4_BURGERS_LF><<<grid, block, 0, s>>>(g, p, u, k0, out, c1, c_out, rho); break;
    case FORM4_BURGERS_LF_FIXED:
      fv2d_tile<STAGE, BND, FORM4_BURGERS_LF_FIXED><<<grid, block, 0, s>>>(g, p, u, k0, out, c1, c_out, rho);
      break;
    case FORM4_TRANSPORT_LINEAR:
      fv2d_tile<STAGE, BND, FORM4_TRANSPORT_LINEAR><<<grid, block, 0, s>>>(g, p, u, k0, out, c1, c_out, rho);
      break;
    case FORM4_BURGERS_EO: fv2d_tile<STAGE, BND, FORM4_BURGERS_EO><<<grid, block, 0, s>>>(g, p, u, k0, out, c1, c_out, rho); break;
    case FORM4_TRANSPORT_EO:
      fv2d_tile<STAGE, BND, FORM4_TRANSPORT_EO><<<grid, block, 0, s>>>(g, p, u, k0, out, c1, c_out, rho);
      break;
    case FORM4_BURGERS_UPWIND:
      fv2d_tile<STAGE, BND, FORM4_BURGERS_UPWIND><<<grid, block, 0, s>>>(g, p, u, k0, out, c1, c_out, rho);
      break;
    default: fv2d_tile<STAGE, BND, FORM4_GENERIC><<<grid, block, 0, s>>>(g, p, u, k0, out, c1, c_out, rho); break;
  }
}

// one stage of the tiled 2D kernel, instantiated for the flux form and the boundary case
template <int STAGE>
void launch_tile(bool bnd, dim3 grid, cudaStream_t s, const GridDesc& g, const FvParams& p, const double* u,
                 const double* k0, double* out, double c1, double c_out, double rho) {
  if (bnd) launch_tile_b<STAGE, true>(grid, s, g, p, u, k0, out, c1, c_out, rho);
  else launch_tile_b<STAGE, false>(grid, s, g, p, u, k0, out, c1, c_out, rho);
}

bool tiled_ok(const GridDesc& g) { return g.dim == 2 && g.n[0] >= 2 && g.n[1] >= 2; }

}  // namespace

gdt_status fv_apply(gdt_context ctx, const gdt_space_s& sp, const gdt_fv_desc* d, const double* u, double* out) {
  const GridDesc& g = sp.g;
  FvParams p = make_params(g, d);
  if (tiled_ok(g)) {
    dim3 grid((unsigned)((g.n[0] + TX - 1) / TX), (unsigned)((g.n[1] + TY - 1) / TY), 1);
    // L(u) = K / (4 h_x), K = dx + (h_x / h_y) dy
    launch_tile<0>(has_boundary(p, 2), grid, ctx->stream, g, p, u, nullptr, out, 0.0, 0.25 / g.h[0], g.h[0] / g.h[1]);
  } else {
    fv_apply_kernel<<<grid_blocks(g.nelem, 256), 256, 0, ctx->stream>>>(g, p, 1, u, out, nullptr, 0.0, 0, nullptr,
                                                                        0.0);
  }
  return check_launch(ctx, "fv_apply");
}

gdt_status fv_estimate_dt(gdt_context ctx, const gdt_space_s& sp, const gdt_fv_desc* d, const double* u0,
                          double* dt) {
  // data range of the (elementwise constant) state, then the reference's formula on the host:
  // f' sampled at the Gauss points of order flux.order() on [min, max]; dt = 1 / (max |I|/|E| * max |f'|)
  const GridDesc& g = sp.g;
  cudaStream_t s = ctx->stream;
  double* dminmax = nullptr;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&dminmax, 2 * sizeof(double), s));
  size_t b1 = 0, b2 = 0;
  cub::DeviceReduce::Min(nullptr, b1, u0, dminmax, (int)g.nelem, s);
  cub::DeviceReduce::Max(nullptr, b2, u0, dminmax + 1, (int)g.nelem, s);
  void* tmp = nullptr;
  GDT_TRY_CUDA(ctx, cudaMallocAsync(&tmp, std::max(b1, b2), s));
  cub::DeviceReduce::Min(tmp, b1, u0, dminmax, (int)g.nelem, s);
  cub::DeviceReduce::Max(tmp, b2, u0, dminmax + 1, (int)g.nelem, s);
  double mm[2];
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(mm, dminmax, sizeof(mm), cudaMemcpyDeviceToHost, s));
  GDT_TRY_CUDA(ctx, cudaFreeAsync(tmp, s));
  GDT_TRY_CUDA(ctx, cudaFreeAsync(dminmax, s));
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
  ctx->launches += 4;
  double data_minimum = std::min(std::numeric_limits<double>::max(), mm[0]);
  double data_maximum = std::max(std::numeric_limits<double>::min(), mm[1]);
  if (!(data_minimum < data_maximum)) data_maximum = data_minimum + 1e-6 * data_minimum;
  double max_df = std::numeric_limits<double>::min();
  // Gauss points on [0,1]: order 2 (Burgers) -> 2 points, order 1 (transport) -> 1 point
  const double g2 = 0.5 / std::sqrt(3.0);
  const double pts2[2] = {0.5 - g2, 0.5 + g2};
  const double pts1[1] = {0.5};
  const double* pts = d->flux == GDT_FLUX_BURGERS ? pts2 : pts1;
  const int npts = d->flux == GDT_FLUX_BURGERS ? 2 : 1;
  for (int q = 0; q < npts; ++q) {
    const double uq = data_minimum + (data_maximum - data_minimum) * pts[q];
    for (int ss = 0; ss < g.dim; ++ss) {
      const double df = d->flux == GDT_FLUX_BURGERS ? uq : d->velocity[ss];
      max_df = std::max(max_df, std::fabs(df));
    }
  }
  double vol = 1.0;
  for (int a = 0; a < g.dim; ++a) vol *= g.h[a];
  double perimeter = 0.0;
  for (int k = 0; k < g.dim; ++k) {
    double area = 1.0;
    for (int j = 0; j < g.dim; ++j)
      if (j != k) area *= g.h[j];
    perimeter += 2 * area;
  }
  const double pov = std::max(std::numeric_limits<double>::min(), perimeter / vol);
  *dt = 1.0 / (pov * max_df);
  return GDT_OK;
}

gdt_status fv_timestep(gdt_context ctx, const gdt_space_s& sp, const gdt_fv_desc* d, int stepper, double dt,
                       long long steps, long long nbatch, double* u, double* work) {
  // work holds 2 * nbatch * N doubles for SSP-RK2 (k0 and the next state), nbatch * N for Euler
  const GridDesc& g = sp.g;
  const FvParams p = make_params(g, d);
  cudaStream_t s = ctx->stream;
  const long long N = g.nelem * nbatch;
  double* cur = u;
  double* nxt = (stepper == GDT_TIMESTEPPER_SSPRK2) ? work + N : work;
  double* k0 = work;
  const bool tiled = tiled_ok(g);
  const bool bnd = has_boundary(p, g.dim);
  dim3 grid((unsigned)((g.n[0] + TX - 1) / TX), (unsigned)((g.n[1] + TY - 1) / TY), (unsigned)nbatch);
  // the tiled kernels' update K = dx + rho dy with L(u) = K / (4 h_x): the stepper keeps K0 = K(u) itself
  // (k0 = L(u) = K0 / (4 h_x)) and folds the factor into its coefficients
  const double rho = tiled ? g.h[0] / g.h[1] : 0.0, ck = 0.25 / g.h[0];
  for (long long st = 0; st < steps; ++st) {
    if (stepper == GDT_TIMESTEPPER_EXPLICIT_EULER) {
      if (tiled)
        launch_tile<1>(bnd, grid, s, g, p, cur, nullptr, nxt, 0.0, -dt * ck, rho);
      else
        fv_apply_kernel<<<grid_blocks(N, 256), 256, 0, s>>>(g, p, nbatch, cur, nullptr, nullptr, 0.0, 1, nxt, dt);
      ctx->launches++;
    } else {
      if (tiled) {
        launch_tile<3>(bnd, grid, s, g, p, cur, nullptr, k0, 0.0, 1.0, rho);
        launch_tile<2>(bnd, grid, s, g, p, cur, k0, nxt, -dt * ck, -0.5 * dt * ck, rho);
      } else {
        fv_apply_kernel<<<grid_blocks(N, 256), 256, 0, s>>>(g, p, nbatch, cur, k0, nullptr, 0.0, 0, nullptr, 0.0);
        fv_apply_kernel<<<grid_blocks(N, 256), 256, 0, s>>>(g, p, nbatch, nullptr, k0, cur, -dt, 2, nxt, -0.5 * dt);
      }
      ctx->launches += 2;
    }
    std::swap(cur, nxt);
  }
  {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, GDT_ECUDA, std::string("fv_timestep: ") + cudaGetErrorString(e));
  }
  if (cur != u) GDT_TRY_CUDA(ctx, cudaMemcpyAsync(u, cur, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
  return GDT_OK;
}

}  // namespace gdt
