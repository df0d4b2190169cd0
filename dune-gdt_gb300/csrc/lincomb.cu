// Parametric linear combinations: out = sum_q theta_q term_q over FP64 arrays, and over the values
// of matrices that share one sparsity pattern. This is the assembled form of pyMOR's LincombOperator
// over dune-gdt matrices (the affine decompositions of the parametric examples: one matrix per
// coefficient function, python/dune/gdt/gamm-2019-talk-on-conservative-rb.cc:74-95, combined with
// the parameter functionals of examples/gamm_2019_talk_on_conservative_rb_OS2015_academic_example.py:62-77).
//
// GB300 design: HBM-bound streaming, (nterms + 1) * 8 bytes per entry. Each thread moves 16-byte
// pairs of every term (all arrays from the caching allocator or the library are 16-byte aligned;
// a misaligned pointer falls back to the scalar loop), the grid is a fixed number of waves over the
// SMs, and the accumulation order is the term order (deterministic).
#include <cstdint>

#include "internal.cuh"

namespace gdt {
namespace {

struct Terms {
  const double* p[GDT_LINCOMB_MAX_TERMS];
  double theta[GDT_LINCOMB_MAX_TERMS];
  int n;
};

template <int Q>
__global__ void __launch_bounds__(256) k_lincomb2(long long npairs, Terms t, double* __restrict__ out) {
  const int nq = Q > 0 ? Q : t.n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npairs;
       i += (long long)gridDim.x * blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
#pragma unroll
    for (int q = 0; q < (Q > 0 ? Q : GDT_LINCOMB_MAX_TERMS); ++q) {
      if (q >= nq) break;
      const double2 v = __ldcs(reinterpret_cast<const double2*>(t.p[q]) + i);
      acc.x = fma(t.theta[q], v.x, acc.x);
      acc.y = fma(t.theta[q], v.y, acc.y);
    }
    __stcs(reinterpret_cast<double2*>(out) + i, acc);
  }
}

__global__ void __launch_bounds__(256) k_lincomb1(long long begin, long long n, Terms t, double* __restrict__ out) {
  for (long long i = begin + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int q = 0; q < t.n; ++q) acc = fma(t.theta[q], t.p[q][i], acc);
    out[i] = acc;
  }
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

gdt_status lincomb(gdt_context ctx, long long n, const Terms& t, double* out) {
  if (n == 0) return GDT_OK;
  bool vec = aligned16(out);
  for (int q = 0; q < t.n; ++q) vec = vec && aligned16(t.p[q]);
  const int blocks_cap = ctx->num_sms * 8;
  long long done = 0;
  if (vec && n >= 2) {
    const long long npairs = n / 2;
    const int blocks = int(std::min<long long>((npairs + 255) / 256, blocks_cap));
    switch (t.n) {
      case 1: k_lincomb2<1><<<blocks, 256, 0, ctx->stream>>>(npairs, t, out); break;
      case 2: k_lincomb2<2><<<blocks, 256, 0, ctx->stream>>>(npairs, t, out); break;
      case 3: k_lincomb2<3><<<blocks, 256, 0, ctx->stream>>>(npairs, t, out); break;
      case 4: k_lincomb2<4><<<blocks, 256, 0, ctx->stream>>>(npairs, t, out); break;
      default: k_lincomb2<0><<<blocks, 256, 0, ctx->stream>>>(npairs, t, out); break;
    }
    ctx->launches++;
    done = 2 * npairs;
  }
  if (done < n) {
    const int blocks = int(std::min<long long>((n - done + 255) / 256, blocks_cap));
    k_lincomb1<<<blocks, 256, 0, ctx->stream>>>(done, n, t, out);
    ctx->launches++;
  }
  return check_launch(ctx, "lincomb");
}

// patterns are built deterministically from the spaces and the stencil: equal inputs, equal patterns
bool same_pattern(const gdt_matrix_s& a, const gdt_matrix_s& b) {
  auto same_space = [](const gdt_space_s& x, const gdt_space_s& y) {
    return x.kind == y.kind && x.order == y.order && x.size == y.size && x.g.dim == y.g.dim &&
           x.g.simplex == y.g.simplex && x.g.periodic == y.g.periodic && x.g.n[0] == y.g.n[0] &&
           x.g.n[1] == y.g.n[1] && x.g.n[2] == y.g.n[2];
  };
  return a.stencil == b.stencil && a.rows == b.rows && a.cols == b.cols && a.nnz == b.nnz &&
         same_space(a.test, b.test) && same_space(a.ansatz, b.ansatz);
}

}  // namespace
}  // namespace gdt

using namespace gdt;

extern "C" {

gdt_status gdt_lincomb(gdt_context ctx, int64_t n, int nterms, const double* const* terms, const double* theta,
                       double* out) {
  if (!ctx || !terms || !theta || !out || n < 0 || nterms < 1 || nterms > GDT_LINCOMB_MAX_TERMS) return GDT_EINVAL;
  Terms t{};
  t.n = nterms;
  for (int q = 0; q < nterms; ++q) {
    if (!terms[q]) return GDT_EINVAL;
    t.p[q] = terms[q];
    t.theta[q] = theta[q];
  }
  return lincomb(ctx, n, t, out);
}

gdt_status gdt_matrix_lincomb(gdt_context ctx, gdt_matrix out, int nterms, const gdt_matrix* terms,
                              const double* theta) {
  if (!ctx || !out || !terms || !theta || nterms < 1 || nterms > GDT_LINCOMB_MAX_TERMS) return GDT_EINVAL;
  Terms t{};
  t.n = nterms;
  for (int q = 0; q < nterms; ++q) {
    if (!terms[q]) return GDT_EINVAL;
    if (!same_pattern(*out, *terms[q])) return fail(ctx, GDT_ESHAPE, "lincomb terms must share the sparsity pattern");
    t.p[q] = terms[q]->val;
    t.theta[q] = theta[q];
  }
  out->mf_valid = 0;
  out->val_version++;
  return lincomb(ctx, out->nnz, t, out->val);
}

}  // extern "C"
