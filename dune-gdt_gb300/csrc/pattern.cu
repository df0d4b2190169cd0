// Sparsity patterns built on the device, equal entry for entry to the reference's
// make_element_sparsity_pattern / make_element_and_intersection_sparsity_pattern + sort()
// (tools/sparsity-pattern.hh:33-50, 117-144) for the structured grids of this library.
#include <cub/device/device_reduce.cuh>
#include <cub/device/device_scan.cuh>

#include "highorder.cuh"
#include "structured.cuh"

namespace gdt {
namespace {

// continuous P1/Q1: row v holds every vertex sharing an element with v, ascending
template <int DIM, bool SIMPLEX, bool FILL>
__global__ void cg_pattern_kernel(GridDesc g, int* __restrict__ row_nnz, const int* __restrict__ rp,
                                  int* __restrict__ col) {
  long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (v >= g.nvert) return;
  long long vi[3];
  vertex_multi(g, v, vi);
  int cnt = 0;
  long long pos = FILL ? rp[v] : 0;
#pragma unroll
  for (int k = 0; k < pow3(DIM); ++k) {
    if (!slot_in_stencil(DIM, SIMPLEX, k)) continue;
    bool ok = true;
    long long w = 0, stride = 1;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      long long x = vi[a] + slot_offset(k, a);
      ok = ok && x >= 0 && x < g.vn[a];
      w += x * stride;
      stride *= g.vn[a];
    }
    if (!ok) continue;
    if (FILL) col[pos + cnt] = int(w);
    ++cnt;
  }
  if (!FILL) row_nnz[v] = cnt;
}

// DG order 1: all local rows of element e share the sorted neighbour blocks
template <bool FILL>
__global__ void dg_pattern_kernel(GridDesc g, int lsize, int stencil, int* __restrict__ row_nnz,
                                  const int* __restrict__ rp, int* __restrict__ col) {
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= g.nelem) return;
  long long nb[8];
  int k = 1;
  if (stencil == GDT_STENCIL_ELEMENT) nb[0] = e;  // the element block only
  else k = dg_neighbours(g, e, stencil != GDT_STENCIL_INTERSECTION, nb);
  for (int i = 0; i < lsize; ++i) {
    long long row = e * lsize + i;
    if (!FILL) {
      row_nnz[row] = k * lsize;
      continue;
    }
    long long pos = rp[row];
    for (int b = 0; b < k; ++b)
      for (int j = 0; j < lsize; ++j) col[pos++] = int(nb[b] * lsize + j);
  }
}

template <int DIM, bool SIMPLEX>
void launch_cg_pattern(const GridDesc& g, bool fill, int* row_nnz, const int* rp, int* col, cudaStream_t s) {
  int th = 256;
  int bl = grid_blocks(g.nvert, th);
  if (fill)
    cg_pattern_kernel<DIM, SIMPLEX, true><<<bl, th, 0, s>>>(g, row_nnz, rp, col);
  else
    cg_pattern_kernel<DIM, SIMPLEX, false><<<bl, th, 0, s>>>(g, row_nnz, rp, col);
}

void dispatch_cg_pattern(const GridDesc& g, bool fill, int* row_nnz, const int* rp, int* col, cudaStream_t s) {
  if (g.dim == 1) launch_cg_pattern<1, false>(g, fill, row_nnz, rp, col, s);
  else if (g.dim == 2 && !g.simplex) launch_cg_pattern<2, false>(g, fill, row_nnz, rp, col, s);
  else if (g.dim == 2) launch_cg_pattern<2, true>(g, fill, row_nnz, rp, col, s);
  else if (!g.simplex) launch_cg_pattern<3, false>(g, fill, row_nnz, rp, col, s);
  else launch_cg_pattern<3, true>(g, fill, row_nnz, rp, col, s);
}

__global__ void global_indices_kernel(GridDesc g, int kind, int lsize, long long* __restrict__ out) {
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= g.nelem) return;
  if (kind == GDT_SPACE_FV) {
    out[e] = e;
    return;
  }
  if (kind == GDT_SPACE_DG) {
    for (int i = 0; i < lsize; ++i) out[e * lsize + i] = e * lsize + i;
    return;
  }
  long long c = e / g.nsub;
  int t = int(e % g.nsub);
  long long ci[3];
  cell_multi(g, c, ci);
  for (int j = 0; j < lsize; ++j) {
    int corner = local_corner(g.dim, g.simplex != 0, t, j);
    long long v = 0, stride = 1;
    for (int a = 0; a < g.dim; ++a) {
      v += (ci[a] + ((corner >> a) & 1)) * stride;
      stride *= g.vn[a];
    }
    out[e * lsize + j] = v;
  }
}

}  // namespace

gdt_status build_pattern(gdt_context ctx, gdt_matrix m) {
  if (m->test.kind == GDT_SPACE_CG && m->test.order == 2) return ho_build_pattern(ctx, m);
  if (m->test.g.mesh) return m->test.kind == GDT_SPACE_DG ? mesh_dg_pattern(ctx, m) : mesh_pattern(ctx, m);
  const GridDesc& g = m->test.g;
  cudaStream_t s = ctx->stream;
  const bool dg = m->test.kind == GDT_SPACE_DG;
  if (dg && g.simplex && g.dim != 2) return fail(ctx, GDT_EUNSUPPORTED, "DG patterns on 3D simplex grids");
  long long rows = m->rows;
  int* row_nnz = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&m->rp, sizeof(int) * (rows + 1)));
  GDT_TRY_CUDA(ctx, cudaMalloc(&row_nnz, sizeof(int) * (rows + 1)));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(row_nnz + rows, 0, sizeof(int), s));
  if (dg)
    dg_pattern_kernel<false><<<grid_blocks(g.nelem, 256), 256, 0, s>>>(g, m->test.lsize, m->stencil, row_nnz, nullptr,
                                                                       nullptr);
  else
    dispatch_cg_pattern(g, false, row_nnz, nullptr, nullptr, s);
  GDT_CHECK(ctx, check_launch(ctx, "pattern count"));
  size_t tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, row_nnz, m->rp, rows + 1, s);
  void* tmp = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&tmp, tmp_bytes));
  cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, row_nnz, m->rp, rows + 1, s);
  GDT_CHECK(ctx, check_launch(ctx, "pattern scan"));
  int nnz = 0;
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&nnz, m->rp + rows, sizeof(int), cudaMemcpyDeviceToHost, s));
  int* dmax = nullptr;
  size_t max_bytes = 0;
  GDT_TRY_CUDA(ctx, cudaMalloc(&dmax, sizeof(int)));
  cub::DeviceReduce::Max(nullptr, max_bytes, row_nnz, dmax, int(rows), s);
  void* tmax = nullptr;
  GDT_TRY_CUDA(ctx, cudaMalloc(&tmax, max_bytes));
  cub::DeviceReduce::Max(tmax, max_bytes, row_nnz, dmax, int(rows), s);
  GDT_TRY_CUDA(ctx, cudaMemcpyAsync(&m->max_row, dmax, sizeof(int), cudaMemcpyDeviceToHost, s));
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(s));
  cudaFree(tmax);
  cudaFree(dmax);
  cudaFree(tmp);
  cudaFree(row_nnz);
  m->nnz = nnz;
  // a few elements of padding so that vectorised/staged loads of a row slice never leave the arrays
  GDT_TRY_CUDA(ctx, cudaMalloc(&m->col, sizeof(int) * (nnz + 8)));
  GDT_TRY_CUDA(ctx, cudaMalloc(&m->val, sizeof(double) * (nnz + 8)));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(m->val, 0, sizeof(double) * (nnz + 8), s));
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(m->col, 0, sizeof(int) * (nnz + 8), s));
  if (dg)
    dg_pattern_kernel<true><<<grid_blocks(g.nelem, 256), 256, 0, s>>>(g, m->test.lsize, m->stencil, nullptr, m->rp,
                                                                      m->col);
  else
    dispatch_cg_pattern(g, true, nullptr, m->rp, m->col, s);
  GDT_CHECK(ctx, check_launch(ctx, "pattern fill"));
  // untuned default schedule: vector-CSR with about four entries per lane (the first SpMV-type call
  // replaces it with the autotuner's choice)
  const double mean = rows ? double(nnz) / double(rows) : 1.0;
  m->spmv_sched = mean <= 16 ? 0 : mean <= 32 ? 1 : mean <= 64 ? 2 : 3;
  m->tuned = 0;
  return GDT_OK;
}

}  // namespace gdt

extern "C" gdt_status gdt_space_global_indices(gdt_context ctx, gdt_space s, int64_t* out) {
  if (!ctx || !s || !out) return GDT_EINVAL;
  if (s->kind == GDT_SPACE_CG && s->order == 2) return gdt::ho_global_indices(ctx, *s, out, nullptr);
  if (s->g.mesh && s->kind == GDT_SPACE_CG) return gdt::mesh_global_indices(ctx, s->g, out);
  gdt::global_indices_kernel<<<gdt::grid_blocks(s->g.nelem, 256), 256, 0, ctx->stream>>>(
      s->g, s->kind, s->lsize, reinterpret_cast<long long*>(out));
  return gdt::check_launch(ctx, "global indices");
}
