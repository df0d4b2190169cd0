// C ABI entry points: handle management, argument validation and dispatch to the kernels.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "highorder.cuh"
#include "internal.cuh"

namespace gdt {

gdt_status fail(gdt_context ctx, gdt_status s, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return s;
}

gdt_status check_launch(gdt_context ctx, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(ctx, GDT_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
  if (ctx) ctx->launches++;
  return GDT_OK;
}

void timing_begin(gdt_context ctx, cudaStream_t s, int kind) {
  if (!ctx->timing) return;
  if (ctx->events_used + 2 > ctx->events.size()) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    ctx->events.push_back(a);
    ctx->events.push_back(b);
    ctx->event_kind.push_back(kind);
  }
  ctx->event_kind[ctx->events_used / 2] = kind;
  cudaEventRecord(ctx->events[ctx->events_used], s);
}

void timing_end(gdt_context ctx, cudaStream_t s) {
  if (!ctx->timing) return;
  cudaEventRecord(ctx->events[ctx->events_used + 1], s);
  ctx->events_used += 2;
}

void timing_harvest(gdt_context ctx) {
  for (size_t k = 0; k + 1 < ctx->events_used; k += 2) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->events[k], ctx->events[k + 1]) == cudaSuccess) {
      const int kind = ctx->event_kind[k / 2];
      ctx->kind_ms[kind] += ms;
      ctx->kind_launches[kind] += 1;
    }
  }
  ctx->events_used = 0;
}

}  // namespace gdt

using namespace gdt;

extern "C" {

const char* gdt_status_string(gdt_status s) {
  switch (s) {
    case GDT_OK: return "ok";
    case GDT_EINVAL: return "invalid argument";
    case GDT_ESHAPE: return "shape mismatch";
    case GDT_ENOCONV: return "linear solver did not converge";
    case GDT_ETIMEOUT: return "device wait exceeded its iteration budget";
    case GDT_ENAN: return "non-finite value";
    case GDT_EUNSUPPORTED: return "not supported by the GPU library";
    case GDT_ECUDA: return "CUDA error";
    case GDT_ENOMEM: return "out of device memory";
  }
  return "unknown status";
}

gdt_status gdt_context_create(int device, void* stream, gdt_context* out) {
  if (!out) return GDT_EINVAL;
  *out = nullptr;
  gdt_context ctx = new (std::nothrow) gdt_context_s;
  if (!ctx) return GDT_ENOMEM;
  ctx->device = device;
  ctx->stream = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->scratch, sizeof(double) * kScratchDoubles);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->counters, sizeof(unsigned int) * kCounters);
  if (e == cudaSuccess) e = cudaMemset(ctx->counters, 0, sizeof(unsigned int) * kCounters);
  if (e == cudaSuccess) e = cudaMallocHost(&ctx->host_pinned, sizeof(double) * 64);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    gdt_context_destroy(ctx);
    return GDT_ECUDA;
  }
  *out = ctx;
  return GDT_OK;
}

gdt_status gdt_context_set_timing(gdt_context ctx, int enable) {
  if (!ctx) return GDT_EINVAL;
  ctx->timing = enable ? 1 : 0;
  return GDT_OK;
}

gdt_status gdt_context_set_solver_launch(gdt_context ctx, int mode) {
  if (!ctx || mode < GDT_SOLVER_LAUNCH_AUTO || mode > GDT_SOLVER_LAUNCH_PERSISTENT) return GDT_EINVAL;
  ctx->solver_launch = mode;
  return GDT_OK;
}

int gdt_context_last_solver_launch(gdt_context ctx) { return ctx ? ctx->last_solver_launch : 0; }

gdt_status gdt_context_set_persistent_limits(gdt_context ctx, int blocks, int64_t wait_limit_ns) {
  if (!ctx || blocks < 0 || wait_limit_ns < 0) return GDT_EINVAL;
  ctx->persistent_blocks = blocks;
  ctx->persistent_wait_ns = wait_limit_ns;
  return GDT_OK;
}

gdt_status gdt_context_spmv_timing(gdt_context ctx, double* fp64_ms, int64_t* fp64_launches, double* fp32_ms,
                                   int64_t* fp32_launches, int reset) {
  if (!ctx) return GDT_EINVAL;
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  timing_harvest(ctx);
  if (fp64_ms) *fp64_ms = ctx->kind_ms[GDT_TIMING_SPMV_FP64];
  if (fp64_launches) *fp64_launches = ctx->kind_launches[GDT_TIMING_SPMV_FP64];
  if (fp32_ms) *fp32_ms = ctx->kind_ms[GDT_TIMING_SPMV_FP32];
  if (fp32_launches) *fp32_launches = ctx->kind_launches[GDT_TIMING_SPMV_FP32];
  if (reset)
    for (int k = 0; k < GDT_TIMING_KINDS; ++k) ctx->kind_ms[k] = 0.0, ctx->kind_launches[k] = 0;
  return GDT_OK;
}

gdt_status gdt_context_kernel_timing(gdt_context ctx, int kind, double* ms, int64_t* launches, int reset) {
  if (!ctx || kind < 0 || kind >= GDT_TIMING_KINDS) return GDT_EINVAL;
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  timing_harvest(ctx);
  if (ms) *ms = ctx->kind_ms[kind];
  if (launches) *launches = ctx->kind_launches[kind];
  if (reset) ctx->kind_ms[kind] = 0.0, ctx->kind_launches[kind] = 0;
  return GDT_OK;
}

gdt_status gdt_context_destroy(gdt_context ctx) {
  if (!ctx) return GDT_EINVAL;
  for (cudaEvent_t e : ctx->events) cudaEventDestroy(e);
  if (ctx->scratch) cudaFree(ctx->scratch);
  if (ctx->counters) cudaFree(ctx->counters);
  if (ctx->host_pinned) cudaFreeHost(ctx->host_pinned);
  delete ctx;
  return GDT_OK;
}

gdt_status gdt_context_set_stream(gdt_context ctx, void* stream) {
  if (!ctx) return GDT_EINVAL;
  ctx->stream = static_cast<cudaStream_t>(stream);
  return GDT_OK;
}

gdt_status gdt_context_synchronize(gdt_context ctx) {
  if (!ctx) return GDT_EINVAL;
  GDT_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GDT_OK;
}

const char* gdt_context_last_error(gdt_context ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int64_t gdt_context_kernel_launches(gdt_context ctx) { return ctx ? ctx->launches : 0; }

// ---------------------------------------------------------------------- grid ---
gdt_status gdt_grid_create_cube(int dim, const int64_t* num_elements, const double* lower_left,
                                const double* upper_right, int simplex, int periodic, gdt_grid* out) {
  if (!out || !num_elements || !lower_left || !upper_right) return GDT_EINVAL;
  *out = nullptr;
  if (dim < 1 || dim > 3) return GDT_EINVAL;
  if (simplex && periodic) return GDT_EUNSUPPORTED;
  gdt_grid g = new (std::nothrow) gdt_grid_s;
  if (!g) return GDT_ENOMEM;
  GridDesc& d = g->d;
  d.dim = dim;
  d.simplex = (simplex && dim >= 2) ? 1 : 0;
  d.periodic = periodic ? 1 : 0;
  d.ncells = 1;
  d.nvert = 1;
  for (int i = 0; i < 3; ++i) {
    if (i < dim) {
      if (num_elements[i] < 1 || !(upper_right[i] > lower_left[i])) {
        delete g;
        return GDT_EINVAL;
      }
      d.n[i] = num_elements[i];
      d.lo[i] = lower_left[i];
      d.hi[i] = upper_right[i];
    } else {
      d.n[i] = 1;
      d.lo[i] = 0.0;
      d.hi[i] = 1.0;
    }
    d.h[i] = (d.hi[i] - d.lo[i]) / double(d.n[i]);
    d.vn[i] = i < dim ? d.n[i] + 1 : 1;
    d.ncells *= d.n[i];
    d.nvert *= d.vn[i];
  }
  d.nsub = 1;
  if (d.simplex)
    for (int i = 2; i <= dim; ++i) d.nsub *= i;
  d.nelem = d.ncells * d.nsub;
  if (d.nvert >= (1LL << 31) || d.nelem >= (1LL << 31)) {
    delete g;
    return GDT_EUNSUPPORTED;
  }
  *out = g;
  return GDT_OK;
}

gdt_status gdt_grid_set_vertices(gdt_grid g, const double* coords) {
  if (!g || !coords) return GDT_EINVAL;
  GridDesc& d = g->d;
  if (d.periodic || d.mesh) return GDT_EUNSUPPORTED;
  const size_t bytes = sizeof(double) * size_t(d.nvert) * d.dim;
  double* buf = nullptr;
  if (cudaMalloc(&buf, bytes) != cudaSuccess) {
    cudaGetLastError();
    return GDT_ENOMEM;
  }
  // host or device coordinates (unified addressing)
  if (cudaMemcpy(buf, coords, bytes, cudaMemcpyDefault) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(buf);
    return GDT_ECUDA;
  }
  g->xv_owner = std::shared_ptr<double>(buf, [](double* q) { cudaFree(q); });
  d.xv = buf;
  return GDT_OK;
}

gdt_status gdt_grid_destroy(gdt_grid g) {
  if (!g) return GDT_EINVAL;
  delete g;
  return GDT_OK;
}

int64_t gdt_grid_num_elements(gdt_grid g) { return g ? g->d.nelem : -1; }
int64_t gdt_grid_num_vertices(gdt_grid g) { return g ? g->d.nvert : -1; }

// --------------------------------------------------------------------- space ---
gdt_status gdt_space_create(gdt_grid g, int kind, int order, gdt_space* out) {
  if (!g || !out) return GDT_EINVAL;
  *out = nullptr;
  const GridDesc& d = g->d;
  gdt_space_s s;
  s.g = d;
  s.xv_owner = g->xv_owner;
  s.mesh_owner = g->mesh_owner;
  s.kind = kind;
  s.order = order;
  // mapped grids: continuous order-1 spaces only (their assembly forms each element's geometry)
  // simplex meshes also: DG order 1 on triangles (SWIPDG)
  if (d.xv && !(kind == GDT_SPACE_CG && order == 1) && !(d.mesh && kind == GDT_SPACE_DG && order == 1 && d.dim == 2))
    return GDT_EUNSUPPORTED;
  if (kind == GDT_SPACE_CG) {
    if (order != 1 && order != 2) return GDT_EUNSUPPORTED;
    if (d.periodic) return GDT_EUNSUPPORTED;
    if (order == 1) {
      s.lsize = d.simplex ? d.dim + 1 : (1 << d.dim);
      s.size = d.nvert;
    } else {
      const ho::HoSpaceInfo info = ho::space_info(d, order);
      s.lsize = info.lsize;
      s.size = info.size;
    }
  } else if (kind == GDT_SPACE_DG) {
    if (order != 1 || d.periodic) return GDT_EUNSUPPORTED;
    s.lsize = d.simplex ? d.dim + 1 : (1 << d.dim);
    s.size = d.nelem * s.lsize;
  } else if (kind == GDT_SPACE_FV) {
    if (order != 0) return GDT_EINVAL;
    if (d.simplex) return GDT_EUNSUPPORTED;
    s.lsize = 1;
    s.size = d.nelem;
  } else {
    return GDT_EINVAL;
  }
  if (s.size >= (1LL << 31)) return GDT_EUNSUPPORTED;
  gdt_space sp = new (std::nothrow) gdt_space_s(s);
  if (!sp) return GDT_ENOMEM;
  *out = sp;
  return GDT_OK;
}

gdt_status gdt_space_destroy(gdt_space s) {
  if (!s) return GDT_EINVAL;
  delete s;
  return GDT_OK;
}

int64_t gdt_space_size(gdt_space s) { return s ? s->size : -1; }
int gdt_space_max_local_size(gdt_space s) { return s ? s->lsize : -1; }

// -------------------------------------------------------------------- matrix ---
gdt_status gdt_matrix_create(gdt_context ctx, gdt_space test, gdt_space ansatz, int stencil, gdt_matrix* out) {
  if (!ctx || !test || !ansatz || !out) return GDT_EINVAL;
  *out = nullptr;
  if (stencil < GDT_STENCIL_ELEMENT || stencil > GDT_STENCIL_ELEMENT_AND_INTERSECTION)
    return fail(ctx, GDT_EINVAL, "unknown stencil");
  if (test->kind != ansatz->kind || test->order != ansatz->order ||
      std::memcmp(test->g.n, ansatz->g.n, sizeof(test->g.n)) != 0 || test->g.simplex != ansatz->g.simplex ||
      test->g.mcells != ansatz->g.mcells)
    return fail(ctx, GDT_EUNSUPPORTED, "test and ansatz space must coincide");
  if (test->kind == GDT_SPACE_FV) return fail(ctx, GDT_EUNSUPPORTED, "no matrix for finite-volume spaces");
  if (test->kind == GDT_SPACE_CG && stencil != GDT_STENCIL_ELEMENT)
    return fail(ctx, GDT_EUNSUPPORTED, "continuous spaces use the element stencil");
  gdt_matrix m = new (std::nothrow) gdt_matrix_s;
  if (!m) return GDT_ENOMEM;
  m->ctx = ctx;
  m->test = *test;
  m->ansatz = *ansatz;
  m->stencil = stencil;
  m->rows = test->size;
  m->cols = ansatz->size;
  gdt_status st = build_pattern(ctx, m);
  if (st != GDT_OK) {
    gdt_matrix_destroy(m);
    return st;
  }
  *out = m;
  return GDT_OK;
}

gdt_status gdt_matrix_destroy(gdt_matrix m) {
  if (!m) return GDT_EINVAL;
  ho_matrix_free(static_cast<HoMatrix*>(m->ho));
  if (m->mf_kappa) cudaFree(m->mf_kappa);
  sell_free(m);
  if (m->rp) cudaFree(m->rp);
  if (m->col) cudaFree(m->col);
  if (m->val) cudaFree(m->val);
  delete m;
  return GDT_OK;
}

int64_t gdt_matrix_rows(gdt_matrix m) { return m ? m->rows : -1; }
int64_t gdt_matrix_cols(gdt_matrix m) { return m ? m->cols : -1; }
int64_t gdt_matrix_nnz(gdt_matrix m) { return m ? m->nnz : -1; }

gdt_status gdt_matrix_device_arrays(gdt_matrix m, const int32_t** rp, const int32_t** col, double** val) {
  if (!m) return GDT_EINVAL;
  if (rp) *rp = m->rp;
  if (col) *col = m->col;
  if (val) {
    *val = m->val;
    m->val_version++;  // the caller may write the values through this pointer
  }
  return GDT_OK;
}

gdt_status gdt_matrix_set_zero(gdt_context ctx, gdt_matrix m) {
  if (!ctx || !m) return GDT_EINVAL;
  m->mf_valid = 0;
  m->val_version++;
  GDT_TRY_CUDA(ctx, cudaMemsetAsync(m->val, 0, sizeof(double) * m->nnz, ctx->stream));
  return GDT_OK;
}

// ------------------------------------------------------------------ assembly ---
gdt_status gdt_assemble_cg_diffusion(gdt_context ctx, gdt_matrix m, const gdt_diffusion_desc* d, double* rhs) {
  if (!ctx || !m || !d) return GDT_EINVAL;
  if (m->test.kind != GDT_SPACE_CG) return fail(ctx, GDT_ESHAPE, "matrix does not belong to a continuous space");
  m->val_version++;
  if (d->force_qp && d->force_quad_order < 0) return fail(ctx, GDT_EINVAL, "negative quadrature order");
  if (m->test.g.xv && (d->kappa_qp || d->kappa_tensor || d->kappa_tensor_qp || d->force_qp))
    return fail(ctx, GDT_EUNSUPPORTED, "mapped grids: kappa and source per element or constant");
  if (m->test.g.mesh) {
    m->mf_valid = 0;
    return mesh_assemble(ctx, m->test.g, m->rp, m->col, m->val, d, rhs, d->dirichlet ? d->dirichlet_values : nullptr,
                         d->dirichlet ? d->dirichlet_value_const : 0.0);
  }
  const bool values = d->dirichlet && (d->dirichlet_values || d->dirichlet_value_const != 0.0);
  if (values && (m->test.order != 1 || d->kappa_qp || d->kappa_tensor || d->kappa_tensor_qp || d->force_qp))
    return fail(ctx, GDT_EUNSUPPORTED, "Dirichlet values are lowered for the order-1 vertex-row assembly");
  // a source at quadrature points: the matrix first, then the load vector from its own pass
  double* rhs_fused = d->force_qp ? nullptr : rhs;
  if (d->kappa_tensor || d->kappa_tensor_qp) {
    m->mf_valid = 0;
    GDT_CHECK(ctx, ho_prepare(ctx, m));
    GDT_CHECK(ctx, ho_assemble_tensor(ctx, m, d->kappa_tensor, d->kappa_tensor_qp, d->force, d->force_const,
                                      rhs_fused, d->dirichlet));
  } else if (m->test.order == 2 || d->kappa_qp) {
    m->mf_valid = 0;
    GDT_CHECK(ctx, ho_prepare(ctx, m));
    GDT_CHECK(ctx, ho_assemble(ctx, m, 0, d->kappa, d->kappa_const, d->kappa_qp, d->force, d->force_const, rhs_fused,
                               d->dirichlet));
  } else {
    GDT_CHECK(ctx, assemble_cg(ctx, m, d, rhs_fused));
  }
  if (d->force_qp && rhs) return ho_rhs_qp(ctx, m->test, d->force_qp, d->force_quad_order, d->dirichlet, rhs);
  return GDT_OK;
}

gdt_status gdt_assemble_cg_rhs(gdt_context ctx, gdt_space s, const gdt_diffusion_desc* d, double* rhs) {
  if (!ctx || !s || !d || !rhs) return GDT_EINVAL;
  if (s->kind != GDT_SPACE_CG) return fail(ctx, GDT_ESHAPE, "not a continuous space");
  if (s->g.mesh && !d->force_qp) return mesh_assemble(ctx, s->g, nullptr, nullptr, nullptr, d, rhs, nullptr, 0.0);
  if (d->force_qp) {
    if (s->g.xv) return fail(ctx, GDT_EUNSUPPORTED, "mapped grids: source per element or constant");
    if (d->force_quad_order < 0) return fail(ctx, GDT_EINVAL, "negative quadrature order");
    return ho_rhs_qp(ctx, *s, d->force_qp, d->force_quad_order, d->dirichlet, rhs);
  }
  if (s->order == 2) return ho_assemble_rhs(ctx, *s, d->force, d->force_const, d->dirichlet, rhs);
  return assemble_cg_rhs(ctx, *s, d, rhs);
}

gdt_status gdt_dirichlet_apply(gdt_context ctx, gdt_matrix m, double* rhs) {
  if (!ctx || !m) return GDT_EINVAL;
  if (m->test.kind != GDT_SPACE_CG) return fail(ctx, GDT_ESHAPE, "matrix does not belong to a continuous space");
  m->val_version++;
  if (m->test.order == 2) return ho_dirichlet(ctx, m, rhs);
  m->mf_dirichlet = 1;
  if (m->test.g.mesh) return mesh_dirichlet(ctx, m, rhs, nullptr, 0.0);
  return dirichlet_apply(ctx, m, rhs);
}

gdt_status gdt_dirichlet_apply_values(gdt_context ctx, gdt_matrix m, double* rhs, const double* values,
                                      double value_const) {
  if (!ctx || !m || !rhs) return GDT_EINVAL;
  if (m->test.kind != GDT_SPACE_CG) return fail(ctx, GDT_ESHAPE, "matrix does not belong to a continuous space");
  if (m->test.order != 1) return fail(ctx, GDT_EUNSUPPORTED, "Dirichlet values are lowered for order 1");
  m->val_version++;
  m->mf_dirichlet = 1;
  if (m->test.g.mesh) return mesh_dirichlet(ctx, m, rhs, values, value_const);
  return dirichlet_apply(ctx, m, rhs, values, value_const);
}

gdt_status gdt_assemble_cg_product(gdt_context ctx, gdt_matrix m, const gdt_product_desc* d) {
  if (!ctx || !m || !d) return GDT_EINVAL;
  if (m->test.kind != GDT_SPACE_CG) return fail(ctx, GDT_ESHAPE, "matrix does not belong to a continuous space");
  if (m->test.g.xv) return fail(ctx, GDT_EUNSUPPORTED, "mapped grids: the Laplace form only");
  m->mf_valid = 0;
  m->val_version++;
  GDT_CHECK(ctx, ho_prepare(ctx, m));
  return ho_assemble(ctx, m, 1, d->weight, d->weight_const, d->weight_qp, nullptr, 0.0, nullptr, 0);
}

int gdt_space_quadrature(gdt_space s, double* x_ref, double* w_ref) {
  if (!s || s->kind != GDT_SPACE_CG) return -1;
  return ho_quadrature(*s, x_ref, w_ref);
}

int gdt_space_quadrature_order(gdt_space s, int quad_order, double* x_ref, double* w_ref) {
  if (!s || quad_order < 0 || quad_order > 40) return -1;
  return quadrature_order(*s, quad_order, x_ref, w_ref);
}

gdt_status gdt_element_error(gdt_context ctx, gdt_space s, int norm, int quad_order, const double* u,
                             const double* ref_qp, double* eta2, double* total) {
  if (!ctx || !s || !u || !ref_qp || !eta2) return GDT_EINVAL;
  if (norm != GDT_NORM_H1_SEMI && norm != GDT_NORM_L2) return fail(ctx, GDT_EINVAL, "unknown norm");
  if (quad_order < 0 || quad_order > 40) return fail(ctx, GDT_EINVAL, "quadrature order out of range");
  if (s->kind == GDT_SPACE_FV || (s->kind == GDT_SPACE_DG && s->order != 1))
    return fail(ctx, GDT_EUNSUPPORTED, "element error of continuous (order 1, 2) and DG (order 1) spaces");
  if (s->g.mesh) return mesh_element_error(ctx, *s, norm, quad_order, u, ref_qp, eta2, total);
  if (s->g.xv) return fail(ctx, GDT_EUNSUPPORTED, "element error on mapped grids");
  return element_error(ctx, *s, norm, quad_order, u, ref_qp, eta2, total);
}

gdt_status gdt_assemble_swipdg(gdt_context ctx, gdt_matrix m, const gdt_ipdg_desc* d, double* rhs) {
  if (!ctx || !m || !d) return GDT_EINVAL;
  if (m->test.kind != GDT_SPACE_DG) return fail(ctx, GDT_ESHAPE, "matrix does not belong to a DG space");
  if (m->stencil != GDT_STENCIL_ELEMENT_AND_INTERSECTION)
    return fail(ctx, GDT_ESHAPE, "SWIPDG needs the element_and_intersection stencil");
  m->val_version++;
  if (m->test.g.mesh) return mesh_swipdg(ctx, m, d, rhs);
  return assemble_swipdg(ctx, m, d, rhs);
}

gdt_status gdt_dg_face_points(gdt_space dg, double* xy) {
  if (!dg || !xy || dg->kind != GDT_SPACE_DG) return GDT_EINVAL;
  if (dg->g.mesh) return mesh_dg_face_points(*dg, xy);
  return dg_face_points(*dg, xy);
}

// local/integrands/elliptic-ipdg.hh:452-501 (inner_sigma, boundary_sigma) and :442-445 (default_beta)
double gdt_elliptic_ipdg_sigma(int pol_order, int boundary) {
  if (boundary) return pol_order <= 1 ? 14.0 : pol_order <= 2 ? 38.0 : pol_order <= 3 ? 74.0 : 100.0;
  return pol_order <= 1 ? 8.0 : pol_order <= 2 ? 20.0 : pol_order <= 3 ? 38.0 : 50.0;
}
double gdt_elliptic_ipdg_beta(int dim) { return dim > 1 ? 1.0 / (dim - 1.0) : 1.0; }

gdt_status gdt_spmv(gdt_context ctx, gdt_matrix m, const double* x, double* y) {
  if (!ctx || !m || !x || !y) return GDT_EINVAL;
  return spmv(ctx, m, x, y);
}

gdt_status gdt_solve(gdt_context ctx, gdt_matrix m, const double* b, double* x, const gdt_solver_opts* o,
                     gdt_solve_info* info) {
  if (!ctx || !m || !b || !x || !o) return GDT_EINVAL;
  if (m->rows != m->cols) return fail(ctx, GDT_ESHAPE, "matrix is not square");
  if (o->solver != GDT_SOLVER_CG && o->solver != GDT_SOLVER_BICGSTAB) return fail(ctx, GDT_EINVAL, "unknown solver");
  if (o->precond < GDT_PREC_NONE || o->precond > GDT_PREC_ILU0) return fail(ctx, GDT_EINVAL, "unknown preconditioner");
  if (o->precision != GDT_PRECISION_FP64 && o->precision != GDT_PRECISION_MIXED)
    return fail(ctx, GDT_EINVAL, "unknown precision");
  if (!(o->tol > 0.0) || o->max_iter < 1) return fail(ctx, GDT_EINVAL, "tol must be > 0 and max_iter >= 1");
  return solve(ctx, m, b, x, o, info);
}

// ------------------------------------------------------------- finite volume ---
static gdt_status fv_check(gdt_context ctx, gdt_space s, const gdt_fv_desc* d) {
  if (!ctx || !s || !d) return GDT_EINVAL;
  if (s->kind != GDT_SPACE_FV) return fail(ctx, GDT_ESHAPE, "not a finite-volume space");
  for (int side = 0; side < 6; ++side) {
    if (d->boundary[side] < GDT_FV_BOUNDARY_NONE || d->boundary[side] > GDT_FV_BOUNDARY_FLUX)
      return fail(ctx, GDT_EINVAL, "unknown boundary treatment");
    if (side >= 2 * s->g.dim && d->boundary[side] != GDT_FV_BOUNDARY_NONE)
      return fail(ctx, GDT_EINVAL, "boundary treatment on a side the grid does not have");
  }
  if (s->g.periodic)
    for (int k = 0; k < s->g.dim; ++k)
      if ((d->boundary[2 * k] == GDT_FV_BOUNDARY_NONE) != (d->boundary[2 * k + 1] == GDT_FV_BOUNDARY_NONE))
        return fail(ctx, GDT_EINVAL, "periodic grid: treat both sides of a direction or neither");
  if (d->flux != GDT_FLUX_BURGERS && d->flux != GDT_FLUX_TRANSPORT) return fail(ctx, GDT_EINVAL, "unknown flux");
  if (d->numflux != GDT_NUMFLUX_LAX_FRIEDRICHS && d->numflux != GDT_NUMFLUX_UPWIND &&
      d->numflux != GDT_NUMFLUX_ENGQUIST_OSHER)
    return fail(ctx, GDT_EINVAL, "unknown numerical flux");
  return GDT_OK;
}

gdt_status gdt_fv_apply(gdt_context ctx, gdt_space s, const gdt_fv_desc* d, const double* u, double* range) {
  GDT_CHECK(ctx, fv_check(ctx, s, d));
  if (!u || !range) return GDT_EINVAL;
  return fv_apply(ctx, *s, d, u, range);
}

gdt_status gdt_fv_estimate_dt(gdt_context ctx, gdt_space s, const gdt_fv_desc* d, const double* u0, double* dt) {
  GDT_CHECK(ctx, fv_check(ctx, s, d));
  if (!u0 || !dt) return GDT_EINVAL;
  return fv_estimate_dt(ctx, *s, d, u0, dt);
}

gdt_status gdt_fv_timestep(gdt_context ctx, gdt_space s, const gdt_fv_desc* d, int timestepper, double dt,
                           int64_t steps, int64_t nbatch, double* u, double* work) {
  GDT_CHECK(ctx, fv_check(ctx, s, d));
  if (!u || !work || steps < 0 || nbatch < 1) return GDT_EINVAL;
  if (timestepper != GDT_TIMESTEPPER_EXPLICIT_EULER && timestepper != GDT_TIMESTEPPER_SSPRK2)
    return fail(ctx, GDT_EINVAL, "unknown time stepper");
  return fv_timestep(ctx, *s, d, timestepper, dt, steps, nbatch, u, work);
}

// ------------------------------------------------------------------- adjoint ---
gdt_status gdt_cg_dlogkappa(gdt_context ctx, gdt_space s, const double* kappa, const double* u, const double* lam,
                            double* out) {
  if (!ctx || !s || !kappa || !u || !lam || !out) return GDT_EINVAL;
  if (s->kind != GDT_SPACE_CG) return fail(ctx, GDT_ESHAPE, "not a continuous space");
  if (s->order != 1) return fail(ctx, GDT_EUNSUPPORTED, "log-kappa gradient of order-2 spaces");
  if (s->g.mesh) return mesh_dlogkappa(ctx, s->g, kappa, u, lam, out);
  if (s->g.xv) return fail(ctx, GDT_EUNSUPPORTED, "log-kappa gradient on mapped grids");
  return cg_dlogkappa(ctx, *s, kappa, u, lam, out);
}

gdt_status gdt_swipdg_dlogkappa(gdt_context ctx, gdt_space s, const gdt_ipdg_desc* d, const double* u,
                                const double* lam, double* out) {
  if (!ctx || !s || !d || !d->kappa || !u || !lam || !out) return GDT_EINVAL;
  if (s->kind != GDT_SPACE_DG) return fail(ctx, GDT_ESHAPE, "not a DG space");
  if (s->g.mesh) return fail(ctx, GDT_EUNSUPPORTED, "SWIPDG log-kappa gradient on simplex meshes");
  return swipdg_dlogkappa(ctx, *s, d, u, lam, out);
}

}  // extern "C"
