// CG + Jacobi solve of a caller-owned CSR system that allocates no memory at all.
//
// Who needs it: callers that may not call cudaMalloc / cudaFree — for example code inside a host
// framework that owns every byte of device memory through its own pool (an allocator that must see
// all allocations), or a time-critical loop that cannot afford the implicit device-wide
// synchronisation of cudaMalloc/cudaFree. gdt_solve allocates its work vectors per call (and a
// context allocates at creation); this entry point needs neither a context nor an allocation.
//
// Its work vectors (r, p, q, the Jacobi diagonal), reduction partials, the last-block ticket and the
// solver scalars live in one file-scope __device__ array of fixed size (GDT_NOALLOC_MAX_ROWS rows,
// about 8 MB), which every GPU keeps until the process exits once this module is loaded there. With
// CUDA's lazy module loading (the default) that happens at the first call on a device, not when the
// library is loaded: that call loads the module (which places the array and may synchronise the
// device), so make it at set-up time, before any stream capture. Host code does not use the array's
// name as an address: that first call (with the device current) looks the address up with
// cudaGetSymbolAddress and all kernels receive that pointer; the lookup is repeated only when the
// device's context changed (after cudaDeviceReset). All calls share the array and it keeps the last
// call's contents, so the ticket is cleared at the start of every call; calls whose work overlaps on
// the GPU (two streams, two host threads) race on it and must be serialised by the caller.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <mutex>

#include "linalg.cuh"

namespace gdt {
namespace {

constexpr long long kMaxRows = GDT_NOALLOC_MAX_ROWS;
constexpr int kTH = 256;
constexpr int kMaxBlocks = 1024;

struct NaState {
  double rho, alpha, beta, rr, rr0, tol2;
  int iter, max_iter, converged, breakdown;
};

struct NaScratch {
  double r[kMaxRows];
  double p[kMaxRows];
  double q[kMaxRows];
  double dinv[kMaxRows];
  double partials[2 * kMaxBlocks];
  NaState state;
  unsigned int ticket;
};

static __device__ __align__(256) NaScratch g_noalloc_scratch;

__device__ __forceinline__ bool na_stopped(const NaScratch* s) {
  return entry_flag(&s->state.converged) != 0;
}

// r = b - A x, dinv = 1 / diag, p = dinv r; rho = r.p, rr0 = r.r
__global__ void __launch_bounds__(kTH) k_na_init(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                const double* __restrict__ val, const double* __restrict__ x,
                                                const double* __restrict__ b, double tol2, int max_iter,
                                                NaScratch* s) {
  double a0 = 0.0, a1 = 0.0;
  for_rows<8, double>(n, rp, col, val, x, [&](int row, bool leader, double ax) {
    if (leader) {
      double d = 1.0;
      for (int k = rp[row]; k < rp[row + 1]; ++k)
        if (col[k] == row) d = val[k];
      const double di = 1.0 / d, ri = b[row] - ax, zi = di * ri;
      s->dinv[row] = di;
      s->r[row] = ri;
      s->p[row] = zi;
      a0 = fma(ri, zi, a0);
      a1 = fma(ri, ri, a1);
    }
  });
  double v[2] = {a0, a1};
  if (grid_reduce<2>(v, s->partials, &s->ticket) && threadIdx.x == 0) {
    s->state.rho = v[0];
    s->state.rr = s->state.rr0 = v[1];
    s->state.tol2 = tol2;
    s->state.iter = 0;
    s->state.max_iter = max_iter;
    s->state.breakdown = 0;
    s->state.converged = (v[1] == 0.0) ? 1 : 0;
  }
}

// q = A p ; alpha = rho / p.q
__global__ void __launch_bounds__(kTH) k_na_spmv(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                const double* __restrict__ val, NaScratch* s) {
  if (na_stopped(s)) return;
  double a0 = 0.0;
  for_rows<8, double>(n, rp, col, val, s->p, [&](int row, bool leader, double ap) {
    if (leader) {
      s->q[row] = ap;
      a0 = fma(s->p[row], ap, a0);
    }
  });
  double v[1] = {a0};
  if (grid_reduce<1>(v, s->partials, &s->ticket) && threadIdx.x == 0) {
    if (!(v[0] > 0.0) || !isfinite(v[0])) {
      s->state.breakdown = 1;
      s->state.converged = 1;
    }
    s->state.alpha = s->state.rho / v[0];
  }
}

// x += alpha p ; r -= alpha q ; rho' = r.(dinv r), rr ; beta ; stop test
__global__ void __launch_bounds__(kTH) k_na_update(int n, double* __restrict__ x, NaScratch* s) {
  if (na_stopped(s)) return;
  const double alpha = s->state.alpha;
  double a0 = 0.0, a1 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = fma(alpha, s->p[i], x[i]);
    const double ri = fma(-alpha, s->q[i], s->r[i]);
    s->r[i] = ri;
    a0 = fma(ri, s->dinv[i] * ri, a0);
    a1 = fma(ri, ri, a1);
  }
  double v[2] = {a0, a1};
  if (grid_reduce<2>(v, s->partials, &s->ticket) && threadIdx.x == 0) {
    NaState& st = s->state;
    st.beta = v[0] / st.rho;
    st.rho = v[0];
    st.rr = v[1];
    st.iter += 1;
    if (v[1] <= st.tol2 * st.rr0 || st.iter >= st.max_iter) st.converged = 1;
    if (!isfinite(v[1])) {
      st.breakdown = 1;
      st.converged = 1;
    }
  }
}

__global__ void __launch_bounds__(kTH) k_na_p(int n, NaScratch* s) {
  if (na_stopped(s)) return;
  const double beta = s->state.beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    s->p[i] = fma(beta, s->p[i], s->dinv[i] * s->r[i]);
}

// Address of the scratch array in the current context of each device. The lookup is cached per
// device together with the context it was made in: after cudaDeviceReset (or any new primary context)
// the module is loaded again, the array may move, and the next call looks it up again.
std::mutex g_noalloc_mutex;
struct NaCached {
  CUcontext ctx;
  NaScratch* ptr;
};
NaCached g_noalloc_ptr[64] = {};

CUcontext current_cu_context() {
  static PFN_cuCtxGetCurrent_v4000 get = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(fn);
  });
  CUcontext c = nullptr;
  if (get) get(&c);
  return c;
}

gdt_status scratch_for_current_device(NaScratch** out, int* device) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return GDT_ECUDA;
  *device = dev;
  CUcontext cur = current_cu_context();  // NULL before the runtime made the primary context current
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!cur || !g_noalloc_ptr[dev].ptr || g_noalloc_ptr[dev].ctx != cur) {
    // the first lookup in a context loads this module (lazy loading), which places the array
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return GDT_ECUDA;
    cur = current_cu_context();  // the lookup made the device's primary context current
    g_noalloc_ptr[dev] = NaCached{cur, static_cast<NaScratch*>(ptr)};
  }
  *out = g_noalloc_ptr[dev].ptr;
  return GDT_OK;
}

}  // namespace
}  // namespace gdt

extern "C" gdt_status gdt_solve_cg_jacobi_noalloc(const int32_t* row_ptr, const int32_t* col, const double* val,
                                                  int64_t n, const double* b, double* x, double tol, int max_iter,
                                                  void* stream, gdt_solve_info* info) {
  using namespace gdt;
  if (!row_ptr || !col || !val || !b || !x || n < 1 || !(tol > 0.0) || max_iter < 1) return GDT_EINVAL;
  if (n > kMaxRows) return GDT_EINVAL;  // larger systems need gdt_solve (which allocates)
  NaScratch* s = nullptr;
  int dev = 0;
  gdt_status st = scratch_for_current_device(&s, &dev);
  if (st != GDT_OK) return st;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const int rows = int(n);
  int sms = 152;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GDT_ECUDA;
  const int vec_blocks = std::max(1, std::min(std::min(grid_blocks(rows, kTH), sms * 4), kMaxBlocks));
  const int csr_blocks = std::max(1, std::min(std::min(grid_blocks((long long)rows * 8, kTH), sms * 4), kMaxBlocks));
  // the array keeps the previous call's contents: the reduction ticket must start at zero
  if (cudaMemsetAsync(&s->ticket, 0, sizeof(unsigned int), cs) != cudaSuccess) return GDT_ECUDA;
  k_na_init<<<csr_blocks, kTH, 0, cs>>>(rows, row_ptr, col, val, x, b, tol * tol, max_iter, s);
  NaState h{};
  const int chunk = 32;
  for (int done = 0; done <= max_iter; done += chunk) {
    for (int k = 0; k < chunk; ++k) {
      k_na_spmv<<<csr_blocks, kTH, 0, cs>>>(rows, row_ptr, col, val, s);
      k_na_update<<<vec_blocks, kTH, 0, cs>>>(rows, x, s);
      k_na_p<<<vec_blocks, kTH, 0, cs>>>(rows, s);
    }
    if (cudaMemcpyAsync(&h, &s->state, sizeof(NaState), cudaMemcpyDeviceToHost, cs) != cudaSuccess ||
        cudaStreamSynchronize(cs) != cudaSuccess)
      return GDT_ECUDA;
    if (h.converged) break;
  }
  if (cudaGetLastError() != cudaSuccess) return GDT_ECUDA;
  const bool ok = !h.breakdown && (h.rr0 == 0.0 || h.rr <= h.tol2 * h.rr0);
  if (info) {
    info->iterations = h.iter;
    info->refinements = 0;
    info->rel_residual = h.rr0 > 0 ? std::sqrt(h.rr / h.rr0) : 0.0;
    info->converged = ok ? 1 : 0;
  }
  return ok ? GDT_OK : GDT_ENOCONV;
}
