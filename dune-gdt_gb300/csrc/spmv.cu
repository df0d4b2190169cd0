// CSR SpMV y = A x (ConstMatrixOperator::apply, operators/matrix-based.hh:121-129).
// Vector-CSR: G lanes per row (G chosen from the mean row length when the pattern is built),
// matrix values/indices streamed with evict-first loads, x gathered through L2.
#include "linalg.cuh"

namespace gdt {

template <int G, class T>
__global__ void __launch_bounds__(256) spmv_kernel(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                   const T* __restrict__ val, const T* __restrict__ x, T* __restrict__ y) {
  for_rows<G, T>(n, rp, col, val, x, [&](int row, bool leader, T s) {
    if (leader) y[row] = s;
  });
}

template <class T>
void launch_spmv(int G, int n, const int* rp, const int* col, const T* val, const T* x, T* y, int num_sms,
                 cudaStream_t s) {
  const int th = 256;
  long long rows_per_block = th / G;
  int blocks = int(std::min<long long>((n + rows_per_block - 1) / rows_per_block, (long long)num_sms * 16));
  if (blocks < 1) blocks = 1;
  switch (G) {
    case 2: spmv_kernel<2, T><<<blocks, th, 0, s>>>(n, rp, col, val, x, y); break;
    case 4: spmv_kernel<4, T><<<blocks, th, 0, s>>>(n, rp, col, val, x, y); break;
    case 8: spmv_kernel<8, T><<<blocks, th, 0, s>>>(n, rp, col, val, x, y); break;
    case 16: spmv_kernel<16, T><<<blocks, th, 0, s>>>(n, rp, col, val, x, y); break;
    default: spmv_kernel<32, T><<<blocks, th, 0, s>>>(n, rp, col, val, x, y); break;
  }
}

template void launch_spmv<double>(int, int, const int*, const int*, const double*, const double*, double*, int,
                                  cudaStream_t);
template void launch_spmv<float>(int, int, const int*, const int*, const float*, const float*, float*, int,
                                 cudaStream_t);

gdt_status spmv(gdt_context ctx, gdt_matrix m, const double* x, double* y) {
  launch_spmv<double>(m->spmv_group, int(m->rows), m->rp, m->col, m->val, x, y, ctx->num_sms, ctx->stream);
  return check_launch(ctx, "spmv");
}

}  // namespace gdt
