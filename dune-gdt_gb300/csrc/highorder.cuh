// Order-2 continuous Lagrange spaces and the element-batched (tensor-core) assembly path.
#pragma once
#include <vector>

#include "internal.cuh"

namespace gdt {
namespace ho {

constexpr int kMaxL = 27;     // local DoFs of Q2 in 3D
constexpr int kMaxTypes = 6;  // Kuhn simplices per cube in 3D

// DoF layout of a continuous Lagrange space of order k on a structured grid
struct HoSpaceInfo {
  int lsize = 0, ntypes = 1;
  int codim[kMaxL] = {};                // codim of each node's support entity
  int has[4] = {};                      // codims that carry DoFs
  long long count[4] = {}, offset[4] = {}, size = 0;  // entities per codim, MCMG offsets, DoFs
  int nsup[kMaxTypes][kMaxL] = {};      // support corners of node i of element type t
  int sup[kMaxTypes][kMaxL][8] = {};    // as cube-corner bit patterns
};
HoSpaceInfo space_info(const GridDesc& g, int order);

// element contraction matrices, per element type, rows = symmetric pairs (i <= j) padded to 8,
// columns = quadrature points padded to 4 (zeros in the padding)
struct ContractionTables {
  int lsize = 0, nq = 0, nq_pad = 0, npair = 0, npair_pad = 0, ntypes = 1;
  std::vector<int> pi, pj;
  std::vector<double> stiff, mass;  // [type][npair_pad][nq_pad]
  std::vector<double> load;         // [type][lsize][nq]
  // tensor diffusion: columns (q, c) over the components c = (a, b), a <= b, of a symmetric d x d
  // tensor (lexicographic), nqt = nq * d (d + 1) / 2 padded to 4: w_q |J| (da phi_i db phi_j + db phi_i
  // da phi_j) for a < b, w_q |J| da phi_i da phi_j for a = b
  int ncomp = 1, nqt = 0, nqt_pad = 0;
  std::vector<double> stiff_t;      // [type][npair_pad][nqt_pad]
};
ContractionTables contraction_tables(const GridDesc& g, int order);

// the quadrature rule of the element-batched path (reference coordinates x[3 q + a], weights)
struct QuadratureInfo {
  int nq = 0;
  std::vector<double> x, w;
};
QuadratureInfo quadrature_info(const GridDesc& g, int order);
QuadratureInfo quadrature_info_order(const GridDesc& g, int quad_order);

// nodal basis values and physical gradients at the points of a quadrature rule, per element type
struct BasisTables {
  int lsize = 0, nq = 0, ntypes = 1;
  std::vector<double> phi;   // [type][q][i]
  std::vector<double> grad;  // [type][q][i][3]
  std::vector<double> wdet;  // [type][q]: w_q |det J|
};
BasisTables basis_tables(const GridDesc& g, int order, int quad_order);

}  // namespace ho

// device work (highorder.cu)
gdt_status ho_global_indices(gdt_context ctx, const gdt_space_s& s, int64_t* out64, int32_t* out32);
gdt_status ho_build_pattern(gdt_context ctx, gdt_matrix m);
gdt_status ho_assemble(gdt_context ctx, gdt_matrix m, int form, const double* coef, double coef_const,
                       const double* coef_qp, const double* force, double force_const, double* rhs, int dirichlet);
gdt_status ho_dirichlet(gdt_context ctx, gdt_matrix m, double* rhs);
// LocalLaplaceIntegrand with a symmetric d x d diffusion tensor, per element ([element][d][d]) or at
// the points of gdt_space_quadrature ([element][q][d][d]); load vector and Dirichlet as ho_assemble
gdt_status ho_assemble_tensor(gdt_context ctx, gdt_matrix m, const double* kt, const double* kt_qp,
                              const double* force, double force_const, double* rhs, int dirichlet);
gdt_status ho_prepare(gdt_context ctx, gdt_matrix m);
gdt_status ho_assemble_rhs(gdt_context ctx, const gdt_space_s& sp, const double* force, double force_const,
                           int dirichlet, double* rhs);
// load vector of a source given at the points of the Gauss rule of quad_order
// (gdt_space_quadrature_order), fqp [element][point]; continuous spaces of order 1 and 2
gdt_status ho_rhs_qp(gdt_context ctx, const gdt_space_s& sp, const double* fqp, int quad_order, int dirichlet,
                     double* rhs);
int ho_quadrature(const gdt_space_s& sp, double* x_ref, double* w_ref);
gdt_status element_error(gdt_context ctx, const gdt_space_s& sp, int norm, int quad_order, const double* u,
                         const double* ref, double* eta2, double* total);
int quadrature_order(const gdt_space_s& sp, int quad_order, double* x_ref, double* w_ref);
struct HoMatrix;
void ho_matrix_free(HoMatrix* h);

}  // namespace gdt
