/* ORACLE — test infrastructure only.
 *
 * CPU restatement (C++17, optional OpenMP) of dune-gdt's discretize-and-solve path, used as the
 * parity checker for the GB300 library and as the timed CPU baseline. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the product never does.
 *
 * Every function cites the reference file it restates (paths relative to the dune-gdt tree).
 * Parity pins: the known answers of dune/gdt/test/integrands/integrands_laplace.cc:131-133 and
 * integrands_product.cc:122-124 (Q2/P2 stiffness and mass), the Burgers FV tables of
 * dune/gdt/test/burgers/burgers__1d__explicit__fv.mini (time-step count, CFL, mass conservation)
 * and the ESV2007 SWIPDG H1 errors (stationary_heat_equation__ESV2007__table_1.mini:28-36).
 */
#ifndef GDT_ORACLE_H
#define GDT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_grid {
  int dim;          /* 1, 2 or 3 */
  long n[3];        /* cells per axis */
  double lo[3];     /* lower-left corner */
  double hi[3];     /* upper-right corner */
  int simplex;      /* 0: cubes (YaspGrid), 1: Kuhn simplices */
  int periodic;     /* periodic in every axis (cube grids, FV only) */
  const double* vertices; /* mapped grid: vertex coordinates [vertex][dim] (x fastest), or NULL */
} orc_grid;

enum { ORC_CG = 0, ORC_DG = 1, ORC_FV = 2 };
enum { ORC_STENCIL_ELEMENT = 0, ORC_STENCIL_INTERSECTION = 1, ORC_STENCIL_ELEMENT_AND_INTERSECTION = 2 };
enum { ORC_FORCE_DATA = 0, ORC_FORCE_ESV2007 = 1 };
enum { ORC_SOLVER_CG = 0, ORC_SOLVER_BICGSTAB = 1 };
enum { ORC_PREC_NONE = 0, ORC_PREC_JACOBI = 1, ORC_PREC_ILU0 = 2 };
enum { ORC_FLUX_BURGERS = 0, ORC_FLUX_TRANSPORT = 1 };
enum { ORC_NUMFLUX_LAX_FRIEDRICHS = 0, ORC_NUMFLUX_UPWIND = 1, ORC_NUMFLUX_ENGQUIST_OSHER = 2 };

typedef struct orc_csr orc_csr;

/* threads used by the parallel loops (OpenMP); 1 keeps the reference walk order */
void orc_set_threads(int nthreads);
int orc_max_threads(void);

long orc_num_elements(const orc_grid* g);
long orc_space_size(const orc_grid* g, int kind, int order);
int orc_local_size(const orc_grid* g, int kind, int order);
/* global indices of every element (row-major [num_elements][local_size]) */
int orc_global_indices(const orc_grid* g, int kind, int order, int64_t* out);
/* Dirichlet DoFs of an all-Dirichlet boundary, ascending; returns the count (out may be NULL) */
long orc_dirichlet_dofs(const orc_grid* g, int order, int64_t* out);

orc_csr* orc_pattern(const orc_grid* g, int kind, int order, int stencil);
long orc_csr_rows(const orc_csr* m);
long orc_csr_nnz(const orc_csr* m);
void orc_csr_export(const orc_csr* m, int64_t* row_ptr, int32_t* col, double* val);
orc_csr* orc_csr_import(long n, const int64_t* row_ptr, const int32_t* col, const double* val);
void orc_csr_free(orc_csr* m);

/* stationary diffusion -div(kappa grad u) = f with continuous Lagrange elements:
 * stiffness (LocalLaplaceIntegrand) + RHS (LocalElementProductIntegrand().with_ansatz(f)),
 * then DirichletConstraints::apply (unit col, unit row, b = 0) when dirichlet != 0. */
orc_csr* orc_assemble_cg(const orc_grid* g, int order, const double* kappa, double kappa_const,
                         const double* force, double force_const, int force_fn, int force_order,
                         int dirichlet, double* rhs);
/* Unstructured simplex mesh (triangles or tetrahedra given by vertex coordinates [nv][dim] and element
 * vertex lists [ne][dim + 1]): continuous P1 stiffness with kappa per element (or constant), load of a
 * source per element (or constant), DirichletConstraints on the boundary vertices (vertices of faces
 * of one element) when dirichlet != 0. */
orc_csr* orc_mesh_assemble(int dim, long nv, const double* coords, long ne, const int64_t* cells, const double* kappa,
                           double kappa_const, const double* force, double force_const, int dirichlet, double* rhs);
/* SWIPDG (DG P1) on a triangle mesh, the terms of orc_assemble_swipdg_data; DoF 3 e + i, face k of an
 * element is the edge opposite its local vertex k */
orc_csr* orc_mesh_assemble_swipdg(long nv, const double* coords, long ne, const int64_t* cells, const double* kappa,
                                  double kappa_const, const double* force, double force_const, double theta,
                                  double sigma_inner, double sigma_boundary, int weight_is_diffusion, double beta,
                                  int dirichlet_fn, double dirichlet_const, int dirichlet_rhs, double* rhs);
/* the boundary vertices of such a mesh, ascending; returns the count (out may be NULL) */
long orc_mesh_boundary(int dim, long nv, long ne, const int64_t* cells, int64_t* out);
/* the same with a d x d diffusion tensor per element, row-major (local/integrands/laplace.hh:81-102) */
orc_csr* orc_assemble_cg_tensor(const orc_grid* g, int order, const double* kappa_tensor, const double* force,
                                double force_const, int dirichlet, double* rhs);
/* the element mass matrix (LocalElementProductIntegrand with weight 1) of a CG/DG space */
orc_csr* orc_assemble_mass(const orc_grid* g, int kind, int order);
/* SWIPDG/IPDG with DG Lagrange elements (element Laplace + InnerCoupling/InnerPenalty on inner
 * intersections once + DirichletCoupling/BoundaryPenalty on boundary intersections), h = |I|. */
orc_csr* orc_assemble_swipdg(const orc_grid* g, int order, const double* kappa, double kappa_const,
                             const double* force, double force_const, int force_fn, int force_order,
                             double symmetry_prefactor, double sigma_inner, double sigma_boundary,
                             int weight_is_diffusion, double* rhs);
/* Dirichlet data of orc_assemble_swipdg_data: a constant, or the test function
 * g = cos(pi x / 2) cos(pi y / 2) + 0.3 x */
enum { ORC_DIRICHLET_CONST = 0, ORC_DIRICHLET_TEST = 1 };
/* orc_assemble_swipdg with the penalty length |I|^beta (local/integrands/elliptic-ipdg.hh:677-741) and the
 * right-hand side terms of Dirichlet data g (rhs_terms bit 0: the unary DirichletCoupling term,
 * local/integrands/laplace-ipdg.hh:292-320; bit 1: the boundary penalty weight times g) */
orc_csr* orc_assemble_swipdg_data(const orc_grid* g, int order, const double* kappa, double kappa_const,
                                  const double* force, double force_const, int force_fn, int force_order,
                                  double theta, double sigma_in, double sigma_bd, int weight_is_diffusion,
                                  double beta, int gfn, double gconst, int rhs_terms, double* rhs);
/* -d/dlog(kappa_e) [lam^T A(kappa) u] for the SWIPDG operator, by Richardson-extrapolated central
 * differences of the element's own local contributions. */
void orc_swipdg_dlogkappa(const orc_grid* g, int order, const double* kappa, double symmetry_prefactor,
                          double sigma_inner, double sigma_boundary, const double* u, const double* lam,
                          double* out);
/* -d/dlog(kappa_e) [lam^T A(kappa) u] for the CG Laplace operator (before Dirichlet rows). */
void orc_cg_dlogkappa(const orc_grid* g, int order, const double* kappa, const double* u, const double* lam,
                      double* out);

void orc_spmv(const orc_csr* m, const double* x, double* y);
/* Krylov solve with relative-residual stop ||b-Ax||/||b-Ax0|| <= tol (x holds x0 on entry). */
int orc_solve(const orc_csr* m, const double* b, double* x, int solver, int prec, double tol, int max_iter,
              int* iterations, double* rel_residual);
/* broken H1 semi-norm error against the ESV2007 test-case-1 solution cos(pi x/2)cos(pi y/2) */
double orc_h1_semi_error_esv2007(const orc_grid* g, int kind, int order, const double* u);
/* L2 norm of a discrete function */
double orc_l2_norm(const orc_grid* g, int kind, int order, const double* u);

/* finite volumes on a structured cube grid, m = 1; boundary treatment per side (-x, +x, -y, +y, -z,
 * +z): bkind ORC_FV_BOUNDARY_*, bval its value; bkind null: none (periodic grids wrap) */
enum { ORC_FV_BOUNDARY_NONE = 0, ORC_FV_BOUNDARY_EXTRAPOLATE = 1, ORC_FV_BOUNDARY_DIRICHLET = 2,
       ORC_FV_BOUNDARY_FLUX = 3 };
double orc_fv_estimate_dt(const orc_grid* g, int flux, const double* velocity, const double* u0);
void orc_fv_apply(const orc_grid* g, int flux, const double* velocity, int numflux, double lf_lambda,
                  const double* u, double* out, const int* bkind, const double* bval);
void orc_fv_explicit_euler(const orc_grid* g, int flux, const double* velocity, int numflux, double lf_lambda,
                           double* u, double dt, long steps, const int* bkind, const double* bval);
void orc_fv_ssprk2(const orc_grid* g, int flux, const double* velocity, int numflux, double lf_lambda, double* u,
                   double dt, long steps, const int* bkind, const double* bval);

#ifdef __cplusplus
}
#endif
#endif
