/* gdt_gb300.h — C ABI of the GB300-native discretize-and-solve library.
 *
 * Plain pointers and sizes only. Vectors and coefficient arrays are caller-owned DEVICE pointers
 * (FP64 unless stated); grids, spaces, matrices and contexts are opaque library-owned handles.
 * Every entry point returns a gdt_status (the reference's exception classes, exceptions.hh:21-76,
 * become status codes); gdt_context_last_error() gives the message. The library is
 * stream-ordered: all work of a context runs on the context's CUDA stream. It is thread-safe
 * across contexts and not re-entrant per context.
 *
 * Reference interfaces replaced (paths inside the dune-gdt tree):
 *   grid + spaces      make_cube_grid + make_{continuous_lagrange,discontinuous_lagrange,
 *                      finite_volume}_space  (spaces/h1/continuous-lagrange.hh:189-203,
 *                      spaces/l2/discontinuous-lagrange.hh:191-205, spaces/l2/finite-volume.hh:209-229)
 *   mappers            ContinuousMapper::global_indices (spaces/mapper/continuous.hh:139-150),
 *                      DiscontinuousMapper (spaces/mapper/discontinuous.hh:102-125),
 *                      FiniteVolumeMapper (spaces/mapper/finite-volume.hh:101-107)
 *   pattern + matrix   make_sparsity_pattern (tools/sparsity-pattern.hh:162-178),
 *                      make_matrix_operator(space, Stencil) (operators/matrix-based.hh:650-658)
 *   assembly           MatrixOperator::append/assemble (operators/matrix-based.hh:346-408, 496-500)
 *                      with LocalElementIntegralBilinearForm(LocalLaplaceIntegrand)
 *                      (local/bilinear-forms/integrals.hh:97-134, local/integrands/laplace.hh:81-102),
 *                      VectorBasedFunctional with LocalElementProductIntegrand().with_ansatz(f)
 *                      (functionals/vector-based.hh:214-222, local/functionals/integrals.hh:72-98),
 *                      DirichletConstraints::apply (tools/dirichlet-constraints.hh:153-184),
 *                      SWIPDG coupling/penalty forms (local/integrands/laplace-ipdg.hh:107-186,
 *                      331-368; local/integrands/ipdg.hh:113-171, 254-282)
 *   apply / solve      ConstMatrixOperator::apply / apply_inverse (operators/matrix-based.hh:121-159)
 *   finite volumes     AdvectionFvOperator::apply (operators/advection-fv.hh:66-115,
 *                      local/operators/advection-fv.hh:127-153) with NumericalLaxFriedrichsFlux /
 *                      NumericalUpwindFlux (local/numerical-fluxes/lax-friedrichs.hh:61-87, upwind.hh:61-73),
 *                      estimate_dt_for_hyperbolic_system (tools/hyperbolic.hh:38-86),
 *                      ExplicitRungeKuttaTimeStepper::step (tools/timestepper/explicit-rungekutta.hh:237-270)
 */
#ifndef GDT_GB300_H
#define GDT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gdt_status {
  GDT_OK = 0,
  GDT_EINVAL = 1,       /* invalid argument (null handle, bad enum, bad size) */
  GDT_ESHAPE = 2,       /* shape mismatch (cf. operators/matrix-based.hh:73-80) */
  GDT_ENOCONV = 3,      /* Krylov solver did not converge (cf. operators/matrix-based.hh:155-158) */
  GDT_ETIMEOUT = 4,     /* a device-side wait ran out of its iteration budget */
  GDT_ENAN = 5,         /* non-finite value detected */
  GDT_EUNSUPPORTED = 6, /* form / element / grid combination not provided by the GPU library */
  GDT_ECUDA = 7,        /* CUDA runtime error */
  GDT_ENOMEM = 8        /* device allocation failed */
} gdt_status;

typedef struct gdt_context_s* gdt_context;
typedef struct gdt_grid_s* gdt_grid;
typedef struct gdt_space_s* gdt_space;
typedef struct gdt_matrix_s* gdt_matrix;

enum { GDT_SPACE_CG = 0, GDT_SPACE_DG = 1, GDT_SPACE_FV = 2 };
enum { GDT_STENCIL_ELEMENT = 0, GDT_STENCIL_INTERSECTION = 1, GDT_STENCIL_ELEMENT_AND_INTERSECTION = 2 };
enum { GDT_SOLVER_CG = 0, GDT_SOLVER_BICGSTAB = 1 };
enum { GDT_PREC_NONE = 0, GDT_PREC_JACOBI = 1, GDT_PREC_ILU0 = 2 };
enum { GDT_PRECISION_FP64 = 0, GDT_PRECISION_MIXED = 1 };
enum { GDT_FLUX_BURGERS = 0, GDT_FLUX_TRANSPORT = 1 };
enum { GDT_NUMFLUX_LAX_FRIEDRICHS = 0, GDT_NUMFLUX_UPWIND = 1, GDT_NUMFLUX_ENGQUIST_OSHER = 2 };
enum { GDT_TIMESTEPPER_EXPLICIT_EULER = 0, GDT_TIMESTEPPER_SSPRK2 = 1 };

/* ------------------------------------------------------------------ context --- */
/* device: CUDA ordinal; stream: a cudaStream_t (NULL = the legacy default stream). */
gdt_status gdt_context_create(int device, void* stream, gdt_context* out);
gdt_status gdt_context_destroy(gdt_context ctx);
gdt_status gdt_context_set_stream(gdt_context ctx, void* stream);
gdt_status gdt_context_synchronize(gdt_context ctx);
const char* gdt_context_last_error(gdt_context ctx);
const char* gdt_status_string(gdt_status s);
/* number of kernels this library launched on the context since creation */
int64_t gdt_context_kernel_launches(gdt_context ctx);
/* kernel timing (tracing aid, no reference counterpart beyond Dune::Timer around solves,
 * test/stationary-eocstudies/base.hh:221-225): while enabled, solver iterations are launched without
 * graph capture and the launches of each kernel class (GDT_TIMING_*) are bracketed by CUDA events on
 * the context stream. */
gdt_status gdt_context_set_timing(gdt_context ctx, int enable);
/* accumulated SpMV kernel time (ms) and launch counts since the last reset, FP64 and FP32 separately */
gdt_status gdt_context_spmv_timing(gdt_context ctx, double* fp64_ms, int64_t* fp64_launches, double* fp32_ms,
                                   int64_t* fp32_launches, int reset);
/* kernel classes timed while timing is on */
#define GDT_TIMING_SPMV_FP64 0      /* CSR SpMV and the SpMV-fused solver kernels, FP64 */
#define GDT_TIMING_SPMV_FP32 1      /* FP32 SpMV of the mixed-precision inner iterations */
#define GDT_TIMING_CG_UPDATE 2      /* x += alpha p, r -= alpha q and their dot products */
#define GDT_TIMING_CG_DIRECTION 3   /* p = M^-1 r + beta p */
#define GDT_TIMING_RELIABLE_UPDATE 4 /* FP64 accumulation and true residual (launched every inner
                                      * iteration, working only when a replacement is due) */
#define GDT_TIMING_MIXED_PERSISTENT 5 /* persistent launches of the mixed-precision inner iterations
                                       * (3D Q1 matrix-free path: one launch per replacement cycle) */
#define GDT_TIMING_KINDS 8
/* accumulated time (ms) and launch count of one kernel class since its last reset (all classes are
 * reset by gdt_context_spmv_timing with reset = 1) */
gdt_status gdt_context_kernel_timing(gdt_context ctx, int kind, double* ms, int64_t* launches, int reset);
/* FP64 throughput of the context's GPU in TFLOP/s, measured with CUDA events on the context stream
 * (no reference counterpart; the denominator of FP64-bound rooflines): independent FMA chains on
 * every SM (fma_tflops) and m8n8k4 FP64 tensor-core products (dmma_tflops). Either may be NULL. */
gdt_status gdt_measure_fp64_peak(gdt_context ctx, double* fma_tflops, double* dmma_tflops);
/* L2 bandwidth (read + write GB/s) of float4 copies between two 24 MB device buffers, 64 passes in one
 * launch, best of 3 after a warm-up (no reference counterpart: the ceiling of the L2-resident mixed
 * inner iteration). Allocates and frees 48 MB on the context stream. */
gdt_status gdt_measure_l2_bandwidth(gdt_context ctx, double* gbs);

/* How gdt_solve runs FP64 CG with Jacobi or no preconditioner (no reference counterpart: the launch
 * form of the device solver). GRAPH: one kernel per step (SpMV, update, direction), iterations
 * captured in CUDA graphs. PERSISTENT: one cooperative launch runs every iteration, with grid
 * barriers between the steps and a SELL-32 copy of the matrix; it takes matrices whose rows hold at
 * most 32 entries. AUTO (default): PERSISTENT wherever it applies (it was faster both for systems
 * that stay in L2 and for ones streamed from HBM), GRAPH otherwise or where no cooperative launch or
 * no room for the copy is available. Timing mode always runs GRAPH's kernels launched one by one. */
#define GDT_SOLVER_LAUNCH_AUTO 0
#define GDT_SOLVER_LAUNCH_GRAPH 1
#define GDT_SOLVER_LAUNCH_PERSISTENT 2
gdt_status gdt_context_set_solver_launch(gdt_context ctx, int mode);
/* launch form (GRAPH or PERSISTENT) of the context's last CG solve (FP64, or mixed precision: the 3D
 * Q1 matrix-free inner iterations run persistent under AUTO and PERSISTENT, the other mixed-precision
 * paths as graphs); 0 before the first */
int gdt_context_last_solver_launch(gdt_context ctx);
/* Limits of the persistent (cooperative) solver launches (no reference counterpart; diagnostics and
 * tests of the launch form): blocks caps the grid (0: one block per SM, the default), wait_limit_ns
 * bounds every wait at a grid barrier (0: the default of one second). A wait that runs out sets a
 * device flag, every block leaves at its next barrier, and the solve returns GDT_ECUDA ("a grid
 * barrier wait ran out"); the context stays usable. */
gdt_status gdt_context_set_persistent_limits(gdt_context ctx, int blocks, int64_t wait_limit_ns);

/* --------------------------------------------------------------------- grid --- */
/* make_cube_grid(lower_left, upper_right, num_elements): equidistant YaspGrid-like cube grid
 * (elements and vertices lexicographic, x fastest) or its Kuhn split into d! simplices per cube
 * (element = cube * d! + permutation in std::next_permutation order). dim in {1,2,3}. */
gdt_status gdt_grid_create_cube(int dim, const int64_t* num_elements, const double* lower_left,
                                const double* upper_right, int simplex, int periodic, gdt_grid* out);
/* Moves the vertices of a cube grid (or its simplex split) to the given coordinates: a mapped
 * structured grid with the same topology and numbering, each element's geometry (J, J^{-T}, |det J|
 * at the quadrature points, as DefaultGlobalBasis::jacobians, spaces/basis/default.hh:152-175, forms
 * them from the element geometry) computed from its own vertices. coords: host or device
 * [num_vertices][dim], vertices lexicographic with x fastest; copied. Call before creating spaces.
 * A mapped grid takes continuous order-1 spaces, their Laplace stiffness and load vector (kappa and
 * source per element or constant, Dirichlet values) and everything that works on assembled matrices
 * (SpMV, solvers, Dirichlet constraints, lincomb); other forms return GDT_EUNSUPPORTED. */
gdt_status gdt_grid_set_vertices(gdt_grid grid, const double* coords);
/* Unstructured simplex mesh: the leaf view of a DUNE simplex grid (ALUGrid, UGGrid, a gmsh import),
 * exported in its index-set order (replaces the grid object that make_cube_grid / GridProvider hand to
 * make_continuous_lagrange_space, spaces/h1/continuous-lagrange.hh:189-203). dim 2 (triangles) or 3
 * (tetrahedra); coords [num_vertices][dim], cells [num_elements][dim + 1] vertex indices; host or
 * device pointers, copied. Elements must have distinct vertices and a volume above rounding (|det J|
 * above 1e-12 times the product of its edge lengths), every vertex must belong to an element, and a
 * face may belong to at most two elements (GDT_EINVAL otherwise). Boundary vertices (the Dirichlet DoFs of
 * DirichletConstraints, tools/dirichlet-constraints.hh:153-184) are the vertices of faces that belong
 * to one element. Such a grid takes continuous order-1 spaces (DoF = vertex index, the ContinuousMapper
 * of spaces/mapper/continuous.hh:139-150), their element pattern, the Laplace stiffness and load
 * vector (kappa and source per element or constant, Dirichlet data homogeneous or given values), the
 * log-kappa gradient and everything that works on assembled matrices; on triangle meshes also DG
 * order-1 spaces (DoF 3 e + i) with the element_and_intersection pattern and the SWIPDG assembly
 * (face k of an element is the edge opposite its local vertex k, for gdt_dg_face_points and
 * gdt_ipdg_desc.dirichlet_face); other forms return GDT_EUNSUPPORTED. */
gdt_status gdt_grid_create_simplex_mesh(int dim, int64_t num_vertices, const double* coords, int64_t num_elements,
                                        const int64_t* cells, gdt_grid* out);
gdt_status gdt_grid_destroy(gdt_grid grid);
int64_t gdt_grid_num_elements(gdt_grid grid);
int64_t gdt_grid_num_vertices(gdt_grid grid);

/* -------------------------------------------------------------------- space --- */
/* kind: GDT_SPACE_CG (order 1 or 2; make_continuous_lagrange_space, spaces/h1/continuous-lagrange.hh:189-203),
 * GDT_SPACE_DG (order 1), GDT_SPACE_FV (order 0, m = 1). Order-2 DoFs: MCMG layout by codim
 * (cells, faces, edges, vertices), edges and faces numbered in order of first appearance in the
 * element walk (ContinuousMapper, spaces/mapper/continuous.hh:117-182). */
gdt_status gdt_space_create(gdt_grid grid, int kind, int order, gdt_space* out);
gdt_status gdt_space_destroy(gdt_space space);
int64_t gdt_space_size(gdt_space space);
int gdt_space_max_local_size(gdt_space space);
/* mapper.global_indices of every element into a DEVICE int64 array [num_elements][local_size] */
gdt_status gdt_space_global_indices(gdt_context ctx, gdt_space space, int64_t* out_dev);

/* ------------------------------------------------------------------- matrix --- */
/* builds the sorted CSR sparsity pattern on the device; values start at zero.
 * row_ptr and col are int32 (nnz < 2^31). */
gdt_status gdt_matrix_create(gdt_context ctx, gdt_space test_space, gdt_space ansatz_space, int stencil,
                             gdt_matrix* out);
gdt_status gdt_matrix_destroy(gdt_matrix m);
int64_t gdt_matrix_rows(gdt_matrix m);
int64_t gdt_matrix_cols(gdt_matrix m);
int64_t gdt_matrix_nnz(gdt_matrix m);
gdt_status gdt_matrix_device_arrays(gdt_matrix m, const int32_t** row_ptr, const int32_t** col, double** val);
gdt_status gdt_matrix_set_zero(gdt_context ctx, gdt_matrix m);
/* SpMV schedule autotuner (no reference counterpart; the reference's ISTL BCRS has one schedule):
 * times every valid SpMV schedule on this matrix with CUDA events and keeps the fastest for all
 * SpMV-type kernels of the matrix. Schedules 0-7 read the CSR arrays (vector CSR with 4/8/16/32
 * lanes per row; warp staging of up to 8/16/32 entries per row; cp.async staging of up to 28);
 * schedule 8 (GDT_SPMV_SCHEDULE_SELL32) reads a SELL-32 copy of the matrix (slices of 32 rows stored
 * column-major, one lane per row; 12 bytes per padded entry held besides the CSR arrays). When it is
 * the fastest, the plain SpMV and the graph-form CG SpMV read the copy and the other kernels keep
 * the fastest CSR schedule. Runs automatically on the first SpMV-type call; schedule (may be NULL)
 * receives the chosen index, times_ms (may be NULL, GDT_SPMV_SCHEDULES entries) the measured ms per
 * launch of each schedule (-1 where a schedule does not apply). */
gdt_status gdt_matrix_tune(gdt_context ctx, gdt_matrix m, int* schedule, double* times_ms);
/* Pins the SpMV schedule of m (0 .. GDT_SPMV_SCHEDULES-1; no reference counterpart) instead of
 * tuning it. GDT_EINVAL when the index is out of range or the schedule cannot hold the matrix's
 * longest row (the staged schedules take rows of at most 8, 16, 32 and 28 entries). */
#define GDT_SPMV_SCHEDULES 9
#define GDT_SPMV_SCHEDULE_SELL32 8
gdt_status gdt_matrix_set_schedule(gdt_matrix m, int schedule);
/* The copy of the values kept for the SELL-32 schedule follows every change the library makes
 * (assembly, constraints, lincomb, set_zero) and every gdt_matrix_device_arrays call that returns the
 * value pointer. A caller that writes values through a pointer obtained earlier calls this before
 * the next gdt_spmv (no reference counterpart; solves copy the values afresh in any case). */
gdt_status gdt_matrix_values_changed(gdt_matrix m);

/* ----------------------------------------------------------------- assembly --- */
typedef struct gdt_diffusion_desc {
  const double* kappa;   /* device, one scalar diffusion value per element, or NULL */
  double kappa_const;    /* used when kappa == NULL (and kappa_qp == NULL) */
  const double* force;   /* device, one source value per element, or NULL */
  double force_const;    /* used when force == NULL */
  int dirichlet;         /* 1: all-Dirichlet boundary, homogeneous (unit row + col, rhs = 0) */
  const double* kappa_qp; /* device, diffusion at the quadrature points of every element
                           * ([element][gdt_space_quadrature point]), or NULL; order-2 spaces (or
                           * any order through the element-batched path) */
  const double* force_qp; /* device, the source at the points of the rule
                           * gdt_space_quadrature_order(space, force_quad_order) of every element
                           * ([element][point]), or NULL: the load vector is then
                           * sum_q w_q |det J| f(x_q) phi_i(x_q), the reference's product integrand
                           * (local/integrands/product.hh:104-130) at its quadrature points, order
                           * = order of f + order of the space (+ over_integrate) */
  int force_quad_order;
  const double* kappa_tensor;    /* device, a symmetric d x d diffusion tensor per element
                                  * ([element][d][d], row-major), or NULL: LocalLaplaceIntegrand's
                                  * (kappa(x) grad phi_j) . grad psi_i (local/integrands/laplace.hh:81-102)
                                  * with a tensor; the element-batched path, any order */
  const double* kappa_tensor_qp; /* device, the same at the points of gdt_space_quadrature
                                  * ([element][q][d][d]), or NULL */
  const double* dirichlet_values; /* device, Dirichlet values per DoF (read on the boundary DoFs), or NULL */
  double dirichlet_value_const;   /* the value where dirichlet_values is NULL (0: homogeneous, the
                                   * reference's DirichletConstraints). Non-zero data (order 1): the
                                   * zeroed columns move to the right-hand side (b_i -= A_ij g_j), then
                                   * unit rows and columns with b_D = g_D */
} gdt_diffusion_desc;

/* continuous Lagrange: stiffness of LocalLaplaceIntegrand(kappa) into m, and (if rhs != NULL) the
 * load vector of LocalElementProductIntegrand().with_ansatz(force); Dirichlet constraints fused.
 * Order 1 (P1/Q1): vertex-row kernel, kappa per element. Order 2 (P2/Q2), or kappa_qp given:
 * element-batched local matrices on the FP64 tensor cores (sum over quadrature points as a small
 * GEMM per batch of elements) and coloured scatter into the CSR pattern. */
gdt_status gdt_assemble_cg_diffusion(gdt_context ctx, gdt_matrix m, const gdt_diffusion_desc* desc, double* rhs);

/* load vector only (VectorBasedFunctional::assemble, functionals/vector-based.hh:276-279); with
 * desc->dirichlet the Dirichlet entries are set to zero (DirichletConstraints::apply(V)). */
gdt_status gdt_assemble_cg_rhs(gdt_context ctx, gdt_space cg, const gdt_diffusion_desc* desc, double* rhs);
/* DirichletConstraints::apply(M, V) (tools/dirichlet-constraints.hh:153-184) on an assembled
 * matrix of a continuous space, all-Dirichlet boundary: unit_col + unit_row, rhs[D] = 0 (rhs may be NULL). */
gdt_status gdt_dirichlet_apply(gdt_context ctx, gdt_matrix m, double* rhs);
/* the same with Dirichlet values (continuous order 1): b_i -= A_ij g_j over the boundary columns j of the
 * other rows, then unit rows and columns and b_D = g_D; values: device per DoF, or NULL for value_const.
 * No counterpart in the reference, whose constraints are homogeneous (the lifting a caller would do). */
gdt_status gdt_dirichlet_apply_values(gdt_context ctx, gdt_matrix m, double* rhs, const double* values,
                                      double value_const);

/* LocalElementIntegralBilinearForm(LocalElementProductIntegrand(weight))
 * (local/bilinear-forms/integrals.hh:97-134, local/integrands/product.hh:89-130): the weighted
 * product (mass) matrix M_ij = int weight phi_i phi_j of a continuous space of order 1 or 2 into m,
 * by the element-batched tensor-core path. */
typedef struct gdt_product_desc {
  const double* weight;     /* device, one value per element, or NULL */
  double weight_const;      /* used when weight == NULL and weight_qp == NULL */
  const double* weight_qp;  /* device, [element][gdt_space_quadrature point], or NULL */
} gdt_product_desc;
gdt_status gdt_assemble_cg_product(gdt_context ctx, gdt_matrix m, const gdt_product_desc* desc);
/* quadrature rule of the element-batched path of a continuous space: returns the number of points
 * nq; x_ref (nq x 3 reference-element coordinates) and w_ref (nq weights on the reference element)
 * may be NULL. The physical point of element e is its first vertex plus J_e x_ref. */
int gdt_space_quadrature(gdt_space s, double* x_ref, double* w_ref);
/* the same for a Gauss rule (Duffy-collapsed on simplices) exact to polynomial order quad_order */
int gdt_space_quadrature_order(gdt_space s, int quad_order, double* x_ref, double* w_ref);

/* element indicators of u_h - u_ref, as the EOC studies compute their norms
 * (test/stationary-eocstudies/base.hh:259-269): per element eta_e^2 = int_e |grad u_h - g|^2
 * (GDT_NORM_H1_SEMI, ref_qp = [element][q][dim] values of the reference gradient g) or
 * int_e (u_h - v)^2 (GDT_NORM_L2, ref_qp = [element][q] values of v), with the points of
 * gdt_space_quadrature_order(s, quad_order). u: device DoF vector of s (continuous order 1 or 2,
 * DG order 1); eta2: device, one value per element; total (host, may be NULL) = sqrt(sum eta2). */
enum { GDT_NORM_H1_SEMI = 0, GDT_NORM_L2 = 1 };
gdt_status gdt_element_error(gdt_context ctx, gdt_space s, int norm, int quad_order, const double* u,
                             const double* ref_qp, double* eta2, double* total);

typedef struct gdt_ipdg_desc {
  const double* kappa;   /* device, per element, or NULL */
  double kappa_const;
  const double* force;   /* device, per element, or NULL */
  double force_const;
  double symmetry_prefactor; /* 1 SIPDG/SWIPDG, 0 IIPDG, -1 NIPDG */
  double sigma_inner;        /* inner penalty */
  double sigma_boundary;     /* Dirichlet penalty */
  int weight_is_diffusion;   /* 1: SWIPDG (weight = kappa), 0: weight = 1 */
  double penalty_beta;       /* penalty sigma gamma / h^beta with h = |I|; 0: beta = 1, the h of
                              * LocalIPDGIntegrands (local/integrands/ipdg.hh:27-38). The deprecated
                              * LocalEllipticIpdgIntegrands use beta = 1 / (d - 1)
                              * (local/integrands/elliptic-ipdg.hh:442-445, 677-741) */
  const double* dirichlet_face; /* device, Dirichlet data g at the two Gauss points of every face of every
                                 * element ([element][face][point], the points of gdt_dg_face_points;
                                 * boundary faces are read), or NULL */
  double dirichlet_const;       /* g where dirichlet_face is NULL */
  int dirichlet_rhs;            /* right-hand side terms of g on the boundary faces: bit 0 the unary
                                 * DirichletCoupling term -theta int g (kappa grad psi_i . n)
                                 * (local/integrands/laplace-ipdg.hh:292-320), bit 1 the boundary penalty's
                                 * counterpart int sigma (n . w n) / h^beta g psi_i (a product integrand on
                                 * the boundary intersections with that weight); 0: homogeneous */
} gdt_ipdg_desc;

/* DG Lagrange order 1: element Laplace + InnerCoupling/InnerPenalty (inner intersections) +
 * DirichletCoupling/BoundaryPenalty (Dirichlet boundary), penalty length h = |I|^beta; the load vector
 * of the force plus the Dirichlet data terms selected by dirichlet_rhs. */
gdt_status gdt_assemble_swipdg(gdt_context ctx, gdt_matrix m, const gdt_ipdg_desc* desc, double* rhs);
/* physical coordinates of the two Gauss points of every face of every element of a DG space on a 2D
 * simplex grid (host array [element][face][point][2]): where gdt_ipdg_desc.dirichlet_face is given */
gdt_status gdt_dg_face_points(gdt_space dg, double* xy);
/* the penalty parameters of the deprecated LocalEllipticIpdgIntegrands (Epshteyn, Riviere 2007;
 * local/integrands/elliptic-ipdg.hh:452-501): sigma by polynomial order for inner (boundary = 0) or
 * Dirichlet boundary (boundary = 1) faces, and beta = 1 / (d - 1) */
double gdt_elliptic_ipdg_sigma(int pol_order, int boundary);
double gdt_elliptic_ipdg_beta(int dim);

/* Inner FP32 operator of the last mixed-precision CG solve with this matrix (-1: none yet):
 * the symmetric stencil of the assembled values (linear or plane-tiled kernel), or, for 3D Q1
 * Laplace matrices whose values are exactly their assembly, the matrix-free element operator
 * (checked against the assembled matrix by a probe product at every solve). */
enum { GDT_MIXED_OPERATOR_STENCIL = 0, GDT_MIXED_OPERATOR_STENCIL_TILED = 1, GDT_MIXED_OPERATOR_MATRIX_FREE = 2 };
int gdt_matrix_mixed_operator(gdt_matrix m);

/* ------------------------------------------------------ parametric lincomb --- */
/* The assembled form of pyMOR's LincombOperator over dune-gdt matrices, as the parametric examples
 * build it (one matrix per coefficient function of an affine decomposition,
 * python/dune/gdt/gamm-2019-talk-on-conservative-rb.cc:74-95, combined with the parameter
 * functionals' values theta_q(mu),
 * examples/gamm_2019_talk_on_conservative_rb_OS2015_academic_example.py:62-77).
 * gdt_lincomb: out[i] = sum_q theta[q] terms[q][i] over n FP64 values (device arrays; out may be one
 * of the terms). gdt_matrix_lincomb: the values of `out` = sum_q theta[q] values of terms[q]; every
 * term must have the pattern of `out` (same spaces and stencil), else GDT_ESHAPE. 1..8 terms. */
#define GDT_LINCOMB_MAX_TERMS 8
gdt_status gdt_lincomb(gdt_context ctx, int64_t n, int nterms, const double* const* terms, const double* theta,
                       double* out);
gdt_status gdt_matrix_lincomb(gdt_context ctx, gdt_matrix out, int nterms, const gdt_matrix* terms,
                              const double* theta);

/* ------------------------------------------------------------ apply / solve --- */
gdt_status gdt_spmv(gdt_context ctx, gdt_matrix m, const double* x, double* y);

typedef struct gdt_solver_opts {
  int solver;            /* GDT_SOLVER_* */
  int precond;           /* GDT_PREC_* */
  int precision;         /* GDT_PRECISION_FP64 or GDT_PRECISION_MIXED (FP32 inner CG, FP64 refinement) */
  double tol;            /* stop when ||b - A x|| <= tol * ||b - A x0|| */
  int max_iter;          /* total inner iterations */
  int check_every;       /* iterations between host convergence checks (0 = library default) */
  double inner_tol;      /* mixed: relative reduction per refinement step (0 = default 1e-3) */
} gdt_solver_opts;

typedef struct gdt_solve_info {
  int iterations;        /* Krylov iterations done */
  int refinements;       /* mixed precision: FP64 refinement steps */
  double rel_residual;   /* final ||b - A x|| / ||b - A x0|| in FP64 */
  int converged;
} gdt_solve_info;

/* x holds the initial guess on entry. Returns GDT_ENOCONV (x = last iterate) if not converged. */
gdt_status gdt_solve(gdt_context ctx, gdt_matrix m, const double* b, double* x, const gdt_solver_opts* opts,
                     gdt_solve_info* info);

/* OperatorInterface::apply_inverse with type "newton" (operators/interfaces.hh:490-599) for the affine
 * residual operator x -> A x - range, as the EOC studies invert `lhs - rhs`
 * (test/stationary-eocstudies/base.hh:186-191). x is the initial guess and receives the solution.
 * Damped Newton with the automatic damping of the reference; the Jacobian is A and the defect systems
 * are solved by gdt_solve with `jacobian_solver` (its tol is replaced by 0.1 * precision, as the
 * reference passes to its linear solvers). GDT_ENOCONV (the reference's operator_error) when max_iter
 * steps or max_dampening_iter halvings do not suffice. */
typedef struct gdt_newton_opts {
  double precision;                /* stop when ||A x - range||_2 < precision (reference default 1e-7) */
  int max_iter;                    /* Newton steps (reference default 100) */
  int max_dampening_iter;          /* damping halvings per step (reference default: that of max_iter, 100) */
  gdt_solver_opts jacobian_solver; /* default: CG + Jacobi, FP64 */
} gdt_newton_opts;
typedef struct gdt_newton_info {
  int iterations;        /* Newton steps taken */
  int dampening_steps;   /* halvings of the damping parameter, summed over the steps */
  int linear_iterations; /* Krylov iterations, summed over the steps */
  double residual;       /* final ||A x - range||_2 */
} gdt_newton_info;
gdt_newton_opts gdt_newton_default_opts(void);
gdt_status gdt_newton_solve(gdt_context ctx, gdt_matrix m, const double* range, double* x, const gdt_newton_opts* opts,
                            gdt_newton_info* info);

/* CG + Jacobi solve (FP64) of a caller-owned CSR system on `stream` that allocates no memory: no
 * context, no cudaMalloc/cudaFree, no allocating library call. No counterpart in the reference. For
 * callers that may not allocate device memory themselves or let a library do it: code inside a host
 * framework that owns all device memory through its own pool, or a time-critical loop that cannot
 * take cudaMalloc's implicit device synchronisation. Its work vectors live in a fixed file-scope
 * device array (about 8 MB, held by a GPU until exit once the library's module is loaded there), so
 * n <= GDT_NOALLOC_MAX_ROWS; larger n returns GDT_EINVAL (use gdt_solve). With CUDA's lazy module
 * loading (the default) the first call on a device loads the module, which places the array there,
 * and looks the array's address up: make that first call at set-up time, before any stream capture.
 * The address is looked up again only after the device's context changed (cudaDeviceReset). All calls share the array:
 * calls that overlap on the GPU race and must be serialised by the caller. x holds the initial guess;
 * stop when ||b - A x|| <= tol ||b - A x0|| (recursive residual), GDT_ENOCONV after max_iter. */
#define GDT_NOALLOC_MAX_ROWS 262144
gdt_status gdt_solve_cg_jacobi_noalloc(const int32_t* row_ptr, const int32_t* col, const double* val, int64_t n,
                                       const double* b, double* x, double tol, int max_iter, void* stream,
                                       gdt_solve_info* info);

/* --------------------------------------------------------------- finite volume --- */
/* Treatment of the intersections on one side of the domain (sides -x, +x, -y, +y, -z, +z). The
 * reference appends a boundary operator to AdvectionFvOperator for them (operators/advection-fv.hh:95-115:
 * LocalAdvectionFvBoundaryTreatmentByCustomExtrapolationOperator, local/operators/advection-fv.hh:307-454,
 * and ...ByCustomNumericalFluxOperator, :187-305, on the boundary intersections, with the periodic
 * coupling restricted away from them). Its user lambdas are lowered to these kinds; g is added to the
 * inside cell as g |I| / |E|, n the unit outer normal:
 *   NONE: periodic coupling on a periodic grid; on a non-periodic grid no operator (no flux)
 *   EXTRAPOLATE: ghost state v = u (outflow), g = numerical flux(u, v, n)
 *   DIRICHLET: ghost state v = value (prescribed inflow state), g = numerical flux(u, v, n)
 *   FLUX: g = value, the boundary flux f.n itself (value 0: impermeable wall)
 * On a periodic grid both sides of a direction are NONE or both are not. */
enum { GDT_FV_BOUNDARY_NONE = 0, GDT_FV_BOUNDARY_EXTRAPOLATE = 1, GDT_FV_BOUNDARY_DIRICHLET = 2,
       GDT_FV_BOUNDARY_FLUX = 3 };

typedef struct gdt_fv_desc {
  int flux;              /* GDT_FLUX_BURGERS: f(u) = u^2/2 (1,..,1); GDT_FLUX_TRANSPORT: f(u) = v u */
  double velocity[3];
  int numflux;           /* GDT_NUMFLUX_* */
  double lf_lambda;      /* 0: local Lax-Friedrichs (max_d |f_d'|); else the reference's fixed lambda */
  int boundary[6];       /* GDT_FV_BOUNDARY_* per side (-x, +x, -y, +y, -z, +z); zero-filled: NONE */
  double boundary_value[6];
} gdt_fv_desc;

/* range = AdvectionFvOperator(u) on a cube grid (FV space, m = 1): inner and periodic intersections
 * once, boundary intersections by the treatment of their side */
gdt_status gdt_fv_apply(gdt_context ctx, gdt_space fv, const gdt_fv_desc* desc, const double* u, double* range);
/* dt of estimate_dt_for_hyperbolic_system for initial data u0 (host result) */
gdt_status gdt_fv_estimate_dt(gdt_context ctx, gdt_space fv, const gdt_fv_desc* desc, const double* u0, double* dt);
/* `steps` explicit steps in place on a batch of `nbatch` states stored one after another
 * (u[b * N + cell]); work must hold nbatch * N doubles for GDT_TIMESTEPPER_EXPLICIT_EULER and
 * 2 * nbatch * N doubles for GDT_TIMESTEPPER_SSPRK2 (the stage vector k0 and the next state: both
 * stages read the neighbours' values, so neither can be updated in place).
 * GDT_FV_WORK_DOUBLES gives the size. */
#define GDT_FV_WORK_DOUBLES(timestepper, nbatch, N) \
  ((timestepper) == GDT_TIMESTEPPER_SSPRK2 ? 2 * (nbatch) * (N) : (nbatch) * (N))
gdt_status gdt_fv_timestep(gdt_context ctx, gdt_space fv, const gdt_fv_desc* desc, int timestepper, double dt,
                           int64_t steps, int64_t nbatch, double* u, double* work);

/* ------------------------------------------------------------------ batched --- */
/* Many parametric stationary problems in one persistent launch (the pyMOR-style parameter sweeps of
 * python/dune/gdt/gamm-2019-talk-on-conservative-rb.cc:74-95 run as one GPU job): problem i is
 * -div(kappa grad u) = force on the unit square with cells[i] x cells[i] squares, continuous P1 on
 * the squares split into two triangles each (GDT_BATCH_P1_SIMPLEX, element e = 2 cell + t) or
 * continuous Q1 on the squares (GDT_BATCH_Q1_CUBE, element e = cell), cells lexicographic with x
 * fastest, homogeneous Dirichlet boundary. Sizes may differ between problems. kappa is given either
 * per quadrant of the 2 x 2 split (GDT_BATCH_KAPPA_QUADRANTS: kappa[4 i + q], q = qx + 2 qy; cells[i]
 * even) or per element (GDT_BATCH_KAPPA_ELEMENTS: kappa[eoff[i] + e] with the element offsets of
 * gdt_batch_element_offsets). */
typedef struct gdt_batch_s* gdt_batch;

enum { GDT_BATCH_P1_SIMPLEX = 0, GDT_BATCH_Q1_CUBE = 1 };
enum { GDT_BATCH_KAPPA_QUADRANTS = 0, GDT_BATCH_KAPPA_ELEMENTS = 1 };
/* who solves a problem: the 8 CTAs of a thread-block cluster together, one CTA, or one warp */
enum { GDT_BATCH_TEAM_CLUSTER = 0, GDT_BATCH_TEAM_CTA = 1, GDT_BATCH_TEAM_WARP = 2 };

typedef struct gdt_batch_info {
  int64_t problems;
  int64_t total_dofs;
  int max_iterations;
  int min_iterations;
  double max_rel_residual;  /* ||b - A x|| / ||b|| of the returned iterates, FP64 */
  int all_converged;
  int64_t nonfinite_problems; /* problems skipped for non-finite kappa or load (x = 0, status GDT_ENAN) */
} gdt_batch_info;

/* P1 batch (gdt_batch_create_ex with GDT_BATCH_P1_SIMPLEX) */
gdt_status gdt_batch_create(gdt_context ctx, int64_t nproblems, const int64_t* cells, gdt_batch* out);
/* cells[i] in [1, 16384]; element GDT_BATCH_P1_SIMPLEX or GDT_BATCH_Q1_CUBE. Every problem starts on
 * cluster teams (gdt_batch_set_teams / gdt_batch_tune change that). */
gdt_status gdt_batch_create_ex(gdt_context ctx, int64_t nproblems, const int64_t* cells, int element, gdt_batch* out);
gdt_status gdt_batch_destroy(gdt_batch b);
int64_t gdt_batch_total_dofs(gdt_batch b);
int64_t gdt_batch_total_elements(gdt_batch b);
/* host arrays of nproblems + 1 offsets into the concatenated solution vector / per-element kappa */
gdt_status gdt_batch_dof_offsets(gdt_batch b, int64_t* offsets);
gdt_status gdt_batch_element_offsets(gdt_batch b, int64_t* offsets);
/* team kind per problem (host array of nproblems GDT_BATCH_TEAM_* values) */
gdt_status gdt_batch_set_teams(gdt_context ctx, gdt_batch b, const int* teams);
gdt_status gdt_batch_teams(gdt_batch b, int* teams);
/* assemble (FP64) and solve every problem to ||b - A x|| <= tol ||b|| in one persistent launch (CUDA
 * graph, re-captured when the arguments or the teams change). kappa: device array (see above); x:
 * device [total_dofs]; stencil_out: optional device [total_dofs][7 (P1) or 9 (Q1)] receiving the
 * assembled rows in CSR column order (NULL to skip); precision: GDT_PRECISION_FP64 or
 * GDT_PRECISION_MIXED. info (optional) makes the call wait; then a problem with non-finite data makes
 * the call return GDT_ENAN and one that did not converge GDT_ENOCONV (the other problems are solved
 * all the same: see gdt_batch_status). */
gdt_status gdt_batch_solve_ex(gdt_context ctx, gdt_batch b, const double* kappa, int kappa_kind, double force,
                              int precision, double tol, int max_iter, double* x, double* stencil_out,
                              gdt_batch_info* info);
/* gdt_batch_solve_ex with kappa per quadrant (mu: device [4 * nproblems]) */
gdt_status gdt_batch_solve(gdt_context ctx, gdt_batch b, const double* mu, double force, int precision, double tol,
                           int max_iter, double* x, double* stencil_out, gdt_batch_info* info);
/* Autotuner of the team kinds: for every size class (problems with the same cells, largest first) the
 * batch solve of that class alone is timed (CUDA events, after one warm-up launch) with cluster, CTA
 * and (for at most 20000 DoFs per problem) warp teams, on the caller's data; the fastest kind is kept
 * for the class. Optional outputs: nsizes (classes), sizes[k] (cells of class k), ms[3 k + team]
 * (-1 where not tried); sizes and ms need room for nproblems classes. Waits; x receives the last
 * timed solve of every class. */
gdt_status gdt_batch_tune(gdt_context ctx, gdt_batch b, const double* kappa, int kappa_kind, double force,
                          int precision, double tol, int max_iter, double* x, int64_t* nsizes, int64_t* sizes,
                          double* ms);
/* per-problem iteration counts (negative: -(count + 1) when not converged) and relative residuals (host) */
gdt_status gdt_batch_iterations(gdt_context ctx, gdt_batch b, int* iterations, double* rel_residuals);
/* per-problem status of the last solve (host): GDT_OK, GDT_ENOCONV or GDT_ENAN */
gdt_status gdt_batch_status(gdt_context ctx, gdt_batch b, int* status);

/* ------------------------------------------------------------------ adjoint --- */
/* out[e] = -d/dlog(kappa_e) [lam^T A(kappa) u]: the gradient of J(u(kappa)) w.r.t. log kappa when
 * lam solves A^T lam = dJ/du. CG: Laplace stiffness (Dirichlet rows excluded); DG: SWIPDG. */
gdt_status gdt_cg_dlogkappa(gdt_context ctx, gdt_space cg, const double* kappa, const double* u,
                            const double* lam, double* out);
gdt_status gdt_swipdg_dlogkappa(gdt_context ctx, gdt_space dg, const gdt_ipdg_desc* desc, const double* u,
                                const double* lam, double* out);

#ifdef __cplusplus
}
#endif
#endif
