// C++ facade of the GB300 discretize-and-solve library: keeps the reference's C++ API names
// (make_cube_grid, make_continuous_lagrange_space, make_matrix_operator, LocalElementIntegralBilinearForm,
// LocalLaplaceIntegrand, make_vector_functional, LocalElementProductIntegrand().with_ansatz(f),
// make_dirichlet_constraints, make_walker, make_discrete_function, AdvectionFvOperator, ...) so a
// driver such as examples/stationary-heat-equation.cc:87-110 ports by changing its includes and
// namespace. Everything below calls the C ABI (include/gdt_gb300.h); device memory is plain
// cudaMalloc memory owned by DeviceVector.
//
// Lowering rules (documented limits of the GPU library): the diffusion is a constant or element-wise
// constant; a function-valued source (std::function of the global point, with its polynomial order as
// dune-xt's GenericFunction(order, lambda)) is evaluated on the host at the quadrature points the
// reference's product integrand uses (a Gauss rule of order f + space order) and the load vector is
// assembled from those values.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "gdt_gb300.h"

namespace Dune {
namespace GDT {
namespace GB300 {

struct Exception : public std::runtime_error {
  gdt_status status;
  Exception(gdt_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(gdt_status s, gdt_context ctx, const char* what) {
  if (s == GDT_OK) return;
  std::string msg = std::string(what) + ": " + gdt_status_string(s);
  if (ctx) msg += std::string(" (") + gdt_context_last_error(ctx) + ")";
  throw Exception(s, msg);
}

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Exception(GDT_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// one context per process and device (stream = legacy default stream)
inline gdt_context default_context() {
  static std::shared_ptr<gdt_context_s> ctx(
      [] {
        gdt_context c = nullptr;
        check(gdt_context_create(0, nullptr, &c), nullptr, "gdt_context_create");
        return c;
      }(),
      [](gdt_context c) { gdt_context_destroy(c); });
  return ctx.get();
}

class DeviceVector {
 public:
  DeviceVector() = default;
  explicit DeviceVector(size_t n, double value = 0.0) : n_(n) {
    cuda_check(cudaMalloc(&p_, sizeof(double) * std::max<size_t>(n, 1)), "cudaMalloc");
    set_all(value);
  }
  DeviceVector(const DeviceVector&) = delete;
  DeviceVector& operator=(const DeviceVector&) = delete;
  DeviceVector(DeviceVector&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; }
  ~DeviceVector() {
    if (p_) cudaFree(p_);
  }
  size_t size() const { return n_; }
  double* data() { return p_; }
  const double* data() const { return p_; }
  void set_all(double v) {
    std::vector<double> h(n_, v);
    upload(h);
  }
  void upload(const std::vector<double>& h) {
    if (h.size() != n_) throw Exception(GDT_ESHAPE, "DeviceVector::upload: size mismatch");
    cuda_check(cudaMemcpy(p_, h.data(), sizeof(double) * n_, cudaMemcpyHostToDevice), "upload");
  }
  std::vector<double> download() const {
    std::vector<double> h(n_);
    cuda_check(cudaDeviceSynchronize(), "synchronize");
    cuda_check(cudaMemcpy(h.data(), p_, sizeof(double) * n_, cudaMemcpyDeviceToHost), "download");
    return h;
  }

 private:
  double* p_ = nullptr;
  size_t n_ = 0;
};

template <int d>
using FieldVector = std::array<double, d>;

// ---------------------------------------------------------------------------------- grid ---
// A grid: make_cube_grid's structured cubes (or their Kuhn simplex split, optionally with moved
// vertices), or an unstructured simplex mesh (make_simplex_mesh)
template <int d>
class Grid {
 public:
  Grid(FieldVector<d> lower, FieldVector<d> upper, std::array<int64_t, d> cells, bool simplex = false,
           bool periodic = false)
      : lower_(lower), upper_(upper), cells_(cells), simplex_(simplex) {
    gdt_grid g = nullptr;
    check(gdt_grid_create_cube(d, cells.data(), lower.data(), upper.data(), simplex, periodic, &g), nullptr,
          "make_cube_grid");
    handle_.reset(g, [](gdt_grid x) { gdt_grid_destroy(x); });
  }
  // An unstructured simplex mesh: the leaf view of a DUNE simplex grid (ALUGrid, UGGrid, a gmsh
  // import) in its index-set order; coords [num_vertices * d], cells [num_elements * (d + 1)] vertex
  // indices. Continuous order-1 spaces (DoF = vertex index) with the Laplace stiffness, load vector
  // (data per element or constant) and Dirichlet constraints on the boundary vertices.
  Grid(const std::vector<double>& coords, const std::vector<int64_t>& cells) : simplex_(true), mapped_(true) {
    const int64_t nv = int64_t(coords.size() / d), ne = int64_t(cells.size() / (d + 1));
    if (coords.size() != size_t(nv) * d || cells.size() != size_t(ne) * (d + 1))
      throw Exception(GDT_ESHAPE, "make_simplex_mesh: coords of d and cells of d + 1 entries each");
    gdt_grid g = nullptr;
    check(gdt_grid_create_simplex_mesh(d, nv, coords.data(), ne, cells.data(), &g), nullptr, "make_simplex_mesh");
    handle_.reset(g, [](gdt_grid x) { gdt_grid_destroy(x); });
  }
  gdt_grid handle() const { return handle_.get(); }
  int64_t num_elements() const { return gdt_grid_num_elements(handle()); }
  // A mapped grid (a Dune::GeometryGrid over this grid's topology): moves every vertex to `coords`
  // ([num_vertices * d], vertices lexicographic with x fastest). Call before making spaces; the
  // continuous order-1 Laplace stiffness and load vector (data per element or constant) then form each
  // element's geometry on the device.
  void set_vertices(const std::vector<double>& coords) {
    if (coords.size() != size_t(gdt_grid_num_vertices(handle())) * d)
      throw Exception(GDT_ESHAPE, "set_vertices: expected num_vertices * d coordinates");
    check(gdt_grid_set_vertices(handle(), coords.data()), nullptr, "set_vertices");
    mapped_ = true;
  }
  bool mapped() const { return mapped_; }
  // element barycentre (elements numbered cube * d! + simplex, cubes lexicographic, x fastest)
  FieldVector<d> barycentre(int64_t e) const {
    if (mapped_) throw Exception(GDT_EUNSUPPORTED, "points of mapped grids and meshes: data per element or constant");
    const int nsub = simplex_ ? (d == 2 ? 2 : d == 3 ? 6 : 1) : 1;
    int64_t c = e / nsub;
    FieldVector<d> x;
    for (int a = 0; a < d; ++a) {
      const double h = (upper_[a] - lower_[a]) / double(cells_[a]);
      const int64_t i = c % cells_[a];
      c /= cells_[a];
      x[a] = lower_[a] + (double(i) + 0.5) * h;
    }
    if (simplex_ && d == 2) {
      // triangles A = (0,0),(1,0),(1,1) and B = (0,0),(0,1),(1,1) in cube coordinates
      const double hx = (upper_[0] - lower_[0]) / double(cells_[0]), hy = (upper_[1] - lower_[1]) / double(cells_[1]);
      const bool a = (e % 2) == 0;
      x[0] += (a ? 1.0 / 6.0 : -1.0 / 6.0) * hx;
      x[1] += (a ? -1.0 / 6.0 : 1.0 / 6.0) * hy;
    }
    return x;
  }
  // the physical point of reference coordinates xref in element e: its first vertex plus J_e xref,
  // J_e the cube's scaling (times the Kuhn simplex's corner matrix: column m is the sum of the unit
  // vectors of the first m + 1 axes of its permutation, permutations in std::next_permutation order)
  FieldVector<d> global(int64_t e, const double* xref) const {
    if (mapped_) throw Exception(GDT_EUNSUPPORTED, "points of mapped grids and meshes: data per element or constant");
    const int nsub = simplex_ ? (d == 2 ? 2 : d == 3 ? 6 : 1) : 1;
    int64_t c = e / nsub;
    std::array<double, d> loc{};
    if (simplex_ && d >= 2) {
      std::array<int, d> perm;
      for (int a = 0; a < d; ++a) perm[a] = a;
      for (int64_t t = 0; t < e % nsub; ++t) std::next_permutation(perm.begin(), perm.end());
      for (int m = 0; m < d; ++m)
        for (int k = 0; k <= m; ++k) loc[perm[k]] += xref[m];
    } else {
      for (int a = 0; a < d; ++a) loc[a] = xref[a];
    }
    FieldVector<d> x;
    for (int a = 0; a < d; ++a) {
      const double h = (upper_[a] - lower_[a]) / double(cells_[a]);
      const int64_t i = c % cells_[a];
      c /= cells_[a];
      x[a] = lower_[a] + (double(i) + loc[a]) * h;
    }
    return x;
  }

 private:
  FieldVector<d> lower_{}, upper_{};
  std::array<int64_t, d> cells_{};
  bool simplex_;
  bool mapped_ = false;
  std::shared_ptr<gdt_grid_s> handle_;
};

template <int d>
using CubeGrid = Grid<d>;

// an unstructured simplex mesh (see Grid)
template <int d>
Grid<d> make_simplex_mesh(const std::vector<double>& coords, const std::vector<int64_t>& cells) {
  return Grid<d>(coords, cells);
}

// XT::Grid::make_cube_grid<G>(lower_left, upper_right, num_elements)
template <int d>
CubeGrid<d> make_cube_grid(double lower, double upper, int64_t cells, bool simplex = false, bool periodic = false) {
  FieldVector<d> lo, hi;
  std::array<int64_t, d> n;
  lo.fill(lower);
  hi.fill(upper);
  n.fill(cells);
  return CubeGrid<d>(lo, hi, n, simplex, periodic);
}

// -------------------------------------------------------------------------------- spaces ---
template <int d>
class Space {
 public:
  Space(const CubeGrid<d>& grid, int kind, int order) : grid_(grid), order_(order) {
    gdt_space s = nullptr;
    check(gdt_space_create(grid.handle(), kind, order, &s), nullptr, "space");
    handle_.reset(s, [](gdt_space x) { gdt_space_destroy(x); });
  }
  gdt_space handle() const { return handle_.get(); }
  int64_t size() const { return gdt_space_size(handle()); }
  int order() const { return order_; }
  const CubeGrid<d>& grid_view() const { return grid_; }

 private:
  CubeGrid<d> grid_;
  int order_;
  std::shared_ptr<gdt_space_s> handle_;
};

template <int d>
Space<d> make_continuous_lagrange_space(const CubeGrid<d>& grid, int order) {
  return Space<d>(grid, GDT_SPACE_CG, order);
}
template <int d>
Space<d> make_discontinuous_lagrange_space(const CubeGrid<d>& grid, int order) {
  return Space<d>(grid, GDT_SPACE_DG, order);
}
template <int d>
Space<d> make_finite_volume_space(const CubeGrid<d>& grid) {
  return Space<d>(grid, GDT_SPACE_FV, 0);
}

enum class Stencil { element = GDT_STENCIL_ELEMENT, intersection = GDT_STENCIL_INTERSECTION,
                     element_and_intersection = GDT_STENCIL_ELEMENT_AND_INTERSECTION };

// ------------------------------------------------------------------- local form descriptors ---
template <int d>
using GridFunction = std::function<double(const FieldVector<d>&)>;

struct LocalLaplaceIntegrand {
  explicit LocalLaplaceIntegrand(double diffusion = 1.0) : constant(diffusion) {}
  explicit LocalLaplaceIntegrand(const DeviceVector* per_element) : elementwise(per_element) {}
  double constant = 1.0;
  const DeviceVector* elementwise = nullptr;
};

template <int d>
struct ProductWithAnsatz {
  GridFunction<d> f;
  double constant = 1.0;
  bool is_constant = true;
  int order = 3;  // polynomial order of f (GenericFunction(order, lambda))
};

struct LocalElementProductIntegrand {
  template <int d>
  ProductWithAnsatz<d> with_ansatz(const GridFunction<d>& f, int order = 3) const {
    return ProductWithAnsatz<d>{f, 0.0, false, order};
  }
  template <int d = 2>
  ProductWithAnsatz<d> with_ansatz(double c) const {
    return ProductWithAnsatz<d>{{}, c, true, 0};
  }
};

struct LocalElementIntegralBilinearForm {
  explicit LocalElementIntegralBilinearForm(LocalLaplaceIntegrand i) : integrand(i) {}
  LocalLaplaceIntegrand integrand;
};

template <int d>
struct LocalElementIntegralFunctional {
  explicit LocalElementIntegralFunctional(ProductWithAnsatz<d> i) : integrand(std::move(i)) {}
  ProductWithAnsatz<d> integrand;
};

// ------------------------------------------------------------------------- matrix operator ---
template <int d>
class MatrixOperator {
 public:
  MatrixOperator(const Space<d>& space, Stencil stencil) : space_(space) {
    gdt_matrix m = nullptr;
    check(gdt_matrix_create(default_context(), space.handle(), space.handle(), int(stencil), &m), default_context(),
          "make_matrix_operator");
    handle_.reset(m, [](gdt_matrix x) { gdt_matrix_destroy(x); });
  }
  void append(const LocalElementIntegralBilinearForm& f) { laplace_ = f.integrand; }
  MatrixOperator& operator+=(const LocalElementIntegralBilinearForm& f) {
    append(f);
    return *this;
  }
  gdt_matrix handle() const { return handle_.get(); }
  MatrixOperator& matrix() { return *this; }
  const Space<d>& source_space() const { return space_; }
  gdt_diffusion_desc desc() const {
    gdt_diffusion_desc desc{};
    desc.kappa = laplace_.elementwise ? laplace_.elementwise->data() : nullptr;
    desc.kappa_const = laplace_.constant;
    desc.force_const = 0.0;
    return desc;
  }
  void assemble(bool /*use_tbb*/ = true) {
    gdt_diffusion_desc ds = desc();
    check(gdt_assemble_cg_diffusion(default_context(), handle(), &ds, nullptr), default_context(), "assemble");
  }
  void apply(const DeviceVector& source, DeviceVector& range) const {
    check(gdt_spmv(default_context(), handle(), source.data(), range.data()), default_context(), "apply");
  }
  // OperatorInterface::apply_inverse(range, source, {{"type", "newton"}, ...}): damped Newton on
  // x -> A x - range, source is the initial guess (operators/interfaces.hh:490-599)
  gdt_newton_info apply_inverse(const DeviceVector& range, DeviceVector& source,
                                gdt_newton_opts opts = gdt_newton_default_opts()) const {
    gdt_newton_info info{};
    check(gdt_newton_solve(default_context(), handle(), range.data(), source.data(), &opts, &info), default_context(),
          "apply_inverse");
    return info;
  }

 private:
  Space<d> space_;
  LocalLaplaceIntegrand laplace_;
  std::shared_ptr<gdt_matrix_s> handle_;
};

template <int d>
MatrixOperator<d> make_matrix_operator(const Space<d>& space, Stencil stencil = Stencil::element) {
  return MatrixOperator<d>(space, stencil);
}

template <int d>
class VectorFunctional {
 public:
  explicit VectorFunctional(const Space<d>& space) : space_(space), vector_(size_t(space.size())) {}
  void append(const LocalElementIntegralFunctional<d>& f) {
    if (f.integrand.is_constant) {
      force_.reset();
      force_qp_.reset();
      constant_ = f.integrand.constant;
      return;
    }
    // the source at the quadrature points of the product integrand (order of f + order of the space)
    const auto& grid = space_.grid_view();
    quad_order_ = f.integrand.order + space_.order();
    const int nq = gdt_space_quadrature_order(space_.handle(), quad_order_, nullptr, nullptr);
    if (nq <= 0) throw Exception(GDT_EUNSUPPORTED, "no quadrature rule for this space");
    std::vector<double> xq(3 * size_t(nq)), wq(static_cast<size_t>(nq));
    gdt_space_quadrature_order(space_.handle(), quad_order_, xq.data(), wq.data());
    std::vector<double> h(size_t(grid.num_elements()) * nq);
    for (int64_t e = 0; e < grid.num_elements(); ++e)
      for (int q = 0; q < nq; ++q) h[size_t(e) * nq + q] = f.integrand.f(grid.global(e, &xq[3 * size_t(q)]));
    force_qp_ = std::make_shared<DeviceVector>(h.size());
    force_qp_->upload(h);
    force_.reset();
  }
  DeviceVector& vector() { return vector_; }
  gdt_diffusion_desc desc(double kappa_const = 1.0, const DeviceVector* kappa = nullptr) const {
    gdt_diffusion_desc ds{};
    ds.kappa = kappa ? kappa->data() : nullptr;
    ds.kappa_const = kappa_const;
    ds.force = force_ ? force_->data() : nullptr;
    ds.force_const = constant_;
    ds.force_qp = force_qp_ ? force_qp_->data() : nullptr;
    ds.force_quad_order = quad_order_;
    return ds;
  }
  void assemble(bool /*use_tbb*/ = true) {
    gdt_diffusion_desc ds = desc();
    check(gdt_assemble_cg_rhs(default_context(), space_.handle(), &ds, vector_.data()), default_context(),
          "assemble");
  }

 private:
  Space<d> space_;
  DeviceVector vector_;
  std::shared_ptr<DeviceVector> force_;
  std::shared_ptr<DeviceVector> force_qp_;
  int quad_order_ = 0;
  double constant_ = 0.0;
};

template <int d>
VectorFunctional<d> make_vector_functional(const Space<d>& space) {
  return VectorFunctional<d>(space);
}

struct AllDirichletBoundaryInfo {};

template <int d>
class DirichletConstraints {
 public:
  explicit DirichletConstraints(const Space<d>& space) : space_(space) {}
  void apply(MatrixOperator<d>& m, DeviceVector& v) {
    if (fused_) return;
    check(gdt_dirichlet_apply(default_context(), m.handle(), v.data()), default_context(), "dirichlet apply");
  }
  bool fused_ = false;

 private:
  Space<d> space_;
};

template <int d>
DirichletConstraints<d> make_dirichlet_constraints(const Space<d>& space, const AllDirichletBoundaryInfo&) {
  return DirichletConstraints<d>(space);
}

// XT::Grid::Walker over the functors of one stationary problem: one fused assembly kernel
template <int d>
class Walker {
 public:
  explicit Walker(const CubeGrid<d>&) {}
  void append(MatrixOperator<d>& op) { op_ = &op; }
  void append(VectorFunctional<d>& f) { f_ = &f; }
  void append(DirichletConstraints<d>& c) { dc_ = &c; }
  void walk(bool /*thread_parallel*/ = true) {
    if (!op_) {
      if (f_) f_->assemble();
      return;
    }
    gdt_diffusion_desc ds = op_->desc();
    if (f_) {
      const gdt_diffusion_desc fd = f_->desc();
      ds.force = fd.force;
      ds.force_const = fd.force_const;
      ds.force_qp = fd.force_qp;
      ds.force_quad_order = fd.force_quad_order;
    }
    ds.dirichlet = dc_ ? 1 : 0;
    check(gdt_assemble_cg_diffusion(default_context(), op_->handle(), &ds, f_ ? f_->vector().data() : nullptr),
          default_context(), "walk");
    if (dc_) dc_->fused_ = true;
  }

 private:
  MatrixOperator<d>* op_ = nullptr;
  VectorFunctional<d>* f_ = nullptr;
  DirichletConstraints<d>* dc_ = nullptr;
};

template <int d>
Walker<d> make_walker(const CubeGrid<d>& g) {
  return Walker<d>(g);
}

// ------------------------------------------------------------------------- discrete function ---
template <int d>
class DiscreteFunction {
 public:
  explicit DiscreteFunction(const Space<d>& space) : space_(space), v_(size_t(space.size())) {}
  DiscreteFunction& dofs() { return *this; }
  DeviceVector& vector() { return v_; }
  const Space<d>& space() const { return space_; }

 private:
  Space<d> space_;
  DeviceVector v_;
};

template <int d>
DiscreteFunction<d> make_discrete_function(const Space<d>& space) {
  return DiscreteFunction<d>(space);
}

// XT::LA::make_solver(matrix).apply(rhs, solution): CG + Jacobi (FP64 or mixed precision)
template <int d>
class Solver {
 public:
  explicit Solver(MatrixOperator<d>& m) : m_(m) {}
  gdt_solve_info apply(const DeviceVector& rhs, DeviceVector& x, double tol = 1e-10,
                       int precision = GDT_PRECISION_FP64, int solver = GDT_SOLVER_CG, int precond = GDT_PREC_JACOBI) {
    gdt_solver_opts o{solver, precond, precision, tol, 1000000, 0, 0.0};
    gdt_solve_info info{};
    check(gdt_solve(default_context(), m_.handle(), rhs.data(), x.data(), &o, &info), default_context(), "solve");
    return info;
  }

 private:
  MatrixOperator<d>& m_;
};

template <int d>
Solver<d> make_solver(MatrixOperator<d>& m) {
  return Solver<d>(m);
}

// ------------------------------------------------------------------------ finite volumes ---
// Flux functions of the FV tests (f(u) = u^2/2 (1, ..., 1) for Burgers, f(u) = v u for linear transport)
// and the numerical fluxes of local/numerical-fluxes/ (lax-friedrichs.hh, upwind.hh, engquist-osher.hh),
// lowered to gdt_fv_desc.
struct BurgersFlux {
  void lower(gdt_fv_desc& d) const { d.flux = GDT_FLUX_BURGERS; }
};
struct LinearTransportFlux {
  std::array<double, 3> velocity{};
  void lower(gdt_fv_desc& d) const {
    d.flux = GDT_FLUX_TRANSPORT;
    for (int k = 0; k < 3; ++k) d.velocity[k] = velocity[k];
  }
};
template <class F>
struct NumericalLaxFriedrichsFlux {
  F flux;
  double lambda = 0.0;  // 0: local speeds; else the reference's fixed lambda_
  explicit NumericalLaxFriedrichsFlux(const F& f, double l = 0.0) : flux(f), lambda(l) {}
  void lower(gdt_fv_desc& d) const {
    flux.lower(d);
    d.numflux = GDT_NUMFLUX_LAX_FRIEDRICHS;
    d.lf_lambda = lambda;
  }
};
template <class F>
struct NumericalUpwindFlux {
  F flux;
  explicit NumericalUpwindFlux(const F& f) : flux(f) {}
  void lower(gdt_fv_desc& d) const {
    flux.lower(d);
    d.numflux = GDT_NUMFLUX_UPWIND;
  }
};
template <class F>
struct NumericalEngquistOsherFlux {
  F flux;
  explicit NumericalEngquistOsherFlux(const F& f) : flux(f) {}
  void lower(gdt_fv_desc& d) const {
    flux.lower(d);
    d.numflux = GDT_NUMFLUX_ENGQUIST_OSHER;
  }
};

// LocalAdvectionFvBoundaryTreatmentByCustomExtrapolationOperator / ...ByCustomNumericalFluxOperator
// (local/operators/advection-fv.hh:187-457) with their lambdas lowered to the GDT_FV_BOUNDARY_* kinds
struct BoundaryTreatmentByCustomExtrapolation {  // ghost state v = u (outflow) or a prescribed state
  int kind = GDT_FV_BOUNDARY_EXTRAPOLATE;
  double value = 0.0;
  BoundaryTreatmentByCustomExtrapolation() = default;
  explicit BoundaryTreatmentByCustomExtrapolation(double state) : kind(GDT_FV_BOUNDARY_DIRICHLET), value(state) {}
};
struct BoundaryTreatmentByCustomNumericalFlux {  // boundary flux f.n = value (0: impermeable wall)
  int kind = GDT_FV_BOUNDARY_FLUX;
  double value = 0.0;
  explicit BoundaryTreatmentByCustomNumericalFlux(double g = 0.0) : value(g) {}
};
enum class Side { minus_x = 0, plus_x = 1, minus_y = 2, plus_y = 3, minus_z = 4, plus_z = 5 };

// AdvectionFvOperator(grid_view, numerical_flux, source_space, range_space) (operators/advection-fv.hh:66-115)
template <int d>
class AdvectionFvOperator {
 public:
  template <class NF>
  AdvectionFvOperator(const CubeGrid<d>& /*grid_view*/, const NF& numerical_flux, const Space<d>& source_space,
                      const Space<d>& /*range_space*/)
      : space_(source_space) {
    numerical_flux.lower(desc_);
  }
  // append(boundary treatment, filter): the sides it applies to (all boundary sides when empty)
  template <class T>
  AdvectionFvOperator& append(const T& treatment, std::vector<Side> sides = {}) {
    if (sides.empty())
      for (int k = 0; k < 2 * d; ++k) sides.push_back(Side(k));
    for (Side sd : sides) {
      desc_.boundary[int(sd)] = treatment.kind;
      desc_.boundary_value[int(sd)] = treatment.value;
    }
    return *this;
  }
  void apply(const DeviceVector& source, DeviceVector& range) const {
    check(gdt_fv_apply(default_context(), space_.handle(), &desc_, source.data(), range.data()), default_context(),
          "AdvectionFvOperator::apply");
  }
  const gdt_fv_desc& desc() const { return desc_; }
  const Space<d>& space() const { return space_; }

 private:
  Space<d> space_;
  gdt_fv_desc desc_{};
};

// estimate_dt_for_hyperbolic_system(grid_view, initial_values, flux) (tools/hyperbolic.hh:38-86)
template <int d>
double estimate_dt_for_hyperbolic_system(const CubeGrid<d>& /*grid_view*/, const DeviceVector& initial_values,
                                         const AdvectionFvOperator<d>& op) {
  double dt = 0.0;
  check(gdt_fv_estimate_dt(default_context(), op.space().handle(), &op.desc(), initial_values.data(), &dt),
        default_context(), "estimate_dt_for_hyperbolic_system");
  return dt;
}

// ExplicitRungeKuttaTimeStepper(op, initial_values, r = -1) with the explicit Euler or the second-order
// SSP tableau (tools/timestepper/explicit-rungekutta.hh:82-97, 237-270); the state lives on the device
template <int d>
class ExplicitRungeKuttaTimeStepper {
 public:
  ExplicitRungeKuttaTimeStepper(const AdvectionFvOperator<d>& op, DeviceVector& initial_values,
                                int method = GDT_TIMESTEPPER_SSPRK2)
      : op_(op), u_(initial_values), method_(method),
        work_(GDT_FV_WORK_DOUBLES(method, 1, initial_values.size())) {}
  // one step of size dt (the reference's step(): u^{n+1} from u^n); returns dt
  double step(double dt, int64_t steps = 1) {
    check(gdt_fv_timestep(default_context(), op_.space().handle(), &op_.desc(), method_, dt, steps, 1, u_.data(),
                          work_.data()),
          default_context(), "ExplicitRungeKuttaTimeStepper::step");
    t_ += dt * double(steps);
    return dt;
  }
  double current_time() const { return t_; }
  const DeviceVector& current_solution() const { return u_; }

 private:
  const AdvectionFvOperator<d>& op_;
  DeviceVector& u_;
  int method_;
  DeviceVector work_;
  double t_ = 0.0;
};

}  // namespace GB300
}  // namespace GDT
}  // namespace Dune
