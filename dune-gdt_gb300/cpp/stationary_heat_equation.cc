// The reference's examples/stationary-heat-equation.cc:58-140 driver on the GB300 library: same
// problem (-laplace u = f on [-1,1]^2, 128^2 cubes, Q1, u = cos(pi x/2) cos(pi y/2), homogeneous
// Dirichlet) and the same sequence of calls, with the namespace Dune::GDT::GB300. Prints the number
// of DoFs, CG iterations, the Newton steps of the residual-operator route and its difference to the
// CG solution, and the discrete maximum error at the vertices.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "gdt_gb300.hh"

using namespace Dune::GDT::GB300;

int main(int argc, char* argv[]) {
  try {
    const int64_t cells = argc > 1 ? std::atoll(argv[1]) : 128;
    const double diffusion = 1;
    const GridFunction<2> source = [](const FieldVector<2>& x) {
      return M_PI_2 * M_PI * std::cos(M_PI_2 * x[0]) * std::cos(M_PI_2 * x[1]);
    };
    auto grid = make_cube_grid<2>(/*lower_left=*/-1., /*upper_right=*/1., /*num_elements=*/cells);
    AllDirichletBoundaryInfo boundary_info;
    auto space = make_continuous_lagrange_space(grid, /*polorder=*/1);
    auto lhs_op = make_matrix_operator(space, Stencil::element);
    lhs_op.append(LocalElementIntegralBilinearForm(LocalLaplaceIntegrand(diffusion)));
    auto rhs_func = make_vector_functional(space);
    rhs_func.append(LocalElementIntegralFunctional<2>(LocalElementProductIntegrand().with_ansatz<2>(source)));
    auto dirichlet_constraints = make_dirichlet_constraints(space, boundary_info);
    auto walker = make_walker(grid);
    walker.append(lhs_op);
    walker.append(rhs_func);
    walker.append(dirichlet_constraints);
    walker.walk(/*thread_parallel=*/true);
    dirichlet_constraints.apply(lhs_op.matrix(), rhs_func.vector());
    auto solution = make_discrete_function(space);
    auto info = make_solver(lhs_op.matrix()).apply(rhs_func.vector(), solution.dofs().vector(), 1e-12);
    // the EOC studies' route to the same solution: Newton on the residual operator x -> A x - b
    auto newton_solution = make_discrete_function(space);
    gdt_newton_opts newton_opts = gdt_newton_default_opts();
    newton_opts.precision = 1e-12;
    const auto newton = lhs_op.apply_inverse(rhs_func.vector(), newton_solution.dofs().vector(), newton_opts);
    // discrete maximum error at the vertices (lexicographic, x fastest)
    const auto u = solution.dofs().vector().download();
    const auto un = newton_solution.dofs().vector().download();
    double newton_diff = 0.0, umax = 0.0;
    for (size_t k = 0; k < u.size(); ++k) {
      newton_diff = std::fmax(newton_diff, std::fabs(un[k] - u[k]));
      umax = std::fmax(umax, std::fabs(u[k]));
    }
    const int64_t nv = cells + 1;
    double err = 0.0;
    for (int64_t j = 0; j < nv; ++j)
      for (int64_t i = 0; i < nv; ++i) {
        const double x = -1.0 + 2.0 * double(i) / double(cells), y = -1.0 + 2.0 * double(j) / double(cells);
        err = std::fmax(err, std::fabs(u[size_t(j * nv + i)] - std::cos(M_PI_2 * x) * std::cos(M_PI_2 * y)));
      }
    std::printf("dofs %lld iterations %d rel_residual %.3e newton_steps %d newton_rel_diff %.3e max_vertex_error %.6e\n",
                (long long)space.size(), info.iterations, info.rel_residual, newton.iterations, newton_diff / umax, err);
  } catch (std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return EXIT_FAILURE;
  }
  return EXIT_SUCCESS;
}
