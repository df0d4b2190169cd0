// The stationary heat equation driver (examples/stationary-heat-equation.cc:87-110) on a mapped grid:
// the `cells` x `cells` cube grid of [0, 1]^2 (split into triangles with simplex = 1) with every vertex
// moved by x_a -> x_a + 0.04 sin(2 pi x_a) (1 + x_{a+1}), as a Dune::GeometryGrid would, unit diffusion
// and source, homogeneous Dirichlet data, continuous Lagrange elements of order 1. Prints the solution,
// one value per line, the DoFs in the space's numbering.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gdt_gb300.hh"

using namespace Dune::GDT::GB300;

int main(int argc, char* argv[]) {
  try {
    const int64_t cells = argc > 1 ? std::atoll(argv[1]) : 8;
    const bool simplex = argc > 2 && std::atoi(argv[2]) != 0;
    auto grid = make_cube_grid<2>(0., 1., cells, simplex);
    const int64_t nv = cells + 1;
    std::vector<double> xv(size_t(2 * nv * nv));
    for (int64_t j = 0; j < nv; ++j)
      for (int64_t i = 0; i < nv; ++i) {
        const double x[2] = {double(i) / double(cells), double(j) / double(cells)};
        for (int a = 0; a < 2; ++a)
          xv[size_t(2 * (j * nv + i) + a)] = x[a] + 0.04 * std::sin(2.0 * M_PI * x[a]) * (1.0 + x[(a + 1) % 2]);
      }
    grid.set_vertices(xv);
    AllDirichletBoundaryInfo boundary_info;
    auto space = make_continuous_lagrange_space(grid, /*polorder=*/1);
    auto lhs_op = make_matrix_operator(space, Stencil::element);
    lhs_op.append(LocalElementIntegralBilinearForm(LocalLaplaceIntegrand(1.0)));
    auto rhs_func = make_vector_functional(space);
    rhs_func.append(LocalElementIntegralFunctional<2>(LocalElementProductIntegrand().with_ansatz(1.0)));
    auto dirichlet_constraints = make_dirichlet_constraints(space, boundary_info);
    auto walker = make_walker(grid);
    walker.append(lhs_op);
    walker.append(rhs_func);
    walker.append(dirichlet_constraints);
    walker.walk(/*thread_parallel=*/true);
    dirichlet_constraints.apply(lhs_op.matrix(), rhs_func.vector());
    auto solution = make_discrete_function(space);
    make_solver(lhs_op.matrix()).apply(rhs_func.vector(), solution.dofs().vector(), 1e-13);
    for (double v : solution.dofs().vector().download()) std::printf("%.17e\n", v);
  } catch (std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return EXIT_FAILURE;
  }
  return EXIT_SUCCESS;
}
