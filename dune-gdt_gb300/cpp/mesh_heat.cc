// The stationary heat equation driver (examples/stationary-heat-equation.cc:87-110) on an unstructured
// simplex mesh: the grid comes from a file instead of make_cube_grid (as a gmsh or ALUGrid import
// would give it), unit diffusion and source, homogeneous Dirichlet data on the boundary vertices,
// continuous Lagrange elements of order 1. Input file: "dim num_vertices num_elements", then the
// vertex coordinates and the element vertex lists (whitespace separated). Prints the solution, one
// value per line, the DoFs in vertex order.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

#include "gdt_gb300.hh"

using namespace Dune::GDT::GB300;

template <int d>
void run(const std::vector<double>& coords, const std::vector<int64_t>& cells) {
  auto grid = make_simplex_mesh<d>(coords, cells);
  AllDirichletBoundaryInfo boundary_info;
  auto space = make_continuous_lagrange_space(grid, /*polorder=*/1);
  auto lhs_op = make_matrix_operator(space, Stencil::element);
  lhs_op.append(LocalElementIntegralBilinearForm(LocalLaplaceIntegrand(1.0)));
  auto rhs_func = make_vector_functional(space);
  rhs_func.append(LocalElementIntegralFunctional<d>(LocalElementProductIntegrand().with_ansatz<d>(1.0)));
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
}

int main(int argc, char* argv[]) {
  try {
    if (argc < 2) throw std::runtime_error("usage: mesh_heat MESHFILE");
    std::ifstream in(argv[1]);
    int dim = 0;
    long long nv = 0, ne = 0;
    if (!(in >> dim >> nv >> ne) || (dim != 2 && dim != 3) || nv < 1 || ne < 1)
      throw std::runtime_error("bad mesh header");
    std::vector<double> coords(size_t(nv) * dim);
    std::vector<int64_t> cells(size_t(ne) * (dim + 1));
    for (double& x : coords)
      if (!(in >> x)) throw std::runtime_error("bad coordinates");
    for (int64_t& c : cells) {
      long long v;
      if (!(in >> v)) throw std::runtime_error("bad element list");
      c = v;
    }
    if (dim == 2) run<2>(coords, cells);
    else run<3>(coords, cells);
  } catch (std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return EXIT_FAILURE;
  }
  return EXIT_SUCCESS;
}
