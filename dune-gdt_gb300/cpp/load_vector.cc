// The load vector of the ESV2007 source (examples/stationary-heat-equation.cc:68-70) through the C++
// facade: make_vector_functional(space) + LocalElementIntegralFunctional(
// LocalElementProductIntegrand().with_ansatz(source)), source a std::function of the global point with
// its polynomial order 3, on [-1, 1]^2 with `cells` squares per axis (split into triangles with
// simplex = 1) and continuous Lagrange elements of `order`. Prints one value per line, the DoFs in
// the space's numbering.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "gdt_gb300.hh"

using namespace Dune::GDT::GB300;

int main(int argc, char* argv[]) {
  try {
    const int64_t cells = argc > 1 ? std::atoll(argv[1]) : 8;
    const bool simplex = argc > 2 && std::atoi(argv[2]) != 0;
    const int order = argc > 3 ? std::atoi(argv[3]) : 1;
    const GridFunction<2> source = [](const FieldVector<2>& x) {
      return M_PI_2 * M_PI * std::cos(M_PI_2 * x[0]) * std::cos(M_PI_2 * x[1]);
    };
    auto grid = make_cube_grid<2>(-1., 1., cells, simplex);
    auto space = make_continuous_lagrange_space(grid, order);
    auto rhs_func = make_vector_functional(space);
    rhs_func.append(LocalElementIntegralFunctional<2>(LocalElementProductIntegrand().with_ansatz<2>(source, 3)));
    rhs_func.assemble();
    for (double v : rhs_func.vector().download()) std::printf("%.17e\n", v);
  } catch (std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return EXIT_FAILURE;
  }
  return EXIT_SUCCESS;
}
