// The reference's 1D Burgers finite-volume test (test/burgers/burgers__1d__explicit__fv.mini with the
// driver of test/instationary-eocstudies/base.hh:428-447: explicit Euler with a fixed dt up to t = 1),
// written against the C++ facade: AdvectionFvOperator with the numerical flux given on the command
// line, estimate_dt_for_hyperbolic_system, ExplicitRungeKuttaTimeStepper. Prints the number of time
// steps, the CFL (dt over the explicit FV dt) and the largest relative mass change.
//
// usage: burgers_1d_fv <lax_friedrichs|upwind|engquist_osher> <cells> <dt>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "gdt_gb300.hh"

using namespace Dune::GDT::GB300;

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s <lax_friedrichs|upwind|engquist_osher> <cells> <dt>\n", argv[0]);
    return 2;
  }
  const std::string nf = argv[1];
  const int64_t n = std::atoll(argv[2]);
  const double dt = std::atof(argv[3]);
  auto grid = make_cube_grid<1>(0.0, 1.0, n, /*simplex=*/false, /*periodic=*/true);
  auto space = make_finite_volume_space(grid);
  // FiniteVolume interpolation of the initial value: element integral with a 2-point Gauss rule
  std::vector<double> u0(n);
  const double h = 1.0 / double(n), g = 0.5 / std::sqrt(3.0);
  for (int64_t i = 0; i < n; ++i) {
    double acc = 0.0;
    for (double xq : {0.5 - g, 0.5 + g}) {
      const double x = (double(i) + xq) * h;
      acc += 0.5 * std::exp(-(x - 0.33) * (x - 0.33) / (2 * 0.075 * 0.075));
    }
    u0[i] = acc;
  }
  DeviceVector u(n);
  u.upload(u0);
  const BurgersFlux flux;
  auto make_op = [&]() {
    if (nf == "upwind") return AdvectionFvOperator<1>(grid, NumericalUpwindFlux<BurgersFlux>(flux), space, space);
    if (nf == "engquist_osher")
      return AdvectionFvOperator<1>(grid, NumericalEngquistOsherFlux<BurgersFlux>(flux), space, space);
    return AdvectionFvOperator<1>(grid, NumericalLaxFriedrichsFlux<BurgersFlux>(flux), space, space);
  };
  const auto op = make_op();
  const double fv_dt = estimate_dt_for_hyperbolic_system(grid, u, op);
  ExplicitRungeKuttaTimeStepper<1> stepper(op, u, GDT_TIMESTEPPER_EXPLICIT_EULER);
  double m0 = 0.0;
  for (double v : u0) m0 += v * h;
  double t = 0.0, max_mass_change = 0.0;
  int count = 1;
  while (t < 1.0 + dt) {
    stepper.step(dt);
    t += dt;
    ++count;
    double m = 0.0;
    for (double v : u.download()) m += v * h;
    max_mass_change = std::max(max_mass_change, std::fabs(m - m0) / m0);
  }
  std::printf("cells %lld timesteps %d cfl %.17g mass_change %.3e\n", (long long)n, count, dt / fv_dt,
              max_mass_change);
  return 0;
}
