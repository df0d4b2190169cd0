"""Pins the CPU oracle to the reference's own known answers (tests/golden/reference_values.json,
extracted from the dune-gdt test sources by tests/golden/extract_reference_values.py)."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl

from conftest import fv_cell_average_1d


@pytest.mark.parametrize("simplex", [False, True])
def test_q2_stiffness_known_answers(oracle, golden, simplex):
    # dune/gdt/test/integrands/integrands_laplace.cc:115-134
    O = oracle
    ref = golden["q2_stiffness"]["simplex" if simplex else "cube"]
    g = O.grid(2, [9, 2], [0, 0], [3, 1], simplex=simplex)
    A, _ = O.assemble_cg(g, order=2, dirichlet=False)
    D = A.dense()
    assert abs(D.min() - ref["min_entry"]) < 1e-13
    assert abs(D.max() - ref["max_entry"]) < 1e-13
    # the reference allows 5e-12 absolute on a sum of 9025 squares; the simplex sum differs from the
    # printed 16-digit value in the 15th digit, so compare relative to 1e-14
    assert abs((D ** 2).sum() - ref["square_sum"]) < 1e-14 * ref["square_sum"]


@pytest.mark.parametrize("simplex", [False, True])
def test_q2_mass_known_answers(oracle, golden, simplex):
    # dune/gdt/test/integrands/integrands_product.cc:107-125
    O = oracle
    ref = golden["q2_mass"]["simplex" if simplex else "cube"]
    g = O.grid(2, [9, 2], [0, 0], [3, 1], simplex=simplex)
    D = O.assemble_mass(g, O.CG, 2).dense()
    assert abs(D.min() - ref["min_entry"]) < 1e-13
    assert abs(D.max() - ref["max_entry"]) < 1e-13
    assert abs((D ** 2).sum() - ref["square_sum"]) < 5e-12


def _burgers_run(O, ncell, numflux, fixed_dt):
    g = O.grid(1, [ncell], [0], [1], periodic=True)
    u0 = fv_cell_average_1d(ncell, lambda x: np.exp(-(x - 0.33) ** 2 / (2 * 0.075 ** 2)), 3)
    fv_dt = O.fv_estimate_dt(g, O.FLUX_BURGERS, u0)
    dt = 0.99 * fixed_dt  # setup.dt_factor default, dune/gdt/test/burgers/base.hh:181
    sols, t, u = [u0.copy()], 0.0, u0.copy()
    while t < 1.0 + dt:  # test/instationary-eocstudies/base.hh:439-446
        u = O.fv_explicit_euler(g, O.FLUX_BURGERS, numflux, u, dt, 1)
        t += dt
        sols.append(u.copy())
    return sols, dt / fv_dt


@pytest.mark.parametrize("flux", ["numerical_upwind_flux", "numerical_lax_friedrichs_flux", "numerical_engquist_osher_flux"])
def test_burgers_1d_fv_tables(oracle, golden, flux):
    # dune/gdt/test/burgers/burgers__1d__explicit__fv.{cc,mini}: 16 and 32 cells, reference on 128
    O = oracle
    case = golden["burgers_1d"][flux]
    res = case["results"]
    nf = {"numerical_upwind_flux": O.NUMFLUX_UPWIND, "numerical_lax_friedrichs_flux": O.NUMFLUX_LAX_FRIEDRICHS,
          "numerical_engquist_osher_flux": O.NUMFLUX_ENGQUIST_OSHER}[flux]
    runs = {n: _burgers_run(O, n, nf, case["setup"]["use_fixed_dt"]) for n in (16, 32, 128)}
    for lvl, n in enumerate((16, 32)):
        sols, cfl = runs[n]
        assert len(sols) == res["quantity.num_timesteps"][lvl]
        assert float("%.2e" % cfl) == pytest.approx(res["quantity.CFL"][lvl], rel=1e-12)
        mass0 = sols[0].sum() / n
        mc = max(abs(mass0 - s.sum() / n) / mass0 for s in sols[1:])
        assert mc < res["zero_tolerance"]
        r = 128 // n
        err = max(np.sqrt(np.sum((np.repeat(a, r) - b) ** 2) / 128) for a, b in zip(sols, runs[128][0]))
        assert float("%.2e" % err) == pytest.approx(res["norm.L_infty_L_2"][lvl], rel=1e-12)


def test_esv2007_swipdg_cube_h1_errors(oracle, golden):
    # NearlyESV2007Table1ButWithCubicGridTest: [-1,1]^2, 8x8 cubes refined twice, DG Q1, SWIPDG with
    # sigma_in = 8, sigma_bd = 14, h = |I| (test/stationary-heat-equation/ESV2007.hh:103-113), force order 4
    O = oracle
    ref = golden["esv2007_cube"]["results"]["norm.H_1_semi"]
    for lvl, n in enumerate((8, 16, 32)):
        g = O.grid(2, [n, n], [-1, -1], [1, 1])
        A, b = O.assemble_swipdg(g, order=1, force_fn=O.FORCE_ESV2007, force_order=4, theta=1.0,
                                 sigma_inner=8.0, sigma_boundary=14.0)
        u = spl.spsolve(A.to_scipy().tocsc(), b)
        err = O.h1_semi_error_esv2007(g, O.DG, 1, u)
        assert float("%.2e" % err) == pytest.approx(ref[lvl], rel=1e-12)


def test_oracle_krylov_matches_direct_solve(oracle):
    O = oracle
    rng = np.random.default_rng(7)
    g = O.grid(2, [12, 10], [0, 0], [1, 1])
    kappa = np.exp(rng.standard_normal(O.num_elements(g)))
    A, b = O.assemble_cg(g, order=1, kappa=kappa)
    xd = spl.spsolve(A.to_scipy().tocsc(), b)
    for solver in (O.SOLVER_CG, O.SOLVER_BICGSTAB):
        for prec in (O.PREC_NONE, O.PREC_JACOBI, O.PREC_ILU0):
            x, it, rr, st = O.solve(A, b, solver=solver, prec=prec, tol=1e-13)
            assert st == 0
            assert np.abs(x - xd).max() < 1e-11 * np.abs(xd).max()
