"""The reference's stationary-heat-equation driver, written against the C++ facade (same calls as
examples/stationary-heat-equation.cc:87-110), runs on the GPU and converges to the exact solution."""
import os
import subprocess

import pytest

from conftest import ROOT, import_gdt

pytestmark = pytest.mark.gpu


def test_stationary_heat_equation_example(gdt):
    exes = gdt._build.build_examples()
    exe = [e for e in exes if e.endswith("stationary_heat_equation")][0]
    errs = []
    for cells in (32, 64):
        out = subprocess.run([exe, str(cells)], capture_output=True, text=True, timeout=300, check=True).stdout
        fields = out.split()
        assert int(fields[1]) == (cells + 1) ** 2
        # Newton on x -> A x - b (OperatorInterface::apply_inverse) reaches the CG solution in one step
        assert fields[6] == "newton_steps" and int(fields[7]) == 1
        assert float(fields[9]) < 1e-8
        errs.append(float(fields[-1]))
    # second-order convergence of the vertex error (the source at the product integrand's quadrature points)
    assert errs[1] < errs[0] / 3.0
    assert errs[1] < 2e-3


@pytest.mark.parametrize("simplex,order", [(0, 1), (1, 1), (0, 2), (1, 2)])
def test_facade_load_vector_matches_oracle(gdt, oracle, simplex, order):
    # a function-valued source through the facade is evaluated at the quadrature points of its product
    # integrand (order of f + order of the space), as the reference does: same load vector as the oracle
    import numpy as np

    exes = gdt._build.build_examples()
    exe = [e for e in exes if e.endswith("load_vector")][0]
    cells = 6
    out = subprocess.run([exe, str(cells), str(simplex), str(order)], capture_output=True, text=True, timeout=300,
                         check=True).stdout.split()
    v = np.array([float(t) for t in out])
    og = oracle.grid(2, [cells, cells], -1.0, 1.0, simplex=bool(simplex))
    _, b = oracle.assemble_cg(og, order, kappa_const=1.0, force_fn=oracle.FORCE_ESV2007, force_order=3,
                              dirichlet=False)
    assert v.shape == b.shape
    assert np.abs(v - b).max() <= 1e-12 * np.abs(b).max()


@pytest.mark.parametrize("flux,name", [("numerical_upwind_flux", "upwind"),
                                       ("numerical_lax_friedrichs_flux", "lax_friedrichs"),
                                       ("numerical_engquist_osher_flux", "engquist_osher")])
def test_burgers_1d_fv_example(gdt, golden, flux, name):
    # test/burgers/burgers__1d__explicit__fv.mini through the C++ facade (AdvectionFvOperator,
    # estimate_dt_for_hyperbolic_system, ExplicitRungeKuttaTimeStepper): step counts and CFL of the
    # reference table, mass conserved
    exes = gdt._build.build_examples()
    exe = [e for e in exes if e.endswith("burgers_1d_fv")][0]
    case = golden["burgers_1d"][flux]
    res = case["results"]
    dt = 0.99 * case["setup"]["use_fixed_dt"]
    for lvl, n in enumerate((16, 32)):
        out = subprocess.run([exe, name, str(n), repr(dt)], capture_output=True, text=True, timeout=300,
                             check=True).stdout.split()
        assert out[0] == "cells" and int(out[1]) == n
        assert int(out[3]) == res["quantity.num_timesteps"][lvl]
        assert float("%.2e" % float(out[5])) == pytest.approx(res["quantity.CFL"][lvl], rel=1e-12)
        assert float(out[7]) < 1e-14


@pytest.mark.parametrize("simplex", [0, 1])
def test_facade_mapped_grid_solution_matches_oracle(gdt, oracle, simplex):
    # CubeGrid::set_vertices (a GeometryGrid-like mapped grid) through the unchanged driver calls: the
    # solution equals a direct solve of the oracle's system on the same moved vertices
    import numpy as np
    import scipy.sparse.linalg as spl

    exes = gdt._build.build_examples()
    exe = [e for e in exes if e.endswith("mapped_grid")][0]
    cells = 12
    out = subprocess.run([exe, str(cells), str(simplex)], capture_output=True, text=True, timeout=300,
                         check=True).stdout.split()
    u = np.array([float(t) for t in out])
    t = np.linspace(0.0, 1.0, cells + 1)
    X = np.stack([np.tile(t, cells + 1), np.repeat(t, cells + 1)], axis=1)
    xv = X.copy()
    for a in range(2):
        xv[:, a] = X[:, a] + 0.04 * np.sin(2 * np.pi * X[:, a]) * (1.0 + X[:, (a + 1) % 2])
    og = oracle.grid(2, [cells, cells], 0.0, 1.0, simplex=bool(simplex), vertices=xv)
    A, b = oracle.assemble_cg(og, 1, kappa_const=1.0, force_const=1.0, dirichlet=True)
    ud = spl.spsolve(A.to_scipy().tocsc(), b)
    assert u.shape == ud.shape
    assert np.abs(u - ud).max() <= 1e-9 * np.abs(ud).max()


@pytest.mark.parametrize("dim,n", [(2, 12), (3, 5)])
def test_facade_mesh_driver_matches_oracle(gdt, oracle, dim, n, tmp_path):
    # make_simplex_mesh<d>(coords, cells) through the unchanged driver calls on a Delaunay mesh read
    # from a file: the solution equals a direct solve of the oracle's system on the same mesh
    import numpy as np
    import scipy.sparse.linalg as spl

    spatial = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(21 + dim)
    t = np.linspace(0.0, 1.0, n + 1)
    X = np.stack(np.meshgrid(*([t] * dim), indexing="ij"), -1).reshape(-1, dim)
    inner = np.all((X > 0) & (X < 1), axis=1)
    X[inner] += (0.3 / n) * rng.uniform(-1, 1, (inner.sum(), dim))
    cells = spatial.Delaunay(X).simplices.astype(np.int64)
    J = np.stack([X[cells[:, k + 1]] - X[cells[:, 0]] for k in range(dim)], axis=-1)
    vol = np.abs(np.linalg.det(J))
    cells = cells[vol > 1e-9 * vol.max()]
    path = tmp_path / "mesh.txt"
    with open(path, "w") as f:
        f.write(f"{dim} {X.shape[0]} {cells.shape[0]}\n")
        np.savetxt(f, X, fmt="%.17e")
        np.savetxt(f, cells, fmt="%d")
    exes = gdt._build.build_examples()
    exe = [e for e in exes if e.endswith("mesh_heat")][0]
    out = subprocess.run([exe, str(path)], capture_output=True, text=True, timeout=300, check=True).stdout.split()
    u = np.array([float(v) for v in out])
    A, b = oracle.mesh_assemble(X, cells, kappa_const=1.0, force_const=1.0, dirichlet=True)
    ud = spl.spsolve(A.to_scipy().tocsc(), b)
    assert u.shape == ud.shape
    assert np.abs(u - ud).max() <= 1e-9 * np.abs(ud).max()
