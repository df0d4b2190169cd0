"""Parity at the sizes the benchmark numbers are quoted on, against the oracle on the same seeded inputs:

* 3D heat equation, 128^3 Q1 hexahedra (2,146,689 DoF, 57,066,625 nonzeros), lognormal kappa per cell:
  pattern bit-exact, matrix and right-hand side within 1e-12, the FP64 solution at a 1e-14 residual and
  the mixed-precision one at 1e-12 (its FP32 Krylov sequence stalls below that) within 1e-12 of the
  oracle's CG at 1e-14;
* SWIPDG P1 on 256^2 squares split into triangles (393,216 DoF) with the high-contrast channels of the
  adjoint workload: pattern bit-exact, matrix and right-hand side within 1e-12, solution within 1e-9
  of the oracle's: both CG solves stop at a 1e-14 residual, and the channels' 1e4 contrast on top of
  the lognormal field makes this the worst conditioned system here, so two solves at that residual
  need not agree to more digits;
* 2D Burgers FV on 4096^2 periodic cells, LF flux: 5 SSP-RK2 steps within 1e-12 of the oracle's;
* the batched parametric workload: 16 problems at its real sides 64..512 (four of each), assembled rows
  within 1e-12 and solutions within 1e-10 of the oracle's.
"""
import numpy as np
import pytest
import torch

from conftest import csr_equal_pattern, rel_err

pytestmark = pytest.mark.gpu


def _threads(oracle):
    oracle.set_threads(oracle.max_threads())


def test_heat3d_128_matches_oracle(gdt, oracle):
    _threads(oracle)
    n = 128
    kappa = np.exp(np.random.default_rng(20261205).standard_normal(n ** 3))
    g = gdt.make_cube_grid([0, 0, 0], [1, 1, 1], [n, n, n])
    space = gdt.ContinuousLagrangeSpace(g, 1)
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(torch.tensor(kappa, device="cuda")))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=1.0, dirichlet=True)
    og = oracle.grid(3, [n, n, n], 0.0, 1.0)
    A, b = oracle.assemble_cg(og, 1, kappa=kappa, force_const=1.0)
    assert (A.n, A.nnz) == (2146689, 57066625)
    rp, col, val = op.csr()
    assert csr_equal_pattern((rp, col, val), A)
    assert rel_err(val.cpu().numpy(), A.val) < 1e-12
    assert rel_err(rhs.cpu().numpy(), b) < 1e-12
    del rp, col, val
    xo, _, _, _ = oracle.solve(A, b, tol=1e-14, max_iter=400000)
    for precision, tol in (("fp64", 1e-14), ("mixed", 1e-12)):
        x = op.apply_inverse(rhs, opts={"tol": tol, "precision": precision, "max_iter": 400000})
        assert op.last_solve_info["converged"]
        assert rel_err(x.cpu().numpy(), xo) < 1e-12, precision


def test_swipdg_256_with_channels_matches_oracle(gdt, oracle):
    _threads(oracle)
    n = 256
    g = gdt.make_cube_grid([0, 0], [1, 1], [n, n], simplex=True)
    ne = g.num_elements
    rng = np.random.default_rng(20261209)
    channel = rng.random((n + 7) // 8) < 0.5
    stripe = channel[((np.arange(ne) // 2) // n) // 8].astype(np.float64)
    kappa = np.exp(rng.standard_normal(ne) + stripe * np.log(1e4))
    prob = gdt.DiffusionProblem(g, dg=True, solver_opts={"tol": 1e-14, "max_iter": 400000})
    kt = torch.tensor(kappa, device="cuda")
    x = prob.solve(kt)
    assert prob.op.last_solve_info["converged"]
    og = oracle.grid(2, [n, n], 0.0, 1.0, simplex=True)
    A, b = oracle.assemble_swipdg(og, 1, kappa=kappa, force_const=1.0, theta=1.0, sigma_inner=8.0,
                                  sigma_boundary=14.0, weight_is_diffusion=True)
    assert A.n == 393216
    rp, col, val = prob.op.csr()
    assert csr_equal_pattern((rp, col, val), A)
    assert rel_err(val.cpu().numpy(), A.val) < 1e-12
    assert rel_err(prob.rhs.cpu().numpy(), b) < 1e-12
    xo, _, _, _ = oracle.solve(A, b, tol=1e-14, max_iter=400000)
    assert rel_err(x.cpu().numpy(), xo) < 1e-9


def _bumps(n, seed, count=32):
    rng = np.random.default_rng(seed)
    xc = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(xc, xc, indexing="xy")
    u = np.zeros((n, n))
    for _ in range(count):
        a = rng.uniform(-1, 1)
        w = rng.uniform(0.01, 0.1)
        cx, cy = rng.uniform(0, 1, 2)
        dx = np.minimum(np.abs(X - cx), 1 - np.abs(X - cx))
        dy = np.minimum(np.abs(Y - cy), 1 - np.abs(Y - cy))
        u += a * np.exp(-(dx * dx + dy * dy) / (2 * w * w))
    return u.reshape(-1)


def test_fv_burgers_4096_ssp2_matches_oracle(gdt, oracle):
    _threads(oracle)
    n, steps = 4096, 5
    u0 = _bumps(n, 20261210)
    g = gdt.make_cube_grid([0, 0], [1, 1], [n, n], periodic=True)
    og = oracle.grid(2, [n, n], 0.0, 1.0, periodic=True)
    op = gdt.AdvectionFvOperator(g, gdt.NumericalLaxFriedrichsFlux(gdt.BurgersFlux()), gdt.FiniteVolumeSpace(g))
    ut = torch.tensor(u0, device="cuda")
    dt_g = gdt.estimate_dt_for_hyperbolic_system(g, ut, op)
    dt_o = oracle.fv_estimate_dt(og, oracle.FLUX_BURGERS, u0)
    assert abs(dt_g - dt_o) <= 1e-14 * dt_o
    dt = 0.5 * dt_o
    gdt.ExplicitRungeKuttaTimeStepper(op, ut, method="ssp2").step(dt, steps)
    ref = oracle.fv_ssprk2(og, oracle.FLUX_BURGERS, oracle.NUMFLUX_LAX_FRIEDRICHS, u0, dt, steps)
    assert rel_err(ut.cpu().numpy(), ref) < 1e-12
    # periodic grid: the mass is conserved to rounding
    assert abs(ut.sum().item() - u0.sum()) <= 1e-12 * np.abs(u0).sum()


OFFS = [(-1, -1), (0, -1), (-1, 0), (0, 0), (1, 0), (0, 1), (1, 1)]


def _quadrant_kappa(n, mu):
    cells = np.arange(n * n)
    cx, cy = cells % n, cells // n
    q = (cx >= n // 2).astype(int) + 2 * (cy >= n // 2).astype(int)
    return np.repeat(mu[q], 2)


def test_batched_sample_at_config_sides_matches_oracle(gdt, oracle):
    _threads(oracle)
    sides = [64, 128, 256, 512] * 4
    rng = np.random.default_rng(20261211)
    np.random.default_rng(0).shuffle(sides)
    mu = rng.uniform(0.1, 10.0, (len(sides), 4))
    b = gdt.BatchedDiffusion(sides)
    x, st = b.solve(torch.tensor(mu, device="cuda"), force=1.0, precision="fp64", tol=1e-14, max_iter=400000,
                    keep_stencil=True)
    assert b.last_info["all_converged"]
    x = x.cpu().numpy()
    st = st.cpu().numpy().reshape(-1, 7)
    for i, n in enumerate(sides):
        og = oracle.grid(2, [n, n], 0.0, 1.0, simplex=True)
        A, rhs = oracle.assemble_cg(og, 1, kappa=_quadrant_kappa(n, mu[i]), force_const=1.0)
        nv = n + 1
        # the oracle's CSR rows in the 7-point layout of the batched stencil output
        rows = np.repeat(np.arange(A.n), np.diff(A.row_ptr))
        dxy = np.stack([A.col % nv - rows % nv, A.col // nv - rows // nv], 1)
        slot = np.full(A.nnz, -1)
        for k, (dx, dy) in enumerate(OFFS):
            slot[(dxy[:, 0] == dx) & (dxy[:, 1] == dy)] = k
        assert (slot >= 0).all()
        dense = np.zeros((A.n, 7))
        dense[rows, slot] = A.val
        S = st[b.offsets[i]:b.offsets[i + 1]]
        assert rel_err(S, dense) < 1e-12, (i, n)
        xo, _, _, _ = oracle.solve(A, rhs, tol=1e-14, max_iter=400000)
        assert rel_err(x[b.offsets[i]:b.offsets[i + 1]], xo) < 1e-10, (i, n)
