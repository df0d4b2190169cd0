"""SWIPDG (DG P1 on triangles) on the GPU against the oracle: matrix + RHS within 1e-12, solve,
and the adjoint log-kappa gradient against the oracle and against central finite differences."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl
import torch

from conftest import csr_equal_pattern, rel_err

pytestmark = pytest.mark.gpu


def _setup(gdt, oracle, n, seed=3, contrast=False, theta=1.0, swipdg=True):
    g = gdt.make_cube_grid([0, 0], [1, 1], n, simplex=True)
    og = oracle.grid(2, n, 0.0, 1.0, simplex=True)
    rng = np.random.default_rng(seed)
    logk = rng.standard_normal(g.num_elements)
    if contrast:
        ne = g.num_elements
        cy = (np.arange(ne) // 2) // n[0]
        logk = logk + np.where((cy // 2) % 2 == 1, np.log(1e4), 0.0)
    kappa = np.exp(logk)
    force = rng.uniform(0.5, 1.5, g.num_elements)
    space = gdt.DiscontinuousLagrangeSpace(g, 1)
    op = gdt.MatrixOperator(g, space, stencil=gdt.Stencil.element_and_intersection)
    kt = torch.tensor(kappa, device="cuda")
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(kt))
    op += gdt.LocalCouplingIntersectionIntegralBilinearForm(
        gdt.LocalLaplaceIPDGInnerCoupling(theta, kt, kt if swipdg else None) + gdt.LocalIPDGInnerPenalty(8.0, kt))
    op += gdt.LocalIntersectionIntegralBilinearForm(
        gdt.LocalLaplaceIPDGDirichletCoupling(theta, kt) + gdt.LocalIPDGBoundaryPenalty(14.0, kt))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=torch.tensor(force, device="cuda"))
    A, b = oracle.assemble_swipdg(og, 1, kappa=kappa, force=force, theta=theta, sigma_inner=8.0,
                                  sigma_boundary=14.0, weight_is_diffusion=swipdg)
    return g, og, space, op, rhs, A, b, kappa


@pytest.mark.parametrize("n", [[5, 4], [12, 9]])
@pytest.mark.parametrize("theta,swipdg", [(1.0, True), (1.0, False), (-1.0, True), (0.0, True)])
def test_swipdg_assembly_matches_oracle(gdt, oracle, n, theta, swipdg):
    g, og, space, op, rhs, A, b, kappa = _setup(gdt, oracle, n, theta=theta, swipdg=swipdg)
    rp, col, val = op.csr()
    assert csr_equal_pattern((rp, col, val), A)
    assert rel_err(val.cpu().numpy(), A.val) < 1e-12
    assert rel_err(rhs.cpu().numpy(), b) < 1e-12


def test_swipdg_high_contrast_solve(gdt, oracle):
    g, og, space, op, rhs, A, b, kappa = _setup(gdt, oracle, [32, 32], contrast=True)
    assert rel_err(op.csr()[2].cpu().numpy(), A.val) < 1e-12
    xd = spl.spsolve(A.to_scipy().tocsc(), b)
    x = op.apply_inverse(rhs, opts={"tol": 1e-13, "max_iter": 200000})
    assert rel_err(x.cpu().numpy(), xd) < 1e-8


def test_swipdg_adjoint_matches_oracle(gdt, oracle):
    g, og, space, op, rhs, A, b, kappa = _setup(gdt, oracle, [10, 8], contrast=True)
    rng = np.random.default_rng(0)
    u = rng.standard_normal(space.num_DoFs)
    lam = rng.standard_normal(space.num_DoFs)
    ref = oracle.swipdg_dlogkappa(og, kappa, u, lam)
    out = gdt.dlogkappa(op, torch.tensor(u, device="cuda"), torch.tensor(lam, device="cuda"),
                        torch.tensor(kappa, device="cuda"))
    assert rel_err(out.cpu().numpy(), ref) < 1e-9


def test_cg_adjoint_matches_oracle(gdt, oracle):
    n = [9, 7]
    g = gdt.make_cube_grid([0, 0], [1, 1], n, simplex=True)
    og = oracle.grid(2, n, 0.0, 1.0, simplex=True)
    rng = np.random.default_rng(1)
    kappa = np.exp(rng.standard_normal(g.num_elements))
    prob = gdt.DiffusionProblem(g)
    prob.assemble(torch.tensor(kappa, device="cuda"))
    nd = prob.space.num_DoFs
    bnd = oracle.dirichlet_dofs(og, 1)
    u = rng.standard_normal(nd)
    lam = rng.standard_normal(nd)
    u[bnd] = 0.0
    lam[bnd] = 0.0
    ref = oracle.cg_dlogkappa(og, kappa, u, lam)
    out = gdt.dlogkappa(prob.op, torch.tensor(u, device="cuda"), torch.tensor(lam, device="cuda"),
                        torch.tensor(kappa, device="cuda"))
    assert rel_err(out.cpu().numpy(), ref) < 1e-12


@pytest.mark.parametrize("dg", [True, False])
def test_autograd_gradient_matches_central_differences(gdt, dg):
    # J = 0.5 ||u - u_d||^2; dJ/dlog(kappa) via DiffusionSolve.backward vs central FD (h = 1e-6)
    n = [16, 16]
    g = gdt.make_cube_grid([0, 0], [1, 1], n, simplex=True)
    prob = gdt.DiffusionProblem(g, dg=dg, solver_opts={"tol": 1e-14, "max_iter": 200000})
    rng = np.random.default_rng(5)
    logk = torch.tensor(rng.standard_normal(g.num_elements), device="cuda", requires_grad=True)
    u_d = prob.solve(torch.exp(torch.tensor(rng.standard_normal(g.num_elements), device="cuda"))).clone()

    def J(lk):
        u = gdt.DiffusionSolve.apply(lk, prob)
        return 0.5 * torch.sum((u - u_d) ** 2)

    j = J(logk)
    j.backward()
    grad = logk.grad.detach().cpu().numpy()
    h = 1e-6
    picks = rng.choice(g.num_elements, 12, replace=False)
    for e in picks:
        with torch.no_grad():
            lp = logk.detach().clone()
            lp[e] += h
            lm = logk.detach().clone()
            lm[e] -= h
            fd = (J(lp).item() - J(lm).item()) / (2 * h)
        assert abs(fd - grad[e]) <= 1e-5 * max(abs(grad).max(), 1e-30)


def _dirichlet_test_fn(x):
    # the oracle's Dirichlet test data g = cos(pi x / 2) cos(pi y / 2) + 0.3 x
    return torch.cos(0.5 * np.pi * x[..., 0]) * torch.cos(0.5 * np.pi * x[..., 1]) + 0.3 * x[..., 0]


def _dg_operator(gdt, g, kt, coupling, penalty):
    space = gdt.DiscontinuousLagrangeSpace(g, 1)
    op = gdt.MatrixOperator(g, space, stencil=gdt.Stencil.element_and_intersection)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(kt))
    op += gdt.LocalCouplingIntersectionIntegralBilinearForm(
        gdt.LocalLaplaceIPDGInnerCoupling(1.0, kt, kt) + gdt.LocalIPDGInnerPenalty(8.0, kt))
    op += gdt.LocalIntersectionIntegralBilinearForm(coupling + penalty)
    return space, op


@pytest.mark.parametrize("terms", [1, 2, 3])
@pytest.mark.parametrize("data", ["function", "constant"])
def test_swipdg_dirichlet_data_matches_oracle(gdt, oracle, terms, data):
    # non-homogeneous Dirichlet data on the right-hand side: the unary DirichletCoupling term
    # -theta int g (kappa grad psi_i . n) (local/integrands/laplace-ipdg.hh:292-320) and/or the boundary
    # penalty's counterpart, g a function evaluated at the face quadrature points or a constant
    n = [12, 9]
    g = gdt.make_cube_grid([-1, -1], [1, 1], n, simplex=True)
    og = oracle.grid(2, n, -1.0, 1.0, simplex=True)
    kappa = np.exp(np.random.default_rng(21).standard_normal(g.num_elements))
    kt = torch.tensor(kappa, device="cuda")
    gd = gdt.GridFunction(_dirichlet_test_fn, order=3) if data == "function" else 0.7
    coupling = gdt.LocalLaplaceIPDGDirichletCoupling(1.0, kt, gd if terms & 1 else 0.0)
    penalty = gdt.LocalIPDGBoundaryPenalty(14.0, kt, dirichlet_data=gd if terms & 2 else None)
    space, op = _dg_operator(gdt, g, kt, coupling, penalty)
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=1.0)
    A, b = oracle.assemble_swipdg(og, 1, kappa=kappa, force_const=1.0,
                                  dirichlet_fn=oracle.DIRICHLET_TEST if data == "function" else oracle.DIRICHLET_CONST,
                                  dirichlet_const=0.7, dirichlet_rhs=terms)
    assert rel_err(op.csr()[2].cpu().numpy(), A.val) < 1e-12
    assert rel_err(rhs.cpu().numpy(), b) < 1e-12
    _, b0 = oracle.assemble_swipdg(og, 1, kappa=kappa, force_const=1.0)
    assert np.abs(b - b0).max() > 1e-6 * np.abs(b0).max()  # the data terms are not negligible


@pytest.mark.parametrize("beta", [None, 0.5])
def test_deprecated_elliptic_ipdg_integrands(gdt, oracle, beta):
    # LocalEllipticIpdgIntegrands (local/integrands/elliptic-ipdg.hh): sigma from the polynomial order
    # (8 inner, 14 boundary for order 1) and the penalty length |I|^beta, beta = 1 / (d - 1) by default;
    # in 2D the default is the LaplaceIPDG form exactly, another beta changes the penalty only
    assert gdt.LocalEllipticIpdgIntegrands.inner_sigma(1) == 8.0
    assert gdt.LocalEllipticIpdgIntegrands.boundary_sigma(1) == 14.0
    assert gdt.LocalEllipticIpdgIntegrands.inner_sigma(2) == 20.0 and gdt.LocalEllipticIpdgIntegrands.boundary_sigma(3) == 74.0
    assert gdt.LocalEllipticIpdgIntegrands.default_beta(2) == 1.0 and gdt.LocalEllipticIpdgIntegrands.default_beta(3) == 0.5
    n = [10, 7]
    g = gdt.make_cube_grid([0, 0], [1, 1], n, simplex=True)
    og = oracle.grid(2, n, 0.0, 1.0, simplex=True)
    kappa = np.exp(np.random.default_rng(22).standard_normal(g.num_elements))
    kt = torch.tensor(kappa, device="cuda")
    space = gdt.DiscontinuousLagrangeSpace(g, 1)
    op = gdt.MatrixOperator(g, space, stencil=gdt.Stencil.element_and_intersection)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(kt))
    op += gdt.LocalCouplingIntersectionIntegralBilinearForm(gdt.LocalEllipticIpdgIntegrands.Inner(kt, beta=beta))
    op += gdt.LocalIntersectionIntegralBilinearForm(gdt.LocalEllipticIpdgIntegrands.DirichletBoundary(kt, beta=beta))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=1.0)
    A, b = oracle.assemble_swipdg(og, 1, kappa=kappa, force_const=1.0, beta=1.0 if beta is None else beta)
    assert rel_err(op.csr()[2].cpu().numpy(), A.val) < 1e-12
    assert rel_err(rhs.cpu().numpy(), b) < 1e-12
    if beta is not None:
        A1, _ = oracle.assemble_swipdg(og, 1, kappa=kappa, force_const=1.0)
        assert np.abs(A.val - A1.val).max() > 1e-3 * np.abs(A1.val).max()
