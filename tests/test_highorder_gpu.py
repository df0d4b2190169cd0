"""Order-2 continuous Lagrange spaces and the element-batched (FP64 tensor-core) assembly on the GPU
against the CPU oracle: DoF numbering and sparsity pattern bit-exact, stiffness / product (mass) /
load vector / Dirichlet constraints within 1e-12, the reference's Q2 known answers
(dune/gdt/test/integrands/integrands_laplace.cc, integrands_product.cc) and solves."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl
import torch

from conftest import csr_equal_pattern, rel_err

pytestmark = pytest.mark.gpu

GRIDS = [(1, [7], False), (2, [5, 4], False), (2, [4, 3], True), (3, [3, 2, 4], False), (3, [2, 3, 2], True)]


def _grid(gdt, oracle, dim, n, simplex):
    lo = [0.0] * dim
    hi = [1.0 + 0.5 * a for a in range(dim)]
    return gdt.make_cube_grid(lo, hi, n, simplex=simplex), oracle.grid(dim, n, lo, hi, simplex=simplex)


@pytest.mark.parametrize("dim,n,simplex", GRIDS)
def test_order2_global_indices_bit_exact(gdt, oracle, dim, n, simplex):
    g, og = _grid(gdt, oracle, dim, n, simplex)
    sp = gdt.ContinuousLagrangeSpace(g, 2)
    assert sp.num_DoFs == oracle.space_size(og, oracle.CG, 2)
    assert np.array_equal(sp.global_indices().cpu().numpy(), oracle.global_indices(og, oracle.CG, 2))


@pytest.mark.parametrize("dim,n,simplex", GRIDS)
def test_order2_pattern_bit_exact(gdt, oracle, dim, n, simplex):
    g, og = _grid(gdt, oracle, dim, n, simplex)
    op = gdt.MatrixOperator(g, gdt.ContinuousLagrangeSpace(g, 2))
    ref = oracle.pattern(og, oracle.CG, 2, oracle.STENCIL_ELEMENT)
    assert op.nnz == ref.nnz
    assert csr_equal_pattern(op.csr(), ref)


@pytest.mark.parametrize("dim,n,simplex", GRIDS)
@pytest.mark.parametrize("dirichlet", [True, False])
def test_order2_assembly_matches_oracle(gdt, oracle, dim, n, simplex, dirichlet):
    g, og = _grid(gdt, oracle, dim, n, simplex)
    rng = np.random.default_rng(17 + dim)
    kappa = np.exp(rng.standard_normal(g.num_elements))
    force = rng.uniform(-1, 2, g.num_elements)
    A, b = oracle.assemble_cg(og, 2, kappa=kappa, force=force, dirichlet=dirichlet)
    space = gdt.ContinuousLagrangeSpace(g, 2)
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(torch.tensor(kappa, device="cuda")))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=torch.tensor(force, device="cuda"), dirichlet=dirichlet)
    rp, col, val = op.csr()
    assert csr_equal_pattern((rp, col, val), A)
    assert rel_err(val.cpu().numpy(), A.val) < 1e-12
    assert rel_err(rhs.cpu().numpy(), b) < 1e-12
    # the load vector alone (VectorBasedFunctional) and the separate Dirichlet pass
    f = gdt.VectorFunctional(g, space)
    f.append(gdt.LocalElementIntegralFunctional(
        gdt.LocalElementProductIntegrand().with_ansatz(torch.tensor(force, device="cuda"))))
    f.assemble()
    _, b0 = oracle.assemble_cg(og, 2, kappa=kappa, force=force, dirichlet=False)
    assert rel_err(f.vector.cpu().numpy(), b0) < 1e-12


@pytest.mark.parametrize("simplex", [False, True])
def test_q2_known_answers_on_gpu(gdt, golden, simplex):
    # dune/gdt/test/integrands/integrands_laplace.cc:115-134 and integrands_product.cc:107-125
    g = gdt.make_cube_grid([0, 0], [3, 1], [9, 2], simplex=simplex)
    space = gdt.ContinuousLagrangeSpace(g, 2)
    for form, key in ((gdt.LocalLaplaceIntegrand(1.0), "q2_stiffness"), (gdt.LocalElementProductIntegrand(1.0), "q2_mass")):
        op = gdt.MatrixOperator(g, space)
        op += gdt.LocalElementIntegralBilinearForm(form)
        op.assemble()
        rp, col, val = (t.cpu().numpy() for t in op.csr())
        n = space.num_DoFs
        import scipy.sparse as sp

        D = sp.csr_matrix((val, col, rp), shape=(n, n)).toarray()
        ref = golden[key]["simplex" if simplex else "cube"]
        assert abs(D.min() - ref["min_entry"]) < 1e-13
        assert abs(D.max() - ref["max_entry"]) < 1e-13
        assert abs((D ** 2).sum() - ref["square_sum"]) < 1e-13 * max(1.0, ref["square_sum"])


@pytest.mark.parametrize("dim,n,simplex", [(2, [5, 4], False), (2, [4, 3], True), (3, [3, 2, 2], False),
                                           (3, [2, 2, 3], True), (1, [6], False)])
@pytest.mark.parametrize("order", [1, 2])
def test_product_form_matches_oracle(gdt, oracle, dim, n, simplex, order):
    g, og = _grid(gdt, oracle, dim, n, simplex)
    M = oracle.assemble_mass(og, oracle.CG, order)
    space = gdt.ContinuousLagrangeSpace(g, order)
    for weight in (1.0, 2.5):
        op = gdt.MatrixOperator(g, space)
        op += gdt.LocalElementIntegralBilinearForm(gdt.LocalElementProductIntegrand(weight))
        op.assemble()
        rp, col, val = op.csr()
        assert csr_equal_pattern((rp, col, val), M)
        assert rel_err(val.cpu().numpy(), weight * M.val) < 1e-12


@pytest.mark.parametrize("dim,n,simplex,order", [(2, [6, 5], False, 2), (2, [5, 4], True, 2), (3, [3, 3, 2], False, 2),
                                                 (2, [6, 5], True, 1), (3, [3, 2, 2], False, 1)])
def test_coefficients_at_quadrature_points(gdt, dim, n, simplex, order):
    # per-quadrature-point diffusion: equal values reproduce the per-element path; the matrix is
    # linear in the coefficient field; constants lie in the kernel of the Laplace stiffness
    g = gdt.make_cube_grid([0.0] * dim, [1.0] * dim, n, simplex=simplex)
    space = gdt.ContinuousLagrangeSpace(g, order)
    nq = space.quadrature()[0].shape[0]
    ne = g.num_elements
    rng = np.random.default_rng(4)

    def stiffness(kappa):
        op = gdt.MatrixOperator(g, space)
        op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(kappa))
        op.assemble()
        return op.csr()[2].clone()

    ke = torch.tensor(np.exp(rng.standard_normal(ne)), device="cuda")
    a_elem = stiffness(ke)
    a_qp = stiffness(ke[:, None].expand(ne, nq).contiguous())
    assert rel_err(a_qp.cpu().numpy(), a_elem.cpu().numpy()) < 1e-13
    k1 = torch.tensor(rng.uniform(0.5, 2.0, (ne, nq)), device="cuda")
    k2 = torch.tensor(rng.uniform(0.5, 2.0, (ne, nq)), device="cuda")
    a1, a2, a12 = stiffness(k1), stiffness(k2), stiffness(k1 + 2.0 * k2)
    assert rel_err(a12.cpu().numpy(), (a1 + 2.0 * a2).cpu().numpy()) < 1e-13
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(k1))
    op.assemble()
    ones = torch.ones(space.num_DoFs, dtype=torch.float64, device="cuda")
    assert op.apply(ones).abs().max().item() < 1e-12 * a1.abs().max().item()


@pytest.mark.parametrize("simplex", [False, True])
def test_order2_solve_matches_direct(gdt, oracle, simplex):
    g, og = _grid(gdt, oracle, 2, [24, 20], simplex)
    rng = np.random.default_rng(5)
    kappa = np.exp(rng.standard_normal(g.num_elements))
    A, b = oracle.assemble_cg(og, 2, kappa=kappa, force_const=1.0)
    space = gdt.ContinuousLagrangeSpace(g, 2)
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(torch.tensor(kappa, device="cuda")))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=1.0, dirichlet=True)
    xd = spl.spsolve(A.to_scipy().tocsc(), b)
    for precision in ("fp64", "mixed"):
        x = op.apply_inverse(rhs, opts={"tol": 1e-12, "precision": precision})
        assert op.last_solve_info["converged"]
        assert rel_err(x.cpu().numpy(), xd) < 1e-9


def _esv2007_force(x):
    # the ESV2007 source f = (pi^2 / 2) cos(pi x / 2) cos(pi y / 2) (examples/stationary-heat-equation.cc:68-70)
    return (0.5 * np.pi) * np.pi * torch.cos(0.5 * np.pi * x[..., 0]) * torch.cos(0.5 * np.pi * x[..., 1])


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("simplex", [False, True])
@pytest.mark.parametrize("fused", [True, False])
def test_source_at_quadrature_points_matches_oracle(gdt, oracle, order, simplex, fused):
    # LocalElementProductIntegrand().with_ansatz(f) with a function-valued f of order 3: the load vector
    # from f at the points of the Gauss rule of order 3 + k, as the reference's product integrand
    # evaluates it (local/integrands/product.hh:104-130), not from one value per element
    n = [6, 5]
    g = gdt.make_cube_grid([-1.0, -1.0], [1.0, 1.0], n, simplex=simplex)
    og = oracle.grid(2, n, -1.0, 1.0, simplex=simplex)
    A, b = oracle.assemble_cg(og, order, kappa_const=1.0, force_fn=oracle.FORCE_ESV2007, force_order=3,
                              dirichlet=True)
    space = gdt.ContinuousLagrangeSpace(g, order)
    f = gdt.GridFunction(_esv2007_force, order=3)
    if fused:
        op = gdt.MatrixOperator(g, space)
        op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(1.0))
        rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
        op.assemble(rhs=rhs, force=f, dirichlet=True)
        assert rel_err(op.csr()[2].cpu().numpy(), A.val) < 1e-12
        assert rel_err(rhs.cpu().numpy(), b) < 1e-12
    else:
        vf = gdt.VectorFunctional(g, space)
        vf.append(gdt.LocalElementIntegralFunctional(gdt.LocalElementProductIntegrand().with_ansatz(f)))
        vf.assemble()
        _, b_free = oracle.assemble_cg(og, order, kappa_const=1.0, force_fn=oracle.FORCE_ESV2007, force_order=3,
                                       dirichlet=False)
        assert rel_err(vf.vector.cpu().numpy(), b_free) < 1e-12


@pytest.mark.parametrize("dim,n,simplex", GRIDS[1:])
@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("per_point", [False, True])
def test_tensor_diffusion_matches_oracle(gdt, oracle, dim, n, simplex, order, per_point):
    # LocalLaplaceIntegrand with a symmetric positive definite d x d diffusion tensor per element
    # (local/integrands/laplace.hh:81-102), given per element or repeated at every quadrature point
    g, og = _grid(gdt, oracle, dim, n, simplex)
    ne = g.num_elements
    rng = np.random.default_rng(40 + dim + order)
    L = rng.standard_normal((ne, dim, dim))
    K = np.einsum("eab,ecb->eac", L, L) + 0.5 * np.eye(dim)[None]
    force = rng.uniform(-1, 2, ne)
    A, b = oracle.assemble_cg_tensor(og, order, K, force=force, dirichlet=True)
    space = gdt.ContinuousLagrangeSpace(g, order)
    kt = torch.tensor(K, device="cuda")
    if per_point:
        nq = space.quadrature()[0].shape[0]
        kt = kt[:, None].expand(ne, nq, dim, dim).contiguous()
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(kt))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=torch.tensor(force, device="cuda"), dirichlet=True)
    rp, col, val = op.csr()
    assert csr_equal_pattern((rp, col, val), A)
    assert rel_err(val.cpu().numpy(), A.val) < 1e-12
    assert rel_err(rhs.cpu().numpy(), b) < 1e-12
    x = op.apply_inverse(rhs, opts={"tol": 1e-13})
    assert rel_err(x.cpu().numpy(), spl.spsolve(A.to_scipy().tocsc(), b)) < 1e-10
