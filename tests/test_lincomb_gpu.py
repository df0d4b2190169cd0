"""Parametric lincomb (pyMOR's LincombOperator over assembled dune-gdt matrices, as in the affine
decompositions of python/dune/gdt/gamm-2019-talk-on-conservative-rb.cc:74-95) on the GPU: the combined
matrix against the oracle's matrices combined on the host, against direct assembly with the combined
coefficient (the Laplace form is linear in kappa), and parametric solves against a direct solve."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _cg_term(gdt, g, space, kappa):
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(torch.tensor(kappa, device="cuda")))
    op.assemble()
    return op


def test_lincomb_of_laplace_terms_equals_assembly_with_combined_kappa(gdt):
    n = [24, 20]
    g = gdt.make_cube_grid([0, 0], [1, 1], n, simplex=True)
    space = gdt.ContinuousLagrangeSpace(g, 1)
    rng = np.random.default_rng(2)
    kappas = [np.exp(rng.standard_normal(g.num_elements)) for _ in range(3)]
    ops = [_cg_term(gdt, g, space, k) for k in kappas]
    lop = gdt.LincombOperator(ops, [lambda mu: mu["a"], 0.5, lambda mu: 1.0 - mu["a"]])
    for a in (0.2, 0.9):
        theta = [a, 0.5, 1.0 - a]
        combined = _cg_term(gdt, g, space, sum(t * k for t, k in zip(theta, kappas)))
        A = lop.assemble({"a": a})
        assert rel_err(A.csr()[2].cpu().numpy(), combined.csr()[2].cpu().numpy()) < 1e-13
        # the pattern is the terms' pattern, bit for bit
        for x, y in zip(A.csr()[:2], ops[0].csr()[:2]):
            assert torch.equal(x, y)


def test_lincomb_of_swipdg_terms_matches_oracle(gdt, oracle):
    n = [10, 8]
    g = gdt.make_cube_grid([0, 0], [1, 1], n, simplex=True)
    og = oracle.grid(2, n, 0.0, 1.0, simplex=True)
    space = gdt.DiscontinuousLagrangeSpace(g, 1)
    rng = np.random.default_rng(4)
    kappas = [np.exp(rng.standard_normal(g.num_elements)), rng.uniform(0.5, 2.0, g.num_elements)]
    ops, refs = [], []
    for k in kappas:
        kt = torch.tensor(k, device="cuda")
        op = gdt.MatrixOperator(g, space, stencil=gdt.Stencil.element_and_intersection)
        op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(kt))
        op += gdt.LocalCouplingIntersectionIntegralBilinearForm(
            gdt.LocalLaplaceIPDGInnerCoupling(1.0, kt, kt) + gdt.LocalIPDGInnerPenalty(8.0, kt))
        op += gdt.LocalIntersectionIntegralBilinearForm(
            gdt.LocalLaplaceIPDGDirichletCoupling(1.0, kt) + gdt.LocalIPDGBoundaryPenalty(14.0, kt))
        op.assemble()
        ops.append(op)
        A, _ = oracle.assemble_swipdg(og, 1, kappa=k, force=np.ones(g.num_elements), theta=1.0, sigma_inner=8.0,
                                      sigma_boundary=14.0, weight_is_diffusion=True)
        refs.append(A)
    theta = [1.7, 0.4]
    lop = gdt.LincombOperator(ops, theta)
    A = lop.assemble()
    ref = theta[0] * refs[0].val + theta[1] * refs[1].val
    assert rel_err(A.csr()[2].cpu().numpy(), ref) < 1e-12
    # parametric solve against a direct solve of the combined oracle matrix
    b = rng.standard_normal(space.num_DoFs)
    x = lop.apply_inverse(torch.tensor(b, device="cuda"), opts={"tol": 1e-13, "max_iter": 100000})
    Ar = refs[0].to_scipy() * theta[0] + refs[1].to_scipy() * theta[1]
    assert rel_err(x.cpu().numpy(), spl.spsolve(Ar.tocsc(), b)) < 1e-8


@pytest.mark.parametrize("n,nterms", [(1, 1), (7, 3), (1000, 2), (4097, 5), (100001, 8)])
def test_vector_lincomb(gdt, n, nterms):
    rng = np.random.default_rng(n)
    vs = [rng.standard_normal(n) for _ in range(nterms)]
    th = rng.standard_normal(nterms)
    out = gdt.lincomb([torch.tensor(v, device="cuda") for v in vs], th).cpu().numpy()
    ref = sum(t * v for t, v in zip(th, vs))
    assert np.abs(out - ref).max() <= 1e-14 * max(1.0, np.abs(ref).max()) * nterms
    # a misaligned view takes the scalar path
    big = torch.tensor(np.concatenate([[0.0], vs[0]]), device="cuda")
    out2 = gdt.lincomb([big[1:]], [2.0]).cpu().numpy()
    assert np.array_equal(out2, 2.0 * vs[0])


def test_lincomb_rejects_other_patterns(gdt):
    g = gdt.make_cube_grid([0, 0], [1, 1], [6, 6], simplex=True)
    g2 = gdt.make_cube_grid([0, 0], [1, 1], [6, 7], simplex=True)
    a = _cg_term(gdt, g, gdt.ContinuousLagrangeSpace(g, 1), np.ones(g.num_elements))
    b = _cg_term(gdt, g2, gdt.ContinuousLagrangeSpace(g2, 1), np.ones(g2.num_elements))
    with pytest.raises(gdt.GdtError) as e:
        gdt.LincombOperator([a, b], [1.0, 1.0]).assemble()
    assert e.value.status == gdt._capi.ESHAPE
