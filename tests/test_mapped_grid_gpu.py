"""Mapped structured grids (gdt_grid_set_vertices): the topology and numbering of make_cube_grid with
every vertex moved, each element's geometry formed from its own vertices. Continuous P1 (Kuhn
simplices) and Q1 (cubes) Laplace stiffness and load vector against the oracle on the same mapped
vertices (pattern bit-exact, values 1e-12), solves against a direct solve, and the forms that a mapped
grid does not lower."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl
import torch

from conftest import csr_equal_pattern, rel_err

pytestmark = pytest.mark.gpu


def vertices(n, kind):
    """Vertex coordinates [vertex, dim] (x fastest) of the unit square / cube under a smooth map."""
    dim = len(n)
    axes = [np.linspace(0.0, 1.0, k + 1) for k in n]
    grids = np.meshgrid(*axes, indexing="ij")  # grids[a][i0, i1, ...]
    X = [gr.transpose(*reversed(range(dim))).reshape(-1) for gr in grids]  # lexicographic, x fastest
    X = np.stack(X, axis=1)
    if kind == "identity":
        return X
    Y = X.copy()
    if kind == "graded":  # x -> (x + x^2) / 2 in every direction
        return 0.5 * (X + X * X)
    # "wavy": interior and tangential boundary motion, Jacobian positive for the amplitude below
    for a in range(dim):
        b = (a + 1) % dim
        Y[:, a] = X[:, a] + 0.04 * np.sin(2 * np.pi * X[:, a]) * (1.0 + X[:, b])
    return Y


CASES = [((12, 10), False), ((12, 10), True), ((6, 5, 7), False), ((6, 5, 7), True)]


@pytest.mark.parametrize("n,simplex", CASES)
@pytest.mark.parametrize("kind", ["wavy", "graded"])
def test_mapped_assembly_matches_oracle(gdt, oracle, n, simplex, kind):
    dim = len(n)
    xv = vertices(n, kind)
    g = gdt.make_cube_grid([0.0] * dim, [1.0] * dim, list(n), simplex=simplex).map_vertices(xv)
    og = oracle.grid(dim, list(n), 0.0, 1.0, simplex=simplex, vertices=xv)
    rng = np.random.default_rng(7 + dim + int(simplex))
    ne = g.num_elements
    kappa = np.exp(rng.standard_normal(ne))
    force = rng.uniform(-1, 2, ne)
    A, b = oracle.assemble_cg(og, 1, kappa=kappa, force=force, dirichlet=True)
    space = gdt.ContinuousLagrangeSpace(g, 1)
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(torch.tensor(kappa, device="cuda")))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=torch.tensor(force, device="cuda"), dirichlet=True)
    rp, col, val = op.csr()
    assert csr_equal_pattern((rp, col, val), A)
    assert rel_err(val.cpu().numpy(), A.val) < 1e-12
    assert rel_err(rhs.cpu().numpy(), b) < 1e-12
    # the solves on the mapped system, FP64 and mixed precision
    xd = spl.spsolve(A.to_scipy().tocsc(), b)
    for precision in ("fp64", "mixed"):
        u = op.apply_inverse(rhs, opts={"tol": 1e-12, "precision": precision})
        assert rel_err(u.cpu().numpy(), xd) < 1e-9, precision


@pytest.mark.parametrize("n,simplex", CASES)
def test_identity_map_equals_equidistant_grid(gdt, n, simplex):
    dim = len(n)
    out = []
    for mapped in (False, True):
        g = gdt.make_cube_grid([0.0] * dim, [1.0] * dim, list(n), simplex=simplex)
        if mapped:
            g.map_vertices(torch.tensor(vertices(n, "identity"), device="cuda"))  # device coordinates
        space = gdt.ContinuousLagrangeSpace(g, 1)
        op = gdt.MatrixOperator(g, space)
        op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(1.0))
        rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
        op.assemble(rhs=rhs, force=1.0, dirichlet=True)
        out.append((op.csr()[2].cpu().numpy(), rhs.cpu().numpy()))
    assert rel_err(out[1][0], out[0][0]) < 1e-13
    assert rel_err(out[1][1], out[0][1]) < 1e-13


@pytest.mark.parametrize("n,simplex", [((10, 9), False), ((5, 4, 6), True)])
def test_mapped_dirichlet_values_match_lifted_oracle(gdt, oracle, n, simplex):
    """Boundary values given as a GridFunction are evaluated at the mapped vertices; the constrained
    system equals the oracle's unconstrained one lifted by those values (b -= A[:, D] g_D, unit rows and
    columns, b_D = g_D)."""
    import scipy.sparse as sp

    dim = len(n)
    xv = vertices(n, "wavy")
    g = gdt.make_cube_grid([0.0] * dim, [1.0] * dim, list(n), simplex=simplex).map_vertices(xv)
    og = oracle.grid(dim, list(n), 0.0, 1.0, simplex=simplex, vertices=xv)
    A, b = oracle.assemble_cg(og, 1, force_const=1.0, dirichlet=False)
    gd = np.sin(3 * xv[:, 0]) + xv[:, 1] ** 2
    dofs = oracle.dirichlet_dofs(og, 1)
    mask = np.zeros(len(b), bool)
    mask[dofs] = True
    S = A.to_scipy().tocsr()
    bb = b - S @ np.where(mask, gd, 0.0)
    bb[mask] = gd[mask]
    keep = sp.diags((~mask).astype(float))
    S = (keep @ S @ keep + sp.diags(mask.astype(float))).tocsr()
    space = gdt.ContinuousLagrangeSpace(g, 1)
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(1.0))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    fn = gdt.GridFunction(lambda x: torch.sin(3 * x[:, 0]) + x[:, 1] ** 2)
    op.assemble(rhs=rhs, force=1.0, dirichlet=True, dirichlet_values=fn)
    rp, col, val = (t.cpu().numpy() for t in op.csr())
    G = sp.csr_matrix((val, col, rp), shape=S.shape)
    assert abs(G - S).max() <= 1e-12 * abs(S).max()
    assert rel_err(rhs.cpu().numpy(), bb) < 1e-12
    u = op.apply_inverse(rhs, opts={"tol": 1e-12})
    assert rel_err(u.cpu().numpy(), spl.spsolve(S.tocsc(), bb)) < 1e-10


def test_mapped_grid_refuses_other_forms(gdt):
    n = (6, 6)
    g = gdt.make_cube_grid([0.0, 0.0], [1.0, 1.0], list(n), simplex=True).map_vertices(vertices(n, "wavy"))
    with pytest.raises(gdt.GdtError) as e:
        gdt.DiscontinuousLagrangeSpace(g, 1)
    assert e.value.status == gdt._capi.EUNSUPPORTED
    with pytest.raises(gdt.GdtError) as e:
        gdt.ContinuousLagrangeSpace(g, 2)
    assert e.value.status == gdt._capi.EUNSUPPORTED
    with pytest.raises(ValueError):
        gdt.make_cube_grid([0.0, 0.0], [1.0, 1.0], list(n)).map_vertices(np.zeros((5, 2)))
