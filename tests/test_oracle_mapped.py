"""CPU checks of the oracle's mapped structured grids (per-element geometry from the vertex coordinates),
which pin the mapped restatement to the equidistant one that the reference's known answers pin:
an axis-aligned affine map equals the equidistant grid on the mapped box, linear functions of the
mapped coordinates pass the patch test, and the load vector of a unit source integrates the area."""
import numpy as np
import pytest

CASES = [(2, [6, 5], False), (2, [6, 5], True), (3, [3, 4, 2], False), (3, [3, 2, 4], True)]


def lattice(n):
    dim = len(n)
    grids = np.meshgrid(*[np.linspace(0.0, 1.0, k + 1) for k in n], indexing="ij")
    return np.stack([gr.transpose(*reversed(range(dim))).reshape(-1) for gr in grids], axis=1)


def wavy(X):
    Y = X.copy()
    dim = X.shape[1]
    for a in range(dim):
        Y[:, a] = X[:, a] + 0.04 * np.sin(2 * np.pi * X[:, a]) * (1.0 + X[:, (a + 1) % dim])
    return Y


@pytest.mark.parametrize("dim,n,simplex", CASES)
def test_affine_map_equals_equidistant_box(oracle, dim, n, simplex):
    lo, hi = np.array([-1.0, 0.5, 2.0][:dim]), np.array([1.5, 1.25, 2.5][:dim])
    xv = lo + (hi - lo) * lattice(n)
    og_m = oracle.grid(dim, n, 0.0, 1.0, simplex=simplex, vertices=xv)
    og_e = oracle.grid(dim, n, list(lo), list(hi), simplex=simplex)
    rng = np.random.default_rng(3)
    ne = oracle.num_elements(og_e)
    kappa, force = np.exp(rng.standard_normal(ne)), rng.uniform(-1, 1, ne)
    Am, bm = oracle.assemble_cg(og_m, 1, kappa=kappa, force=force, dirichlet=True)
    Ae, be = oracle.assemble_cg(og_e, 1, kappa=kappa, force=force, dirichlet=True)
    assert np.array_equal(Am.col, Ae.col)
    assert np.abs(Am.val - Ae.val).max() <= 1e-13 * np.abs(Ae.val).max()
    assert np.abs(bm - be).max() <= 1e-13 * np.abs(be).max()


@pytest.mark.parametrize("dim,n,simplex", CASES)
def test_patch_test_on_wavy_map(oracle, dim, n, simplex):
    # P1 (exact) and Q1 (isoparametric, tensor Gauss rule of two points) reproduce linear functions:
    # the stiffness matrix maps u = c0 + c . x to zero on every interior row
    xv = wavy(lattice(n))
    og = oracle.grid(dim, n, 0.0, 1.0, simplex=simplex, vertices=xv)
    A, _ = oracle.assemble_cg(og, 1, dirichlet=False)
    S = A.to_scipy().tocsr()
    u = 0.7 + xv @ np.array([1.0, -2.0, 0.5][:dim])
    r = S @ u
    interior = np.ones(len(u), bool)
    interior[oracle.dirichlet_dofs(og, 1)] = False
    assert interior.any()
    assert np.abs(r[interior]).max() <= 1e-12 * abs(S).max() * np.abs(u).max()
    assert np.abs(S @ np.ones(len(u))).max() <= 1e-12 * abs(S).max()
    assert abs(S - S.T).max() <= 1e-14 * abs(S).max()


@pytest.mark.parametrize("dim,n,simplex", [c for c in CASES if c[0] == 2 or c[2]])
def test_unit_source_integrates_mapped_area(oracle, dim, n, simplex):
    # the wavy map keeps the unit box; the midpoint rule is exact for the area of bilinear quadrilaterals
    # and of simplices, and the basis is a partition of unity
    og = oracle.grid(dim, n, 0.0, 1.0, simplex=simplex, vertices=wavy(lattice(n)))
    _, b = oracle.assemble_cg(og, 1, force_const=1.0, dirichlet=False)
    assert abs(b.sum() - 1.0) <= 1e-13
