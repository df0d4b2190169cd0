"""CPU checks of the oracle's unstructured simplex meshes, pinning the mesh restatement to the structured
one that the reference's known answers pin: the Kuhn split of a cube grid handed over as a mesh gives
the same pattern, matrix, load vector and boundary; on Delaunay meshes, linear functions pass the patch
test and a unit source integrates the area."""
import numpy as np
import pytest

spatial = pytest.importorskip("scipy.spatial")


def kuhn_mesh(oracle, dim, n):
    """The Kuhn simplex grid of the unit box as (oracle grid, coords, cells)."""
    og = oracle.grid(dim, n, 0.0, 1.0, simplex=True)
    ne = oracle.num_elements(og)
    cells = oracle.global_indices(og, oracle.CG, 1).reshape(ne, dim + 1)
    grids = np.meshgrid(*[np.linspace(0.0, 1.0, k + 1) for k in n], indexing="ij")
    coords = np.stack([gr.transpose(*reversed(range(dim))).reshape(-1) for gr in grids], axis=1)
    return og, coords, cells


def delaunay_mesh(dim, n, seed):
    """Delaunay simplices of a jittered lattice of (n + 1)^dim points in the unit box (corners kept)."""
    rng = np.random.default_rng(seed)
    t = np.linspace(0.0, 1.0, n + 1)
    X = np.stack(np.meshgrid(*([t] * dim), indexing="ij"), -1).reshape(-1, dim)
    inner = np.all((X > 0) & (X < 1), axis=1)
    X[inner] += (0.3 / n) * rng.uniform(-1, 1, (inner.sum(), dim))
    cells = spatial.Delaunay(X).simplices.astype(np.int64)
    # the flat simplices Delaunay leaves on the box faces (coplanar boundary points) have no volume
    J = np.stack([X[cells[:, k + 1]] - X[cells[:, 0]] for k in range(dim)], axis=-1)
    vol = np.abs(np.linalg.det(J))
    return X, cells[vol > 1e-9 * vol.max()]


@pytest.mark.parametrize("dim,n", [(2, [6, 5]), (3, [3, 4, 2])])
def test_kuhn_grid_as_mesh_equals_structured(oracle, dim, n):
    og, coords, cells = kuhn_mesh(oracle, dim, n)
    rng = np.random.default_rng(4)
    ne = cells.shape[0]
    kappa, force = np.exp(rng.standard_normal(ne)), rng.uniform(-1, 2, ne)
    for dirichlet in (False, True):
        A, b = oracle.assemble_cg(og, 1, kappa=kappa, force=force, dirichlet=dirichlet)
        M, bm = oracle.mesh_assemble(coords, cells, kappa=kappa, force=force, dirichlet=dirichlet)
        assert np.array_equal(M.row_ptr, A.row_ptr) and np.array_equal(M.col, A.col)
        assert np.abs(M.val - A.val).max() <= 1e-14 * np.abs(A.val).max()
        assert np.abs(bm - b).max() <= 1e-14 * np.abs(b).max()
    assert np.array_equal(oracle.mesh_boundary(coords.shape[0], cells), oracle.dirichlet_dofs(og, 1))


@pytest.mark.parametrize("dim,n", [(2, 9), (3, 4)])
def test_delaunay_mesh_patch_test_and_area(oracle, dim, n):
    X, cells = delaunay_mesh(dim, n, 11)
    A, b = oracle.mesh_assemble(X, cells, force_const=1.0, dirichlet=False)
    S = A.to_scipy().tocsr()
    assert abs(S - S.T).max() <= 1e-14 * abs(S).max()
    u = 0.3 + X @ np.array([1.0, -0.5, 2.0][:dim])
    r = S @ u
    inner = np.ones(X.shape[0], bool)
    inner[oracle.mesh_boundary(X.shape[0], cells)] = False
    assert inner.any()
    assert np.abs(r[inner]).max() <= 1e-12 * abs(S).max() * np.abs(u).max()
    assert abs(b.sum() - 1.0) <= 1e-13


@pytest.mark.parametrize("n", [[5, 4], [7, 7]])
@pytest.mark.parametrize("theta,rhs_terms", [(1.0, 0), (1.0, 3), (-1.0, 1)])
def test_kuhn_grid_as_mesh_swipdg_equals_structured(oracle, n, theta, rhs_terms):
    # SWIPDG on the Kuhn triangles handed over as a mesh: the structured restatement's system
    og, coords, cells = kuhn_mesh(oracle, 2, n)
    rng = np.random.default_rng(9)
    ne = cells.shape[0]
    kappa, force = np.exp(rng.standard_normal(ne)), rng.uniform(-1, 2, ne)
    kw = dict(kappa=kappa, force=force, theta=theta, sigma_inner=8.0, sigma_boundary=14.0, beta=1.0,
              dirichlet_fn=oracle.DIRICHLET_TEST, dirichlet_rhs=rhs_terms)
    A, b = oracle.assemble_swipdg(og, 1, **kw)
    M, bm = oracle.mesh_assemble_swipdg(coords, cells, **kw)
    assert np.array_equal(M.row_ptr, A.row_ptr) and np.array_equal(M.col, A.col)
    assert np.abs(M.val - A.val).max() <= 1e-13 * np.abs(A.val).max()
    assert np.abs(bm - b).max() <= 1e-13 * np.abs(b).max()


@pytest.mark.parametrize("dim,n", [(2, 8), (3, 4)])
def test_mesh_boundary_is_the_convex_hull(oracle, dim, n):
    # on a Delaunay mesh of points in a box, the faces of one element are the convex hull's facets
    X, cells = delaunay_mesh(dim, n, 17)
    hull = spatial.ConvexHull(X)
    on_box = np.any((X <= 1e-12) | (X >= 1 - 1e-12), axis=1)
    bnd = oracle.mesh_boundary(X.shape[0], cells)
    assert np.array_equal(np.sort(bnd), np.flatnonzero(on_box))
    assert set(np.unique(hull.simplices)) <= set(bnd.tolist())


@pytest.mark.parametrize("n,theta", [(9, 1.0), (14, -1.0)])
def test_mesh_swipdg_reproduces_constants(oracle, n, theta):
    # SWIPDG is consistent: with f = 0 and Dirichlet data g = c on both right-hand side terms, the
    # discrete solution is u = c on every DoF, whatever the coefficient
    import scipy.sparse.linalg as spl

    X, cells = delaunay_mesh(2, n, 41)
    kappa = np.exp(np.random.default_rng(41).standard_normal(cells.shape[0]) * 2.0)
    A, b = oracle.mesh_assemble_swipdg(X, cells, kappa=kappa, force_const=0.0, theta=theta,
                                       dirichlet_const=0.7, dirichlet_rhs=3)
    u = spl.spsolve(A.to_scipy().tocsc(), b)
    assert np.abs(u - 0.7).max() <= 1e-10


@pytest.mark.parametrize("dim,n", [(2, 10), (3, 5)])
def test_mesh_p1_reproduces_linear_functions(oracle, dim, n):
    # P1 on a mesh with f = 0 and Dirichlet values of a linear function: the solution is that function
    import scipy.sparse.linalg as spl

    X, cells = delaunay_mesh(dim, n, 43)
    A, _ = oracle.mesh_assemble(X, cells, kappa=np.ones(cells.shape[0]), force_const=0.0, dirichlet=False)
    lin = 0.2 + X @ np.array([1.0, -0.7, 0.4][:dim])
    bnd = oracle.mesh_boundary(X.shape[0], cells)
    inner = np.setdiff1d(np.arange(X.shape[0]), bnd)
    S = A.to_scipy().tocsr()
    u = np.zeros(X.shape[0])
    u[bnd] = lin[bnd]
    rhs = -S[inner][:, bnd] @ lin[bnd]
    u[inner] = spl.spsolve(S[inner][:, inner].tocsc(), rhs)
    assert np.abs(u - lin).max() <= 1e-11
