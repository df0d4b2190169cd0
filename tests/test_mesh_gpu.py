"""Unstructured simplex meshes (gdt_grid_create_simplex_mesh) on the GPU against the oracle: the pattern
bit-exact, stiffness, load vector and Dirichlet constraints within 1e-12 on Delaunay meshes of 2D and 3D
boxes; the Kuhn split of a cube grid handed over as a mesh gives the structured path's system; solves,
Dirichlet values, the log-kappa gradient, SWIPDG (DG P1) on triangle meshes, and the forms a mesh does
not lower."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl
import torch

from conftest import csr_equal_pattern, rel_err

pytestmark = pytest.mark.gpu
spatial = pytest.importorskip("scipy.spatial")


def delaunay_mesh(dim, n, seed):
    """Delaunay simplices of a jittered lattice of (n + 1)^dim points in the unit box."""
    rng = np.random.default_rng(seed)
    t = np.linspace(0.0, 1.0, n + 1)
    X = np.stack(np.meshgrid(*([t] * dim), indexing="ij"), -1).reshape(-1, dim)
    inner = np.all((X > 0) & (X < 1), axis=1)
    X[inner] += (0.3 / n) * rng.uniform(-1, 1, (inner.sum(), dim))
    cells = spatial.Delaunay(X).simplices.astype(np.int64)
    J = np.stack([X[cells[:, k + 1]] - X[cells[:, 0]] for k in range(dim)], axis=-1)
    vol = np.abs(np.linalg.det(J))
    return X, cells[vol > 1e-9 * vol.max()]


MESHES = [(2, 14, 3), (2, 25, 4), (3, 5, 5), (3, 7, 6)]


def _assemble(gdt, mesh, kappa, force, dirichlet, values=None):
    space = gdt.ContinuousLagrangeSpace(mesh, 1)
    op = gdt.MatrixOperator(mesh, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(kappa))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=force, dirichlet=dirichlet, dirichlet_values=values)
    return space, op, rhs


@pytest.mark.parametrize("dim,n,seed", MESHES)
@pytest.mark.parametrize("dirichlet", [True, False])
def test_mesh_assembly_matches_oracle(gdt, oracle, dim, n, seed, dirichlet):
    X, cells = delaunay_mesh(dim, n, seed)
    mesh = gdt.make_simplex_mesh(X, torch.tensor(cells, device="cuda"))
    ne = cells.shape[0]
    rng = np.random.default_rng(seed)
    kappa, force = np.exp(rng.standard_normal(ne)), rng.uniform(-1, 2, ne)
    A, b = oracle.mesh_assemble(X, cells, kappa=kappa, force=force, dirichlet=dirichlet)
    space, op, rhs = _assemble(gdt, mesh, torch.tensor(kappa, device="cuda"), torch.tensor(force, device="cuda"),
                               dirichlet)
    assert space.num_DoFs == X.shape[0] and mesh.num_elements == ne
    rp, col, val = op.csr()
    assert csr_equal_pattern((rp, col, val), A)
    assert rel_err(val.cpu().numpy(), A.val) < 1e-12
    assert rel_err(rhs.cpu().numpy(), b) < 1e-12
    # the DoF map is the element vertex lists, and the load vector alone matches the fused one
    assert np.array_equal(space.global_indices().cpu().numpy().reshape(ne, dim + 1), cells)
    fn = gdt.VectorFunctional(mesh, space)
    fn.append(gdt.LocalElementIntegralFunctional(gdt.LocalElementProductIntegrand().with_ansatz(
        torch.tensor(force, device="cuda"))))
    fn.assemble()
    _, b0 = oracle.mesh_assemble(X, cells, kappa=kappa, force=force, dirichlet=False)
    assert rel_err(fn.vector.cpu().numpy(), b0) < 1e-12
    if dirichlet:
        xd = spl.spsolve(A.to_scipy().tocsc(), b)
        for precision in ("fp64", "mixed"):
            u = op.apply_inverse(rhs, opts={"tol": 1e-12, "precision": precision})
            assert op.last_solve_info["converged"]
            assert rel_err(u.cpu().numpy(), xd) < 1e-9, precision


@pytest.mark.parametrize("dim,n", [(2, [9, 7]), (3, [4, 5, 3])])
def test_kuhn_grid_as_mesh_equals_structured_path(gdt, dim, n):
    # the structured Kuhn grid exported as coordinates and element vertex lists: same system
    g = gdt.make_cube_grid([0.0] * dim, [1.0] * dim, n, simplex=True)
    sg = gdt.ContinuousLagrangeSpace(g, 1)
    cells = sg.global_indices().reshape(g.num_elements, dim + 1)
    grids = np.meshgrid(*[np.linspace(0.0, 1.0, k + 1) for k in n], indexing="ij")
    X = np.stack([gr.transpose(*reversed(range(dim))).reshape(-1) for gr in grids], axis=1)
    mesh = gdt.make_simplex_mesh(torch.tensor(X, device="cuda"), cells)
    kappa = torch.exp(torch.tensor(np.random.default_rng(2).standard_normal(g.num_elements), device="cuda"))
    out = []
    for grid in (g, mesh):
        _, op, rhs = _assemble(gdt, grid, kappa, 1.0, True)
        out.append([t.cpu().numpy() for t in op.csr()] + [rhs.cpu().numpy()])
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert rel_err(out[1][2], out[0][2]) < 1e-13
    assert rel_err(out[1][3], out[0][3]) < 1e-13


@pytest.mark.parametrize("dim,n,seed", [(2, 12, 8), (3, 5, 9)])
def test_mesh_dirichlet_values_match_lifted_oracle(gdt, oracle, dim, n, seed):
    X, cells = delaunay_mesh(dim, n, seed)
    mesh = gdt.make_simplex_mesh(X, cells)
    A, b = oracle.mesh_assemble(X, cells, force_const=1.0, dirichlet=False)
    gd = np.sin(3 * X[:, 0]) + X[:, 1] ** 2
    mask = np.zeros(X.shape[0], bool)
    mask[oracle.mesh_boundary(X.shape[0], cells)] = True
    S = A.to_scipy().tocsr()
    bb = b - S @ np.where(mask, gd, 0.0)
    bb[mask] = gd[mask]
    keep = sp.diags((~mask).astype(float))
    S = (keep @ S @ keep + sp.diags(mask.astype(float))).tocsr()
    fn = gdt.GridFunction(lambda x: torch.sin(3 * x[:, 0]) + x[:, 1] ** 2)
    for fused in (True, False):
        if fused:
            space, op, rhs = _assemble(gdt, mesh, 1.0, 1.0, True, values=fn)
        else:
            space, op, rhs = _assemble(gdt, mesh, 1.0, 1.0, False)
            gdt.DirichletConstraints("dirichlet", space).apply(op, rhs, values=torch.tensor(gd, device="cuda"))
        rp, col, val = (t.cpu().numpy() for t in op.csr())
        G = sp.csr_matrix((val, col, rp), shape=S.shape)
        assert abs(G - S).max() <= 1e-12 * abs(S).max()
        assert rel_err(rhs.cpu().numpy(), bb) < 1e-12
    u = op.apply_inverse(rhs, opts={"tol": 1e-12})
    assert rel_err(u.cpu().numpy(), spl.spsolve(S.tocsc(), bb)) < 1e-10


@pytest.mark.parametrize("dim,n,seed", [(2, 10, 12), (3, 4, 13)])
def test_mesh_log_kappa_gradient(gdt, oracle, dim, n, seed):
    # -kappa_e lam_e^T K_e u_e with the boundary rows and columns excluded, against a numpy restatement
    X, cells = delaunay_mesh(dim, n, seed)
    mesh = gdt.make_simplex_mesh(X, cells)
    space = gdt.ContinuousLagrangeSpace(mesh, 1)
    rng = np.random.default_rng(seed)
    ne, nv = cells.shape[0], X.shape[0]
    kappa, u, lam = np.exp(rng.standard_normal(ne)), rng.standard_normal(nv), rng.standard_normal(nv)
    lib = gdt._capi.load()
    out = torch.zeros(ne, dtype=torch.float64, device="cuda")
    kt, ut, lt = (torch.tensor(a, device="cuda") for a in (kappa, u, lam))
    gdt._capi.check(lib.gdt_cg_dlogkappa(gdt.default_context().handle, space.handle, kt.data_ptr(), ut.data_ptr(),
                                         lt.data_ptr(), out.data_ptr()), what="gdt_cg_dlogkappa")
    bnd = np.zeros(nv, bool)
    bnd[oracle.mesh_boundary(nv, cells)] = True
    uz, lz = np.where(bnd, 0.0, u), np.where(bnd, 0.0, lam)
    ref = np.empty(ne)
    for e in range(ne):
        w = cells[e]
        J = np.stack([X[w[k + 1]] - X[w[0]] for k in range(dim)], axis=1)
        Gr = np.vstack([-np.ones(dim), np.eye(dim)]) @ np.linalg.inv(J)  # rows: gradients of the P1 basis
        K = abs(np.linalg.det(J)) / (2.0 if dim == 2 else 6.0) * Gr @ Gr.T
        ref[e] = -kappa[e] * lz[w] @ K @ uz[w]
    assert rel_err(out.cpu().numpy(), ref) < 1e-12


def test_mesh_refusals(gdt):
    X, cells = delaunay_mesh(2, 6, 1)
    mesh = gdt.make_simplex_mesh(X, cells)
    X3, cells3 = delaunay_mesh(3, 3, 1)
    mesh3 = gdt.make_simplex_mesh(X3, cells3)
    for make in (lambda: gdt.DiscontinuousLagrangeSpace(mesh3, 1), lambda: gdt.ContinuousLagrangeSpace(mesh, 2)):
        with pytest.raises(gdt.GdtError) as e:
            make()
        assert e.value.status == gdt._capi.EUNSUPPORTED
    lib = gdt._capi.load()
    assert lib.gdt_grid_set_vertices(mesh.handle, X.ctypes.data) == gdt._capi.EUNSUPPORTED
    bad = [cells.copy(), cells.copy(), cells.copy()]
    bad[0][3, 1] = X.shape[0]          # vertex index out of range
    bad[1][2, 2] = bad[1][2, 0]        # repeated vertex
    Xf = X.copy()
    Xf[cells[0, 2]] = 0.5 * (Xf[cells[0, 0]] + Xf[cells[0, 1]])  # a flat triangle
    Xextra = np.vstack([X, [[2.0, 2.0]]])  # a vertex of no element
    for Xi, ci in ((X, bad[0]), (X, bad[1]), (Xf, cells), (Xextra, cells)):
        with pytest.raises(gdt.GdtError) as e:
            gdt.make_simplex_mesh(Xi, ci)
        assert e.value.status == gdt._capi.EINVAL
    space = gdt.ContinuousLagrangeSpace(mesh, 1)
    op = gdt.MatrixOperator(mesh, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalElementProductIntegrand())
    with pytest.raises(gdt.GdtError) as e:
        op.assemble()
    assert e.value.status == gdt._capi.EUNSUPPORTED


def _swipdg(gdt, grid, kappa, force, theta=1.0, dirichlet=None):
    space = gdt.DiscontinuousLagrangeSpace(grid, 1)
    op = gdt.MatrixOperator(grid, space, stencil=gdt.Stencil.element_and_intersection)
    kt = torch.tensor(kappa, device="cuda")
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(kt))
    op += gdt.LocalCouplingIntersectionIntegralBilinearForm(
        gdt.LocalLaplaceIPDGInnerCoupling(theta, kt, kt) + gdt.LocalIPDGInnerPenalty(8.0, kt))
    coupling = gdt.LocalLaplaceIPDGDirichletCoupling(theta, kt, 0.0 if dirichlet is None else dirichlet)
    penalty = gdt.LocalIPDGBoundaryPenalty(14.0, kt, dirichlet_data=dirichlet)
    op += gdt.LocalIntersectionIntegralBilinearForm(coupling + penalty)
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=torch.tensor(force, device="cuda"))
    return space, op, rhs


@pytest.mark.parametrize("n,seed", [(10, 31), (24, 32)])
@pytest.mark.parametrize("theta", [1.0, -1.0, 0.0])
def test_mesh_swipdg_matches_oracle(gdt, oracle, n, seed, theta):
    X, cells = delaunay_mesh(2, n, seed)
    mesh = gdt.make_simplex_mesh(X, cells)
    rng = np.random.default_rng(seed)
    ne = cells.shape[0]
    kappa, force = np.exp(rng.standard_normal(ne)), rng.uniform(0.5, 1.5, ne)
    space, op, rhs = _swipdg(gdt, mesh, kappa, force, theta)
    A, b = oracle.mesh_assemble_swipdg(X, cells, kappa=kappa, force=force, theta=theta)
    rp, col, val = op.csr()
    assert csr_equal_pattern((rp, col, val), A)
    assert rel_err(val.cpu().numpy(), A.val) < 1e-12
    assert rel_err(rhs.cpu().numpy(), b) < 1e-12
    if theta == 1.0:
        u = op.apply_inverse(rhs, opts={"tol": 1e-13, "max_iter": 200000})
        assert rel_err(u.cpu().numpy(), spl.spsolve(A.to_scipy().tocsc(), b)) < 1e-9


def test_mesh_swipdg_dirichlet_data_matches_oracle(gdt, oracle):
    # Dirichlet data g = cos(pi x / 2) cos(pi y / 2) + 0.3 x at the face points of the mesh's faces: both
    # right-hand side terms (unary DirichletCoupling and the penalty's counterpart)
    X, cells = delaunay_mesh(2, 12, 33)
    mesh = gdt.make_simplex_mesh(X, cells)
    rng = np.random.default_rng(33)
    ne = cells.shape[0]
    kappa, force = np.exp(rng.standard_normal(ne)), rng.uniform(0.5, 1.5, ne)
    g = gdt.GridFunction(lambda x: torch.cos(np.pi / 2 * x[..., 0]) * torch.cos(np.pi / 2 * x[..., 1]) + 0.3 * x[..., 0])
    space, op, rhs = _swipdg(gdt, mesh, kappa, force, 1.0, dirichlet=g)
    A, b = oracle.mesh_assemble_swipdg(X, cells, kappa=kappa, force=force, dirichlet_fn=oracle.DIRICHLET_TEST,
                                       dirichlet_rhs=3)
    assert rel_err(op.csr()[2].cpu().numpy(), A.val) < 1e-12
    assert rel_err(rhs.cpu().numpy(), b) < 1e-12


def test_kuhn_grid_as_mesh_swipdg_equals_structured_path(gdt):
    n = [9, 7]
    g = gdt.make_cube_grid([0.0, 0.0], [1.0, 1.0], n, simplex=True)
    cells = gdt.ContinuousLagrangeSpace(g, 1).global_indices()
    t = [np.linspace(0.0, 1.0, k + 1) for k in n]
    X = np.stack(np.meshgrid(*t, indexing="ij"), -1).transpose(1, 0, 2).reshape(-1, 2)
    mesh = gdt.make_simplex_mesh(X, cells)
    rng = np.random.default_rng(5)
    kappa, force = np.exp(rng.standard_normal(g.num_elements)), rng.uniform(0.5, 1.5, g.num_elements)
    out = []
    for grid in (g, mesh):
        _, op, rhs = _swipdg(gdt, grid, kappa, force)
        out.append([t.cpu().numpy() for t in op.csr()] + [rhs.cpu().numpy()])
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert rel_err(out[1][2], out[0][2]) < 1e-13
    assert rel_err(out[1][3], out[0][3]) < 1e-13


@pytest.mark.parametrize("dim,n,kind", [(2, 9, "cg"), (3, 4, "cg"), (2, 8, "dg")])
@pytest.mark.parametrize("norm", ["h1_semi", "l2"])
def test_mesh_element_error_matches_numpy(gdt, dim, n, kind, norm):
    # the EOC studies' element indicators on a mesh against a numpy restatement at the same points
    X, cells = delaunay_mesh(dim, n, 51)
    mesh = gdt.make_simplex_mesh(X, cells)
    space = gdt.ContinuousLagrangeSpace(mesh, 1) if kind == "cg" else gdt.DiscontinuousLagrangeSpace(mesh, 1)
    rng = np.random.default_rng(51)
    u = rng.standard_normal(space.num_DoFs)
    order = 4
    xq = space.quadrature_points(order)  # [element, q, dim]
    xr, wr = space.quadrature(order)
    if norm == "h1_semi":
        ref = torch.stack([torch.cos(3 * xq[..., a]) for a in range(dim)], -1)
    else:
        ref = torch.sin(2 * xq[..., 0]) + xq[..., 1]
    eta2, total = gdt.element_error(space, torch.tensor(u, device="cuda"), ref.contiguous(), norm=norm,
                                    quad_order=order)
    refn = ref.cpu().numpy()
    exp = np.empty(cells.shape[0])
    for e in range(cells.shape[0]):
        w = cells[e]
        J = np.stack([X[w[k + 1]] - X[w[0]] for k in range(dim)], axis=1)
        Gr = np.vstack([-np.ones(dim), np.eye(dim)]) @ np.linalg.inv(J)
        ue = u[w] if kind == "cg" else u[(dim + 1) * e:(dim + 1) * (e + 1)]
        wq = wr * abs(np.linalg.det(J))
        if norm == "h1_semi":
            d = (ue @ Gr)[None, :] - refn[e]
            exp[e] = wq @ (d * d).sum(1)
        else:
            phi = np.hstack([1.0 - xr[:, :dim].sum(1, keepdims=True), xr[:, :dim]])
            d = phi @ ue - refn[e]
            exp[e] = wq @ (d * d)
    assert rel_err(eta2.cpu().numpy(), exp) < 1e-12
    assert abs(total - np.sqrt(exp.sum())) <= 1e-12 * np.sqrt(exp.sum())
