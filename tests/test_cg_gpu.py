"""Continuous Lagrange path on the GPU against the CPU oracle: DoF numbering and sparsity pattern
bit-exact, stiffness/RHS/Dirichlet within 1e-12 relative, SpMV and Krylov solves."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl
import torch

from conftest import csr_equal_pattern, rel_err

pytestmark = pytest.mark.gpu

GRIDS = [
    (1, [7], False),
    (2, [5, 4], False),
    (2, [6, 3], True),
    (3, [4, 3, 5], False),
    (3, [3, 4, 2], True),
]


def _grid(gdt, oracle, dim, n, simplex, lo=None, hi=None):
    lo = lo or [0.0] * dim
    hi = hi or [1.0 + 0.5 * a for a in range(dim)]
    return gdt.make_cube_grid(lo, hi, n, simplex=simplex), oracle.grid(dim, n, lo, hi, simplex=simplex)


@pytest.mark.parametrize("dim,n,simplex", GRIDS)
def test_global_indices_bit_exact(gdt, oracle, dim, n, simplex):
    g, og = _grid(gdt, oracle, dim, n, simplex)
    for kind, cls in ((oracle.CG, gdt.ContinuousLagrangeSpace), (oracle.DG, gdt.DiscontinuousLagrangeSpace)):
        if kind == oracle.DG and simplex and dim == 3:
            continue
        sp = cls(g, 1)
        assert sp.num_DoFs == oracle.space_size(og, kind, 1)
        gi = sp.global_indices().cpu().numpy()
        assert np.array_equal(gi, oracle.global_indices(og, kind, 1))


@pytest.mark.parametrize("dim,n,simplex", GRIDS)
def test_pattern_bit_exact(gdt, oracle, dim, n, simplex):
    g, og = _grid(gdt, oracle, dim, n, simplex)
    op = gdt.MatrixOperator(g, gdt.ContinuousLagrangeSpace(g, 1))
    ref = oracle.pattern(og, oracle.CG, 1, oracle.STENCIL_ELEMENT)
    assert op.nnz == ref.nnz
    assert csr_equal_pattern(op.csr(), ref)


@pytest.mark.parametrize("dim,n,simplex", [(2, [5, 4], True), (2, [4, 6], False)])
def test_dg_pattern_bit_exact(gdt, oracle, dim, n, simplex):
    g, og = _grid(gdt, oracle, dim, n, simplex)
    sp = gdt.DiscontinuousLagrangeSpace(g, 1)
    for st, ost in ((gdt.Stencil.element_and_intersection, oracle.STENCIL_ELEMENT_AND_INTERSECTION),
                    (gdt.Stencil.intersection, oracle.STENCIL_INTERSECTION),
                    (gdt.Stencil.element, oracle.STENCIL_ELEMENT)):
        op = gdt.MatrixOperator(g, sp, stencil=st)
        ref = oracle.pattern(og, oracle.DG, 1, ost)
        assert csr_equal_pattern(op.csr(), ref)


@pytest.mark.parametrize("dim,n,simplex", GRIDS)
@pytest.mark.parametrize("dirichlet", [True, False])
def test_assembly_matches_oracle(gdt, oracle, dim, n, simplex, dirichlet):
    g, og = _grid(gdt, oracle, dim, n, simplex)
    rng = np.random.default_rng(11 + dim)
    ne = g.num_elements
    kappa = np.exp(rng.standard_normal(ne))
    force = rng.uniform(-1, 2, ne)
    A, b = oracle.assemble_cg(og, 1, kappa=kappa, force=force, dirichlet=dirichlet)
    space = gdt.ContinuousLagrangeSpace(g, 1)
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(torch.tensor(kappa, device="cuda")))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=torch.tensor(force, device="cuda"), dirichlet=dirichlet)
    rp, col, val = op.csr()
    assert csr_equal_pattern((rp, col, val), A)
    assert rel_err(val.cpu().numpy(), A.val) < 1e-12
    assert rel_err(rhs.cpu().numpy(), b) < 1e-12


def test_walker_fused_equals_separate_dirichlet(gdt, oracle):
    # the reference example's walker (examples/stationary-heat-equation.cc:94-110) vs separate passes
    g = gdt.make_cube_grid([-1, -1], [1, 1], [16, 16])
    space = gdt.ContinuousLagrangeSpace(g, 1)
    ops = []
    for fused in (True, False):
        lhs = gdt.MatrixOperator(g, space)
        lhs.append(gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(1.0)))
        rhs = gdt.VectorFunctional(g, space)
        rhs.append(gdt.LocalElementIntegralFunctional(gdt.LocalElementProductIntegrand().with_ansatz(1.0)))
        dc = gdt.DirichletConstraints("all_dirichlet", space)
        if fused:
            w = gdt.Walker(g)
            w.append(lhs).append(rhs).append(dc)
            w.walk(thread_parallel=True)
        else:
            lhs.assemble()
            rhs.assemble()
        dc.apply(lhs, rhs.vector)
        ops.append((lhs.csr()[2].cpu().numpy().copy(), rhs.vector.cpu().numpy().copy()))
    og = oracle.grid(2, [16, 16], [-1, -1], [1, 1])
    A, b = oracle.assemble_cg(og, 1)
    for val, vec in ops:
        assert rel_err(val, A.val) < 1e-12
        assert rel_err(vec, b) < 1e-12


@pytest.mark.parametrize("dim,n,simplex", [(2, [9, 7], True), (3, [5, 4, 6], False), (1, [9], False)])
def test_spmv_matches_oracle(gdt, oracle, dim, n, simplex):
    g, og = _grid(gdt, oracle, dim, n, simplex)
    rng = np.random.default_rng(3)
    kappa = np.exp(rng.standard_normal(g.num_elements))
    A, _ = oracle.assemble_cg(og, 1, kappa=kappa, dirichlet=False)
    space = gdt.ContinuousLagrangeSpace(g, 1)
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(torch.tensor(kappa, device="cuda")))
    op.assemble()
    x = rng.standard_normal(space.num_DoFs)
    y = op.apply(torch.tensor(x, device="cuda")).cpu().numpy()
    assert rel_err(y, oracle.spmv(A, x)) < 1e-13


def _heat_problem(gdt, oracle, dim, n, simplex, seed=5):
    g, og = _grid(gdt, oracle, dim, n, simplex)
    rng = np.random.default_rng(seed)
    kappa = np.exp(rng.standard_normal(g.num_elements))
    A, b = oracle.assemble_cg(og, 1, kappa=kappa, force_const=1.0)
    space = gdt.ContinuousLagrangeSpace(g, 1)
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(torch.tensor(kappa, device="cuda")))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=1.0, dirichlet=True)
    return op, rhs, A, b


@pytest.mark.parametrize("solver,precond", [("cg", "jacobi"), ("cg", "none"), ("cg", "ilu0"),
                                            ("bicgstab", "jacobi"), ("bicgstab", "ilu0"), ("bicgstab", "none")])
def test_solvers_match_direct(gdt, oracle, solver, precond):
    op, rhs, A, b = _heat_problem(gdt, oracle, 2, [24, 20], True)
    xd = spl.spsolve(A.to_scipy().tocsc(), b)
    x = op.apply_inverse(rhs, opts={"type": solver, "precond": precond, "tol": 1e-13})
    info = op.last_solve_info
    assert info["converged"]
    assert rel_err(x.cpu().numpy(), xd) < 1e-10
    # iteration counts agree with the oracle's restatement of the same algorithm
    xo, it, rr, st = oracle.solve(A, b, solver={"cg": 0, "bicgstab": 1}[solver],
                                  prec={"none": 0, "jacobi": 1, "ilu0": 2}[precond], tol=1e-13)
    assert abs(info["iterations"] - it) <= max(2, 0.05 * it)


def _solve_in(op, rhs, launch, opts):
    op.ctx.set_solver_launch(launch)
    try:
        x = op.apply_inverse(rhs, opts=opts).clone()
    finally:
        op.ctx.set_solver_launch("auto")
    return x, dict(op.last_solve_info)


def _scipy(op):
    import scipy.sparse as sp

    rp, col, val = (t.cpu().numpy() for t in op.csr())
    return sp.csr_matrix((val, col, rp), shape=op.shape)


@pytest.mark.parametrize("case", ["p1_2d", "q1_3d", "swipdg_2d", "q1_1d"])
@pytest.mark.parametrize("precond", ["jacobi", "none"])
def test_persistent_cg_matches_graph_and_direct(gdt, oracle, case, precond):
    # FP64 CG in one cooperative launch (grid barriers between the steps, every block reducing the
    # per-block partials itself) against the graph form of the same iteration and a direct solve;
    # rows of 3 (1D), 7 (P1 triangles), 12 (SWIPDG) and 27 (Q1 hexahedra) entries
    dim, n, simplex, dg = {"p1_2d": (2, [40, 33], True, False), "q1_3d": (3, [9, 8, 7], False, False),
                           "swipdg_2d": (2, [12, 9], True, True), "q1_1d": (1, [1001], False, False)}[case]
    g = gdt.make_cube_grid([0.0] * dim, [1.0] * dim, n, simplex=simplex)
    kappa = torch.exp(torch.tensor(np.random.default_rng(8).standard_normal(g.num_elements), device="cuda"))
    prob = gdt.DiffusionProblem(g, dg=dg)
    prob.assemble(kappa)
    op, rhs = prob.op, prob.rhs
    opts = {"tol": 1e-12, "precond": precond, "max_iter": 100000}
    xg, ig = _solve_in(op, rhs, "graph", opts)
    xp, ip = _solve_in(op, rhs, "persistent", opts)
    xa, ia = _solve_in(op, rhs, "auto", opts)
    assert ig["launch"] == "graph" and ip["launch"] == "persistent" and ia["launch"] == "persistent"
    assert ig["converged"] and ip["converged"]
    assert abs(ig["iterations"] - ip["iterations"]) <= max(2, 0.02 * ig["iterations"])
    assert rel_err(xp.cpu().numpy(), xg.cpu().numpy()) < 1e-9
    xd = spl.spsolve(_scipy(op).tocsc(), rhs.cpu().numpy())
    assert rel_err(xp.cpu().numpy(), xd) < 1e-9
    # the reductions are deterministic: the same iterates launch after launch
    assert ia["iterations"] == ip["iterations"] and torch.equal(xa, xp)


def test_persistent_cg_reports_non_convergence_and_skips_long_rows(gdt, oracle):
    op, rhs, A, b = _heat_problem(gdt, oracle, 2, [30, 30], False)
    lib = gdt._capi.load()
    assert lib.gdt_context_set_solver_launch(op.ctx.handle, 3) == gdt._capi.EINVAL
    assert lib.gdt_context_set_solver_launch(None, 0) == gdt._capi.EINVAL
    op.ctx.set_solver_launch("persistent")
    try:
        with pytest.raises(gdt.GdtError) as e:
            op.apply_inverse(rhs, opts={"tol": 1e-12, "max_iter": 3})
        assert e.value.status == gdt._capi.ENOCONV
        # Q2 hexahedra: rows of up to 125 entries run in the graph form even when persistent is asked for
        g = gdt.make_cube_grid([0.0] * 3, [1.0] * 3, [4, 3, 5])
        space = gdt.ContinuousLagrangeSpace(g, 2)
        op2 = gdt.MatrixOperator(g, space)
        op2 += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(
            torch.ones(g.num_elements, dtype=torch.float64, device="cuda")))
        rhs2 = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
        op2.assemble(rhs=rhs2, force=1.0, dirichlet=True)
        x2 = op2.apply_inverse(rhs2, opts={"tol": 1e-12})
        assert op2.last_solve_info["launch"] == "graph" and op2.last_solve_info["converged"]
        assert rel_err(x2.cpu().numpy(), spl.spsolve(_scipy(op2).tocsc(), rhs2.cpu().numpy())) < 1e-9
    finally:
        op.ctx.set_solver_launch("auto")


@pytest.mark.parametrize("dim,n,blocks", [(2, [200, 200], 1), (3, [40, 40, 40], 2)])
def test_persistent_cg_on_few_blocks_reaches_later_slices(gdt, dim, n, blocks):
    # A warp of the persistent kernel keeps the (offset, width) of its first 32 SELL-32 slices in
    # registers and loads those of later slices from memory. With the grid capped at 1 or 2 blocks
    # (32 or 64 warps) the 1,263 slices of the 200^2 Q1 system and the 2,154 of the 40^3 one give
    # warps a 33rd and later slice, so that branch runs here (a full grid reaches it only above
    # ~5 M rows).
    g = gdt.make_cube_grid([0.0] * dim, [1.0] * dim, n)
    kappa = torch.exp(torch.tensor(np.random.default_rng(12).standard_normal(g.num_elements), device="cuda"))
    prob = gdt.DiffusionProblem(g)
    prob.assemble(kappa)
    op, rhs = prob.op, prob.rhs
    nslices = (op.shape[0] + 31) // 32
    assert nslices > 32 * 32 * blocks
    opts = {"tol": 1e-12, "precond": "jacobi", "max_iter": 100000}
    xg, ig = _solve_in(op, rhs, "graph", opts)
    op.ctx.set_persistent_limits(blocks=blocks)
    try:
        xp, ip = _solve_in(op, rhs, "persistent", opts)
    finally:
        op.ctx.set_persistent_limits()
    assert ip["launch"] == "persistent" and ip["converged"]
    assert abs(ig["iterations"] - ip["iterations"]) <= max(2, 0.02 * ig["iterations"])
    xd = spl.spsolve(_scipy(op).tocsc(), rhs.cpu().numpy())
    assert rel_err(xp.cpu().numpy(), xd) < 1e-10
    assert rel_err(xp.cpu().numpy(), xg.cpu().numpy()) < 1e-10


def test_persistent_cg_barrier_wait_limit_reports_and_recovers(gdt):
    # Every grid-barrier wait of the persistent solver is bounded. With the limit set to 1 ns the
    # first wait runs out: the waiting block sets the fault flag, every block leaves at its next
    # barrier, and the solve reports GDT_ECUDA. The same context then solves normally.
    g = gdt.make_cube_grid([0.0] * 3, [1.0] * 3, [30, 30, 30])
    kappa = torch.exp(torch.tensor(np.random.default_rng(13).standard_normal(g.num_elements), device="cuda"))
    prob = gdt.DiffusionProblem(g)
    prob.assemble(kappa)
    op, rhs = prob.op, prob.rhs
    opts = {"tol": 1e-12, "precond": "jacobi", "max_iter": 100000}
    op.ctx.set_persistent_limits(wait_limit_ns=1)
    try:
        op.ctx.set_solver_launch("persistent")
        with pytest.raises(gdt.GdtError) as e:
            op.apply_inverse(rhs, opts=opts)
    finally:
        op.ctx.set_persistent_limits()
        op.ctx.set_solver_launch("auto")
    assert e.value.status == gdt._capi.ECUDA
    assert "grid barrier wait ran out" in str(e.value)
    x, info = _solve_in(op, rhs, "persistent", opts)
    assert info["launch"] == "persistent" and info["converged"]
    xd = spl.spsolve(_scipy(op).tocsc(), rhs.cpu().numpy())
    assert rel_err(x.cpu().numpy(), xd) < 1e-10


def test_mixed_precision_refinement_reaches_fp64_accuracy(gdt, oracle):
    op, rhs, A, b = _heat_problem(gdt, oracle, 3, [12, 10, 14], False)
    xd = spl.spsolve(A.to_scipy().tocsc(), b)
    x = op.apply_inverse(rhs, opts={"precision": "mixed", "tol": 1e-12})
    info = op.last_solve_info
    assert info["converged"] and info["refinements"] >= 2
    assert rel_err(x.cpu().numpy(), xd) < 1e-9


@pytest.mark.parametrize("n,simplex", [([37, 11, 6], False), ([13, 9, 7], True), ([40, 2, 9], True),
                                       ([1, 5, 6], False), ([33, 8, 3], False)])
def test_mixed_precision_3d_grids_match_direct(gdt, oracle, n, simplex):
    # 3D vertex grids run the plane-tiled FP32 stencil SpMV (ragged 32 x 8 tiles, z chunks); grids
    # only one cell wide fall back to the linear stencil kernel
    op, rhs, A, b = _heat_problem(gdt, oracle, 3, n, simplex)
    xd = spl.spsolve(A.to_scipy().tocsc(), b)
    x = op.apply_inverse(rhs, opts={"precision": "mixed", "tol": 1e-12})
    assert op.last_solve_info["converged"]
    assert rel_err(x.cpu().numpy(), xd) < 1e-9


def test_mixed_precision_matrix_free_operator_follows_the_matrix(gdt, oracle):
    # 3D Q1 Laplace matrices run the inner FP32 operator matrix-free from the element coefficients
    # kept at assembly; a probe product against the assembled matrix guards it at every solve
    op, rhs, A, b = _heat_problem(gdt, oracle, 3, [20, 18, 17], False)
    Asp = A.to_scipy().tocsc()
    x = op.apply_inverse(rhs, opts={"precision": "mixed", "tol": 1e-12})
    assert op.last_solve_info["converged"] and op.last_solve_info["inner_operator"] == "matrix_free"
    assert rel_err(x.cpu().numpy(), spl.spsolve(Asp, b)) < 1e-9
    # values changed behind the library's back (through the zero-copy CSR view): the probe product no
    # longer matches, the solve falls back to the stencil of the actual values
    op.csr()[2].mul_(2.0)
    x2 = op.apply_inverse(rhs, opts={"precision": "mixed", "tol": 1e-12})
    assert op.last_solve_info["converged"] and op.last_solve_info["inner_operator"].startswith("stencil")
    assert rel_err(x2.cpu().numpy(), spl.spsolve(2.0 * Asp, b)) < 1e-9


@pytest.mark.parametrize("n", [[20, 18, 17], [12, 10, 14]])
def test_mixed_precision_direct_launches_match_graphs(gdt, oracle, n):
    # with kernel timing on, the iterations run as direct launches (no graph capture) and the
    # reliable-update kernels run every iteration as early exits: same iterates as the graphs
    op, rhs, A, b = _heat_problem(gdt, oracle, 3, n, False)
    x1 = op.apply_inverse(rhs, opts={"precision": "mixed", "tol": 1e-12}).clone()
    it1 = op.last_solve_info["iterations"]
    lib = gdt._capi.load()
    lib.gdt_context_set_timing(op.ctx.handle, 1)
    try:
        x2 = op.apply_inverse(rhs, opts={"precision": "mixed", "tol": 1e-12})
        it2 = op.last_solve_info["iterations"]
    finally:
        lib.gdt_context_set_timing(op.ctx.handle, 0)
    assert it1 == it2
    assert torch.equal(x1, x2)


@pytest.mark.parametrize("n", [[9, 8, 7], [20, 18, 17], [33, 5, 12], [2, 3, 40]])
@pytest.mark.parametrize("precond", ["jacobi", "none"])
def test_mixed_persistent_matches_graph_form_and_direct(gdt, oracle, n, precond):
    # 3D Q1 Laplace matrices: the matrix-free inner iterations in persistent launches (AUTO) against the
    # graph form of the same Chronopoulos-Gear iteration (element-form operator kernel) and a direct
    # solve; the two operators round differently in FP32, so iteration counts agree only closely
    op, rhs, A, b = _heat_problem(gdt, oracle, 3, n, False)
    xd = spl.spsolve(A.to_scipy().tocsc(), b)
    opts = {"precision": "mixed", "tol": 1e-12, "precond": precond, "max_iter": 100000}
    xp, ip = _solve_in(op, rhs, "auto", opts)
    xg, ig = _solve_in(op, rhs, "graph", opts)
    assert ip["launch"] == "persistent" and ip["inner_operator"] == "matrix_free" and ip["converged"]
    assert ig["launch"] == "graph" and ig["converged"]
    assert abs(ip["iterations"] - ig["iterations"]) <= max(3, 0.05 * ig["iterations"])
    assert rel_err(xp.cpu().numpy(), xd) < 1e-10
    assert rel_err(xg.cpu().numpy(), xd) < 1e-10
    # deterministic reductions: a second solve repeats the iterates bit for bit
    xp2, ip2 = _solve_in(op, rhs, "auto", opts)
    assert ip2["iterations"] == ip["iterations"] and torch.equal(xp2, xp)


@pytest.mark.parametrize("blocks", [1, 3])
def test_mixed_persistent_on_few_blocks(gdt, oracle, blocks):
    # a grid capped at 1 or 3 blocks: every thread walks several (column, z chunk) items and the update
    # pass several float4 groups
    op, rhs, A, b = _heat_problem(gdt, oracle, 3, [30, 28, 26], False)
    op.ctx.set_persistent_limits(blocks=blocks)
    try:
        x, info = _solve_in(op, rhs, "auto", {"precision": "mixed", "tol": 1e-12})
    finally:
        op.ctx.set_persistent_limits()
    assert info["launch"] == "persistent" and info["inner_operator"] == "matrix_free" and info["converged"]
    assert rel_err(x.cpu().numpy(), spl.spsolve(A.to_scipy().tocsc(), b)) < 1e-10


def test_mixed_persistent_barrier_wait_limit_reports_and_recovers(gdt, oracle):
    op, rhs, A, b = _heat_problem(gdt, oracle, 3, [30, 30, 30], False)
    op.ctx.set_persistent_limits(wait_limit_ns=1)
    try:
        with pytest.raises(gdt.GdtError) as e:
            op.apply_inverse(rhs, opts={"precision": "mixed", "tol": 1e-12})
    finally:
        op.ctx.set_persistent_limits()
    assert e.value.status == gdt._capi.ECUDA
    assert "grid barrier wait ran out" in str(e.value)
    x = op.apply_inverse(rhs, opts={"precision": "mixed", "tol": 1e-12})
    assert op.last_solve_info["launch"] == "persistent" and op.last_solve_info["converged"]
    assert rel_err(x.cpu().numpy(), spl.spsolve(A.to_scipy().tocsc(), b)) < 1e-10


def test_mixed_precision_matrix_free_with_separate_dirichlet(gdt, oracle):
    # assembly without constraints, then DirichletConstraints::apply: the operator takes the unit rows
    # and zero columns from the constraint pass
    n = [16, 15, 14]
    g, og = _grid(gdt, oracle, 3, n, False)
    rng = np.random.default_rng(8)
    kappa = np.exp(rng.standard_normal(g.num_elements))
    A, b = oracle.assemble_cg(og, 1, kappa=kappa, force_const=1.0)
    space = gdt.ContinuousLagrangeSpace(g, 1)
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(torch.tensor(kappa, device="cuda")))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    op.assemble(rhs=rhs, force=1.0, dirichlet=False)
    gdt.DirichletConstraints("dirichlet", space).apply(op, rhs)
    x = op.apply_inverse(rhs, opts={"precision": "mixed", "tol": 1e-12})
    assert op.last_solve_info["converged"] and op.last_solve_info["inner_operator"] == "matrix_free"
    assert rel_err(x.cpu().numpy(), spl.spsolve(A.to_scipy().tocsc(), b)) < 1e-9


@pytest.mark.parametrize("dim,n,simplex", [(2, [24, 20], True), (3, [9, 8, 7], False)])
def test_newton_apply_inverse_matches_direct(gdt, oracle, dim, n, simplex):
    # OperatorInterface::apply_inverse, type "newton" (operators/interfaces.hh:490-599) on the affine
    # residual operator x -> A x - b: one undamped step with an exact-enough defect solve
    op, rhs, A, b = _heat_problem(gdt, oracle, dim, n, simplex)
    xd = spl.spsolve(A.to_scipy().tocsc(), b)
    x = op.apply_inverse(rhs, opts={"type": "newton", "precision": 1e-10})
    info = op.last_solve_info
    assert info["iterations"] == 1 and info["dampening_steps"] == 0 and info["linear_iterations"] > 0
    assert info["residual"] < 1e-10
    assert np.linalg.norm(A.to_scipy() @ x.cpu().numpy() - b) < 1e-10
    assert rel_err(x.cpu().numpy(), xd) < 1e-8
    # the reference's defaults (precision 1e-7, max_iter 100) and an initial guess already at the solution
    x2 = op.apply_inverse(rhs, x.clone(), opts={"type": "newton"})
    assert op.last_solve_info["iterations"] == 0
    assert torch.equal(x2, x)


def test_newton_reports_operator_error(gdt, oracle):
    op, rhs, A, b = _heat_problem(gdt, oracle, 2, [16, 16], False)
    with pytest.raises(gdt.GdtError) as e:
        op.apply_inverse(rhs, opts={"type": "newton", "max_iter": 0})
    assert e.value.status == gdt._capi.ENOCONV
    # the defect system cannot be solved (one Krylov iteration allowed)
    with pytest.raises(gdt.GdtError) as e:
        op.apply_inverse(rhs, opts={"type": "newton", "jacobian": {"max_iter": 1}})
    assert e.value.status == gdt._capi.ENOCONV
    assert "defect" in str(e.value)


def test_solver_reports_non_convergence(gdt, oracle):
    op, rhs, A, b = _heat_problem(gdt, oracle, 2, [30, 30], False)
    with pytest.raises(gdt.GdtError) as e:
        op.apply_inverse(rhs, opts={"tol": 1e-12, "max_iter": 3})
    assert e.value.status == gdt._capi.ENOCONV


def test_shape_errors_are_status_codes(gdt):
    g = gdt.make_cube_grid([0, 0], [1, 1], [4, 4])
    op = gdt.MatrixOperator(g, gdt.ContinuousLagrangeSpace(g, 1))
    with pytest.raises(ValueError):
        op.apply(torch.zeros(3, dtype=torch.float64, device="cuda"))
    with pytest.raises(gdt.GdtError) as e:
        gdt.MatrixOperator(g, gdt.ContinuousLagrangeSpace(g, 1), stencil=gdt.Stencil.element_and_intersection)
    assert e.value.status == gdt._capi.EUNSUPPORTED


def _lifted(A, b, dofs, gvals):
    # the Dirichlet-constrained system with values g on the boundary DoFs: b -= A[:, D] g_D on the other
    # rows, then unit rows and columns and b_D = g_D
    import scipy.sparse as sp

    S = A.to_scipy().tolil()
    n = S.shape[0]
    gfull = np.zeros(n)
    gfull[dofs] = gvals[dofs]
    mask = np.zeros(n, bool)
    mask[dofs] = True
    bb = b - S.tocsr() @ gfull
    bb[mask] = gvals[mask]
    S = S.tocsr()
    keep = sp.diags((~mask).astype(float))
    S = keep @ S @ keep + sp.diags(mask.astype(float))
    return S.tocsr(), bb


@pytest.mark.parametrize("dim,n,simplex", [(2, [7, 6], True), (2, [6, 5], False), (3, [4, 3, 5], False),
                                           (3, [3, 3, 2], True)])
@pytest.mark.parametrize("fused", [True, False])
def test_dirichlet_values_match_lifted_oracle_system(gdt, oracle, dim, n, simplex, fused):
    g, og = _grid(gdt, oracle, dim, n, simplex)
    rng = np.random.default_rng(23)
    kappa = np.exp(rng.standard_normal(g.num_elements))
    A, b = oracle.assemble_cg(og, 1, kappa=kappa, force_const=1.0, dirichlet=False)
    space = gdt.ContinuousLagrangeSpace(g, 1)
    gvals = rng.uniform(-1, 1, space.num_DoFs)
    dofs = oracle.dirichlet_dofs(og, 1)
    S, bb = _lifted(A, b, dofs, gvals)
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(torch.tensor(kappa, device="cuda")))
    rhs = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    gt = torch.tensor(gvals, device="cuda")
    if fused:
        op.assemble(rhs=rhs, force=1.0, dirichlet=True, dirichlet_values=gt)
    else:
        op.assemble(rhs=rhs, force=1.0)
        gdt.DirichletConstraints("dirichlet", space).apply(op, rhs, values=gt)
    rp, col, val = (t.cpu().numpy() for t in op.csr())
    import scipy.sparse as sp

    G = sp.csr_matrix((val, col, rp), shape=S.shape)
    assert abs(G - S).max() <= 1e-12 * abs(S).max()
    assert rel_err(rhs.cpu().numpy(), bb) < 1e-12
    for precision in ("fp64", "mixed"):
        x = op.apply_inverse(rhs, opts={"tol": 1e-12, "precision": precision})
        xd = spl.spsolve(S.tocsc(), bb)
        assert rel_err(x.cpu().numpy(), xd) < 1e-10
        assert np.abs(x.cpu().numpy()[dofs] - gvals[dofs]).max() < 1e-12
