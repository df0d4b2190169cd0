"""Every SpMV schedule of the library, pinned with gdt_matrix_set_schedule, against scipy's CSR product
(ConstMatrixOperator::apply, operators/matrix-based.hh:121-129) and through the FP64 and
mixed-precision CG solvers (apply_inverse, operators/matrix-based.hh:131-159).

The autotuner keeps whichever schedule is fastest on the GPU at hand, so each one has to be right on
its own. Schedule 8 reads a SELL-32 copy of the matrix, which has to follow every change of the values. Cases cover row lengths 7 (P1 2D), 12 (SWIPDG P1 2D), 15 (P1 3D) and 27 (Q1 3D), row counts
that are not multiples of a warp, and sizes large enough that every warp of the staged schedules
walks several row slices (the double-buffered path).
"""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

pytestmark = pytest.mark.gpu

# longest row each staged schedule holds (vector-CSR schedules 0-3 hold any row)
_CAPS = {4: 8, 5: 16, 6: 32, 7: 28}

CASES = {
    "p1_2d_ragged": dict(lower=[0, 0], upper=[1, 1], cells=[61, 47], simplex=True, dg=False),
    "p1_2d_large": dict(lower=[0, 0], upper=[1, 1], cells=[300, 300], simplex=True, dg=False),
    "swipdg_p1_2d": dict(lower=[0, 0], upper=[1, 1], cells=[20, 17], simplex=True, dg=True),
    "p1_3d": dict(lower=[0, 0, 0], upper=[1, 1, 1], cells=[11, 9, 7], simplex=True, dg=False),
    "q1_3d_ragged": dict(lower=[0, 0, 0], upper=[1, 1, 1], cells=[13, 11, 9], simplex=False, dg=False),
    "q1_3d_large": dict(lower=[0, 0, 0], upper=[1, 1, 1], cells=[40, 40, 40], simplex=False, dg=False),
}


def _problem(gdt, case):
    c = CASES[case]
    g = gdt.make_cube_grid(c["lower"], c["upper"], c["cells"], simplex=c["simplex"])
    rng = np.random.default_rng(7)
    kappa = torch.tensor(np.exp(0.5 * rng.standard_normal(g.num_elements)), device="cuda")
    prob = gdt.DiffusionProblem(g, dg=c["dg"])
    prob.assemble(kappa)
    rp, col, val = prob.op.csr()
    n = prob.space.num_DoFs
    A = sp.csr_matrix((val.cpu().numpy(), col.cpu().numpy(), rp.cpu().numpy()), shape=(n, n))
    return prob, A


def _valid(schedule, max_row):
    return schedule not in _CAPS or max_row <= _CAPS[schedule]


@pytest.mark.parametrize("case", list(CASES))
def test_every_schedule_matches_scipy_spmv(gdt, case):
    prob, A = _problem(gdt, case)
    max_row = int(np.diff(A.indptr).max())
    x = np.random.default_rng(3).standard_normal(A.shape[1])
    y_ref = A @ x
    xd = torch.tensor(x, device="cuda")
    ran = 0
    for k in range(gdt._capi.SPMV_SCHEDULES):
        st = gdt._capi.load().gdt_matrix_set_schedule(prob.op.handle, k)
        if not _valid(k, max_row):
            assert st == gdt._capi.EINVAL, f"schedule {k} accepted rows of {max_row} entries"
            continue
        assert st == gdt._capi.OK
        y = prob.op.apply(xd).cpu().numpy()
        err = np.abs(y - y_ref).max() / np.abs(y_ref).max()
        assert err < 1e-13, f"schedule {k}: relative difference {err}"
        ran += 1
    assert ran >= 4


@pytest.mark.parametrize("case", ["p1_2d_large", "q1_3d_large", "swipdg_p1_2d"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_every_schedule_solves_alike(gdt, case, precision):
    prob, A = _problem(gdt, case)
    max_row = int(np.diff(A.indptr).max())
    opts = {"type": "cg", "precond": "jacobi", "precision": precision, "tol": 1e-11}
    ref = None
    for k in range(gdt._capi.SPMV_SCHEDULES):
        if not _valid(k, max_row):
            continue
        prob.op.set_spmv_schedule(k)
        u = prob.op.apply_inverse(prob.rhs, opts=opts)
        info = prob.op.last_solve_info
        assert info["converged"], f"schedule {k}: {info}"
        r = prob.rhs.cpu().numpy() - A @ u.cpu().numpy()
        assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(prob.rhs.cpu().numpy()), f"schedule {k}"
        if ref is None:
            ref = u
        else:
            err = ((u - ref).abs().max() / ref.abs().max()).item()
            assert err < 1e-8, f"schedule {k}: relative difference {err}"


def test_set_schedule_rejects_bad_indices(gdt):
    prob, A = _problem(gdt, "q1_3d_ragged")
    L = gdt._capi.load()
    assert L.gdt_matrix_set_schedule(prob.op.handle, -1) == gdt._capi.EINVAL
    assert L.gdt_matrix_set_schedule(prob.op.handle, gdt._capi.SPMV_SCHEDULES) == gdt._capi.EINVAL
    # rows of 27 entries do not fit the 8- and 16-entry staged windows
    assert L.gdt_matrix_set_schedule(prob.op.handle, 4) == gdt._capi.EINVAL
    assert L.gdt_matrix_set_schedule(prob.op.handle, 5) == gdt._capi.EINVAL
    with pytest.raises(gdt._capi.GdtError):
        prob.op.set_spmv_schedule(4)


def test_sell_copy_follows_value_changes(gdt):
    prob, A = _problem(gdt, "q1_3d_ragged")
    op = prob.op
    op.set_spmv_schedule(gdt._capi.SPMV_SCHEDULE_SELL32)
    x = np.random.default_rng(5).standard_normal(A.shape[1])
    xd = torch.tensor(x, device="cuda")

    def check(ref):
        y = op.apply(xd).cpu().numpy()
        y_ref = ref @ x
        assert np.abs(y - y_ref).max() <= 1e-13 * np.abs(y_ref).max()

    check(A)
    # a new assembly
    kappa2 = torch.tensor(np.exp(np.random.default_rng(9).standard_normal(prob.grid.num_elements)), device="cuda")
    prob.assemble(kappa2)
    rp, col, val = op.csr()
    A2 = sp.csr_matrix((val.cpu().numpy(), col.cpu().numpy(), rp.cpu().numpy()), shape=A.shape)
    assert abs(A2 - A).max() > 0
    check(A2)
    # values written through a fresh view (csr() marks the values as changed)
    op.csr()[2].mul_(2.0)
    check(2.0 * A2)
    # values written through a view taken before an apply: values_changed() tells the library
    view = op.csr()[2]
    check(2.0 * A2)
    view.mul_(0.5)
    op.values_changed()
    check(A2)


@pytest.mark.parametrize("case", ["q1_3d_large", "swipdg_p1_2d"])
def test_graph_form_cg_on_the_sell_copy(gdt, case):
    import scipy.sparse.linalg as spl

    prob, A = _problem(gdt, case)
    op = prob.op
    op.set_spmv_schedule(gdt._capi.SPMV_SCHEDULE_SELL32)
    op.ctx.set_solver_launch("graph")
    try:
        u = op.apply_inverse(prob.rhs, opts={"tol": 1e-12, "precond": "jacobi"})
        info = dict(op.last_solve_info)
    finally:
        op.ctx.set_solver_launch("auto")
    assert info["launch"] == "graph" and info["converged"]
    xd = spl.spsolve(A.tocsc(), prob.rhs.cpu().numpy())
    assert np.abs(u.cpu().numpy() - xd).max() <= 1e-10 * np.abs(xd).max()
