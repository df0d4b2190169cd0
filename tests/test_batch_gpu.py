"""Batched persistent assemble + solve against the oracle (per problem: assembled rows within 1e-12,
solutions vs a direct solve) and against the single-problem GPU path (iteration counts)."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu

OFFS = [(-1, -1), (0, -1), (-1, 0), (0, 0), (1, 0), (0, 1), (1, 1)]


def quadrant_kappa(n, mu):
    # element e = 2 * cell + t, cell lexicographic (x fastest); quadrant q = qx + 2 qy
    cells = np.arange(n * n)
    cx, cy = cells % n, cells // n
    q = (cx >= n // 2).astype(int) + 2 * (cy >= n // 2).astype(int)
    return np.repeat(mu[q], 2)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_oracle(gdt, oracle, precision):
    cells = [6, 10, 4, 16, 8, 12, 2, 20]
    rng = np.random.default_rng(17)
    mu = rng.uniform(0.1, 10.0, (len(cells), 4))
    b = gdt.BatchedDiffusion(cells)
    x, st = b.solve(torch.tensor(mu, device="cuda"), force=1.0, precision=precision, tol=1e-12, keep_stencil=True)
    assert b.last_info["all_converged"]
    x = x.cpu().numpy()
    st = st.cpu().numpy().reshape(-1, 7)
    for i, n in enumerate(cells):
        og = oracle.grid(2, [n, n], 0.0, 1.0, simplex=True)
        A, rhs = oracle.assemble_cg(og, 1, kappa=quadrant_kappa(n, mu[i]), force_const=1.0)
        nv = n + 1
        S = st[b.offsets[i]:b.offsets[i + 1]]
        dense = np.zeros_like(S)
        for r in range(A.n):
            ix, iy = r % nv, r // nv
            cols = A.col[A.row_ptr[r]:A.row_ptr[r + 1]]
            vals = A.val[A.row_ptr[r]:A.row_ptr[r + 1]]
            for k, (dx, dy) in enumerate(OFFS):
                jx, jy = ix + dx, iy + dy
                if 0 <= jx < nv and 0 <= jy < nv:
                    c = jx + nv * jy
                    hit = np.nonzero(cols == c)[0]
                    assert len(hit) == 1
                    dense[r, k] = vals[hit[0]]
        assert rel_err(S, dense) < 1e-12
        xd = spl.spsolve(A.to_scipy().tocsc(), rhs)
        assert rel_err(x[b.offsets[i]:b.offsets[i + 1]], xd) < 1e-9


def test_batch_iterations_match_single_problem_path(gdt, oracle):
    cells = [32, 16, 24]
    rng = np.random.default_rng(3)
    mu = rng.uniform(0.1, 10.0, (len(cells), 4))
    b = gdt.BatchedDiffusion(cells)
    x = b.solve(torch.tensor(mu, device="cuda"), tol=1e-10)
    its, rr = b.iterations()
    for i, n in enumerate(cells):
        g = gdt.make_cube_grid([0, 0], [1, 1], [n, n], simplex=True)
        prob = gdt.DiffusionProblem(g, solver_opts={"tol": 1e-10})
        u = prob.solve(torch.tensor(quadrant_kappa(n, mu[i]), device="cuda"))
        single = prob.op.last_solve_info["iterations"]
        assert abs(its[i] - single) <= max(2, 0.02 * single)
        assert rel_err(b.unpack(x, i).cpu().numpy(), u.cpu().numpy()) < 1e-8


def test_batch_reports_non_convergence(gdt):
    b = gdt.BatchedDiffusion([16, 8])
    mu = torch.ones(8, dtype=torch.float64, device="cuda")
    with pytest.raises(gdt.GdtError) as e:
        b.solve(mu, tol=1e-12, max_iter=3)
    assert e.value.status == gdt._capi.ENOCONV
    its, _ = b.iterations()
    assert (its < 0).all()


def test_batch_mixed_keeps_the_krylov_rate(gdt):
    # one FP32 sequence with reliable updates: no restarts, so the iteration count stays near the FP64 one
    cells = [64, 40, 24]
    rng = np.random.default_rng(5)
    mu = torch.tensor(rng.uniform(0.1, 10.0, (len(cells), 4)), device="cuda")
    b = gdt.BatchedDiffusion(cells)
    x64 = b.solve(mu, tol=1e-10, precision="fp64").cpu().numpy()
    its64, _ = b.iterations()
    xmx = b.solve(mu, tol=1e-10, precision="mixed").cpu().numpy()
    itsmx, rr = b.iterations()
    assert (itsmx > 0).all() and (rr <= 1e-10).all()
    assert (itsmx <= 1.3 * its64 + 10).all(), (itsmx, its64)
    assert rel_err(xmx, x64) < 1e-8


def test_batch_mixed_reports_non_convergence(gdt):
    b = gdt.BatchedDiffusion([16, 8])
    mu = torch.ones(8, dtype=torch.float64, device="cuda")
    with pytest.raises(gdt.GdtError) as e:
        b.solve(mu, tol=1e-12, max_iter=3, precision="mixed")
    assert e.value.status == gdt._capi.ENOCONV
    its, rr = b.iterations()
    assert (its < 0).all() and (rr > 1e-12).all()
