"""The generalised batched solver against the oracle: P1 (Kuhn triangles) and Q1 (squares), kappa per
element or per quadrant, meshes of uneven size, each team kind (cluster of 8 CTAs, one CTA, one warp
per problem) in FP64 and mixed precision; the autotuner's choice; a problem with non-finite data
skipped and reported while the others are solved (the batched scheduler's failure path, injected on
the host)."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu

# stencil slot k -> vertex offset (k % 3 - 1, k // 3 - 1); P1 keeps 7 of the 9 (CSR column order)
SLOTS = {"p1": [0, 1, 3, 4, 5, 7, 8], "q1": list(range(9))}


def quadrant_kappa(n, mu, per_cell):
    cells = np.arange(n * n)
    cx, cy = cells % n, cells // n
    q = (cx >= n // 2).astype(int) + 2 * (cy >= n // 2).astype(int)
    return np.repeat(mu[q], per_cell)


def oracle_problem(oracle, element, n, kappa):
    og = oracle.grid(2, [n, n], 0.0, 1.0, simplex=element == "p1")
    return oracle.assemble_cg(og, 1, kappa=kappa, force_const=1.0)


def dense_rows(A, n, slots):
    nv = n + 1
    out = np.zeros((A.n, len(slots)))
    for r in range(A.n):
        ix, iy = r % nv, r // nv
        cols = A.col[A.row_ptr[r]:A.row_ptr[r + 1]]
        vals = A.val[A.row_ptr[r]:A.row_ptr[r + 1]]
        for k, sl in enumerate(slots):
            jx, jy = ix + sl % 3 - 1, iy + sl // 3 - 1
            if 0 <= jx < nv and 0 <= jy < nv:
                hit = np.nonzero(cols == jx + nv * jy)[0]
                assert len(hit) == 1
                out[r, k] = vals[hit[0]]
    return out


def check_against_oracle(oracle, b, element, kappa_of, x, st, tol_x):
    x = x.cpu().numpy()
    st = st.cpu().numpy().reshape(-1, len(SLOTS[element]))
    for i, n in enumerate(b.cells):
        A, rhs = oracle_problem(oracle, element, n, kappa_of(i))
        S = st[b.offsets[i]:b.offsets[i + 1]]
        assert rel_err(S, dense_rows(A, n, SLOTS[element])) < 1e-12, (element, n)
        xd = spl.spsolve(A.to_scipy().tocsc(), rhs)
        assert rel_err(x[b.offsets[i]:b.offsets[i + 1]], xd) < tol_x, (element, n)


@pytest.mark.parametrize("element", ["p1", "q1"])
@pytest.mark.parametrize("team", ["cluster", "cta", "warp"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_per_element_kappa_each_team(gdt, oracle, element, team, precision):
    cells = [6, 11, 4, 16, 9, 12, 3, 20, 1, 7]
    b = gdt.BatchedDiffusion(cells, element=element)
    rng = np.random.default_rng(100 + len(team))
    kap = np.exp(rng.standard_normal(b.total_elements))  # lognormal per element
    b.set_teams(team)
    assert b.teams() == [team] * len(cells)
    x, st = b.solve(kappa=torch.tensor(kap, device="cuda"), precision=precision, tol=1e-12, keep_stencil=True)
    assert b.last_info["all_converged"]
    eo = b.element_offsets
    check_against_oracle(oracle, b, element, lambda i: kap[eo[i]:eo[i + 1]], x, st, 1e-9)
    its, rr = b.iterations()
    assert (its >= 0).all() and (rr <= 1e-12).all()
    assert (b.status() == gdt._capi.OK).all()


@pytest.mark.parametrize("element", ["p1", "q1"])
def test_quadrant_kappa_mixed_teams(gdt, oracle, element):
    # one batch, all three team kinds at once; more problems per kind than one cluster item holds
    # (8 CTA teams, 64 warp teams per item)
    rng = np.random.default_rng(7)
    cells = list(rng.choice([2, 4, 6, 8], size=80)) + [10, 12, 14, 16, 18, 20, 22, 24, 26, 28] + [40, 32]
    b = gdt.BatchedDiffusion(cells, element=element)
    teams = ["warp"] * 80 + ["cta"] * 10 + ["cluster"] * 2
    b.set_teams(teams)
    mu = rng.uniform(0.1, 10.0, (len(cells), 4))
    x, st = b.solve(torch.tensor(mu, device="cuda"), tol=1e-12, keep_stencil=True)
    per_cell = 2 if element == "p1" else 1
    check_against_oracle(oracle, b, element, lambda i: quadrant_kappa(cells[i], mu[i], per_cell), x, st, 1e-9)


def test_teams_give_the_same_solve(gdt):
    # the same problem on every team kind: the same CG sequence up to the order of the reductions, whose
    # rounding moves the iteration count by a few per cent at a tight tolerance
    cells = [24, 24, 24]
    b = gdt.BatchedDiffusion(cells)
    mu = np.random.default_rng(3).uniform(0.1, 10.0, 4)
    b.set_teams(["cluster", "cta", "warp"])
    x = b.solve(torch.tensor(np.tile(mu, (3, 1)), device="cuda"), tol=1e-10)
    its, _ = b.iterations()
    assert abs(its[0] - its[1]) <= max(2, 0.06 * its[0]) and abs(its[0] - its[2]) <= max(2, 0.06 * its[0])
    assert rel_err(b.unpack(x, 1).cpu().numpy(), b.unpack(x, 0).cpu().numpy()) < 1e-9
    assert rel_err(b.unpack(x, 2).cpu().numpy(), b.unpack(x, 0).cpu().numpy()) < 1e-9


def test_autotuner_picks_the_fastest_team_per_size(gdt, oracle):
    cells = [8] * 40 + [24] * 12 + [64] * 3
    b = gdt.BatchedDiffusion(cells)
    rng = np.random.default_rng(11)
    mu = torch.tensor(rng.uniform(0.1, 10.0, (len(cells), 4)), device="cuda")
    times = b.tune(mu, tol=1e-10)
    assert sorted(times) == [8, 24, 64]
    for size, t in times.items():
        assert set(t) >= {"cluster", "cta"} and all(v > 0 for v in t.values())
        assert ("warp" in t) == ((size + 1) ** 2 <= 20000)
    chosen = b.teams()
    for i, c in enumerate(cells):
        assert chosen[i] == min(times[c], key=times[c].get)
    x, st = b.solve(mu, tol=1e-12, keep_stencil=True)
    check_against_oracle(oracle, b, "p1", lambda i: quadrant_kappa(cells[i], mu[i].cpu().numpy(), 2), x, st, 1e-9)


@pytest.mark.parametrize("team", ["cluster", "cta", "warp"])
def test_nonfinite_kappa_is_skipped_and_reported(gdt, oracle, team):
    cells = [8, 12, 8, 6]
    b = gdt.BatchedDiffusion(cells)
    b.set_teams(team)
    rng = np.random.default_rng(5)
    kap = np.exp(rng.standard_normal(b.total_elements))
    eo = b.element_offsets
    kap[eo[1] + 17] = np.nan  # problem 1 poisoned
    kap[eo[3]] = np.inf       # problem 3 poisoned
    x = torch.full((b.total_dofs,), 7.0, dtype=torch.float64, device="cuda")
    with pytest.raises(gdt.GdtError) as e:
        b.solve(kappa=torch.tensor(kap, device="cuda"), tol=1e-12, x=x)
    assert e.value.status == gdt._capi.ENAN
    assert b.last_info["nonfinite_problems"] == 2
    st = b.status()
    assert list(st) == [gdt._capi.OK, gdt._capi.ENAN, gdt._capi.OK, gdt._capi.ENAN]
    xs = x.cpu().numpy()
    for i in (1, 3):
        assert (xs[b.offsets[i]:b.offsets[i + 1]] == 0).all()
    for i in (0, 2):
        A, rhs = oracle_problem(oracle, "p1", cells[i], kap[eo[i]:eo[i + 1]])
        xd = spl.spsolve(A.to_scipy().tocsc(), rhs)
        assert rel_err(xs[b.offsets[i]:b.offsets[i + 1]], xd) < 1e-9


def test_argument_checks(gdt):
    b = gdt.BatchedDiffusion([3, 4])
    with pytest.raises(gdt.GdtError) as e:  # kappa per quadrant needs even sides
        b.solve(torch.ones(8, dtype=torch.float64, device="cuda"))
    assert e.value.status == gdt._capi.EINVAL
    with pytest.raises(ValueError):
        b.solve()
    with pytest.raises(KeyError):
        b.set_teams("block")
