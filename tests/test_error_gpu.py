"""Element error indicators on the GPU (the EOC studies' norms, test/stationary-eocstudies/base.hh:259-269):
the ESV2007 H1-semi errors of SWIPDG on cube grids against the reference table
(stationary_heat_equation__ESV2007__table_1.mini) and the oracle, L2 norms against the oracle, and
exactness for nodal interpolants of quadratics in P2/Q2."""
import itertools
import math

import numpy as np
import pytest
import scipy.sparse.linalg as spl
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _esv2007_grad(X):
    hp = 0.5 * np.pi
    gx = -hp * torch.sin(hp * X[..., 0]) * torch.cos(hp * X[..., 1])
    gy = -hp * torch.cos(hp * X[..., 0]) * torch.sin(hp * X[..., 1])
    return torch.stack([gx, gy], -1).contiguous()


def test_esv2007_h1_semi_table(gdt, oracle, golden):
    # NearlyESV2007Table1ButWithCubicGridTest: [-1,1]^2, 8x8 cubes refined twice, DG Q1, SWIPDG (sigma 8/14, h = |I|)
    O = oracle
    ref = golden["esv2007_cube"]["results"]["norm.H_1_semi"]
    for lvl, n in enumerate((8, 16, 32)):
        og = O.grid(2, [n, n], [-1, -1], [1, 1])
        A, b = O.assemble_swipdg(og, order=1, force_fn=O.FORCE_ESV2007, force_order=4, theta=1.0,
                                 sigma_inner=8.0, sigma_boundary=14.0)
        u = spl.spsolve(A.to_scipy().tocsc(), b)
        g = gdt.make_cube_grid([-1, -1], [1, 1], [n, n])
        space = gdt.DiscontinuousLagrangeSpace(g, 1)
        X = space.quadrature_points(12)
        eta2, total = gdt.element_error(space, torch.tensor(u, device="cuda"), _esv2007_grad(X), "h1_semi", 12)
        assert abs(total - O.h1_semi_error_esv2007(og, O.DG, 1, u)) < 1e-11 * total
        assert float("%.2e" % total) == pytest.approx(ref[lvl], rel=1e-12)
        assert abs(math.sqrt(eta2.sum().item()) - total) < 1e-13 * total


@pytest.mark.parametrize("dim,n,simplex,order", [(2, [6, 5], True, 1), (2, [6, 5], False, 2), (2, [5, 4], True, 2),
                                                 (3, [3, 2, 3], False, 2), (3, [2, 3, 2], True, 2)])
def test_l2_norm_matches_oracle(gdt, oracle, dim, n, simplex, order):
    og = oracle.grid(dim, n, 0.0, 1.0, simplex=simplex)
    g = gdt.make_cube_grid([0.0] * dim, [1.0] * dim, n, simplex=simplex)
    space = gdt.ContinuousLagrangeSpace(g, order)
    u = np.random.default_rng(8).standard_normal(space.num_DoFs)
    ne, nq = g.num_elements, space.quadrature(2 * order + 2)[0].shape[0]
    zero = torch.zeros((ne, nq), dtype=torch.float64, device="cuda")
    _, total = gdt.element_error(space, torch.tensor(u, device="cuda"), zero, "l2", 2 * order + 2)
    assert abs(total - oracle.l2_norm(og, oracle.CG, order, u)) < 1e-12 * total


@pytest.mark.parametrize("dim,n,simplex", [(2, [5, 4], False), (2, [4, 5], True), (3, [3, 2, 2], False), (3, [2, 2, 3], True)])
def test_order2_interpolant_of_quadratic_is_exact(gdt, dim, n, simplex):
    # u = 1 + x + 2 y^2 - x y (+ z^2 - y z): its P2/Q2 nodal interpolant is u itself, both errors vanish
    lo, hi = [0.0] * dim, [1.0 + 0.25 * a for a in range(dim)]
    g = gdt.make_cube_grid(lo, hi, n, simplex=simplex)
    space = gdt.ContinuousLagrangeSpace(g, 2)

    def ufun(X):
        x, y = X[..., 0], X[..., 1]
        v = 1 + x + 2 * y ** 2 - x * y
        if dim == 3:
            v = v + X[..., 2] ** 2 - y * X[..., 2]
        return v

    def ugrad(X):
        x, y = X[..., 0], X[..., 1]
        cols = [1 - y, 4 * y - x]
        if dim == 3:
            z = X[..., 2]
            cols = [1 - y, 4 * y - x - z, 2 * z - y]
        return torch.stack(cols, -1).contiguous()

    # DoF values: the function at the local nodes (a, b, c) / 2 of every element (lexicographic, first
    # coordinate fastest, a + b + c <= 2 on simplices), mapped like the quadrature points
    nodes = [(a / 2, b / 2, c / 2) for c in range(3 if dim == 3 else 1) for b in range(3) for a in range(3)
             if not simplex or a + b + c <= 2]
    d = dim
    h = torch.tensor([(hi[a] - lo[a]) / n[a] for a in range(d)], dtype=torch.float64, device="cuda")
    nsub = math.factorial(d) if simplex else 1
    e = torch.arange(g.num_elements, device="cuda")
    cube, t = e // nsub, e % nsub
    idx, rest = [], cube
    for a in range(d):
        idx.append(rest % n[a])
        rest = rest // n[a]
    ci = torch.stack(idx, 1).to(torch.float64)
    xr = torch.tensor([p[:d] for p in nodes], dtype=torch.float64, device="cuda")
    if simplex:
        J = torch.zeros((nsub, d, d), dtype=torch.float64, device="cuda")
        for k, perm in enumerate(itertools.permutations(range(d))):
            for m in range(d):
                for a in perm[:m + 1]:
                    J[k, a, m] = 1.0
        local = torch.einsum("tam,qm->tqa", J, xr)[t]
    else:
        local = xr[None].expand(g.num_elements, -1, -1)
    Xn = torch.tensor(lo, dtype=torch.float64, device="cuda") + h * (ci[:, None, :] + local)
    gi = space.global_indices()
    u = torch.zeros(space.num_DoFs, dtype=torch.float64, device="cuda")
    u[gi.reshape(-1)] = ufun(Xn).reshape(-1)
    Xq = space.quadrature_points(6)
    _, e_h1 = gdt.element_error(space, u, ugrad(Xq), "h1_semi", 6)
    _, e_l2 = gdt.element_error(space, u, ufun(Xq).contiguous(), "l2", 6)
    assert e_h1 < 1e-12 and e_l2 < 1e-12
