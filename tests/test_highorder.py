"""Host logic of the order-2 continuous Lagrange spaces (no GPU): DoF counts of the MCMG layout
against the oracle (ContinuousMapper, spaces/mapper/continuous.hh:117-182) and the quadrature rule of
the element-batched assembly path."""
import itertools
import math

import numpy as np
import pytest

from conftest import import_gdt

GRIDS = [(1, [7], False), (2, [5, 4], False), (2, [4, 3], True), (3, [3, 2, 4], False), (3, [2, 3, 2], True)]


@pytest.mark.parametrize("dim,n,simplex", GRIDS)
def test_order2_space_size_matches_oracle(oracle, dim, n, simplex):
    gdt = import_gdt()
    g = gdt.make_cube_grid([0.0] * dim, [1.0] * dim, n, simplex=simplex)
    og = oracle.grid(dim, n, 0.0, 1.0, simplex=simplex)
    space = gdt.ContinuousLagrangeSpace(g, 2)
    assert space.num_DoFs == oracle.space_size(og, oracle.CG, 2)
    assert space.max_local_size == {1: 3, 2: 6 if simplex else 9, 3: 10 if simplex else 27}[dim]


@pytest.mark.parametrize("dim,simplex", [(1, False), (2, False), (2, True), (3, False), (3, True)])
def test_quadrature_rule_is_exact(dim, simplex):
    gdt = import_gdt()
    g = gdt.make_cube_grid([0.0] * dim, [1.0] * dim, [2] * dim, simplex=simplex)
    for order in (1, 2):
        x, w = gdt.ContinuousLagrangeSpace(g, order).quadrature()
        deg = 2 * order + 2
        for e in itertools.product(range(deg + 1), repeat=dim):
            if (sum(e) if simplex else max(e)) > deg:
                continue
            num = float(np.sum(w * np.prod([x[:, a] ** e[a] for a in range(dim)], axis=0)))
            if simplex:  # int over the unit simplex of x^a y^b z^c = a! b! c! / (a + b + c + d)!
                exact = math.prod(math.factorial(k) for k in e) / math.factorial(sum(e) + dim)
            else:
                exact = math.prod(1.0 / (k + 1) for k in e)
            assert abs(num - exact) <= 1e-14, (order, e, num, exact)
