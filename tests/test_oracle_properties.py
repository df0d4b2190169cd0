"""CPU checks of the oracle and of the algebra the GPU kernels rely on: FV boundary treatments (exact
discrete values, mass balance), the element-coefficient form of the Q1 Laplace operator that the
matrix-free inner operator applies, and the Chronopoulos-Gear CG recurrences of the mixed solver."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl

NONE, EXTRAPOLATE, DIRICHLET, FLUX = 0, 1, 2, 3


def test_fv_upwind_inflow_outflow_exact_values(oracle):
    # linear transport a = 1 on 1D cells of width 1/4, upwind flux: inflow state 0.5 on the left,
    # extrapolation on the right: L(u)_i = (u_i - u_{i-1}) / h with u_{-1} = 0.5
    g = oracle.grid(1, [4], 0.0, 1.0, periodic=False)
    u = np.array([1.0, 2.0, 3.0, 4.0])
    out = oracle.fv_apply(g, oracle.FLUX_TRANSPORT, oracle.NUMFLUX_UPWIND, u, velocity=[1.0],
                          boundary=[DIRICHLET, EXTRAPOLATE], boundary_value=[0.5, 0.0])
    assert np.allclose(out, [(1.0 - 0.5) * 4, (2.0 - 1.0) * 4, (3.0 - 2.0) * 4, (4.0 - 3.0) * 4], rtol=0, atol=1e-14)


@pytest.mark.parametrize("numflux", ["lf", "upwind", "eo"])
def test_fv_walls_conserve_mass_and_flux_boundaries_balance(oracle, numflux):
    nf = {"lf": oracle.NUMFLUX_LAX_FRIEDRICHS, "upwind": oracle.NUMFLUX_UPWIND,
          "eo": oracle.NUMFLUX_ENGQUIST_OSHER}[numflux]
    n = [7, 5]
    g = oracle.grid(2, n, 0.0, 1.0, periodic=False)
    u = np.random.default_rng(2).uniform(-1, 1, 35)
    vol = 1.0 / 35
    for kinds in ([NONE] * 4, [FLUX] * 4):
        out = oracle.fv_apply(g, oracle.FLUX_BURGERS, nf, u, boundary=kinds, boundary_value=[0.0] * 4)
        assert abs(out.sum() * vol) < 1e-14
    # prescribed boundary fluxes g on each side: d/dt sum(u |E|) = -sum_sides g |side|
    gb = [0.3, -0.2, 0.7, 0.1]
    out = oracle.fv_apply(g, oracle.FLUX_BURGERS, nf, u, boundary=[FLUX] * 4, boundary_value=gb)
    side = [1.0, 1.0, 1.0, 1.0]  # unit square: every side has length 1
    assert abs(out.sum() * vol - sum(a * b for a, b in zip(gb, side))) < 1e-13


def _q1_reference_stiffness(h):
    m1 = lambda a: np.array([[a / 3, a / 6], [a / 6, a / 3]])
    s1 = lambda a: np.array([[1 / a, -1 / a], [-1 / a, 1 / a]])
    # corner index x + 2 y + 4 z
    return (np.kron(m1(h[2]), np.kron(m1(h[1]), s1(h[0]))) + np.kron(m1(h[2]), np.kron(s1(h[1]), m1(h[0])))
            + np.kron(s1(h[2]), np.kron(m1(h[1]), m1(h[0]))))


@pytest.mark.parametrize("ncell", [[6, 5, 4], [3, 7, 2]])
def test_q1_laplace_is_the_sum_of_coefficient_scaled_element_matrices(oracle, ncell):
    # the matrix-free inner operator applies q_v = sum_cells kappa_c sum_j K[l_v][j] v_j, with unit rows
    # and zero columns on the Dirichlet boundary; it must equal the assembled matrix
    og = oracle.grid(3, ncell, 0.0, 1.0)
    rng = np.random.default_rng(4)
    kappa = np.exp(rng.standard_normal(int(np.prod(ncell))))
    A, _ = oracle.assemble_cg(og, 1, kappa=kappa, force_const=1.0)
    nx, ny, nz = (c + 1 for c in ncell)
    K = _q1_reference_stiffness([1.0 / c for c in ncell])
    v = rng.uniform(-1, 1, nx * ny * nz)
    V = v.reshape(nz, ny, nx)
    bnd = np.zeros((nz, ny, nx), bool)
    bnd[0], bnd[-1], bnd[:, 0], bnd[:, -1], bnd[:, :, 0], bnd[:, :, -1] = (True,) * 6
    Vm = np.where(bnd, 0.0, V)
    Kap = kappa.reshape(ncell[2], ncell[1], ncell[0])
    q = np.zeros_like(V)
    for cz in range(ncell[2]):
        for cy in range(ncell[1]):
            for cx in range(ncell[0]):
                loc = np.array([Vm[cz + (j >> 2), cy + ((j >> 1) & 1), cx + (j & 1)] for j in range(8)])
                y = Kap[cz, cy, cx] * (K @ loc)
                for i in range(8):
                    q[cz + (i >> 2), cy + ((i >> 1) & 1), cx + (i & 1)] += y[i]
    q = np.where(bnd, V, q)
    ref = A.to_scipy() @ v
    assert np.abs(q.reshape(-1) - ref).max() <= 1e-12 * np.abs(ref).max()


def test_chronopoulos_gear_recurrences_match_cg(oracle):
    # the mixed matrix-free path runs CG in the Chronopoulos-Gear form (one reduction phase per
    # iteration); in exact arithmetic its iterates are those of preconditioned CG
    og = oracle.grid(2, [14, 11], 0.0, 1.0, simplex=True)
    kappa = np.exp(np.random.default_rng(6).standard_normal(14 * 11 * 2))  # two triangles per square
    A, b = oracle.assemble_cg(og, 1, kappa=kappa, force_const=1.0)
    A = A.to_scipy()
    d = 1.0 / A.diagonal()
    x = np.zeros_like(b)
    r = b.copy()
    z = d * r
    w = A @ z
    gamma, delta = r @ z, z @ w
    alpha, beta = gamma / delta, 0.0
    p = np.zeros_like(b)
    s = np.zeros_like(b)
    its = 0
    while np.linalg.norm(r) > 1e-12 * np.linalg.norm(b) and its < 1000:
        p = z + beta * p
        s = w + beta * s
        x += alpha * p
        r -= alpha * s
        z = d * r
        w = A @ z
        gamma_new, delta = r @ z, z @ w
        beta = gamma_new / gamma
        alpha = gamma_new / (delta - beta * gamma_new / alpha)
        gamma = gamma_new
        its += 1
    xd = spl.spsolve(A.tocsc(), b)
    assert np.linalg.norm(x - xd) <= 1e-9 * np.linalg.norm(xd)
    _, it_cg, _, _ = oracle.solve(oracle.assemble_cg(og, 1, kappa=kappa, force_const=1.0)[0], b, tol=1e-12)
    assert abs(its - it_cg) <= 2


@pytest.mark.parametrize("dim,n,simplex,order", [(2, [4, 3], False, 1), (2, [3, 3], True, 2), (3, [2, 3, 2], False, 1),
                                                 (3, [2, 2, 2], True, 1)])
def test_tensor_diffusion_restatement_reduces_to_scalar(oracle, dim, n, simplex, order):
    # LocalLaplaceIntegrand with a tensor (local/integrands/laplace.hh:81-102): kappa_e * I gives the
    # scalar assembly (pinned to the reference's known answers) to rounding, and the transpose of an
    # anisotropic tensor's matrix is the matrix of the transposed tensor
    og = oracle.grid(dim, n, 0.0, 1.0, simplex=simplex)
    ne = oracle.num_elements(og)
    rng = np.random.default_rng(31)
    kappa = np.exp(rng.standard_normal(ne))
    A, b = oracle.assemble_cg(og, order, kappa=kappa, force_const=1.0, dirichlet=False)
    At, bt = oracle.assemble_cg_tensor(og, order, kappa[:, None, None] * np.eye(dim)[None], force_const=1.0,
                                       dirichlet=False)
    assert np.array_equal(A.col, At.col)
    assert np.abs(A.val - At.val).max() <= 1e-14 * np.abs(A.val).max()
    assert np.abs(b - bt).max() <= 1e-14 * np.abs(b).max()
    K = rng.standard_normal((ne, dim, dim))
    M1, _ = oracle.assemble_cg_tensor(og, order, K, dirichlet=False)
    M2, _ = oracle.assemble_cg_tensor(og, order, np.transpose(K, (0, 2, 1)), dirichlet=False)
    S1, S2 = M1.to_scipy(), M2.to_scipy()
    assert abs(S1 - S2.T).max() <= 1e-13 * abs(S1).max()


@pytest.mark.parametrize("dim,n,order", [(2, [5, 4], 1), (2, [4, 3], 2), (3, [3, 2, 3], 1), (3, [2, 2, 2], 2)])
def test_threaded_walk_equals_serial_on_simplices(oracle, dim, n, order):
    # the threaded grid walk colours elements so that no two of one colour share a DoF: with the d!
    # simplices of a cube in different colours its results are those of the serial walk
    og = oracle.grid(dim, n, 0.0, 1.0, simplex=True)
    ne = oracle.num_elements(og)
    rng = np.random.default_rng(7)
    kappa, force = np.exp(rng.standard_normal(ne)), rng.uniform(-1, 1, ne)
    try:
        oracle.set_threads(1)
        A1, b1 = oracle.assemble_cg(og, order, kappa=kappa, force=force)
        oracle.set_threads(8)
        A8, b8 = oracle.assemble_cg(og, order, kappa=kappa, force=force)
    finally:
        oracle.set_threads(1)
    assert np.abs(A1.val - A8.val).max() <= 1e-14 * np.abs(A1.val).max()
    assert np.abs(b1 - b8).max() <= 1e-14 * np.abs(b1).max()
