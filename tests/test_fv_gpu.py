"""Finite-volume path on the GPU against the oracle: AdvectionFvOperator apply, dt estimate,
explicit Euler and SSP-RK2 (single and batched), and the reference's Burgers 1D tables."""
import numpy as np
import pytest
import torch

from conftest import fv_cell_average_1d, rel_err

pytestmark = pytest.mark.gpu


def _bumps(dim, n, seed, nb=6):
    rng = np.random.default_rng(seed)
    axes = [(np.arange(k) + 0.5) / k for k in n]
    X = np.meshgrid(*axes, indexing="ij")
    u = np.zeros([k for k in n])
    for _ in range(nb):
        c = rng.uniform(0, 1, dim)
        w = rng.uniform(0.05, 0.2)
        a = rng.uniform(-1, 1)
        r2 = sum((X[a_] - c[a_]) ** 2 for a_ in range(dim))
        u += a * np.exp(-r2 / (2 * w * w))
    # lexicographic, x fastest
    return np.ascontiguousarray(u.transpose(list(range(dim))[::-1]).reshape(-1))


CASES = [
    (1, [37]),
    (2, [40, 33]),
    (2, [64, 64]),
    (3, [9, 7, 6]),
]
FLUXES = [("burgers", "lf"), ("burgers", "upwind"), ("burgers", "eo"), ("transport", "lf"), ("transport", "upwind"),
          ("transport", "eo")]


def _op(gdt, g, flux, numflux, dim):
    fl = gdt.BurgersFlux() if flux == "burgers" else gdt.LinearTransportFlux([0.7, -0.4, 0.25][:dim])
    nf = {"lf": gdt.NumericalLaxFriedrichsFlux, "upwind": gdt.NumericalUpwindFlux,
          "eo": gdt.NumericalEngquistOsherFlux}[numflux](fl)
    space = gdt.FiniteVolumeSpace(g)
    return gdt.AdvectionFvOperator(g, nf, space), space


def _orc_args(oracle, flux, numflux, dim):
    return dict(flux=oracle.FLUX_BURGERS if flux == "burgers" else oracle.FLUX_TRANSPORT,
                numflux={"lf": oracle.NUMFLUX_LAX_FRIEDRICHS, "upwind": oracle.NUMFLUX_UPWIND,
                         "eo": oracle.NUMFLUX_ENGQUIST_OSHER}[numflux],
                velocity=[0.7, -0.4, 0.25][:dim])


@pytest.mark.parametrize("dim,n", CASES)
@pytest.mark.parametrize("flux,numflux", FLUXES)
def test_fv_apply_matches_oracle(gdt, oracle, dim, n, flux, numflux):
    g = gdt.make_cube_grid([0] * dim, [1] * dim, n, periodic=True)
    og = oracle.grid(dim, n, 0.0, 1.0, periodic=True)
    op, space = _op(gdt, g, flux, numflux, dim)
    u = _bumps(dim, n, 4)
    a = _orc_args(oracle, flux, numflux, dim)
    ref = oracle.fv_apply(og, a["flux"], a["numflux"], u, velocity=a["velocity"])
    out = op.apply(torch.tensor(u, device="cuda")).cpu().numpy()
    assert rel_err(out, ref) < 1e-13


@pytest.mark.parametrize("dim,n", CASES)
@pytest.mark.parametrize("flux,numflux", FLUXES)
@pytest.mark.parametrize("method", ["euler", "ssp2"])
def test_fv_timesteppers_match_oracle(gdt, oracle, dim, n, flux, numflux, method):
    g = gdt.make_cube_grid([0] * dim, [1] * dim, n, periodic=True)
    og = oracle.grid(dim, n, 0.0, 1.0, periodic=True)
    op, space = _op(gdt, g, flux, numflux, dim)
    u0 = _bumps(dim, n, 9)
    a = _orc_args(oracle, flux, numflux, dim)
    dt_o = oracle.fv_estimate_dt(og, a["flux"], u0, velocity=a["velocity"])
    ut = torch.tensor(u0, device="cuda")
    dt_g = gdt.estimate_dt_for_hyperbolic_system(g, ut, op)
    assert abs(dt_g - dt_o) <= 1e-14 * dt_o
    dt = 0.5 * dt_o
    steps = 25
    stepper = gdt.ExplicitRungeKuttaTimeStepper(op, ut, method=method)
    stepper.step(dt, steps)
    if method == "euler":
        ref = oracle.fv_explicit_euler(og, a["flux"], a["numflux"], u0, dt, steps, velocity=a["velocity"])
    else:
        ref = oracle.fv_ssprk2(og, a["flux"], a["numflux"], u0, dt, steps, velocity=a["velocity"])
    assert rel_err(ut.cpu().numpy(), ref) < 1e-12


def test_fv_batched_equals_single(gdt, oracle):
    n = [48, 40]
    g = gdt.make_cube_grid([0, 0], [1, 1], n, periodic=True)
    og = oracle.grid(2, n, 0.0, 1.0, periodic=True)
    op, space = _op(gdt, g, "burgers", "lf", 2)
    states = [_bumps(2, n, s) for s in (1, 2, 3)]
    ut = torch.tensor(np.concatenate(states), device="cuda")
    dt = 0.4 * min(oracle.fv_estimate_dt(og, oracle.FLUX_BURGERS, s) for s in states)
    gdt.ExplicitRungeKuttaTimeStepper(op, ut, method="ssp2").step(dt, 30)
    out = ut.cpu().numpy().reshape(3, -1)
    for b, s in enumerate(states):
        ref = oracle.fv_ssprk2(og, oracle.FLUX_BURGERS, oracle.NUMFLUX_LAX_FRIEDRICHS, s, dt, 30)
        assert rel_err(out[b], ref) < 1e-12


@pytest.mark.parametrize("flux", ["numerical_upwind_flux", "numerical_lax_friedrichs_flux", "numerical_engquist_osher_flux"])
def test_burgers_1d_tables_on_gpu(gdt, oracle, golden, flux):
    # dune/gdt/test/burgers/burgers__1d__explicit__fv.mini through the GPU path
    case = golden["burgers_1d"][flux]
    res = case["results"]
    for lvl, n in enumerate((16, 32)):
        g = gdt.make_cube_grid([0.0], [1.0], [n], periodic=True)
        fl = gdt.BurgersFlux()
        nf = {"numerical_upwind_flux": gdt.NumericalUpwindFlux, "numerical_lax_friedrichs_flux": gdt.NumericalLaxFriedrichsFlux,
              "numerical_engquist_osher_flux": gdt.NumericalEngquistOsherFlux}[flux](fl)
        op = gdt.AdvectionFvOperator(g, nf, gdt.FiniteVolumeSpace(g))
        u0 = fv_cell_average_1d(n, lambda x: np.exp(-(x - 0.33) ** 2 / (2 * 0.075 ** 2)), 3)
        ut = torch.tensor(u0, device="cuda")
        fv_dt = gdt.estimate_dt_for_hyperbolic_system(g, ut, op)
        dt = 0.99 * case["setup"]["use_fixed_dt"]
        stepper = gdt.ExplicitRungeKuttaTimeStepper(op, ut, method="euler")
        t, count, masses = 0.0, 1, []
        while t < 1.0 + dt:
            stepper.step(dt, 1)
            t += dt
            count += 1
            masses.append(ut.sum().item() / n)
        assert count == res["quantity.num_timesteps"][lvl]
        assert float("%.2e" % (dt / fv_dt)) == pytest.approx(res["quantity.CFL"][lvl], rel=1e-12)
        m0 = u0.sum() / n
        assert max(abs(m - m0) / m0 for m in masses) < 1e-14


@pytest.mark.parametrize("dim,n", [(1, [37]), (2, [40, 33]), (3, [9, 7, 6])])
@pytest.mark.parametrize("method", ["euler", "ssp2"])
def test_fv_timestep_stays_inside_its_work_buffer(gdt, oracle, dim, n, method):
    # gdt_fv_timestep through the C ABI with a work buffer of exactly GDT_FV_WORK_DOUBLES doubles,
    # followed by a guard band of sentinels inside the same allocation: the guard must come back intact
    import ctypes as C

    g = gdt.make_cube_grid([0] * dim, [1] * dim, n, periodic=True)
    og = oracle.grid(dim, n, 0.0, 1.0, periodic=True)
    op, space = _op(gdt, g, "burgers", "lf", dim)
    N, nbatch = space.num_DoFs, 2
    states = [_bumps(dim, n, s) for s in (11, 12)]
    u = torch.tensor(np.concatenate(states), device="cuda")
    stepper = gdt.ExplicitRungeKuttaTimeStepper(op, u, method=method)
    need = stepper.work_doubles(nbatch)
    assert need == (2 if method == "ssp2" else 1) * nbatch * N
    guard = 4096
    buf = torch.full((need + guard,), 1.2345e300, dtype=torch.float64, device="cuda")
    dt = 0.4 * min(oracle.fv_estimate_dt(og, oracle.FLUX_BURGERS, s) for s in states)
    tsm = gdt._capi.TIMESTEPPER_SSPRK2 if method == "ssp2" else gdt._capi.TIMESTEPPER_EXPLICIT_EULER
    op.ctx.call("gdt_fv_timestep", space.handle, C.byref(op.desc), tsm, C.c_double(dt), C.c_int64(7),
                C.c_int64(nbatch), C.c_void_p(u.data_ptr()), C.c_void_p(buf.data_ptr()))
    torch.cuda.synchronize()
    assert bool((buf[need:] == 1.2345e300).all()), "gdt_fv_timestep wrote past its documented work size"
    step_ref = oracle.fv_ssprk2 if method == "ssp2" else oracle.fv_explicit_euler
    out = u.cpu().numpy().reshape(nbatch, -1)
    for b, s in enumerate(states):
        assert rel_err(out[b], step_ref(og, oracle.FLUX_BURGERS, oracle.NUMFLUX_LAX_FRIEDRICHS, s, dt, 7)) < 1e-12


# ------------------------------------------------------------------ non-periodic boundaries ---
# (grid periodic?, per-side treatment: None, ("extrapolate",), ("inflow", state) or ("flux", g))
BOUNDARY_SETUPS = {
    "walls_by_absence": (False, {}),
    "outflow_all": (False, {s: ("extrapolate",) for s in ("-x", "+x", "-y", "+y", "-z", "+z")}),
    "inflow_outflow_walls": (False, {"-x": ("inflow", 0.8), "+x": ("extrapolate",), "-y": ("flux", 0.0),
                                     "+y": ("flux", 0.0), "-z": ("inflow", -0.3), "+z": ("extrapolate",)}),
    "periodic_but_x": (True, {"-x": ("inflow", 0.6), "+x": ("flux", 0.25)}),
}


def _apply_setup(gdt, op, dim, setup):
    kinds, vals = [0] * 6, [0.0] * 6
    sides = ("-x", "+x", "-y", "+y", "-z", "+z")[: 2 * dim]
    for side, t in setup.items():
        if side not in sides:
            continue
        if t[0] == "extrapolate":
            tr = gdt.BoundaryTreatmentByCustomExtrapolation()
        elif t[0] == "inflow":
            tr = gdt.BoundaryTreatmentByCustomExtrapolation(state=t[1])
        else:
            tr = gdt.BoundaryTreatmentByCustomNumericalFlux(t[1])
        op.append(tr, filter=side)
        kinds[sides.index(side)], vals[sides.index(side)] = tr.kind, tr.value
    return kinds, vals


BND_CASES = [(1, [37]), (2, [40, 33]), (2, [1, 9]), (3, [9, 7, 6])]


@pytest.mark.parametrize("dim,n", BND_CASES)
@pytest.mark.parametrize("flux,numflux", FLUXES)
@pytest.mark.parametrize("setup", list(BOUNDARY_SETUPS))
def test_fv_boundary_treatments_match_oracle(gdt, oracle, dim, n, flux, numflux, setup):
    periodic, sides = BOUNDARY_SETUPS[setup]
    g = gdt.make_cube_grid([0] * dim, [1] * dim, n, periodic=periodic)
    og = oracle.grid(dim, n, 0.0, 1.0, periodic=periodic)
    op, space = _op(gdt, g, flux, numflux, dim)
    kinds, vals = _apply_setup(gdt, op, dim, sides)
    u = _bumps(dim, n, 6) + 0.2
    a = _orc_args(oracle, flux, numflux, dim)
    ref = oracle.fv_apply(og, a["flux"], a["numflux"], u, velocity=a["velocity"], boundary=kinds, boundary_value=vals)
    out = op.apply(torch.tensor(u, device="cuda")).cpu().numpy()
    assert rel_err(out, ref) < 1e-13


@pytest.mark.parametrize("flux,numflux", FLUXES)
@pytest.mark.parametrize("method", ["euler", "ssp2"])
@pytest.mark.parametrize("setup", ["inflow_outflow_walls", "periodic_but_x"])
def test_fv_boundary_timesteppers_match_oracle(gdt, oracle, flux, numflux, method, setup):
    dim, n = 2, [70, 45]  # tiled 2D stepper, partial tiles on both axes
    periodic, sides = BOUNDARY_SETUPS[setup]
    g = gdt.make_cube_grid([0, 0], [1, 1], n, periodic=periodic)
    og = oracle.grid(dim, n, 0.0, 1.0, periodic=periodic)
    op, space = _op(gdt, g, flux, numflux, dim)
    kinds, vals = _apply_setup(gdt, op, dim, sides)
    u0 = _bumps(dim, n, 11) + 0.2
    a = _orc_args(oracle, flux, numflux, dim)
    dt = 0.4 * oracle.fv_estimate_dt(og, a["flux"], u0, velocity=a["velocity"])
    ut = torch.tensor(np.concatenate([u0, u0[::-1].copy()]), device="cuda")  # a batch of two states
    gdt.ExplicitRungeKuttaTimeStepper(op, ut, method=method).step(dt, 20)
    run = oracle.fv_explicit_euler if method == "euler" else oracle.fv_ssprk2
    out = ut.cpu().numpy().reshape(2, -1)
    for b, s in enumerate([u0, u0[::-1].copy()]):
        ref = run(og, a["flux"], a["numflux"], s, dt, 20, velocity=a["velocity"], boundary=kinds, boundary_value=vals)
        assert rel_err(out[b], ref) < 1e-12


def test_fv_impermeable_walls_conserve_mass(gdt):
    n = [96, 80]
    g = gdt.make_cube_grid([0, 0], [1, 1], n)
    op, space = _op(gdt, g, "burgers", "lf", 2)
    op.append(gdt.BoundaryTreatmentByCustomNumericalFlux(0.0))
    u0 = torch.tensor(_bumps(2, n, 3), device="cuda")
    ut = u0.clone()
    dt = 0.4 * gdt.estimate_dt_for_hyperbolic_system(g, ut, op)
    gdt.ExplicitRungeKuttaTimeStepper(op, ut, method="ssp2").step(dt, 50)
    assert abs(float(ut.sum() - u0.sum())) <= 1e-12 * float(u0.abs().sum())
    assert float((ut - u0).abs().max()) > 1e-3  # the state did move


def test_fv_boundary_treatment_rejects_half_periodic_directions(gdt):
    g = gdt.make_cube_grid([0, 0], [1, 1], [8, 8], periodic=True)
    op, space = _op(gdt, g, "burgers", "lf", 2)
    op.append(gdt.BoundaryTreatmentByCustomExtrapolation(), filter="-x")
    with pytest.raises(gdt.GdtError) as e:
        op.apply(torch.zeros(64, dtype=torch.float64, device="cuda"))
    assert e.value.status == gdt._capi.EINVAL
