"""GB300-native drop-in for dune-gdt's discretize-and-solve path (Python side).

Mirrors the names of the reference's Python bindings (python/dune/gdt/*: spaces, MatrixOperator,
VectorFunctional, DirichletConstraints, DiscreteFunction, AdvectionFvOperator, ...). DoF vectors
and coefficients are CUDA torch tensors (float64); all compute goes through the C ABI of
libgdtgb300.so (include/gdt_gb300.h). There is no CPU fallback: without the library or a GPU every
compute call raises.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _capi as capi
from . import replicas
from ._capi import GdtError

__all__ = [
    "Context", "default_context", "make_cube_grid", "Grid", "make_simplex_mesh", "SimplexMesh",
    "ContinuousLagrangeSpace",
    "DiscontinuousLagrangeSpace", "FiniteVolumeSpace", "Stencil", "LocalLaplaceIntegrand",
    "LocalElementProductIntegrand", "LocalElementIntegralBilinearForm", "LocalElementIntegralFunctional",
    "LocalLaplaceIPDGInnerCoupling", "LocalLaplaceIPDGDirichletCoupling", "LocalIPDGInnerPenalty",
    "LocalEllipticIpdgIntegrands",
    "LocalIPDGBoundaryPenalty", "LocalCouplingIntersectionIntegralBilinearForm",
    "LocalIntersectionIntegralBilinearForm", "MatrixOperator", "VectorFunctional", "DirichletConstraints",
    "Walker", "DiscreteFunction", "BurgersFlux", "LinearTransportFlux", "NumericalLaxFriedrichsFlux",
    "NumericalUpwindFlux", "NumericalEngquistOsherFlux", "AdvectionFvOperator", "BoundaryTreatmentByCustomExtrapolation",
    "BoundaryTreatmentByCustomNumericalFlux", "ExplicitRungeKuttaTimeStepper",
    "estimate_dt_for_hyperbolic_system", "GdtError", "element_error", "LincombOperator", "lincomb", "GridFunction",
]


def _ptr(t):
    if t is None:
        return None
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("expected a CUDA tensor")
    return C.c_void_p(t.data_ptr())


def _f64(t, n=None, name="vector"):
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64 or not t.is_contiguous():
        raise TypeError(f"{name} must be a contiguous float64 CUDA tensor")
    if n is not None and t.numel() != n:
        raise ValueError(f"{name} has {t.numel()} entries, expected {n}")
    return t


# ---------------------------------------------------------------------------- context ---
class Context:
    """Device + CUDA stream the library works on (the torch current stream by default)."""

    def __init__(self, device=0, stream=None):
        self.lib = capi.load()
        self.device = torch.device("cuda", device)
        self.stream = stream if stream is not None else torch.cuda.current_stream(self.device)
        h = C.c_void_p()
        capi.check(self.lib.gdt_context_create(device, C.c_void_p(self.stream.cuda_stream), C.byref(h)))
        self.handle = h

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.lib.gdt_context_destroy(self.handle)
        except Exception:
            pass

    def call(self, name, *args):
        capi.check(getattr(self.lib, name)(self.handle, *args), self.handle, name)

    def synchronize(self):
        self.call("gdt_context_synchronize")

    @property
    def kernel_launches(self):
        return int(self.lib.gdt_context_kernel_launches(self.handle))

    def set_solver_launch(self, mode):
        """Launch form of FP64 CG solves: 'auto' (persistent wherever it applies), 'graph'
        (one kernel per step, CUDA graphs) or 'persistent' (one cooperative launch for all iterations)."""
        self.call("gdt_context_set_solver_launch", {"auto": capi.SOLVER_LAUNCH_AUTO, "graph": capi.SOLVER_LAUNCH_GRAPH,
                                                    "persistent": capi.SOLVER_LAUNCH_PERSISTENT}[mode])

    def set_persistent_limits(self, blocks=0, wait_limit_ns=0):
        """Grid size cap (0: one block per SM) and grid-barrier wait limit in ns (0: one second) of the
        persistent solver launches."""
        self.call("gdt_context_set_persistent_limits", int(blocks), int(wait_limit_ns))


_default = {}


def default_context() -> Context:
    dev = torch.cuda.current_device()
    if dev not in _default:
        _default[dev] = Context(dev)
    return _default[dev]


# ------------------------------------------------------------------------------- grid ---
class Grid:
    """make_cube_grid: equidistant YaspGrid-like cube grid or its Kuhn simplex split."""

    def __init__(self, lower_left, upper_right, num_elements, simplex=False, periodic=False):
        dim = len(num_elements)
        self.dimension = dim
        self.lower_left = [float(x) for x in lower_left]
        self.upper_right = [float(x) for x in upper_right]
        self.num_cells = [int(n) for n in num_elements]
        self.simplex = bool(simplex)
        self.periodic = bool(periodic)
        self.vertices = None  # the coordinates of a mapped grid ([num_vertices, dim] float64)
        self.lib = capi.load()
        h = C.c_void_p()
        n = (C.c_int64 * 3)(*self.num_cells, *([1] * (3 - dim)))
        lo = (C.c_double * 3)(*self.lower_left, *([0.0] * (3 - dim)))
        hi = (C.c_double * 3)(*self.upper_right, *([1.0] * (3 - dim)))
        capi.check(self.lib.gdt_grid_create_cube(dim, n, lo, hi, int(simplex), int(periodic), C.byref(h)),
                   what="make_cube_grid")
        self.handle = h

    def map_vertices(self, coords):
        """Moves the vertices to `coords` ([num_vertices, dim], vertices lexicographic with x fastest;
        numpy or torch, host or device): a mapped structured grid whose elements take their geometry
        from their own vertices (gdt_grid_set_vertices). Call before creating spaces; a mapped grid
        takes continuous order-1 spaces and the Laplace stiffness / load vector assembly."""
        import numpy as np

        nv = int(self.lib.gdt_grid_num_vertices(self.handle))
        if isinstance(coords, torch.Tensor):
            keep = coords.detach().to(torch.float64).contiguous()
            shape, ptr = tuple(keep.shape), keep.data_ptr()
        else:
            keep = np.ascontiguousarray(coords, dtype=np.float64)
            shape, ptr = keep.shape, keep.ctypes.data
        if shape != (nv, self.dimension):
            raise ValueError(f"coords must have shape ({nv}, {self.dimension}), got {shape}")
        capi.check(self.lib.gdt_grid_set_vertices(self.handle, C.c_void_p(ptr)), what="map_vertices")
        self.vertices = torch.as_tensor(keep).clone()
        return self

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.lib.gdt_grid_destroy(self.handle)
        except Exception:
            pass

    @property
    def num_elements(self):
        return int(self.lib.gdt_grid_num_elements(self.handle))

    @property
    def num_vertices(self):
        return int(self.lib.gdt_grid_num_vertices(self.handle))

    @property
    def cell_volume(self):
        v = 1.0
        for a in range(self.dimension):
            v *= (self.upper_right[a] - self.lower_left[a]) / self.num_cells[a]
        if self.simplex:
            import math

            v /= math.factorial(self.dimension)
        return v


class SimplexMesh:
    """An unstructured simplex mesh: the leaf view of a DUNE simplex grid (ALUGrid, UGGrid, a gmsh
    import) exported in its index-set order (gdt_grid_create_simplex_mesh). coords [num_vertices, dim]
    (dim 2 or 3), cells [num_elements, dim + 1] vertex indices; numpy or torch, host or device.
    Continuous order-1 spaces (DoF = vertex index), their Laplace stiffness and load vector (kappa and
    source per element or constant), Dirichlet constraints on the boundary vertices (vertices of faces
    of one element), the solvers and the log-kappa gradient work on it."""

    def __init__(self, coords, cells):
        import numpy as np

        self.lib = capi.load()
        if isinstance(coords, torch.Tensor):
            xk = coords.detach().to(torch.float64).contiguous()
            xp = xk.data_ptr()
        else:
            xk = np.ascontiguousarray(coords, dtype=np.float64)
            xp = xk.ctypes.data
        if isinstance(cells, torch.Tensor):
            ck = cells.detach().to(torch.int64).contiguous()
            cp = ck.data_ptr()
        else:
            ck = np.ascontiguousarray(cells, dtype=np.int64)
            cp = ck.ctypes.data
        if len(xk.shape) != 2 or xk.shape[1] not in (2, 3) or len(ck.shape) != 2 or ck.shape[1] != xk.shape[1] + 1:
            raise ValueError(f"coords [num_vertices, 2 or 3] and cells [num_elements, dim + 1] expected, got "
                             f"{tuple(xk.shape)} and {tuple(ck.shape)}")
        self.dimension = int(xk.shape[1])
        self.simplex, self.periodic = True, False
        h = C.c_void_p()
        capi.check(self.lib.gdt_grid_create_simplex_mesh(self.dimension, int(xk.shape[0]), C.c_void_p(xp),
                                                         int(ck.shape[0]), C.c_void_p(cp), C.byref(h)),
                   what="make_simplex_mesh")
        self.handle = h
        self.vertices = torch.as_tensor(xk).clone()
        self.cells = torch.as_tensor(ck).clone()

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.lib.gdt_grid_destroy(self.handle)
        except Exception:
            pass

    @property
    def num_elements(self):
        return int(self.lib.gdt_grid_num_elements(self.handle))

    @property
    def num_vertices(self):
        return int(self.lib.gdt_grid_num_vertices(self.handle))


def make_simplex_mesh(coords, cells) -> SimplexMesh:
    return SimplexMesh(coords, cells)


def make_cube_grid(lower_left, upper_right, num_elements, simplex=False, periodic=False) -> Grid:
    dim = len(num_elements)
    if not hasattr(lower_left, "__len__"):
        lower_left = [lower_left] * dim
    if not hasattr(upper_right, "__len__"):
        upper_right = [upper_right] * dim
    return Grid(lower_left, upper_right, num_elements, simplex, periodic)


# ----------------------------------------------------------------------------- spaces ---
class _Space:
    kind = None

    def __init__(self, grid: Grid, order: int):
        self.grid = grid
        self.order = order
        self.lib = capi.load()
        h = C.c_void_p()
        capi.check(self.lib.gdt_space_create(grid.handle, self.kind, order, C.byref(h)), what=type(self).__name__)
        self.handle = h

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.lib.gdt_space_destroy(self.handle)
        except Exception:
            pass

    @property
    def num_DoFs(self):
        return int(self.lib.gdt_space_size(self.handle))

    size = num_DoFs

    @property
    def max_local_size(self):
        return int(self.lib.gdt_space_max_local_size(self.handle))

    def quadrature(self, order=None):
        """(x_ref [nq, 3], w_ref [nq]) on the reference element: with order=None the rule of the
        element-batched assembly path (coefficients given per quadrature point are [element, q] at
        these points), else a rule exact to that polynomial order (element_error)."""
        import numpy as np

        if order is None:
            fn, args = self.lib.gdt_space_quadrature, ()
        else:
            fn, args = self.lib.gdt_space_quadrature_order, (int(order),)
        nq = int(fn(self.handle, *args, None, None))
        if nq < 0:
            raise GdtError(capi.EUNSUPPORTED, "no quadrature rule for this space")
        x = np.zeros((nq, 3))
        w = np.zeros(nq)
        fn(self.handle, *args, x.ctypes.data_as(C.c_void_p), w.ctypes.data_as(C.c_void_p))
        return x, w

    def quadrature_points(self, order=None, device=None):
        """Physical quadrature points of every element, a float64 tensor [element, q, dim]."""
        import itertools
        import math

        x, _ = self.quadrature(order)
        g = self.grid
        if isinstance(g, SimplexMesh):  # the affine map of every element: x_0 + sum_k xi_k (x_{k+1} - x_0)
            device = device or torch.device("cuda", torch.cuda.current_device())
            d = g.dimension
            X = g.vertices.to(device)[g.cells.to(device)]  # [element, d + 1, d]
            xr = torch.tensor(x[:, :d], device=device)  # [q, d]
            return X[:, None, 0, :] + torch.einsum("qk,ekd->eqd", xr, X[:, 1:, :] - X[:, None, 0, :])
        if getattr(g, "vertices", None) is not None:
            raise GdtError(capi.EUNSUPPORTED, "quadrature points of mapped grids")
        d = g.dimension
        device = device or torch.device("cuda", torch.cuda.current_device())
        lo = torch.tensor(g.lower_left, dtype=torch.float64, device=device)
        h = torch.tensor([(g.upper_right[a] - g.lower_left[a]) / g.num_cells[a] for a in range(d)],
                         dtype=torch.float64, device=device)
        xr = torch.tensor(x[:, :d], device=device)
        simplex = g.simplex and d >= 2
        nsub = math.factorial(d) if simplex else 1
        e = torch.arange(g.num_elements, device=device)
        cube, t = e // nsub, e % nsub
        idx, rest = [], cube
        for a in range(d):
            idx.append(rest % g.num_cells[a])
            rest = rest // g.num_cells[a]
        ci = torch.stack(idx, 1).to(torch.float64)  # [ne, d]
        if simplex:  # type t maps the reference simplex onto corners 0, e_pi0, e_pi0 + e_pi1, ...
            J = torch.zeros((nsub, d, d), dtype=torch.float64, device=device)
            for k, perm in enumerate(itertools.permutations(range(d))):
                for m in range(d):
                    for a in perm[:m + 1]:
                        J[k, a, m] = 1.0
            local = torch.einsum("tam,qm->tqa", J, xr)[t]  # [ne, nq, d]
        else:
            local = xr[None].expand(g.num_elements, -1, -1)
        return lo + h * (ci[:, None, :] + local)

    def face_points(self, device=None):
        """Physical coordinates of the two Gauss points of every face of every element (DG spaces on 2D
        simplex grids): float64 tensor [element, 3, 2, 2] (gdt_dg_face_points)."""
        import numpy as np

        out = np.zeros((self.grid.num_elements, 3, 2, 2))
        capi.check(self.lib.gdt_dg_face_points(self.handle, out.ctypes.data_as(C.c_void_p)),
                   what="gdt_dg_face_points")
        return torch.tensor(out, device=device or torch.device("cuda", torch.cuda.current_device()))

    def global_indices(self, ctx: Context | None = None):
        """mapper.global_indices of every element: int64 CUDA tensor [num_elements, local_size]."""
        ctx = ctx or default_context()
        out = torch.empty((self.grid.num_elements, self.max_local_size), dtype=torch.int64, device=ctx.device)
        ctx.call("gdt_space_global_indices", self.handle, _ptr(out))
        return out


class ContinuousLagrangeSpace(_Space):
    kind = capi.SPACE_CG

    def __init__(self, grid, order=1):
        super().__init__(grid, order)


class DiscontinuousLagrangeSpace(_Space):
    kind = capi.SPACE_DG

    def __init__(self, grid, order=1):
        super().__init__(grid, order)


class FiniteVolumeSpace(_Space):
    kind = capi.SPACE_FV

    def __init__(self, grid):
        super().__init__(grid, 0)


class Stencil:
    element = capi.STENCIL_ELEMENT
    intersection = capi.STENCIL_INTERSECTION
    element_and_intersection = capi.STENCIL_ELEMENT_AND_INTERSECTION


# ------------------------------------------------------------------- local forms (descriptors) ---
def _coef(c):
    """A diffusion / source coefficient: a Python number or a per-element float64 CUDA tensor."""
    if isinstance(c, torch.Tensor):
        return _f64(c, name="coefficient"), 0.0
    return None, float(c)


def _coef_qp(c):
    """(per-element tensor, constant, per-quadrature-point tensor): a number, a 1D tensor with one value
    per element, or a 2D tensor [element, quadrature point] (points of _Space.quadrature())."""
    if isinstance(c, torch.Tensor) and c.dim() == 2:
        return None, 0.0, _f64(c.contiguous() if c.is_contiguous() else c, name="coefficient")
    t, k = _coef(c)
    return t, k, None


class GridFunction:
    """A function of the global point x with its polynomial order, as dune-xt's
    GenericFunction(order, lambda) (examples/stationary-heat-equation.cc:68-70): `fn` maps a float64
    tensor of points [..., dim] to the values [...]. As the source of a load vector it is evaluated at
    the points of the Gauss rule of order `order` + the space's order (the reference's product
    integrand at its own quadrature points), not sampled per element."""

    def __init__(self, fn, order=3):
        self.fn = fn
        self.order = int(order)

    def at_quadrature_points(self, space):
        quad_order = self.order + space.order
        pts = space.quadrature_points(order=quad_order)
        vals = self.fn(pts)
        vals = torch.as_tensor(vals, dtype=torch.float64, device=pts.device)
        if tuple(vals.shape) != tuple(pts.shape[:2]):
            raise ValueError(f"GridFunction returned shape {tuple(vals.shape)}, expected {tuple(pts.shape[:2])}")
        return vals.contiguous(), quad_order


def _force_fields(d, force, space):
    """Sets force / force_const / force_qp / force_quad_order of a DiffusionDesc; returns the tensors
    that must stay alive while the descriptor is used."""
    if isinstance(force, GridFunction):
        vals, quad_order = force.at_quadrature_points(space)
        d.force, d.force_const = None, 0.0
        d.force_qp, d.force_quad_order = vals.data_ptr(), quad_order
        return [vals]
    ft, fc = _coef(force)
    d.force = ft.data_ptr() if ft is not None else None
    d.force_const = fc
    d.force_qp, d.force_quad_order = None, 0
    return [ft]


def _dirichlet_values(d, values, space, ctx):
    """Sets dirichlet_values / dirichlet_value_const of a DiffusionDesc: a number, a per-DoF float64
    tensor or a GridFunction (evaluated at the vertices, the DoFs of order-1 continuous spaces)."""
    d.dirichlet_values, d.dirichlet_value_const = None, 0.0
    if values is None:
        return []
    if isinstance(values, (int, float)):
        d.dirichlet_value_const = float(values)
        return []
    if isinstance(values, GridFunction) and getattr(space.grid, "vertices", None) is not None:
        values = torch.as_tensor(values.fn(space.grid.vertices.to(ctx.device)), dtype=torch.float64, device=ctx.device)
    elif isinstance(values, GridFunction):
        g = space.grid
        dim = g.dimension
        vn = [c + 1 for c in g.num_cells]
        idx = torch.arange(space.num_DoFs, device=ctx.device)
        coords = []
        for a in range(dim):
            i = idx % vn[a]
            idx = idx // vn[a]
            h = (g.upper_right[a] - g.lower_left[a]) / g.num_cells[a]
            coords.append(g.lower_left[a] + h * i.to(torch.float64))
        values = torch.as_tensor(values.fn(torch.stack(coords, -1)), dtype=torch.float64, device=ctx.device)
    t = _f64(values.contiguous(), space.num_DoFs, "Dirichlet values")
    d.dirichlet_values = t.data_ptr()
    return [t]


class LocalLaplaceIntegrand:
    def __init__(self, diffusion=1.0):
        self.diffusion = diffusion


class _ProductWithAnsatz:
    def __init__(self, weight, function):
        self.weight = weight
        self.function = function


class LocalElementProductIntegrand:
    """weight * phi_i * phi_j (local/integrands/product.hh:89-130): as a bilinear form the weighted
    product (mass) matrix, weight a number, a per-element tensor or a [element, quadrature point]
    tensor; with_ansatz(f) lowers the load-vector integrand (unit weight)."""

    def __init__(self, weight=1.0):
        self.weight = weight

    def with_ansatz(self, function):
        if isinstance(self.weight, torch.Tensor) or self.weight != 1.0:
            raise GdtError(capi.EUNSUPPORTED, "only the unit weight is lowered for load vectors")
        return _ProductWithAnsatz(self.weight, function)


class LocalElementIntegralBilinearForm:
    def __init__(self, integrand, over_integrate=0):
        self.integrand = integrand


class LocalElementIntegralFunctional:
    def __init__(self, integrand, over_integrate=0):
        self.integrand = integrand


class _Sum:
    def __init__(self, *terms):
        self.terms = list(terms)

    def __add__(self, other):
        return _Sum(*self.terms, other)


class _Term:
    def __add__(self, other):
        return _Sum(self, other)


class LocalLaplaceIPDGInnerCoupling(_Term):
    def __init__(self, symmetry_prefactor, diffusion, weight=None):
        self.symmetry_prefactor, self.diffusion, self.weight = float(symmetry_prefactor), diffusion, weight


class LocalLaplaceIPDGDirichletCoupling(_Term):
    """Dirichlet boundary terms (local/integrands/laplace-ipdg.hh:231-368). dirichlet_data (a number, a
    GridFunction, or a [element, 3, 2] tensor of values at the face points of gdt_dg_face_points) is read
    only for the right-hand side, the unary term -theta int g (kappa grad psi_i . n)."""

    def __init__(self, symmetry_prefactor, diffusion, dirichlet_data=0.0):
        self.symmetry_prefactor, self.diffusion = float(symmetry_prefactor), diffusion
        self.dirichlet_data = dirichlet_data


class LocalIPDGInnerPenalty(_Term):
    def __init__(self, penalty, weight=None, beta=None):
        self.penalty, self.weight, self.beta = float(penalty), weight, beta


class LocalIPDGBoundaryPenalty(_Term):
    """Dirichlet penalty sigma (n . w n) / h; with dirichlet_data, the right-hand side also gets its
    counterpart int sigma (n . w n) / h g psi_i."""

    def __init__(self, penalty, weight=None, beta=None, dirichlet_data=None):
        self.penalty, self.weight, self.beta = float(penalty), weight, beta
        self.dirichlet_data = dirichlet_data


class LocalEllipticIpdgIntegrands:
    """The deprecated combined SWIPDG integrands (local/integrands/elliptic-ipdg.hh): the same bilinear form
    as InnerCoupling + InnerPenalty and DirichletCoupling + BoundaryPenalty, with the penalty sigma from
    the polynomial order (Epshteyn, Riviere 2007; :452-501) and the length h^beta, beta = 1 / (d - 1)."""

    @staticmethod
    def default_beta(dim):
        return float(capi.load().gdt_elliptic_ipdg_beta(int(dim)))

    @staticmethod
    def inner_sigma(pol_order):
        return float(capi.load().gdt_elliptic_ipdg_sigma(int(pol_order), 0))

    @staticmethod
    def boundary_sigma(pol_order):
        return float(capi.load().gdt_elliptic_ipdg_sigma(int(pol_order), 1))

    @staticmethod
    def Inner(diffusion, pol_order=1, dim=2, beta=None):
        b = LocalEllipticIpdgIntegrands.default_beta(dim) if beta is None else float(beta)
        return (LocalLaplaceIPDGInnerCoupling(1.0, diffusion, diffusion)
                + LocalIPDGInnerPenalty(LocalEllipticIpdgIntegrands.inner_sigma(pol_order), diffusion, beta=b))

    @staticmethod
    def DirichletBoundary(diffusion, pol_order=1, dim=2, beta=None):
        b = LocalEllipticIpdgIntegrands.default_beta(dim) if beta is None else float(beta)
        return (LocalLaplaceIPDGDirichletCoupling(1.0, diffusion)
                + LocalIPDGBoundaryPenalty(LocalEllipticIpdgIntegrands.boundary_sigma(pol_order), diffusion, beta=b))


class LocalCouplingIntersectionIntegralBilinearForm:
    def __init__(self, integrand):
        self.integrand = integrand


class LocalIntersectionIntegralBilinearForm:
    def __init__(self, integrand):
        self.integrand = integrand


def _terms(x):
    return x.terms if isinstance(x, _Sum) else [x]


# ---------------------------------------------------------------------------- matrix operator ---
class MatrixOperator:
    """make_matrix_operator(space, stencil): CSR matrix on the device + the appended local forms."""

    def __init__(self, grid, source_space, range_space=None, stencil=Stencil.element, ctx: Context | None = None):
        self.grid = grid
        self.source_space = source_space
        self.range_space = range_space or source_space
        self.ctx = ctx or default_context()
        self.stencil = stencil
        h = C.c_void_p()
        self.ctx.call("gdt_matrix_create", self.range_space.handle, self.source_space.handle, int(stencil),
                      C.byref(h))
        self.handle = h
        self.forms = []
        self._keep = []

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                capi.load().gdt_matrix_destroy(self.handle)
        except Exception:
            pass

    def append(self, local_form):
        self.forms.append(local_form)
        return self

    def __iadd__(self, local_form):
        return self.append(local_form)

    @property
    def shape(self):
        L = capi.load()
        return int(L.gdt_matrix_rows(self.handle)), int(L.gdt_matrix_cols(self.handle))

    @property
    def nnz(self):
        return int(capi.load().gdt_matrix_nnz(self.handle))

    def csr(self):
        """(row_ptr, col, val) as zero-copy CUDA tensors over the library-owned CSR arrays. Values written
        through these tensors after a later apply() need values_changed() before the next apply()."""
        rp, col, val = C.c_void_p(), C.c_void_p(), C.c_void_p()
        capi.check(capi.load().gdt_matrix_device_arrays(self.handle, C.byref(rp), C.byref(col), C.byref(val)))
        n, nnz = self.shape[0], self.nnz
        return (_wrap(rp.value, n + 1, torch.int32, self.ctx.device), _wrap(col.value, nnz, torch.int32, self.ctx.device),
                _wrap(val.value, nnz, torch.float64, self.ctx.device))

    def values_changed(self):
        """Tell the library that the values were written through csr() tensors (gdt_matrix_values_changed)."""
        capi.check(capi.load().gdt_matrix_values_changed(self.handle), what="gdt_matrix_values_changed")

    @property
    def matrix(self):
        return self.csr()

    def set_spmv_schedule(self, schedule):
        """Pin the SpMV schedule (0 .. capi.SPMV_SCHEDULES-1) of every SpMV-type kernel of this matrix
        instead of autotuning it; raises GdtError(EINVAL) when it cannot hold the longest row."""
        capi.check(capi.load().gdt_matrix_set_schedule(self.handle, int(schedule)), what="gdt_matrix_set_schedule")
        return self

    def _check_qp(self, t):
        if t is None:
            return
        nq = self.source_space.quadrature()[0].shape[0]
        if tuple(t.shape) != (self.grid.num_elements, nq):
            raise ValueError(f"per-quadrature-point coefficient has shape {tuple(t.shape)}, expected "
                             f"({self.grid.num_elements}, {nq})")

    def _diffusion_desc(self, rhs_force=None, dirichlet=False):
        kappa = 1.0
        for f in self.forms:
            if isinstance(f, LocalElementIntegralBilinearForm) and isinstance(f.integrand, LocalLaplaceIntegrand):
                kappa = f.integrand.diffusion
        d = capi.DiffusionDesc()
        if isinstance(kappa, torch.Tensor) and kappa.dim() in (3, 4):
            # a symmetric d x d tensor per element [element, d, d] or per quadrature point [element, q, d, d]
            tt = _f64(kappa.contiguous(), name="diffusion tensor")
            dim = self.grid.dimension
            if tuple(tt.shape[-2:]) != (dim, dim) or tt.shape[0] != self.grid.num_elements:
                raise ValueError(f"diffusion tensor has shape {tuple(tt.shape)}")
            if tt.dim() == 4:
                self._check_qp(tt[..., 0, 0])
            d.kappa, d.kappa_const, d.kappa_qp = None, 0.0, None
            d.kappa_tensor = tt.data_ptr() if tt.dim() == 3 else None
            d.kappa_tensor_qp = tt.data_ptr() if tt.dim() == 4 else None
            keep = [tt]
        else:
            kt, kc, kq = _coef_qp(kappa)
            self._check_qp(kq)
            d.kappa = kt.data_ptr() if kt is not None else None
            d.kappa_const = kc
            d.kappa_qp = kq.data_ptr() if kq is not None else None
            keep = [kt, kq]
        self._keep = keep + _force_fields(d, 1.0 if rhs_force is None else rhs_force, self.source_space)
        d.dirichlet = int(dirichlet)
        return d

    def _ipdg_desc(self, force=0.0):
        kappa, theta, sig_in, sig_bd, wdiff, beta = 1.0, 1.0, 8.0, 14.0, True, None
        g_coupling, g_penalty = None, None
        for f in self.forms:
            if isinstance(f, LocalElementIntegralBilinearForm) and isinstance(f.integrand, LocalLaplaceIntegrand):
                kappa = f.integrand.diffusion
            for t in _terms(getattr(f, "integrand", None)):
                if isinstance(t, LocalLaplaceIPDGInnerCoupling):
                    theta = t.symmetry_prefactor
                    wdiff = t.weight is not None
                if isinstance(t, LocalLaplaceIPDGDirichletCoupling):
                    g_coupling = t.dirichlet_data
                if isinstance(t, LocalIPDGInnerPenalty):
                    sig_in = t.penalty
                    beta = t.beta if t.beta is not None else beta
                if isinstance(t, LocalIPDGBoundaryPenalty):
                    sig_bd = t.penalty
                    beta = t.beta if t.beta is not None else beta
                    g_penalty = t.dirichlet_data
        kt, kc = _coef(kappa)
        ft, fc = _coef(force)
        d = capi.IpdgDesc()
        d.kappa = kt.data_ptr() if kt is not None else None
        d.kappa_const = kc
        d.force = ft.data_ptr() if ft is not None else None
        d.force_const = fc
        d.symmetry_prefactor, d.sigma_inner, d.sigma_boundary, d.weight_is_diffusion = theta, sig_in, sig_bd, int(wdiff)
        d.penalty_beta = 0.0 if beta is None else float(beta)
        # Dirichlet data on the right-hand side (the coupling's unary term, the penalty's counterpart)
        data = [g for g in (g_coupling, g_penalty) if g is not None and not (isinstance(g, (int, float)) and g == 0)]
        if len(data) == 2 and data[0] is not data[1]:
            raise GdtError(capi.EUNSUPPORTED, "the coupling and the penalty take the same Dirichlet data")
        d.dirichlet_rhs = (1 if data and g_coupling is data[0] else 0) | (2 if data and g_penalty is data[0] else 0)
        self._keep_dg = []
        if data:
            g = data[0]
            if isinstance(g, (int, float)):
                d.dirichlet_face, d.dirichlet_const = None, float(g)
            else:
                if isinstance(g, GridFunction):
                    g = g.fn(self.source_space.face_points())
                g = _f64(torch.as_tensor(g, dtype=torch.float64, device=self.ctx.device).contiguous(),
                         self.grid.num_elements * 6, "Dirichlet data")
                d.dirichlet_face, d.dirichlet_const = g.data_ptr(), 0.0
                self._keep_dg.append(g)
        return d

    def assemble(self, parallel=True, rhs=None, force=None, dirichlet=False, dirichlet_values=None):
        """MatrixOperator::assemble; optionally fused with the load vector / Dirichlet constraints.
        dirichlet_values (continuous order 1): a number, a per-DoF tensor or a GridFunction of the
        boundary values; the constrained columns move to the right-hand side."""
        if isinstance(self.source_space, DiscontinuousLagrangeSpace):
            d = self._ipdg_desc(0.0 if force is None else force)
            self.ctx.call("gdt_assemble_swipdg", self.handle, C.byref(d), _ptr(rhs))
        else:
            products = [f for f in self.forms if isinstance(f, LocalElementIntegralBilinearForm)
                        and isinstance(f.integrand, LocalElementProductIntegrand)]
            if products:
                if len(products) != len(self.forms) or len(products) > 1 or rhs is not None or dirichlet:
                    raise GdtError(capi.EUNSUPPORTED, "a product (mass) form is assembled on its own")
                wt, wc, wq = _coef_qp(products[0].integrand.weight)
                self._check_qp(wq)
                if wt is not None and wt.numel() != self.grid.num_elements:
                    raise ValueError(f"weight has {wt.numel()} entries, expected {self.grid.num_elements}")
                pd = capi.ProductDesc()
                pd.weight = wt.data_ptr() if wt is not None else None
                pd.weight_const = wc
                pd.weight_qp = wq.data_ptr() if wq is not None else None
                self.ctx.call("gdt_assemble_cg_product", self.handle, C.byref(pd))
                return self
            d = self._diffusion_desc(force, dirichlet)
            keep = _dirichlet_values(d, dirichlet_values, self.source_space, self.ctx)
            self.ctx.call("gdt_assemble_cg_diffusion", self.handle, C.byref(d), _ptr(rhs))
            del keep
        return self

    def apply(self, source, range=None):
        n, m = self.shape
        _f64(source, m, "source")
        if range is None:
            range = torch.empty(n, dtype=torch.float64, device=self.ctx.device)
        self.ctx.call("gdt_spmv", self.handle, _ptr(source), _ptr(_f64(range, n, "range")))
        return range

    @staticmethod
    def _solver_opts(opts):
        o = capi.SolverOpts()
        o.solver = {"cg": capi.SOLVER_CG, "bicgstab": capi.SOLVER_BICGSTAB}[opts.get("type", "cg")]
        o.precond = {"none": capi.PREC_NONE, "jacobi": capi.PREC_JACOBI, "ilu0": capi.PREC_ILU0}[
            opts.get("precond", "jacobi")]
        o.precision = {"fp64": capi.PRECISION_FP64, "mixed": capi.PRECISION_MIXED}[opts.get("precision", "fp64")]
        o.tol = float(opts.get("tol", 1e-10))
        o.max_iter = int(opts.get("max_iter", 100000))
        o.check_every = int(opts.get("check_every", 0))
        o.inner_tol = float(opts.get("inner_tol", 0.0))
        return o

    def apply_inverse(self, range, source=None, opts=None):
        """Solve A source = range; opts: type ('cg'|'bicgstab'), precond ('jacobi'|'ilu0'|'none'),
        precision ('fp64'|'mixed'), tol (relative residual), max_iter, check_every, inner_tol.

        type 'newton' runs the damped Newton of OperatorInterface::apply_inverse on x -> A x - range
        (keys precision, max_iter, max_dampening_iter as in the reference, and 'jacobian': the linear
        solver options of the defect systems); `source` is the initial guess."""
        opts = dict(opts or {})
        n = self.shape[0]
        _f64(range, n, "range")
        if source is None:
            source = torch.zeros(n, dtype=torch.float64, device=self.ctx.device)
        if opts.get("type") == "newton":
            no = capi.load().gdt_newton_default_opts()
            no.precision = float(opts.get("precision", no.precision))
            no.max_iter = int(opts.get("max_iter", no.max_iter))
            no.max_dampening_iter = int(opts.get("max_dampening_iter", no.max_dampening_iter))
            if "jacobian" in opts:
                no.jacobian_solver = self._solver_opts(dict(opts["jacobian"]))
            ninfo = capi.NewtonInfo()
            self.ctx.call("gdt_newton_solve", self.handle, _ptr(range), _ptr(_f64(source, n, "source")), C.byref(no),
                          C.byref(ninfo))
            self.last_solve_info = {"iterations": ninfo.iterations, "dampening_steps": ninfo.dampening_steps,
                                    "linear_iterations": ninfo.linear_iterations, "residual": ninfo.residual,
                                    "converged": True}
            return source
        o = self._solver_opts(opts)
        info = capi.SolveInfo()
        self.ctx.call("gdt_solve", self.handle, _ptr(range), _ptr(_f64(source, n, "source")), C.byref(o),
                      C.byref(info))
        self.last_solve_info = {"iterations": info.iterations, "refinements": info.refinements,
                                "rel_residual": info.rel_residual, "converged": bool(info.converged)}
        launch = int(capi.load().gdt_context_last_solver_launch(self.ctx.handle))
        if launch:
            self.last_solve_info["launch"] = {capi.SOLVER_LAUNCH_GRAPH: "graph",
                                              capi.SOLVER_LAUNCH_PERSISTENT: "persistent"}[launch]
        if o.precision == capi.PRECISION_MIXED:
            kind = int(capi.load().gdt_matrix_mixed_operator(self.handle))
            self.last_solve_info["inner_operator"] = {0: "stencil", 1: "stencil_tiled", 2: "matrix_free"}.get(kind)
        return source


class LincombOperator:
    """pyMOR's LincombOperator over assembled MatrixOperators that share one space and stencil, as the
    parametric examples build it (python/dune/gdt/gamm-2019-talk-on-conservative-rb.cc:74-95,
    examples/gamm_2019_talk_on_conservative_rb_OS2015_academic_example.py:62-77): the operator at mu is
    sum_q theta_q(mu) A_q. `coefficients` are numbers or callables of mu (parameter functionals).
    `assemble(mu)` forms the combined matrix on the device (one streaming kernel over the values) into
    a MatrixOperator that is reused across parameters; `apply` and `apply_inverse` act on it."""

    def __init__(self, operators, coefficients):
        if not operators or len(operators) != len(coefficients) or len(operators) > 8:
            raise GdtError(capi.EINVAL, "LincombOperator: 1..8 operators, one coefficient each")
        self.operators, self.coefficients = list(operators), list(coefficients)
        op0 = self.operators[0]
        self.ctx = op0.ctx
        self._target = None
        self._mu = object()

    def evaluate_coefficients(self, mu=None):
        return [float(c(mu)) if callable(c) else float(c) for c in self.coefficients]

    def assemble(self, mu=None):
        theta = self.evaluate_coefficients(mu)
        op0 = self.operators[0]
        if self._target is None:
            self._target = MatrixOperator(op0.grid, op0.source_space, op0.range_space, op0.stencil, ctx=self.ctx)
        handles = (C.c_void_p * len(self.operators))(*[op.handle.value for op in self.operators])
        th = (C.c_double * len(theta))(*theta)
        self.ctx.call("gdt_matrix_lincomb", self._target.handle, len(theta), handles, th)
        self._mu = mu
        return self._target

    def apply(self, U, mu=None, range=None):
        return self.assemble(mu).apply(U, range)

    def apply_inverse(self, V, mu=None, source=None, opts=None):
        return self.assemble(mu).apply_inverse(V, source, opts)


def lincomb(vectors, coefficients, out=None):
    """sum_q coefficients[q] vectors[q] over FP64 device vectors of one length (gdt_lincomb)."""
    if not vectors or len(vectors) != len(coefficients) or len(vectors) > 8:
        raise GdtError(capi.EINVAL, "lincomb: 1..8 vectors, one coefficient each")
    n = vectors[0].numel()
    for v in vectors:
        _f64(v, n, "vector")
    if out is None:
        out = torch.empty(n, dtype=torch.float64, device=vectors[0].device)
    ptrs = (C.c_void_p * len(vectors))(*[v.data_ptr() for v in vectors])
    th = (C.c_double * len(coefficients))(*[float(c) for c in coefficients])
    default_context().call("gdt_lincomb", C.c_int64(n), len(vectors), ptrs, th, _ptr(_f64(out, n, "out")))
    return out


def _wrap(ptr, n, dtype, device):
    """Zero-copy CUDA tensor over library-owned device memory (lifetime: the owning handle)."""
    if n == 0:
        return torch.empty(0, dtype=dtype, device=device)
    itemsize = torch.empty((), dtype=dtype).element_size()
    cai = {"shape": (n,), "typestr": {torch.int32: "<i4", torch.int64: "<i8", torch.float64: "<f8",
                                       torch.float32: "<f4"}[dtype],
           "data": (ptr, False), "version": 3, "strides": (itemsize,)}

    class _Holder:
        __cuda_array_interface__ = cai

    return torch.as_tensor(_Holder(), device=device)


class VectorFunctional:
    """make_vector_functional(space) with LocalElementIntegralFunctional(product.with_ansatz(f))."""

    def __init__(self, grid, source_space, ctx: Context | None = None):
        self.grid, self.space = grid, source_space
        self.ctx = ctx or default_context()
        self.forms = []
        self.vector = torch.zeros(source_space.num_DoFs, dtype=torch.float64, device=self.ctx.device)

    def append(self, local_functional):
        self.forms.append(local_functional)
        return self

    __iadd__ = append

    def force(self):
        f = 0.0
        for lf in self.forms:
            if isinstance(lf.integrand, _ProductWithAnsatz):
                f = lf.integrand.function
        return f

    def assemble(self, parallel=True):
        d = capi.DiffusionDesc()
        d.kappa, d.kappa_const = None, 1.0
        keep = _force_fields(d, self.force(), self.space)
        d.dirichlet = 0
        self.ctx.call("gdt_assemble_cg_rhs", self.space.handle, C.byref(d), _ptr(self.vector))
        del keep
        return self


class DirichletConstraints:
    """make_dirichlet_constraints(space, AllDirichletBoundaryInfo) + apply(M, V)."""

    def __init__(self, boundary_info, space, ctx: Context | None = None):
        if boundary_info not in ("dirichlet", "all_dirichlet", None):
            raise GdtError(capi.EUNSUPPORTED, "only the all-Dirichlet boundary info is lowered")
        self.space = space
        self.ctx = ctx or default_context()
        self.applied_in_walk = False

    def apply(self, matrix_operator, vector=None, values=None):
        """DirichletConstraints::apply(M, V); with values (continuous order 1: a number, a per-DoF tensor
        or a GridFunction) the boundary rows get those values and the constrained columns move to V."""
        if self.applied_in_walk:
            return
        if values is None:
            self.ctx.call("gdt_dirichlet_apply", matrix_operator.handle, _ptr(vector))
            return
        d = capi.DiffusionDesc()
        keep = _dirichlet_values(d, values, self.space, self.ctx)
        self.ctx.call("gdt_dirichlet_apply_values", matrix_operator.handle, _ptr(vector), C.c_void_p(d.dirichlet_values),
                      C.c_double(d.dirichlet_value_const))
        del keep


class Walker:
    """XT::Grid::Walker over (MatrixOperator, VectorFunctional, DirichletConstraints): one fused kernel."""

    def __init__(self, grid):
        self.grid = grid
        self.functors = []

    def append(self, functor):
        self.functors.append(functor)
        return self

    def walk(self, thread_parallel=True):
        ops = [f for f in self.functors if isinstance(f, MatrixOperator)]
        funcs = [f for f in self.functors if isinstance(f, VectorFunctional)]
        dcs = [f for f in self.functors if isinstance(f, DirichletConstraints)]
        if len(ops) == 1 and len(funcs) <= 1 and not isinstance(ops[0].source_space, DiscontinuousLagrangeSpace):
            rhs = funcs[0].vector if funcs else None
            force = funcs[0].force() if funcs else None
            # the Dirichlet constraints are applied by DirichletConstraints.apply in the reference;
            # here they are fused into the same pass and apply() becomes a no-op
            ops[0].assemble(rhs=rhs, force=force, dirichlet=bool(dcs))
            for d in dcs:
                d.applied_in_walk = True
            return
        for o in ops:
            o.assemble()
        for f in funcs:
            f.assemble()


class DiscreteFunction:
    def __init__(self, space, vector=None, name="dune.gdt.discretefunction"):
        self.space = space
        self.name = name
        self._vector = vector if vector is not None else torch.zeros(space.num_DoFs, dtype=torch.float64,
                                                                     device=default_context().device)

    def dofs(self):
        return self

    @property
    def vector(self):
        return self._vector


# ---------------------------------------------------------------------------- finite volumes ---
class BurgersFlux:
    """f(u) = u^2/2 (1, ..., 1)"""
    kind = capi.FLUX_BURGERS
    velocity = (0.0, 0.0, 0.0)


class LinearTransportFlux:
    """f(u) = v u"""
    kind = capi.FLUX_TRANSPORT

    def __init__(self, velocity):
        self.velocity = tuple(float(v) for v in velocity) + (0.0,) * (3 - len(velocity))


class NumericalLaxFriedrichsFlux:
    numflux = capi.NUMFLUX_LAX_FRIEDRICHS

    def __init__(self, flux, lambda_=0.0):
        self.flux, self.lf_lambda = flux, float(lambda_)


class NumericalUpwindFlux:
    numflux = capi.NUMFLUX_UPWIND

    def __init__(self, flux):
        self.flux, self.lf_lambda = flux, 0.0


class NumericalEngquistOsherFlux:
    numflux = capi.NUMFLUX_ENGQUIST_OSHER

    def __init__(self, flux):
        self.flux, self.lf_lambda = flux, 0.0


def _fv_desc(numerical_flux):
    d = capi.FvDesc()
    d.flux = numerical_flux.flux.kind
    for i, v in enumerate(numerical_flux.flux.velocity[:3]):
        d.velocity[i] = v
    d.numflux = numerical_flux.numflux
    d.lf_lambda = numerical_flux.lf_lambda
    return d


FV_SIDES = ("-x", "+x", "-y", "+y", "-z", "+z")


class BoundaryTreatmentByCustomExtrapolation:
    """LocalAdvectionFvBoundaryTreatmentByCustomExtrapolationOperator (local/operators/advection-fv.hh:
    307-454) with its extrapolation lowered: the ghost state is the inside state (state=None, outflow)
    or a prescribed state (inflow); the boundary flux is the operator's numerical flux g(u, v, n)."""

    def __init__(self, state=None):
        self.kind = capi.FV_BOUNDARY_EXTRAPOLATE if state is None else capi.FV_BOUNDARY_DIRICHLET
        self.value = 0.0 if state is None else float(state)


class BoundaryTreatmentByCustomNumericalFlux:
    """LocalAdvectionFvBoundaryTreatmentByCustomNumericalFluxOperator (local/operators/advection-fv.hh:
    187-305) with a constant boundary flux g = f.n in the outer normal direction (0: impermeable wall)."""

    def __init__(self, flux=0.0):
        self.kind = capi.FV_BOUNDARY_FLUX
        self.value = float(flux)


class AdvectionFvOperator:
    """AdvectionFvOperator(grid_view, numerical_flux, source_space, range_space): the coupling on inner
    and periodic intersections; `append` adds a boundary treatment on sides of the domain (on a
    periodic grid those sides stop being periodic, as with the reference's periodicity restriction)."""

    def __init__(self, grid, numerical_flux, source_space, range_space=None, ctx: Context | None = None):
        self.grid, self.numerical_flux = grid, numerical_flux
        self.space = source_space
        self.ctx = ctx or default_context()
        self.desc = _fv_desc(numerical_flux)

    def append(self, treatment, filter=None):
        """append(boundary_treatment, filter): filter = the sides ("-x", "+x", "-y", ...) it applies
        to; None: every boundary side of the grid (ApplyOn::BoundaryIntersections)."""
        dim = self.grid.dimension
        sides = FV_SIDES[: 2 * dim] if filter is None else ([filter] if isinstance(filter, str) else list(filter))
        for side in sides:
            if side not in FV_SIDES[: 2 * dim]:
                raise GdtError(capi.EINVAL, f"no side {side!r} on a {dim}D grid")
            k = FV_SIDES.index(side)
            self.desc.boundary[k] = treatment.kind
            self.desc.boundary_value[k] = treatment.value
        return self

    __iadd__ = append

    def apply(self, source, range=None, param=None):
        n = self.space.num_DoFs
        _f64(source, n, "source")
        if range is None:
            range = torch.empty(n, dtype=torch.float64, device=self.ctx.device)
        self.ctx.call("gdt_fv_apply", self.space.handle, C.byref(self.desc), _ptr(source), _ptr(range))
        return range


def estimate_dt_for_hyperbolic_system(grid, state, flux_operator: AdvectionFvOperator):
    dt = C.c_double()
    op = flux_operator
    op.ctx.call("gdt_fv_estimate_dt", op.space.handle, C.byref(op.desc), _ptr(_f64(state, op.space.num_DoFs)),
                C.byref(dt))
    return dt.value


class ExplicitRungeKuttaTimeStepper:
    """ExplicitRungeKuttaTimeStepper(op, initial_values, r=-1) with the explicit Euler or SSP2 tableau.
    `u` may hold a batch of states one after another (independent initial conditions)."""

    def __init__(self, op: AdvectionFvOperator, initial_values, r=-1.0, method="ssp2"):
        if r != -1.0:
            raise GdtError(capi.EUNSUPPORTED, "only r = -1 (u_t + L(u) = 0) is lowered")
        self.op = op
        self.u = initial_values
        self.method = {"ssp2": capi.TIMESTEPPER_SSPRK2, "euler": capi.TIMESTEPPER_EXPLICIT_EULER}[method]
        self.work = torch.empty(0, dtype=torch.float64, device=initial_values.device)
        self.t = 0.0

    def work_doubles(self, nbatch):
        """Size of the work buffer gdt_fv_timestep needs: the SSP2 stage vector and the next state
        (2 N per state), or the next state alone for explicit Euler."""
        n = self.op.space.num_DoFs
        return (2 if self.method == capi.TIMESTEPPER_SSPRK2 else 1) * nbatch * n

    def step(self, dt, steps=1):
        n = self.op.space.num_DoFs
        if self.u.numel() == 0 or self.u.numel() % n:
            raise GdtError(capi.ESHAPE, f"state of {self.u.numel()} values is not a batch of {n}-cell states")
        _f64(self.u, self.u.numel(), "state")
        nbatch = self.u.numel() // n
        if self.work.numel() < self.work_doubles(nbatch):
            self.work = torch.empty(self.work_doubles(nbatch), dtype=torch.float64, device=self.u.device)
        self.op.ctx.call("gdt_fv_timestep", self.op.space.handle, C.byref(self.op.desc), self.method,
                         C.c_double(dt), C.c_int64(steps), C.c_int64(nbatch), _ptr(self.u), _ptr(self.work))
        self.t += dt * steps
        return dt


# ---------------------------------------------------------------------------- adjoint / autograd ---
def dlogkappa(op: MatrixOperator, u, lam, kappa):
    """out[e] = -d/dlog(kappa_e) [lam^T A(kappa) u] for the operator's Laplace (CG) or SWIPDG (DG) forms:
    the log-kappa gradient of J(u(kappa)) when lam solves A^T lam = dJ/du."""
    ne = op.grid.num_elements
    out = torch.empty(ne, dtype=torch.float64, device=op.ctx.device)
    n = op.shape[0]
    _f64(u, n, "u")
    _f64(lam, n, "lam")
    _f64(kappa, ne, "kappa")
    if isinstance(op.source_space, DiscontinuousLagrangeSpace):
        d = op._ipdg_desc()
        d.kappa = kappa.data_ptr()
        op.ctx.call("gdt_swipdg_dlogkappa", op.source_space.handle, C.byref(d), _ptr(u), _ptr(lam), _ptr(out))
    else:
        op.ctx.call("gdt_cg_dlogkappa", op.source_space.handle, _ptr(kappa), _ptr(u), _ptr(lam), _ptr(out))
    return out


class DiffusionProblem:
    """-div(kappa grad u) = f with kappa = exp(log_kappa) per element: continuous P1/Q1 with homogeneous
    Dirichlet constraints, or SWIPDG P1 (sigma_inner, sigma_boundary, theta = 1, weight = kappa)."""

    def __init__(self, grid, dg=False, force=1.0, sigma_inner=8.0, sigma_boundary=14.0, solver_opts=None):
        self.grid = grid
        self.dg = dg
        self.force = force
        self.sigma = (sigma_inner, sigma_boundary)
        self.solver_opts = dict(solver_opts or {"tol": 1e-12})
        if dg:
            self.space = DiscontinuousLagrangeSpace(grid, 1)
            self.op = MatrixOperator(grid, self.space, stencil=Stencil.element_and_intersection)
        else:
            self.space = ContinuousLagrangeSpace(grid, 1)
            self.op = MatrixOperator(grid, self.space)
        self.rhs = torch.zeros(self.space.num_DoFs, dtype=torch.float64, device=self.op.ctx.device)

    def assemble(self, kappa):
        op = self.op
        op.forms = [LocalElementIntegralBilinearForm(LocalLaplaceIntegrand(kappa))]
        if self.dg:
            op.forms += [
                LocalCouplingIntersectionIntegralBilinearForm(
                    LocalLaplaceIPDGInnerCoupling(1.0, kappa, kappa) + LocalIPDGInnerPenalty(self.sigma[0], kappa)),
                LocalIntersectionIntegralBilinearForm(
                    LocalLaplaceIPDGDirichletCoupling(1.0, kappa) + LocalIPDGBoundaryPenalty(self.sigma[1], kappa)),
            ]
            op.assemble(rhs=self.rhs, force=self.force)
        else:
            op.assemble(rhs=self.rhs, force=self.force, dirichlet=True)

    def solve(self, kappa, rhs=None):
        self.assemble(kappa)
        return self.op.apply_inverse(self.rhs if rhs is None else rhs, opts=self.solver_opts)


class DiffusionSolve(torch.autograd.Function):
    """u = solve(A(exp(log_kappa)) u = f). Backward: one adjoint solve A^T lam = grad_u (A is symmetric
    for CG Laplace and SWIPDG with theta = 1) and the element kernel -lam^T dA/dlog(kappa_e) u."""

    @staticmethod
    def forward(ctx, log_kappa, problem: DiffusionProblem):
        kappa = torch.exp(log_kappa.detach()).contiguous()
        u = problem.solve(kappa).clone()
        ctx.problem = problem
        ctx.save_for_backward(kappa, u)
        return u

    @staticmethod
    def backward(ctx, grad_u):
        kappa, u = ctx.saved_tensors
        problem = ctx.problem
        problem.assemble(kappa)  # the operator may have been reassembled since forward
        lam = problem.op.apply_inverse(grad_u.contiguous().to(torch.float64), opts=problem.solver_opts)
        return dlogkappa(problem.op, u, lam, kappa), None


# ------------------------------------------------------------------------------ error norms ---
def element_error(space, u, reference, norm="h1_semi", quad_order=None, ctx: Context | None = None):
    """Element indicators of u - u_ref as the EOC studies' norms (test/stationary-eocstudies/base.hh:259-269):
    eta_e^2 = int_e |grad u - g|^2 ("h1_semi", reference = g at space.quadrature_points(quad_order),
    [element, q, dim]) or int_e (u - v)^2 ("l2", reference [element, q]). Returns (eta2 tensor, total),
    total = sqrt(sum eta2)."""
    ctx = ctx or default_context()
    if quad_order is None:
        quad_order = 2 * space.order + 2
    nq = space.quadrature(quad_order)[0].shape[0]
    ne = space.grid.num_elements
    kind = {"h1_semi": capi.NORM_H1_SEMI, "l2": capi.NORM_L2}[norm]
    shape = (ne, nq, space.grid.dimension) if kind == capi.NORM_H1_SEMI else (ne, nq)
    ref = _f64(reference.contiguous(), name="reference")
    if tuple(ref.shape) != shape:
        raise ValueError(f"reference has shape {tuple(ref.shape)}, expected {shape}")
    _f64(u, space.num_DoFs, "u")
    eta2 = torch.empty(ne, dtype=torch.float64, device=ctx.device)
    total = C.c_double()
    ctx.call("gdt_element_error", space.handle, kind, int(quad_order), _ptr(u), _ptr(ref), _ptr(eta2),
             C.byref(total))
    return eta2, total.value


# ---------------------------------------------------------------------------------- batched ---
class BatchedDiffusion:
    """Many parametric problems -div(kappa grad u) = f on the unit square, one mesh of cells[i]^2
    squares each (sizes may differ), assembled and solved in one persistent launch: continuous P1 on
    the squares split into two triangles (element="p1", element e = 2 cell + t) or continuous Q1 on
    the squares (element="q1", element e = cell), homogeneous Dirichlet. kappa per quadrant of the
    2 x 2 split (`mu`, [n, 4]) or per element (`kappa`, concatenated at `element_offsets`).
    Each problem is solved by a team of threads: the 8 CTAs of a cluster, one CTA or one warp;
    `tune()` times the team kinds per size class and keeps the fastest (the autotuner),
    `set_teams()` sets them by hand."""

    TEAMS = {"cluster": capi.BATCH_TEAM_CLUSTER, "cta": capi.BATCH_TEAM_CTA, "warp": capi.BATCH_TEAM_WARP}

    def __init__(self, cells, ctx: Context | None = None, element="p1"):
        self.ctx = ctx or default_context()
        self.cells = [int(c) for c in cells]
        self.element = element
        kind = {"p1": capi.BATCH_P1_SIMPLEX, "q1": capi.BATCH_Q1_CUBE}[element]
        arr = (C.c_int64 * len(self.cells))(*self.cells)
        h = C.c_void_p()
        self.ctx.call("gdt_batch_create_ex", C.c_int64(len(self.cells)), arr, kind, C.byref(h))
        self.handle = h
        L = capi.load()
        self.total_dofs = int(L.gdt_batch_total_dofs(h))
        self.total_elements = int(L.gdt_batch_total_elements(h))
        off = (C.c_int64 * (len(self.cells) + 1))()
        capi.check(L.gdt_batch_dof_offsets(h, off))
        self.offsets = [int(v) for v in off]
        capi.check(L.gdt_batch_element_offsets(h, off))
        self.element_offsets = [int(v) for v in off]
        self.stencil_width = 7 if element == "p1" else 9

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                capi.load().gdt_batch_destroy(self.handle)
        except Exception:
            pass

    def _kappa(self, mu, kappa):
        if (mu is None) == (kappa is None):
            raise ValueError("give exactly one of mu (per quadrant) and kappa (per element)")
        if mu is not None:
            return _f64(mu.contiguous().reshape(-1), 4 * len(self.cells), "mu"), capi.BATCH_KAPPA_QUADRANTS
        return _f64(kappa.contiguous().reshape(-1), self.total_elements, "kappa"), capi.BATCH_KAPPA_ELEMENTS

    def solve(self, mu=None, force=1.0, precision="fp64", tol=1e-10, max_iter=100000, x=None, keep_stencil=False,
              wait=True, kappa=None):
        """Assemble and solve every problem; raises GdtError(ENAN) when a problem has non-finite data
        (that problem is skipped with x = 0, see status()) or GdtError(ENOCONV) when one did not
        converge; the other problems are solved all the same."""
        k, kind = self._kappa(mu, kappa)
        if x is None:
            x = torch.empty(self.total_dofs, dtype=torch.float64, device=self.ctx.device)
        stencil = (torch.empty(self.total_dofs * self.stencil_width, dtype=torch.float64, device=self.ctx.device)
                   if keep_stencil else None)
        info = capi.BatchInfo()
        prec = {"fp64": capi.PRECISION_FP64, "mixed": capi.PRECISION_MIXED}[precision]
        try:
            self.ctx.call("gdt_batch_solve_ex", self.handle, _ptr(k), kind, C.c_double(force), prec, C.c_double(tol),
                          int(max_iter), _ptr(_f64(x, self.total_dofs, "x")), _ptr(stencil),
                          C.byref(info) if wait else None)
        finally:  # filled also when some problem failed (the others are solved all the same)
            self.last_info = {"max_iterations": info.max_iterations, "min_iterations": info.min_iterations,
                              "max_rel_residual": info.max_rel_residual, "all_converged": bool(info.all_converged),
                              "nonfinite_problems": info.nonfinite_problems}
        return (x, stencil) if keep_stencil else x

    def tune(self, mu=None, force=1.0, precision="fp64", tol=1e-10, max_iter=100000, kappa=None):
        """The autotuner: per size class, the batch solve of that class timed with every allowed team
        kind; the fastest is kept. Returns {cells: {team: ms}} of the timings (teams not tried absent)."""
        k, kind = self._kappa(mu, kappa)
        n = len(self.cells)
        x = torch.empty(self.total_dofs, dtype=torch.float64, device=self.ctx.device)
        nsizes = C.c_int64()
        sizes = (C.c_int64 * n)()
        ms = (C.c_double * (3 * n))()
        prec = {"fp64": capi.PRECISION_FP64, "mixed": capi.PRECISION_MIXED}[precision]
        self.ctx.call("gdt_batch_tune", self.handle, _ptr(k), kind, C.c_double(force), prec, C.c_double(tol),
                      int(max_iter), _ptr(x), C.byref(nsizes), sizes, ms)
        names = {v: name for name, v in self.TEAMS.items()}
        return {int(sizes[c]): {names[t]: ms[3 * c + t] for t in range(3) if ms[3 * c + t] >= 0}
                for c in range(nsizes.value)}

    def teams(self):
        t = (C.c_int * len(self.cells))()
        capi.check(capi.load().gdt_batch_teams(self.handle, t))
        names = {v: name for name, v in self.TEAMS.items()}
        return [names[v] for v in t]

    def set_teams(self, teams):
        """teams: one name ("cluster", "cta", "warp") for all, a list per problem, or {cells: name}."""
        if isinstance(teams, str):
            per = [teams] * len(self.cells)
        elif isinstance(teams, dict):
            cur = self.teams()
            per = [teams.get(c, cur[i]) for i, c in enumerate(self.cells)]
        else:
            per = list(teams)
        arr = (C.c_int * len(self.cells))(*[self.TEAMS[t] for t in per])
        self.ctx.call("gdt_batch_set_teams", self.handle, arr)
        return self

    def iterations(self):
        import numpy as np

        n = len(self.cells)
        it = (C.c_int * n)()
        rr = (C.c_double * n)()
        self.ctx.call("gdt_batch_iterations", self.handle, it, rr)
        return np.array(it[:]), np.array(rr[:])

    def status(self):
        """per-problem status of the last solve: capi.OK, capi.ENOCONV or capi.ENAN"""
        import numpy as np

        st = (C.c_int * len(self.cells))()
        self.ctx.call("gdt_batch_status", self.handle, st)
        return np.array(st[:])

    def unpack(self, x, i):
        return x[self.offsets[i]:self.offsets[i + 1]]
