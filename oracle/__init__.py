"""ORACLE — test infrastructure only.

ctypes bindings of the CPU restatement in ``oracle.cpp`` (see ``oracle.h``). Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import this package; the
product library never loads it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

CG, DG, FV = 0, 1, 2
STENCIL_ELEMENT, STENCIL_INTERSECTION, STENCIL_ELEMENT_AND_INTERSECTION = 0, 1, 2
FORCE_DATA, FORCE_ESV2007 = 0, 1
DIRICHLET_CONST, DIRICHLET_TEST = 0, 1
SOLVER_CG, SOLVER_BICGSTAB = 0, 1
PREC_NONE, PREC_JACOBI, PREC_ILU0 = 0, 1, 2
FLUX_BURGERS, FLUX_TRANSPORT = 0, 1
NUMFLUX_LAX_FRIEDRICHS, NUMFLUX_UPWIND, NUMFLUX_ENGQUIST_OSHER = 0, 1, 2


def build(verbose: bool = False) -> str:
    """Compile liboracle.so with g++ (portable flags: the same source builds on x86-64 and aarch64)."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    src = os.path.join(HERE, "oracle.cpp")
    deps = [src, os.path.join(HERE, "fem.hpp"), os.path.join(HERE, "oracle.h")]
    if os.path.exists(LIB_PATH) and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(d) for d in deps):
        return LIB_PATH
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", src, "-o", LIB_PATH]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return LIB_PATH


class Grid(C.Structure):
    _fields_ = [
        ("dim", C.c_int),
        ("n", C.c_long * 3),
        ("lo", C.c_double * 3),
        ("hi", C.c_double * 3),
        ("simplex", C.c_int),
        ("periodic", C.c_int),
        ("vertices", C.c_void_p),
    ]


def grid(dim, n, lo=0.0, hi=1.0, simplex=False, periodic=False, vertices=None) -> Grid:
    """vertices: optional coordinates [vertex, dim] (vertices lexicographic, x fastest) of a mapped grid;
    the array is kept alive by the returned structure."""
    g = Grid()
    g.dim = dim
    ns = list(n) if hasattr(n, "__len__") else [n] * dim
    los = list(lo) if hasattr(lo, "__len__") else [lo] * dim
    his = list(hi) if hasattr(hi, "__len__") else [hi] * dim
    for i in range(3):
        g.n[i] = ns[i] if i < dim else 1
        g.lo[i] = los[i] if i < dim else 0.0
        g.hi[i] = his[i] if i < dim else 1.0
    g.simplex = int(bool(simplex))
    g.periodic = int(bool(periodic))
    if vertices is not None:
        import numpy as np

        xv = np.ascontiguousarray(vertices, dtype=np.float64)
        g._vertices = xv  # keeps the buffer alive
        g.vertices = xv.ctypes.data
    else:
        g.vertices = None
    return g


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        dp, lp, ip = P(C.c_double), P(C.c_int64), P(C.c_int32)
        g = P(Grid)
        sig = {
            "orc_set_threads": (None, [C.c_int]),
            "orc_max_threads": (C.c_int, []),
            "orc_num_elements": (C.c_long, [g]),
            "orc_space_size": (C.c_long, [g, C.c_int, C.c_int]),
            "orc_local_size": (C.c_int, [g, C.c_int, C.c_int]),
            "orc_global_indices": (C.c_int, [g, C.c_int, C.c_int, lp]),
            "orc_dirichlet_dofs": (C.c_long, [g, C.c_int, lp]),
            "orc_pattern": (C.c_void_p, [g, C.c_int, C.c_int, C.c_int]),
            "orc_csr_rows": (C.c_long, [C.c_void_p]),
            "orc_csr_nnz": (C.c_long, [C.c_void_p]),
            "orc_csr_export": (None, [C.c_void_p, lp, ip, dp]),
            "orc_csr_import": (C.c_void_p, [C.c_long, lp, ip, dp]),
            "orc_csr_free": (None, [C.c_void_p]),
            "orc_assemble_cg": (C.c_void_p, [g, C.c_int, dp, C.c_double, dp, C.c_double, C.c_int, C.c_int, C.c_int, dp]),
            "orc_assemble_cg_tensor": (C.c_void_p, [g, C.c_int, dp, dp, C.c_double, C.c_int, dp]),
            "orc_assemble_mass": (C.c_void_p, [g, C.c_int, C.c_int]),
            "orc_assemble_swipdg": (C.c_void_p, [g, C.c_int, dp, C.c_double, dp, C.c_double, C.c_int, C.c_int,
                                                 C.c_double, C.c_double, C.c_double, C.c_int, dp]),
            "orc_assemble_swipdg_data": (C.c_void_p, [g, C.c_int, dp, C.c_double, dp, C.c_double, C.c_int, C.c_int,
                                                      C.c_double, C.c_double, C.c_double, C.c_int, C.c_double,
                                                      C.c_int, C.c_double, C.c_int, dp]),
            "orc_swipdg_dlogkappa": (None, [g, C.c_int, dp, C.c_double, C.c_double, C.c_double, dp, dp, dp]),
            "orc_cg_dlogkappa": (None, [g, C.c_int, dp, dp, dp, dp]),
            "orc_spmv": (None, [C.c_void_p, dp, dp]),
            "orc_solve": (C.c_int, [C.c_void_p, dp, dp, C.c_int, C.c_int, C.c_double, C.c_int, P(C.c_int), dp]),
            "orc_h1_semi_error_esv2007": (C.c_double, [g, C.c_int, C.c_int, dp]),
            "orc_l2_norm": (C.c_double, [g, C.c_int, C.c_int, dp]),
            "orc_fv_estimate_dt": (C.c_double, [g, C.c_int, dp, dp]),
            "orc_fv_apply": (None, [g, C.c_int, dp, C.c_int, C.c_double, dp, dp, ip, dp]),
            "orc_fv_explicit_euler": (None, [g, C.c_int, dp, C.c_int, C.c_double, dp, C.c_double, C.c_long, ip,
                                             dp]),
            "orc_fv_ssprk2": (None, [g, C.c_int, dp, C.c_int, C.c_double, dp, C.c_double, C.c_long, ip, dp]),
            "orc_mesh_assemble": (C.c_void_p, [C.c_int, C.c_long, dp, C.c_long, lp, dp, C.c_double, dp, C.c_double,
                                               C.c_int, dp]),
            "orc_mesh_boundary": (C.c_long, [C.c_int, C.c_long, C.c_long, lp, lp]),
            "orc_mesh_assemble_swipdg": (C.c_void_p, [C.c_long, dp, C.c_long, lp, dp, C.c_double, dp, C.c_double,
                                                      C.c_double, C.c_double, C.c_double, C.c_int, C.c_double,
                                                      C.c_int, C.c_double, C.c_int, dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _dp(a):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _lp(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return int(lib().orc_max_threads())


class CSR:
    """Owned copy of an oracle CSR matrix (row_ptr int64, col int32, val float64)."""

    def __init__(self, handle):
        L = lib()
        n = L.orc_csr_rows(handle)
        nnz = L.orc_csr_nnz(handle)
        self.row_ptr = np.empty(n + 1, np.int64)
        self.col = np.empty(nnz, np.int32)
        self.val = np.empty(nnz, np.float64)
        L.orc_csr_export(handle, _lp(self.row_ptr), _ip(self.col), _dp(self.val))
        L.orc_csr_free(handle)
        self.n = n

    @property
    def nnz(self):
        return len(self.col)

    def handle(self):
        return lib().orc_csr_import(self.n, _lp(self.row_ptr), _ip(self.col), _dp(self.val))

    def to_scipy(self):
        import scipy.sparse as sp

        return sp.csr_matrix((self.val, self.col, self.row_ptr), shape=(self.n, self.n))

    def dense(self):
        return self.to_scipy().toarray()


def space_size(g, kind, order):
    return int(lib().orc_space_size(C.byref(g), kind, order))


def num_elements(g):
    return int(lib().orc_num_elements(C.byref(g)))


def global_indices(g, kind, order):
    ls = lib().orc_local_size(C.byref(g), kind, order)
    out = np.empty(num_elements(g) * ls, np.int64)
    lib().orc_global_indices(C.byref(g), kind, order, _lp(out))
    return out.reshape(-1, ls)


def mesh_assemble(coords, cells, kappa=None, kappa_const=1.0, force=None, force_const=1.0, dirichlet=True):
    """P1 stiffness + load vector on an unstructured simplex mesh (coords [nv, dim], cells [ne, dim + 1])."""
    x = np.ascontiguousarray(coords, dtype=np.float64)
    c = np.ascontiguousarray(cells, dtype=np.int64)
    rhs = np.zeros(x.shape[0])
    kap = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
    frc = None if force is None else np.ascontiguousarray(force, dtype=np.float64)
    h = lib().orc_mesh_assemble(x.shape[1], x.shape[0], _dp(x), c.shape[0], _lp(c), _dp(kap), kappa_const, _dp(frc),
                                force_const, int(dirichlet), _dp(rhs))
    return CSR(h), rhs


def mesh_assemble_swipdg(coords, cells, kappa=None, kappa_const=1.0, force=None, force_const=1.0, theta=1.0,
                         sigma_inner=8.0, sigma_boundary=14.0, weight_is_diffusion=True, beta=1.0,
                         dirichlet_fn=DIRICHLET_CONST, dirichlet_const=0.0, dirichlet_rhs=0):
    """SWIPDG (DG P1) matrix + right-hand side on a triangle mesh (coords [nv, 2], cells [ne, 3])."""
    x = np.ascontiguousarray(coords, dtype=np.float64)
    c = np.ascontiguousarray(cells, dtype=np.int64)
    rhs = np.zeros(3 * c.shape[0])
    kap = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
    frc = None if force is None else np.ascontiguousarray(force, dtype=np.float64)
    h = lib().orc_mesh_assemble_swipdg(x.shape[0], _dp(x), c.shape[0], _lp(c), _dp(kap), kappa_const, _dp(frc),
                                       force_const, theta, sigma_inner, sigma_boundary, int(weight_is_diffusion),
                                       float(beta), int(dirichlet_fn), float(dirichlet_const), int(dirichlet_rhs),
                                       _dp(rhs))
    return CSR(h), rhs


def mesh_boundary(num_vertices, cells):
    c = np.ascontiguousarray(cells, dtype=np.int64)
    dim = c.shape[1] - 1
    n = lib().orc_mesh_boundary(dim, num_vertices, c.shape[0], _lp(c), None)
    out = np.empty(n, np.int64)
    lib().orc_mesh_boundary(dim, num_vertices, c.shape[0], _lp(c), _lp(out))
    return out


def dirichlet_dofs(g, order):
    n = lib().orc_dirichlet_dofs(C.byref(g), order, None)
    out = np.empty(n, np.int64)
    lib().orc_dirichlet_dofs(C.byref(g), order, _lp(out))
    return out


def pattern(g, kind, order, stencil):
    return CSR(lib().orc_pattern(C.byref(g), kind, order, stencil))


def assemble_cg(g, order=1, kappa=None, kappa_const=1.0, force=None, force_const=1.0, force_fn=FORCE_DATA,
                force_order=0, dirichlet=True):
    n = space_size(g, CG, order)
    rhs = np.zeros(n)
    kap = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
    frc = None if force is None else np.ascontiguousarray(force, dtype=np.float64)
    h = lib().orc_assemble_cg(C.byref(g), order, _dp(kap), kappa_const, _dp(frc), force_const, force_fn,
                              force_order, int(dirichlet), _dp(rhs))
    return CSR(h), rhs


def assemble_cg_tensor(g, order, kappa_tensor, force=None, force_const=1.0, dirichlet=True):
    """Laplace stiffness with a d x d diffusion tensor per element ([element, d, d]) + load vector."""
    n = space_size(g, CG, order)
    rhs = np.zeros(n)
    kt = np.ascontiguousarray(kappa_tensor, dtype=np.float64)
    frc = None if force is None else np.ascontiguousarray(force, dtype=np.float64)
    h = lib().orc_assemble_cg_tensor(C.byref(g), order, _dp(kt), _dp(frc), force_const, int(dirichlet), _dp(rhs))
    return CSR(h), rhs


def assemble_mass(g, kind, order):
    return CSR(lib().orc_assemble_mass(C.byref(g), kind, order))


def assemble_swipdg(g, order=1, kappa=None, kappa_const=1.0, force=None, force_const=1.0, force_fn=FORCE_DATA,
                    force_order=0, theta=1.0, sigma_inner=8.0, sigma_boundary=14.0, weight_is_diffusion=True,
                    beta=1.0, dirichlet_fn=DIRICHLET_CONST, dirichlet_const=0.0, dirichlet_rhs=0):
    """SWIPDG matrix + right-hand side; beta: penalty length |I|^beta; dirichlet_rhs: bit 0 the unary
    DirichletCoupling term, bit 1 the boundary penalty weight times g (g = dirichlet_const, or the test
    function cos(pi x / 2) cos(pi y / 2) + 0.3 x with dirichlet_fn = DIRICHLET_TEST)."""
    n = space_size(g, DG, order)
    rhs = np.zeros(n)
    kap = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
    frc = None if force is None else np.ascontiguousarray(force, dtype=np.float64)
    h = lib().orc_assemble_swipdg_data(C.byref(g), order, _dp(kap), kappa_const, _dp(frc), force_const, force_fn,
                                       force_order, theta, sigma_inner, sigma_boundary, int(weight_is_diffusion),
                                       float(beta), int(dirichlet_fn), float(dirichlet_const), int(dirichlet_rhs),
                                       _dp(rhs))
    return CSR(h), rhs


def swipdg_dlogkappa(g, kappa, u, lam, order=1, theta=1.0, sigma_inner=8.0, sigma_boundary=14.0):
    out = np.empty(num_elements(g))
    k = np.ascontiguousarray(kappa, np.float64)
    lib().orc_swipdg_dlogkappa(C.byref(g), order, _dp(k), theta, sigma_inner, sigma_boundary,
                               _dp(np.ascontiguousarray(u, np.float64)), _dp(np.ascontiguousarray(lam, np.float64)),
                               _dp(out))
    return out


def cg_dlogkappa(g, kappa, u, lam, order=1):
    out = np.empty(num_elements(g))
    lib().orc_cg_dlogkappa(C.byref(g), order, _dp(np.ascontiguousarray(kappa, np.float64)),
                           _dp(np.ascontiguousarray(u, np.float64)), _dp(np.ascontiguousarray(lam, np.float64)),
                           _dp(out))
    return out


def spmv(A: CSR, x):
    h = A.handle()
    y = np.empty(A.n)
    lib().orc_spmv(h, _dp(np.ascontiguousarray(x, np.float64)), _dp(y))
    lib().orc_csr_free(h)
    return y


def solve(A: CSR, b, x0=None, solver=SOLVER_CG, prec=PREC_JACOBI, tol=1e-10, max_iter=100000):
    h = A.handle()
    x = np.zeros(A.n) if x0 is None else np.array(x0, dtype=np.float64)
    it = C.c_int(0)
    rr = C.c_double(0)
    st = lib().orc_solve(h, _dp(np.ascontiguousarray(b, np.float64)), _dp(x), solver, prec, tol, max_iter,
                         C.byref(it), C.byref(rr))
    lib().orc_csr_free(h)
    return x, int(it.value), float(rr.value), int(st)


def h1_semi_error_esv2007(g, kind, order, u):
    return float(lib().orc_h1_semi_error_esv2007(C.byref(g), kind, order, _dp(np.ascontiguousarray(u, np.float64))))


def l2_norm(g, kind, order, u):
    return float(lib().orc_l2_norm(C.byref(g), kind, order, _dp(np.ascontiguousarray(u, np.float64))))


def _vel(v):
    a = np.zeros(3)
    if v is not None:
        a[: len(v)] = v
    return a


def fv_estimate_dt(g, flux, u0, velocity=None):
    return float(lib().orc_fv_estimate_dt(C.byref(g), flux, _dp(_vel(velocity)),
                                          _dp(np.ascontiguousarray(u0, np.float64))))


def _boundary(boundary, boundary_value):
    """(kinds, values) per side (-x, +x, -y, +y, -z, +z) as C arrays, or (None, None)"""
    if boundary is None:
        return None, None
    kinds = (C.c_int * 6)(*([int(k) for k in boundary] + [0] * (6 - len(boundary))))
    vals = list(boundary_value) if boundary_value is not None else []
    values = (C.c_double * 6)(*([float(v) for v in vals] + [0.0] * (6 - len(vals))))
    return kinds, C.cast(values, C.POINTER(C.c_double))


def fv_apply(g, flux, numflux, u, velocity=None, lf_lambda=0.0, boundary=None, boundary_value=None):
    out = np.empty(len(u))
    bk, bv = _boundary(boundary, boundary_value)
    lib().orc_fv_apply(C.byref(g), flux, _dp(_vel(velocity)), numflux, lf_lambda,
                       _dp(np.ascontiguousarray(u, np.float64)), _dp(out), bk, bv)
    return out


def fv_explicit_euler(g, flux, numflux, u, dt, steps, velocity=None, lf_lambda=0.0, boundary=None,
                      boundary_value=None):
    x = np.array(u, dtype=np.float64)
    bk, bv = _boundary(boundary, boundary_value)
    lib().orc_fv_explicit_euler(C.byref(g), flux, _dp(_vel(velocity)), numflux, lf_lambda, _dp(x), dt, steps, bk,
                                bv)
    return x


def fv_ssprk2(g, flux, numflux, u, dt, steps, velocity=None, lf_lambda=0.0, boundary=None, boundary_value=None):
    x = np.array(u, dtype=np.float64)
    bk, bv = _boundary(boundary, boundary_value)
    lib().orc_fv_ssprk2(C.byref(g), flux, _dp(_vel(velocity)), numflux, lf_lambda, _dp(x), dt, steps, bk, bv)
    return x
