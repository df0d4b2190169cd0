"""ctypes binding of include/gdt_gb300.h (the C ABI of libgdtgb300.so).

The library is the only compute path: when it is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

SPMV_SCHEDULES = 9
SPMV_SCHEDULE_SELL32 = 8
NORM_H1_SEMI, NORM_L2 = 0, 1
(TIMING_SPMV_FP64, TIMING_SPMV_FP32, TIMING_CG_UPDATE, TIMING_CG_DIRECTION, TIMING_RELIABLE_UPDATE,
 TIMING_MIXED_PERSISTENT) = range(6)
TIMING_KINDS = 8
OK, EINVAL, ESHAPE, ENOCONV, ETIMEOUT, ENAN, EUNSUPPORTED, ECUDA, ENOMEM = range(9)
SPACE_CG, SPACE_DG, SPACE_FV = 0, 1, 2
STENCIL_ELEMENT, STENCIL_INTERSECTION, STENCIL_ELEMENT_AND_INTERSECTION = 0, 1, 2
SOLVER_CG, SOLVER_BICGSTAB = 0, 1
PREC_NONE, PREC_JACOBI, PREC_ILU0 = 0, 1, 2
PRECISION_FP64, PRECISION_MIXED = 0, 1
FLUX_BURGERS, FLUX_TRANSPORT = 0, 1
NUMFLUX_LAX_FRIEDRICHS, NUMFLUX_UPWIND, NUMFLUX_ENGQUIST_OSHER = 0, 1, 2
FV_BOUNDARY_NONE, FV_BOUNDARY_EXTRAPOLATE, FV_BOUNDARY_DIRICHLET, FV_BOUNDARY_FLUX = 0, 1, 2, 3
TIMESTEPPER_EXPLICIT_EULER, TIMESTEPPER_SSPRK2 = 0, 1
MIXED_OPERATOR_STENCIL, MIXED_OPERATOR_STENCIL_TILED, MIXED_OPERATOR_MATRIX_FREE = 0, 1, 2
SOLVER_LAUNCH_AUTO, SOLVER_LAUNCH_GRAPH, SOLVER_LAUNCH_PERSISTENT = 0, 1, 2
BATCH_P1_SIMPLEX, BATCH_Q1_CUBE = 0, 1
BATCH_KAPPA_QUADRANTS, BATCH_KAPPA_ELEMENTS = 0, 1
BATCH_TEAM_CLUSTER, BATCH_TEAM_CTA, BATCH_TEAM_WARP = 0, 1, 2


class DiffusionDesc(C.Structure):
    _fields_ = [("kappa", C.c_void_p), ("kappa_const", C.c_double), ("force", C.c_void_p),
                ("force_const", C.c_double), ("dirichlet", C.c_int), ("kappa_qp", C.c_void_p),
                ("force_qp", C.c_void_p), ("force_quad_order", C.c_int), ("kappa_tensor", C.c_void_p),
                ("kappa_tensor_qp", C.c_void_p), ("dirichlet_values", C.c_void_p),
                ("dirichlet_value_const", C.c_double)]


class ProductDesc(C.Structure):
    _fields_ = [("weight", C.c_void_p), ("weight_const", C.c_double), ("weight_qp", C.c_void_p)]


class IpdgDesc(C.Structure):
    _fields_ = [("kappa", C.c_void_p), ("kappa_const", C.c_double), ("force", C.c_void_p),
                ("force_const", C.c_double), ("symmetry_prefactor", C.c_double), ("sigma_inner", C.c_double),
                ("sigma_boundary", C.c_double), ("weight_is_diffusion", C.c_int), ("penalty_beta", C.c_double),
                ("dirichlet_face", C.c_void_p), ("dirichlet_const", C.c_double), ("dirichlet_rhs", C.c_int)]


class SolverOpts(C.Structure):
    _fields_ = [("solver", C.c_int), ("precond", C.c_int), ("precision", C.c_int), ("tol", C.c_double),
                ("max_iter", C.c_int), ("check_every", C.c_int), ("inner_tol", C.c_double)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("refinements", C.c_int), ("rel_residual", C.c_double),
                ("converged", C.c_int)]


class NewtonOpts(C.Structure):
    _fields_ = [("precision", C.c_double), ("max_iter", C.c_int), ("max_dampening_iter", C.c_int),
                ("jacobian_solver", SolverOpts)]


class NewtonInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("dampening_steps", C.c_int), ("linear_iterations", C.c_int),
                ("residual", C.c_double)]


class FvDesc(C.Structure):
    _fields_ = [("flux", C.c_int), ("velocity", C.c_double * 3), ("numflux", C.c_int), ("lf_lambda", C.c_double),
                ("boundary", C.c_int * 6), ("boundary_value", C.c_double * 6)]


class BatchInfo(C.Structure):
    _fields_ = [("problems", C.c_int64), ("total_dofs", C.c_int64), ("max_iterations", C.c_int),
                ("min_iterations", C.c_int), ("max_rel_residual", C.c_double), ("all_converged", C.c_int),
                ("nonfinite_problems", C.c_int64)]


class GdtError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


# name: (restype, argtypes); every entry point of include/gdt_gb300.h
P = C.c_void_p
_SIGNATURES = {
    "gdt_status_string": (C.c_char_p, [C.c_int]),
    "gdt_context_create": (C.c_int, [C.c_int, P, C.POINTER(P)]),
    "gdt_context_destroy": (C.c_int, [P]),
    "gdt_context_set_stream": (C.c_int, [P, P]),
    "gdt_context_synchronize": (C.c_int, [P]),
    "gdt_context_last_error": (C.c_char_p, [P]),
    "gdt_context_kernel_launches": (C.c_int64, [P]),
    "gdt_context_set_timing": (C.c_int, [P, C.c_int]),
    "gdt_context_set_solver_launch": (C.c_int, [P, C.c_int]),
    "gdt_context_last_solver_launch": (C.c_int, [P]),
    "gdt_context_set_persistent_limits": (C.c_int, [P, C.c_int, C.c_int64]),
    "gdt_context_spmv_timing": (C.c_int, [P, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_double),
                                          C.POINTER(C.c_int64), C.c_int]),
    "gdt_context_kernel_timing": (C.c_int, [P, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.c_int]),
    "gdt_measure_fp64_peak": (C.c_int, [P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "gdt_measure_l2_bandwidth": (C.c_int, [P, C.POINTER(C.c_double)]),
    "gdt_grid_create_cube": (C.c_int, [C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), C.c_int, C.c_int, C.POINTER(P)]),
    "gdt_grid_set_vertices": (C.c_int, [P, P]),
    "gdt_grid_create_simplex_mesh": (C.c_int, [C.c_int, C.c_int64, P, C.c_int64, P, C.POINTER(P)]),
    "gdt_grid_destroy": (C.c_int, [P]),
    "gdt_grid_num_elements": (C.c_int64, [P]),
    "gdt_grid_num_vertices": (C.c_int64, [P]),
    "gdt_space_create": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(P)]),
    "gdt_space_destroy": (C.c_int, [P]),
    "gdt_space_size": (C.c_int64, [P]),
    "gdt_space_max_local_size": (C.c_int, [P]),
    "gdt_space_global_indices": (C.c_int, [P, P, P]),
    "gdt_matrix_create": (C.c_int, [P, P, P, C.c_int, C.POINTER(P)]),
    "gdt_matrix_destroy": (C.c_int, [P]),
    "gdt_matrix_rows": (C.c_int64, [P]),
    "gdt_matrix_cols": (C.c_int64, [P]),
    "gdt_matrix_nnz": (C.c_int64, [P]),
    "gdt_matrix_device_arrays": (C.c_int, [P, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "gdt_matrix_set_zero": (C.c_int, [P, P]),
    "gdt_matrix_tune": (C.c_int, [P, P, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "gdt_matrix_set_schedule": (C.c_int, [P, C.c_int]),
    "gdt_matrix_values_changed": (C.c_int, [P]),
    "gdt_matrix_mixed_operator": (C.c_int, [P]),
    "gdt_assemble_cg_diffusion": (C.c_int, [P, P, C.POINTER(DiffusionDesc), P]),
    "gdt_assemble_cg_rhs": (C.c_int, [P, P, C.POINTER(DiffusionDesc), P]),
    "gdt_dirichlet_apply": (C.c_int, [P, P, P]),
    "gdt_dirichlet_apply_values": (C.c_int, [P, P, P, P, C.c_double]),
    "gdt_assemble_cg_product": (C.c_int, [P, P, C.POINTER(ProductDesc)]),
    "gdt_space_quadrature": (C.c_int, [P, P, P]),
    "gdt_space_quadrature_order": (C.c_int, [P, C.c_int, P, P]),
    "gdt_element_error": (C.c_int, [P, P, C.c_int, C.c_int, P, P, P, C.POINTER(C.c_double)]),
    "gdt_assemble_swipdg": (C.c_int, [P, P, C.POINTER(IpdgDesc), P]),
    "gdt_dg_face_points": (C.c_int, [P, P]),
    "gdt_elliptic_ipdg_sigma": (C.c_double, [C.c_int, C.c_int]),
    "gdt_elliptic_ipdg_beta": (C.c_double, [C.c_int]),
    "gdt_lincomb": (C.c_int, [P, C.c_int64, C.c_int, C.POINTER(P), C.POINTER(C.c_double), P]),
    "gdt_matrix_lincomb": (C.c_int, [P, P, C.c_int, C.POINTER(P), C.POINTER(C.c_double)]),
    "gdt_spmv": (C.c_int, [P, P, P, P]),
    "gdt_solve": (C.c_int, [P, P, P, P, C.POINTER(SolverOpts), C.POINTER(SolveInfo)]),
    "gdt_newton_default_opts": (NewtonOpts, []),
    "gdt_newton_solve": (C.c_int, [P, P, P, P, C.POINTER(NewtonOpts), C.POINTER(NewtonInfo)]),
    "gdt_solve_cg_jacobi_noalloc": (C.c_int, [P, P, P, C.c_int64, P, P, C.c_double, C.c_int, P,
                                              C.POINTER(SolveInfo)]),
    "gdt_fv_apply": (C.c_int, [P, P, C.POINTER(FvDesc), P, P]),
    "gdt_fv_estimate_dt": (C.c_int, [P, P, C.POINTER(FvDesc), P, C.POINTER(C.c_double)]),
    "gdt_fv_timestep": (C.c_int, [P, P, C.POINTER(FvDesc), C.c_int, C.c_double, C.c_int64, C.c_int64, P, P]),
    "gdt_batch_create": (C.c_int, [P, C.c_int64, C.POINTER(C.c_int64), C.POINTER(P)]),
    "gdt_batch_create_ex": (C.c_int, [P, C.c_int64, C.POINTER(C.c_int64), C.c_int, C.POINTER(P)]),
    "gdt_batch_destroy": (C.c_int, [P]),
    "gdt_batch_total_dofs": (C.c_int64, [P]),
    "gdt_batch_total_elements": (C.c_int64, [P]),
    "gdt_batch_dof_offsets": (C.c_int, [P, C.POINTER(C.c_int64)]),
    "gdt_batch_element_offsets": (C.c_int, [P, C.POINTER(C.c_int64)]),
    "gdt_batch_set_teams": (C.c_int, [P, P, C.POINTER(C.c_int)]),
    "gdt_batch_teams": (C.c_int, [P, C.POINTER(C.c_int)]),
    "gdt_batch_solve": (C.c_int, [P, P, P, C.c_double, C.c_int, C.c_double, C.c_int, P, P, P]),
    "gdt_batch_solve_ex": (C.c_int, [P, P, P, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, P, P, P]),
    "gdt_batch_tune": (C.c_int, [P, P, P, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, P,
                                 C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "gdt_batch_iterations": (C.c_int, [P, P, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "gdt_batch_status": (C.c_int, [P, P, C.POINTER(C.c_int)]),
    "gdt_cg_dlogkappa": (C.c_int, [P, P, P, P, P, P]),
    "gdt_swipdg_dlogkappa": (C.c_int, [P, P, C.POINTER(IpdgDesc), P, P, P]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libgdtgb300.so (and bind every C-ABI symbol). Raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(f"libgdtgb300.so not built ({path}); run __graft_entry__.build()")
    L = C.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def symbols():
    return list(_SIGNATURES)


def check(status, ctx=None, what=""):
    if status != OK:
        L = load()
        msg = L.gdt_status_string(status).decode()
        if ctx is not None:
            detail = L.gdt_context_last_error(ctx)
            if detail:
                msg += ": " + detail.decode()
        raise GdtError(status, f"{what}: {msg}" if what else msg)
