"""ctypes mirror of include/covof_gpu.h.

Loads the in-tree libcovof_gpu.so.  There is no CPU fallback: if the library
is missing or cannot be loaded, importing the package raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libcovof_gpu.so"
# the bounds-check build (build.py: checked=True) for runs that ask for it
CHECKED_LIB_PATH = PKG / "_build_checked" / "libcovof_gpu.so"

# status codes (include/covof_gpu.h)
OK, MAXITER, BREAKDOWN, NAN, TIMEOUT, UNSUPPORTED, CUDA_ERROR, INVALID, TOO_LARGE = range(9)
STATUS_NAMES = {0: "OK", 1: "MAXITER", 2: "BREAKDOWN", 3: "NAN", 4: "TIMEOUT",
                5: "UNSUPPORTED", 6: "CUDA_ERROR", 7: "INVALID", 8: "TOO_LARGE"}
# codes shared with src/module_constants.f90
BC_DIRICHLET, BC_NEUMANN, BC_PERIODIC, BC_FREESLIP = 1, 2, 3, 4
LINEAR_BICGSTAB2, LINEAR_BICGSTAB, LINEAR_CG = 1, 2, 3
PRECOND_NONE, PRECOND_JACOBI, PRECOND_SSOR, PRECOND_ILU0, PRECOND_BLOCK_TRIANGULAR = 0, 1, 2, 3, 4
CONV_UPWIND, CONV_CENTERED, CONV_TVD_SUPERBEE = 1, 2, 3
TIME_EULER, TIME_GEAR = 1, 2
CONV_LIN_PICARD, CONV_LIN_AB2, CONV_LIN_NEWTON = 1, 2, 3
RECON_PLIC, RECON_ELVIRA = 0, 1
ADVECT_WEYMOUTH_YUE, ADVECT_CIAM, ADVECT_TVD = 0, 1, 2
SOLVER_AUGMENTED_LAGRANGIAN, SOLVER_MONOLITHIC, SOLVER_STANDARD_PROJECTION, SOLVER_AAL, SOLVER_CAAL = 1, 2, 3, 4, 5
LIMITER_SUPERBEE, LIMITER_VAN_LEER, LIMITER_MUSCL, LIMITER_HRIC = 0, 1, 2, 3
GAUGE_REFERENCE, GAUGE_PINNED = 0, 1
PREC_FP64, PREC_MIXED, PREC_FP64_MG = 0, 1, 2
INNER_CHEBYSHEV, INNER_CG, INNER_CHEBYSHEV_STREAM, INNER_MG = 0, 1, 2, 3
# resident fields (COVOF_FIELD_*), in header order; names follow the Fields dataclass
FIELD_NAMES = ("u", "v", "p", "C", "rho", "rho_u", "rho_v", "mu", "mu_node", "fx_sigma",
               "fy_sigma", "curvature", "u_old", "v_old", "u_nm1", "v_nm1", "C_s", "C_tilde")
FIELD = {name: k for k, name in enumerate(FIELD_NAMES)}
RUN_GRAPH = 1


class Params(C.Structure):
    """covof_params (include/covof_gpu.h)."""
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("dx", C.c_double), ("dy", C.c_double),
        ("bc_type", C.c_int * 4), ("bc_u", C.c_double * 4), ("bc_v", C.c_double * 4),
        ("linear_solver", C.c_int), ("precond", C.c_int), ("use_precond", C.c_int),
        ("max_iter", C.c_int), ("tol", C.c_double),
        ("enable_convection", C.c_int), ("convective_scheme", C.c_int),
        ("p_precond", C.c_int), ("p_max_iter", C.c_int), ("p_gauge", C.c_int),
        ("p_precision", C.c_int), ("p_tol", C.c_double), ("p_inner_tol", C.c_double),
        ("p_inner_max_iter", C.c_int), ("p_max_refine", C.c_int),
        ("enable_two_phase", C.c_int), ("enable_surface_tension", C.c_int),
        ("rho1", C.c_double), ("rho2", C.c_double), ("mu1", C.c_double), ("mu2", C.c_double),
        ("sigma", C.c_double), ("gx", C.c_double), ("gy", C.c_double),
        ("recon", C.c_int),
        ("p_inner_kind", C.c_int), ("p_cheb_lo", C.c_double),
        ("p_mg_nu", C.c_int), ("p_mg_cw", C.c_double), ("p_mg_tail", C.c_int),
        ("time_scheme", C.c_int), ("convective_linearization", C.c_int),
        ("enable_svof_smoothing", C.c_int), ("svof_filter_width", C.c_double),
        ("enable_diffusion_smoothing", C.c_int), ("diffusion_smoothing_steps", C.c_int),
        ("advection_method", C.c_int), ("tvd_limiter", C.c_int),
        ("solver_type", C.c_int), ("r_al", C.c_double), ("adaptative_al", C.c_int), ("k_aal", C.c_double),
        ("l0_ref", C.c_double), ("t0_ref", C.c_double), ("u0_ref", C.c_double), ("p0_ref", C.c_double),
        ("ic_radius", C.c_double), ("uzawa_iter", C.c_int), ("uzawa_tol", C.c_double),
        ("p_mg_nuc", C.c_int),
    ]

    def copy(self) -> "Params":
        p = Params()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(Params))
        return p

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


class RunStats(C.Structure):
    """covof_run_stats (include/covof_gpu.h)."""
    _fields_ = [
        ("steps", C.c_int), ("first_bad_step", C.c_int), ("first_bad_status", C.c_int),
        ("graph", C.c_int), ("mom_iters", C.c_longlong), ("poisson_iters", C.c_longlong),
        ("refine_steps", C.c_longlong), ("last_relres", C.c_double), ("max_relres", C.c_double),
        ("ms", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class Launch(C.Structure):
    """covof_launch (include/covof_gpu.h)."""
    _fields_ = [("p_threads", C.c_int), ("p_blocks", C.c_int), ("p_inner_form", C.c_int),
                ("vof_cell_min", C.c_int)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class CovofError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} ({describe(status)})")


_lib = None
_DP = C.POINTER(C.c_double)
_VP = C.c_void_p
_IP = C.POINTER(C.c_int)

# name -> argument types; every function returns int except where noted
_SIGS = {
    "covof_create": [C.POINTER(Params), C.POINTER(C.c_void_p)],
    "covof_destroy": [_VP],
    "covof_abi_version": [],
    "covof_set_wait_budget": [C.c_longlong],
    "covof_bounds_check": [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)],
    "covof_device_info": [_VP, _IP, _IP],
    "covof_get_stream": [_VP, C.POINTER(C.c_void_p)],
    "covof_last_solve_ms": [_VP, _DP],
    "covof_last_refine_steps": [_VP, _IP],
    "covof_get_vof_step_count": [_VP, _IP],
    "covof_set_vof_step_count": [_VP, C.c_int],
    "covof_sp_step": [_VP, C.c_double] + [_VP] * 11 + [_IP, _DP],
    "covof_sp_step_dev": [_VP, C.c_double] + [_VP] * 11 + [_IP, _DP],
    "covof_predictor": [_VP, C.c_double] + [_VP] * 10 + [_IP],
    "covof_predictor_dev": [_VP, C.c_double] + [_VP] * 10 + [_IP],
    "covof_momentum_apply": [_VP, C.c_double] + [_VP] * 10,
    "covof_poisson_solve": [_VP, C.c_double] + [_VP] * 5 + [_IP, _DP],
    "covof_poisson_solve_dev": [_VP, C.c_double] + [_VP] * 5 + [_IP, _DP],
    "covof_poisson_solve_rhs": [_VP, C.c_double] + [_VP] * 4 + [_IP, _DP],
    "covof_poisson_solve_rhs_dev": [_VP, C.c_double] + [_VP] * 4 + [_IP, _DP],
    "covof_poisson_apply": [_VP, C.c_double] + [_VP] * 4,
    "covof_poisson_apply_dev": [_VP, C.c_double] + [_VP] * 4,
    "covof_project_correct": [_VP, C.c_double] + [_VP] * 5,
    "covof_vof_reconstruct": [_VP, _VP, _VP],
    "covof_vof_reconstruct_dev": [_VP, _VP, _VP],
    "covof_vof_wy_step": [_VP, C.c_double, C.c_int, _VP, _VP, _VP],
    "covof_vof_wy_step_dev": [_VP, C.c_double, C.c_int, _VP, _VP, _VP],
    "covof_vof_advect": [_VP, C.c_double] + [_VP] * 11,
    "covof_vof_advect_dev": [_VP, C.c_double] + [_VP] * 11,
    "covof_projection": [_VP, C.c_double] + [_VP] * 7 + [_IP, _DP],
    "covof_projection_dev": [_VP, C.c_double] + [_VP] * 7 + [_IP, _DP],
    "covof_projection_vjp": [_VP, C.c_double] + [_VP] * 10 + [_IP, _DP],
    "covof_projection_vjp_dev": [_VP, C.c_double] + [_VP] * 10 + [_IP, _DP],
    "covof_poisson_solve_rhs_static_dev": [C.POINTER(Params), C.c_double] + [_VP] * 4 + [_IP, _DP],
    "covof_update_physical_properties": [_VP] + [_VP] * 6,
    "covof_compute_curvature_and_csf": [_VP] + [_VP] * 4,
    "covof_apply_velocity_bc": [_VP, _VP, _VP],
    "covof_apply_vof_bc": [_VP, _VP],
    "covof_state_set": [_VP, C.c_int, _VP],
    "covof_state_get": [_VP, C.c_int, _VP],
    "covof_state_field_dev": [_VP, C.c_int, C.POINTER(C.c_void_p)],
    "covof_set_has_nm1": [_VP, C.c_int],
    "covof_svof_smooth": [_VP, _VP, _VP],
    "covof_al_step": [_VP, C.c_double] + [_VP] * 12 + [_IP, _IP],
    "covof_monolithic_step": [_VP, C.c_double] + [_VP] * 11 + [_IP],
    "covof_precond_apply": [_VP, C.c_double] + [_VP] * 13,
    "covof_fp64_peak": [_VP, C.POINTER(C.c_double)],
    "covof_vtk_write_async": [_VP, C.c_char_p, C.c_char_p, C.c_int],
    "covof_vtk_wait": [_VP],
    "covof_history_open": [_VP, C.c_char_p, C.c_char_p],
    "covof_history_write_async": [_VP, C.c_char_p, C.c_char_p, C.c_int, C.c_double, C.c_double],
    "covof_diffusion_smooth": [_VP, _VP, _VP],
    "covof_get_has_nm1": [_VP, C.POINTER(C.c_int)],
    "covof_batch_set_has_nm1": [_VP, C.c_int],
    "covof_run_steps": [_VP, C.c_double, C.c_int, C.c_int, C.POINTER(RunStats)],
    "covof_set_launch": [_VP, C.POINTER(Launch)],
    "covof_get_launch": [_VP, C.POINTER(Launch)],
    "covof_batch_create": [C.POINTER(Params), C.c_int, C.POINTER(C.c_void_p)],
    "covof_batch_destroy": [_VP],
    "covof_batch_state_set": [_VP, C.c_int, C.c_int, _VP],
    "covof_batch_state_get": [_VP, C.c_int, C.c_int, _VP],
    "covof_batch_run_steps": [_VP, _DP, C.c_int, C.c_int, C.POINTER(RunStats), _DP],
    "covof_batch_info": [_VP, _IP, _IP, _IP, _IP],
}


def load_library(path: Path | str | None = None):
    """Load libcovof_gpu.so once; raise if it is absent (no fallback path)."""
    global _lib
    if _lib is not None:
        return _lib
    if path is None and os.environ.get("COVOF_GPU_CHECKED") == "1":
        path = CHECKED_LIB_PATH
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"GB300 library not built ({p} missing): run __graft_entry__.build(); "
            "this package has no CPU fallback")
    lib = C.CDLL(str(p), mode=C.RTLD_GLOBAL)
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.covof_strerror.argtypes = [C.c_int]
    lib.covof_strerror.restype = C.c_char_p
    lib.covof_params_default.argtypes = [C.POINTER(Params), C.c_int, C.c_int, C.c_double, C.c_double]
    lib.covof_params_default.restype = None
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    """Every entry point the header declares (for the export test)."""
    return sorted(list(_SIGS) + ["covof_strerror", "covof_params_default"])


def describe(status: int) -> str:
    try:
        return load_library().covof_strerror(status).decode()
    except Exception:  # library not loadable: fall back to the name only
        return STATUS_NAMES.get(status, str(status))


def default_params(nx: int, ny: int, lx: float, ly: float) -> Params:
    p = Params()
    load_library().covof_params_default(C.byref(p), nx, ny, lx, ly)
    return p


def library_path() -> str:
    return os.fspath(LIB_PATH)
