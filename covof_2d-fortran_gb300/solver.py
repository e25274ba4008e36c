"""Host-side mirror of the reference's hot-path subroutines over the C ABI.

Arrays follow the reference layout: a Fortran (0:nx+1, 0:ny+1) array is a
C-contiguous numpy array of shape (ny+2, nx+2) with a[j, i] == f(i, j); the
two are the same bytes.  Method names follow the reference:

* ``sim_solve_standard_projection`` -- src/module_simulation.f90:2424-2666
* ``advect_vof``                    -- src/module_interface_vof.f90:792-825
* ``advect_vof_weymouth_yue``       -- src/module_interface_vof.f90:1162-1377
* ``reconstruct_interface``         -- src/module_interface_reconstruction.f90:580-683
* ``update_physical_properties``    -- src/module_interface_vof.f90:479-616
* ``compute_curvature_and_csf``     -- src/module_interface_vof.f90:627-789

Error behaviour mirrors the reference: a Krylov loop that stops on its
iteration cap or on a breakdown guard still returns its iterate (the status
is returned, not raised); invalid arguments, unsupported options, CUDA errors
and device-side wait timeouts raise CovofError.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .capi import CovofError, Params

_RAISE = {capi.INVALID, capi.UNSUPPORTED, capi.CUDA_ERROR, capi.TIMEOUT}


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
        raise TypeError("fields must be C-contiguous float64 numpy arrays of shape (ny+2, nx+2)")
    return a.ctypes.data


def _dptr(t):
    """Device pointer of a torch CUDA tensor (float64, contiguous) or an int."""
    if t is None:
        return None
    if isinstance(t, int):
        return t
    if not t.is_cuda or not t.is_contiguous():
        raise TypeError("device arguments must be contiguous CUDA tensors")
    return t.data_ptr()


def new_field(p: Params, value: float = 0.0) -> np.ndarray:
    return np.full((p.ny + 2, p.nx + 2), value, dtype=np.float64)


@dataclass
class Fields:
    """The subset of flow_fields_t (src/module_fields.f90:27-92) on the hot path,
    with reset_fields defaults (:232-278)."""
    u: np.ndarray
    v: np.ndarray
    p: np.ndarray
    C: np.ndarray
    rho: np.ndarray
    rho_u: np.ndarray
    rho_v: np.ndarray
    mu: np.ndarray
    mu_node: np.ndarray
    fx_sigma: np.ndarray
    fy_sigma: np.ndarray
    curvature: np.ndarray
    u_old: np.ndarray
    v_old: np.ndarray
    u_nm1: np.ndarray   # velocity of step n-1 (Gear / BDF2, Adams-Bashforth)
    v_nm1: np.ndarray
    C_s: np.ndarray     # SVOF-smoothed indicator
    C_tilde: np.ndarray  # diffusion-smoothed indicator (CSF normals)

    @classmethod
    def allocate(cls, p: Params) -> "Fields":
        z = lambda val=0.0: new_field(p, val)  # noqa: E731
        return cls(u=z(), v=z(), p=z(), C=z(1.0), rho=z(1.0), rho_u=z(1.0), rho_v=z(1.0),
                   mu=z(1.0e-3), mu_node=z(1.0e-3), fx_sigma=z(), fy_sigma=z(), curvature=z(),
                   u_old=z(), v_old=z(), u_nm1=z(), v_nm1=z(), C_s=z(1.0), C_tilde=z(1.0))

    def copy(self) -> "Fields":
        return Fields(**{k: getattr(self, k).copy() for k in self.__dataclass_fields__})


class Solver:
    """One handle (device buffers + stream) for one mesh and parameter set."""

    def __init__(self, params: Params):
        self.lib = capi.load_library()
        self.params = params.copy()
        h = C.c_void_p()
        st = self.lib.covof_create(C.byref(self.params), C.byref(h))
        if st != capi.OK:
            raise CovofError(st, "covof_create")
        self.h = h

    # -- life cycle -----------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.covof_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int, where: str) -> int:
        if st in _RAISE:
            raise CovofError(st, where)
        return st

    @property
    def stream_ptr(self) -> int:
        s = C.c_void_p()
        self.lib.covof_get_stream(self.h, C.byref(s))
        return s.value or 0

    def last_solve_ms(self) -> float:
        ms = C.c_double()
        self.lib.covof_last_solve_ms(self.h, C.byref(ms))
        return ms.value

    def last_refine_steps(self) -> int:
        n = C.c_int()
        self.lib.covof_last_refine_steps(self.h, C.byref(n))
        return n.value

    @property
    def vof_step_count(self) -> int:
        n = C.c_int()
        self.lib.covof_get_vof_step_count(self.h, C.byref(n))
        return n.value

    @vof_step_count.setter
    def vof_step_count(self, n: int):
        self._check(self.lib.covof_set_vof_step_count(self.h, int(n)), "set_vof_step_count")

    # -- time history (Gear / BDF2, Adams-Bashforth) ---------------------------
    @property
    def has_nm1(self) -> int:
        n = C.c_int()
        self._check(self.lib.covof_get_has_nm1(self.h, C.byref(n)), "get_has_nm1")
        return n.value

    @has_nm1.setter
    def has_nm1(self, flag: int):
        self._check(self.lib.covof_set_has_nm1(self.h, int(bool(flag))), "set_has_nm1")

    def _history(self, f: Fields | None, has_nm1):
        """Upload f.u_nm1 / f.v_nm1 and set has_nm1 (when given) before a
        predictor call; the C entry points read the handle's history."""
        if has_nm1 is not None:
            self.has_nm1 = has_nm1
        if f is not None:
            for name in ("u_nm1", "v_nm1"):
                self._check(self.lib.covof_state_set(self.h, capi.FIELD[name], _ptr(getattr(f, name))),
                            "covof_state_set")

    # -- STANDARD_PROJECTION --------------------------------------------------
    def sim_solve_standard_projection(self, dt: float, f: Fields, has_nm1=None):
        """One SP step on host fields; returns (total_iters, poisson_relres, status).
        has_nm1 (with f.u_nm1, f.v_nm1): the n-1 history for Gear / AB2."""
        self._history(f, has_nm1)
        it, rr = C.c_int(), C.c_double()
        st = self.lib.covof_sp_step(self.h, dt, _ptr(f.u), _ptr(f.v), _ptr(f.p), _ptr(f.rho_u),
                                    _ptr(f.rho_v), _ptr(f.mu), _ptr(f.mu_node), _ptr(f.fx_sigma),
                                    _ptr(f.fy_sigma), _ptr(f.u_old), _ptr(f.v_old),
                                    C.byref(it), C.byref(rr))
        return it.value, rr.value, self._check(st, "covof_sp_step")

    def al_step(self, dt: float, f: Fields, has_nm1=None):
        """One augmented-Lagrangian step on host fields; returns
        (predictor iterations, Uzawa iterations, status)."""
        self._history(f, has_nm1)
        it, ud = C.c_int(), C.c_int()
        st = self.lib.covof_al_step(self.h, dt, _ptr(f.u), _ptr(f.v), _ptr(f.p), _ptr(f.rho), _ptr(f.rho_u),
                                    _ptr(f.rho_v), _ptr(f.mu), _ptr(f.mu_node), _ptr(f.fx_sigma),
                                    _ptr(f.fy_sigma), _ptr(f.u_old), _ptr(f.v_old), C.byref(it), C.byref(ud))
        return it.value, ud.value, self._check(st, "covof_al_step")

    def precond_apply(self, dt, zu, zv, zp, u_n, v_n, rho_u, rho_v, mu, mu_node, r_al=None):
        """The Krylov preconditioner M^-1 on host arrays (zp / yp: the
        MONOLITHIC pressure block); returns (yu, yv, yp)."""
        yu, yv, yp = np.zeros_like(zu), np.zeros_like(zv), np.zeros_like(zu)
        st = self.lib.covof_precond_apply(self.h, dt, _ptr(zu), _ptr(zv), _ptr(zp), _ptr(yu), _ptr(yv),
                                          _ptr(yp), _ptr(u_n), _ptr(v_n), _ptr(rho_u), _ptr(rho_v), _ptr(mu),
                                          _ptr(mu_node), _ptr(r_al))
        self._check(st, "covof_precond_apply")
        return yu, yv, yp

    def monolithic_step(self, dt: float, f: Fields, has_nm1=None):
        """One MONOLITHIC step on host fields (the coupled u, v, p solve);
        returns (Krylov iterations, status)."""
        self._history(f, has_nm1)
        it = C.c_int()
        st = self.lib.covof_monolithic_step(self.h, dt, _ptr(f.u), _ptr(f.v), _ptr(f.p), _ptr(f.rho_u),
                                            _ptr(f.rho_v), _ptr(f.mu), _ptr(f.mu_node), _ptr(f.fx_sigma),
                                            _ptr(f.fy_sigma), _ptr(f.u_old), _ptr(f.v_old), C.byref(it))
        return it.value, self._check(st, "covof_monolithic_step")

    def predictor(self, dt: float, f: Fields, has_nm1=None):
        self._history(f, has_nm1)
        it = C.c_int()
        st = self.lib.covof_predictor(self.h, dt, _ptr(f.u), _ptr(f.v), _ptr(f.rho_u), _ptr(f.rho_v),
                                      _ptr(f.mu), _ptr(f.mu_node), _ptr(f.fx_sigma), _ptr(f.fy_sigma),
                                      _ptr(f.u_old), _ptr(f.v_old), C.byref(it))
        return it.value, self._check(st, "covof_predictor")

    def momentum_apply(self, dt, xu, xv, u_n, v_n, rho_u, rho_v, mu, mu_node, u_old=None, v_old=None,
                       u_nm1=None, v_nm1=None, has_nm1=0):
        """A x on host arrays.  u_old .. has_nm1: the history Adams-Bashforth
        and Gear read (uploaded to the resident u_old / v_old / u_nm1 / v_nm1)."""
        for name, a in (("u_old", u_old), ("v_old", v_old), ("u_nm1", u_nm1), ("v_nm1", v_nm1)):
            if a is not None:
                self._check(self.lib.covof_state_set(self.h, capi.FIELD[name], _ptr(a)), "covof_state_set")
        self.has_nm1 = has_nm1
        yu = np.zeros_like(xu)
        yv = np.zeros_like(xv)
        st = self.lib.covof_momentum_apply(self.h, dt, _ptr(xu), _ptr(xv), _ptr(yu), _ptr(yv),
                                           _ptr(u_n), _ptr(v_n), _ptr(rho_u), _ptr(rho_v),
                                           _ptr(mu), _ptr(mu_node))
        self._check(st, "covof_momentum_apply")
        return yu, yv

    def poisson_solve(self, dt, u_star, v_star, rho_u, rho_v, p):
        it, rr = C.c_int(), C.c_double()
        st = self.lib.covof_poisson_solve(self.h, dt, _ptr(u_star), _ptr(v_star), _ptr(rho_u),
                                          _ptr(rho_v), _ptr(p), C.byref(it), C.byref(rr))
        return it.value, rr.value, self._check(st, "covof_poisson_solve")

    def poisson_solve_rhs(self, dt, b, rho_u, rho_v, p):
        it, rr = C.c_int(), C.c_double()
        st = self.lib.covof_poisson_solve_rhs(self.h, dt, _ptr(b), _ptr(rho_u), _ptr(rho_v), _ptr(p),
                                              C.byref(it), C.byref(rr))
        return it.value, rr.value, self._check(st, "covof_poisson_solve_rhs")

    def poisson_apply(self, dt, rho_u, rho_v, x):
        y = np.zeros_like(x)
        st = self.lib.covof_poisson_apply(self.h, dt, _ptr(rho_u), _ptr(rho_v), _ptr(x), _ptr(y))
        self._check(st, "covof_poisson_apply")
        return y

    def project_correct(self, dt, u, v, p, rho_u, rho_v):
        st = self.lib.covof_project_correct(self.h, dt, _ptr(u), _ptr(v), _ptr(p), _ptr(rho_u), _ptr(rho_v))
        self._check(st, "covof_project_correct")

    # device-resident variants (torch CUDA tensors or raw device pointers)
    def poisson_solve_rhs_dev(self, dt, b, rho_u, rho_v, p):
        it, rr = C.c_int(), C.c_double()
        st = self.lib.covof_poisson_solve_rhs_dev(self.h, dt, _dptr(b), _dptr(rho_u), _dptr(rho_v),
                                                  _dptr(p), C.byref(it), C.byref(rr))
        return it.value, rr.value, self._check(st, "covof_poisson_solve_rhs_dev")

    def poisson_solve_dev(self, dt, u_star, v_star, rho_u, rho_v, p):
        it, rr = C.c_int(), C.c_double()
        st = self.lib.covof_poisson_solve_dev(self.h, dt, _dptr(u_star), _dptr(v_star), _dptr(rho_u),
                                              _dptr(rho_v), _dptr(p), C.byref(it), C.byref(rr))
        return it.value, rr.value, self._check(st, "covof_poisson_solve_dev")

    def sp_step_dev(self, dt, u, v, p, rho_u, rho_v, mu, mu_node, fx, fy, u_old, v_old):
        it, rr = C.c_int(), C.c_double()
        st = self.lib.covof_sp_step_dev(self.h, dt, _dptr(u), _dptr(v), _dptr(p), _dptr(rho_u),
                                        _dptr(rho_v), _dptr(mu), _dptr(mu_node), _dptr(fx), _dptr(fy),
                                        _dptr(u_old), _dptr(v_old), C.byref(it), C.byref(rr))
        return it.value, rr.value, self._check(st, "covof_sp_step_dev")

    def vof_advect_dev(self, dt, u, v, Cf, rho, rho_u, rho_v, mu, mu_node, fx, fy, curv):
        st = self.lib.covof_vof_advect_dev(self.h, dt, _dptr(u), _dptr(v), _dptr(Cf), _dptr(rho),
                                           _dptr(rho_u), _dptr(rho_v), _dptr(mu), _dptr(mu_node),
                                           _dptr(fx), _dptr(fy), _dptr(curv))
        return self._check(st, "covof_vof_advect_dev")

    # -- projection and its adjoint ---------------------------------------------
    def projection(self, dt, u_star, v_star, rho_u, rho_v, p):
        """u = u* - dt/rho grad p with p from the Poisson solve; returns (u, v, iters, relres, status)."""
        u, v = u_star.copy(), v_star.copy()
        it, rr = C.c_int(), C.c_double()
        st = self.lib.covof_projection(self.h, dt, _ptr(u_star), _ptr(v_star), _ptr(rho_u), _ptr(rho_v),
                                       _ptr(p), _ptr(u), _ptr(v), C.byref(it), C.byref(rr))
        return u, v, it.value, rr.value, self._check(st, "covof_projection")

    def projection_vjp(self, dt, rho_u, rho_v, p, gu, gv, gp=None):
        """(dL/du*, dL/dv*, dL/d(1/rho_u), dL/d(1/rho_v), iters, relres, status)."""
        out = [np.zeros_like(gu) for _ in range(4)]
        it, rr = C.c_int(), C.c_double()
        st = self.lib.covof_projection_vjp(self.h, dt, _ptr(rho_u), _ptr(rho_v), _ptr(p), _ptr(gu), _ptr(gv),
                                           _ptr(gp), *[_ptr(o) for o in out], C.byref(it), C.byref(rr))
        return (*out, it.value, rr.value, self._check(st, "covof_projection_vjp"))

    def projection_dev(self, dt, u_star, v_star, rho_u, rho_v, p, u, v):
        it, rr = C.c_int(), C.c_double()
        st = self.lib.covof_projection_dev(self.h, dt, _dptr(u_star), _dptr(v_star), _dptr(rho_u),
                                           _dptr(rho_v), _dptr(p), _dptr(u), _dptr(v), C.byref(it), C.byref(rr))
        return it.value, rr.value, self._check(st, "covof_projection_dev")

    def projection_vjp_dev(self, dt, rho_u, rho_v, p, gu, gv, gp, gxu, gxv, gbu, gbv):
        it, rr = C.c_int(), C.c_double()
        st = self.lib.covof_projection_vjp_dev(self.h, dt, _dptr(rho_u), _dptr(rho_v), _dptr(p), _dptr(gu),
                                               _dptr(gv), _dptr(gp), _dptr(gxu), _dptr(gxv), _dptr(gbu),
                                               _dptr(gbv), C.byref(it), C.byref(rr))
        return it.value, rr.value, self._check(st, "covof_projection_vjp_dev")

    def fp64_peak(self) -> float:
        """GFLOP/s of independent FP64 FMA chains on this GPU."""
        g = C.c_double()
        self._check(self.lib.covof_fp64_peak(self.h, C.byref(g)), "covof_fp64_peak")
        return g.value

    # -- geometric VOF ----------------------------------------------------------
    def reconstruct_interface(self, Cf: np.ndarray) -> np.ndarray:
        seg = np.zeros(Cf.shape + (3,), dtype=np.float64)
        st = self.lib.covof_vof_reconstruct(self.h, _ptr(Cf), seg.ctypes.data)
        self._check(st, "covof_vof_reconstruct")
        return seg

    def advect_vof_weymouth_yue(self, dt: float, u, v, Cf, x_first: bool):
        st = self.lib.covof_vof_wy_step(self.h, dt, int(bool(x_first)), _ptr(u), _ptr(v), _ptr(Cf))
        self._check(st, "covof_vof_wy_step")

    def _smoothed(self, f: Fields, upload: bool):
        """Move f.C_s / f.C_tilde to (upload) or from the resident copies the
        property and CSF entry points read, for the enabled smoothings."""
        fn = self.lib.covof_state_set if upload else self.lib.covof_state_get
        for name, on in (("C_s", self.params.enable_svof_smoothing),
                         ("C_tilde", self.params.enable_diffusion_smoothing)):
            if on:
                self._check(fn(self.h, capi.FIELD[name], _ptr(getattr(f, name))), "covof_state_" +
                            ("set" if upload else "get"))

    def advect_vof(self, dt: float, f: Fields):
        st = self.lib.covof_vof_advect(self.h, dt, _ptr(f.u), _ptr(f.v), _ptr(f.C), _ptr(f.rho),
                                       _ptr(f.rho_u), _ptr(f.rho_v), _ptr(f.mu), _ptr(f.mu_node),
                                       _ptr(f.fx_sigma), _ptr(f.fy_sigma), _ptr(f.curvature))
        self._check(st, "covof_vof_advect")
        self._smoothed(f, upload=False)

    def svof_smooth(self, f: Fields):
        """smooth_svof_helmholtz: f.C -> f.C_s."""
        self._check(self.lib.covof_svof_smooth(self.h, _ptr(f.C), _ptr(f.C_s)), "covof_svof_smooth")

    def diffusion_smooth(self, f: Fields):
        """vof_smooth_diffusion: f.C -> f.C_tilde."""
        self._check(self.lib.covof_diffusion_smooth(self.h, _ptr(f.C), _ptr(f.C_tilde)),
                    "covof_diffusion_smooth")

    def apply_velocity_bc(self, f: Fields):
        """apply_velocity_bc (src/module_mpi_comm.f90:290-537): ghosts of f.u, f.v."""
        self._check(self.lib.covof_apply_velocity_bc(self.h, _ptr(f.u), _ptr(f.v)), "covof_apply_velocity_bc")

    def apply_vof_bc(self, f: Fields):
        """apply_vof_bc (src/module_mpi_comm.f90:636-683): ghosts of f.C."""
        self._check(self.lib.covof_apply_vof_bc(self.h, _ptr(f.C)), "covof_apply_vof_bc")

    def update_physical_properties(self, f: Fields):
        self._smoothed(f, upload=True)
        st = self.lib.covof_update_physical_properties(self.h, _ptr(f.C), _ptr(f.rho), _ptr(f.rho_u),
                                                       _ptr(f.rho_v), _ptr(f.mu), _ptr(f.mu_node))
        self._check(st, "covof_update_physical_properties")

    def compute_curvature_and_csf(self, f: Fields):
        self._smoothed(f, upload=True)
        st = self.lib.covof_compute_curvature_and_csf(self.h, _ptr(f.C), _ptr(f.fx_sigma),
                                                      _ptr(f.fy_sigma), _ptr(f.curvature))
        self._check(st, "covof_compute_curvature_and_csf")

    # -- device-resident time stepping ----------------------------------------
    def state_set(self, f: Fields):
        """Upload every resident field from host Fields."""
        for name in capi.FIELD_NAMES:
            self._check(self.lib.covof_state_set(self.h, capi.FIELD[name], _ptr(getattr(f, name))),
                        "covof_state_set")

    def state_get(self, f: Fields):
        """Download every resident field into host Fields."""
        for name in capi.FIELD_NAMES:
            self._check(self.lib.covof_state_get(self.h, capi.FIELD[name], _ptr(getattr(f, name))),
                        "covof_state_get")

    def state_field_dev(self, name: str) -> int:
        """Device address of one resident field."""
        ptr = C.c_void_p()
        self._check(self.lib.covof_state_field_dev(self.h, capi.FIELD[name], C.byref(ptr)),
                    "covof_state_field_dev")
        return ptr.value

    def vtk_write_async(self, out_dir: str, case_name: str, step: int) -> int:
        """Snapshot the resident fields into the reference's .vtr / .pvtr
        files without waiting; returns the previous snapshot's status."""
        return self._check(self.lib.covof_vtk_write_async(self.h, str(out_dir).encode(), case_name.encode(),
                                                          int(step)), "covof_vtk_write_async")

    def vtk_wait(self) -> int:
        return self._check(self.lib.covof_vtk_wait(self.h), "covof_vtk_wait")

    def history_open(self, out_dir: str, case_name: str) -> int:
        return self._check(self.lib.covof_history_open(self.h, str(out_dir).encode(), case_name.encode()),
                           "covof_history_open")

    def history_write_async(self, out_dir: str, case_name: str, step: int, time: float, dt: float) -> int:
        """Append the diagnostics record of the resident fields at this point."""
        return self._check(self.lib.covof_history_write_async(self.h, str(out_dir).encode(), case_name.encode(),
                                                              int(step), float(time), float(dt)),
                           "covof_history_write_async")

    def run_steps(self, dt: float, nsteps: int, graph: bool = True) -> tuple[int, dict]:
        """nsteps time-loop iterations of sim_run (src/module_simulation.f90:492-559)
        on the resident fields; returns (status, run statistics)."""
        stats = capi.RunStats()
        st = self.lib.covof_run_steps(self.h, dt, int(nsteps), capi.RUN_GRAPH if graph else 0,
                                      C.byref(stats))
        return self._check(st, "covof_run_steps"), stats.as_dict()


class Batch:
    """Many independent cases stepped together (covof_batch_*): one entry of
    params per case, uneven mesh sizes allowed."""

    def __init__(self, params_list):
        self.lib = capi.load_library()
        self.params = [p.copy() for p in params_list]
        self.n = len(self.params)
        arr = (Params * self.n)(*self.params)
        h = C.c_void_p()
        st = self.lib.covof_batch_create(arr, self.n, C.byref(h))
        if st != capi.OK:
            raise CovofError(st, "covof_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.covof_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int, where: str) -> int:
        if st in _RAISE:
            raise CovofError(st, where)
        return st

    def set_has_nm1(self, flag: int):
        self._check(self.lib.covof_batch_set_has_nm1(self.h, int(bool(flag))), "covof_batch_set_has_nm1")

    def state_set(self, i: int, f: Fields):
        for name in capi.FIELD_NAMES:
            self._check(self.lib.covof_batch_state_set(self.h, i, capi.FIELD[name], _ptr(getattr(f, name))),
                        "covof_batch_state_set")

    def state_get(self, i: int, f: Fields):
        for name in capi.FIELD_NAMES:
            self._check(self.lib.covof_batch_state_get(self.h, i, capi.FIELD[name], _ptr(getattr(f, name))),
                        "covof_batch_state_get")

    def run_steps(self, dt, nsteps: int, graph: bool = True):
        """nsteps steps of every case (dt: one value per case, or a scalar);
        returns (status, per-case statistics, device ms)."""
        dts = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (self.n,)))
        stats = (capi.RunStats * self.n)()
        ms = C.c_double()
        st = self.lib.covof_batch_run_steps(self.h, dts.ctypes.data_as(C.POINTER(C.c_double)), int(nsteps),
                                            capi.RUN_GRAPH if graph else 0, stats, C.byref(ms))
        return self._check(st, "covof_batch_run_steps"), [x.as_dict() for x in stats], ms.value

    def info(self) -> dict:
        v = [C.c_int() for _ in range(4)]
        self._check(self.lib.covof_batch_info(self.h, *[C.byref(x) for x in v]), "covof_batch_info")
        return dict(zip(("poisson_teams", "poisson_blocks", "predictor_teams", "predictor_blocks"),
                        (x.value for x in v)))

