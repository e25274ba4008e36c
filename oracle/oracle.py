"""TEST INFRASTRUCTURE ONLY: ctypes loader of the CPU oracle (covof_oracle.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use this
module, and only as the checker / the timed CPU restatement.  Arrays use the
reference layout (ny+2, nx+2), float64, C-contiguous.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libcovof_oracle.so"
_lib = None


def build(force: bool = False) -> Path:
    srcs = [HERE / "covof_oracle.cpp", HERE / "covof_oracle.h", HERE.parent / "include" / "covof_gpu.h"]
    if force or not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in srcs):
        subprocess.run(["make", "-s", "-C", str(HERE)] + (["-B"] if force else []), check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        d, i, v = C.c_double, C.c_int, C.c_void_p
        sig = {
            "orc_hypot": (d, [d, d]),
            "orc_cut_box_area": (d, [d] * 7),
            "orc_compute_alpha": (d, [d] * 7),
            "orc_apply_velocity_bc": (i, [v, v, v, i]),
            "orc_apply_vof_bc": (i, [v, v]),
            "orc_poisson_assemble": (i, [v, d] + [v] * 10),
            "orc_poisson_matvec": (i, [v, d] + [v] * 4),
            "orc_poisson_solve": (i, [v, d] + [v] * 5 + [v, v, i]),
            "orc_poisson_solve_rhs": (i, [v, d] + [v] * 4 + [v, v, i]),
            "orc_poisson_fixed_iters": (i, [v, d] + [v] * 4 + [i, i, v]),
            "orc_project_correct": (i, [v, d] + [v] * 5),
            "orc_momentum_apply": (i, [v, d] + [v] * 10 + [v] * 4 + [i]),
            "orc_momentum_diag": (i, [v, d] + [v] * 8 + [v] * 4 + [i]),
            "orc_momentum_rhs": (i, [v, d] + [v] * 11 + [v, v, i]),
            "orc_predictor": (i, [v, d] + [v] * 10 + [v, v, i] + [v]),
            "orc_sp_step": (i, [v, d] + [v] * 11 + [v, v, i] + [v, v, v]),
            "orc_set_step_threads": (i, [i]),
            "orc_reconstruct": (i, [v, v, v]),
            "orc_wy_step": (i, [v, d, i, v, v, v]),
            "orc_update_physical_properties": (i, [v] * 8),
            "orc_compute_curvature_and_csf": (i, [v] * 7),
            "orc_vof_advect": (i, [v, d, i] + [v] * 13),
            "orc_svof_smooth": (i, [v, v, v]),
            "orc_vof_transport": (i, [v, d, i, v, v, v]),
            "orc_al_step": (i, [v, d] + [v] * 14 + [i, v, v]),
            "orc_mono_step": (i, [v, d] + [v] * 13 + [i, v]),
            "orc_mono_apply": (i, [v, d] + [v] * 16 + [i]),
            "orc_schur_diag": (i, [v, d, v, v, v]),
            "orc_precond_apply": (i, [v, d] + [v] * 16 + [i, v]),
            "orc_prec_blocks": (i, [v, d] + [v] * 10 + [i, v, v]),
            "orc_diffusion_smooth": (i, [v, v, v]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data


def _params(prm):
    return C.byref(prm)


def hypot(x, y): return lib().orc_hypot(x, y)
def cut_box_area(*a): return lib().orc_cut_box_area(*[float(x) for x in a])
def compute_alpha(*a): return lib().orc_compute_alpha(*[float(x) for x in a])


def apply_velocity_bc(prm, u, v, homogeneous=False):
    return lib().orc_apply_velocity_bc(_params(prm), _p(u), _p(v), int(homogeneous))


def apply_vof_bc(prm, Cf):
    return lib().orc_apply_vof_bc(_params(prm), _p(Cf))


def poisson_assemble(prm, dt, u, v, rho_u, rho_v):
    n = prm.nx * prm.ny
    out = [np.zeros(n) for _ in range(6)]
    st = lib().orc_poisson_assemble(_params(prm), dt, _p(u), _p(v), _p(rho_u), _p(rho_v), *[_p(o) for o in out])
    assert st == 0, st
    return [o.reshape(prm.ny, prm.nx) for o in out]


def poisson_matvec(prm, dt, rho_u, rho_v, x):
    y = np.zeros_like(x)
    st = lib().orc_poisson_matvec(_params(prm), dt, _p(rho_u), _p(rho_v), _p(x), _p(y))
    assert st == 0, st
    return y


def poisson_solve(prm, dt, u, v, rho_u, rho_v, p, nthreads=1):
    it, rr = C.c_int(), C.c_double()
    st = lib().orc_poisson_solve(_params(prm), dt, _p(u), _p(v), _p(rho_u), _p(rho_v), _p(p),
                                 C.byref(it), C.byref(rr), nthreads)
    return it.value, rr.value, st


def poisson_solve_rhs(prm, dt, b, rho_u, rho_v, p, nthreads=1):
    it, rr = C.c_int(), C.c_double()
    st = lib().orc_poisson_solve_rhs(_params(prm), dt, _p(b), _p(rho_u), _p(rho_v), _p(p),
                                     C.byref(it), C.byref(rr), nthreads)
    return it.value, rr.value, st


def poisson_fixed_iters(prm, dt, b, rho_u, rho_v, p, n_iter, nthreads=1):
    rr = C.c_double()
    st = lib().orc_poisson_fixed_iters(_params(prm), dt, _p(b), _p(rho_u), _p(rho_v), _p(p),
                                       int(n_iter), int(nthreads), C.byref(rr))
    return rr.value, st


def set_step_threads(n):
    """Host threads of the Poisson solve inside sp_step / time_step (1 by
    default, the reference's serial loop)."""
    st = lib().orc_set_step_threads(int(n))
    assert st == 0, st


def project_correct(prm, dt, u, v, p, rho_u, rho_v):
    return lib().orc_project_correct(_params(prm), dt, _p(u), _p(v), _p(p), _p(rho_u), _p(rho_v))


# Momentum entry points take the time history (u_old, v_old, u_nm1, v_nm1,
# has_nm1; src/module_simulation.f90:508-529), read by Gear / BDF2 and
# Adams-Bashforth only; None leaves it out.
def momentum_apply(prm, dt, xu, xv, u_n, v_n, rho_u, rho_v, mu, mu_node, u_old=None, v_old=None,
                   u_nm1=None, v_nm1=None, has_nm1=0):
    yu, yv = np.zeros_like(xu), np.zeros_like(xv)
    st = lib().orc_momentum_apply(_params(prm), dt, _p(xu), _p(xv), _p(yu), _p(yv), _p(u_n), _p(v_n),
                                  _p(rho_u), _p(rho_v), _p(mu), _p(mu_node), _p(u_old), _p(v_old),
                                  _p(u_nm1), _p(v_nm1), int(has_nm1))
    assert st == 0, st
    return yu, yv


def mono_apply(prm, dt, xu, xv, xp, u_n, v_n, rho_u, rho_v, mu, mu_node, u_old=None, v_old=None,
               u_nm1=None, v_nm1=None, has_nm1=0):
    """The MONOLITHIC operator on (xu, xv, xp); returns (yu, yv, yp)."""
    yu, yv, yp = np.zeros_like(xu), np.zeros_like(xv), np.zeros_like(xp)
    st = lib().orc_mono_apply(_params(prm), dt, _p(xu), _p(xv), _p(xp), _p(yu), _p(yv), _p(yp), _p(u_n),
                              _p(v_n), _p(rho_u), _p(rho_v), _p(mu), _p(mu_node), _p(u_old), _p(v_old),
                              _p(u_nm1), _p(v_nm1), int(has_nm1))
    assert st == 0, st
    return yu, yv, yp


def precond_apply(prm, dt, zu, zv, zp, u_n, v_n, rho_u, rho_v, mu, mu_node, u_old=None, v_old=None,
                  u_nm1=None, v_nm1=None, has_nm1=0, r_al=None):
    """M^-1 of prm.precond on (zu, zv, zp); returns (yu, yv, yp)."""
    yu, yv, yp = np.zeros_like(zu), np.zeros_like(zv), np.zeros_like(zp)
    st = lib().orc_precond_apply(_params(prm), dt, _p(zu), _p(zv), _p(zp), _p(yu), _p(yv), _p(yp), _p(u_n),
                                 _p(v_n), _p(rho_u), _p(rho_v), _p(mu), _p(mu_node), _p(u_old), _p(v_old),
                                 _p(u_nm1), _p(v_nm1), int(has_nm1), _p(r_al))
    assert st == 0, st
    return yu, yv, yp


def prec_blocks(prm, dt, u_n, v_n, rho_u, rho_v, mu, mu_node, u_old=None, v_old=None, u_nm1=None,
                v_nm1=None, has_nm1=0, r_al=None):
    """The sweep preconditioners' stencils: dict block -> dict W/E/S/N/P arrays."""
    shape = u_n.shape
    out = np.zeros((15,) + shape)
    st = lib().orc_prec_blocks(_params(prm), dt, _p(u_n), _p(v_n), _p(rho_u), _p(rho_v), _p(mu), _p(mu_node),
                               _p(u_old), _p(v_old), _p(u_nm1), _p(v_nm1), int(has_nm1), _p(r_al), _p(out))
    assert st == 0, st
    return {b: {c: out[5 * q + k] for k, c in enumerate("WESNP")} for q, b in enumerate("uvs")}


def schur_diag(prm, dt, du, dv):
    dp = np.zeros_like(du)
    st = lib().orc_schur_diag(_params(prm), dt, _p(du), _p(dv), _p(dp))
    assert st == 0, st
    return dp


def momentum_diag(prm, dt, u_n, v_n, rho_u, rho_v, mu, mu_node, u_old=None, v_old=None, u_nm1=None,
                  v_nm1=None, has_nm1=0):
    du, dv = np.zeros_like(u_n), np.zeros_like(v_n)
    st = lib().orc_momentum_diag(_params(prm), dt, _p(u_n), _p(v_n), _p(rho_u), _p(rho_v), _p(mu),
                                 _p(mu_node), _p(du), _p(dv), _p(u_old), _p(v_old), _p(u_nm1), _p(v_nm1),
                                 int(has_nm1))
    assert st == 0, st
    return du, dv


def momentum_rhs(prm, dt, u_n, v_n, rho_u, rho_v, mu_node, fx, fy, u_old, v_old, u_nm1=None, v_nm1=None,
                 has_nm1=0):
    ru, rv = np.zeros_like(u_n), np.zeros_like(v_n)
    st = lib().orc_momentum_rhs(_params(prm), dt, _p(u_n), _p(v_n), _p(rho_u), _p(rho_v), _p(mu_node),
                                _p(fx), _p(fy), _p(u_old), _p(v_old), _p(ru), _p(rv), _p(u_nm1), _p(v_nm1),
                                int(has_nm1))
    assert st == 0, st
    return ru, rv


def predictor(prm, dt, f, has_nm1=0):
    it = C.c_int()
    st = lib().orc_predictor(_params(prm), dt, _p(f.u), _p(f.v), _p(f.rho_u), _p(f.rho_v), _p(f.mu),
                             _p(f.mu_node), _p(f.fx_sigma), _p(f.fy_sigma), _p(f.u_old), _p(f.v_old),
                             _p(f.u_nm1), _p(f.v_nm1), int(has_nm1), C.byref(it))
    return it.value, st


def sp_step(prm, dt, f, has_nm1=0):
    iu, ip, rr = C.c_int(), C.c_int(), C.c_double()
    st = lib().orc_sp_step(_params(prm), dt, _p(f.u), _p(f.v), _p(f.p), _p(f.rho_u), _p(f.rho_v),
                           _p(f.mu), _p(f.mu_node), _p(f.fx_sigma), _p(f.fy_sigma), _p(f.u_old),
                           _p(f.v_old), _p(f.u_nm1), _p(f.v_nm1), int(has_nm1), C.byref(iu), C.byref(ip),
                           C.byref(rr))
    return iu.value, ip.value, rr.value, st


def al_step(prm, dt, f, has_nm1=0):
    """One augmented-Lagrangian step (Uzawa); returns (iters, uzawa_done, status)."""
    it, ud = C.c_int(), C.c_int()
    st = lib().orc_al_step(_params(prm), dt, _p(f.u), _p(f.v), _p(f.p), _p(f.rho), _p(f.rho_u), _p(f.rho_v),
                           _p(f.mu), _p(f.mu_node), _p(f.fx_sigma), _p(f.fy_sigma), _p(f.u_old), _p(f.v_old),
                           _p(f.u_nm1), _p(f.v_nm1), int(has_nm1), C.byref(it), C.byref(ud))
    return it.value, ud.value, st


def reconstruct(prm, Cf):
    seg = np.zeros(Cf.shape + (3,))
    st = lib().orc_reconstruct(_params(prm), _p(Cf), seg.ctypes.data)
    assert st == 0, st
    return seg


def wy_step(prm, dt, x_first, u, v, Cf):
    st = lib().orc_wy_step(_params(prm), dt, int(bool(x_first)), _p(u), _p(v), _p(Cf))
    assert st == 0, st


def vof_transport(prm, dt, x_first, u, v, Cf):
    """The configured transport (Weymouth-Yue / CIAM / TVD) alone."""
    st = lib().orc_vof_transport(_params(prm), dt, int(bool(x_first)), _p(u), _p(v), _p(Cf))
    assert st == 0, st


def svof_smooth(prm, f):
    """smooth_svof_helmholtz: f.C -> f.C_s."""
    st = lib().orc_svof_smooth(_params(prm), _p(f.C), _p(f.C_s))
    assert st == 0, st


def diffusion_smooth(prm, f):
    """vof_smooth_diffusion: f.C -> f.C_tilde."""
    st = lib().orc_diffusion_smooth(_params(prm), _p(f.C), _p(f.C_tilde))
    assert st == 0, st


def update_physical_properties(prm, f):
    st = lib().orc_update_physical_properties(_params(prm), _p(f.C), _p(f.rho), _p(f.rho_u), _p(f.rho_v),
                                              _p(f.mu), _p(f.mu_node), _p(f.C_s))
    assert st == 0, st


def compute_curvature_and_csf(prm, f):
    st = lib().orc_compute_curvature_and_csf(_params(prm), _p(f.C), _p(f.fx_sigma), _p(f.fy_sigma),
                                             _p(f.curvature), _p(f.C_s), _p(f.C_tilde))
    assert st == 0, st


def prepare_interface(prm, f):
    """The interface-derived fields at t = 0, as after advect_vof: C_s
    (SVOF), properties, C_tilde (diffusion smoothing), curvature + CSF."""
    if prm.enable_svof_smoothing:
        svof_smooth(prm, f)
    update_physical_properties(prm, f)
    if prm.enable_diffusion_smoothing:
        diffusion_smooth(prm, f)
    compute_curvature_and_csf(prm, f)


def vof_advect(prm, dt, step_count, f):
    st = lib().orc_vof_advect(_params(prm), dt, int(step_count), _p(f.u), _p(f.v), _p(f.C), _p(f.rho),
                              _p(f.rho_u), _p(f.rho_v), _p(f.mu), _p(f.mu_node), _p(f.fx_sigma),
                              _p(f.fy_sigma), _p(f.curvature), _p(f.C_s), _p(f.C_tilde))
    assert st == 0, st


def mono_step(prm, dt, f, has_nm1=0):
    """One MONOLITHIC step (the coupled u, v, p solve); returns (iters, status)."""
    it = C.c_int()
    st = lib().orc_mono_step(_params(prm), dt, _p(f.u), _p(f.v), _p(f.p), _p(f.rho_u), _p(f.rho_v), _p(f.mu),
                             _p(f.mu_node), _p(f.fx_sigma), _p(f.fy_sigma), _p(f.u_old), _p(f.v_old),
                             _p(f.u_nm1), _p(f.v_nm1), int(has_nm1), C.byref(it))
    return it.value, st


def time_step(prm, dt, step_count, f):
    """One iteration of the time loop body of sim_run (src/module_simulation.f90:
    492-559) for a fixed dt and STANDARD_PROJECTION: the n-1 history
    (u_nm1 = u_old from step 2 on, has_nm1; :508-520), u_old = u, v_old = v;
    advect_vof + apply_velocity_bc when two-phase;
    sim_solve_standard_projection.  step_count counts the steps already
    taken (the reference's step - 1).  Returns (iters_u, iters_p, relres,
    status)."""
    has_nm1 = 1 if step_count > 0 else 0
    if has_nm1:
        f.u_nm1[...] = f.u_old
        f.v_nm1[...] = f.v_old
    else:
        f.u_nm1[...] = f.u
        f.v_nm1[...] = f.v
    f.u_old[...] = f.u
    f.v_old[...] = f.v
    if prm.enable_two_phase:
        vof_advect(prm, dt, step_count, f)
        apply_velocity_bc(prm, f.u, f.v, False)
    if prm.solver_type in (1, 4):  # AUGMENTED_LAGRANGIAN / AAL
        it, ud, st = al_step(prm, dt, f, has_nm1)
        return it, 0, 0.0, st
    if prm.solver_type == 2:  # MONOLITHIC
        it, st = mono_step(prm, dt, f, has_nm1)
        return it, 0, 0.0, st
    return sp_step(prm, dt, f, has_nm1)
