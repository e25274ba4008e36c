/*
 * covof_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement (FP64, serial, -ffp-contract=off) of the COVOF 2D reference
 * hot path, used as the parity checker for the GPU library.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline legs may load it; the
 * product path never links or calls it.
 *
 * Parity status: the reference (Fortran 2018 + MPI) cannot be compiled on
 * these machines (no Fortran compiler, no MPI), and it ships no golden
 * vectors.  The restatement is pinned by the reference's own documented
 * acceptance checks (vortex-shear volume conservation |dV|/V0 < 1e-12,
 * README.md:219; Laplacian Krylov accuracy), by known-answer tests derived
 * from the algorithms' mathematics, and by structural invariants; element
 * values of the SP step are otherwise "parity unpinned" against the
 * reference binary.
 *
 * One deliberate deviation: the reference calls the Fortran intrinsic
 * hypot (libm), which is not correctly rounded and differs between x86-64
 * and aarch64 builds.  The oracle and the GPU both use covof_hypot(), a
 * fused (FMA-corrected) hypot, so that both sides compute identical bits.
 *
 * All arrays use the reference layout (0:nx+1, 0:ny+1), i fastest.
 */
#ifndef COVOF_ORACLE_H
#define COVOF_ORACLE_H
#include "../include/covof_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

double orc_hypot(double x, double y);
double orc_cut_box_area(double xmin, double xmax, double ymin, double ymax,
                        double nx, double ny, double alpha);
double orc_compute_alpha(double xmin, double xmax, double ymin, double ymax,
                         double nx, double ny, double c_target);

/* velocity / VOF ghost conditions (np = 1) */
int orc_apply_velocity_bc(const covof_params* prm, double* u, double* v, int homogeneous);
int orc_apply_vof_bc(const covof_params* prm, double* C);

/* Poisson (SP section of sim_solve_standard_projection) */
int orc_poisson_assemble(const covof_params* prm, double dt, const double* u_star,
                         const double* v_star, const double* rho_u, const double* rho_v,
                         double* aW, double* aE, double* aS, double* aN, double* aP,
                         double* b);
int orc_poisson_matvec(const covof_params* prm, double dt, const double* rho_u,
                       const double* rho_v, const double* x, double* y);
int orc_poisson_solve(const covof_params* prm, double dt, const double* u_star,
                      const double* v_star, const double* rho_u, const double* rho_v,
                      double* p, int* iters, double* relres, int nthreads);
int orc_poisson_solve_rhs(const covof_params* prm, double dt, const double* b,
                          const double* rho_u, const double* rho_v, double* p, int* iters,
                          double* relres, int nthreads);
/* Timing helper for the CPU baseline: run exactly n_iter Jacobi-PCG
 * iterations (no convergence exit) on the explicit-RHS system. */
int orc_poisson_fixed_iters(const covof_params* prm, double dt, const double* b,
                            const double* rho_u, const double* rho_v, double* p, int n_iter,
                            int nthreads, double* relres);
int orc_project_correct(const covof_params* prm, double dt, double* u, double* v,
                        const double* p, const double* rho_u, const double* rho_v);

/* momentum predictor */
/* The momentum entry points take the time history: u_old / v_old
 * (fields%u_old), u_nm1 / v_nm1 and has_nm1 (src/module_simulation.f90:
 * 508-529), read by Gear / BDF2 and Adams-Bashforth only. */
int orc_momentum_apply(const covof_params* prm, double dt, const double* xu, const double* xv,
                       double* yu, double* yv, const double* u_n, const double* v_n,
                       const double* rho_u, const double* rho_v, const double* mu,
                       const double* mu_node, const double* u_old, const double* v_old,
                       const double* u_nm1, const double* v_nm1, int has_nm1);
int orc_mono_apply(const covof_params* prm, double dt, const double* xu, const double* xv, const double* xp,
                   double* yu, double* yv, double* yp, const double* u_n, const double* v_n,
                   const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                   const double* u_old, const double* v_old, const double* u_nm1, const double* v_nm1,
                   int has_nm1);
int orc_schur_diag(const covof_params* prm, double dt, const double* du, const double* dv, double* dp);
/* the SSOR / BLOCK_TRIANGULAR stencils: 15 arrays (u, v, Schur; W E S N P) */
int orc_prec_blocks(const covof_params* prm, double dt, const double* u_n, const double* v_n,
                    const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                    const double* u_old, const double* v_old, const double* u_nm1, const double* v_nm1,
                    int has_nm1, const double* r_al, double* out);
/* the Krylov preconditioner M^-1 of prm->precond on (zu, zv, zp) (zp, yp:
 * MONOLITHIC only); r_al: the AL penalty field or NULL */
int orc_precond_apply(const covof_params* prm, double dt, const double* zu, const double* zv, const double* zp,
                      double* yu, double* yv, double* yp, const double* u_n, const double* v_n,
                      const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                      const double* u_old, const double* v_old, const double* u_nm1, const double* v_nm1,
                      int has_nm1, const double* r_al);
int orc_momentum_diag(const covof_params* prm, double dt, const double* u_n, const double* v_n,
                      const double* rho_u, const double* rho_v, const double* mu,
                      const double* mu_node, double* diag_u, double* diag_v, const double* u_old,
                      const double* v_old, const double* u_nm1, const double* v_nm1, int has_nm1);
int orc_momentum_rhs(const covof_params* prm, double dt, const double* u_n, const double* v_n,
                     const double* rho_u, const double* rho_v, const double* mu_node,
                     const double* fx_sigma, const double* fy_sigma, const double* u_old,
                     const double* v_old, double* rhs_u, double* rhs_v, const double* u_nm1,
                     const double* v_nm1, int has_nm1);
int orc_predictor(const covof_params* prm, double dt, double* u, double* v, const double* rho_u,
                  const double* rho_v, const double* mu, const double* mu_node,
                  const double* fx_sigma, const double* fy_sigma, const double* u_old,
                  const double* v_old, const double* u_nm1, const double* v_nm1, int has_nm1,
                  int* iters);
/* host threads of the Poisson solve inside orc_sp_step (default 1; the
 * Jacobi-PCG then runs the fused parallel loop, SGS stays serial) */
int orc_set_step_threads(int n);
int orc_sp_step(const covof_params* prm, double dt, double* u, double* v, double* p,
                const double* rho_u, const double* rho_v, const double* mu,
                const double* mu_node, const double* fx_sigma, const double* fy_sigma,
                const double* u_old, const double* v_old, const double* u_nm1, const double* v_nm1,
                int has_nm1, int* iters_u, int* iters_p, double* relres);

/* one augmented-Lagrangian step (solver_type AUGMENTED_LAGRANGIAN / AAL):
 * Uzawa iterations of the penalised momentum solve and p -= r div u;
 * iters = Krylov iterations summed, uzawa_done = Uzawa iterations run */
int orc_al_step(const covof_params* prm, double dt, double* u, double* v, double* p, const double* rho,
                const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                const double* fx_sigma, const double* fy_sigma, const double* u_old, const double* v_old,
                const double* u_nm1, const double* v_nm1, int has_nm1, int* iters, int* uzawa_done);
/* one MONOLITHIC step: the coupled (u, v, p) system with the Schur
 * diagonal as the pressure block's Jacobi preconditioner; iters = Krylov
 * iterations */
int orc_mono_step(const covof_params* prm, double dt, double* u, double* v, double* p, const double* rho_u,
                  const double* rho_v, const double* mu, const double* mu_node, const double* fx_sigma,
                  const double* fy_sigma, const double* u_old, const double* v_old, const double* u_nm1,
                  const double* v_nm1, int has_nm1, int* iters);

/* geometric VOF */
int orc_reconstruct(const covof_params* prm, const double* C, double* seg);
int orc_wy_step(const covof_params* prm, double dt, int x_first, const double* u,
                const double* v, double* C);
/* the configured VOF transport alone (advection_method), pass order x_first */
int orc_vof_transport(const covof_params* prm, double dt, int x_first, const double* u,
                      const double* v, double* C);
/* interface smoothing: SVOF (C -> C_s) and diffusion (C -> C_tilde) */
int orc_svof_smooth(const covof_params* prm, const double* C, double* C_s);
int orc_diffusion_smooth(const covof_params* prm, const double* C, double* C_tilde);
/* C_s / C_tilde: read when the matching smoothing is enabled (may be NULL otherwise) */
int orc_update_physical_properties(const covof_params* prm, double* C, double* rho,
                                   double* rho_u, double* rho_v, double* mu, double* mu_node,
                                   const double* C_s);
int orc_compute_curvature_and_csf(const covof_params* prm, const double* C, double* fx_sigma,
                                  double* fy_sigma, double* curvature, const double* C_s,
                                  const double* C_tilde);
int orc_vof_advect(const covof_params* prm, double dt, int step_count, const double* u,
                   const double* v, double* C, double* rho, double* rho_u, double* rho_v,
                   double* mu, double* mu_node, double* fx_sigma, double* fy_sigma,
                   double* curvature, double* C_s, double* C_tilde);

#ifdef __cplusplus
}
#endif
#endif
