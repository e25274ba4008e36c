/*
 * covof_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the COVOF 2D
 * per-timestep hot path: the STANDARD_PROJECTION step (momentum predictor,
 * variable-density pressure Poisson solve, velocity correction) and the
 * geometric VOF step (PLIC / ELVIRA reconstruction + Weymouth-Yue fluxes).
 *
 * Layout contract (identical to the reference's flow_fields_t,
 * src/module_fields.f90:129-169): every field argument is a Fortran array
 * dimensioned (0:nx+1, 0:ny+1), column-major, i fastest, one ghost layer,
 * i.e. (nx+2)*(ny+2) contiguous doubles with element (i,j) at i + (nx+2)*j.
 * u(i,j) is the normal velocity on the west face of cell i (x = (i-1)*dx),
 * v(i,j) on the south face of cell j (y = (j-1)*dy); p, C, rho, mu at cell
 * centres; mu_node(i,j) at the south-west node of cell (i,j).
 *
 * Host-pointer entry points copy in, compute on the device and copy out;
 * the caller owns every host array and nothing is retained past the call.
 * The *_dev entry points take device pointers with the same layout and run on
 * the handle's stream; all calls are synchronous on return.  A handle is not
 * thread-safe.  No entry point throws; every one returns a COVOF_* status.
 */
#ifndef COVOF_GPU_H
#define COVOF_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define COVOF_ABI_VERSION 1

/* Status codes.  MAXITER and BREAKDOWN mirror the reference's silent Krylov
 * exits (src/module_linear_solvers.f90:565,576,715; src/module_simulation.f90:2558):
 * the result is still written, the code tells the caller why the loop ended. */
enum {
  COVOF_OK = 0,
  COVOF_MAXITER = 1,
  COVOF_BREAKDOWN = 2,
  COVOF_NAN = 3,
  COVOF_TIMEOUT = 4,      /* a bounded device-side wait gave up */
  COVOF_UNSUPPORTED = 5,  /* option outside the implemented path */
  COVOF_CUDA_ERROR = 6,
  COVOF_INVALID = 7,      /* bad argument (null pointer, size, code) */
  COVOF_TOO_LARGE = 8     /* mesh exceeds a fixed-size buffer (covof_poisson_solve_rhs_static_dev) */
};

/* Boundary codes: same values as BC_* in src/module_constants.f90:41-44. */
enum { COVOF_BC_DIRICHLET = 1, COVOF_BC_NEUMANN = 2, COVOF_BC_PERIODIC = 3, COVOF_BC_FREESLIP = 4 };
/* Linear solvers: LINEAR_* in src/module_constants.f90:53-58. */
enum { COVOF_LINEAR_BICGSTAB2 = 1, COVOF_LINEAR_BICGSTAB = 2, COVOF_LINEAR_CG = 3 };
/* Preconditioners: PRECOND_* in src/module_constants.f90:67-72.
 * ILU0 is the same diagonal scaling as JACOBI in the reference
 * (src/module_linear_solvers.f90:280-304).  For the pressure Poisson
 * (p_precond) SSOR names the reference's symmetric Gauss-Seidel sweep pair
 * (src/module_simulation.f90:2709-2758).  In the momentum / coupled
 * Krylov solves SSOR is two symmetric lexicographic sweeps per block and
 * BLOCK_TRIANGULAR the Schur-complement sweeps then the velocity sweeps
 * (src/module_linear_solvers.f90:137-278); their Krylov iterations are driven
 * from the host, so covof_run_steps runs them eagerly. */
enum { COVOF_PRECOND_NONE = 0, COVOF_PRECOND_JACOBI = 1, COVOF_PRECOND_SSOR = 2, COVOF_PRECOND_ILU0 = 3,
       COVOF_PRECOND_BLOCK_TRIANGULAR = 4 };
/* Convective schemes: CONV_* in src/module_constants.f90:81-85. */
enum { COVOF_CONV_UPWIND = 1, COVOF_CONV_CENTERED = 2, COVOF_CONV_TVD_SUPERBEE = 3 };
/* Momentum time scheme: TIME_SCHEME_* in src/module_constants.f90:132-134
 * (0 is read as EULER).  GEAR (BDF2) applies once the velocity of step n-1
 * is known (has_nm1, covof_set_has_nm1). */
enum { COVOF_TIME_EULER = 1, COVOF_TIME_GEAR = 2 };
/* Linearisation of the convective term: CONV_LIN_* in
 * src/module_constants.f90:137-140 (0 is read as PICARD).  PICARD advects with
 * the current velocity, AB2 with the velocity at the start of the step,
 * extrapolated 2 u^n - u^(n-1) once has_nm1 holds.  NEWTON returns
 * COVOF_UNSUPPORTED. */
enum { COVOF_CONV_LIN_PICARD = 1, COVOF_CONV_LIN_AB2 = 2, COVOF_CONV_LIN_NEWTON = 3 };
/* Interface reconstruction (cfg%reconstruction_method). */
enum { COVOF_RECON_PLIC = 0, COVOF_RECON_ELVIRA = 1 };
/* VOF transport (cfg%advection_method, src/module_interface_vof.f90:801-808):
 * WEYMOUTH_YUE (:1162-1377), CIAM (:938-1159, geometric with a Lagrangian
 * remap of the cell width) or the algebraic TVD scheme (:828-935). */
enum { COVOF_ADVECT_WEYMOUTH_YUE = 0, COVOF_ADVECT_CIAM = 1, COVOF_ADVECT_TVD = 2 };
/* Velocity-pressure coupling (cfg%solver_type, src/module_constants.f90:41-49;
 * 0 reads as STANDARD_PROJECTION).  AUGMENTED_LAGRANGIAN / AAL: Uzawa
 * iterations of the momentum solve with the penalty r grad(div u) and the
 * update p -= r div u (src/module_simulation.f90:561-607); r is r_al, or the
 * adaptive field of src/module_navier_stokes.f90:1106-1218 with adaptative_al.
 * MONOLITHIC: one Krylov solve of the coupled (u, v, p) system with the
 * continuity rows (src/module_navier_stokes.f90:730-777) and the Schur
 * diagonal as the pressure block's Jacobi preconditioner (:1541-1590).  The
 * compressible CAAL returns COVOF_UNSUPPORTED. */
enum { COVOF_SOLVER_AUGMENTED_LAGRANGIAN = 1, COVOF_SOLVER_MONOLITHIC = 2, COVOF_SOLVER_STANDARD_PROJECTION = 3,
       COVOF_SOLVER_AAL = 4, COVOF_SOLVER_CAAL = 5 };
/* Limiter of the TVD transport (cfg%tvd_limiter,
 * src/module_interface_reconstruction.f90:686-725). */
enum { COVOF_LIMITER_SUPERBEE = 0, COVOF_LIMITER_VAN_LEER = 1, COVOF_LIMITER_MUSCL = 2, COVOF_LIMITER_HRIC = 3 };
/* Pressure gauge.  REFERENCE: 1e-12*dvol diagonal shift + mean removal
 * (src/module_simulation.f90:2531,2579-2582).  PINNED: same operator with
 * cell (1,1) held at p = 0 (no mean removal). */
enum { COVOF_GAUGE_REFERENCE = 0, COVOF_GAUGE_PINNED = 1 };
/* Poisson arithmetic.  FP64: plain FP64 PCG (the reference's algorithm).
 * MIXED: FP64 flexible CG on the true FP64 residual, preconditioned by an
 * FP32 inner iteration (p_inner_kind; FP64 solution).  FP64_MG: the MIXED
 * path with COVOF_INNER_MG and the V-cycle in FP64 (same kernels, same
 * p_mg_* settings, same gauge handling): beside MIXED it isolates what the
 * FP32 arithmetic of the inner iteration buys.  No reference counterpart. */
enum { COVOF_PREC_FP64 = 0, COVOF_PREC_MIXED = 1, COVOF_PREC_FP64_MG = 2 };

/* Plain-old-data parameter block (the subset of config_t,
 * src/module_config.f90:31-184, that the hot path reads). */
typedef struct covof_params {
  int nx, ny;            /* cells */
  double dx, dy;         /* mesh%dx, mesh%dy */
  int bc_type[4];        /* left, right, bottom, top: COVOF_BC_* */
  double bc_u[4];        /* wall velocity (cfg%bc_*%u) */
  double bc_v[4];        /* wall velocity (cfg%bc_*%v) */
  /* momentum predictor (cfg%linear_solver, precond_type, tol, max_iter) */
  int linear_solver;
  int precond;
  int use_precond;
  int max_iter;
  double tol;
  int enable_convection;
  int convective_scheme;
  /* pressure Poisson */
  int p_precond;         /* JACOBI, or SSOR: the symmetric Gauss-Seidel pair (FP64 only;
                            the PCG then iterates from the host, steps run eagerly) */
  int p_max_iter;
  int p_gauge;
  int p_precision;
  double p_tol;          /* ||r||/||b|| target */
  double p_inner_tol;    /* MIXED: relative reduction asked of each FP32 inner solve */
  int p_inner_max_iter;  /* MIXED: cap per inner solve */
  int p_max_refine;      /* MIXED: cap on outer refinement steps */
  /* two-phase properties */
  int enable_two_phase;
  int enable_surface_tension;
  double rho1, rho2, mu1, mu2, sigma, gx, gy;
  int recon;             /* COVOF_RECON_* */
  /* MIXED inner preconditioner (default COVOF_INNER_MG, the fastest measured
   * on every mesh from 256^2 to 4096^2): COVOF_INNER_CHEBYSHEV (degree p_inner_max_iter,
   * at most 128, on [p_cheb_lo * 2, 2], no inner reductions; its state lives
   * in shared-memory row strips on every SM when a strip fits, else it
   * streams through L2/HBM; covof_set_launch can place it in one
   * thread-block cluster instead), COVOF_INNER_CHEBYSHEV_STREAM (the
   * streaming form always), COVOF_INNER_MG (one geometric multigrid V-cycle
   * per outer iteration: Galerkin piecewise-constant coarsening, damped
   * Jacobi smoothing; p_max_iter then counts V-cycles) or
   * COVOF_INNER_CG (Jacobi-PCG, at most p_inner_max_iter iterations or
   * p_inner_tol reduction). */
  int p_inner_kind;
  double p_cheb_lo;      /* lower end of the Chebyshev interval, as a fraction of 2 */
  int p_mg_nu;           /* COVOF_INNER_MG: Jacobi sweeps before and after each coarse correction (1-8) */
  double p_mg_cw;        /* COVOF_INNER_MG: coarse-correction weight (0, 4]; about 1.8 offsets the
                          * stiffness of aggregation coarse operators (over-correction) */
  int p_mg_tail;         /* COVOF_INNER_MG: levels of at most this many cells run in one block's
                          * shared memory (0: 2048) */
  /* momentum time scheme and convective linearisation (cfg%time_scheme,
   * cfg%convective_linearization): COVOF_TIME_*, COVOF_CONV_LIN_* */
  int time_scheme;
  int convective_linearization;
  /* interface smoothing (cfg%enable_svof_smoothing, svof_filter_width,
   * enable_diffusion_smoothing, diffusion_smoothing_steps;
   * src/module_interface_vof.f90:387-476, 1416-1461): SVOF smooths C into
   * C_s (25 symmetric Gauss-Seidel sweeps of (I - D lap) C_s = C, D =
   * width * dx * dy; 0 reads as 1), which then gives rho, mu, mu_node and
   * the CSF normals; diffusion smoothing gives C_tilde (explicit steps; 0
   * reads as 3), which takes over the CSF normals. */
  int enable_svof_smoothing;
  double svof_filter_width;
  int enable_diffusion_smoothing;
  int diffusion_smoothing_steps;
  int advection_method;  /* COVOF_ADVECT_* */
  int tvd_limiter;       /* COVOF_LIMITER_* (TVD transport only) */
  /* coupling (cfg%solver_type, r_al, adaptative_al, k_aal, l0_ref, t0_ref,
   * u0_ref, p0_ref, ic_radius, uzawa_iter, uzawa_tol) */
  int solver_type;       /* COVOF_SOLVER_* */
  double r_al;           /* penalty (100) */
  int adaptative_al;     /* adaptive penalty field */
  double k_aal;          /* adaptive amplification (100) */
  double l0_ref, t0_ref, u0_ref, p0_ref;  /* reference scales, 0 = automatic */
  double ic_radius;      /* two-phase length scale 2 ic_radius when l0_ref = 0 (0.25) */
  int uzawa_iter;        /* Uzawa iterations per step (1) */
  double uzawa_tol;      /* stop when max |div u| <= uzawa_tol (1e-12; with uzawa_iter > 1) */
  int p_mg_nuc;          /* COVOF_INNER_MG: Jacobi sweeps on the coarsest level; < 0 (default):
                            solved exactly by a dense inverse formed once per solve when that
                            level has at most 64 cells and sits in block 0's shared memory
                            (else 64 sweeps); 0: 64 sweeps */
} covof_params;
enum { COVOF_INNER_CHEBYSHEV = 0, COVOF_INNER_CG = 1, COVOF_INNER_CHEBYSHEV_STREAM = 2, COVOF_INNER_MG = 3 };

typedef struct covof_handle covof_handle;

/* Reference-default parameters for an nx*ny mesh of lx*ly: no-slip walls,
 * BiCGSTAB(2)+Jacobi tol 1e-5 / 300 its (src/module_config.f90:576-636),
 * UPWIND, Poisson Jacobi-PCG tol 1e-7 / 1000 its, reference gauge, FP64. */
void covof_params_default(covof_params* p, int nx, int ny, double lx, double ly);

int covof_create(const covof_params* params, covof_handle** out);
int covof_destroy(covof_handle* h);
const char* covof_strerror(int status);
int covof_abi_version(void);
/* Failure-detection hook (no reference counterpart): the number of polls
 * every bounded device-side wait (grid and team barriers, neighbour
 * counters, wavefront progress) makes before it gives up, records
 * COVOF_TIMEOUT and returns; 0 restores the default of 2^21 polls (about a
 * second).  A test lowers it to make waits run out -- the solve returns
 * COVOF_TIMEOUT, no GPU fault -- and restores it; the handle stays usable.
 * Applies to the current device; set it while no kernel of this library runs. */
int covof_set_wait_budget(long long polls);
/* Bounds-check build (no reference counterpart): in a library compiled with
 * -DCOVOF_CHECKED every cell index formed on the device and every stencil
 * centre of the operators is checked against the (nx+2) x (ny+2) ghosted
 * extents; a bad index is counted, the first recorded, and the access
 * redirected inside the array.  Returns the count since the last call (bad)
 * and the first record (first: site << 40 | index + 2^39), then clears them.
 * The normal build returns COVOF_UNSUPPORTED. */
int covof_bounds_check(long long* bad, long long* first);
/* Device the handle was created on and the number of SMs it uses. */
int covof_device_info(const covof_handle* h, int* device, int* sm_count);

/* ---- STANDARD_PROJECTION --------------------------------------------- */

/* Whole SP step: replaces sim_solve_standard_projection
 * (src/module_simulation.f90:2424-2666).  u, v hold u^n on entry and u^{n+1}
 * on exit (ghosts set by the non-homogeneous velocity BC, as
 * src/module_mpi_comm.f90:290-537); p is the warm start on entry and the
 * projected pressure on exit.  total_iters = predictor + Poisson iterations. */
int covof_sp_step(covof_handle* h, double dt, double* u, double* v, double* p,
                  const double* rho_u, const double* rho_v, const double* mu,
                  const double* mu_node, const double* fx_sigma, const double* fy_sigma,
                  const double* u_old, const double* v_old,
                  int* total_iters, double* final_relres);
int covof_sp_step_dev(covof_handle* h, double dt, double* u, double* v, double* p,
                      const double* rho_u, const double* rho_v, const double* mu,
                      const double* mu_node, const double* fx_sigma, const double* fy_sigma,
                      const double* u_old, const double* v_old,
                      int* total_iters, double* final_relres);

/* Momentum predictor only (src/module_simulation.f90:2454-2470): u, v in/out. */
int covof_predictor(covof_handle* h, double dt, double* u, double* v,
                    const double* rho_u, const double* rho_v, const double* mu,
                    const double* mu_node, const double* fx_sigma, const double* fy_sigma,
                    const double* u_old, const double* v_old, int* iters);
int covof_predictor_dev(covof_handle* h, double dt, double* u, double* v,
                        const double* rho_u, const double* rho_v, const double* mu,
                        const double* mu_node, const double* fx_sigma, const double* fy_sigma,
                        const double* u_old, const double* v_old, int* iters);

/* Momentum operator y = A x on one (u,v) pair (ns_apply_system_matrix,
 * src/module_navier_stokes.f90:380-780), fields_old = (u_n, v_n, rho_u, rho_v,
 * mu, mu_node); x and y are ghosted (u,v) arrays, only DOF entries of y are
 * written.  Exposed for parity tests of the operator itself. */
int covof_momentum_apply(covof_handle* h, double dt, const double* xu, const double* xv,
                         double* yu, double* yv, const double* u_n, const double* v_n,
                         const double* rho_u, const double* rho_v, const double* mu,
                         const double* mu_node);

/* The momentum / coupled Krylov solve's preconditioner M^-1 on one operand
 * (apply_precond, src/module_linear_solvers.f90:88-304): JACOBI / ILU0
 * diagonal scaling, or the SSOR / BLOCK_TRIANGULAR sweeps over the stencils
 * of ns_assemble_preconditioner_blocks (src/module_navier_stokes.f90:
 * 1268-1595), assembled from fields_old = (u_n, v_n, rho_u, rho_v, mu,
 * mu_node) and the handle's history.  zp / yp: the pressure block
 * (MONOLITHIC only, else may be NULL); r_al: the penalty field for
 * AUGMENTED_LAGRANGIAN / AAL (else NULL).  Exposed for parity tests of the
 * preconditioner itself. */
int covof_precond_apply(covof_handle* h, double dt, const double* zu, const double* zv, const double* zp,
                        double* yu, double* yv, double* yp, const double* u_n, const double* v_n,
                        const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                        const double* r_al);

/* Pressure Poisson from a predicted velocity (src/module_simulation.f90:2476-2584):
 * assembly, PCG, gauge.  p: warm start in, solution out (interior). */
int covof_poisson_solve(covof_handle* h, double dt, const double* u_star, const double* v_star,
                        const double* rho_u, const double* rho_v, double* p,
                        int* iters, double* relres);
int covof_poisson_solve_dev(covof_handle* h, double dt, const double* u_star, const double* v_star,
                            const double* rho_u, const double* rho_v, double* p,
                            int* iters, double* relres);
/* Same operator with an explicit right-hand side b (ghosted layout, interior
 * read) in place of -div(u*): the standalone variable-density Poisson. */
int covof_poisson_solve_rhs(covof_handle* h, double dt, const double* b,
                            const double* rho_u, const double* rho_v, double* p,
                            int* iters, double* relres);
int covof_poisson_solve_rhs_dev(covof_handle* h, double dt, const double* b,
                                const double* rho_u, const double* rho_v, double* p,
                                int* iters, double* relres);
/* Velocity correction u -= dt/rho_u dp/dx, v -= dt/rho_v dp/dy
 * (src/module_simulation.f90:2586-2660). */
int covof_project_correct(covof_handle* h, double dt, double* u, double* v, const double* p,
                          const double* rho_u, const double* rho_v);

/* Poisson operator y = A x (interior of y written), assembled from rho_u,
 * rho_v and dt as in covof_poisson_solve.  Exposed for parity tests of the
 * operator (src/module_simulation.f90:2668-2707). */
int covof_poisson_apply(covof_handle* h, double dt, const double* rho_u, const double* rho_v,
                        const double* x, double* y);
int covof_poisson_apply_dev(covof_handle* h, double dt, const double* rho_u, const double* rho_v,
                            const double* x, double* y);

/* The handle's CUDA stream (a blocking stream: it orders after work on the
 * legacy default stream) and the device time of the last Poisson solve
 * kernel, measured with CUDA events on that stream. */
int covof_get_stream(const covof_handle* h, void** stream);
int covof_last_solve_ms(const covof_handle* h, double* ms);
/* Outer FP64 refinement steps of the last MIXED Poisson solve. */
int covof_last_refine_steps(const covof_handle* h, int* steps);

/* Allocation-free plain FP64 Poisson solve (no counterpart in the reference,
 * which has no GPU path).  For callers that cannot allocate device memory at
 * the call: a host code whose pool allocator reserved the whole GPU at
 * start-up, or a time loop that must not pay cudaMalloc's device-wide
 * synchronisation.  Same operator, solver and results as
 * covof_poisson_solve_rhs_dev with prm->p_precision = FP64 and the Jacobi
 * preconditioner (other p_precision values and p_precond = SSOR return
 * COVOF_UNSUPPORTED), but no handle: inputs and outputs are the caller's
 * device pointers, the scratch is a fixed static device array (about 5.4 MB,
 * held by every GPU that loads the library until exit) and nothing is
 * allocated.  Limit: (nx+2)*(ny+2) <= 258*258 (256 x 256 cells); larger
 * meshes return COVOF_TOO_LARGE.  Every call looks up the array's device
 * address on the current device; the first call on a device also loads the
 * library's device code there, so make it before any stream capture.  An
 * error pending from the caller's earlier work is returned as
 * COVOF_CUDA_ERROR before anything is launched.  Runs on the legacy default
 * stream and is synchronous.  All calls share the array: calls that overlap
 * on the GPU (from several host threads or streams) race. */
int covof_poisson_solve_rhs_static_dev(const covof_params* prm, double dt, const double* b,
                                       const double* rho_u, const double* rho_v, double* p,
                                       int* iters, double* relres);

/* ---- projection adjoint ------------------------------------------------ */

/* Forward projection: p from the Poisson solve on -div(u*) (as
 * covof_poisson_solve), then u = u* - dt/rho_u dp/dx, v likewise (as
 * covof_project_correct) into separate outputs u, v (DOF faces written). */
int covof_projection(covof_handle* h, double dt, const double* u_star, const double* v_star,
                     const double* rho_u, const double* rho_v, double* p, double* u, double* v,
                     int* iters, double* relres);
int covof_projection_dev(covof_handle* h, double dt, const double* u_star, const double* v_star,
                         const double* rho_u, const double* rho_v, double* p, double* u, double* v,
                         int* iters, double* relres);
/* Vector-Jacobian product of covof_projection (no counterpart in the
 * reference, which has no derivatives; built on its operators).  Given the
 * forward pressure p and upstream gradients gu, gv (faces) and gp (cells, may
 * be NULL), solves one adjoint Poisson problem with the same symmetric
 * operator and writes dL/du* (grad_u, grad_v, every DOF face) and
 * dL/d(1/rho_face) (grad_bu, grad_bv, interior faces; zero elsewhere). */
int covof_projection_vjp(covof_handle* h, double dt, const double* rho_u, const double* rho_v,
                         const double* p, const double* gu, const double* gv, const double* gp,
                         double* grad_u, double* grad_v, double* grad_bu, double* grad_bv,
                         int* iters, double* relres);
int covof_projection_vjp_dev(covof_handle* h, double dt, const double* rho_u, const double* rho_v,
                             const double* p, const double* gu, const double* gv, const double* gp,
                             double* grad_u, double* grad_v, double* grad_bu, double* grad_bv,
                             int* iters, double* relres);

/* ---- geometric VOF ---------------------------------------------------- */

/* reconstruct_interface (src/module_interface_reconstruction.f90:580-683):
 * seg = 3*(nx+2)*(ny+2) doubles, AoS {nx, ny, alpha} per cell. */
int covof_vof_reconstruct(covof_handle* h, const double* C, double* seg);
int covof_vof_reconstruct_dev(covof_handle* h, const double* C, double* seg);
/* advect_vof_weymouth_yue (src/module_interface_vof.f90:1162-1377) with the
 * pass order given explicitly (x_first = mod(vof_step_count,2)==0). */
int covof_vof_wy_step(covof_handle* h, double dt, int x_first, const double* u, const double* v,
                      double* C);
int covof_vof_wy_step_dev(covof_handle* h, double dt, int x_first, const double* u,
                          const double* v, double* C);
/* advect_vof (src/module_interface_vof.f90:792-825) for WEYMOUTH_YUE: the WY
 * step with the handle's vof_step_count, the count increment, the VOF BC,
 * update_physical_properties and compute_curvature_and_csf. */
int covof_vof_advect(covof_handle* h, double dt, const double* u, const double* v, double* C,
                     double* rho, double* rho_u, double* rho_v, double* mu, double* mu_node,
                     double* fx_sigma, double* fy_sigma, double* curvature);
int covof_vof_advect_dev(covof_handle* h, double dt, const double* u, const double* v, double* C,
                         double* rho, double* rho_u, double* rho_v, double* mu, double* mu_node,
                         double* fx_sigma, double* fy_sigma, double* curvature);
int covof_get_vof_step_count(const covof_handle* h, int* count);
int covof_set_vof_step_count(covof_handle* h, int count);
/* smooth_svof_helmholtz (src/module_interface_vof.f90:387-476): C -> C_s,
 * also kept as the resident C_s that the property and CSF entry points read
 * when enable_svof_smoothing is set.  C_s may be NULL (resident copy only).
 * On the device the Gauss-Seidel sweeps run as a wavefront and give the
 * serial loop's values. */
int covof_svof_smooth(covof_handle* h, const double* C, double* C_s);
/* vof_smooth_diffusion (:1416-1461): C -> C_tilde, also kept resident (the
 * CSF normals read it when enable_diffusion_smoothing is set). */
int covof_diffusion_smooth(covof_handle* h, const double* C, double* C_tilde);
/* update_physical_properties (src/module_interface_vof.f90:479-616); C's
 * physical corners are rewritten as in the reference.  With SVOF the cell
 * properties and mu_node follow the resident C_s. */
int covof_update_physical_properties(covof_handle* h, double* C, double* rho, double* rho_u,
                                     double* rho_v, double* mu, double* mu_node);
/* apply_velocity_bc (src/module_mpi_comm.f90:290-537, one rank, constant
 * wall values bc_u / bc_v): the ghost values of u and v for the boundary
 * types of the parameter block; interior faces untouched. */
int covof_apply_velocity_bc(covof_handle* h, double* u, double* v);
/* apply_vof_bc (src/module_mpi_comm.f90:636-683, one rank): the ghost values
 * of C (zero gradient at walls). */
int covof_apply_vof_bc(covof_handle* h, double* C);
/* compute_curvature_and_csf (src/module_interface_vof.f90:627-789); the
 * normals come from the resident C_tilde (diffusion smoothing) or C_s (SVOF)
 * when those are enabled. */
int covof_compute_curvature_and_csf(covof_handle* h, const double* C, double* fx_sigma,
                                    double* fy_sigma, double* curvature);

/* One augmented-Lagrangian step (solver_type AUGMENTED_LAGRANGIAN / AAL,
 * src/module_simulation.f90:546-607): the penalty field r_aal (r_al, or the
 * adaptive field with adaptative_al), the predictor's Jacobi diagonal, then
 * up to uzawa_iter Uzawa iterations of the penalised momentum solve and
 * p -= r div u, stopping when max |div u| <= uzawa_tol.  Gear / AB2 read the
 * handle's history as in covof_predictor.  total_iters: predictor Krylov
 * iterations summed over the Uzawa iterations; uzawa_done: iterations run.
 * covof_run_steps runs this coupling in place of STANDARD_PROJECTION when
 * solver_type asks for it (eagerly when the Uzawa exit test is on). */
int covof_al_step(covof_handle* h, double dt, double* u, double* v, double* p, const double* rho,
                  const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                  const double* fx_sigma, const double* fy_sigma, const double* u_old, const double* v_old,
                  int* total_iters, int* uzawa_done);

/* One MONOLITHIC step (solver_type MONOLITHIC, src/module_simulation.f90:
 * 552-583): the preconditioner blocks (momentum diagonals, Schur diagonal
 * diag_p), the right-hand side without a pressure term, one Krylov solve
 * (linear_solver) of the coupled system for (u, v, p) from the given fields,
 * then the velocity boundary conditions.  Replaces the reference's
 * assemble_preconditioner_blocks + assemble_rhs + pack_vector +
 * solve_linear_system + unpack_vector sequence (src/module_simulation.f90:
 * 552-583, src/module_navier_stokes.f90:231-375, 785-1101, 1268-1595).
 * Gear / AB2 read the handle's history as in covof_predictor.  Returns the
 * Krylov status; iters: Krylov iterations. */
int covof_monolithic_step(covof_handle* h, double dt, double* u, double* v, double* p, const double* rho_u,
                          const double* rho_v, const double* mu, const double* mu_node, const double* fx_sigma,
                          const double* fy_sigma, const double* u_old, const double* v_old, int* iters);

/* The FP64 rate this GPU sustains on independent FMA chains (GFLOP/s, two
 * flops per FMA), measured on the handle's stream: the denominator of the
 * interface reconstruction's FP64 rate. */
int covof_fp64_peak(covof_handle* h, double* gflops);

/* ---- device-resident time stepping ------------------------------------ */

/* The members of flow_fields_t (src/module_fields.f90:27-92) that the hot
 * path reads or writes, kept on the device inside the handle. */
enum {
  COVOF_FIELD_U = 0, COVOF_FIELD_V = 1, COVOF_FIELD_P = 2, COVOF_FIELD_C = 3,
  COVOF_FIELD_RHO = 4, COVOF_FIELD_RHO_U = 5, COVOF_FIELD_RHO_V = 6, COVOF_FIELD_MU = 7,
  COVOF_FIELD_MU_NODE = 8, COVOF_FIELD_FX_SIGMA = 9, COVOF_FIELD_FY_SIGMA = 10,
  COVOF_FIELD_CURVATURE = 11, COVOF_FIELD_U_OLD = 12, COVOF_FIELD_V_OLD = 13,
  COVOF_FIELD_U_NM1 = 14, COVOF_FIELD_V_NM1 = 15, COVOF_FIELD_C_S = 16, COVOF_FIELD_C_TILDE = 17,
  COVOF_NFIELDS = 18
};
/* Copy one (nx+2)*(ny+2) field between the host and the handle's resident
 * copy (synchronous). */
int covof_state_set(covof_handle* h, int field, const double* host);
int covof_state_get(covof_handle* h, int field, double* host);
/* Device address of the resident copy (valid until covof_destroy). */
int covof_state_field_dev(covof_handle* h, int field, double** dev);
/* Whether the resident u_nm1 / v_nm1 hold the velocity of step n-1
 * (fields%has_nm1, src/module_simulation.f90:508-520): Gear / BDF2 and the
 * Adams-Bashforth extrapolation use them only then.  Every predictor entry
 * point reads the handle's u_nm1 / v_nm1 and this flag; covof_run_steps
 * rotates u_nm1 = u_old (or u on a first step) itself and sets the flag
 * after its first step.  A new handle starts with has_nm1 = 0. */
int covof_set_has_nm1(covof_handle* h, int has_nm1);
int covof_get_has_nm1(const covof_handle* h, int* has_nm1);

typedef struct covof_run_stats {
  int steps;               /* time steps run */
  int first_bad_step;      /* -1 when every solve returned COVOF_OK */
  int first_bad_status;    /* status of that step's first failing solve */
  int graph;               /* 1 when the steps replayed captured CUDA graphs */
  long long mom_iters;     /* predictor Krylov iterations, summed over steps */
  long long poisson_iters; /* Poisson iterations (mixed: FP32 inner steps), summed */
  long long refine_steps;  /* mixed: FP64 outer steps, summed */
  double last_relres;      /* Poisson ||r||/||b|| of the last step */
  double max_relres;       /* largest Poisson ||r||/||b|| of the run */
  double ms;               /* device time of the run (CUDA events) */
} covof_run_stats;

#define COVOF_RUN_GRAPH 1  /* flag: replay each step as a captured CUDA graph */

/* nsteps iterations of the time loop body of sim_run
 * (src/module_simulation.f90:492-559) on the resident fields, for a fixed dt
 * (adaptive_dt = .false.), Euler time stepping and STANDARD_PROJECTION:
 *   u_old = u, v_old = v;
 *   if enable_two_phase: advect_vof (WEYMOUTH_YUE), apply_velocity_bc;
 *   sim_solve_standard_projection.
 * No host synchronisation between steps: each solve's status is folded into
 * device-side statistics that are read once at the end.  A failing step does
 * not stop the run (the reference's Krylov exits are silent too); the first
 * one is reported.  With COVOF_RUN_GRAPH each step is one graph launch (two
 * graphs, for the two Weymouth-Yue pass orders), captured on the first call
 * for a given dt; where capture is refused the steps run eagerly and
 * stats->graph is 0. */
int covof_run_steps(covof_handle* h, double dt, int nsteps, int flags, covof_run_stats* stats);

/* ---- snapshot output --------------------------------------------------- */

/* The files of the reference's vtk_write_step for one rank
 * (src/module_vtk_writer.f90:90-386): <dir>/<case_name>_p0_<step>.vtr and
 * <dir>/<case_name>_<step>.pvtr (step as 6 digits), ASCII, every value as
 * Fortran ES16.8, from the resident fields at the point of the call in stream
 * order.  Asynchronous: a device-side snapshot on the handle's stream, the
 * host copy on a side stream and the formatting on a host thread; steps
 * enqueued afterwards do not wait for it.  Returns the status of the previous
 * snapshot's write.  Temperature is written as 300 (the reference's reset
 * value; no energy equation here). */
int covof_vtk_write_async(covof_handle* h, const char* dir, const char* case_name, int step);
/* Waits for the last snapshot's files; returns their status. */
int covof_vtk_wait(covof_handle* h);
/* vtk_init's history file (src/module_vtk_writer.f90:61-70): creates dir and
 * <dir>/<case_name>_history.csv with its header line. */
int covof_history_open(covof_handle* h, const char* dir, const char* case_name);
/* Appends the record of vtk_write_diagnostics (src/module_vtk_writer.f90:
 * 392-470: bubble centroid height, rise velocity, volume, kinetic energy, max
 * speed, max |div u|, gas density and pressure averages) for the resident
 * fields at the call, computed on a host thread in the reference's serial
 * order, like covof_vtk_write_async (which it shares the writer with). */
int covof_history_write_async(covof_handle* h, const char* dir, const char* case_name, int step, double time,
                              double dt);

/* ---- launch shapes (autotuning) --------------------------------------- */

/* Launch shape of the Poisson solver of a handle.  Zero fields leave the
 * choice to the built-in rules; the autotuner (autotune.py) times candidates
 * and sets the fastest.  No reference counterpart. */
typedef struct covof_launch {
  int p_threads;     /* threads per block, 128, 256, 512 or 1024, of the plain FP64 PCG and of
                      * the multigrid solve (0: the built-in choice by mesh size) */
  int p_blocks;      /* blocks of the persistent solve (mixed: row strips), at most one per SM */
  int p_inner_form;  /* mixed Chebyshev inner state: 1 shared-memory strips on every SM,
                      * 2 streamed through L2 / HBM, 3 one thread-block cluster of p_blocks
                      * (<= 16) CTAs exchanging rows through distributed shared memory */
  int vof_cell_min;  /* interface reconstruction: from this many interface cells on, one
                      * thread per cell instead of one warp per cell (same results bit for
                      * bit); 0 = the built-in 16384 */
} covof_launch;
/* Set the overrides (validated: COVOF_INVALID for out-of-range values,
 * COVOF_UNSUPPORTED for shared-memory strips that do not fit); drops the
 * handle's launch plan and captured graphs. */
int covof_set_launch(covof_handle* h, const covof_launch* launch);
/* The shape in effect (after planning): every field filled in. */
int covof_get_launch(covof_handle* h, covof_launch* launch);

/* ---- batches of independent cases ------------------------------------- */

/* Many independent cases (each its own mesh size and parameters) stepped
 * together.  No reference counterpart: the reference runs one case per MPI
 * job.  A batch step runs, for every case, what covof_run_steps runs, with
 * the predictor and Poisson Krylov solves of ALL cases in one persistent
 * cooperative launch each (teams of blocks, one case per team at a time);
 * with COVOF_RUN_GRAPH a whole batch step is one CUDA-graph launch.  All
 * cases of a batch use the same Poisson arithmetic (p_precision).  A mixed
 * batch runs COVOF_INNER_MG for every case (each case its own hierarchy) or
 * the Chebyshev inner iteration for every case, with each case's state in
 * shared-memory row strips of a team sized to fit (at most 32 blocks), or
 * streamed through L2 / HBM when a case does not fit or any case asks for
 * COVOF_INNER_CHEBYSHEV_STREAM; COVOF_INNER_CG, and multigrid mixed with
 * Chebyshev cases, are rejected (COVOF_UNSUPPORTED).  The Weymouth-Yue pass
 * order follows the batch's own step count (x first on its first step). */
typedef struct covof_batch covof_batch;
int covof_batch_create(const covof_params* cases, int ncases, covof_batch** out);
int covof_batch_destroy(covof_batch* b);
/* Resident fields of one case (COVOF_FIELD_*), as covof_state_set/get. */
/* covof_set_has_nm1 for every case of the batch (a new batch starts with 0;
 * its first step sets it). */
int covof_batch_set_has_nm1(covof_batch* b, int has_nm1);
int covof_batch_state_set(covof_batch* b, int icase, int field, const double* host);
int covof_batch_state_get(covof_batch* b, int icase, int field, double* host);
/* nsteps steps of every case, dt[icase] each (fixed per call); stats (one per
 * case, may be NULL) as covof_run_steps; ms = device time of the call.
 * Returns the first failing case's first failing status, else COVOF_OK. */
int covof_batch_run_steps(covof_batch* b, const double* dt, int nsteps, int flags,
                          covof_run_stats* stats, double* ms);
/* Team layout of the two batched solves. */
int covof_batch_info(const covof_batch* b, int* poisson_teams, int* poisson_blocks,
                     int* predictor_teams, int* predictor_blocks);

#ifdef __cplusplus
}
#endif
#endif /* COVOF_GPU_H */
