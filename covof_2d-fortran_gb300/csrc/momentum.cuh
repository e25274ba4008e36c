// momentum.cuh -- argument blocks for the momentum predictor (momentum.cu).
#pragma once
#include "common.cuh"

namespace covof {

struct KrylovResult {
  int iters;
  int status;
};

struct MomArgs {
  Dims D;
  double dx, dy, dt, gx, gy;
  int bc[4];
  double bcu[4], bcv[4];
  int conv, scheme;
  // time scheme and linearisation with the history they need
  // (src/module_navier_stokes.f90:481-486, 2427-2457): alpha = 1.5 for Gear
  // once step n-1 is known, else 1; gear_rhs: the BDF2 inertial term; ab2:
  // advect with u_old / v_old; ab2_ext: extrapolate 2 u^n - u^(n-1)
  double alpha;
  int gear_rhs, ab2, ab2_ext;
  const double* u_nm1; const double* v_nm1;
  // augmented Lagrangian (solver_type AL / AAL): penalty field r_aal and the
  // pressure of the right-hand side's -grad p term; nullptr for projection
  const double* r_al; const double* p_al;
  // MONOLITHIC coupling (src/module_navier_stokes.f90:281-294, 597-602,
  // 723-777): the pressure is a third block of Krylov unknowns (cell DOFs
  // at offset 2g of every Krylov vector); pm: the pressure field packed from
  // and unpacked into
  int mono;
  double* pm;
  // fields_old of the operator (u^n with ghosts) and material properties
  const double* u_n; const double* v_n;
  const double* rho_u; const double* rho_v; const double* mu; const double* mu_node;
  // right-hand side inputs
  const double* fx; const double* fy; const double* u_old; const double* v_old;
  // Krylov storage: each vector 2*(nx+2)*(ny+2) doubles (u block, v block),
  // 3*(nx+2)*(ny+2) with the MONOLITHIC pressure block
  double* x; double* rhs; double* diag;
  double* coef;   // assembled rows: 9 slots x 2*(nx+2)*(ny+2), slot-major (k_mom_assemble)
  double* idiag;  // inverse Jacobi diagonal (1 where no division applies)
  double* v0; double* v1; double* v2; double* v3; double* v4; double* v5; double* v6;
  int precond_on, max_iter;
  int method;  // COVOF_LINEAR_* (the batch kernel dispatches on it)
  double tol;
  unsigned int* bar; int* err; double* part;  // part: 16 * nblocks doubles
  KrylovResult* res;
};

struct BcArgs {
  Dims D;
  int bc[4];
  double bcu[4], bcv[4];
};

// Five-point stencils of the SSOR / BLOCK_TRIANGULAR preconditioners
// (ns_assemble_preconditioner_blocks, src/module_navier_stokes.f90:
// 1268-1595): per block (u faces, v faces, Schur cells) the neighbour
// coefficients W, E, S, N (M-matrix form), the centre P (the reference's
// aP, or 1 where |aP| < 1e-30 as the sweeps read it) and rP = RN(1 / P).
// Each array (nx+2)*(ny+2) doubles in the field layout.
struct Stencil {
  double *W, *E, *S, *N, *P, *rP;
};
struct PBlk {
  Stencil u, v, s;
};

__global__ void k_mom_diag(MomArgs a);
__global__ void k_mono_diag(MomArgs a);
__global__ void k_prec_blocks(MomArgs a, PBlk b);
__global__ void k_prec_schur(MomArgs a, PBlk b);
__global__ void k_mom_matvec(MomArgs a, const double* x, double* y);

// Augmented Lagrangian (momentum.cu)
struct AlArgs {
  Dims D;
  double dx, dy, dt;
  const double *u, *v, *rho, *mu;
  double* p;
  double* r;                     // penalty field r_aal
  unsigned long long* maxv;      // [0] max |u_cell|, [1] max |p|, [2] max |div u| (bit patterns)
  // penalty parameters (src/module_navier_stokes.f90:1106-1218)
  int adaptive;
  double r_al, k_aal, L0, t0, g_norm, sigma, alpha_time, u0_ref, p0_ref, mu_max;
};
__global__ void k_al_maxima(AlArgs a);
__global__ void k_al_penalty(AlArgs a);
__global__ void k_al_pressure(AlArgs a);
__global__ void k_al_divmax(AlArgs a);
__global__ void k_mom_rhs(MomArgs a);
__global__ void k_mom_assemble(MomArgs a);
__global__ void k_mom_apply(MomArgs a, const double* xu, const double* xv, double* yu, double* yv);
__global__ void k_bicgstab(MomArgs a);
__global__ void k_bicgstab2(MomArgs a);
__global__ void k_cg(MomArgs a);
__global__ void k_mom_krylov_batch(const MomArgs* __restrict__ cases, BatchTeams bt);
__global__ void k_mom_bicgstab_batch(const MomArgs* __restrict__ cases, BatchTeams bt);
__global__ void k_mom_cg_batch(const MomArgs* __restrict__ cases, BatchTeams bt);
__global__ void k_mom_unpack(MomArgs a, double* u, double* v);
__global__ void k_mom_pack(MomArgs a, const double* u, const double* v);
__global__ void k_vbc_we(BcArgs b, double* u, double* v);
__global__ void k_vbc_sn(BcArgs b, double* u, double* v);
__global__ void k_vbc_periodic(BcArgs b, double* u, double* v);
__global__ void k_vbc_corners(BcArgs b, double* u, double* v);

}  // namespace covof
