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
  // fields_old of the operator (u^n with ghosts) and material properties
  const double* u_n; const double* v_n;
  const double* rho_u; const double* rho_v; const double* mu; const double* mu_node;
  // right-hand side inputs
  const double* fx; const double* fy; const double* u_old; const double* v_old;
  // Krylov storage: each vector 2*(nx+2)*(ny+2) doubles (u block, v block)
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

__global__ void k_mom_diag(MomArgs a);
__global__ void k_mom_rhs(MomArgs a);
__global__ void k_mom_assemble(MomArgs a);
__global__ void k_mom_apply(MomArgs a, const double* xu, const double* xv, double* yu, double* yv);
__global__ void k_bicgstab(MomArgs a);
__global__ void k_bicgstab2(MomArgs a);
__global__ void k_cg(MomArgs a);
__global__ void k_mom_krylov_batch(const MomArgs* __restrict__ cases, BatchTeams bt);
__global__ void k_mom_unpack(MomArgs a, double* u, double* v);
__global__ void k_mom_pack(MomArgs a, const double* u, const double* v);
__global__ void k_vbc_we(BcArgs b, double* u, double* v);
__global__ void k_vbc_sn(BcArgs b, double* u, double* v);
__global__ void k_vbc_corners(BcArgs b, double* u, double* v);

}  // namespace covof
