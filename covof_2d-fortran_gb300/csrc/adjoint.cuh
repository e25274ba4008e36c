// adjoint.cuh -- argument block of the projection adjoint (adjoint.cu).
#pragma once
#include "common.cuh"

namespace covof {

struct AdjArgs {
  Dims D;
  double dx, dy, dt;
  int4 wall;
  const double* rho_u; const double* rho_v;
  const double* p;                       // forward pressure
  const double* gu; const double* gv;    // upstream gradient on faces
  const double* gp;                      // upstream gradient on cells (may be null)
  double* rhs; const double* psi;        // adjoint Poisson right-hand side / solution
  double* grad_u; double* grad_v;        // dL/du*, dL/dv*
  double* grad_bu; double* grad_bv;      // dL/d(1/rho_u), dL/d(1/rho_v)
};

__global__ void k_adj_rhs(AdjArgs a, double gp_mean);
__global__ void k_adj_grad(AdjArgs a);
__global__ void k_sum_interior(Dims D, const double* __restrict__ x, double* __restrict__ part);
__global__ void k_sum_final(const double* __restrict__ part, int n, double* __restrict__ out);

}  // namespace covof
