// precond.cuh -- internal: the sequential preconditioners of the momentum /
// coupled Krylov solves (SSOR, BLOCK_TRIANGULAR) and the host-driven Krylov
// iterations that apply them.  Not part of the C ABI.
#pragma once
#include "momentum.cuh"

namespace covof {

constexpr int kSsorMaxJobs = 3;

// One lexicographic SSOR solve (src/module_linear_solvers.f90:1278-1401) of
// the stencil st on DOFs i = 1..ni, j = 1..nj of the field layout.
struct SsorJob {
  Stencil st;
  const double* z;     // right-hand side
  double* r;           // solution; zero on entry (its ghost entries stay zero)
  int ni, nj;
  int sweeps;          // symmetric pairs
  double omega;
  unsigned int* prog;  // per band (stride 32): chunks published, zero at launch
  // kind 0: the relaxed sweeps above.  kind 1: the pressure Poisson's
  // symmetric Gauss-Seidel pair (src/module_simulation.f90:2709-2758):
  // forward r = (z + aW r_W + aS r_S) / aP, backward
  // r = (aP r + aE r_E + aN r_N) / aP, neighbours inside the domain only;
  // pin: cell (1,1) held at zero (the pinned gauge)
  int kind, pin;
};

// Independent solves run side by side in one launch.
struct SsorArgs {
  Dims D;
  SsorJob job[kSsorMaxJobs];
  int njob;
  int band0[kSsorMaxJobs + 1];  // prefix sums of the jobs' band counts
  int* err;
};

__global__ void k_ssor(SsorArgs a);

}  // namespace covof
