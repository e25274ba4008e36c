// vof.cuh -- argument blocks for the VOF kernels (vof.cu).
#pragma once
#include "common.cuh"

namespace covof {

struct VofArgs {
  Dims D;
  double dx, dy, dt;
  int method;              // COVOF_RECON_*
  const double* C;         // field reconstructed by k_vof_classify / k_vof_mixed / k_vof_ring_warp
  double* seg;             // 3 * (nx+2)*(ny+2), AoS {nx, ny, alpha}
  const double* Cn;        // C at time n (dilatation indicator source)
  const double* u;
  const double* v;
};

struct PropsArgs {
  Dims D;
  int two_phase;
  double rho1, rho2, mu1, mu2;
  double* C; double* rho; double* rho_u; double* rho_v; double* mu; double* mu_node;
  const double* Cs;  // SVOF-smoothed indicator, nullptr without SVOF
};

struct CsfArgs {
  Dims D;
  double dx, dy, sigma;
  const double* C;
  const double* N;   // field the normals are taken from (C, C_s or C_tilde)
  double* nxv; double* nyv; double* kappa;   // scratch, zero ghost ring
  double* fx; double* fy; double* curv;
};

__global__ void k_vof_classify(VofArgs a, int* __restrict__ list, int* __restrict__ count);
__global__ void k_vof_mixed(VofArgs a, const int* __restrict__ list, const int* __restrict__ count, int min_count,
                            int max_count);
__global__ void k_vof_elvira_block(VofArgs a, const int* __restrict__ list, const int* __restrict__ count,
                                   int max_count);
__global__ void k_vof_mixed_cell(VofArgs a, const int* __restrict__ list, const int* __restrict__ count,
                                 int min_count);
__global__ void k_vof_ring_warp(VofArgs a);
__global__ void k_vof_pass(VofArgs a, int dir, int clamp, const double* __restrict__ Cin,
                           double* __restrict__ Cout);
__global__ void k_ciam_pass(VofArgs a, int dir, const double* __restrict__ Cin, double* __restrict__ Cout);
__global__ void k_tvd_advect(VofArgs a, int lim, const double* __restrict__ Cin, double* __restrict__ Cout);
__global__ void k_vof_bc(Dims D, double* __restrict__ C);
__global__ void k_vof_halo_bc(Dims D, double* __restrict__ C, int halo);
__global__ void k_props_cells(PropsArgs a);
__global__ void k_props_faces(PropsArgs a);
__global__ void k_csf_normals(CsfArgs a);
__global__ void k_csf_kappa(CsfArgs a);
__global__ void k_csf_force(CsfArgs a);

// Interface smoothing (svof.cu)
constexpr int kSvofIters = 25;  // sweep pairs (src/module_interface_vof.f90:409)
struct SvofArgs {
  Dims D;
  double wx, wy;             // D / dx^2, D / dy^2
  // per wall pattern f = (i==nx) | (i==1)<<1 | (j==ny)<<2 | (j==1)<<3:
  // aP = 1 + aE + aW + aN + aS in the reference's order, and RN(1 / aP)
  double aP[16], rP[16];
  const double* C;
  double* Cs;                // in: a copy of C; out: before the clamp
  unsigned int* prog;        // per band (stride 32): chunks published, zero at launch
  int* err;
};
__global__ void k_svof_sgs(SvofArgs a);
__global__ void k_svof_finish(Dims D, double* __restrict__ Cs);
__global__ void k_diffusion_step(Dims D, double dtau, double dx2, double dy2, const double* __restrict__ src,
                                 double* __restrict__ dst);
__global__ void k_diffusion_ghosts(Dims D, double* __restrict__ Ct);

}  // namespace covof
