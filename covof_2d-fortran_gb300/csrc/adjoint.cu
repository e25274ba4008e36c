// adjoint.cu -- hand-written adjoint (vector-Jacobian product) of the
// projection step of STANDARD_PROJECTION (src/module_simulation.f90:2476-2654).
//
// Forward, in matrix form over MAC faces f and cells c (walls excluded from
// G, whose rows are the interior faces):
//   b = -D u*,  D = -dvol G^T           (b_c = -[(u_{i+1}-u_i) dy + (v_{j+1}-v_j) dx])
//   A p = b,    A = dt dvol G^T B G     (B = diag(beta), beta = 1/rho_face;
//                                        a_face = dt dy/(rho dx) etc.)
//   u = u* - dt B G p                   ((G p)_f = (p_R - p_L)/h_f)
// Reverse for upstream gradients (g_u on faces, g_p on cells):
//   A psi = g_p' - dt G^T B g_u         (g_p' = g_p minus its mean in the
//                                        reference gauge, since p has its
//                                        mean removed; the same operator,
//                                        solved by the same solver)
//   dL/du*   = g_u - D^T psi            ((D^T psi)_f = len_f (psi_L - psi_R))
//   dL/dbeta = -dt (G p)_f [g_u,f + dvol (G psi)_f]   on interior faces
// The second line of the beta gradient is the face kernel -grad(lambda).grad(p)
// with lambda = -psi.
#include "common.cuh"
#include "adjoint.cuh"

namespace covof {

__device__ __forceinline__ double beta_of(double rho) { return 1.0 / (rho < 1.0e-12 ? 1.0 : rho); }

// rhs_c = g_p,c - gp_mean - dt [ (beta_w g_w - beta_e g_e)/dx + (beta_s g_s - beta_n g_n)/dy ]
// (wall faces carry no G row and drop out).
__global__ void k_adj_rhs(AdjArgs a, double gp_mean) {
  const Dims& D = a.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > D.nx || j > D.ny) return;
  const int k = D.id(i, j);
  const bool wW = (i == 1 && a.wall.x), wE = (i == D.nx && a.wall.y);
  const bool wS = (j == 1 && a.wall.z), wN = (j == D.ny && a.wall.w);
  const double fw = wW ? 0.0 : beta_of(a.rho_u[k]) * a.gu[k];
  const double fe = wE ? 0.0 : beta_of(a.rho_u[k + 1]) * a.gu[k + 1];
  const double fs = wS ? 0.0 : beta_of(a.rho_v[k]) * a.gv[k];
  const double fn = wN ? 0.0 : beta_of(a.rho_v[k + D.P]) * a.gv[k + D.P];
  const double gpc = a.gp ? a.gp[k] - gp_mean : 0.0;
  a.rhs[k] = gpc - a.dt * ((fw - fe) / a.dx + (fs - fn) / a.dy);
}

// Face gradients.  Thread (i, j) handles u-face (i, j) and v-face (i, j).
__global__ void k_adj_grad(AdjArgs a) {
  const Dims& D = a.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int nx = D.nx, ny = D.ny;
  const double dvol = a.dx * a.dy;
  // psi outside the interior is zero (solver vectors keep a zero ghost ring)
  if (i <= nx + 1 && j <= ny) {
    const int k = D.id(i, j);
    const double psiL = (i > 1) ? a.psi[k - 1] : 0.0, psiR = (i <= nx) ? a.psi[k] : 0.0;
    a.grad_u[k] = a.gu[k] - a.dy * (psiL - psiR);
    const bool wall = (i == 1 && a.wall.x) || (i == nx + 1 && a.wall.y);
    double gb = 0.0;
    if (!wall && i > 1 && i <= nx) {
      const double gpf = (a.p[k] - a.p[k - 1]) / a.dx;
      const double gpsi = (psiR - psiL) / a.dx;
      gb = -a.dt * gpf * (a.gu[k] + dvol * gpsi);
    }
    a.grad_bu[k] = gb;
  }
  if (i <= nx && j <= ny + 1) {
    const int k = D.id(i, j);
    const double psiL = (j > 1) ? a.psi[k - D.P] : 0.0, psiR = (j <= ny) ? a.psi[k] : 0.0;
    a.grad_v[k] = a.gv[k] - a.dx * (psiL - psiR);
    const bool wall = (j == 1 && a.wall.z) || (j == ny + 1 && a.wall.w);
    double gb = 0.0;
    if (!wall && j > 1 && j <= ny) {
      const double gpf = (a.p[k] - a.p[k - D.P]) / a.dy;
      const double gpsi = (psiR - psiL) / a.dy;
      gb = -a.dt * gpf * (a.gv[k] + dvol * gpsi);
    }
    a.grad_bv[k] = gb;
  }
}

// Deterministic interior sum: per-block partials (fixed tree) ...
__global__ void k_sum_interior(Dims D, const double* __restrict__ x, double* __restrict__ part) {
  double acc[1] = {0.0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < D.nx * D.ny; c += gridDim.x * blockDim.x) {
    const int j = c / D.nx + 1, i = c - (j - 1) * D.nx + 1;
    acc[0] += x[D.id(i, j)];
  }
  block_sum<double, 1>(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc[0];
}
// ... then one block adds the partials in a fixed order.
__global__ void k_sum_final(const double* __restrict__ part, int n, double* __restrict__ out) {
  double acc[1] = {0.0};
  for (int b = threadIdx.x; b < n; b += blockDim.x) acc[0] += part[b];
  block_sum<double, 1>(acc);
  if (threadIdx.x == 0) *out = acc[0];
}

}  // namespace covof

COVOF_UNIT_HOOKS(adjoint)
