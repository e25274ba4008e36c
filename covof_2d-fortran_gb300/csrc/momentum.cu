// momentum.cu -- momentum predictor of the STANDARD_PROJECTION step on one
// GB300: matrix-free MAC momentum operator (Euler or Gear/BDF2 unsteady
// term + upwind / centred / TVD-Superbee convection, Picard or
// Adams-Bashforth linearisation + 2 mu normal stress + mu_node shear),
// its Jacobi diagonal and right-hand side, and persistent cooperative
// BiCGSTAB / BiCGSTAB(2) / CG kernels that run a whole Krylov solve in one
// launch with device-side convergence tests.
//
// Krylov vectors hold the u DOFs (i=1..nx+1, j=1..ny) in the first
// (nx+2)*(ny+2) block and the v DOFs (i=1..nx, j=1..ny+1) in the second, in
// the field layout itself; ghost entries are never read: the operator
// evaluates the homogeneous ghost conditions of
// src/module_mpi_comm.f90:290-537 on the fly from the DOF values, as the
// reference does when ns_unpack_vector applies them before every product
// (src/module_navier_stokes.f90:397-458).  Expressions follow the reference
// term order and the unit is built with -fmad=false, so one operator
// application is bit-identical to a serial FP64 evaluation.
#include "common.cuh"
#include "momentum.cuh"

namespace covof {

enum { SL = 0, SR = 1, SB = 2, ST = 3 };

__device__ __forceinline__ bool is_wall(const MomArgs& a, int s) {
  return a.bc[s] == COVOF_BC_DIRICHLET || a.bc[s] == COVOF_BC_FREESLIP;
}

// Operand u with homogeneous ghosts.  Reads bypass L1: other blocks of the
// persistent kernel wrote the vector.
__device__ __forceinline__ double tu(const MomArgs& a, const double* xu, int i, int j) {
  const Dims& D = a.D;
  const int nx = D.nx, ny = D.ny;
  if (j >= 1 && j <= ny) {
    if (i >= 1) return __ldcg(xu + D.id(i, j));  // i <= nx+1 for every read made
    return 0.0;                                   // west wall: u(0,j) = u_l = 0
  }
  if (j == 0) {
    const double u1 = __ldcg(xu + D.id(i, 1));
    if (a.bc[SB] == COVOF_BC_DIRICHLET) {
      if (ny >= 2) return (8.0 * 0.0 - 6.0 * u1 + __ldcg(xu + D.id(i, 2))) / 3.0;
      return 2.0 * 0.0 - u1;
    }
    return u1;  // FREESLIP
  }
  // j == ny + 1
  const double un = __ldcg(xu + D.id(i, ny));
  if (a.bc[ST] == COVOF_BC_DIRICHLET) {
    if (ny >= 2) return (8.0 * 0.0 - 6.0 * un + __ldcg(xu + D.id(i, ny - 1))) / 3.0;
    return 2.0 * 0.0 - un;
  }
  return un;
}

// Operand v with homogeneous ghosts.
__device__ __forceinline__ double tv(const MomArgs& a, const double* xv, int i, int j) {
  const Dims& D = a.D;
  const int nx = D.nx;
  if (j == 0) return 0.0;  // south wall: v(i,0) = v_b = 0
  if (i == 0) {
    const double v1 = __ldcg(xv + D.id(1, j));
    return a.bc[SL] == COVOF_BC_DIRICHLET ? 2.0 * 0.0 - v1 : v1;
  }
  if (i == nx + 1) {
    const double vn = __ldcg(xv + D.id(nx, j));
    return a.bc[SR] == COVOF_BC_DIRICHLET ? 2.0 * 0.0 - vn : vn;
  }
  return __ldcg(xv + D.id(i, j));
}

// src/module_navier_stokes.f90:2388-2416 conv_face_flux.  The operand
// values pl, pr are of type T (doubles, or linear forms for the row
// coefficients); the TVD limiter reads only fields_old values (q*), so the
// face flux stays linear in the operand.
template <class T>
__device__ __forceinline__ T conv_face_flux(int scheme, double flux, const T& pl, const T& pr, double qLL,
                                            double qL, double qR, double qRR, bool hasLL, bool hasRR) {
  if (scheme == COVOF_CONV_CENTERED) return 0.5 * flux * (pl + pr);
  if (scheme == COVOF_CONV_UPWIND) return (flux >= 0.0) ? flux * pl : flux * pr;
  // TVD, Superbee limiter
  const double dq = qR - qL;
  double psi = 0.0;
  if (flux >= 0.0) {
    if (hasLL && fabs(dq) > 1.0e-14) {
      const double r = (qL - qLL) / dq;
      psi = fmax(fmax(0.0, fmin(2.0 * r, 1.0)), fmin(r, 2.0));
    }
    return flux * (pl + 0.5 * psi * (pr - pl));
  }
  if (hasRR && fabs(dq) > 1.0e-14) {
    const double r = (qRR - qR) / dq;
    psi = fmax(fmax(0.0, fmin(2.0 * r, 1.0)), fmin(r, 2.0));
  }
  return flux * (pr + 0.5 * psi * (pl - pr));
}

// src/module_navier_stokes.f90:2418-2457 compute_u_conv_fluxes: the
// advecting velocity is fields%u (PICARD) or fields%u_old (AB2),
// extrapolated 2 u^n - u^(n-1) when the history exists
__device__ __forceinline__ void u_fluxes(const MomArgs& a, int i, int j, double& FE, double& FW,
                                         double& FN, double& FS) {
  const Dims& D = a.D;
  const double* ub = a.ab2 ? a.u_old : a.u_n;
  const double* vb = a.ab2 ? a.v_old : a.v_n;
  double un = ub[D.id(i, j)], unE = ub[D.id(i + 1, j)], unW = ub[D.id(i - 1, j)];
  double vnN = 0.5 * (vb[D.id(i - 1, j + 1)] + vb[D.id(i, j + 1)]);
  double vnS = 0.5 * (vb[D.id(i - 1, j)] + vb[D.id(i, j)]);
  if (a.ab2_ext) {
    un = 2.0 * un - a.u_nm1[D.id(i, j)];
    unE = 2.0 * unE - a.u_nm1[D.id(i + 1, j)];
    unW = 2.0 * unW - a.u_nm1[D.id(i - 1, j)];
    const double vmN = 0.5 * (a.v_nm1[D.id(i - 1, j + 1)] + a.v_nm1[D.id(i, j + 1)]);
    const double vmS = 0.5 * (a.v_nm1[D.id(i - 1, j)] + a.v_nm1[D.id(i, j)]);
    vnN = 2.0 * vnN - vmN;
    vnS = 2.0 * vnS - vmS;
  }
  FE = 0.5 * (un + unE) * a.dy;
  FW = 0.5 * (unW + un) * a.dy;
  FN = vnN * a.dx;
  FS = vnS * a.dx;
}
// src/module_navier_stokes.f90:2459-2498 compute_v_conv_fluxes
__device__ __forceinline__ void v_fluxes(const MomArgs& a, int i, int j, double& FE, double& FW,
                                         double& FN, double& FS) {
  const Dims& D = a.D;
  const double* ub = a.ab2 ? a.u_old : a.u_n;
  const double* vb = a.ab2 ? a.v_old : a.v_n;
  double vn = vb[D.id(i, j)], vnN = vb[D.id(i, j + 1)], vnS = vb[D.id(i, j - 1)];
  double unE = 0.5 * (ub[D.id(i + 1, j - 1)] + ub[D.id(i + 1, j)]);
  double unW = 0.5 * (ub[D.id(i, j - 1)] + ub[D.id(i, j)]);
  if (a.ab2_ext) {
    vn = 2.0 * vn - a.v_nm1[D.id(i, j)];
    vnN = 2.0 * vnN - a.v_nm1[D.id(i, j + 1)];
    vnS = 2.0 * vnS - a.v_nm1[D.id(i, j - 1)];
    const double umE = 0.5 * (a.u_nm1[D.id(i + 1, j - 1)] + a.u_nm1[D.id(i + 1, j)]);
    const double umW = 0.5 * (a.u_nm1[D.id(i, j - 1)] + a.u_nm1[D.id(i, j)]);
    unE = 2.0 * unE - umE;
    unW = 2.0 * unW - umW;
  }
  FE = unE * a.dy;
  FW = unW * a.dy;
  FN = 0.5 * (vn + vnN) * a.dx;
  FS = 0.5 * (vnS + vn) * a.dx;
}

// Operand sources of mom_apply_gen.
struct XSrc {
  const MomArgs& a;
  const double* xu;
  const double* xv;
  __device__ __forceinline__ double u(int i, int j) const { return tu(a, xu, i, j); }
  __device__ __forceinline__ double v(int i, int j) const { return tv(a, xv, i, j); }
};

// A row of the operator as a linear form over 9 slots: same component
// centre, east, west, north, south (0-4) and the 4 cross-component values the
// row reads (5-8; u rows: v(i,j+1), v(i-1,j+1), v(i,j), v(i-1,j); v rows:
// u(i+1,j), u(i+1,j-1), u(i,j), u(i,j-1)).  Wall ghosts fold into the slots
// of the DOFs they are built from.
struct LF {
  double c[9];
};
__device__ __forceinline__ LF lf_zero() { LF r; for (int q = 0; q < 9; ++q) r.c[q] = 0.0; return r; }
__device__ __forceinline__ LF lf_unit(int q) { LF r = lf_zero(); if (q >= 0) r.c[q] = 1.0; return r; }
__device__ __forceinline__ LF operator+(const LF& x, const LF& y) { LF r; for (int q = 0; q < 9; ++q) r.c[q] = x.c[q] + y.c[q]; return r; }
__device__ __forceinline__ LF operator-(const LF& x, const LF& y) { LF r; for (int q = 0; q < 9; ++q) r.c[q] = x.c[q] - y.c[q]; return r; }
// constant - form: the constants of the ghost formulas are the homogeneous wall values, 0
__device__ __forceinline__ LF operator-(double, const LF& y) { LF r; for (int q = 0; q < 9; ++q) r.c[q] = -y.c[q]; return r; }
__device__ __forceinline__ LF operator*(double x, const LF& y) { LF r; for (int q = 0; q < 9; ++q) r.c[q] = x * y.c[q]; return r; }
__device__ __forceinline__ LF operator*(const LF& y, double x) { return x * y; }
// one FP64 division per form, not nine: the assembled rows feed only the
// Krylov solves, which already differ from the matrix-free product at
// round-off (the product itself, XSrc, divides exactly as the reference)
__device__ __forceinline__ LF operator/(const LF& y, double x) {
  const double rx = 1.0 / x;
  LF r;
  for (int q = 0; q < 9; ++q) r.c[q] = y.c[q] * rx;
  return r;
}

struct LFSrc {
  const MomArgs& a;
  int part, i0, j0;
  // slot of DOF (i, j) of component comp (0 u, 1 v) in this row, -1 if none
  __device__ int slot(int comp, int i, int j) const {
    if (comp == part) {
      if (i == i0 && j == j0) return 0;
      if (i == i0 + 1 && j == j0) return 1;
      if (i == i0 - 1 && j == j0) return 2;
      if (i == i0 && j == j0 + 1) return 3;
      if (i == i0 && j == j0 - 1) return 4;
      return -1;
    }
    if (part == 0) {  // v values read by a u row
      if (i == i0 && j == j0 + 1) return 5;
      if (i == i0 - 1 && j == j0 + 1) return 6;
      if (i == i0 && j == j0) return 7;
      if (i == i0 - 1 && j == j0) return 8;
      return -1;
    }
    if (i == i0 + 1 && j == j0) return 5;  // u values read by a v row
    if (i == i0 + 1 && j == j0 - 1) return 6;
    if (i == i0 && j == j0) return 7;
    if (i == i0 && j == j0 - 1) return 8;
    return -1;
  }
  // tu / tv with the operand replaced by unit forms (same ghost rules)
  __device__ LF u(int i, int j) const {
    const int ny = a.D.ny;
    if (j >= 1 && j <= ny) return i >= 1 ? lf_unit(slot(0, i, j)) : lf_zero();
    if (j == 0) {
      const LF u1 = lf_unit(slot(0, i, 1));
      if (a.bc[SB] == COVOF_BC_DIRICHLET) {
        if (ny >= 2) return (8.0 * 0.0 - 6.0 * u1 + lf_unit(slot(0, i, 2))) / 3.0;
        return 2.0 * 0.0 - u1;
      }
      return u1;
    }
    const LF un = lf_unit(slot(0, i, ny));
    if (a.bc[ST] == COVOF_BC_DIRICHLET) {
      if (ny >= 2) return (8.0 * 0.0 - 6.0 * un + lf_unit(slot(0, i, ny - 1))) / 3.0;
      return 2.0 * 0.0 - un;
    }
    return un;
  }
  __device__ LF v(int i, int j) const {
    const int nx = a.D.nx;
    if (j == 0) return lf_zero();
    if (i == 0) {
      const LF v1 = lf_unit(slot(1, 1, j));
      return a.bc[SL] == COVOF_BC_DIRICHLET ? 2.0 * 0.0 - v1 : v1;
    }
    if (i == nx + 1) {
      const LF vn = lf_unit(slot(1, nx, j));
      return a.bc[SR] == COVOF_BC_DIRICHLET ? 2.0 * 0.0 - vn : vn;
    }
    return lf_unit(slot(1, i, j));
  }
};

// (A x) at one DOF (src/module_navier_stokes.f90:474-617 for u, :624-750 for v),
// written once over a value source: src.u(i, j) / src.v(i, j) give the
// operand with its homogeneous ghost values.  Evaluated on doubles (XSrc) it
// is the operator application, bit for bit the reference's term order;
// evaluated on linear forms (LFSrc) it yields the row's coefficients.
template <class S>
__device__ auto mom_apply_gen(const MomArgs& a, int part, int i, int j, const S& src) -> decltype(src.u(0, 0)) {
  const Dims& D = a.D;
  const int nx = D.nx, ny = D.ny;
  const double dx = a.dx, dy = a.dy, dvol = dx * dy, dt = a.dt;
  const int k = D.id(i, j);
  if (part == 0) {
    const double rho = a.rho_u[k];
    const double diag_bc = ((a.alpha * rho) / dt) * dvol;
    if (i == 1) return diag_bc * src.u(1, j);        // DIRICHLET / FREESLIP west
    if (i == nx + 1) return diag_bc * src.u(nx + 1, j);
    const auto uc = src.u(i, j);
    auto val = (((a.alpha * rho) / dt) * uc) * dvol;
    const auto uE = src.u(i + 1, j), uW = src.u(i - 1, j);
    const auto uN = src.u(i, j + 1), uS = src.u(i, j - 1);
    if (a.conv) {
      double FE, FW, FN, FS;
      u_fluxes(a, i, j, FE, FW, FN, FS);
      // limiter inputs: fields_old%u around the face (:533-547)
      const double* q = a.u_n;
      const bool has_ee = i + 2 <= nx + 1, has_ww = i - 2 >= 0, has_nn = j + 2 <= ny + 1, has_ss = j - 2 >= 0;
      const double q_ee = has_ee ? q[D.id(i + 2, j)] : 0.0;
      const double q_ww = has_ww ? q[D.id(i - 2, j)] : 0.0;
      const double q_nn = has_nn ? q[D.id(i, j + 2)] : 0.0;
      const double q_ss = has_ss ? q[D.id(i, j - 2)] : 0.0;
      const double qc = q[k], qE = q[k + 1], qW = q[k - 1], qN = q[k + D.P], qS = q[k - D.P];
      const auto pE = conv_face_flux(a.scheme, FE, uc, uE, qW, qc, qE, q_ee, true, has_ee);
      const auto pW = conv_face_flux(a.scheme, FW, uW, uc, q_ww, qW, qc, qE, has_ww, true);
      const auto pN = conv_face_flux(a.scheme, FN, uc, uN, qS, qc, qN, q_nn, true, has_nn);
      const auto pS = conv_face_flux(a.scheme, FS, uS, uc, q_ss, qS, qc, qN, has_ss, true);
      val = val + rho * (pE - pW + pN - pS);
    }
    const double muE = a.mu[k], muW = a.mu[k - 1];
    const auto dE = 2.0 * muE * (uE - uc) / dx * dy;
    const auto dW = 2.0 * muW * (uc - uW) / dx * dy;
    val = val - (dE - dW);
    const double mN = a.mu_node[k + D.P], mS = a.mu_node[k];
    const auto sN = mN * ((uN - uc) / dy + (src.v(i, j + 1) - src.v(i - 1, j + 1)) / dx) * dx;
    const auto sS = mS * ((uc - uS) / dy + (src.v(i, j) - src.v(i - 1, j)) / dx) * dx;
    val = val - (sN - sS);
    if (a.r_al) {
      // :584-595: -(r_E div(i,j) - r_W div(i-1,j)) dy, div of the operand
      const auto dE = (uE - uc) / dx + (src.v(i, j + 1) - src.v(i, j)) / dy;
      const auto dW = (uc - uW) / dx + (src.v(i - 1, j + 1) - src.v(i - 1, j)) / dy;
      val = val - (a.r_al[k] * dE - a.r_al[k - 1] * dW) * dy;
    }
    return val;
  }
  const double rho = a.rho_v[k];
  const double diag_bc = ((a.alpha * rho) / dt) * dvol;
  if ((j == 1 && is_wall(a, SB)) || (j == ny + 1 && is_wall(a, ST))) return diag_bc * src.v(i, j);
  const auto vc = src.v(i, j);
  auto val = (((a.alpha * rho) / dt) * vc) * dvol;
  const auto vE = src.v(i + 1, j), vW = src.v(i - 1, j);
  const auto vN = src.v(i, j + 1), vS = src.v(i, j - 1);
  if (a.conv) {
    double FE, FW, FN, FS;
    v_fluxes(a, i, j, FE, FW, FN, FS);
    // limiter inputs: fields_old%v around the face (:666-680)
    const double* q = a.v_n;
    const bool has_ee = i + 2 <= nx + 1, has_ww = i - 2 >= 0, has_nn = j + 2 <= ny + 1, has_ss = j - 2 >= 0;
    const double q_ee = has_ee ? q[D.id(i + 2, j)] : 0.0;
    const double q_ww = has_ww ? q[D.id(i - 2, j)] : 0.0;
    const double q_nn = has_nn ? q[D.id(i, j + 2)] : 0.0;
    const double q_ss = has_ss ? q[D.id(i, j - 2)] : 0.0;
    const double qc = q[k], qE = q[k + 1], qW = q[k - 1], qN = q[k + D.P], qS = q[k - D.P];
    const auto pE = conv_face_flux(a.scheme, FE, vc, vE, qW, qc, qE, q_ee, true, has_ee);
    const auto pW = conv_face_flux(a.scheme, FW, vW, vc, q_ww, qW, qc, qE, has_ww, true);
    const auto pN = conv_face_flux(a.scheme, FN, vc, vN, qS, qc, qN, q_nn, true, has_nn);
    const auto pS = conv_face_flux(a.scheme, FS, vS, vc, q_ss, qS, qc, qN, has_ss, true);
    val = val + rho * (pE - pW + pN - pS);
  }
  const double muN = a.mu[k], muS = a.mu[k - D.P];
  const auto dN = 2.0 * muN * (vN - vc) / dy * dx;
  const auto dS = 2.0 * muS * (vc - vS) / dy * dx;
  val = val - (dN - dS);
  const double mE = a.mu_node[k + 1], mW = a.mu_node[k];
  const auto sE = mE * ((vE - vc) / dx + (src.u(i + 1, j) - src.u(i + 1, j - 1)) / dy) * dy;
  const auto sW = mW * ((vc - vW) / dx + (src.u(i, j) - src.u(i, j - 1)) / dy) * dy;
  val = val - (sE - sW);
  if (a.r_al) {
    // :711-721: -(r_N div(i,j) - r_S div(i,j-1)) dx
    const auto dN = (src.u(i + 1, j) - src.u(i, j)) / dx + (vN - vc) / dy;
    const auto dS = (src.u(i + 1, j - 1) - src.u(i, j - 1)) / dx + (vc - vS) / dy;
    val = val - (a.r_al[k] * dN - a.r_al[k - D.P] * dS) * dx;
  }
  return val;
}

__device__ double mom_apply_dof(const MomArgs& a, int part, int i, int j, const double* xu,
                                const double* xv) {
  return mom_apply_gen(a, part, i, j, XSrc{a, xu, xv});
}

// ---------------------------------------------------------------------------
// Jacobi diagonal, src/module_navier_stokes.f90:1313-1539 (diag_u / diag_v).
__global__ void k_mom_diag(MomArgs a) {
  const Dims& D = a.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int nx = D.nx, ny = D.ny;
  const double dx = a.dx, dy = a.dy, dvol = dx * dy;
  const double dt_safe = a.dt > 1.0e-30 ? a.dt : 1.0;
  const int g = D.P * (ny + 2);
  if (i <= nx + 1 && j <= ny) {
    const int k = D.id(i, j);
    const double rho = a.rho_u[k];
    double Du = ((a.alpha * rho) / dt_safe) * dvol;
    if (Du <= 1.0e-30) Du = 1.0;
    double out;
    if (i == 1 || i == nx + 1) {
      out = Du;
    } else {
      const double mue = a.mu[k], muw = a.mu[k - 1];
      const double cE = 2.0 * mue * (dy / dx), cW = 2.0 * muw * (dy / dx);
      const double cNr = a.mu_node[k + D.P] * (dx / dy);
      const double cSr = a.mu_node[k] * (dx / dy);
      double cNv = cNr, cSv = cSr, dwy = 0.0;
      if (j == 1) {
        if (a.bc[SB] == COVOF_BC_DIRICHLET) dwy = dwy + (ny >= 2 ? 3.0 * cSr : 2.0 * cSr);
        cSv = 0.0;
      }
      if (j == ny) {
        if (a.bc[ST] == COVOF_BC_DIRICHLET) dwy = dwy + (ny >= 2 ? 3.0 * cNr : 2.0 * cNr);
        cNv = 0.0;
      }
      double conv_diag = 0.0;
      if (a.conv) {
        double FE, FW, FN, FS;
        u_fluxes(a, i, j, FE, FW, FN, FS);
        conv_diag = rho * (fmax(FE, 0.0) + fmax(-FW, 0.0) + fmax(FN, 0.0) + fmax(-FS, 0.0));
      }
      double alW = 0.0, alE = 0.0;
      if (a.r_al) { alW = a.r_al[k - 1] * (dy / dx); alE = a.r_al[k] * (dy / dx); }
      double aP = Du + dwy + conv_diag + 0.0 + 0.0 + cW + cE + cSv + cNv + alW + alE;
      if (aP <= 1.0e-15) aP = 1.0;
      out = aP;
    }
    a.diag[k] = out;
  }
  if (i <= nx && j <= ny + 1) {
    const int k = D.id(i, j);
    const double rho = a.rho_v[k];
    double Dv = ((a.alpha * rho) / dt_safe) * dvol;
    if (Dv <= 1.0e-30) Dv = 1.0;
    double out;
    if ((j == 1 && is_wall(a, SB)) || (j == ny + 1 && is_wall(a, ST))) {
      out = Dv;
    } else {
      const double mun = a.mu[k], mus = a.mu[k - D.P];
      const double cN = 2.0 * mun * (dx / dy), cS = 2.0 * mus * (dx / dy);
      const double cEr = a.mu_node[k + 1] * (dy / dx);
      const double cWr = a.mu_node[k] * (dy / dx);
      double cEv = cEr, cWv = cWr, dwx = 0.0;
      if (i == 1) {
        if (a.bc[SL] == COVOF_BC_DIRICHLET) dwx = dwx + 2.0 * cWr;
        cWv = 0.0;
      }
      if (i == nx) {
        if (a.bc[SR] == COVOF_BC_DIRICHLET) dwx = dwx + 2.0 * cEr;
        cEv = 0.0;
      }
      double conv_diag = 0.0;
      if (a.conv) {
        double FE, FW, FN, FS;
        v_fluxes(a, i, j, FE, FW, FN, FS);
        conv_diag = rho * (fmax(FE, 0.0) + fmax(-FW, 0.0) + fmax(FN, 0.0) + fmax(-FS, 0.0));
      }
      double alS = 0.0, alN = 0.0;
      if (a.r_al) { alS = a.r_al[k - D.P] * (dx / dy); alN = a.r_al[k] * (dx / dy); }
      double aP = Dv + dwx + conv_diag + 0.0 + 0.0 + cWv + cEv + cS + cN + alS + alN;
      if (aP <= 1.0e-15) aP = 1.0;
      out = aP;
    }
    a.diag[g + k] = out;
  }
}

// Stencils of the sweep preconditioners, src/module_navier_stokes.f90:
// 1312-1590 (the u block :1312-1425, v block :1428-1539, Schur :1542-1590);
// the centres equal k_mom_diag's diagonals.  Every DOF entry of every array
// is written (zero where the reference leaves a coefficient at zero), so the
// arrays need no clearing between assemblies.  One thread per (i, j).
__device__ __forceinline__ void put_stencil(const Stencil& t, int k, double W, double E, double S, double N,
                                            double P) {
  // the sweeps divide by aP, or by 1 where |aP| < 1e-30
  const double d = fabs(P) < 1.0e-30 ? 1.0 : P;
  t.W[k] = W; t.E[k] = E; t.S[k] = S; t.N[k] = N; t.P[k] = d;
  t.rP[k] = __drcp_rn(d);
}

__global__ void k_prec_blocks(MomArgs a, PBlk b) {
  const Dims& D = a.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int nx = D.nx, ny = D.ny;
  const double dx = a.dx, dy = a.dy, dvol = dx * dy;
  const double dt_safe = a.dt > 1.0e-30 ? a.dt : 1.0;
  if (i <= nx + 1 && j <= ny) {
    const int k = D.id(i, j);
    const double rho = a.rho_u[k];
    double Du = ((a.alpha * rho) / dt_safe) * dvol;
    if (Du <= 1.0e-30) Du = 1.0;
    if (i == 1) {
      put_stencil(b.u, k, 0.0, (a.bc[SL] == COVOF_BC_NEUMANN && nx + 1 >= 2) ? Du : 0.0, 0.0, 0.0, Du);
    } else if (i == nx + 1) {
      put_stencil(b.u, k, (a.bc[SR] == COVOF_BC_NEUMANN && nx + 1 >= 2) ? Du : 0.0, 0.0, 0.0, 0.0, Du);
    } else {
      const double mue = a.mu[k], muw = a.mu[k - 1];
      const double cE = 2.0 * mue * (dy / dx), cW = 2.0 * muw * (dy / dx);
      const double cNr = a.mu_node[k + D.P] * (dx / dy);
      const double cSr = a.mu_node[k] * (dx / dy);
      double cNv = cNr, cSv = cSr, dwy = 0.0, cNx = 0.0, cSx = 0.0;
      if (j == 1) {
        if (a.bc[SB] == COVOF_BC_DIRICHLET) {
          if (ny >= 2) { dwy = dwy + 3.0 * cSr; cNx = cNx + cSr / 3.0; }
          else dwy = dwy + 2.0 * cSr;
        }
        cSv = 0.0;
      }
      if (j == ny) {
        if (a.bc[ST] == COVOF_BC_DIRICHLET) {
          if (ny >= 2) { dwy = dwy + 3.0 * cNr; cSx = cSx + cNr / 3.0; }
          else dwy = dwy + 2.0 * cNr;
        }
        cNv = 0.0;
      }
      double cd = 0.0, cvW = 0.0, cvE = 0.0, cvS = 0.0, cvN = 0.0;
      if (a.conv) {
        double FE, FW, FN, FS;
        u_fluxes(a, i, j, FE, FW, FN, FS);
        cd = rho * (fmax(FE, 0.0) + fmax(-FW, 0.0) + fmax(FN, 0.0) + fmax(-FS, 0.0));
        cvE = rho * fmax(-FE, 0.0);
        cvW = rho * fmax(FW, 0.0);
        cvN = (j == ny) ? 0.0 : rho * fmax(-FN, 0.0);
        cvS = (j == 1) ? 0.0 : rho * fmax(FS, 0.0);
      }
      double alE = 0.0, alW = 0.0;
      if (a.r_al) { alE = a.r_al[k] * (dy / dx); alW = a.r_al[k - 1] * (dy / dx); }
      double aP = Du + dwy + cd + 0.0 + 0.0 + cW + cE + cSv + cNv + alW + alE;
      if (aP <= 1.0e-15) aP = 1.0;
      put_stencil(b.u, k, cW + cvW + alW, cE + cvE + alE, cSv + cvS + cSx, cNv + cvN + cNx, aP);
    }
  }
  if (i <= nx && j <= ny + 1) {
    const int k = D.id(i, j);
    const double rho = a.rho_v[k];
    double Dv = ((a.alpha * rho) / dt_safe) * dvol;
    if (Dv <= 1.0e-30) Dv = 1.0;
    if ((j == 1 && is_wall(a, SB)) || (j == ny + 1 && is_wall(a, ST))) {
      put_stencil(b.v, k, 0.0, 0.0, 0.0, 0.0, Dv);
    } else if (j == 1 && a.bc[SB] == COVOF_BC_NEUMANN && ny + 1 >= 2) {
      put_stencil(b.v, k, 0.0, 0.0, 0.0, Dv, Dv);
    } else if (j == ny + 1 && a.bc[ST] == COVOF_BC_NEUMANN && ny + 1 >= 2) {
      put_stencil(b.v, k, 0.0, 0.0, Dv, 0.0, Dv);
    } else {
      const double mun = a.mu[k], mus = a.mu[k - D.P];
      const double cN = 2.0 * mun * (dx / dy), cS = 2.0 * mus * (dx / dy);
      const double cEr = a.mu_node[k + 1] * (dy / dx);
      const double cWr = a.mu_node[k] * (dy / dx);
      double cEv = cEr, cWv = cWr, dwx = 0.0;
      if (i == 1) {
        if (a.bc[SL] == COVOF_BC_DIRICHLET) dwx = dwx + 2.0 * cWr;
        cWv = 0.0;
      }
      if (i == nx) {
        if (a.bc[SR] == COVOF_BC_DIRICHLET) dwx = dwx + 2.0 * cEr;
        cEv = 0.0;
      }
      double cd = 0.0, cvW = 0.0, cvE = 0.0, cvS = 0.0, cvN = 0.0;
      if (a.conv) {
        double FE, FW, FN, FS;
        v_fluxes(a, i, j, FE, FW, FN, FS);
        cd = rho * (fmax(FE, 0.0) + fmax(-FW, 0.0) + fmax(FN, 0.0) + fmax(-FS, 0.0));
        cvE = (i == nx) ? 0.0 : rho * fmax(-FE, 0.0);
        cvW = (i == 1) ? 0.0 : rho * fmax(FW, 0.0);
        cvN = rho * fmax(-FN, 0.0);
        cvS = rho * fmax(FS, 0.0);
      }
      double alN = 0.0, alS = 0.0;
      if (a.r_al) { alN = a.r_al[k] * (dx / dy); alS = a.r_al[k - D.P] * (dx / dy); }
      double aP = Dv + dwx + cd + 0.0 + 0.0 + cWv + cEv + cS + cN + alS + alN;
      if (aP <= 1.0e-15) aP = 1.0;
      put_stencil(b.v, k, cWv + cvW, cEv + cvE, cS + cvS + alS, cN + cvN + alN, aP);
    }
  }
}

// The Schur stencil from the u / v centres (after k_prec_blocks).
__global__ void k_prec_schur(MomArgs a, PBlk b) {
  const Dims& D = a.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > D.nx || j > D.ny) return;
  const double dx = a.dx, dy = a.dy, dvol = dx * dy;
  double sW = 0.0, sE = 0.0, sS = 0.0, sN = 0.0;
  if (!(i == 1 && is_wall(a, SL))) sW = __ddiv_rn(dy * dy, fmax(1.0e-30, b.u.P[D.id(i, j)]));
  if (!(i == D.nx && is_wall(a, SR))) sE = __ddiv_rn(dy * dy, fmax(1.0e-30, b.u.P[D.id(i + 1, j)]));
  if (!(j == 1 && is_wall(a, SB))) sS = __ddiv_rn(dx * dx, fmax(1.0e-30, b.v.P[D.id(i, j)]));
  if (!(j == D.ny && is_wall(a, ST))) sN = __ddiv_rn(dx * dx, fmax(1.0e-30, b.v.P[D.id(i, j + 1)]));
  const double reg = (i == 1 && j == 1) ? 1.0e-10 * dvol : 1.0e-12 * dvol;
  put_stencil(b.s, D.id(i, j), sW, sE, sS, sN, sW + sE + sS + sN + 0.0 + reg);
}

// Right-hand side, src/module_navier_stokes.f90:817-1088 (SP, constant walls;
// Euler, or the Gear / BDF2 inertial term rho (2 u^n - u^(n-1) / 2) / dt).
__global__ void k_mom_rhs(MomArgs a) {
  const Dims& D = a.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int nx = D.nx, ny = D.ny;
  const double dx = a.dx, dy = a.dy, dvol = dx * dy, dt = a.dt;
  const int g = D.P * (ny + 2);
  if (i <= nx + 1 && j <= ny) {
    const int k = D.id(i, j);
    const double rho = a.rho_u[k];
    const double diag_bc = ((a.alpha * rho) / dt) * dvol;
    double out;
    if (i == 1) {
      out = diag_bc * (a.bc[SL] == COVOF_BC_DIRICHLET ? a.bcu[SL] : 0.0);
    } else if (i == nx + 1) {
      out = diag_bc * (a.bc[SR] == COVOF_BC_DIRICHLET ? a.bcu[SR] : 0.0);
    } else {
      double val;
      if (a.gear_rhs) {
        const double u_in = rho * (2.0 * a.u_old[k] - 0.5 * a.u_nm1[k]);
        val = (u_in / dt) * dvol;
      } else {
        val = (rho / dt) * a.u_old[k] * dvol;
      }
      val = val + rho * a.gx * dvol;
      val = val + a.fx[k] * dvol;
      if (a.p_al) val = val - (a.p_al[k] - a.p_al[k - 1]) * dy;  // :908-913
      if (j == ny && a.bc[ST] == COVOF_BC_DIRICHLET) {
        const double mN = a.mu_node[k + D.P];
        if (ny >= 2) val = val + mN * ((8.0 / 3.0) * a.bcu[ST] / dy) * dx;
        else val = val + mN * (2.0 * a.bcu[ST] / dy) * dx;
      }
      if (j == 1 && a.bc[SB] == COVOF_BC_DIRICHLET) {
        const double mS = a.mu_node[k];
        if (ny >= 2) val = val + mS * ((8.0 / 3.0) * a.bcu[SB] / dy) * dx;
        else val = val + mS * (2.0 * a.bcu[SB] / dy) * dx;
      }
      out = val;
    }
    a.rhs[k] = out;
  }
  if (i <= nx && j <= ny + 1) {
    const int k = D.id(i, j);
    const double rho = a.rho_v[k];
    const double diag_bc = ((a.alpha * rho) / dt) * dvol;
    double out;
    if (j == 1 && is_wall(a, SB)) {
      out = diag_bc * (a.bc[SB] == COVOF_BC_DIRICHLET ? a.bcv[SB] : 0.0);
    } else if (j == ny + 1 && is_wall(a, ST)) {
      out = diag_bc * (a.bc[ST] == COVOF_BC_DIRICHLET ? a.bcv[ST] : 0.0);
    } else {
      double val;
      if (a.gear_rhs) {
        const double v_in = rho * (2.0 * a.v_old[k] - 0.5 * a.v_nm1[k]);
        val = (v_in / dt) * dvol;
      } else {
        val = (rho / dt) * a.v_old[k] * dvol;
      }
      val = val + rho * a.gy * dvol;
      val = val + a.fy[k] * dvol;
      if (a.p_al) val = val - (a.p_al[k] - a.p_al[k - D.P]) * dx;  // :1053-1058
      if (i == 1 && a.bc[SL] == COVOF_BC_DIRICHLET) {
        const double mW = a.mu_node[k];
        val = val + mW * (2.0 * a.bcv[SL] / dx) * dy;
      }
      if (i == nx && a.bc[SR] == COVOF_BC_DIRICHLET) {
        const double mE = a.mu_node[k + 1];
        val = val + mE * (2.0 * a.bcv[SR] / dx) * dy;
      }
      out = val;
    }
    a.rhs[g + k] = out;
  }
}

// One operator application over all DOFs (tests; also the reference's
// ns_apply_system_matrix on unpacked vectors).
__global__ void k_mom_apply(MomArgs a, const double* xu, const double* xv, double* yu, double* yv) {
  const Dims& D = a.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i <= D.nx + 1 && j <= D.ny) yu[D.id(i, j)] = mom_apply_dof(a, 0, i, j, xu, xv);
  if (i <= D.nx && j <= D.ny + 1) yv[D.id(i, j)] = mom_apply_dof(a, 1, i, j, xu, xv);
}

// Rows of the operator for the Krylov solve (coef: 9 slots x 2g, slot-major)
// and the inverse Jacobi diagonal (after k_mom_diag).  One thread per DOF.
__global__ void k_mom_assemble(MomArgs a) {
  const Dims& D = a.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int g = D.P * (D.ny + 2);
  const size_t g2 = 2 * (size_t)g;
  for (int part = 0; part < 2; ++part) {
    const bool in = part == 0 ? (i <= D.nx + 1 && j <= D.ny) : (i <= D.nx && j <= D.ny + 1);
    if (!in) continue;
    const int k = (part == 0 ? 0 : g) + D.id(i, j);
    const LF row = mom_apply_gen(a, part, i, j, LFSrc{a, part, i, j});
    for (int q = 0; q < 9; ++q) a.coef[q * g2 + k] = row.c[q];
    const double d = a.diag[k];
    a.idiag[k] = (a.precond_on && fabs(d) > 1.0e-15) ? 1.0 / d : 1.0;
  }
}

// The pressure block's Jacobi diagonal for MONOLITHIC,
// src/module_navier_stokes.f90:1541-1590: diag_p = schur_aP, the row sum of
// B D^-1 B^T from the momentum diagonals (after k_mom_diag), plus 1e-10 dvol
// in cell (1,1) and 1e-12 dvol elsewhere.  One thread per cell.
__global__ void k_mono_diag(MomArgs a) {
  const Dims& D = a.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > D.nx || j > D.ny) return;
  const int g = D.P * (D.ny + 2);
  const double dx = a.dx, dy = a.dy, dvol = dx * dy;
  const double* du = a.diag;
  const double* dv = a.diag + g;
  double aW = 0.0, aE = 0.0, aS = 0.0, aN = 0.0;
  if (!(i == 1 && is_wall(a, SL))) aW = __ddiv_rn(dy * dy, fmax(1.0e-30, du[D.id(i, j)]));
  if (!(i == D.nx && is_wall(a, SR))) aE = __ddiv_rn(dy * dy, fmax(1.0e-30, du[D.id(i + 1, j)]));
  if (!(j == 1 && is_wall(a, SB))) aS = __ddiv_rn(dx * dx, fmax(1.0e-30, dv[D.id(i, j)]));
  if (!(j == D.ny && is_wall(a, ST))) aN = __ddiv_rn(dx * dx, fmax(1.0e-30, dv[D.id(i, j + 1)]));
  const double reg = (i == 1 && j == 1) ? 1.0e-10 * dvol : 1.0e-12 * dvol;
  const double d = aW + aE + aS + aN + 0.0 + reg;
  const size_t k = 2 * (size_t)g + D.id(i, j);
  a.diag[k] = d;
  a.idiag[k] = (a.precond_on && fabs(d) > 1.0e-15) ? 1.0 / d : 1.0;
}

// ---------------------------------------------------------------------------
// Persistent Krylov solvers.  DOF ownership: warp w walks 32-wide row
// segments of the u block, then of the v block, then (MONOLITHIC) of the
// pressure block.
struct DofWalker {
  int nsu, nsv, nsp, su, suv, stot, gw, nw, lane, g;
  __device__ DofWalker(const Dims& D, const Team& tm, int mono = 0) {
    nsu = (D.nx + 1 + 31) >> 5;
    nsv = (D.nx + 31) >> 5;
    nsp = nsv;
    su = nsu * D.ny;
    suv = su + nsv * (D.ny + 1);
    stot = suv + (mono ? nsp * D.ny : 0);
    lane = threadIdx.x & 31;
    gw = (tm.rank * (int)blockDim.x + (int)threadIdx.x) >> 5;
    nw = (tm.size * (int)blockDim.x) >> 5;
    g = D.P * (D.ny + 2);
  }
  // Decode segment s; returns false when this lane has no DOF there.
  __device__ __forceinline__ bool at(const Dims& D, int s, int& part, int& i, int& j, int& k) const {
    if (s < su) {
      part = 0; j = s / nsu + 1; i = (s - (j - 1) * nsu) * 32 + lane + 1;
      if (i > D.nx + 1) return false;
      k = D.id(i, j);
    } else if (s < suv) {
      const int t = s - su;
      part = 1; j = t / nsv + 1; i = (t - (j - 1) * nsv) * 32 + lane + 1;
      if (i > D.nx) return false;
      k = g + D.id(i, j);
    } else {
      const int t = s - suv;
      part = 2; j = t / nsp + 1; i = (t - (j - 1) * nsp) * 32 + lane + 1;
      if (i > D.nx) return false;
      k = 2 * g + D.id(i, j);
    }
    return true;
  }
};
#define FOR_DOFS(A, W, part, i, j, k)                                 \
  for (int s_ = (W).gw; s_ < (W).stot; s_ += (W).nw)                 \
    for (int part = 0, i = 0, j = 0, k = 0, once_ = (W).at((A).D, s_, part, i, j, k); once_; once_ = 0)

// Jacobi preconditioner (src/module_linear_solvers.f90:88-135): a multiply by
// the inverse diagonal k_mom_assemble stored (1 where the reference skips
// the division).
__device__ __forceinline__ double prec(const MomArgs& a, int k, double src) { return src * a.idiag[k]; }

// y = M^-1 A x (or A x when with_prec = false) at own DOFs, from the
// assembled rows: 9 FMAs instead of the matrix-free expression (which costs
// tens of FP64 divisions per DOF; FP64 issue bounds these solves on GB300).
// Wall rows keep only their centre coefficient and read nothing else.
// MONOLITHIC: momentum rows add B^T p, (p(i,j) - p(i-1,j)) dy for u and
// (p(i,j) - p(i,j-1)) dx for v (src/module_navier_stokes.f90:597-602,
// 723-728); continuity rows are div u dvol (as (du) dy + (dv) dx) plus
// 1e-10 dvol p(1,1) in cell (1,1) (:730-777).
__device__ __forceinline__ double pa_at(const MomArgs& a, const DofWalker& W, int part, int i,
                                        int j, int k, const double* x, bool with_prec) {
  const Dims& D = a.D;
  const size_t g2 = 2 * (size_t)W.g;
  if (part == 2) {
    const int ku = k - 2 * W.g, kv = ku + W.g;
    double y = (__ldcg(x + ku + 1) - __ldcg(x + ku)) * a.dy + (__ldcg(x + kv + D.P) - __ldcg(x + kv)) * a.dx;
    if (i == 1 && j == 1) y = y + (1.0e-10 * (a.dx * a.dy)) * __ldcg(x + k);
    return with_prec ? y * a.idiag[k] : y;
  }
  const double* __restrict__ cf = a.coef;
  double y = cf[k] * __ldcg(x + k);
  const bool wall_row = part == 0 ? (i == 1 || i == D.nx + 1)
                                  : ((j == 1 && is_wall(a, SB)) || (j == D.ny + 1 && is_wall(a, ST)));
  // checked builds: a row that reads neighbours has its neighbourhood in its block
  if (!wall_row && D.nbhd(k - part * W.g, 7) != k - part * W.g) return 0.0;
  if (!wall_row) {
    const int P = D.P;
    const int o = part == 0 ? W.g : -W.g;  // offset of the other component's block
    const int kc = k + o;                   // same (i, j) in the other block
    y = fma(cf[1 * g2 + k], __ldcg(x + k + 1), y);
    y = fma(cf[2 * g2 + k], __ldcg(x + k - 1), y);
    y = fma(cf[3 * g2 + k], __ldcg(x + k + P), y);
    y = fma(cf[4 * g2 + k], __ldcg(x + k - P), y);
    if (part == 0) {
      y = fma(cf[5 * g2 + k], __ldcg(x + kc + P), y);
      y = fma(cf[6 * g2 + k], __ldcg(x + kc + P - 1), y);
      y = fma(cf[7 * g2 + k], __ldcg(x + kc), y);
      y = fma(cf[8 * g2 + k], __ldcg(x + kc - 1), y);
    } else {
      y = fma(cf[5 * g2 + k], __ldcg(x + kc + 1), y);
      y = fma(cf[6 * g2 + k], __ldcg(x + kc + 1 - P), y);
      y = fma(cf[7 * g2 + k], __ldcg(x + kc), y);
      y = fma(cf[8 * g2 + k], __ldcg(x + kc - P), y);
    }
    if (a.mono) {
      // the same (i, j) in the pressure block, and its west / south neighbour
      const int kp = k + (part == 0 ? 2 * W.g : W.g);
      y = y + (__ldcg(x + kp) - __ldcg(x + kp - (part == 0 ? 1 : P))) * (part == 0 ? a.dy : a.dx);
    }
  }
  return with_prec ? y * a.idiag[k] : y;
}

// y = A x at every DOF from the assembled rows (one launch; the Krylov
// iterations driven from the host for the sweep preconditioners).
__global__ void k_mom_matvec(MomArgs a, const double* x, double* y) {
  const Team tm{(int)blockIdx.x, (int)gridDim.x};
  DofWalker W(a.D, tm, a.mono);
  FOR_DOFS(a, W, part, i, j, k) y[k] = pa_at(a, W, part, i, j, k, x, false);
}

struct KCtx {
  GridReducer R;
  bool ok;
};

__device__ void krylov_finish(const MomArgs& a, const Team& tm, int iters, int status, bool ok) {
  if (tm.rank == 0 && threadIdx.x == 0) {
    a.res->iters = iters;
    a.res->status = ok ? status : COVOF_TIMEOUT;
  }
}

// src/module_linear_solvers.f90:584-730 solve_bicgstab (left Jacobi).
// Every division and square root of the recurrences runs once per block, in
// thread 0, inside the reductions (GridReducer::sum_map), and is broadcast:
// FP64 issue is the scarce resource of a GB300 SM.
__device__ void bicgstab_case(const MomArgs& a, const Team& tm, GridReducer& R) {
  DofWalker W(a.D, tm, a.mono);
  double *x = a.x, *bh = a.v0, *r = a.v1, *rt = a.v2, *p = a.v3, *v = a.v4, *s = a.v5, *t = a.v6;
  const double tol = a.tol;
  const int max_iter = a.max_iter;
  // b_hat = M^-1 b ; r = b_hat - M^-1 A x ; ||r||
  double acc[1] = {0.0};
  FOR_DOFS(a, W, part, i, j, k) {
    const double bb = prec(a, k, a.rhs[k]);
    bh[k] = bb;
    const double rr = bb - pa_at(a, W, part, i, j, k, x, true);
    r[k] = rr; rt[k] = rr;
    acc[0] += rr * rr;
  }
  double o0[2];
  bool ok = R.sum_map<1, 2>(acc, o0, [&](const double* w, double* o) { o[0] = w[0]; o[1] = sqrt(w[0]); });
  const double rsq0 = o0[0];
  const double r0 = o0[1];
  if (!ok || r0 < 1.0e-12) { krylov_finish(a, tm, 0, COVOF_OK, ok); return; }
  double rho_old = 1.0, alpha = 1.0, omega = 1.0, rho = rsq0, beta = 0.0;
  int iters = max_iter, status = COVOF_MAXITER;
  for (int it = 1; it <= max_iter && ok; ++it) {
    if (fabs(rho) < 1.0e-30) { status = COVOF_BREAKDOWN; break; }
    // beta = (rho / rho_old) (alpha / omega), formed in the previous reduction
    FOR_DOFS(a, W, part, i, j, k) {
      p[k] = (it == 1) ? r[k] : r[k] + beta * (p[k] - omega * v[k]);
    }
    ok = R.gs.sync();
    if (!ok) break;
    double a1[1] = {0.0};
    FOR_DOFS(a, W, part, i, j, k) {
      const double vv = pa_at(a, W, part, i, j, k, p, true);
      v[k] = vv;
      a1[0] += rt[k] * vv;
    }
    double o1[2];
    ok = R.sum_map<1, 2>(a1, o1, [&](const double* w, double* o) {
      o[0] = w[0];
      o[1] = fabs(w[0]) < 1.0e-30 ? 0.0 : rho / w[0];
    });
    if (!ok) break;
    if (fabs(o1[0]) < 1.0e-30) { status = COVOF_BREAKDOWN; break; }
    alpha = o1[1];
    double a2[1] = {0.0};
    FOR_DOFS(a, W, part, i, j, k) {
      const double sv = r[k] - alpha * v[k];
      s[k] = sv;
      a2[0] += sv * sv;
    }
    double o2[2];
    ok = R.sum_map<1, 2>(a2, o2, [&](const double* w, double* o) {
      const double sn = sqrt(w[0]);
      o[0] = sn;
      o[1] = sn / r0;
    });
    if (!ok) break;
    const double sn = o2[0];
    if (sn != sn || sn > 1.0e30) { status = COVOF_NAN; break; }
    if (o2[1] < tol || sn < 1.0e-12) {
      FOR_DOFS(a, W, part, i, j, k) x[k] = x[k] + alpha * p[k];
      iters = it; status = COVOF_OK;
      break;
    }
    double a3[2] = {0.0, 0.0};
    FOR_DOFS(a, W, part, i, j, k) {
      const double tt = pa_at(a, W, part, i, j, k, s, true);
      t[k] = tt;
      a3[0] += tt * tt;
      a3[1] += tt * s[k];
    }
    double o3[1];
    ok = R.sum_map<2, 1>(a3, o3, [&](const double* w, double* o) { o[0] = w[0] > 1.0e-30 ? w[1] / w[0] : 0.0; });
    if (!ok) break;
    omega = o3[0];
    double a4[2] = {0.0, 0.0};
    FOR_DOFS(a, W, part, i, j, k) {
      x[k] = x[k] + alpha * p[k] + omega * s[k];
      const double rr = s[k] - omega * t[k];
      r[k] = rr;
      a4[0] += rr * rr;
      a4[1] += rt[k] * rr;  // next iteration's rho = <r~, r>
    }
    double o4[4];
    ok = R.sum_map<2, 4>(a4, o4, [&](const double* w, double* o) {
      const double rn = sqrt(w[0]);
      o[0] = rn;
      o[1] = rn / r0;
      // the next iteration's beta (rho_old is this iteration's rho)
      o[2] = (w[1] / rho) * (alpha / omega);
      o[3] = w[1];
    });
    if (!ok) break;
    rho_old = rho;
    rho = o4[3];
    beta = o4[2];
    const double rn = o4[0];
    if (rn != rn || rn > 1.0e30) { status = COVOF_NAN; break; }
    if (o4[1] < tol || rn < 1.0e-12) { iters = it; status = COVOF_OK; break; }
    if (fabs(omega) < 1.0e-30) { status = COVOF_BREAKDOWN; break; }
  }
  (void)rho_old;
  krylov_finish(a, tm, iters, status, ok);
}

__global__ void __launch_bounds__(512) k_bicgstab(MomArgs a) {
  const Team tm = grid_team();
  GridReducer R{a.part, GridSync{a.bar, a.err, (unsigned)tm.size, 0u}, 0, tm.rank};
  bicgstab_case(a, tm, R);
}

// src/module_linear_solvers.f90:735-838 solve_cg (unpreconditioned operator,
// separate Jacobi application).
__device__ void cg_case(const MomArgs& a, const Team& tm, GridReducer& R) {
  DofWalker W(a.D, tm, a.mono);
  double *x = a.x, *r = a.v1, *p = a.v3, *Ap = a.v4;
  const double tol = a.tol;
  const int max_iter = a.max_iter;
  double acc[2] = {0.0, 0.0};
  FOR_DOFS(a, W, part, i, j, k) {
    const double rr = a.rhs[k] - pa_at(a, W, part, i, j, k, x, false);
    r[k] = rr;
    const double z = prec(a, k, rr);
    p[k] = z;
    acc[0] += rr * rr;
    acc[1] += rr * z;
  }
  double o0[2];
  bool ok = R.sum_map<2, 2>(acc, o0, [&](const double* w, double* o) { o[0] = sqrt(w[0]); o[1] = w[1]; });
  const double r0 = o0[0];
  if (!ok || r0 < 1.0e-12) { krylov_finish(a, tm, 0, COVOF_OK, ok); return; }
  double rz_old = o0[1];
  int iters = max_iter, status = COVOF_MAXITER;
  for (int it = 1; it <= max_iter && ok; ++it) {
    double a1[1] = {0.0};
    FOR_DOFS(a, W, part, i, j, k) {
      const double y = pa_at(a, W, part, i, j, k, p, false);
      Ap[k] = y;
      a1[0] += p[k] * y;
    }
    double o1[2];
    ok = R.sum_map<1, 2>(a1, o1, [&](const double* w, double* o) {
      o[0] = w[0];
      o[1] = fabs(w[0]) < 1.0e-30 ? 0.0 : rz_old / w[0];
    });
    if (!ok) break;
    if (fabs(o1[0]) < 1.0e-30) { status = COVOF_BREAKDOWN; break; }
    const double alpha = o1[1];
    double a2[2] = {0.0, 0.0};
    FOR_DOFS(a, W, part, i, j, k) {
      x[k] = x[k] + alpha * p[k];
      const double rr = r[k] - alpha * Ap[k];
      r[k] = rr;
      a2[0] += rr * rr;
      a2[1] += rr * prec(a, k, rr);
    }
    double o2[4];
    ok = R.sum_map<2, 4>(a2, o2, [&](const double* w, double* o) {
      const double rn = sqrt(w[0]);
      o[0] = rn;
      o[1] = rn / r0;
      o[2] = w[1] / rz_old;  // beta
      o[3] = w[1];
    });
    if (!ok) break;
    const double rn = o2[0];
    if (o2[1] < tol || rn < 1.0e-13) { iters = it; status = COVOF_OK; break; }
    const double beta = o2[2];
    rz_old = o2[3];
    FOR_DOFS(a, W, part, i, j, k) p[k] = prec(a, k, r[k]) + beta * p[k];
    ok = R.gs.sync();
  }
  krylov_finish(a, tm, iters, status, ok);
}

__global__ void __launch_bounds__(512) k_cg(MomArgs a) {
  const Team tm = grid_team();
  GridReducer R{a.part, GridSync{a.bar, a.err, (unsigned)tm.size, 0u}, 0, tm.rank};
  cg_case(a, tm, R);
}

// src/module_linear_solvers.f90:361-579 solve_bicgstab2 (left Jacobi).
// Divisions and square roots run once per block inside the reductions, as
// in bicgstab_case; each reduction also forms the next step's coefficients.
__device__ void bicgstab2_case(const MomArgs& a, const Team& tm, GridReducer& R) {
  DofWalker W(a.D, tm, a.mono);
  double *x = a.x, *rt = a.v0, *r0 = a.v1, *r1 = a.v2, *r2 = a.v3, *u0 = a.v4, *u1 = a.v5, *u2 = a.v6;
  const double tol = a.tol;
  const int max_iter = a.max_iter;
  double acc[1] = {0.0};
  FOR_DOFS(a, W, part, i, j, k) {
    const double bb = prec(a, k, a.rhs[k]);
    const double rr = bb - pa_at(a, W, part, i, j, k, x, true);
    r0[k] = rr; rt[k] = rr;
    u0[k] = 0.0; u1[k] = 0.0; u2[k] = 0.0; r1[k] = 0.0; r2[k] = 0.0;
    acc[0] += rr * rr;
  }
  double rho0 = 1.0, alpha = 0.0, omega = 1.0;
  // the loop head's rho0 = -omega rho0 and beta = alpha (rho1 / rho0), with
  // rho1 = <r~, r0>, formed in the reduction before it
  auto head = [&](double rho1, double* o) {
    const double rn0 = -omega * rho0;
    o[0] = rn0;
    o[1] = alpha * (rho1 / rn0);
    o[2] = rho1;
  };
  double i0[4];
  bool ok = R.sum_map<1, 4>(acc, i0, [&](const double* w, double* o) {
    head(w[0], o);
    o[3] = sqrt(w[0]);
  });
  const double r0n = i0[3];
  if (!ok || r0n < 1.0e-12) { krylov_finish(a, tm, 0, COVOF_OK, ok); return; }
  double hd[3] = {i0[0], i0[1], i0[2]};
  int iter = 0, status = COVOF_MAXITER;
  while (iter < max_iter && ok) {
    iter += 2;
    rho0 = hd[0];
    if (fabs(rho0) < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    double beta = hd[1];
    rho0 = hd[2];
    FOR_DOFS(a, W, part, i, j, k) u0[k] = r0[k] - beta * u0[k];
    ok = R.gs.sync();
    if (!ok) break;
    double g1[1] = {0.0};
    FOR_DOFS(a, W, part, i, j, k) {
      const double y = pa_at(a, W, part, i, j, k, u0, true);
      u1[k] = y;
      g1[0] += rt[k] * y;
    }
    double o1[2];
    ok = R.sum_map<1, 2>(g1, o1, [&](const double* w, double* o) {
      o[0] = w[0];
      o[1] = fabs(w[0]) < 1.0e-300 ? 0.0 : rho0 / w[0];
    });
    if (!ok) break;
    if (fabs(o1[0]) < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    alpha = o1[1];
    FOR_DOFS(a, W, part, i, j, k) {
      r0[k] = r0[k] - alpha * u1[k];
      x[k] = x[k] + alpha * u0[k];
    }
    ok = R.gs.sync();
    if (!ok) break;
    double g2[1] = {0.0};
    FOR_DOFS(a, W, part, i, j, k) {
      const double y = pa_at(a, W, part, i, j, k, r0, true);
      r1[k] = y;
      g2[0] += rt[k] * y;
    }
    double o2[2];
    ok = R.sum_map<1, 2>(g2, o2, [&](const double* w, double* o) {
      o[0] = w[0];
      o[1] = alpha * (w[0] / rho0);
    });
    if (!ok) break;
    if (fabs(rho0) < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    beta = o2[1];
    rho0 = o2[0];
    FOR_DOFS(a, W, part, i, j, k) {
      u0[k] = r0[k] - beta * u0[k];
      u1[k] = r1[k] - beta * u1[k];
    }
    ok = R.gs.sync();
    if (!ok) break;
    double g3[1] = {0.0};
    FOR_DOFS(a, W, part, i, j, k) {
      const double y = pa_at(a, W, part, i, j, k, u1, true);
      u2[k] = y;
      g3[0] += rt[k] * y;
    }
    double o3[2];
    ok = R.sum_map<1, 2>(g3, o3, [&](const double* w, double* o) {
      o[0] = w[0];
      o[1] = fabs(w[0]) < 1.0e-300 ? 0.0 : rho0 / w[0];
    });
    if (!ok) break;
    if (fabs(o3[0]) < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    alpha = o3[1];
    FOR_DOFS(a, W, part, i, j, k) {
      x[k] = x[k] + alpha * u0[k];
      r0[k] = r0[k] - alpha * u1[k];
      r1[k] = r1[k] - alpha * u2[k];
    }
    ok = R.gs.sync();
    if (!ok) break;
    double sg[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    FOR_DOFS(a, W, part, i, j, k) {
      const double y = pa_at(a, W, part, i, j, k, r1, true);
      r2[k] = y;
      sg[0] += r1[k] * r1[k];
      sg[1] += y * r1[k];
      sg[2] += y * y;
      sg[3] += r0[k] * r1[k];
      sg[4] += r0[k] * y;
    }
    // the minimal-residual pair (gamma1, gamma2); o[0] = 1: breakdown
    double gm[3];
    ok = R.sum_map<5, 3>(sg, gm, [&](const double* w, double* o) {
      const double s11 = w[0], s12 = w[1], s22 = w[2], rhs1 = w[3], rhs2 = w[4];
      const double rn1 = sqrt(s11), rn2 = sqrt(s22);
      double gm1 = 0.0, gm2 = 0.0;
      o[0] = 0.0;
      if (rn1 < 1.0e-300) { o[0] = 1.0; }
      else if (rn2 < 1.0e-300) { gm2 = 0.0; gm1 = rhs1 / s11; }
      else {
        const double i1 = 1.0 / rn1, i2 = 1.0 / rn2;
        const double c12 = s12 * i1 * i2;
        const double b1 = rhs1 * i1, b2 = rhs2 * i2;
        const double det = 1.0 - c12 * c12;
        if (fabs(det) < 1.0e-14) { gm2 = 0.0; gm1 = b1 * i1; }
        else { gm1 = (b1 - c12 * b2) / (det * rn1); gm2 = (b2 - c12 * b1) / (det * rn2); }
      }
      o[1] = gm1;
      o[2] = gm2;
    });
    if (!ok) break;
    if (gm[0] != 0.0) { status = COVOF_BREAKDOWN; break; }
    const double gm1 = gm[1], gm2 = gm[2];
    double fin[2] = {0.0, 0.0};
    FOR_DOFS(a, W, part, i, j, k) {
      x[k] = x[k] + gm1 * r0[k] + gm2 * r1[k];
      const double rr = r0[k] - (gm1 * r1[k] + gm2 * r2[k]);
      r0[k] = rr;
      u0[k] = u0[k] - (gm1 * u1[k] + gm2 * u2[k]);
      fin[0] += rr * rr;
      fin[1] += rt[k] * rr;  // rho1 of the next sweep
    }
    if (gm2 != 0.0) omega = gm2;
    else if (fabs(gm1) > 1.0e-300) omega = gm1;
    else omega = 1.0;
    double of[5];
    ok = R.sum_map<2, 5>(fin, of, [&](const double* w, double* o) {
      head(w[1], o);
      const double rn = sqrt(w[0]);
      o[3] = rn;
      o[4] = rn / r0n;
    });
    if (!ok) break;
    hd[0] = of[0]; hd[1] = of[1]; hd[2] = of[2];
    const double rn = of[3];
    if (rn != rn || rn > 1.0e30) { status = COVOF_NAN; break; }
    if (of[4] < tol || rn < 1.0e-12) { status = COVOF_OK; break; }
  }
  krylov_finish(a, tm, iter, status, ok);
}

__global__ void __launch_bounds__(512) k_bicgstab2(MomArgs a) {
  const Team tm = grid_team();
  GridReducer R{a.part, GridSync{a.bar, a.err, (unsigned)tm.size, 0u}, 0, tm.rank};
  bicgstab2_case(a, tm, R);
}

// ---------------------------------------------------------------------------
// Copy the solution DOFs back into (u, v); ghosts come from k_vbc_*.
__global__ void k_mom_unpack(MomArgs a, double* u, double* v) {
  const Dims& D = a.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int g = D.P * (D.ny + 2);
  if (i <= D.nx + 1 && j <= D.ny) u[D.id(i, j)] = a.x[D.id(i, j)];
  if (i <= D.nx && j <= D.ny + 1) v[D.id(i, j)] = a.x[g + D.id(i, j)];
  if (a.mono && i <= D.nx && j <= D.ny) a.pm[D.id(i, j)] = a.x[2 * (size_t)g + D.id(i, j)];
}
// Pack (u, v) DOFs into the Krylov start vector.
__global__ void k_mom_pack(MomArgs a, const double* u, const double* v) {
  const Dims& D = a.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int g = D.P * (D.ny + 2);
  if (i <= D.nx + 1 && j <= D.ny) a.x[D.id(i, j)] = u[D.id(i, j)];
  if (i <= D.nx && j <= D.ny + 1) a.x[g + D.id(i, j)] = v[D.id(i, j)];
  if (a.mono && i <= D.nx && j <= D.ny) a.x[2 * (size_t)g + D.id(i, j)] = a.pm[D.id(i, j)];
}

// Non-homogeneous velocity ghost conditions, src/module_mpi_comm.f90:290-537,
// in the reference's order: west/east columns, then south/north rows, then
// the physical corners.
__global__ void k_vbc_we(BcArgs b, double* u, double* v) {
  const Dims& D = b.D;
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int nx = D.nx;
  if (j > D.ny) return;
  // west
  if (b.bc[SL] == COVOF_BC_DIRICHLET) {
    u[D.id(1, j)] = b.bcu[SL];
    u[D.id(0, j)] = b.bcu[SL];
    v[D.id(0, j)] = 2.0 * b.bcv[SL] - v[D.id(1, j)];
  } else if (b.bc[SL] == COVOF_BC_FREESLIP) {
    u[D.id(1, j)] = 0.0;
    u[D.id(0, j)] = 0.0;
    v[D.id(0, j)] = v[D.id(1, j)];
  }
  // east
  if (b.bc[SR] == COVOF_BC_DIRICHLET) {
    u[D.id(nx + 1, j)] = b.bcu[SR];
    v[D.id(nx + 1, j)] = 2.0 * b.bcv[SR] - v[D.id(nx, j)];
  } else if (b.bc[SR] == COVOF_BC_FREESLIP) {
    u[D.id(nx + 1, j)] = 0.0;
    v[D.id(nx + 1, j)] = v[D.id(nx, j)];
  }
}
__global__ void k_vbc_sn(BcArgs b, double* u, double* v) {
  const Dims& D = b.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int ny = D.ny;
  if (i > D.nx) return;
  if (b.bc[SB] == COVOF_BC_DIRICHLET) {
    v[D.id(i, 1)] = b.bcv[SB];
    v[D.id(i, 0)] = b.bcv[SB];
    if (ny >= 2) u[D.id(i, 0)] = (8.0 * b.bcu[SB] - 6.0 * u[D.id(i, 1)] + u[D.id(i, 2)]) / 3.0;
    else u[D.id(i, 0)] = 2.0 * b.bcu[SB] - u[D.id(i, 1)];
  } else if (b.bc[SB] == COVOF_BC_FREESLIP) {
    v[D.id(i, 1)] = 0.0;
    v[D.id(i, 0)] = 0.0;
    u[D.id(i, 0)] = u[D.id(i, 1)];
  }
  if (b.bc[ST] == COVOF_BC_DIRICHLET) {
    v[D.id(i, ny + 1)] = b.bcv[ST];
    if (ny >= 2) u[D.id(i, ny + 1)] = (8.0 * b.bcu[ST] - 6.0 * u[D.id(i, ny)] + u[D.id(i, ny - 1)]) / 3.0;
    else u[D.id(i, ny + 1)] = 2.0 * b.bcu[ST] - u[D.id(i, ny)];
  } else if (b.bc[ST] == COVOF_BC_FREESLIP) {
    v[D.id(i, ny + 1)] = 0.0;
    u[D.id(i, ny + 1)] = u[D.id(i, ny)];
  }
}
// The periodic directions of apply_velocity_bc at np = 1
// (src/module_mpi_comm.f90:332-351), before the wall sides: x first (rows
// 1..ny of u and v), then y (v columns 1..nx, u columns 0..nx+1); one block.
__global__ void k_vbc_periodic(BcArgs b, double* u, double* v) {
  const Dims& D = b.D;
  const int nx = D.nx, ny = D.ny;
  if (D.perx)
    for (int j = 1 + (int)threadIdx.x; j <= ny; j += blockDim.x) {
      u[D.id(0, j)] = u[D.id(nx, j)];
      u[D.id(nx + 1, j)] = u[D.id(1, j)];
      v[D.id(0, j)] = v[D.id(nx, j)];
      v[D.id(nx + 1, j)] = v[D.id(1, j)];
    }
  __syncthreads();
  if (D.pery) {
    for (int i = 1 + (int)threadIdx.x; i <= nx; i += blockDim.x) {
      v[D.id(i, 0)] = v[D.id(i, ny)];
      v[D.id(i, ny + 1)] = v[D.id(i, 1)];
    }
    for (int i = (int)threadIdx.x; i <= nx + 1; i += blockDim.x) {
      u[D.id(i, 0)] = u[D.id(i, ny)];
      u[D.id(i, ny + 1)] = u[D.id(i, 1)];
    }
  }
}
// physical corners (:512-526): none when a direction is periodic
__global__ void k_vbc_corners(BcArgs b, double* u, double* v) {
  const Dims& D = b.D;
  const int nx = D.nx, ny = D.ny;
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  if (D.perx || D.pery) return;
  u[D.id(nx + 1, 0)] = u[D.id(nx + 1, 1)];
  v[D.id(nx + 1, 0)] = v[D.id(nx, 0)];
  u[D.id(nx + 1, ny + 1)] = u[D.id(nx + 1, ny)];
  v[D.id(nx + 1, ny + 1)] = v[D.id(nx, ny + 1)];
  v[D.id(0, ny + 1)] = v[D.id(1, ny + 1)];
}

// Predictor Krylov solves of many cases in one persistent launch (teams,
// see BatchTeams); each case's method is its own linear_solver.
__device__ __forceinline__ void mom_krylov_batch(const MomArgs* __restrict__ cases, const BatchTeams& bt,
                                                 int method) {
  int4 T;
  const Team tm = batch_team(bt, T);
  const int t = bt.block_team[blockIdx.x];
  GridReducer R{bt.part + (size_t)16 * T.x, GridSync{bt.bar + 32 * t, bt.err + t, (unsigned)T.y, 0u}, 0, tm.rank};
  for (int q = T.z; q < T.w; ++q) {
    const MomArgs& a = cases[bt.case_list[q]];
    const int m = method >= 0 ? method : a.method;
    if (m == COVOF_LINEAR_BICGSTAB) bicgstab_case(a, tm, R);
    else if (m == COVOF_LINEAR_CG) cg_case(a, tm, R);
    else bicgstab2_case(a, tm, R);
  }
}

__global__ void __launch_bounds__(512) k_mom_krylov_batch(const MomArgs* __restrict__ cases, BatchTeams bt) {
  mom_krylov_batch(cases, bt, -1);
}

// Every case with the same method: that method alone, in 64 registers, so
// two 512-thread blocks share an SM (twice the loads in flight for these
// HBM-streaming loops; the mixed-method kernel above needs 128 registers).
__global__ void __launch_bounds__(512, 2) k_mom_bicgstab_batch(const MomArgs* __restrict__ cases, BatchTeams bt) {
  mom_krylov_batch(cases, bt, COVOF_LINEAR_BICGSTAB);
}
__global__ void __launch_bounds__(512, 2) k_mom_cg_batch(const MomArgs* __restrict__ cases, BatchTeams bt) {
  mom_krylov_batch(cases, bt, COVOF_LINEAR_CG);
}

// ---------------------------------------------------------------------------
// Augmented Lagrangian (solver_type AUGMENTED_LAGRANGIAN / AAL).
// Maxima of nonnegative doubles through their bit patterns (monotone for
// x >= 0), so the order of the atomics does not matter.
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* p, double x) {
  atomicMax(p, (unsigned long long)__double_as_longlong(x));
}
__device__ __forceinline__ double block_max(double x) {
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// max over interior cells of the cell-centre speed and of |p|
// (src/module_navier_stokes.f90:1149-1160); maxv[0..1] zero at launch.
__global__ void k_al_maxima(AlArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  double spd = 0.0, pa = 0.0;
  if (i <= a.D.nx && j <= a.D.ny) {
    const int k = a.D.id(i, j);
    const double uc = 0.5 * (a.u[k] + a.u[k + 1]);
    const double vc = 0.5 * (a.v[k] + a.v[k + a.D.P]);
    spd = sqrt(uc * uc + vc * vc);
    pa = fabs(a.p[k]);
  }
  spd = block_max(spd);
  pa = block_max(pa);
  if ((threadIdx.x + threadIdx.y * blockDim.x) % 32 == 0) {
    atomic_max_nonneg(a.maxv + 0, spd);
    atomic_max_nonneg(a.maxv + 1, pa);
  }
}

// r_aal (src/module_navier_stokes.f90:1120-1216, incompressible): r_al
// everywhere, or k_aal * max(unsteady, inertial, gravity, pressure, viscous,
// capillary) per interior cell with the velocity / pressure scales from
// k_al_maxima.
__global__ void k_al_penalty(AlArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.D.nx, ny = a.D.ny;
  if (i > nx + 1 || j > ny + 1) return;
  const int k = a.D.id(i, j);
  if (!a.adaptive) { a.r[k] = a.r_al; return; }
  if (i < 1 || i > nx || j < 1 || j > ny) return;  // ghosts are never read
  const double u_max = __longlong_as_double((long long)a.maxv[0]);
  const double p_max = __longlong_as_double((long long)a.maxv[1]);
  const double L0 = a.L0, t0 = a.t0;
  double u0 = a.u0_ref > 0.0 ? a.u0_ref : u_max;
  if (u0 < 1.0e-12) {
    const double u_grav = a.g_norm > 0.0 ? sqrt(a.g_norm * L0) : 0.0;
    const double u_cap = (a.sigma > 0.0 && a.mu_max > 1.0e-30) ? a.sigma / a.mu_max : 0.0;
    u0 = fmax(fmax(fmax(u_grav, u_cap), L0 / fmax(t0, 1.0e-12)), 1.0e-3);
  }
  const double p0 = a.p0_ref > 0.0 ? a.p0_ref : p_max;
  const double rM = a.rho[k], mM = a.mu[k];
  const double t_uns = a.alpha_time * rM * (L0 * L0) / fmax(t0, 1.0e-30);
  const double t_in = rM * u0 * L0;
  const double t_gr = rM * (L0 * L0 / u0) * a.g_norm;
  const double t_pr = (p0 * L0) / u0;
  const double t_vi = mM;
  const double t_ca = a.sigma / u0;
  const double mx = fmax(fmax(fmax(t_uns, t_in), fmax(t_gr, t_pr)), fmax(fmax(t_vi, 0.0), t_ca));
  double r = a.k_aal * mx;
  if (r <= 1.0e-15) r = a.r_al;
  a.r[k] = r;
}

// p -= r div u on interior cells (src/module_navier_stokes.f90:1223-1263)
__global__ void k_al_pressure(AlArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > a.D.nx || j > a.D.ny) return;
  const int k = a.D.id(i, j);
  const double dv = (a.u[k + 1] - a.u[k]) / a.dx + (a.v[k + a.D.P] - a.v[k]) / a.dy;
  a.p[k] = a.p[k] - a.r[k] * dv;
}

// max |div u| over interior cells into maxv[2] (zero at launch)
__global__ void k_al_divmax(AlArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  double d = 0.0;
  if (i <= a.D.nx && j <= a.D.ny) {
    const int k = a.D.id(i, j);
    d = fabs((a.u[k + 1] - a.u[k]) / a.dx + (a.v[k + a.D.P] - a.v[k]) / a.dy);
  }
  d = block_max(d);
  if ((threadIdx.x + threadIdx.y * blockDim.x) % 32 == 0) atomic_max_nonneg(a.maxv + 2, d);
}

}  // namespace covof

COVOF_UNIT_HOOKS(momentum)
