// covof_oracle.cpp -- TEST INFRASTRUCTURE ONLY (see covof_oracle.h).
//
// Serial FP64 CPU restatement of the COVOF 2D hot path, following the
// reference subroutines line by line (cited per function).  Built with
// -O2 -ffp-contract=off so that no multiply-add is fused behind our back; the
// evaluation order of every expression follows the Fortran source (left to
// right, parentheses respected).  np = 1 semantics throughout: the MPI halo
// exchanges of the reference are no-ops on a single non-periodic domain
// (src/module_mpi_comm.f90:46-56) and are omitted.
#include "covof_oracle.h"

#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { L = 0, R = 1, B = 2, T = 3 };

struct Mesh {
  int nx, ny;
  double dx, dy;
  int P;  // pitch = nx + 2
  inline size_t id(int i, int j) const { return (size_t)j * (size_t)P + (size_t)i; }
  // src/module_mesh.f90:177-206, single domain: i_start_global = 1
  inline double x_face(int i) const { return (double)(i - 1) * dx; }
  inline double y_face(int j) const { return (double)(j - 1) * dy; }
  inline double x_center(int i) const { return ((double)(i - 1) + 0.5) * dx; }
  inline double y_center(int j) const { return ((double)(j - 1) + 0.5) * dy; }
};

inline Mesh mesh_of(const covof_params* p) {
  Mesh m;
  m.nx = p->nx; m.ny = p->ny; m.dx = p->dx; m.dy = p->dy; m.P = p->nx + 2;
  return m;
}

inline bool is_wall(const covof_params* p, int side) {
  return p->bc_type[side] == COVOF_BC_DIRICHLET || p->bc_type[side] == COVOF_BC_FREESLIP;
}

// Periodic directions at np = 1: the reference makes a direction periodic
// when either side names BC_PERIODIC (src/module_simulation.f90:116-118) but
// then tests one side or the other (bc_left in apply_vof_bc, bc_right in
// poisson_matvec's east term); this restatement takes a pair only.
inline bool per_x(const covof_params* p) { return p->bc_type[L] == COVOF_BC_PERIODIC; }
inline bool per_y(const covof_params* p) { return p->bc_type[B] == COVOF_BC_PERIODIC; }
// the periodic VOF branches restated here are Weymouth-Yue's (CIAM's, TVD's
// and the smoothing filters' are not)
inline int check_periodic_vof(const covof_params* p) {
  if (!(per_x(p) || per_y(p))) return COVOF_OK;
  if (p->advection_method != COVOF_ADVECT_WEYMOUTH_YUE || p->enable_svof_smoothing ||
      p->enable_diffusion_smoothing)
    return COVOF_UNSUPPORTED;
  return COVOF_OK;
}

// allow_periodic: the routine follows the reference's periodic branches
// (Poisson, projection correction, VOF); the momentum path does not (its
// velocity DOF count changes with periodicity) and refuses them.
int check_params(const covof_params* p, bool allow_neumann, bool allow_periodic = false) {
  if (!p || p->nx < 2 || p->ny < 2 || !(p->dx > 0) || !(p->dy > 0)) return COVOF_INVALID;
  for (int s = 0; s < 4; ++s) {
    int t = p->bc_type[s];
    if (t == COVOF_BC_PERIODIC) {
      const int other = s ^ 1;  // L<->R, B<->T
      if (p->bc_type[other] != COVOF_BC_PERIODIC) return COVOF_INVALID;
      if (!allow_periodic) return COVOF_UNSUPPORTED;
      continue;
    }
    if (t == COVOF_BC_NEUMANN && !allow_neumann) return COVOF_UNSUPPORTED;
    if (t != COVOF_BC_DIRICHLET && t != COVOF_BC_FREESLIP && t != COVOF_BC_NEUMANN)
      return COVOF_INVALID;
  }
  return COVOF_OK;
}

// ---------------------------------------------------------------------------
// Fused hypot: sqrt(x^2+y^2) with an FMA-based residual correction (after
// C. F. Borges, "An improved algorithm for hypot(a,b)", ACM TOMS 2021).
// Stands in for the Fortran intrinsic; bit-identical to the GPU's version.
double fhypot(double x, double y) {
  double ax = std::fabs(x), ay = std::fabs(y);
  if (std::isinf(ax) || std::isinf(ay)) return INFINITY;
  if (std::isnan(ax) || std::isnan(ay)) return ax + ay;
  if (ax < ay) std::swap(ax, ay);
  if (ay == 0.0) return ax;
  if (ay < ax * 0x1p-30) return ax;  // ay^2 below half an ulp of ax^2
  double scale = 1.0;
  if (ax > 0x1p+500) { ax *= 0x1p-600; ay *= 0x1p-600; scale = 0x1p+600; }
  else if (ax < 0x1p-450) { ax *= 0x1p+600; ay *= 0x1p+600; scale = 0x1p-600; }
  double h = std::sqrt(std::fma(ax, ax, ay * ay));
  double h_sq = h * h, h_lo = std::fma(h, h, -h_sq);
  double x_sq = ax * ax, x_lo = std::fma(ax, ax, -x_sq);
  double y_sq = ay * ay, y_lo = std::fma(ay, ay, -y_sq);
  double r = ((x_sq - h_sq) + y_sq) + ((x_lo - h_lo) + y_lo);
  h = h + r / (2.0 * h);
  return h * scale;
}

// ---------------------------------------------------------------------------
// src/module_interface_reconstruction.f90:33-101  cut_box_area
double cut_box_area(double xmin, double xmax, double ymin, double ymax, double nx, double ny,
                    double alpha) {
  if ((xmax - xmin) <= 1.0e-14 || (ymax - ymin) <= 1.0e-14) return 0.0;
  double bx[4] = {xmin, xmax, xmax, xmin};
  double by[4] = {ymin, ymin, ymax, ymax};
  double d[4];
  for (int i = 0; i < 4; ++i) d[i] = nx * bx[i] + ny * by[i] + alpha;
  double cx[8], cy[8];
  int n = 0;
  for (int i = 0; i < 4; ++i) {
    int ni = (i + 1) % 4;
    double d1 = d[i], d2 = d[ni];
    if (d1 <= 0.0) {
      if (d2 <= 0.0) {
        cx[n] = bx[ni]; cy[n] = by[ni]; ++n;
      } else {
        double t = -d1 / (d2 - d1);
        cx[n] = bx[i] + t * (bx[ni] - bx[i]);
        cy[n] = by[i] + t * (by[ni] - by[i]);
        ++n;
      }
    } else {
      if (d2 <= 0.0) {
        double t = -d1 / (d2 - d1);
        cx[n] = bx[i] + t * (bx[ni] - bx[i]);
        cy[n] = by[i] + t * (by[ni] - by[i]);
        ++n;
        cx[n] = bx[ni]; cy[n] = by[ni]; ++n;
      }
    }
  }
  if (n < 3) return 0.0;
  double s = 0.0;
  for (int q = 0; q < n; ++q) {
    int nq = (q + 1) % n;
    s = s + (cx[q] * cy[nq] - cx[nq] * cy[q]);
  }
  return 0.5 * std::fabs(s);
}

// src/module_interface_reconstruction.f90:105-147  compute_alpha (45-step bisection)
double compute_alpha(double xmin, double xmax, double ymin, double ymax, double nx, double ny,
                     double c_target) {
  double total_area = (xmax - xmin) * (ymax - ymin);
  if (c_target <= 1.0e-7) return 1.0e9;
  if (c_target >= 1.0 - 1.0e-7) return -1.0e9;
  double target_area = std::max(0.0, std::min(1.0, c_target)) * total_area;
  double v1 = nx * xmin + ny * ymin;
  double v2 = nx * xmax + ny * ymin;
  double v3 = nx * xmax + ny * ymax;
  double v4 = nx * xmin + ny * ymax;
  double min_val = std::min(v1, std::min(v2, std::min(v3, v4)));
  double max_val = std::max(v1, std::max(v2, std::max(v3, v4)));
  double lo = -max_val - 1.0e-12;
  double hi = -min_val + 1.0e-12;
  for (int it = 0; it < 45; ++it) {
    double mid = 0.5 * (lo + hi);
    double a = cut_box_area(xmin, xmax, ymin, ymax, nx, ny, mid);
    if (a < target_area) hi = mid; else lo = mid;
  }
  return 0.5 * (lo + hi);
}

// ---------------------------------------------------------------------------
// src/module_mpi_comm.f90:290-537 apply_velocity_bc (np=1, constant walls,
// no PARABOLIC / JET_INLET / obstacle profiles).
void velocity_bc(const covof_params* prm, const Mesh& m, double* u, double* v, bool homog) {
  const int nx = m.nx, ny = m.ny;
  double ul = homog ? 0.0 : prm->bc_u[L], vl = homog ? 0.0 : prm->bc_v[L];
  double ur = homog ? 0.0 : prm->bc_u[R], vr = homog ? 0.0 : prm->bc_v[R];
  double ub = homog ? 0.0 : prm->bc_u[B], vb = homog ? 0.0 : prm->bc_v[B];
  double ut = homog ? 0.0 : prm->bc_u[T], vt = homog ? 0.0 : prm->bc_v[T];
  // periodic directions at np = 1 (:332-351); the wall branches below then
  // skip those sides (their types are PERIODIC)
  if (per_x(prm))
    for (int j = 1; j <= ny; ++j) {
      u[m.id(0, j)] = u[m.id(nx, j)];
      u[m.id(nx + 1, j)] = u[m.id(1, j)];
      v[m.id(0, j)] = v[m.id(nx, j)];
      v[m.id(nx + 1, j)] = v[m.id(1, j)];
    }
  if (per_y(prm)) {
    for (int i = 1; i <= nx; ++i) {
      v[m.id(i, 0)] = v[m.id(i, ny)];
      v[m.id(i, ny + 1)] = v[m.id(i, 1)];
    }
    for (int i = 0; i <= nx + 1; ++i) {
      u[m.id(i, 0)] = u[m.id(i, ny)];
      u[m.id(i, ny + 1)] = u[m.id(i, 1)];
    }
  }
  // west (:339-373)
  for (int j = 1; j <= ny; ++j) {
    int t = prm->bc_type[L];
    if (t == COVOF_BC_DIRICHLET) {
      if (!homog) u[m.id(1, j)] = ul;
      u[m.id(0, j)] = ul;
      v[m.id(0, j)] = 2.0 * vl - v[m.id(1, j)];
    } else if (t == COVOF_BC_FREESLIP) {
      if (!homog) u[m.id(1, j)] = 0.0;
      u[m.id(0, j)] = 0.0;
      v[m.id(0, j)] = v[m.id(1, j)];
    } else if (t == COVOF_BC_NEUMANN) {
      u[m.id(0, j)] = u[m.id(1, j)];
      v[m.id(0, j)] = v[m.id(1, j)];
    }
  }
  // east (:377-394)
  for (int j = 1; j <= ny; ++j) {
    int t = prm->bc_type[R];
    if (t == COVOF_BC_DIRICHLET) {
      if (!homog) u[m.id(nx + 1, j)] = ur;
      v[m.id(nx + 1, j)] = 2.0 * vr - v[m.id(nx, j)];
    } else if (t == COVOF_BC_FREESLIP) {
      if (!homog) u[m.id(nx + 1, j)] = 0.0;
      v[m.id(nx + 1, j)] = v[m.id(nx, j)];
    } else if (t == COVOF_BC_NEUMANN) {
      if (!homog) u[m.id(nx + 1, j)] = u[m.id(nx, j)];
      v[m.id(nx + 1, j)] = v[m.id(nx, j)];
    }
  }
  // south (:397-425)
  for (int i = 1; i <= nx; ++i) {
    int t = prm->bc_type[B];
    if (t == COVOF_BC_DIRICHLET) {
      if (!homog) v[m.id(i, 1)] = vb;
      v[m.id(i, 0)] = vb;
      if (ny >= 2)
        u[m.id(i, 0)] = (8.0 * ub - 6.0 * u[m.id(i, 1)] + u[m.id(i, 2)]) / 3.0;
      else
        u[m.id(i, 0)] = 2.0 * ub - u[m.id(i, 1)];
    } else if (t == COVOF_BC_FREESLIP) {
      if (!homog) v[m.id(i, 1)] = 0.0;
      v[m.id(i, 0)] = 0.0;
      u[m.id(i, 0)] = u[m.id(i, 1)];
    } else if (t == COVOF_BC_NEUMANN) {
      u[m.id(i, 0)] = u[m.id(i, 1)];
      v[m.id(i, 0)] = v[m.id(i, 1)];
    }
  }
  // north (:456-479)
  for (int i = 1; i <= nx; ++i) {
    int t = prm->bc_type[T];
    if (t == COVOF_BC_DIRICHLET) {
      if (!homog) v[m.id(i, ny + 1)] = vt;
      if (ny >= 2)
        u[m.id(i, ny + 1)] = (8.0 * ut - 6.0 * u[m.id(i, ny)] + u[m.id(i, ny - 1)]) / 3.0;
      else
        u[m.id(i, ny + 1)] = 2.0 * ut - u[m.id(i, ny)];
    } else if (t == COVOF_BC_FREESLIP) {
      if (!homog) v[m.id(i, ny + 1)] = 0.0;
      u[m.id(i, ny + 1)] = u[m.id(i, ny)];
    } else if (t == COVOF_BC_NEUMANN) {
      u[m.id(i, ny + 1)] = u[m.id(i, ny)];
      if (!homog) v[m.id(i, ny + 1)] = v[m.id(i, ny)];
    }
  }
  // physical corners, non-homogeneous only (:512-526; none on a periodic side)
  if (!homog && !per_x(prm) && !per_y(prm)) {
    u[m.id(nx + 1, 0)] = u[m.id(nx + 1, 1)];
    v[m.id(nx + 1, 0)] = v[m.id(nx, 0)];
    u[m.id(nx + 1, ny + 1)] = u[m.id(nx + 1, ny)];
    v[m.id(nx + 1, ny + 1)] = v[m.id(nx, ny + 1)];
    v[m.id(0, ny + 1)] = v[m.id(1, ny + 1)];
  }
}

// src/module_mpi_comm.f90:25-56 exchange_halos_scalar at np = 1: the
// periodic wrap of the ghost ring (x first, rows 0..ny+1, then y, columns
// 0..nx+1, so the corners take the doubly wrapped values); nothing on a
// non-periodic domain.
void halo_scalar(const covof_params* prm, const Mesh& m, double* f) {
  const int nx = m.nx, ny = m.ny;
  if (per_x(prm))
    for (int j = 0; j <= ny + 1; ++j) {
      f[m.id(0, j)] = f[m.id(nx, j)];
      f[m.id(nx + 1, j)] = f[m.id(1, j)];
    }
  if (per_y(prm))
    for (int i = 0; i <= nx + 1; ++i) {
      f[m.id(i, 0)] = f[m.id(i, ny)];
      f[m.id(i, ny + 1)] = f[m.id(i, 1)];
    }
}

// src/module_mpi_comm.f90:636-683 apply_vof_bc (np=1, no JET_INLET):
// periodic wrap (rows / columns 1..n) or zero gradient per direction.
void vof_bc(const covof_params* prm, const Mesh& m, double* C) {
  const int nx = m.nx, ny = m.ny;
  if (per_x(prm)) {
    for (int j = 1; j <= ny; ++j) {
      C[m.id(0, j)] = C[m.id(nx, j)];
      C[m.id(nx + 1, j)] = C[m.id(1, j)];
    }
  } else {
    for (int j = 1; j <= ny; ++j) {
      C[m.id(0, j)] = C[m.id(1, j)];
      C[m.id(nx + 1, j)] = C[m.id(nx, j)];
    }
  }
  if (per_y(prm)) {
    for (int i = 1; i <= nx; ++i) {
      C[m.id(i, 0)] = C[m.id(i, ny)];
      C[m.id(i, ny + 1)] = C[m.id(i, 1)];
    }
  } else {
    for (int i = 1; i <= nx; ++i) C[m.id(i, 0)] = C[m.id(i, 1)];
    for (int i = 1; i <= nx; ++i) C[m.id(i, ny + 1)] = C[m.id(i, ny)];
  }
}

// ---------------------------------------------------------------------------
// Pressure Poisson.  Coefficient arrays are (nx, ny), index (i-1)+nx*(j-1).
struct Poisson {
  int nx, ny;
  bool perx = false, pery = false;  // periodic wrap of the stencil (np = 1)
  std::vector<double> aW, aE, aS, aN, aP, b;
  inline size_t k(int i, int j) const { return (size_t)(i - 1) + (size_t)nx * (size_t)(j - 1); }
};

// src/module_simulation.f90:2483-2533 (obstacles disabled)
void poisson_assemble(const covof_params* prm, const Mesh& m, double dt, const double* rho_u,
                      const double* rho_v, Poisson& P) {
  const int nx = m.nx, ny = m.ny;
  const double dx = m.dx, dy = m.dy, dvol = dx * dy;
  P.nx = nx; P.ny = ny;
  P.perx = per_x(prm); P.pery = per_y(prm);
  size_t n = (size_t)nx * ny;
  P.aW.assign(n, 0.0); P.aE.assign(n, 0.0); P.aS.assign(n, 0.0); P.aN.assign(n, 0.0);
  P.aP.assign(n, 0.0); P.b.assign(n, 0.0);
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t q = P.k(i, j);
      bool wW = (i == 1 && is_wall(prm, L));
      if (!wW) {
        double r = rho_u[m.id(i, j)];
        if (r < 1.0e-12) r = 1.0;
        P.aW[q] = (dt * dy) / (r * dx);
      }
      bool wE = (i == nx && is_wall(prm, R));
      if (!wE) {
        double r = rho_u[m.id(i + 1, j)];
        if (r < 1.0e-12) r = 1.0;
        P.aE[q] = (dt * dy) / (r * dx);
      }
      bool wS = (j == 1 && is_wall(prm, B));
      if (!wS) {
        double r = rho_v[m.id(i, j)];
        if (r < 1.0e-12) r = 1.0;
        P.aS[q] = (dt * dx) / (r * dy);
      }
      bool wN = (j == ny && is_wall(prm, T));
      if (!wN) {
        double r = rho_v[m.id(i, j + 1)];
        if (r < 1.0e-12) r = 1.0;
        P.aN[q] = (dt * dx) / (r * dy);
      }
      P.aP[q] = P.aW[q] + P.aE[q] + P.aS[q] + P.aN[q] + 1.0e-12 * dvol;
    }
}

// src/module_simulation.f90:2484-2487 b = -div(u*)
void poisson_rhs_from_velocity(const Mesh& m, const double* u, const double* v, Poisson& P) {
  for (int j = 1; j <= m.ny; ++j)
    for (int i = 1; i <= m.nx; ++i) {
      double div = (u[m.id(i + 1, j)] - u[m.id(i, j)]) * m.dy + (v[m.id(i, j + 1)] - v[m.id(i, j)]) * m.dx;
      P.b[P.k(i, j)] = -div;
    }
}

// src/module_simulation.f90:2668-2707 poisson_matvec, one row: the
// neighbours across a periodic boundary wrap (x(nx,j) west of cell 1,
// x(1,j) east of cell nx; likewise in y).
inline double poisson_row(const Poisson& P, const double* x, int i, int j) {
  const int nx = P.nx, ny = P.ny;
  const size_t q = P.k(i, j);
  double val = P.aP[q] * x[q];
  if (i > 1) val = val - P.aW[q] * x[q - 1];
  else if (P.perx) val = val - P.aW[q] * x[P.k(nx, j)];
  if (i < nx) val = val - P.aE[q] * x[q + 1];
  else if (P.perx) val = val - P.aE[q] * x[P.k(1, j)];
  if (j > 1) val = val - P.aS[q] * x[q - nx];
  else if (P.pery) val = val - P.aS[q] * x[P.k(i, ny)];
  if (j < ny) val = val - P.aN[q] * x[q + nx];
  else if (P.pery) val = val - P.aN[q] * x[P.k(i, 1)];
  return val;
}

void poisson_matvec(const Poisson& P, const double* x, double* y) {
  for (int j = 1; j <= P.ny; ++j)
    for (int i = 1; i <= P.nx; ++i) y[P.k(i, j)] = poisson_row(P, x, i, j);
}

void poisson_matvec_omp(const Poisson& P, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= P.ny; ++j)
    for (int i = 1; i <= P.nx; ++i) y[P.k(i, j)] = poisson_row(P, x, i, j);
}

// src/module_simulation.f90:2709-2758 poisson_ssor (SGS, omega = 1).
// pinned: cell (1,1) is held at zero in both sweeps.
void poisson_sgs(const Poisson& P, const double* r, double* z, bool pinned) {
  const int nx = P.nx, ny = P.ny;
  std::fill(z, z + (size_t)nx * ny, 0.0);
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t q = P.k(i, j);
      double val = r[q];
      if (i > 1) val = val + P.aW[q] * z[q - 1];
      else if (P.perx) val = val + P.aW[q] * z[P.k(nx, j)];
      if (j > 1) val = val + P.aS[q] * z[q - nx];
      else if (P.pery) val = val + P.aS[q] * z[P.k(i, ny)];
      z[q] = val / P.aP[q];
      if (pinned && i == 1 && j == 1) z[q] = 0.0;
    }
  for (int j = ny; j >= 1; --j)
    for (int i = nx; i >= 1; --i) {
      size_t q = P.k(i, j);
      double val = P.aP[q] * z[q];
      if (i < nx) val = val + P.aE[q] * z[q + 1];
      else if (P.perx) val = val + P.aE[q] * z[P.k(1, j)];
      if (j < ny) val = val + P.aN[q] * z[q + nx];
      else if (P.pery) val = val + P.aN[q] * z[P.k(i, 1)];
      z[q] = val / P.aP[q];
      if (pinned && i == 1 && j == 1) z[q] = 0.0;
    }
}

// Jacobi alternative (diagonal scaling by a_P), an option of this build.
void poisson_jacobi(const Poisson& P, const double* r, double* z, bool pinned) {
  size_t n = (size_t)P.nx * P.ny;
  for (size_t q = 0; q < n; ++q) z[q] = r[q] / P.aP[q];
  if (pinned) z[0] = 0.0;
}

// src/module_simulation.f90:2760-2774 dot / norm (sequential, column-major order)
double dot(const double* x, const double* y, size_t n) {
  double s = 0.0;
  for (size_t q = 0; q < n; ++q) s = s + x[q] * y[q];
  return s;
}
double dot_omp(const double* x, const double* y, size_t n) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (long q = 0; q < (long)n; ++q) s += x[q] * y[q];
  return s;
}

// The Jacobi-PCG of poisson_pcg on nthreads host threads: the same
// recurrences (z = r / a_P, alpha = <r,z>/<d,Ad>, beta = <r,z>_new/<r,z>_old,
// exit on ||r||/||b||), with every vector pass inside one parallel region.
// Rows are split statically among the threads; each thread writes its
// partial sums to its own slot, and every thread combines the slots in
// thread order, so all threads hold the same scalars and the result is
// reproducible for a given thread count (it differs from the serial loop's
// only in the association of the sums).  Three barriers per iteration:
// after A d and <d,Ad>, after the x, r updates and their sums, after the
// direction update (the next product reads the neighbours' rows).
int poisson_pcg_par(const covof_params* prm, Poisson& P, std::vector<double>& x, int* iters_out,
                    double* relres_out, int nthreads, int fixed_iters) {
  const int nx = P.nx, ny = P.ny;
  const size_t n = (size_t)nx * ny;
  const bool pinned = prm->p_gauge == COVOF_GAUGE_PINNED;
  const double tol = prm->p_tol;
  const int max_iter = fixed_iters > 0 ? fixed_iters : prm->p_max_iter;
  if (pinned) { P.b[0] = 0.0; x[0] = 0.0; }
  std::vector<double> r(n), d(n), Ad(n);
  constexpr int kPad = 8;  // one 64-byte line per thread and buffer
  std::vector<double> part(2 * (size_t)nthreads * kPad, 0.0);
  const double* aP = P.aP.data(); const double* aW = P.aW.data(); const double* aE = P.aE.data();
  const double* aS = P.aS.data(); const double* aN = P.aN.data();
  double* xp = x.data(); double* rp = r.data(); double* dp = d.data(); double* Adp = Ad.data();
  const double* bp = P.b.data();
  int iters = 0, status = COVOF_OK;
  double r_norm = 0.0, b_norm = 1.0;
  auto Arow = [&](const double* v, double* y, int j) {
    if (P.perx || P.pery) {
      for (int i = 1; i <= nx; ++i) y[P.k(i, j)] = poisson_row(P, v, i, j);
    } else {
      for (int i = 1; i <= nx; ++i) {
        const size_t q = P.k(i, j);
        double val = aP[q] * v[q];
        if (i > 1) val = val - aW[q] * v[q - 1];
        if (i < nx) val = val - aE[q] * v[q + 1];
        if (j > 1) val = val - aS[q] * v[q - nx];
        if (j < ny) val = val - aN[q] * v[q + nx];
        y[q] = val;
      }
    }
    if (pinned && j == 1) y[0] = 0.0;
  };
  auto zval = [&](size_t q) { return (pinned && q == 0) ? 0.0 : rp[q] / aP[q]; };
#pragma omp parallel num_threads(nthreads)
  {
    const int T = omp_get_num_threads(), t = omp_get_thread_num();
    const int j0 = 1 + (int)((long long)ny * t / T), j1 = (int)((long long)ny * (t + 1) / T);
    int buf = 0;
    // combine NV partial sums of every thread, in thread order
    auto reduce = [&](const double* mine, int nv, double* out) {
      double* slot = part.data() + ((size_t)buf * T + t) * kPad;
      for (int q = 0; q < nv; ++q) slot[q] = mine[q];
#pragma omp barrier
      for (int q = 0; q < nv; ++q) out[q] = 0.0;
      for (int s = 0; s < T; ++s) {
        const double* o = part.data() + ((size_t)buf * T + s) * kPad;
        for (int q = 0; q < nv; ++q) out[q] += o[q];
      }
      buf ^= 1;  // the next reduction writes the other buffer: no second barrier
    };
    // r = b - A x; ||b||, ||r||, <r,z>; d = z
    for (int j = j0; j <= j1; ++j) Arow(xp, Adp, j);
    double acc[3] = {0.0, 0.0, 0.0};
    for (int j = j0; j <= j1; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t q = P.k(i, j);
        rp[q] = bp[q] - Adp[q];
        const double z = zval(q);
        dp[q] = z;
        acc[0] += bp[q] * bp[q];
        acc[1] += rp[q] * rp[q];
        acc[2] += rp[q] * z;
      }
    double s3[3];
    reduce(acc, 3, s3);
    double bn = std::sqrt(s3[0]);
    if (bn < 1.0e-30) bn = 1.0;
    double rn = std::sqrt(s3[1]), rz_old = s3[2];
    int it_local = 0, st_local = COVOF_OK;
    bool converged = false;
    if (std::isnan(rn)) st_local = COVOF_NAN;
    else if (fixed_iters > 0 || rn / bn > tol) {
#pragma omp barrier
      for (int it = 1; it <= max_iter; ++it) {
        it_local = it;
        double a1 = 0.0;
        for (int j = j0; j <= j1; ++j) {
          Arow(dp, Adp, j);
          for (int i = 1; i <= nx; ++i) { const size_t q = P.k(i, j); a1 += dp[q] * Adp[q]; }
        }
        double dAd;
        reduce(&a1, 1, &dAd);
        if (std::fabs(dAd) < 1.0e-35) { st_local = COVOF_BREAKDOWN; break; }
        const double alpha = rz_old / dAd;
        double a2[2] = {0.0, 0.0};
        for (int j = j0; j <= j1; ++j)
          for (int i = 1; i <= nx; ++i) {
            const size_t q = P.k(i, j);
            xp[q] = xp[q] + alpha * dp[q];
            rp[q] = rp[q] - alpha * Adp[q];
            a2[0] += rp[q] * rp[q];
            a2[1] += rp[q] * zval(q);
          }
        double s2[2];
        reduce(a2, 2, s2);
        rn = std::sqrt(s2[0]);
        if (std::isnan(rn)) { st_local = COVOF_NAN; break; }
        if (fixed_iters == 0 && rn / bn <= tol) { converged = true; break; }
        if (std::fabs(rz_old) < 1.0e-35) { st_local = COVOF_BREAKDOWN; break; }
        const double beta = s2[1] / rz_old;
        rz_old = s2[1];
        for (int j = j0; j <= j1; ++j)
          for (int i = 1; i <= nx; ++i) { const size_t q = P.k(i, j); dp[q] = zval(q) + beta * dp[q]; }
#pragma omp barrier
      }
      if (st_local == COVOF_OK && !converged && fixed_iters == 0) st_local = COVOF_MAXITER;
    }
    if (!pinned) {
      // src/module_simulation.f90:2579-2582
#pragma omp barrier
      double s = 0.0;
      for (int j = j0; j <= j1; ++j)
        for (int i = 1; i <= nx; ++i) s += xp[P.k(i, j)];
      double tot;
      reduce(&s, 1, &tot);
      const double mean = tot / (double)((long long)nx * ny);
      for (int j = j0; j <= j1; ++j)
        for (int i = 1; i <= nx; ++i) { const size_t q = P.k(i, j); xp[q] = xp[q] - mean; }
    }
    if (t == 0) { iters = it_local; status = st_local; r_norm = rn; b_norm = bn; }
  }
  if (iters_out) *iters_out = iters;
  if (relres_out) *relres_out = r_norm / b_norm;
  return status;
}

// src/module_simulation.f90:2535-2584  PCG + gauge.  x: (nx,ny) warm start / result.
int poisson_pcg(const covof_params* prm, Poisson& P, std::vector<double>& x, int* iters_out,
                double* relres_out, int nthreads, int fixed_iters) {
  const size_t n = (size_t)P.nx * P.ny;
  const bool pinned = prm->p_gauge == COVOF_GAUGE_PINNED;
  const bool sgs = prm->p_precond == COVOF_PRECOND_SSOR;
  if (nthreads > 1 && !sgs) return poisson_pcg_par(prm, P, x, iters_out, relres_out, nthreads, fixed_iters);
  const bool par = nthreads > 1;
  const double tol = prm->p_tol;
  const int max_iter = fixed_iters > 0 ? fixed_iters : prm->p_max_iter;
#ifdef _OPENMP
  if (par) omp_set_num_threads(nthreads);
#endif
  auto DOT = [&](const double* a, const double* b) { return par ? dot_omp(a, b, n) : dot(a, b, n); };
  auto MATVEC = [&](const double* a, double* y) {
    if (par) poisson_matvec_omp(P, a, y); else poisson_matvec(P, a, y);
    if (pinned) y[0] = 0.0;
  };
  auto PREC = [&](const double* r, double* z) {
    if (sgs) poisson_sgs(P, r, z, pinned); else poisson_jacobi(P, r, z, pinned);
  };
  if (pinned) { P.b[0] = 0.0; x[0] = 0.0; }
  std::vector<double> r(n), Ap(n), z(n), d(n), Ad(n);
  MATVEC(x.data(), Ap.data());
  for (size_t q = 0; q < n; ++q) r[q] = P.b[q] - Ap[q];
  double b_norm = std::sqrt(DOT(P.b.data(), P.b.data()));
  if (b_norm < 1.0e-30) b_norm = 1.0;
  double r_norm = std::sqrt(DOT(r.data(), r.data()));
  int iters = 0, status = COVOF_OK;
  bool converged = false;
  // a NaN in b or x: the reference's loop test (r_norm / b_norm > tol) is
  // false and it returns silently; the status says so here
  if (std::isnan(r_norm)) status = COVOF_NAN;
  else if (fixed_iters > 0 || r_norm / b_norm > tol) {
    PREC(r.data(), z.data());
    d = z;
    double rz_old = DOT(r.data(), z.data());
    for (int it = 1; it <= max_iter; ++it) {
      iters = iters + 1;
      MATVEC(d.data(), Ad.data());
      double dAd = DOT(d.data(), Ad.data());
      if (std::fabs(dAd) < 1.0e-35) { status = COVOF_BREAKDOWN; break; }
      double alpha = rz_old / dAd;
      for (size_t q = 0; q < n; ++q) x[q] = x[q] + alpha * d[q];
      for (size_t q = 0; q < n; ++q) r[q] = r[q] - alpha * Ad[q];
      r_norm = std::sqrt(DOT(r.data(), r.data()));
      if (std::isnan(r_norm)) { status = COVOF_NAN; break; }
      if (fixed_iters == 0 && r_norm / b_norm <= tol) { converged = true; break; }
      PREC(r.data(), z.data());
      double rz_new = DOT(r.data(), z.data());
      if (std::fabs(rz_old) < 1.0e-35) { status = COVOF_BREAKDOWN; break; }
      double beta = rz_new / rz_old;
      rz_old = rz_new;
      for (size_t q = 0; q < n; ++q) d[q] = z[q] + beta * d[q];
    }
    if (status == COVOF_OK && !converged && fixed_iters == 0) status = COVOF_MAXITER;
  }
  if (!pinned) {
    // src/module_simulation.f90:2579-2582
    double s = 0.0;
    for (size_t q = 0; q < n; ++q) s = s + x[q];
    double mean = s / (double)((long long)P.nx * P.ny);
    for (size_t q = 0; q < n; ++q) x[q] = x[q] - mean;
  }
  if (iters_out) *iters_out = iters;
  if (relres_out) *relres_out = r_norm / b_norm;
  return status;
}

int poisson_driver(const covof_params* prm, double dt, const double* u_star, const double* v_star,
                   const double* b_in, const double* rho_u, const double* rho_v, double* p,
                   int* iters, double* relres, int nthreads, int fixed_iters) {
  Mesh m = mesh_of(prm);
  Poisson P;
  poisson_assemble(prm, m, dt, rho_u, rho_v, P);
  if (b_in) {
    for (int j = 1; j <= m.ny; ++j)
      for (int i = 1; i <= m.nx; ++i) P.b[P.k(i, j)] = b_in[m.id(i, j)];
  } else {
    poisson_rhs_from_velocity(m, u_star, v_star, P);
  }
  std::vector<double> x((size_t)m.nx * m.ny);
  for (int j = 1; j <= m.ny; ++j)
    for (int i = 1; i <= m.nx; ++i) x[P.k(i, j)] = p[m.id(i, j)];
  int st = poisson_pcg(prm, P, x, iters, relres, nthreads, fixed_iters);
  for (int j = 1; j <= m.ny; ++j)
    for (int i = 1; i <= m.nx; ++i) p[m.id(i, j)] = x[P.k(i, j)];
  return st;
}

// src/module_simulation.f90:2586-2654 projection correction.  With a
// periodic direction the last face is the first one's image and is not
// corrected (u_nx = nx, :2446-2449); the west / south neighbour of the first
// face wraps.
void project_correct(const covof_params* prm, const Mesh& m, double dt, double* u, double* v,
                     const double* p, const double* rho_u, const double* rho_v) {
  const int nx = m.nx, ny = m.ny;
  const int u_nx = per_x(prm) ? nx : nx + 1, v_ny = per_y(prm) ? ny : ny + 1;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= u_nx; ++i) {
      bool wall = (i == 1 && is_wall(prm, L)) || (i == u_nx && is_wall(prm, R));
      if (wall) continue;
      double r = rho_u[m.id(i, j)];
      if (r < 1.0e-12) r = 1.0;
      double pw = (i > 1) ? p[m.id(i - 1, j)] : (per_x(prm) ? p[m.id(nx, j)] : p[m.id(1, j)]);
      double pe = (i <= nx) ? p[m.id(i, j)] : (per_x(prm) ? p[m.id(1, j)] : p[m.id(nx, j)]);
      double g = (pe - pw) / m.dx;
      u[m.id(i, j)] = u[m.id(i, j)] - (dt / r) * g;
    }
  for (int j = 1; j <= v_ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      bool wall = (j == 1 && is_wall(prm, B)) || (j == v_ny && is_wall(prm, T));
      if (wall) continue;
      double r = rho_v[m.id(i, j)];
      if (r < 1.0e-12) r = 1.0;
      double ps = (j > 1) ? p[m.id(i, j - 1)] : (per_y(prm) ? p[m.id(i, ny)] : p[m.id(i, 1)]);
      double pn = (j <= ny) ? p[m.id(i, j)] : (per_y(prm) ? p[m.id(i, 1)] : p[m.id(i, ny)]);
      double g = (pn - ps) / m.dy;
      v[m.id(i, j)] = v[m.id(i, j)] - (dt / r) * g;
    }
}

// ---------------------------------------------------------------------------
// Momentum predictor (SP: DOFs = u then v, src/module_navier_stokes.f90:164-169)
// Time history of the predictor (fields%u_old, u_nm1, has_nm1;
// src/module_simulation.f90:508-529).
struct Hist {
  const double *u_old = nullptr, *v_old = nullptr, *u_nm1 = nullptr, *v_nm1 = nullptr;
  int has_nm1 = 0;
};

struct MomCtx {
  const covof_params* prm;
  Mesh m;
  double dt;
  const double *u_n, *v_n, *rho_u, *rho_v, *mu, *mu_node;
  double alpha;                  // 1.5: Gear / BDF2 with history (:481-486), else 1
  bool gear_rhs;                 // BDF2 inertial term (:841-848)
  const double *u_adv, *v_adv;   // advecting velocity: fields%u (PICARD) or u_old (AB2)
  const double *u_nm1, *v_nm1;   // AB2 extrapolation partner, nullptr without history
  const double *u_nm1_rhs, *v_nm1_rhs;  // fields%u_nm1 for the Gear right-hand side
  // augmented Lagrangian (solver_type AL / AAL): the penalty field r_aal and
  // the pressure of the right-hand side's gradient term; nullptr for SP
  const double* r_al = nullptr;
  const double* p_al = nullptr;
  // MONOLITHIC coupling: the pressure is a Krylov unknown (np cell DOFs
  // after the velocity DOFs), src/module_navier_stokes.f90:281-294
  bool mono = false;
  int u_nx, v_ny;
  size_t nu, nv, np = 0;
};

// src/module_navier_stokes.f90:2388-2416 conv_face_flux (UPWIND / CENTERED /
// TVD_SUPERBEE; the limiter reads fields_old values q*)
inline double conv_face_flux(int scheme, double flux, double phiL, double phiR, double qLL, double qL,
                             double qR, double qRR, bool hasLL, bool hasRR) {
  if (scheme == COVOF_CONV_CENTERED) return 0.5 * flux * (phiL + phiR);
  if (scheme == COVOF_CONV_UPWIND) return (flux >= 0.0) ? flux * phiL : flux * phiR;
  double dq = qR - qL;
  double psi = 0.0;
  if (flux >= 0.0) {
    if (hasLL && std::fabs(dq) > 1.0e-14) {
      double r = (qL - qLL) / dq;
      psi = std::max(std::max(0.0, std::min(2.0 * r, 1.0)), std::min(r, 2.0));
    }
    return flux * (phiL + 0.5 * psi * (phiR - phiL));
  }
  if (hasRR && std::fabs(dq) > 1.0e-14) {
    double r = (qRR - qR) / dq;
    psi = std::max(std::max(0.0, std::min(2.0 * r, 1.0)), std::min(r, 2.0));
  }
  return flux * (phiR + 0.5 * psi * (phiL - phiR));
}

// src/module_navier_stokes.f90:2418-2457 compute_u_conv_fluxes
inline void u_conv_fluxes(const MomCtx& c, int i, int j, double& FE, double& FW, double& FN,
                          double& FS) {
  const Mesh& m = c.m;
  double un = c.u_adv[m.id(i, j)], unE = c.u_adv[m.id(i + 1, j)], unW = c.u_adv[m.id(i - 1, j)];
  double vnN = 0.5 * (c.v_adv[m.id(i - 1, j + 1)] + c.v_adv[m.id(i, j + 1)]);
  double vnS = 0.5 * (c.v_adv[m.id(i - 1, j)] + c.v_adv[m.id(i, j)]);
  if (c.u_nm1) {
    un = 2.0 * un - c.u_nm1[m.id(i, j)];
    unE = 2.0 * unE - c.u_nm1[m.id(i + 1, j)];
    unW = 2.0 * unW - c.u_nm1[m.id(i - 1, j)];
    double vmN = 0.5 * (c.v_nm1[m.id(i - 1, j + 1)] + c.v_nm1[m.id(i, j + 1)]);
    double vmS = 0.5 * (c.v_nm1[m.id(i - 1, j)] + c.v_nm1[m.id(i, j)]);
    vnN = 2.0 * vnN - vmN;
    vnS = 2.0 * vnS - vmS;
  }
  FE = 0.5 * (un + unE) * m.dy;
  FW = 0.5 * (unW + un) * m.dy;
  FN = vnN * m.dx;
  FS = vnS * m.dx;
}
// src/module_navier_stokes.f90:2459-2498 compute_v_conv_fluxes
inline void v_conv_fluxes(const MomCtx& c, int i, int j, double& FE, double& FW, double& FN,
                          double& FS) {
  const Mesh& m = c.m;
  double vn = c.v_adv[m.id(i, j)], vnN = c.v_adv[m.id(i, j + 1)], vnS = c.v_adv[m.id(i, j - 1)];
  double unE = 0.5 * (c.u_adv[m.id(i + 1, j - 1)] + c.u_adv[m.id(i + 1, j)]);
  double unW = 0.5 * (c.u_adv[m.id(i, j - 1)] + c.u_adv[m.id(i, j)]);
  if (c.u_nm1) {
    vn = 2.0 * vn - c.v_nm1[m.id(i, j)];
    vnN = 2.0 * vnN - c.v_nm1[m.id(i, j + 1)];
    vnS = 2.0 * vnS - c.v_nm1[m.id(i, j - 1)];
    double umE = 0.5 * (c.u_nm1[m.id(i + 1, j - 1)] + c.u_nm1[m.id(i + 1, j)]);
    double umW = 0.5 * (c.u_nm1[m.id(i, j - 1)] + c.u_nm1[m.id(i, j)]);
    unE = 2.0 * unE - umE;
    unW = 2.0 * unW - umW;
  }
  FE = unE * m.dy;
  FW = unW * m.dy;
  FN = 0.5 * (vn + vnN) * m.dx;
  FS = 0.5 * (vnS + vn) * m.dx;
}

// src/module_navier_stokes.f90:380-780 ns_apply_system_matrix (SP; Euler or
// Gear; PICARD or AB2; UPWIND / CENTERED / TVD_SUPERBEE; AL penalty; no
// obstacle terms).  tu/tv: the unpacked operand with the homogeneous ghost
// conditions applied (:458 -> src/module_mpi_comm.f90:290-537).  tp/yp
// (MONOLITHIC only): the operand's pressure (ghosts zero) and the
// continuity rows' image.
void mom_apply(const MomCtx& c, const double* tu, const double* tv, double* yu, double* yv,
               const double* tp = nullptr, double* yp = nullptr) {
  const Mesh& m = c.m;
  const covof_params* prm = c.prm;
  const double dx = m.dx, dy = m.dy, dvol = dx * dy, dt = c.dt;
  const int nx = m.nx, ny = m.ny, u_nx = c.u_nx, v_ny = c.v_ny;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= u_nx; ++i) {
      size_t k = m.id(i, j);
      double rho = c.rho_u[k];
      double diag_bc = ((c.alpha * rho) / dt) * dvol;
      if (i == 1) {
        if (prm->bc_type[L] == COVOF_BC_NEUMANN) yu[k] = diag_bc * (tu[m.id(1, j)] - tu[m.id(2, j)]);
        else yu[k] = diag_bc * tu[m.id(1, j)];
        continue;
      }
      if (i == u_nx) {
        if (prm->bc_type[R] == COVOF_BC_NEUMANN)
          yu[k] = diag_bc * (tu[m.id(u_nx, j)] - tu[m.id(u_nx - 1, j)]);
        else yu[k] = diag_bc * tu[m.id(u_nx, j)];
        continue;
      }
      double val = (((c.alpha * rho) / dt) * tu[k]) * dvol;
      if (prm->enable_convection) {
        double FE, FW, FN, FS;
        u_conv_fluxes(c, i, j, FE, FW, FN, FS);
        // :533-547: the limiter's neighbours come from fields_old%u
        const double* q = c.u_n;
        bool has_ee = i + 2 <= nx + 1, has_ww = i - 2 >= 0, has_nn = j + 2 <= ny + 1, has_ss = j - 2 >= 0;
        double q_ee = has_ee ? q[m.id(std::min(i + 2, nx + 1), j)] : 0.0;
        double q_ww = has_ww ? q[m.id(std::max(i - 2, 0), j)] : 0.0;
        double q_nn = has_nn ? q[m.id(i, std::min(j + 2, ny + 1))] : 0.0;
        double q_ss = has_ss ? q[m.id(i, std::max(j - 2, 0))] : 0.0;
        int s = prm->convective_scheme;
        double pE = conv_face_flux(s, FE, tu[k], tu[m.id(i + 1, j)], q[m.id(i - 1, j)], q[k],
                                   q[m.id(i + 1, j)], q_ee, true, has_ee);
        double pW = conv_face_flux(s, FW, tu[m.id(i - 1, j)], tu[k], q_ww, q[m.id(i - 1, j)], q[k],
                                   q[m.id(i + 1, j)], has_ww, true);
        double pN = conv_face_flux(s, FN, tu[k], tu[m.id(i, j + 1)], q[m.id(i, j - 1)], q[k],
                                   q[m.id(i, j + 1)], q_nn, true, has_nn);
        double pS = conv_face_flux(s, FS, tu[m.id(i, j - 1)], tu[k], q_ss, q[m.id(i, j - 1)], q[k],
                                   q[m.id(i, j + 1)], has_ss, true);
        val = val + rho * (pE - pW + pN - pS);
      }
      double muE = c.mu[m.id(i, j)], muW = c.mu[m.id(i - 1, j)];
      double dE = 2.0 * muE * (tu[m.id(i + 1, j)] - tu[k]) / dx * dy;
      double dW = 2.0 * muW * (tu[k] - tu[m.id(i - 1, j)]) / dx * dy;
      val = val - (dE - dW);
      double mN = c.mu_node[m.id(i, j + 1)], mS = c.mu_node[m.id(i, j)];
      double sN = mN * ((tu[m.id(i, j + 1)] - tu[k]) / dy + (tv[m.id(i, j + 1)] - tv[m.id(i - 1, j + 1)]) / dx) * dx;
      double sS = mS * ((tu[k] - tu[m.id(i, j - 1)]) / dy + (tv[m.id(i, j)] - tv[m.id(i - 1, j)]) / dx) * dx;
      val = val - (sN - sS);
      if (c.r_al) {
        // :584-595: -(r_E div(i,j) - r_W div(i-1,j)) dy, div of the operand
        double dE = (tu[m.id(i + 1, j)] - tu[k]) / dx + (tv[m.id(i, j + 1)] - tv[k]) / dy;
        double dW = (tu[k] - tu[m.id(i - 1, j)]) / dx + (tv[m.id(i - 1, j + 1)] - tv[m.id(i - 1, j)]) / dy;
        val = val - (c.r_al[k] * dE - c.r_al[m.id(i - 1, j)] * dW) * dy;
      }
      if (tp) val = val + (tp[k] - tp[m.id(i - 1, j)]) * dy;  // :597-602, B_u^T p
      yu[k] = val;
    }
  for (int j = 1; j <= v_ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = m.id(i, j);
      double rho = c.rho_v[k];
      double diag_bc = ((c.alpha * rho) / dt) * dvol;
      bool wb = (j == 1 && is_wall(prm, B));
      bool wt = (j == v_ny && is_wall(prm, T));
      if (wb || wt) { yv[k] = diag_bc * tv[k]; continue; }
      double val = (((c.alpha * rho) / dt) * tv[k]) * dvol;
      if (prm->enable_convection) {
        double FE, FW, FN, FS;
        v_conv_fluxes(c, i, j, FE, FW, FN, FS);
        // :666-680: the limiter's neighbours come from fields_old%v
        const double* q = c.v_n;
        bool has_ee = i + 2 <= nx + 1, has_ww = i - 2 >= 0, has_nn = j + 2 <= ny + 1, has_ss = j - 2 >= 0;
        double q_ee = has_ee ? q[m.id(std::min(i + 2, nx + 1), j)] : 0.0;
        double q_ww = has_ww ? q[m.id(std::max(i - 2, 0), j)] : 0.0;
        double q_nn = has_nn ? q[m.id(i, std::min(j + 2, ny + 1))] : 0.0;
        double q_ss = has_ss ? q[m.id(i, std::max(j - 2, 0))] : 0.0;
        int s = prm->convective_scheme;
        double pE = conv_face_flux(s, FE, tv[k], tv[m.id(i + 1, j)], q[m.id(i - 1, j)], q[k],
                                   q[m.id(i + 1, j)], q_ee, true, has_ee);
        double pW = conv_face_flux(s, FW, tv[m.id(i - 1, j)], tv[k], q_ww, q[m.id(i - 1, j)], q[k],
                                   q[m.id(i + 1, j)], has_ww, true);
        double pN = conv_face_flux(s, FN, tv[k], tv[m.id(i, j + 1)], q[m.id(i, j - 1)], q[k],
                                   q[m.id(i, j + 1)], q_nn, true, has_nn);
        double pS = conv_face_flux(s, FS, tv[m.id(i, j - 1)], tv[k], q_ss, q[m.id(i, j - 1)], q[k],
                                   q[m.id(i, j + 1)], has_ss, true);
        val = val + rho * (pE - pW + pN - pS);
      }
      double muN = c.mu[m.id(i, j)], muS = c.mu[m.id(i, j - 1)];
      double dN = 2.0 * muN * (tv[m.id(i, j + 1)] - tv[k]) / dy * dx;
      double dS = 2.0 * muS * (tv[k] - tv[m.id(i, j - 1)]) / dy * dx;
      val = val - (dN - dS);
      double mE = c.mu_node[m.id(i + 1, j)], mW = c.mu_node[m.id(i, j)];
      double sE = mE * ((tv[m.id(i + 1, j)] - tv[k]) / dx + (tu[m.id(i + 1, j)] - tu[m.id(i + 1, j - 1)]) / dy) * dy;
      double sW = mW * ((tv[k] - tv[m.id(i - 1, j)]) / dx + (tu[m.id(i, j)] - tu[m.id(i, j - 1)]) / dy) * dy;
      val = val - (sE - sW);
      if (c.r_al) {
        // :711-721: -(r_N div(i,j) - r_S div(i,j-1)) dx
        double dN = (tu[m.id(i + 1, j)] - tu[k]) / dx + (tv[m.id(i, j + 1)] - tv[k]) / dy;
        double dS = (tu[m.id(i + 1, j - 1)] - tu[m.id(i, j - 1)]) / dx + (tv[k] - tv[m.id(i, j - 1)]) / dy;
        val = val - (c.r_al[k] * dN - c.r_al[m.id(i, j - 1)] * dS) * dx;
      }
      if (tp) val = val + (tp[k] - tp[m.id(i, j - 1)]) * dx;  // :723-728
      yv[k] = val;
    }
  if (!tp || !yp) return;
  // :730-777 continuity rows: div u dvol, plus 1e-10 p(1,1) dvol in cell
  // (1,1) (the pressure level of the incompressible system)
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = m.id(i, j);
      double div = (tu[m.id(i + 1, j)] - tu[k]) / dx + (tv[m.id(i, j + 1)] - tv[k]) / dy;
      if (i == 1 && j == 1) yp[k] = div * dvol + 1.0e-10 * tp[k] * dvol;
      else yp[k] = div * dvol;
    }
}

// src/module_navier_stokes.f90:1541-1590: the pressure block's diagonal
// diag_p = schur_aP, the row sum of the Schur complement approximation
// B D^-1 B^T with D the momentum diagonals (du, dv after mom_diag), plus
// 1e-10 dvol in cell (1,1) and 1e-12 dvol elsewhere.
void schur_diag(const MomCtx& c, const double* du, const double* dv, double* dp) {
  const Mesh& m = c.m;
  const covof_params* prm = c.prm;
  const double dx = m.dx, dy = m.dy, dvol = dx * dy;
  const int nx = m.nx, ny = m.ny;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      double aW = 0.0, aE = 0.0, aS = 0.0, aN = 0.0;
      if (!(i == 1 && is_wall(prm, L))) aW = (dy * dy) / std::max(1.0e-30, du[m.id(i, j)]);
      if (!(i == nx && is_wall(prm, R))) aE = (dy * dy) / std::max(1.0e-30, du[m.id(i + 1, j)]);
      if (!(j == 1 && is_wall(prm, B))) aS = (dx * dx) / std::max(1.0e-30, dv[m.id(i, j)]);
      if (!(j == ny && is_wall(prm, T))) aN = (dx * dx) / std::max(1.0e-30, dv[m.id(i, j + 1)]);
      const double reg = (i == 1 && j == 1) ? 1.0e-10 * dvol : 1.0e-12 * dvol;
      dp[m.id(i, j)] = aW + aE + aS + aN + 0.0 + reg;
    }
}

// src/module_navier_stokes.f90:1268-1539 ns_assemble_preconditioner_blocks
// (diag_u / diag_v only; no AL / obstacle / Newton terms).
void mom_diag(const MomCtx& c, double* du, double* dv) {
  const Mesh& m = c.m;
  const covof_params* prm = c.prm;
  const double dx = m.dx, dy = m.dy, dvol = dx * dy;
  const double dt_safe = c.dt > 1.0e-30 ? c.dt : 1.0;
  const int nx = m.nx, ny = m.ny, u_nx = c.u_nx, v_ny = c.v_ny;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= u_nx; ++i) {
      size_t k = m.id(i, j);
      double rho = c.rho_u[k];
      double Du = ((c.alpha * rho) / dt_safe) * dvol;
      if (Du <= 1.0e-30) Du = 1.0;
      if (i == 1 || i == u_nx) { du[k] = Du; continue; }
      double mue = c.mu[m.id(i, j)], muw = c.mu[m.id(i - 1, j)];
      double cE = 2.0 * mue * (dy / dx), cW = 2.0 * muw * (dy / dx);
      double cNr = c.mu_node[m.id(i, j + 1)] * (dx / dy);
      double cSr = c.mu_node[m.id(i, j)] * (dx / dy);
      double cNv = cNr, cSv = cSr, dwy = 0.0;
      if (j == 1) {
        if (prm->bc_type[B] == COVOF_BC_DIRICHLET) dwy = dwy + (ny >= 2 ? 3.0 * cSr : 2.0 * cSr);
        cSv = 0.0;
      }
      if (j == ny) {
        if (prm->bc_type[T] == COVOF_BC_DIRICHLET) dwy = dwy + (ny >= 2 ? 3.0 * cNr : 2.0 * cNr);
        cNv = 0.0;
      }
      double conv_diag = 0.0;
      if (prm->enable_convection) {
        double FE, FW, FN, FS;
        u_conv_fluxes(c, i, j, FE, FW, FN, FS);
        conv_diag = rho * (std::max(FE, 0.0) + std::max(-FW, 0.0) + std::max(FN, 0.0) + std::max(-FS, 0.0));
      }
      double alW = 0.0, alE = 0.0;
      if (c.r_al) { alW = c.r_al[m.id(i - 1, j)] * (dy / dx); alE = c.r_al[k] * (dy / dx); }
      double aP = Du + dwy + conv_diag + 0.0 + 0.0 + cW + cE + cSv + cNv + alW + alE;
      if (aP <= 1.0e-15) aP = 1.0;
      du[k] = aP;
    }
  for (int j = 1; j <= v_ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = m.id(i, j);
      double rho = c.rho_v[k];
      double Dv = ((c.alpha * rho) / dt_safe) * dvol;
      if (Dv <= 1.0e-30) Dv = 1.0;
      bool wall = (j == 1 && is_wall(prm, B)) || (j == v_ny && is_wall(prm, T));
      if (wall) { dv[k] = Dv; continue; }
      if ((j == 1 && prm->bc_type[B] == COVOF_BC_NEUMANN) ||
          (j == v_ny && prm->bc_type[T] == COVOF_BC_NEUMANN)) { dv[k] = Dv; continue; }
      double mun = c.mu[m.id(i, j)], mus = c.mu[m.id(i, j - 1)];
      double cN = 2.0 * mun * (dx / dy), cS = 2.0 * mus * (dx / dy);
      double cEr = c.mu_node[m.id(i + 1, j)] * (dy / dx);
      double cWr = c.mu_node[m.id(i, j)] * (dy / dx);
      double cEv = cEr, cWv = cWr, dwx = 0.0;
      if (i == 1) {
        if (prm->bc_type[L] == COVOF_BC_DIRICHLET) dwx = dwx + 2.0 * cWr;
        cWv = 0.0;
      }
      if (i == nx) {
        if (prm->bc_type[R] == COVOF_BC_DIRICHLET) dwx = dwx + 2.0 * cEr;
        cEv = 0.0;
      }
      double conv_diag = 0.0;
      if (prm->enable_convection) {
        double FE, FW, FN, FS;
        v_conv_fluxes(c, i, j, FE, FW, FN, FS);
        conv_diag = rho * (std::max(FE, 0.0) + std::max(-FW, 0.0) + std::max(FN, 0.0) + std::max(-FS, 0.0));
      }
      double alS = 0.0, alN = 0.0;
      if (c.r_al) { alS = c.r_al[m.id(i, j - 1)] * (dx / dy); alN = c.r_al[k] * (dx / dy); }
      double aP = Dv + dwx + conv_diag + 0.0 + 0.0 + cWv + cEv + cS + cN + alS + alN;
      if (aP <= 1.0e-15) aP = 1.0;
      dv[k] = aP;
    }
}

// src/module_navier_stokes.f90:785-1101 ns_assemble_rhs (SP, constant walls;
// Euler or the Gear / BDF2 inertial term, :841-848 and :1022-1029)
void mom_rhs(const MomCtx& c, const double* mu_node, const double* fx, const double* fy,
             const double* u_old, const double* v_old, double* ru, double* rv) {
  const Mesh& m = c.m;
  const covof_params* prm = c.prm;
  const double dx = m.dx, dy = m.dy, dvol = dx * dy, dt = c.dt;
  const int nx = m.nx, ny = m.ny, u_nx = c.u_nx, v_ny = c.v_ny;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= u_nx; ++i) {
      size_t k = m.id(i, j);
      double rho = c.rho_u[k];
      double diag_bc = ((c.alpha * rho) / dt) * dvol;
      if (i == 1) {
        double ubc = prm->bc_type[L] == COVOF_BC_DIRICHLET ? prm->bc_u[L] : 0.0;
        ru[k] = diag_bc * ubc;
        continue;
      }
      if (i == u_nx) {
        double ubc = prm->bc_type[R] == COVOF_BC_DIRICHLET ? prm->bc_u[R] : 0.0;
        ru[k] = diag_bc * ubc;
        continue;
      }
      double val;
      if (c.gear_rhs) {
        double u_in = rho * (2.0 * u_old[k] - 0.5 * c.u_nm1_rhs[k]);
        val = (u_in / dt) * dvol;
      } else {
        val = (rho / dt) * u_old[k] * dvol;
      }
      val = val + rho * prm->gx * dvol;
      val = val + fx[k] * dvol;
      if (c.p_al) val = val - (c.p_al[k] - c.p_al[m.id(i - 1, j)]) * dy;  // :908-913
      if (j == ny && prm->bc_type[T] == COVOF_BC_DIRICHLET) {
        double mN = mu_node[m.id(i, j + 1)];
        if (ny >= 2) val = val + mN * ((8.0 / 3.0) * prm->bc_u[T] / dy) * dx;
        else val = val + mN * (2.0 * prm->bc_u[T] / dy) * dx;
      }
      if (j == 1 && prm->bc_type[B] == COVOF_BC_DIRICHLET) {
        double mS = mu_node[m.id(i, j)];
        if (ny >= 2) val = val + mS * ((8.0 / 3.0) * prm->bc_u[B] / dy) * dx;
        else val = val + mS * (2.0 * prm->bc_u[B] / dy) * dx;
      }
      ru[k] = val;
    }
  for (int j = 1; j <= v_ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = m.id(i, j);
      double rho = c.rho_v[k];
      double diag_bc = ((c.alpha * rho) / dt) * dvol;
      if (j == 1 && is_wall(prm, B)) {
        double vbc = prm->bc_type[B] == COVOF_BC_DIRICHLET ? prm->bc_v[B] : 0.0;
        rv[k] = diag_bc * vbc;
        continue;
      }
      if (j == v_ny && is_wall(prm, T)) {
        double vbc = prm->bc_type[T] == COVOF_BC_DIRICHLET ? prm->bc_v[T] : 0.0;
        rv[k] = diag_bc * vbc;
        continue;
      }
      double val;
      if (c.gear_rhs) {
        double v_in = rho * (2.0 * v_old[k] - 0.5 * c.v_nm1_rhs[k]);
        val = (v_in / dt) * dvol;
      } else {
        val = (rho / dt) * v_old[k] * dvol;
      }
      val = val + rho * prm->gy * dvol;
      val = val + fy[k] * dvol;
      if (c.p_al) val = val - (c.p_al[k] - c.p_al[m.id(i, j - 1)]) * dx;  // :1053-1058
      if (i == 1 && prm->bc_type[L] == COVOF_BC_DIRICHLET) {
        double mW = mu_node[m.id(i, j)];
        val = val + mW * (2.0 * prm->bc_v[L] / dx) * dy;
      }
      if (i == nx && prm->bc_type[R] == COVOF_BC_DIRICHLET) {
        double mE = mu_node[m.id(i + 1, j)];
        val = val + mE * (2.0 * prm->bc_v[R] / dx) * dy;
      }
      rv[k] = val;
    }
}

// src/module_navier_stokes.f90:1268-1595 ns_assemble_preconditioner_blocks:
// the five-point stencils of the u and v blocks for the SSOR sweeps (M-matrix
// form: aP r = z + aW r_W + aE r_E + aS r_S + aN r_N, convection upwinded),
// and for MONOLITHIC the Schur complement approximation B D^-1 B^T.  All
// arrays in the (0:nx+1, 0:ny+1) layout; u at faces i = 1..u_nx, v at faces
// j = 1..v_ny, the Schur stencil at cells.
struct PBlocks {
  std::vector<double> uW, uE, uS, uN, uP, vW, vE, vS, vN, vP, sW, sE, sS, sN, sP;
};

void prec_blocks(const MomCtx& c, PBlocks& Q) {
  const Mesh& m = c.m;
  const covof_params* prm = c.prm;
  const double dx = m.dx, dy = m.dy, dvol = dx * dy;
  const double dt_safe = c.dt > 1.0e-30 ? c.dt : 1.0;
  const int nx = m.nx, ny = m.ny, u_nx = c.u_nx, v_ny = c.v_ny;
  const size_t g = (size_t)(nx + 2) * (ny + 2);
  for (auto* v : {&Q.uW, &Q.uE, &Q.uS, &Q.uN, &Q.vW, &Q.vE, &Q.vS, &Q.vN, &Q.sW, &Q.sE, &Q.sS, &Q.sN})
    v->assign(g, 0.0);
  for (auto* v : {&Q.uP, &Q.vP, &Q.sP}) v->assign(g, 1.0);
  // 1. u block (:1312-1425)
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= u_nx; ++i) {
      size_t k = m.id(i, j);
      double rho = c.rho_u[k];
      double Du = ((c.alpha * rho) / dt_safe) * dvol;
      if (Du <= 1.0e-30) Du = 1.0;
      if (i == 1) {
        Q.uP[k] = Du;
        Q.uE[k] = (prm->bc_type[L] == COVOF_BC_NEUMANN && u_nx >= 2) ? Du : 0.0;
        continue;
      }
      if (i == u_nx) {
        Q.uP[k] = Du;
        Q.uW[k] = (prm->bc_type[R] == COVOF_BC_NEUMANN && u_nx >= 2) ? Du : 0.0;
        continue;
      }
      double mue = c.mu[m.id(i, j)], muw = c.mu[m.id(i - 1, j)];
      double cE = 2.0 * mue * (dy / dx), cW = 2.0 * muw * (dy / dx);
      double cNr = c.mu_node[m.id(i, j + 1)] * (dx / dy);
      double cSr = c.mu_node[m.id(i, j)] * (dx / dy);
      double cNv = cNr, cSv = cSr, dwy = 0.0, cNx = 0.0, cSx = 0.0;
      if (j == 1) {
        if (prm->bc_type[B] == COVOF_BC_DIRICHLET) {
          if (ny >= 2) { dwy = dwy + 3.0 * cSr; cNx = cNx + cSr / 3.0; }
          else dwy = dwy + 2.0 * cSr;
        }
        cSv = 0.0;
      }
      if (j == ny) {
        if (prm->bc_type[T] == COVOF_BC_DIRICHLET) {
          if (ny >= 2) { dwy = dwy + 3.0 * cNr; cSx = cSx + cNr / 3.0; }
          else dwy = dwy + 2.0 * cNr;
        }
        cNv = 0.0;
      }
      double cd = 0.0, cvW = 0.0, cvE = 0.0, cvS = 0.0, cvN = 0.0;
      if (prm->enable_convection) {
        double FE, FW, FN, FS;
        u_conv_fluxes(c, i, j, FE, FW, FN, FS);
        cd = rho * (std::max(FE, 0.0) + std::max(-FW, 0.0) + std::max(FN, 0.0) + std::max(-FS, 0.0));
        cvE = rho * std::max(-FE, 0.0);
        cvW = rho * std::max(FW, 0.0);
        cvN = (j == ny) ? 0.0 : rho * std::max(-FN, 0.0);
        cvS = (j == 1) ? 0.0 : rho * std::max(FS, 0.0);
      }
      double alE = 0.0, alW = 0.0;
      if (c.r_al) { alE = c.r_al[k] * (dy / dx); alW = c.r_al[m.id(i - 1, j)] * (dy / dx); }
      Q.uW[k] = cW + cvW + alW;
      Q.uE[k] = cE + cvE + alE;
      Q.uS[k] = cSv + cvS + cSx;
      Q.uN[k] = cNv + cvN + cNx;
      double aP = Du + dwy + cd + 0.0 + 0.0 + cW + cE + cSv + cNv + alW + alE;
      if (aP <= 1.0e-15) aP = 1.0;
      Q.uP[k] = aP;
    }
  // 2. v block (:1428-1539)
  for (int j = 1; j <= v_ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = m.id(i, j);
      double rho = c.rho_v[k];
      double Dv = ((c.alpha * rho) / dt_safe) * dvol;
      if (Dv <= 1.0e-30) Dv = 1.0;
      bool wall = (j == 1 && is_wall(prm, B)) || (j == v_ny && is_wall(prm, T));
      if (wall) { Q.vP[k] = Dv; continue; }
      if (j == 1 && prm->bc_type[B] == COVOF_BC_NEUMANN && v_ny >= 2) { Q.vP[k] = Dv; Q.vN[k] = Dv; continue; }
      if (j == v_ny && prm->bc_type[T] == COVOF_BC_NEUMANN && v_ny >= 2) { Q.vP[k] = Dv; Q.vS[k] = Dv; continue; }
      double mun = c.mu[m.id(i, j)], mus = c.mu[m.id(i, j - 1)];
      double cN = 2.0 * mun * (dx / dy), cS = 2.0 * mus * (dx / dy);
      double cEr = c.mu_node[m.id(i + 1, j)] * (dy / dx);
      double cWr = c.mu_node[m.id(i, j)] * (dy / dx);
      double cEv = cEr, cWv = cWr, dwx = 0.0;
      if (i == 1) {
        if (prm->bc_type[L] == COVOF_BC_DIRICHLET) dwx = dwx + 2.0 * cWr;
        cWv = 0.0;
      }
      if (i == nx) {
        if (prm->bc_type[R] == COVOF_BC_DIRICHLET) dwx = dwx + 2.0 * cEr;
        cEv = 0.0;
      }
      double cd = 0.0, cvW = 0.0, cvE = 0.0, cvS = 0.0, cvN = 0.0;
      if (prm->enable_convection) {
        double FE, FW, FN, FS;
        v_conv_fluxes(c, i, j, FE, FW, FN, FS);
        cd = rho * (std::max(FE, 0.0) + std::max(-FW, 0.0) + std::max(FN, 0.0) + std::max(-FS, 0.0));
        cvE = (i == nx) ? 0.0 : rho * std::max(-FE, 0.0);
        cvW = (i == 1) ? 0.0 : rho * std::max(FW, 0.0);
        cvN = rho * std::max(-FN, 0.0);
        cvS = rho * std::max(FS, 0.0);
      }
      double alN = 0.0, alS = 0.0;
      if (c.r_al) { alN = c.r_al[k] * (dx / dy); alS = c.r_al[m.id(i, j - 1)] * (dx / dy); }
      Q.vW[k] = cWv + cvW;
      Q.vE[k] = cEv + cvE;
      Q.vS[k] = cS + cvS + alS;
      Q.vN[k] = cN + cvN + alN;
      double aP = Dv + dwx + cd + 0.0 + 0.0 + cWv + cEv + cS + cN + alS + alN;
      if (aP <= 1.0e-15) aP = 1.0;
      Q.vP[k] = aP;
    }
  // 3 & 4. Schur stencil (:1542-1590), from the blocks' diagonals
  if (!c.mono) return;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = m.id(i, j);
      if (!(i == 1 && is_wall(prm, L))) Q.sW[k] = (dy * dy) / std::max(1.0e-30, Q.uP[m.id(i, j)]);
      if (!(i == nx && is_wall(prm, R))) Q.sE[k] = (dy * dy) / std::max(1.0e-30, Q.uP[m.id(i + 1, j)]);
      if (!(j == 1 && is_wall(prm, B))) Q.sS[k] = (dx * dx) / std::max(1.0e-30, Q.vP[m.id(i, j)]);
      if (!(j == ny && is_wall(prm, T))) Q.sN[k] = (dx * dx) / std::max(1.0e-30, Q.vP[m.id(i, j + 1)]);
      const double reg = (i == 1 && j == 1) ? 1.0e-10 * dvol : 1.0e-12 * dvol;
      Q.sP[k] = Q.sW[k] + Q.sE[k] + Q.sS[k] + Q.sN[k] + 0.0 + reg;
    }
}

// src/module_linear_solvers.f90:1278-1401 ssor_solve_p / _u / _v: r = 0,
// then n_sweeps pairs of lexicographic Gauss-Seidel sweeps (rows j = 1..nj,
// columns i = 1..ni, then the reverse), each cell relaxed
// r = (1 - omega) r + omega (z + sum of the non-zero a_nb r_nb) / aP.
// Ghost entries of r stay zero (one rank, no halo exchange).
void ssor_solve(const Mesh& m, int ni, int nj, const double* aW, const double* aE, const double* aS,
                const double* aN, const double* aP, const double* z, double* r, int n_sweeps, double omega) {
  const size_t g = (size_t)(m.nx + 2) * (m.ny + 2);
  std::fill(r, r + g, 0.0);
  auto cell = [&](int i, int j) {
    const size_t k = m.id(i, j);
    double d = aP[k];
    if (std::fabs(d) < 1.0e-30) d = 1.0;
    double val = z[k];
    if (aW[k] != 0.0) val = val + aW[k] * r[k - 1];
    if (aE[k] != 0.0) val = val + aE[k] * r[k + 1];
    if (aS[k] != 0.0) val = val + aS[k] * r[k - m.P];
    if (aN[k] != 0.0) val = val + aN[k] * r[k + m.P];
    r[k] = (1.0 - omega) * r[k] + omega * (val / d);
  };
  for (int s = 0; s < n_sweeps; ++s) {
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) cell(i, j);
    for (int j = nj; j >= 1; --j)
      for (int i = ni; i >= 1; --i) cell(i, j);
  }
}

inline bool uses_sweeps(const covof_params* prm) {
  return prm->use_precond && (prm->precond == COVOF_PRECOND_SSOR || prm->precond == COVOF_PRECOND_BLOCK_TRIANGULAR);
}

// Packed Krylov vectors: u DOFs (i=1..u_nx, j=1..ny) then v DOFs
// (i=1..nx, j=1..v_ny), src/module_navier_stokes.f90:231-296.
// MONOLITHIC adds the pressure DOFs (i=1..nx, j=1..ny) after them
// (:281-294, :352-371).
struct Packer {
  const MomCtx& c;
  size_t n() const { return c.nu + c.nv + (c.mono ? c.np : 0); }
  void pack(const double* u, const double* v, double* x, const double* p = nullptr) const {
    const Mesh& m = c.m;
    size_t d = 0;
    for (int j = 1; j <= m.ny; ++j) for (int i = 1; i <= c.u_nx; ++i) x[d++] = u[m.id(i, j)];
    for (int j = 1; j <= c.v_ny; ++j) for (int i = 1; i <= m.nx; ++i) x[d++] = v[m.id(i, j)];
    if (c.mono)
      for (int j = 1; j <= m.ny; ++j) for (int i = 1; i <= m.nx; ++i) x[d++] = p ? p[m.id(i, j)] : 0.0;
  }
  void unpack(const double* x, double* u, double* v, double* p = nullptr) const {
    const Mesh& m = c.m;
    size_t d = 0;
    for (int j = 1; j <= m.ny; ++j) for (int i = 1; i <= c.u_nx; ++i) u[m.id(i, j)] = x[d++];
    for (int j = 1; j <= c.v_ny; ++j) for (int i = 1; i <= m.nx; ++i) v[m.id(i, j)] = x[d++];
    if (c.mono && p)
      for (int j = 1; j <= m.ny; ++j) for (int i = 1; i <= m.nx; ++i) p[m.id(i, j)] = x[d++];
  }
};

struct Krylov {
  const MomCtx& c;
  Packer pk;
  std::vector<double> tu, tv, yu, yv, tp, yp, diag;  // tf (saved operand), diag packed
  PBlocks blk;  // SSOR / BLOCK_TRIANGULAR stencils (prec_blocks)
  explicit Krylov(const MomCtx& cc) : c(cc), pk{cc} {
    size_t g = (size_t)(c.m.nx + 2) * (c.m.ny + 2);
    tu.assign(g, 0.0); tv.assign(g, 0.0); yu.assign(g, 0.0); yv.assign(g, 0.0);
    tp.assign(g, 0.0); yp.assign(g, 0.0);  // tf%p: ghosts stay zero
  }
  // ns_apply_system_matrix with unpack + homogeneous BC (:397-458)
  void A(const double* x, double* y) {
    pk.unpack(x, tu.data(), tv.data(), tp.data());
    velocity_bc(c.prm, c.m, tu.data(), tv.data(), true);
    if (c.mono) {
      mom_apply(c, tu.data(), tv.data(), yu.data(), yv.data(), tp.data(), yp.data());
      pk.pack(yu.data(), yv.data(), y, yp.data());
    } else {
      mom_apply(c, tu.data(), tv.data(), yu.data(), yv.data());
      pk.pack(yu.data(), yv.data(), y);
    }
  }
  // src/module_linear_solvers.f90:88-117 (JACOBI) / :280-304 (ILU0 = same),
  // :137-278 (SSOR, BLOCK_TRIANGULAR)
  void M(const double* src, double* dst) {
    size_t n = pk.n();
    const int pc = c.prm->use_precond ? c.prm->precond : COVOF_PRECOND_NONE;
    if (pc == COVOF_PRECOND_SSOR || pc == COVOF_PRECOND_BLOCK_TRIANGULAR) { sweeps(src, dst, pc); return; }
    bool on = pc == COVOF_PRECOND_JACOBI || pc == COVOF_PRECOND_ILU0;
    for (size_t q = 0; q < n; ++q) {
      double d = diag[q];
      dst[q] = (on && std::fabs(d) > 1.0e-15) ? src[q] / d : src[q];
    }
  }
  // SSOR: two symmetric sweeps with omega = 1 on each block (the Schur
  // stencil for the pressure).  BLOCK_TRIANGULAR with MONOLITHIC: twelve
  // sweeps with omega = 1.25 on the Schur complement, its mean removed, then
  // four sweeps on each velocity block with the right-hand side z - B^T r_p
  // (wall DOFs keep z); without MONOLITHIC it is the SSOR of the velocity
  // blocks (:265-276).
  void sweeps(const double* src, double* dst, int pc) {
    const Mesh& m = c.m;
    const size_t g = (size_t)(m.nx + 2) * (m.ny + 2);
    const int nx = m.nx, ny = m.ny, u_nx = c.u_nx, v_ny = c.v_ny;
    std::vector<double> zu(g, 0.0), zv(g, 0.0), zp(g, 0.0), ru(g), rv(g), rp(g, 0.0);
    pk.unpack(src, zu.data(), zv.data(), zp.data());
    const PBlocks& Q = blk;
    if (pc == COVOF_PRECOND_SSOR || !c.mono) {
      ssor_solve(m, u_nx, ny, Q.uW.data(), Q.uE.data(), Q.uS.data(), Q.uN.data(), Q.uP.data(), zu.data(),
                 ru.data(), 2, 1.0);
      ssor_solve(m, nx, v_ny, Q.vW.data(), Q.vE.data(), Q.vS.data(), Q.vN.data(), Q.vP.data(), zv.data(),
                 rv.data(), 2, 1.0);
      if (c.mono)
        ssor_solve(m, nx, ny, Q.sW.data(), Q.sE.data(), Q.sS.data(), Q.sN.data(), Q.sP.data(), zp.data(),
                   rp.data(), 2, 1.0);
      pk.pack(ru.data(), rv.data(), dst, rp.data());
      return;
    }
    ssor_solve(m, nx, ny, Q.sW.data(), Q.sE.data(), Q.sS.data(), Q.sN.data(), Q.sP.data(), zp.data(),
               rp.data(), 12, 1.25);
    double sum = 0.0;
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) sum += rp[m.id(i, j)];
    const double mean = sum / (double)((long long)nx * ny);
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) rp[m.id(i, j)] = rp[m.id(i, j)] - mean;
    std::vector<double> hu(g, 0.0), hv(g, 0.0);
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= u_nx; ++i) {
        const size_t k = m.id(i, j);
        hu[k] = (i == 1 || i == u_nx) ? zu[k] : zu[k] - (rp[k] - rp[k - 1]) * m.dy;
      }
    ssor_solve(m, u_nx, ny, Q.uW.data(), Q.uE.data(), Q.uS.data(), Q.uN.data(), Q.uP.data(), hu.data(),
               ru.data(), 4, 1.0);
    for (int j = 1; j <= v_ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t k = m.id(i, j);
        const bool wall = (j == 1 && is_wall(c.prm, B)) || (j == v_ny && is_wall(c.prm, T));
        hv[k] = wall ? zv[k] : zv[k] - (rp[k] - rp[k - m.P]) * m.dx;
      }
    ssor_solve(m, nx, v_ny, Q.vW.data(), Q.vE.data(), Q.vS.data(), Q.vN.data(), Q.vP.data(), hv.data(),
               rv.data(), 4, 1.0);
    pk.pack(ru.data(), rv.data(), dst, rp.data());
  }
  void PA(const double* src, double* dst) {  // apply_PA (:323-356)
    std::vector<double> tmp(pk.n());
    A(src, tmp.data());
    M(tmp.data(), dst);
  }
};

// src/module_linear_solvers.f90:584-730 solve_bicgstab
int solve_bicgstab(Krylov& K, const double* b, double* x, int* iters) {
  const covof_params* prm = K.c.prm;
  size_t n = K.pk.n();
  double tol = prm->tol;
  int max_iter = prm->max_iter;
  *iters = max_iter;
  std::vector<double> bh(n), r(n), rt(n), p(n), v(n), s(n), t(n);
  K.M(b, bh.data());
  K.PA(x, r.data());
  for (size_t q = 0; q < n; ++q) r[q] = bh[q] - r[q];
  double r0 = std::sqrt(dot(r.data(), r.data(), n));
  if (r0 < 1.0e-12) { *iters = 0; return COVOF_OK; }
  rt = r;
  double rho_old = 1.0, alpha = 1.0, omega = 1.0;
  for (int it = 1; it <= max_iter; ++it) {
    double rho = dot(rt.data(), r.data(), n);
    if (std::fabs(rho) < 1.0e-30) return COVOF_BREAKDOWN;
    if (it == 1) p = r;
    else {
      double beta = (rho / rho_old) * (alpha / omega);
      for (size_t q = 0; q < n; ++q) p[q] = r[q] + beta * (p[q] - omega * v[q]);
    }
    K.PA(p.data(), v.data());
    double den = dot(rt.data(), v.data(), n);
    if (std::fabs(den) < 1.0e-30) return COVOF_BREAKDOWN;
    alpha = rho / den;
    for (size_t q = 0; q < n; ++q) s[q] = r[q] - alpha * v[q];
    double sn = std::sqrt(dot(s.data(), s.data(), n));
    if (sn != sn || sn > 1.0e30) return COVOF_NAN;
    if (sn / r0 < tol || sn < 1.0e-12) {
      for (size_t q = 0; q < n; ++q) x[q] = x[q] + alpha * p[q];
      *iters = it;
      return COVOF_OK;
    }
    K.PA(s.data(), t.data());
    double tt = dot(t.data(), t.data(), n);
    omega = tt > 1.0e-30 ? dot(t.data(), s.data(), n) / tt : 0.0;
    for (size_t q = 0; q < n; ++q) x[q] = x[q] + alpha * p[q] + omega * s[q];
    for (size_t q = 0; q < n; ++q) r[q] = s[q] - omega * t[q];
    rho_old = rho;
    double rn = std::sqrt(dot(r.data(), r.data(), n));
    if (rn != rn || rn > 1.0e30) return COVOF_NAN;
    if (rn / r0 < tol || rn < 1.0e-12) { *iters = it; return COVOF_OK; }
    if (std::fabs(omega) < 1.0e-30) return COVOF_BREAKDOWN;
  }
  return COVOF_MAXITER;
}

// src/module_linear_solvers.f90:361-579 solve_bicgstab2
int solve_bicgstab2(Krylov& K, const double* b, double* x, int* iters) {
  const covof_params* prm = K.c.prm;
  size_t n = K.pk.n();
  double tol = prm->tol;
  int max_iter = prm->max_iter;
  *iters = 0;
  std::vector<double> bh(n), rt(n), r0(n), r1(n, 0.0), r2(n, 0.0), u0(n, 0.0), u1(n, 0.0), u2(n, 0.0);
  K.M(b, bh.data());
  K.PA(x, r0.data());
  for (size_t q = 0; q < n; ++q) r0[q] = bh[q] - r0[q];
  double r0n = std::sqrt(dot(r0.data(), r0.data(), n));
  if (r0n < 1.0e-12) return COVOF_OK;
  rt = r0;
  double rho0 = 1.0, alpha = 0.0, omega = 1.0;
  int iter = 0;
  int status = COVOF_MAXITER;
  while (iter < max_iter) {
    iter = iter + 2;
    rho0 = -omega * rho0;
    double rho1 = dot(rt.data(), r0.data(), n);
    if (std::fabs(rho0) < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    double beta = alpha * (rho1 / rho0);
    rho0 = rho1;
    for (size_t q = 0; q < n; ++q) u0[q] = r0[q] - beta * u0[q];
    K.PA(u0.data(), u1.data());
    double gamma = dot(rt.data(), u1.data(), n);
    if (std::fabs(gamma) < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    alpha = rho0 / gamma;
    for (size_t q = 0; q < n; ++q) r0[q] = r0[q] - alpha * u1[q];
    for (size_t q = 0; q < n; ++q) x[q] = x[q] + alpha * u0[q];
    K.PA(r0.data(), r1.data());
    rho1 = dot(rt.data(), r1.data(), n);
    if (std::fabs(rho0) < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    beta = alpha * (rho1 / rho0);
    rho0 = rho1;
    for (size_t q = 0; q < n; ++q) u0[q] = r0[q] - beta * u0[q];
    for (size_t q = 0; q < n; ++q) u1[q] = r1[q] - beta * u1[q];
    K.PA(u1.data(), u2.data());
    gamma = dot(rt.data(), u2.data(), n);
    if (std::fabs(gamma) < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    alpha = rho0 / gamma;
    for (size_t q = 0; q < n; ++q) x[q] = x[q] + alpha * u0[q];
    for (size_t q = 0; q < n; ++q) r0[q] = r0[q] - alpha * u1[q];
    for (size_t q = 0; q < n; ++q) r1[q] = r1[q] - alpha * u2[q];
    K.PA(r1.data(), r2.data());
    double s11 = dot(r1.data(), r1.data(), n);
    double s12 = dot(r2.data(), r1.data(), n);
    double s22 = dot(r2.data(), r2.data(), n);
    double rhs1 = dot(r0.data(), r1.data(), n);
    double rhs2 = dot(r0.data(), r2.data(), n);
    double rn1 = std::sqrt(s11), rn2 = std::sqrt(s22), g1, g2;
    if (rn1 < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    else if (rn2 < 1.0e-300) { g2 = 0.0; g1 = rhs1 / s11; }
    else {
      double i1 = 1.0 / rn1, i2 = 1.0 / rn2;
      double c12 = s12 * i1 * i2;
      double b1 = rhs1 * i1, b2 = rhs2 * i2;
      double det = 1.0 - c12 * c12;
      if (std::fabs(det) < 1.0e-14) { g2 = 0.0; g1 = b1 * i1; }
      else { g1 = (b1 - c12 * b2) / (det * rn1); g2 = (b2 - c12 * b1) / (det * rn2); }
    }
    for (size_t q = 0; q < n; ++q) x[q] = x[q] + g1 * r0[q] + g2 * r1[q];
    for (size_t q = 0; q < n; ++q) r0[q] = r0[q] - (g1 * r1[q] + g2 * r2[q]);
    for (size_t q = 0; q < n; ++q) u0[q] = u0[q] - (g1 * u1[q] + g2 * u2[q]);
    if (g2 != 0.0) omega = g2;
    else if (std::fabs(g1) > 1.0e-300) omega = g1;
    else omega = 1.0;
    double rn = std::sqrt(dot(r0.data(), r0.data(), n));
    if (rn != rn || rn > 1.0e30) { status = COVOF_NAN; break; }
    if (rn / r0n < tol || rn < 1.0e-12) { *iters = iter; return COVOF_OK; }
  }
  *iters = iter;
  return status;
}

// src/module_linear_solvers.f90:735-838 solve_cg
int solve_cg(Krylov& K, const double* b, double* x, int* iters) {
  const covof_params* prm = K.c.prm;
  size_t n = K.pk.n();
  double tol = prm->tol;
  int max_iter = prm->max_iter;
  *iters = max_iter;
  std::vector<double> Ax(n), r(n), z(n), p(n), Ap(n);
  K.A(x, Ax.data());
  for (size_t q = 0; q < n; ++q) r[q] = b[q] - Ax[q];
  double r0 = std::sqrt(dot(r.data(), r.data(), n));
  if (r0 < 1.0e-12) { *iters = 0; return COVOF_OK; }
  K.M(r.data(), z.data());
  p = z;
  double rz_old = dot(r.data(), z.data(), n);
  for (int it = 1; it <= max_iter; ++it) {
    K.A(p.data(), Ap.data());
    double pAp = dot(p.data(), Ap.data(), n);
    if (std::fabs(pAp) < 1.0e-30) return COVOF_BREAKDOWN;
    double alpha = rz_old / pAp;
    for (size_t q = 0; q < n; ++q) x[q] = x[q] + alpha * p[q];
    for (size_t q = 0; q < n; ++q) r[q] = r[q] - alpha * Ap[q];
    double rn = std::sqrt(dot(r.data(), r.data(), n));
    if (rn / r0 < tol || rn < 1.0e-13) { *iters = it; return COVOF_OK; }
    K.M(r.data(), z.data());
    double rz_new = dot(r.data(), z.data(), n);
    double beta = rz_new / rz_old;
    rz_old = rz_new;
    for (size_t q = 0; q < n; ++q) p[q] = z[q] + beta * p[q];
  }
  return COVOF_MAXITER;
}

MomCtx make_ctx(const covof_params* prm, double dt, const double* u_n, const double* v_n,
                const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                const Hist& h = Hist()) {
  MomCtx c;
  c.prm = prm; c.m = mesh_of(prm); c.dt = dt;
  c.u_n = u_n; c.v_n = v_n; c.rho_u = rho_u; c.rho_v = rho_v; c.mu = mu; c.mu_node = mu_node;
  const bool gear = prm->time_scheme == COVOF_TIME_GEAR && h.has_nm1;
  const bool ab2 = prm->convective_linearization == COVOF_CONV_LIN_AB2;
  c.alpha = gear ? 1.5 : 1.0;
  c.gear_rhs = gear;
  c.u_adv = (ab2 && h.u_old) ? h.u_old : u_n;
  c.v_adv = (ab2 && h.v_old) ? h.v_old : v_n;
  c.u_nm1 = (ab2 && h.has_nm1) ? h.u_nm1 : nullptr;
  c.v_nm1 = (ab2 && h.has_nm1) ? h.v_nm1 : nullptr;
  c.u_nm1_rhs = h.u_nm1; c.v_nm1_rhs = h.v_nm1;
  c.u_nx = prm->nx + 1; c.v_ny = prm->ny + 1;
  c.nu = (size_t)c.u_nx * prm->ny; c.nv = (size_t)prm->nx * c.v_ny;
  return c;
}

// src/module_simulation.f90:2454-2470: diag, rhs, pack, solve, unpack, BC
int predictor(const covof_params* prm, double dt, double* u, double* v, const double* rho_u,
              const double* rho_v, const double* mu, const double* mu_node, const double* fx,
              const double* fy, const double* u_old, const double* v_old, const Hist& hist,
              int* iters) {
  // fields_old for the operator is the current field (u^n) itself.
  size_t g = (size_t)(prm->nx + 2) * (prm->ny + 2);
  std::vector<double> un(u, u + g), vn(v, v + g);
  MomCtx c = make_ctx(prm, dt, un.data(), vn.data(), rho_u, rho_v, mu, mu_node, hist);
  Krylov K(c);
  std::vector<double> du(g, 1.0), dv(g, 1.0), ru(g, 0.0), rv(g, 0.0);
  mom_diag(c, du.data(), dv.data());
  K.diag.resize(K.pk.n());
  K.pk.pack(du.data(), dv.data(), K.diag.data());
  if (uses_sweeps(prm)) prec_blocks(c, K.blk);
  mom_rhs(c, mu_node, fx, fy, u_old, v_old, ru.data(), rv.data());
  std::vector<double> rhs(K.pk.n()), x(K.pk.n());
  K.pk.pack(ru.data(), rv.data(), rhs.data());
  K.pk.pack(un.data(), vn.data(), x.data());
  int st;
  switch (prm->linear_solver) {
    case COVOF_LINEAR_BICGSTAB: st = solve_bicgstab(K, rhs.data(), x.data(), iters); break;
    case COVOF_LINEAR_CG: st = solve_cg(K, rhs.data(), x.data(), iters); break;
    default: st = solve_bicgstab2(K, rhs.data(), x.data(), iters); break;
  }
  K.pk.unpack(x.data(), u, v);
  velocity_bc(prm, c.m, u, v, false);
  return st;
}

// src/module_navier_stokes.f90:1106-1218 ns_compute_adaptative_r_al
// (incompressible): r_aal = r_al everywhere, or with adaptative_al the
// per-cell k_aal * max(unsteady, inertial, gravity, pressure, viscous,
// capillary scales).
void al_penalty(const covof_params* prm, const Mesh& m, double dt, const double* u, const double* v,
                const double* p, const double* rho, const double* mu, int has_nm1, double* r) {
  const int nx = m.nx, ny = m.ny;
  size_t g = (size_t)(nx + 2) * (ny + 2);
  if (!prm->adaptative_al) {
    for (size_t k = 0; k < g; ++k) r[k] = prm->r_al;
    return;
  }
  const double lx = nx * m.dx, ly = ny * m.dy;
  double L0;
  if (prm->l0_ref > 0.0) L0 = prm->l0_ref;
  else if (prm->enable_two_phase && prm->ic_radius > 0.0) L0 = 2.0 * prm->ic_radius;
  else L0 = std::min(lx, ly);
  const double t0 = prm->t0_ref > 0.0 ? prm->t0_ref : dt;
  const double g_norm = std::sqrt(prm->gx * prm->gx + prm->gy * prm->gy);
  const double sigma_val = prm->enable_two_phase ? prm->sigma : 0.0;
  const double alpha_time = (prm->time_scheme == COVOF_TIME_GEAR && has_nm1) ? 1.5 : 1.0;
  double u_max = 0.0, p_max = 0.0;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      double uc = 0.5 * (u[m.id(i, j)] + u[m.id(i + 1, j)]);
      double vc = 0.5 * (v[m.id(i, j)] + v[m.id(i, j + 1)]);
      double spd = std::sqrt(uc * uc + vc * vc);
      if (spd > u_max) u_max = spd;
      double pa = std::fabs(p[m.id(i, j)]);
      if (pa > p_max) p_max = pa;
    }
  double u0 = prm->u0_ref > 0.0 ? prm->u0_ref : u_max;
  if (u0 < 1.0e-12) {
    double u_grav = g_norm > 0.0 ? std::sqrt(g_norm * L0) : 0.0;
    double mu_max = std::max(prm->mu1, prm->mu2);
    double u_cap = (sigma_val > 0.0 && mu_max > 1.0e-30) ? sigma_val / mu_max : 0.0;
    u0 = std::max(std::max(std::max(u_grav, u_cap), L0 / std::max(t0, 1.0e-12)), 1.0e-3);
  }
  const double p0 = prm->p0_ref > 0.0 ? prm->p0_ref : p_max;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = m.id(i, j);
      double rM = rho[k], mM = mu[k];
      double t_uns = alpha_time * rM * (L0 * L0) / std::max(t0, 1.0e-30);
      double t_in = rM * u0 * L0;
      double t_gr = rM * (L0 * L0 / u0) * g_norm;
      double t_pr = (p0 * L0) / u0;
      double t_vi = mM;
      double t_ca = sigma_val / u0;
      double mx = std::max(std::max(std::max(t_uns, t_in), std::max(t_gr, t_pr)),
                           std::max(std::max(t_vi, 0.0), t_ca));
      double rl = prm->k_aal * mx;
      if (rl <= 1.0e-15) rl = prm->r_al;
      r[k] = rl;
    }
}

// max over interior cells of |div u| (src/module_simulation.f90:590-604)
double max_div(const Mesh& m, const double* u, const double* v) {
  double mx = 0.0;
  for (int j = 1; j <= m.ny; ++j)
    for (int i = 1; i <= m.nx; ++i) {
      double d = std::fabs((u[m.id(i + 1, j)] - u[m.id(i, j)]) / m.dx + (v[m.id(i, j + 1)] - v[m.id(i, j)]) / m.dy);
      if (d > mx) mx = d;
    }
  return mx;
}

// src/module_simulation.f90:553-607 for solver_type AUGMENTED_LAGRANGIAN /
// AAL: penalty field, preconditioner diagonal once, then Uzawa iterations of
// rhs (with -grad p), pack, Krylov solve (operator linearised about the
// current u), unpack + velocity BC, p -= r div u (:1223-1263), with the
// max |div u| exit test when uzawa_iter > 1 and uzawa_tol > 0.
int al_step(const covof_params* prm, double dt, double* u, double* v, double* p, const double* rho,
            const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
            const double* fx, const double* fy, const Hist& hist, int* iters, int* uzawa_done) {
  const Mesh m = mesh_of(prm);
  const size_t g = (size_t)(prm->nx + 2) * (prm->ny + 2);
  std::vector<double> r(g, 0.0);
  al_penalty(prm, m, dt, u, v, p, rho, mu, hist.has_nm1, r.data());
  std::vector<double> un(u, u + g), vn(v, v + g);
  MomCtx c = make_ctx(prm, dt, un.data(), vn.data(), rho_u, rho_v, mu, mu_node, hist);
  c.r_al = r.data();
  c.p_al = p;
  Krylov K(c);
  std::vector<double> du(g, 1.0), dv(g, 1.0), ru(g, 0.0), rv(g, 0.0);
  mom_diag(c, du.data(), dv.data());
  K.diag.resize(K.pk.n());
  K.pk.pack(du.data(), dv.data(), K.diag.data());
  if (uses_sweeps(prm)) prec_blocks(c, K.blk);
  const int umax = prm->uzawa_iter > 0 ? prm->uzawa_iter : 1;
  int total = 0, st = COVOF_OK, m_done = 0;
  for (int mi = 1; mi <= umax; ++mi) {
    m_done = mi;
    mom_rhs(c, mu_node, fx, fy, hist.u_old, hist.v_old, ru.data(), rv.data());
    std::vector<double> rhs(K.pk.n()), x(K.pk.n());
    K.pk.pack(ru.data(), rv.data(), rhs.data());
    K.pk.pack(u, v, x.data());
    // the operator's fields_old is the current field
    std::memcpy(un.data(), u, g * sizeof(double));
    std::memcpy(vn.data(), v, g * sizeof(double));
    int it = 0;
    switch (prm->linear_solver) {
      case COVOF_LINEAR_BICGSTAB: st = solve_bicgstab(K, rhs.data(), x.data(), &it); break;
      case COVOF_LINEAR_CG: st = solve_cg(K, rhs.data(), x.data(), &it); break;
      default: st = solve_bicgstab2(K, rhs.data(), x.data(), &it); break;
    }
    total += it;
    if (st == COVOF_NAN) break;
    K.pk.unpack(x.data(), u, v);
    velocity_bc(prm, m, u, v, false);
    for (int j = 1; j <= m.ny; ++j)
      for (int i = 1; i <= m.nx; ++i) {
        size_t k = m.id(i, j);
        double dv_ = (u[m.id(i + 1, j)] - u[k]) / m.dx + (v[m.id(i, j + 1)] - v[k]) / m.dy;
        p[k] = p[k] - r[k] * dv_;
      }
    if (umax > 1 && prm->uzawa_tol > 0.0 && max_div(m, u, v) <= prm->uzawa_tol) break;
  }
  if (iters) *iters = total;
  if (uzawa_done) *uzawa_done = m_done;
  return st;
}

// src/module_simulation.f90:552-583 for solver_type MONOLITHIC: the
// preconditioner blocks (momentum diagonals and the Schur diagonal diag_p),
// the right-hand side (momentum without a pressure term, zero continuity
// block, :1079-1100), pack (u, v, p), one Krylov solve of the coupled system,
// unpack (u, v, p) and the velocity boundary conditions.
int mono_step(const covof_params* prm, double dt, double* u, double* v, double* p, const double* rho_u,
              const double* rho_v, const double* mu, const double* mu_node, const double* fx,
              const double* fy, const Hist& hist, int* iters) {
  const Mesh m = mesh_of(prm);
  const size_t g = (size_t)(prm->nx + 2) * (prm->ny + 2);
  std::vector<double> un(u, u + g), vn(v, v + g);
  MomCtx c = make_ctx(prm, dt, un.data(), vn.data(), rho_u, rho_v, mu, mu_node, hist);
  c.mono = true;
  c.np = (size_t)prm->nx * prm->ny;
  Krylov K(c);
  std::vector<double> du(g, 1.0), dv(g, 1.0), dp(g, 1.0), ru(g, 0.0), rv(g, 0.0);
  mom_diag(c, du.data(), dv.data());
  schur_diag(c, du.data(), dv.data(), dp.data());
  K.diag.resize(K.pk.n());
  K.pk.pack(du.data(), dv.data(), K.diag.data(), dp.data());
  if (uses_sweeps(prm)) prec_blocks(c, K.blk);
  mom_rhs(c, mu_node, fx, fy, hist.u_old, hist.v_old, ru.data(), rv.data());
  std::vector<double> rhs(K.pk.n()), x(K.pk.n());
  K.pk.pack(ru.data(), rv.data(), rhs.data(), nullptr);
  K.pk.pack(u, v, x.data(), p);
  int st, it = 0;
  switch (prm->linear_solver) {
    case COVOF_LINEAR_BICGSTAB: st = solve_bicgstab(K, rhs.data(), x.data(), &it); break;
    case COVOF_LINEAR_CG: st = solve_cg(K, rhs.data(), x.data(), &it); break;
    default: st = solve_bicgstab2(K, rhs.data(), x.data(), &it); break;
  }
  if (iters) *iters = it;
  if (st == COVOF_NAN) return st;
  K.pk.unpack(x.data(), u, v, p);
  velocity_bc(prm, m, u, v, false);
  return st;
}

// ---------------------------------------------------------------------------
// Geometric VOF
struct Seg { double nx, ny, alpha; };

// src/module_interface_reconstruction.f90:283-343 reconstruct_plic
void reconstruct_plic(const Mesh& m, const double* C, Seg* s) {
  const int nx = m.nx, ny = m.ny;
  for (int j = 0; j <= ny + 1; ++j)
    for (int i = 0; i <= nx + 1; ++i) {
      size_t k = m.id(i, j);
      double c = C[k];
      if (c <= 1.0e-6) { s[k] = {1.0, 0.0, 1.0e9}; continue; }
      if (c >= 1.0 - 1.0e-6) { s[k] = {1.0, 0.0, -1.0e9}; continue; }
      double mx, my;
      if (i >= 1 && i <= nx && j >= 1 && j <= ny) {
        double cmm = C[m.id(i - 1, j - 1)], c0m = C[m.id(i, j - 1)], cpm = C[m.id(i + 1, j - 1)];
        double cm0 = C[m.id(i - 1, j)], cp0 = C[m.id(i + 1, j)];
        double cmp = C[m.id(i - 1, j + 1)], c0p = C[m.id(i, j + 1)], cpp = C[m.id(i + 1, j + 1)];
        mx = -((cpp + 2.0 * cp0 + cpm) - (cmp + 2.0 * cm0 + cmm)) / (8.0 * m.dx);
        my = -((cpp + 2.0 * c0p + cmp) - (cpm + 2.0 * c0m + cmm)) / (8.0 * m.dy);
      } else {
        mx = 1.0; my = 0.0;
      }
      double nrm = fhypot(mx, my), pnx, pny;
      if (nrm > 1.0e-12) { pnx = mx / nrm; pny = my / nrm; }
      else { pnx = 1.0; pny = 0.0; }
      double a = compute_alpha(m.x_face(i), m.x_face(i + 1), m.y_face(j), m.y_face(j + 1), pnx, pny, c);
      s[k] = {pnx, pny, a};
    }
}

// src/module_interface_reconstruction.f90:346-457 reconstruct_elvira
void reconstruct_elvira(const Mesh& m, const double* C, Seg* s) {
  const int nx = m.nx, ny = m.ny;
  const double dx = m.dx, dy = m.dy;
  for (int j = 0; j <= ny + 1; ++j)
    for (int i = 0; i <= nx + 1; ++i) {
      size_t k = m.id(i, j);
      double c = C[k];
      if (c <= 1.0e-6) { s[k] = {1.0, 0.0, 1.0e9}; continue; }
      if (c >= 1.0 - 1.0e-6) { s[k] = {1.0, 0.0, -1.0e9}; continue; }
      double xmin = m.x_face(i), xmax = m.x_face(i + 1), ymin = m.y_face(j), ymax = m.y_face(j + 1);
      if (!(i >= 1 && i <= nx && j >= 1 && j <= ny)) {
        s[k] = {1.0, 0.0, compute_alpha(xmin, xmax, ymin, ymax, 1.0, 0.0, c)};
        continue;
      }
      auto Cq = [&](int a, int b) { return C[m.id(a, b)]; };
      double Hm1 = (Cq(i - 1, j - 1) + Cq(i - 1, j) + Cq(i - 1, j + 1)) * dy;
      double H0 = (Cq(i, j - 1) + Cq(i, j) + Cq(i, j + 1)) * dy;
      double Hp1 = (Cq(i + 1, j - 1) + Cq(i + 1, j) + Cq(i + 1, j + 1)) * dy;
      double Wm1 = (Cq(i - 1, j - 1) + Cq(i, j - 1) + Cq(i + 1, j - 1)) * dx;
      double W0 = (Cq(i - 1, j) + Cq(i, j) + Cq(i + 1, j)) * dx;
      double Wp1 = (Cq(i - 1, j + 1) + Cq(i, j + 1) + Cq(i + 1, j + 1)) * dx;
      double sgy = (Cq(i, j + 1) < Cq(i, j - 1)) ? 1.0 : -1.0;
      double sgx = (Cq(i + 1, j) < Cq(i - 1, j)) ? 1.0 : -1.0;
      double cnx[7], cny[7];
      cnx[0] = -sgy * (Hp1 - Hm1) / (2.0 * dx); cny[0] = sgy * 1.0;
      cnx[1] = -sgy * (Hp1 - H0) / (dx);        cny[1] = sgy * 1.0;
      cnx[2] = -sgy * (H0 - Hm1) / (dx);        cny[2] = sgy * 1.0;
      cnx[3] = sgx * 1.0; cny[3] = -sgx * (Wp1 - Wm1) / (2.0 * dy);
      cnx[4] = sgx * 1.0; cny[4] = -sgx * (Wp1 - W0) / (dy);
      cnx[5] = sgx * 1.0; cny[5] = -sgx * (W0 - Wm1) / (dy);
      double mx = -((Cq(i + 1, j + 1) + 2.0 * Cq(i + 1, j) + Cq(i + 1, j - 1)) -
                    (Cq(i - 1, j + 1) + 2.0 * Cq(i - 1, j) + Cq(i - 1, j - 1))) / (8.0 * dx);
      double my = -((Cq(i + 1, j + 1) + 2.0 * Cq(i, j + 1) + Cq(i - 1, j + 1)) -
                    (Cq(i + 1, j - 1) + 2.0 * Cq(i, j - 1) + Cq(i - 1, j - 1))) / (8.0 * dy);
      cnx[6] = mx; cny[6] = my;
      double best_err = 1.0e30, bnx = 1.0, bny = 0.0, ba = 0.0;
      for (int q = 0; q < 7; ++q) {
        double cn = fhypot(cnx[q], cny[q]);
        if (cn < 1.0e-12) continue;
        double ux = cnx[q] / cn, uy = cny[q] / cn;
        double ca = compute_alpha(xmin, xmax, ymin, ymax, ux, uy, c);
        double err = 0.0;
        for (int dj = -1; dj <= 1; ++dj)
          for (int di = -1; di <= 1; ++di) {
            if (di == 0 && dj == 0) continue;
            double vt = Cq(i + di, j + dj) * dx * dy;
            double vr = cut_box_area(m.x_face(i + di), m.x_face(i + di + 1), m.y_face(j + dj),
                                     m.y_face(j + dj + 1), ux, uy, ca);
            double df = vr - vt;
            err = err + df * df;
          }
        if (err < best_err) { best_err = err; bnx = ux; bny = uy; ba = ca; }
      }
      s[k] = {bnx, bny, ba};
    }
}

// src/module_interface_reconstruction.f90:580-683 reconstruct_interface (np=1)
void reconstruct_interface(const covof_params* prm, const Mesh& m, const double* C, Seg* s) {
  const int nx = m.nx, ny = m.ny;
  if (prm->recon == COVOF_RECON_ELVIRA) reconstruct_elvira(m, C, s);
  else reconstruct_plic(m, C, s);
  size_t g = (size_t)(nx + 2) * (ny + 2);
  std::vector<double> snx(g, 0.0), sny(g, 0.0);
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) { snx[m.id(i, j)] = s[m.id(i, j)].nx; sny[m.id(i, j)] = s[m.id(i, j)].ny; }
  // :606-627: the normals' halo exchange (the periodic wrap), then the
  // first interior ring copied out on the non-periodic sides
  halo_scalar(prm, m, snx.data());
  halo_scalar(prm, m, sny.data());
  if (!per_x(prm))
    for (int j = 1; j <= ny; ++j) {
      snx[m.id(0, j)] = snx[m.id(1, j)]; sny[m.id(0, j)] = sny[m.id(1, j)];
      snx[m.id(nx + 1, j)] = snx[m.id(nx, j)]; sny[m.id(nx + 1, j)] = sny[m.id(nx, j)];
    }
  if (!per_y(prm))
    for (int i = 0; i <= nx + 1; ++i) {
      snx[m.id(i, 0)] = snx[m.id(i, 1)]; sny[m.id(i, 0)] = sny[m.id(i, 1)];
      snx[m.id(i, ny + 1)] = snx[m.id(i, ny)]; sny[m.id(i, ny + 1)] = sny[m.id(i, ny)];
    }
  auto ring = [&](int i, int j) {
    size_t k = m.id(i, j);
    double c = C[k];
    if (c > 1.0e-6 && c < 1.0 - 1.0e-6) {
      double a = snx[k], b = sny[k];
      double nr = fhypot(a, b);
      if (nr > 1.0e-12) {
        a = a / nr; b = b / nr;
        s[k].nx = a; s[k].ny = b;
        s[k].alpha = compute_alpha(m.x_face(i), m.x_face(i + 1), m.y_face(j), m.y_face(j + 1), a, b, c);
      }
    }
  };
  for (int j = 1; j <= ny; ++j) { ring(0, j); ring(nx + 1, j); }
  for (int i = 0; i <= nx + 1; ++i) { ring(i, 0); ring(i, ny + 1); }
}

// One direction pass of src/module_interface_vof.f90:1162-1377.
// dir 0 = x (:1203-1243), dir 1 = y (:1246-1285).  Cin -> Cout (interior),
// ghosts of Cout copied from Cin; clamp applied when requested (pass 2).
void wy_pass(const covof_params* prm, const Mesh& m, double dt, int dir, const double* u,
             const double* v, const double* cd, const double* Cin, double* Cout, bool clamp) {
  const int nx = m.nx, ny = m.ny;
  const double dx = m.dx, dy = m.dy, area = dx * dy;
  size_t g = (size_t)(nx + 2) * (ny + 2);
  std::vector<Seg> seg(g);
  reconstruct_interface(prm, m, Cin, seg.data());
  std::vector<double> flux(g, 0.0);
  if (dir == 0) {
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx + 1; ++i) {
        double uf = u[m.id(i, j)];
        double d = std::fabs(uf) * dt;
        if (d <= 1.0e-14) continue;
        double xp = m.x_face(i);
        if (uf > 0.0) {
          const Seg& s = seg[m.id(i - 1, j)];
          flux[m.id(i, j)] = cut_box_area(xp - d, xp, m.y_face(j), m.y_face(j + 1), s.nx, s.ny, s.alpha);
        } else {
          const Seg& s = seg[m.id(i, j)];
          flux[m.id(i, j)] = -cut_box_area(xp, xp + d, m.y_face(j), m.y_face(j + 1), s.nx, s.ny, s.alpha);
        }
      }
    // :1223-1231: the two images of the periodic face carry the upwind one's flux
    if (per_x(prm))
      for (int j = 1; j <= ny; ++j) {
        if (u[m.id(1, j)] >= 0.0) flux[m.id(1, j)] = flux[m.id(nx + 1, j)];
        else flux[m.id(nx + 1, j)] = flux[m.id(1, j)];
      }
    std::memcpy(Cout, Cin, g * sizeof(double));
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double c = Cin[m.id(i, j)] - (flux[m.id(i + 1, j)] - flux[m.id(i, j)]) / area +
                   cd[m.id(i, j)] * (dt / dx) * (u[m.id(i + 1, j)] - u[m.id(i, j)]);
        if (clamp) c = std::max(0.0, std::min(1.0, c));
        Cout[m.id(i, j)] = c;
      }
  } else {
    for (int j = 1; j <= ny + 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        double vf = v[m.id(i, j)];
        double d = std::fabs(vf) * dt;
        if (d <= 1.0e-14) continue;
        double yp = m.y_face(j);
        if (vf > 0.0) {
          const Seg& s = seg[m.id(i, j - 1)];
          flux[m.id(i, j)] = cut_box_area(m.x_face(i), m.x_face(i + 1), yp - d, yp, s.nx, s.ny, s.alpha);
        } else {
          const Seg& s = seg[m.id(i, j)];
          flux[m.id(i, j)] = -cut_box_area(m.x_face(i), m.x_face(i + 1), yp, yp + d, s.nx, s.ny, s.alpha);
        }
      }
    // :1268-1276
    if (per_y(prm))
      for (int i = 1; i <= nx; ++i) {
        if (v[m.id(i, 1)] >= 0.0) flux[m.id(i, 1)] = flux[m.id(i, ny + 1)];
        else flux[m.id(i, ny + 1)] = flux[m.id(i, 1)];
      }
    std::memcpy(Cout, Cin, g * sizeof(double));
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double c = Cin[m.id(i, j)] - (flux[m.id(i, j + 1)] - flux[m.id(i, j)]) / area +
                   cd[m.id(i, j)] * (dt / dy) * (v[m.id(i, j + 1)] - v[m.id(i, j)]);
        if (clamp) c = std::max(0.0, std::min(1.0, c));
        Cout[m.id(i, j)] = c;
      }
  }
}

// src/module_interface_vof.f90:1162-1377 advect_vof_weymouth_yue
// src/module_interface_vof.f90:938-1159 advect_vof_ciam: the same donor-cell
// flux volumes as Weymouth-Yue, then a Lagrangian remap of the cell width
// (denom = dh - dt (u_e - u_w)), clamped after each pass.
void ciam_pass(const covof_params* prm, const Mesh& m, double dt, int dir, const double* u,
               const double* v, const double* Cin, double* Cout) {
  const int nx = m.nx, ny = m.ny;
  const double dx = m.dx, dy = m.dy;
  size_t g = (size_t)(nx + 2) * (ny + 2);
  std::vector<Seg> seg(g);
  reconstruct_interface(prm, m, Cin, seg.data());
  std::vector<double> flux(g, 0.0);
  std::memcpy(Cout, Cin, g * sizeof(double));
  if (dir == 0) {
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx + 1; ++i) {
        double uf = u[m.id(i, j)];
        double d = std::fabs(uf) * dt;
        if (d <= 1.0e-14) continue;
        double xp = m.x_face(i);
        if (uf > 0.0) {
          const Seg& s = seg[m.id(i - 1, j)];
          flux[m.id(i, j)] = cut_box_area(xp - d, xp, m.y_face(j), m.y_face(j + 1), s.nx, s.ny, s.alpha);
        } else {
          const Seg& s = seg[m.id(i, j)];
          flux[m.id(i, j)] = -cut_box_area(xp, xp + d, m.y_face(j), m.y_face(j + 1), s.nx, s.ny, s.alpha);
        }
      }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double denom = dx - dt * (u[m.id(i + 1, j)] - u[m.id(i, j)]);
        double df = flux[m.id(i + 1, j)] - flux[m.id(i, j)];
        double c = denom > 1.0e-12 ? (Cin[m.id(i, j)] * dx - df / dy) / denom : Cin[m.id(i, j)] - df / (dx * dy);
        Cout[m.id(i, j)] = std::max(0.0, std::min(1.0, c));
      }
  } else {
    for (int j = 1; j <= ny + 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        double vf = v[m.id(i, j)];
        double d = std::fabs(vf) * dt;
        if (d <= 1.0e-14) continue;
        double yp = m.y_face(j);
        if (vf > 0.0) {
          const Seg& s = seg[m.id(i, j - 1)];
          flux[m.id(i, j)] = cut_box_area(m.x_face(i), m.x_face(i + 1), yp - d, yp, s.nx, s.ny, s.alpha);
        } else {
          const Seg& s = seg[m.id(i, j)];
          flux[m.id(i, j)] = -cut_box_area(m.x_face(i), m.x_face(i + 1), yp, yp + d, s.nx, s.ny, s.alpha);
        }
      }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double denom = dy - dt * (v[m.id(i, j + 1)] - v[m.id(i, j)]);
        double df = flux[m.id(i, j + 1)] - flux[m.id(i, j)];
        double c = denom > 1.0e-12 ? (Cin[m.id(i, j)] * dy - df / dx) / denom : Cin[m.id(i, j)] - df / (dx * dy);
        Cout[m.id(i, j)] = std::max(0.0, std::min(1.0, c));
      }
  }
}

void ciam_step(const covof_params* prm, const Mesh& m, double dt, bool x_first, const double* u,
               const double* v, double* C) {
  size_t g = (size_t)(m.nx + 2) * (m.ny + 2);
  std::vector<double> cs(g), cf(g);
  int d1 = x_first ? 0 : 1, d2 = x_first ? 1 : 0;
  ciam_pass(prm, m, dt, d1, u, v, C, cs.data());
  vof_bc(prm, m, cs.data());  // :1002-1004
  ciam_pass(prm, m, dt, d2, u, v, cs.data(), cf.data());
  std::memcpy(C, cf.data(), g * sizeof(double));
}

// src/module_interface_reconstruction.f90:686-725 evaluate_limiter
double tvd_limiter(int lim, double r, double c_donor, double c_upwind, double c_acceptor) {
  switch (lim) {
    case COVOF_LIMITER_VAN_LEER:
      return r > 0.0 ? 2.0 * r / (1.0 + r) : 0.0;
    case COVOF_LIMITER_MUSCL:
      return std::max(0.0, std::min(2.0 * r, std::min(0.5 * (1.0 + r), 2.0)));
    case COVOF_LIMITER_HRIC: {
      double denom = c_acceptor - c_upwind;
      if (std::fabs(denom) < 1.0e-12) return 0.0;
      double ctD = (c_donor - c_upwind) / denom;
      double ctf = ctD;
      if (ctD >= 0.0 && ctD <= 1.0) ctf = ctD < 0.5 ? 2.0 * ctD : 1.0;
      if (std::fabs(1.0 - ctD) > 1.0e-12) {
        double phi = 2.0 * (ctf - ctD) / (1.0 - ctD);
        return std::max(0.0, std::min(2.0, phi));
      }
      return 1.0;
    }
    default:
      return std::max(0.0, std::max(std::min(2.0 * r, 1.0), std::min(r, 2.0)));
  }
}

// src/module_interface_vof.f90:828-935 advect_vof_tvd: limited upwind face
// fluxes in both directions from C^n, one conservative update, clamp.
void tvd_step(const covof_params* prm, const Mesh& m, double dt, const double* u, const double* v,
              double* C) {
  const int nx = m.nx, ny = m.ny;
  const double dx = m.dx, dy = m.dy;
  size_t g = (size_t)(nx + 2) * (ny + 2);
  std::vector<double> fx(g, 0.0), fy(g, 0.0), cn(C, C + g);
  const int lim = prm->tvd_limiter;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx + 1; ++i) {
      double uf = u[m.id(i, j)];
      double cl = C[m.id(i - 1, j)], cr = C[m.id(i, j)];
      double cfl = 1.0 - std::min(1.0, std::fabs(uf) * dt / dx);
      if (uf >= 0.0) {
        double cu = C[m.id(std::max(0, i - 2), j)];
        double dup = cl - cu, dloc = cr - cl;
        double r = std::fabs(dloc) > 1.0e-12 ? dup / dloc : 0.0;
        double phi = tvd_limiter(lim, r, cl, cu, cr);
        fx[m.id(i, j)] = uf * (cl + 0.5 * phi * cfl * dloc);
      } else {
        double cu = C[m.id(std::min(nx + 1, i + 1), j)];
        double dup = cu - cr, dloc = cr - cl;
        double r = std::fabs(dloc) > 1.0e-12 ? dup / dloc : 0.0;
        double phi = tvd_limiter(lim, r, cr, cu, cl);
        fx[m.id(i, j)] = uf * (cr - 0.5 * phi * cfl * dloc);
      }
    }
  for (int j = 1; j <= ny + 1; ++j)
    for (int i = 1; i <= nx; ++i) {
      double vf = v[m.id(i, j)];
      double cb = C[m.id(i, j - 1)], ct = C[m.id(i, j)];
      double cfl = 1.0 - std::min(1.0, std::fabs(vf) * dt / dy);
      if (vf >= 0.0) {
        double cu = C[m.id(i, std::max(0, j - 2))];
        double dup = cb - cu, dloc = ct - cb;
        double r = std::fabs(dloc) > 1.0e-12 ? dup / dloc : 0.0;
        double phi = tvd_limiter(lim, r, cb, cu, ct);
        fy[m.id(i, j)] = vf * (cb + 0.5 * phi * cfl * dloc);
      } else {
        double cu = C[m.id(i, std::min(ny + 1, j + 1))];
        double dup = cu - ct, dloc = ct - cb;
        double r = std::fabs(dloc) > 1.0e-12 ? dup / dloc : 0.0;
        double phi = tvd_limiter(lim, r, ct, cu, cb);
        fy[m.id(i, j)] = vf * (ct - 0.5 * phi * cfl * dloc);
      }
    }
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = m.id(i, j);
      double c = C[k] - (dt / dx) * (fx[m.id(i + 1, j)] - fx[k]) - (dt / dy) * (fy[m.id(i, j + 1)] - fy[k]);
      cn[k] = std::max(0.0, std::min(1.0, c));
    }
  std::memcpy(C, cn.data(), g * sizeof(double));
}

// src/module_interface_vof.f90:801-808: the transport method of advect_vof
void vof_transport(const covof_params* prm, const Mesh& m, double dt, bool x_first, const double* u,
                   const double* v, double* C);

void wy_step(const covof_params* prm, const Mesh& m, double dt, bool x_first, const double* u,
             const double* v, double* C) {
  size_t g = (size_t)(m.nx + 2) * (m.ny + 2);
  std::vector<double> cd(g), cs(g), cf(g);
  for (size_t k = 0; k < g; ++k) cd[k] = C[k] >= 0.5 ? 1.0 : 0.0;  // :1189-1197
  int d1 = x_first ? 0 : 1, d2 = x_first ? 1 : 0;
  wy_pass(prm, m, dt, d1, u, v, cd.data(), C, cs.data(), false);
  halo_scalar(prm, m, cs.data());  // :1238-1242
  vof_bc(prm, m, cs.data());
  wy_pass(prm, m, dt, d2, u, v, cd.data(), cs.data(), cf.data(), true);
  std::memcpy(C, cf.data(), g * sizeof(double));
}

void vof_transport(const covof_params* prm, const Mesh& m, double dt, bool x_first, const double* u,
                   const double* v, double* C) {
  if (prm->advection_method == COVOF_ADVECT_CIAM) ciam_step(prm, m, dt, x_first, u, v, C);
  else if (prm->advection_method == COVOF_ADVECT_TVD) tvd_step(prm, m, dt, u, v, C);
  else wy_step(prm, m, dt, x_first, u, v, C);
}

// src/module_interface_vof.f90:387-476 smooth_svof_helmholtz: 25 symmetric
// Gauss-Seidel sweep pairs of (I - D lap) C_s = C with dC_s/dn = 0, then
// the clamp to [0, 1] and the ghost ring (corners included).
void svof_smooth(const covof_params* prm, const Mesh& m, const double* C, double* Cs) {
  const int nx = m.nx, ny = m.ny;
  const double dx = m.dx, dy = m.dy;
  double kw = prm->svof_filter_width;
  if (kw <= 0.0) kw = 1.0;
  const double D = kw * dx * dy;
  const double wx = D / (dx * dx), wy = D / (dy * dy);
  size_t g = (size_t)(nx + 2) * (ny + 2);
  for (size_t k = 0; k < g; ++k) Cs[k] = C[k];
  auto cell = [&](int i, int j) {
    double aE = (i == nx) ? 0.0 : wx;
    double aW = (i == 1) ? 0.0 : wx;
    double aN = (j == ny) ? 0.0 : wy;
    double aS = (j == 1) ? 0.0 : wy;
    double aP = 1.0 + aE + aW + aN + aS;
    double sum = aE * Cs[m.id(i + 1, j)] + aW * Cs[m.id(i - 1, j)] + aN * Cs[m.id(i, j + 1)] +
                 aS * Cs[m.id(i, j - 1)];
    Cs[m.id(i, j)] = (C[m.id(i, j)] + sum) / aP;
  };
  for (int it = 0; it < 25; ++it) {
    for (int j = 1; j <= ny; ++j) { Cs[m.id(0, j)] = Cs[m.id(1, j)]; Cs[m.id(nx + 1, j)] = Cs[m.id(nx, j)]; }
    for (int i = 1; i <= nx; ++i) { Cs[m.id(i, 0)] = Cs[m.id(i, 1)]; Cs[m.id(i, ny + 1)] = Cs[m.id(i, ny)]; }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) cell(i, j);
    for (int j = ny; j >= 1; --j)
      for (int i = nx; i >= 1; --i) cell(i, j);
  }
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) Cs[m.id(i, j)] = std::max(0.0, std::min(1.0, Cs[m.id(i, j)]));
  for (int j = 1; j <= ny; ++j) { Cs[m.id(0, j)] = Cs[m.id(1, j)]; Cs[m.id(nx + 1, j)] = Cs[m.id(nx, j)]; }
  for (int i = 1; i <= nx; ++i) { Cs[m.id(i, 0)] = Cs[m.id(i, 1)]; Cs[m.id(i, ny + 1)] = Cs[m.id(i, ny)]; }
  Cs[m.id(0, 0)] = Cs[m.id(1, 1)];
  Cs[m.id(nx + 1, 0)] = Cs[m.id(nx, 1)];
  Cs[m.id(0, ny + 1)] = Cs[m.id(1, ny)];
  Cs[m.id(nx + 1, ny + 1)] = Cs[m.id(nx, ny)];
}

// src/module_interface_vof.f90:1416-1461 vof_smooth_diffusion: explicit
// diffusion steps (dtau = 0.2 min(dx^2, dy^2)) of C into C_tilde.
void diffusion_smooth(const covof_params* prm, const Mesh& m, const double* C, double* Ct) {
  const int nx = m.nx, ny = m.ny;
  const double dx = m.dx, dy = m.dy;
  size_t g = (size_t)(nx + 2) * (ny + 2);
  for (size_t k = 0; k < g; ++k) Ct[k] = C[k];
  const double dtau = 0.2 * std::min(dx * dx, dy * dy);
  int steps = prm->diffusion_smoothing_steps;
  if (steps < 1) steps = 3;
  auto ghosts = [&]() {
    for (int j = 1; j <= ny; ++j) Ct[m.id(0, j)] = Ct[m.id(1, j)];
    for (int j = 1; j <= ny; ++j) Ct[m.id(nx + 1, j)] = Ct[m.id(nx, j)];
    for (int i = 0; i <= nx + 1; ++i) Ct[m.id(i, 0)] = Ct[m.id(i, 1)];
    for (int i = 0; i <= nx + 1; ++i) Ct[m.id(i, ny + 1)] = Ct[m.id(i, ny)];
  };
  std::vector<double> next(g);
  for (int s = 0; s < steps; ++s) {
    ghosts();
    for (size_t k = 0; k < g; ++k) next[k] = Ct[k];
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        size_t k = m.id(i, j);
        double lx = (Ct[m.id(i + 1, j)] - 2.0 * Ct[k] + Ct[m.id(i - 1, j)]) / (dx * dx);
        double ly = (Ct[m.id(i, j + 1)] - 2.0 * Ct[k] + Ct[m.id(i, j - 1)]) / (dy * dy);
        next[k] = Ct[k] + dtau * (lx + ly);
      }
    for (size_t k = 0; k < g; ++k) Ct[k] = next[k];
  }
  ghosts();
}

// src/module_interface_vof.f90:479-616 (two-phase, incompressible; with
// SVOF the cell properties and mu_node come from C_s, :541-545, 596-601)
void update_props(const covof_params* prm, const Mesh& m, double* C, double* rho, double* rho_u,
                  double* rho_v, double* mu, double* mu_node, const double* Cs) {
  const int nx = m.nx, ny = m.ny;
  size_t g = (size_t)(nx + 2) * (ny + 2);
  if (!prm->enable_two_phase) {
    for (size_t k = 0; k < g; ++k) {
      rho[k] = prm->rho1; rho_u[k] = prm->rho1; rho_v[k] = prm->rho1;
      mu[k] = prm->mu1; mu_node[k] = prm->mu1;
    }
    return;
  }
  // physical corners only (:532-535): a periodic side has no boundary
  if (!per_x(prm) && !per_y(prm)) {
    C[m.id(0, 0)] = C[m.id(1, 1)];
    C[m.id(nx + 1, 0)] = C[m.id(nx, 1)];
    C[m.id(0, ny + 1)] = C[m.id(1, ny)];
    C[m.id(nx + 1, ny + 1)] = C[m.id(nx, ny)];
  }
  const bool svof = prm->enable_svof_smoothing && Cs;
  for (int j = 0; j <= ny + 1; ++j)
    for (int i = 0; i <= nx + 1; ++i) {
      size_t k = m.id(i, j);
      double c = std::max(0.0, std::min(1.0, svof ? Cs[k] : C[k]));
      rho[k] = c * prm->rho1 + (1.0 - c) * prm->rho2;
      mu[k] = c * prm->mu1 + (1.0 - c) * prm->mu2;
    }
  mu[m.id(0, 0)] = mu[m.id(1, 1)];
  mu[m.id(nx + 1, 0)] = mu[m.id(nx, 1)];
  mu[m.id(0, ny + 1)] = mu[m.id(1, ny)];
  mu[m.id(nx + 1, ny + 1)] = mu[m.id(nx, ny)];
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx + 1; ++i)
      rho_u[m.id(i, j)] = 0.5 * (rho[m.id(i - 1, j)] + rho[m.id(i, j)]);
  for (int j = 1; j <= ny + 1; ++j)
    for (int i = 1; i <= nx; ++i)
      rho_v[m.id(i, j)] = 0.5 * (rho[m.id(i, j - 1)] + rho[m.id(i, j)]);
  for (int j = 1; j <= ny + 1; ++j)
    for (int i = 1; i <= nx + 1; ++i) {
      if (svof) {
        double cn = 0.25 * (Cs[m.id(i - 1, j - 1)] + Cs[m.id(i, j - 1)] + Cs[m.id(i - 1, j)] + Cs[m.id(i, j)]);
        cn = std::max(0.0, std::min(1.0, cn));
        double denom = prm->mu2 * cn + prm->mu1 * (1.0 - cn);
        mu_node[m.id(i, j)] = (prm->mu1 * prm->mu2) / std::max(1.0e-30, denom);
      } else {
        double sw = mu[m.id(i - 1, j - 1)], se = mu[m.id(i, j - 1)];
        double nw = mu[m.id(i - 1, j)], ne = mu[m.id(i, j)];
        mu_node[m.id(i, j)] = 4.0 / (1.0 / sw + 1.0 / se + 1.0 / nw + 1.0 / ne);
      }
    }
}

// src/module_interface_vof.f90:627-789 (no markers): the normals come from
// C_tilde (diffusion smoothing), else C_s (SVOF), else C (:682-690); the
// face gradient from C.
void csf(const covof_params* prm, const Mesh& m, const double* C, double* fx, double* fy,
         double* curv, const double* Cs, const double* Ct) {
  const int nx = m.nx, ny = m.ny;
  const double dx = m.dx, dy = m.dy;
  size_t g = (size_t)(nx + 2) * (ny + 2);
  if (!prm->enable_surface_tension || prm->sigma <= 0.0) {
    for (size_t k = 0; k < g; ++k) { fx[k] = 0.0; fy[k] = 0.0; curv[k] = 0.0; }
    return;
  }
  std::vector<double> nxv(g, 0.0), nyv(g, 0.0), kap(g, 0.0);
  const double* N = (prm->enable_diffusion_smoothing && Ct) ? Ct : (prm->enable_svof_smoothing && Cs) ? Cs : C;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      double dcx = (N[m.id(i + 1, j)] - N[m.id(i - 1, j)]) / (2.0 * dx);
      double dcy = (N[m.id(i, j + 1)] - N[m.id(i, j - 1)]) / (2.0 * dy);
      double gm = std::sqrt(dcx * dcx + dcy * dcy);
      if (gm > 1.0e-3 / dx) { nxv[m.id(i, j)] = dcx / gm; nyv[m.id(i, j)] = dcy / gm; }
    }
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = m.id(i, j);
      if (nxv[k] != 0.0 || nyv[k] != 0.0)
        kap[k] = -((nxv[m.id(i + 1, j)] - nxv[m.id(i - 1, j)]) / (2.0 * dx) +
                   (nyv[m.id(i, j + 1)] - nyv[m.id(i, j - 1)]) / (2.0 * dy));
    }
  for (size_t k = 0; k < g; ++k) curv[k] = kap[k];
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx + 1; ++i) {
      double ka = 0.5 * (kap[m.id(i - 1, j)] + kap[m.id(i, j)]);
      double gc = (C[m.id(i, j)] - C[m.id(i - 1, j)]) / dx;
      fx[m.id(i, j)] = prm->sigma * ka * gc;
    }
  for (int j = 1; j <= ny + 1; ++j)
    for (int i = 1; i <= nx; ++i) {
      double ka = 0.5 * (kap[m.id(i, j - 1)] + kap[m.id(i, j)]);
      double gc = (C[m.id(i, j)] - C[m.id(i, j - 1)]) / dy;
      fy[m.id(i, j)] = prm->sigma * ka * gc;
    }
}

}  // namespace

// ===========================================================================
extern "C" {

double orc_hypot(double x, double y) { return fhypot(x, y); }
double orc_cut_box_area(double a, double b, double c, double d, double nx, double ny, double al) {
  return cut_box_area(a, b, c, d, nx, ny, al);
}
double orc_compute_alpha(double a, double b, double c, double d, double nx, double ny, double ct) {
  return compute_alpha(a, b, c, d, nx, ny, ct);
}

int orc_apply_velocity_bc(const covof_params* prm, double* u, double* v, int homogeneous) {
  int st = check_params(prm, true, true);
  if (st) return st;
  velocity_bc(prm, mesh_of(prm), u, v, homogeneous != 0);
  return COVOF_OK;
}
int orc_apply_vof_bc(const covof_params* prm, double* C) {
  int st = check_params(prm, true, true);
  if (st) return st;
  vof_bc(prm, mesh_of(prm), C);
  return COVOF_OK;
}

int orc_poisson_assemble(const covof_params* prm, double dt, const double* u_star,
                         const double* v_star, const double* rho_u, const double* rho_v,
                         double* aW, double* aE, double* aS, double* aN, double* aP, double* b) {
  int st = check_params(prm, true, true);
  if (st) return st;
  Mesh m = mesh_of(prm);
  Poisson P;
  poisson_assemble(prm, m, dt, rho_u, rho_v, P);
  poisson_rhs_from_velocity(m, u_star, v_star, P);
  size_t n = (size_t)m.nx * m.ny;
  std::memcpy(aW, P.aW.data(), n * 8); std::memcpy(aE, P.aE.data(), n * 8);
  std::memcpy(aS, P.aS.data(), n * 8); std::memcpy(aN, P.aN.data(), n * 8);
  std::memcpy(aP, P.aP.data(), n * 8); std::memcpy(b, P.b.data(), n * 8);
  return COVOF_OK;
}

int orc_poisson_matvec(const covof_params* prm, double dt, const double* rho_u,
                       const double* rho_v, const double* x, double* y) {
  int st = check_params(prm, true, true);
  if (st) return st;
  Mesh m = mesh_of(prm);
  Poisson P;
  poisson_assemble(prm, m, dt, rho_u, rho_v, P);
  std::vector<double> xi((size_t)m.nx * m.ny), yi(xi.size());
  for (int j = 1; j <= m.ny; ++j) for (int i = 1; i <= m.nx; ++i) xi[P.k(i, j)] = x[m.id(i, j)];
  poisson_matvec(P, xi.data(), yi.data());
  for (int j = 1; j <= m.ny; ++j) for (int i = 1; i <= m.nx; ++i) y[m.id(i, j)] = yi[P.k(i, j)];
  return COVOF_OK;
}

int orc_poisson_solve(const covof_params* prm, double dt, const double* u_star,
                      const double* v_star, const double* rho_u, const double* rho_v, double* p,
                      int* iters, double* relres, int nthreads) {
  int st = check_params(prm, true, true);
  if (st) return st;
  return poisson_driver(prm, dt, u_star, v_star, nullptr, rho_u, rho_v, p, iters, relres, nthreads, 0);
}

int orc_poisson_solve_rhs(const covof_params* prm, double dt, const double* b,
                          const double* rho_u, const double* rho_v, double* p, int* iters,
                          double* relres, int nthreads) {
  int st = check_params(prm, true, true);
  if (st) return st;
  return poisson_driver(prm, dt, nullptr, nullptr, b, rho_u, rho_v, p, iters, relres, nthreads, 0);
}

int orc_poisson_fixed_iters(const covof_params* prm, double dt, const double* b,
                            const double* rho_u, const double* rho_v, double* p, int n_iter,
                            int nthreads, double* relres) {
  int st = check_params(prm, true, true);
  if (st) return st;
  if (n_iter < 1) return COVOF_INVALID;
  int it = 0;
  return poisson_driver(prm, dt, nullptr, nullptr, b, rho_u, rho_v, p, &it, relres, nthreads, n_iter);
}

int orc_project_correct(const covof_params* prm, double dt, double* u, double* v, const double* p,
                        const double* rho_u, const double* rho_v) {
  int st = check_params(prm, true, true);
  if (st) return st;
  project_correct(prm, mesh_of(prm), dt, u, v, p, rho_u, rho_v);
  return COVOF_OK;
}

Hist hist_of(const double* u_old, const double* v_old, const double* u_nm1, const double* v_nm1,
             int has_nm1) {
  Hist h;
  h.u_old = u_old; h.v_old = v_old; h.u_nm1 = u_nm1; h.v_nm1 = v_nm1;
  h.has_nm1 = (has_nm1 && u_nm1 && v_nm1) ? 1 : 0;
  return h;
}

int check_mom(const covof_params* prm, const double* u_old, const double* u_nm1, int has_nm1) {
  if (prm->time_scheme != 0 && prm->time_scheme != COVOF_TIME_EULER && prm->time_scheme != COVOF_TIME_GEAR)
    return COVOF_UNSUPPORTED;
  if (prm->convective_linearization != 0 && prm->convective_linearization != COVOF_CONV_LIN_PICARD &&
      prm->convective_linearization != COVOF_CONV_LIN_AB2)
    return COVOF_UNSUPPORTED;
  if (prm->convective_scheme != COVOF_CONV_UPWIND && prm->convective_scheme != COVOF_CONV_CENTERED &&
      prm->convective_scheme != COVOF_CONV_TVD_SUPERBEE)
    return COVOF_UNSUPPORTED;
  if (prm->convective_linearization == COVOF_CONV_LIN_AB2 && !u_old) return COVOF_INVALID;
  if (has_nm1 && !u_nm1 && (prm->time_scheme == COVOF_TIME_GEAR ||
                            prm->convective_linearization == COVOF_CONV_LIN_AB2))
    return COVOF_INVALID;
  return COVOF_OK;
}

int orc_momentum_apply(const covof_params* prm, double dt, const double* xu, const double* xv,
                       double* yu, double* yv, const double* u_n, const double* v_n,
                       const double* rho_u, const double* rho_v, const double* mu,
                       const double* mu_node, const double* u_old, const double* v_old,
                       const double* u_nm1, const double* v_nm1, int has_nm1) {
  int st = check_params(prm, false);
  if (st) return st;
  if ((st = check_mom(prm, u_old, u_nm1, has_nm1))) return st;
  MomCtx c = make_ctx(prm, dt, u_n, v_n, rho_u, rho_v, mu, mu_node, hist_of(u_old, v_old, u_nm1, v_nm1, has_nm1));
  size_t g = (size_t)(prm->nx + 2) * (prm->ny + 2);
  // tf is a fresh field set: ghosts start at zero, then the DOFs are copied
  // in and the homogeneous ghost conditions applied.
  std::vector<double> tu(g, 0.0), tv(g, 0.0);
  Packer pk{c};
  std::vector<double> x(pk.n());
  pk.pack(xu, xv, x.data());
  pk.unpack(x.data(), tu.data(), tv.data());
  velocity_bc(prm, c.m, tu.data(), tv.data(), true);
  mom_apply(c, tu.data(), tv.data(), yu, yv);
  return COVOF_OK;
}

// The MONOLITHIC operator (:380-780 with the pressure DOFs): momentum rows
// with B^T p, continuity rows; the operand's pressure ghosts are zero.
int orc_mono_apply(const covof_params* prm, double dt, const double* xu, const double* xv, const double* xp,
                   double* yu, double* yv, double* yp, const double* u_n, const double* v_n,
                   const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                   const double* u_old, const double* v_old, const double* u_nm1, const double* v_nm1,
                   int has_nm1) {
  int st = check_params(prm, false);
  if (st) return st;
  if ((st = check_mom(prm, u_old, u_nm1, has_nm1))) return st;
  MomCtx c = make_ctx(prm, dt, u_n, v_n, rho_u, rho_v, mu, mu_node, hist_of(u_old, v_old, u_nm1, v_nm1, has_nm1));
  c.mono = true;
  c.np = (size_t)prm->nx * prm->ny;
  size_t g = (size_t)(prm->nx + 2) * (prm->ny + 2);
  std::vector<double> tu(g, 0.0), tv(g, 0.0), tp(g, 0.0);
  Packer pk{c};
  std::vector<double> x(pk.n());
  pk.pack(xu, xv, x.data(), xp);
  pk.unpack(x.data(), tu.data(), tv.data(), tp.data());
  velocity_bc(prm, c.m, tu.data(), tv.data(), true);
  mom_apply(c, tu.data(), tv.data(), yu, yv, tp.data(), yp);
  return COVOF_OK;
}

// diag_p (the Schur diagonal) from the momentum diagonals du, dv
int orc_schur_diag(const covof_params* prm, double dt, const double* du, const double* dv, double* dp) {
  int st = check_params(prm, false);
  if (st) return st;
  MomCtx c = make_ctx(prm, dt, du, dv, du, dv, du, du);
  schur_diag(c, du, dv, dp);
  return COVOF_OK;
}

// The Krylov preconditioner M^-1 of the configured precond (JACOBI / ILU0 /
// SSOR / BLOCK_TRIANGULAR, or none) on (zu, zv[, zp]) -> (yu, yv[, yp]),
// assembled from the fields as the solve would (r_al: the AL penalty field
// for AUGMENTED_LAGRANGIAN / AAL, else nullptr).
int orc_precond_apply(const covof_params* prm, double dt, const double* zu, const double* zv, const double* zp,
                      double* yu, double* yv, double* yp, const double* u_n, const double* v_n,
                      const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                      const double* u_old, const double* v_old, const double* u_nm1, const double* v_nm1,
                      int has_nm1, const double* r_al) {
  int st = check_params(prm, false);
  if (st) return st;
  if ((st = check_mom(prm, u_old, u_nm1, has_nm1))) return st;
  MomCtx c = make_ctx(prm, dt, u_n, v_n, rho_u, rho_v, mu, mu_node, hist_of(u_old, v_old, u_nm1, v_nm1, has_nm1));
  const bool al = prm->solver_type == COVOF_SOLVER_AUGMENTED_LAGRANGIAN || prm->solver_type == COVOF_SOLVER_AAL;
  if (al) c.r_al = r_al;
  c.mono = prm->solver_type == COVOF_SOLVER_MONOLITHIC;
  c.np = c.mono ? (size_t)prm->nx * prm->ny : 0;
  const size_t g = (size_t)(prm->nx + 2) * (prm->ny + 2);
  Krylov K(c);
  std::vector<double> du(g, 1.0), dv(g, 1.0), dp(g, 1.0);
  mom_diag(c, du.data(), dv.data());
  if (c.mono) schur_diag(c, du.data(), dv.data(), dp.data());
  K.diag.resize(K.pk.n());
  K.pk.pack(du.data(), dv.data(), K.diag.data(), dp.data());
  if (uses_sweeps(prm)) prec_blocks(c, K.blk);
  std::vector<double> z(K.pk.n()), y(K.pk.n());
  K.pk.pack(zu, zv, z.data(), zp);
  K.M(z.data(), y.data());
  K.pk.unpack(y.data(), yu, yv, yp);
  return COVOF_OK;
}

// The sweep preconditioners' stencils: out holds 15 arrays of (nx+2)*(ny+2)
// doubles, u W E S N P, v W E S N P, Schur W E S N P (the Schur ones for
// MONOLITHIC only, else W..N zero and P one).
int orc_prec_blocks(const covof_params* prm, double dt, const double* u_n, const double* v_n,
                    const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                    const double* u_old, const double* v_old, const double* u_nm1, const double* v_nm1,
                    int has_nm1, const double* r_al, double* out) {
  int st = check_params(prm, false);
  if (st) return st;
  if ((st = check_mom(prm, u_old, u_nm1, has_nm1))) return st;
  MomCtx c = make_ctx(prm, dt, u_n, v_n, rho_u, rho_v, mu, mu_node, hist_of(u_old, v_old, u_nm1, v_nm1, has_nm1));
  const bool al = prm->solver_type == COVOF_SOLVER_AUGMENTED_LAGRANGIAN || prm->solver_type == COVOF_SOLVER_AAL;
  if (al) c.r_al = r_al;
  c.mono = prm->solver_type == COVOF_SOLVER_MONOLITHIC;
  PBlocks Q;
  prec_blocks(c, Q);
  const size_t g = (size_t)(prm->nx + 2) * (prm->ny + 2);
  const std::vector<double>* arr[15] = {&Q.uW, &Q.uE, &Q.uS, &Q.uN, &Q.uP, &Q.vW, &Q.vE, &Q.vS, &Q.vN, &Q.vP,
                                        &Q.sW, &Q.sE, &Q.sS, &Q.sN, &Q.sP};
  for (int q = 0; q < 15; ++q) std::memcpy(out + q * g, arr[q]->data(), g * sizeof(double));
  return COVOF_OK;
}

int orc_momentum_diag(const covof_params* prm, double dt, const double* u_n, const double* v_n,
                      const double* rho_u, const double* rho_v, const double* mu,
                      const double* mu_node, double* diag_u, double* diag_v, const double* u_old,
                      const double* v_old, const double* u_nm1, const double* v_nm1, int has_nm1) {
  int st = check_params(prm, false);
  if (st) return st;
  if ((st = check_mom(prm, u_old, u_nm1, has_nm1))) return st;
  MomCtx c = make_ctx(prm, dt, u_n, v_n, rho_u, rho_v, mu, mu_node, hist_of(u_old, v_old, u_nm1, v_nm1, has_nm1));
  mom_diag(c, diag_u, diag_v);
  return COVOF_OK;
}

int orc_momentum_rhs(const covof_params* prm, double dt, const double* u_n, const double* v_n,
                     const double* rho_u, const double* rho_v, const double* mu_node,
                     const double* fx_sigma, const double* fy_sigma, const double* u_old,
                     const double* v_old, double* rhs_u, double* rhs_v, const double* u_nm1,
                     const double* v_nm1, int has_nm1) {
  int st = check_params(prm, false);
  if (st) return st;
  if ((st = check_mom(prm, u_old, u_nm1, has_nm1))) return st;
  MomCtx c = make_ctx(prm, dt, u_n, v_n, rho_u, rho_v, nullptr, mu_node, hist_of(u_old, v_old, u_nm1, v_nm1, has_nm1));
  mom_rhs(c, mu_node, fx_sigma, fy_sigma, u_old, v_old, rhs_u, rhs_v);
  return COVOF_OK;
}

int orc_predictor(const covof_params* prm, double dt, double* u, double* v, const double* rho_u,
                  const double* rho_v, const double* mu, const double* mu_node,
                  const double* fx_sigma, const double* fy_sigma, const double* u_old,
                  const double* v_old, const double* u_nm1, const double* v_nm1, int has_nm1,
                  int* iters) {
  int st = check_params(prm, false);
  if (st) return st;
  if ((st = check_mom(prm, u_old, u_nm1, has_nm1))) return st;
  int it = 0;
  st = predictor(prm, dt, u, v, rho_u, rho_v, mu, mu_node, fx_sigma, fy_sigma, u_old, v_old,
                 hist_of(u_old, v_old, u_nm1, v_nm1, has_nm1), &it);
  if (iters) *iters = it;
  return st;
}

// one augmented-Lagrangian step (solver_type AUGMENTED_LAGRANGIAN / AAL)
int orc_al_step(const covof_params* prm, double dt, double* u, double* v, double* p, const double* rho,
                const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                const double* fx_sigma, const double* fy_sigma, const double* u_old, const double* v_old,
                const double* u_nm1, const double* v_nm1, int has_nm1, int* iters, int* uzawa_done) {
  int st = check_params(prm, false);
  if (st) return st;
  if ((st = check_mom(prm, u_old, u_nm1, has_nm1))) return st;
  if (prm->solver_type != COVOF_SOLVER_AUGMENTED_LAGRANGIAN && prm->solver_type != COVOF_SOLVER_AAL)
    return COVOF_INVALID;
  return al_step(prm, dt, u, v, p, rho, rho_u, rho_v, mu, mu_node, fx_sigma, fy_sigma,
                 hist_of(u_old, v_old, u_nm1, v_nm1, has_nm1), iters, uzawa_done);
}

int orc_mono_step(const covof_params* prm, double dt, double* u, double* v, double* p, const double* rho_u,
                  const double* rho_v, const double* mu, const double* mu_node, const double* fx_sigma,
                  const double* fy_sigma, const double* u_old, const double* v_old, const double* u_nm1,
                  const double* v_nm1, int has_nm1, int* iters) {
  int st = check_params(prm, false);
  if (st) return st;
  if ((st = check_mom(prm, u_old, u_nm1, has_nm1))) return st;
  if (prm->solver_type != COVOF_SOLVER_MONOLITHIC) return COVOF_INVALID;
  return mono_step(prm, dt, u, v, p, rho_u, rho_v, mu, mu_node, fx_sigma, fy_sigma,
                   hist_of(u_old, v_old, u_nm1, v_nm1, has_nm1), iters);
}

// Host threads of the Poisson solve inside orc_sp_step (and so of the time
// loop): 1 by default, the reference's serial per-rank loop.
static int g_step_threads = 1;
int orc_set_step_threads(int n) {
  if (n < 1) return COVOF_INVALID;
  g_step_threads = n;
  return COVOF_OK;
}

// src/module_simulation.f90:2424-2666 sim_solve_standard_projection
int orc_sp_step(const covof_params* prm, double dt, double* u, double* v, double* p,
                const double* rho_u, const double* rho_v, const double* mu,
                const double* mu_node, const double* fx_sigma, const double* fy_sigma,
                const double* u_old, const double* v_old, const double* u_nm1, const double* v_nm1,
                int has_nm1, int* iters_u, int* iters_p, double* relres) {
  int st = check_params(prm, false);
  if (st) return st;
  if ((st = check_mom(prm, u_old, u_nm1, has_nm1))) return st;
  int iu = 0, ip = 0;
  int s1 = predictor(prm, dt, u, v, rho_u, rho_v, mu, mu_node, fx_sigma, fy_sigma, u_old, v_old,
                     hist_of(u_old, v_old, u_nm1, v_nm1, has_nm1), &iu);
  if (s1 == COVOF_NAN) return s1;
  int s2 = poisson_driver(prm, dt, u, v, nullptr, rho_u, rho_v, p, &ip, relres, g_step_threads, 0);
  Mesh m = mesh_of(prm);
  project_correct(prm, m, dt, u, v, p, rho_u, rho_v);
  velocity_bc(prm, m, u, v, false);
  if (iters_u) *iters_u = iu;
  if (iters_p) *iters_p = ip;
  return s2 != COVOF_OK ? s2 : s1;
}

int orc_reconstruct(const covof_params* prm, const double* C, double* seg) {
  int st = check_params(prm, true, true);
  if (st) return st;
  Mesh m = mesh_of(prm);
  size_t g = (size_t)(m.nx + 2) * (m.ny + 2);
  std::vector<Seg> s(g);
  reconstruct_interface(prm, m, C, s.data());
  for (size_t k = 0; k < g; ++k) { seg[3 * k] = s[k].nx; seg[3 * k + 1] = s[k].ny; seg[3 * k + 2] = s[k].alpha; }
  return COVOF_OK;
}

int orc_wy_step(const covof_params* prm, double dt, int x_first, const double* u, const double* v,
                double* C) {
  int st = check_params(prm, true, true);
  if (st) return st;
  if ((st = check_periodic_vof(prm))) return st;
  wy_step(prm, mesh_of(prm), dt, x_first != 0, u, v, C);
  return COVOF_OK;
}

// the configured transport alone (Weymouth-Yue, CIAM or TVD)
int orc_vof_transport(const covof_params* prm, double dt, int x_first, const double* u,
                      const double* v, double* C) {
  int st = check_params(prm, true, true);
  if (st) return st;
  if ((st = check_periodic_vof(prm))) return st;
  if (prm->advection_method < 0 || prm->advection_method > COVOF_ADVECT_TVD) return COVOF_INVALID;
  vof_transport(prm, mesh_of(prm), dt, x_first != 0, u, v, C);
  return COVOF_OK;
}

int orc_svof_smooth(const covof_params* prm, const double* C, double* C_s) {
  int st = check_params(prm, true);
  if (st) return st;
  svof_smooth(prm, mesh_of(prm), C, C_s);
  return COVOF_OK;
}

int orc_diffusion_smooth(const covof_params* prm, const double* C, double* C_tilde) {
  int st = check_params(prm, true);
  if (st) return st;
  diffusion_smooth(prm, mesh_of(prm), C, C_tilde);
  return COVOF_OK;
}

int orc_update_physical_properties(const covof_params* prm, double* C, double* rho,
                                   double* rho_u, double* rho_v, double* mu, double* mu_node,
                                   const double* C_s) {
  int st = check_params(prm, true, true);
  if (st) return st;
  update_props(prm, mesh_of(prm), C, rho, rho_u, rho_v, mu, mu_node, C_s);
  return COVOF_OK;
}

int orc_compute_curvature_and_csf(const covof_params* prm, const double* C, double* fx_sigma,
                                  double* fy_sigma, double* curvature, const double* C_s,
                                  const double* C_tilde) {
  int st = check_params(prm, true, true);
  if (st) return st;
  csf(prm, mesh_of(prm), C, fx_sigma, fy_sigma, curvature, C_s, C_tilde);
  return COVOF_OK;
}

// src/module_interface_vof.f90:792-825 advect_vof (WEYMOUTH_YUE branch):
// transport, VOF BC, SVOF, properties, diffusion smoothing, curvature + CSF
int orc_vof_advect(const covof_params* prm, double dt, int step_count, const double* u,
                   const double* v, double* C, double* rho, double* rho_u, double* rho_v,
                   double* mu, double* mu_node, double* fx_sigma, double* fy_sigma,
                   double* curvature, double* C_s, double* C_tilde) {
  int st = check_params(prm, true, true);
  if (st) return st;
  if ((st = check_periodic_vof(prm))) return st;
  Mesh m = mesh_of(prm);
  vof_transport(prm, m, dt, (step_count % 2) == 0, u, v, C);
  halo_scalar(prm, m, C);  // src/module_interface_vof.f90:809-810
  vof_bc(prm, m, C);
  if (prm->enable_svof_smoothing && C_s) svof_smooth(prm, m, C, C_s);
  update_props(prm, m, C, rho, rho_u, rho_v, mu, mu_node, C_s);
  if (prm->enable_diffusion_smoothing && C_tilde) diffusion_smooth(prm, m, C, C_tilde);
  csf(prm, m, C, fx_sigma, fy_sigma, curvature, C_s, C_tilde);
  return COVOF_OK;
}

}  // extern "C"
