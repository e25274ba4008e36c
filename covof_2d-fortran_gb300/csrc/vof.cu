// vof.cu -- geometric VOF step on one GB300: PLIC / ELVIRA reconstruction,
// Weymouth-Yue direction passes, VOF ghost conditions, physical properties
// and CSF surface-tension forces.
//
// Every floating-point expression is evaluated in the order of the reference
// Fortran (left to right, parentheses respected) and this translation unit is
// compiled with -fmad=false, so no multiply-add is contracted.  The VOF
// results are therefore bit-identical to a serial FP64 evaluation; the only
// libm call (hypot) is replaced by the fused hypot in common.cuh.
//
// One thread per cell.  Pure cells (C <= 1e-6 or >= 1-1e-6) short-circuit,
// so the cost concentrates on interface cells: ELVIRA runs 7 candidates x
// (45 bisection steps + 8 neighbour clips) = 371 polygon clips per mixed
// cell and pass.
#include "common.cuh"
#include "vof.cuh"

namespace covof {

struct VMesh {
  Dims D;
  double dx, dy;
  // src/module_mesh.f90:177-206 (single domain, i_start_global = 1)
  __device__ __forceinline__ double xf(int i) const { return (double)(i - 1) * dx; }
  __device__ __forceinline__ double yf(int j) const { return (double)(j - 1) * dy; }
};

// src/module_interface_reconstruction.f90:33-101 cut_box_area.
// Sutherland-Hodgman clip of the box by {nx*x + ny*y + alpha <= 0}, then the
// shoelace area.  The shoelace terms are accumulated as the clipped vertices
// are emitted -- (1,2), (2,3), ..., (n-1,n), then (n,1) -- which is the
// reference's summation order, so no vertex list is stored.
struct Shoelace {
  double x0, y0, px, py, s;
  int n;
  __device__ __forceinline__ void emit(double x, double y) {
    if (n == 0) { x0 = x; y0 = y; }
    else s = s + (px * y - x * py);
    px = x; py = y; ++n;
  }
};

__device__ double cut_box_area(double xmin, double xmax, double ymin, double ymax, double nx,
                               double ny, double alpha) {
  if ((xmax - xmin) <= 1.0e-14 || (ymax - ymin) <= 1.0e-14) return 0.0;
  const double bx[4] = {xmin, xmax, xmax, xmin};
  const double by[4] = {ymin, ymin, ymax, ymax};
  double d[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) d[q] = nx * bx[q] + ny * by[q] + alpha;
  Shoelace sl{0.0, 0.0, 0.0, 0.0, 0.0, 0};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int nq = (q + 1) & 3;
    const double d1 = d[q], d2 = d[nq];
    if (d1 <= 0.0) {
      if (d2 <= 0.0) {
        sl.emit(bx[nq], by[nq]);
      } else {
        const double t = -d1 / (d2 - d1);
        sl.emit(bx[q] + t * (bx[nq] - bx[q]), by[q] + t * (by[nq] - by[q]));
      }
    } else if (d2 <= 0.0) {
      const double t = -d1 / (d2 - d1);
      sl.emit(bx[q] + t * (bx[nq] - bx[q]), by[q] + t * (by[nq] - by[q]));
      sl.emit(bx[nq], by[nq]);
    }
  }
  if (sl.n < 3) return 0.0;
  const double s = sl.s + (sl.px * sl.y0 - sl.x0 * sl.py);
  return 0.5 * fabs(s);
}

// src/module_interface_reconstruction.f90:105-147 compute_alpha
__device__ double compute_alpha(double xmin, double xmax, double ymin, double ymax, double nx,
                                double ny, double c_target) {
  const double total = (xmax - xmin) * (ymax - ymin);
  if (c_target <= 1.0e-7) return 1.0e9;
  if (c_target >= 1.0 - 1.0e-7) return -1.0e9;
  const double target = fmax(0.0, fmin(1.0, c_target)) * total;
  const double v1 = nx * xmin + ny * ymin;
  const double v2 = nx * xmax + ny * ymin;
  const double v3 = nx * xmax + ny * ymax;
  const double v4 = nx * xmin + ny * ymax;
  const double mn = fmin(v1, fmin(v2, fmin(v3, v4)));
  const double mx = fmax(v1, fmax(v2, fmax(v3, v4)));
  double lo = -mx - 1.0e-12;
  double hi = -mn + 1.0e-12;
  for (int it = 0; it < 45; ++it) {
    const double mid = 0.5 * (lo + hi);
    const double a = cut_box_area(xmin, xmax, ymin, ymax, nx, ny, mid);
    if (a < target) hi = mid; else lo = mid;
  }
  return 0.5 * (lo + hi);
}

__device__ __forceinline__ void put_seg(double* seg, int k, double a, double b, double c) {
  seg[3 * k] = a; seg[3 * k + 1] = b; seg[3 * k + 2] = c;
}

// src/module_interface_reconstruction.f90:283-343 (PLIC) and :346-457 (ELVIRA),
// every cell of (0:nx+1, 0:ny+1).
__global__ void k_vof_reconstruct(VofArgs a) {
  const VMesh m{a.D, a.dx, a.dy};
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.D.nx, ny = a.D.ny;
  if (i > nx + 1 || j > ny + 1) return;
  const double* __restrict__ C = a.C;
  const int k = a.D.id(i, j);
  const double c = C[k];
  if (c <= 1.0e-6) { put_seg(a.seg, k, 1.0, 0.0, 1.0e9); return; }
  if (c >= 1.0 - 1.0e-6) { put_seg(a.seg, k, 1.0, 0.0, -1.0e9); return; }
  const double xmin = m.xf(i), xmax = m.xf(i + 1), ymin = m.yf(j), ymax = m.yf(j + 1);
  const bool inner = (i >= 1 && i <= nx && j >= 1 && j <= ny);
  const double dx = a.dx, dy = a.dy;
  auto Cq = [&](int p, int q) { return C[a.D.id(p, q)]; };
  if (a.method != COVOF_RECON_ELVIRA) {
    double mxv, myv;
    if (inner) {
      const double cmm = Cq(i - 1, j - 1), c0m = Cq(i, j - 1), cpm = Cq(i + 1, j - 1);
      const double cm0 = Cq(i - 1, j), cp0 = Cq(i + 1, j);
      const double cmp = Cq(i - 1, j + 1), c0p = Cq(i, j + 1), cpp = Cq(i + 1, j + 1);
      mxv = -((cpp + 2.0 * cp0 + cpm) - (cmp + 2.0 * cm0 + cmm)) / (8.0 * dx);
      myv = -((cpp + 2.0 * c0p + cmp) - (cpm + 2.0 * c0m + cmm)) / (8.0 * dy);
    } else {
      mxv = 1.0; myv = 0.0;
    }
    const double nrm = fhypot(mxv, myv);
    double pnx, pny;
    if (nrm > 1.0e-12) { pnx = mxv / nrm; pny = myv / nrm; }
    else { pnx = 1.0; pny = 0.0; }
    put_seg(a.seg, k, pnx, pny, compute_alpha(xmin, xmax, ymin, ymax, pnx, pny, c));
    return;
  }
  if (!inner) {
    put_seg(a.seg, k, 1.0, 0.0, compute_alpha(xmin, xmax, ymin, ymax, 1.0, 0.0, c));
    return;
  }
  const double Hm1 = (Cq(i - 1, j - 1) + Cq(i - 1, j) + Cq(i - 1, j + 1)) * dy;
  const double H0 = (Cq(i, j - 1) + Cq(i, j) + Cq(i, j + 1)) * dy;
  const double Hp1 = (Cq(i + 1, j - 1) + Cq(i + 1, j) + Cq(i + 1, j + 1)) * dy;
  const double Wm1 = (Cq(i - 1, j - 1) + Cq(i, j - 1) + Cq(i + 1, j - 1)) * dx;
  const double W0 = (Cq(i - 1, j) + Cq(i, j) + Cq(i + 1, j)) * dx;
  const double Wp1 = (Cq(i - 1, j + 1) + Cq(i, j + 1) + Cq(i + 1, j + 1)) * dx;
  const double sgy = (Cq(i, j + 1) < Cq(i, j - 1)) ? 1.0 : -1.0;
  const double sgx = (Cq(i + 1, j) < Cq(i - 1, j)) ? 1.0 : -1.0;
  double cnx[7], cny[7];
  cnx[0] = -sgy * (Hp1 - Hm1) / (2.0 * dx); cny[0] = sgy * 1.0;
  cnx[1] = -sgy * (Hp1 - H0) / (dx);        cny[1] = sgy * 1.0;
  cnx[2] = -sgy * (H0 - Hm1) / (dx);        cny[2] = sgy * 1.0;
  cnx[3] = sgx * 1.0; cny[3] = -sgx * (Wp1 - Wm1) / (2.0 * dy);
  cnx[4] = sgx * 1.0; cny[4] = -sgx * (Wp1 - W0) / (dy);
  cnx[5] = sgx * 1.0; cny[5] = -sgx * (W0 - Wm1) / (dy);
  cnx[6] = -((Cq(i + 1, j + 1) + 2.0 * Cq(i + 1, j) + Cq(i + 1, j - 1)) -
             (Cq(i - 1, j + 1) + 2.0 * Cq(i - 1, j) + Cq(i - 1, j - 1))) / (8.0 * dx);
  cny[6] = -((Cq(i + 1, j + 1) + 2.0 * Cq(i, j + 1) + Cq(i - 1, j + 1)) -
             (Cq(i + 1, j - 1) + 2.0 * Cq(i, j - 1) + Cq(i - 1, j - 1))) / (8.0 * dy);
  double best_err = 1.0e30, bnx = 1.0, bny = 0.0, ba = 0.0;
  for (int q = 0; q < 7; ++q) {
    const double cn = fhypot(cnx[q], cny[q]);
    if (cn < 1.0e-12) continue;
    const double ux = cnx[q] / cn, uy = cny[q] / cn;
    const double ca = compute_alpha(xmin, xmax, ymin, ymax, ux, uy, c);
    double err = 0.0;
    for (int dj = -1; dj <= 1; ++dj)
      for (int di = -1; di <= 1; ++di) {
        if (di == 0 && dj == 0) continue;
        const double vt = Cq(i + di, j + dj) * dx * dy;
        const double vr = cut_box_area(m.xf(i + di), m.xf(i + di + 1), m.yf(j + dj),
                                       m.yf(j + dj + 1), ux, uy, ca);
        const double df = vr - vt;
        err = err + df * df;
      }
    if (err < best_err) { best_err = err; bnx = ux; bny = uy; ba = ca; }
  }
  put_seg(a.seg, k, bnx, bny, ba);
}

// src/module_interface_reconstruction.f90:602-681: ghost-ring cells take the
// normal of the nearest interior cell and get a fresh line constant.
__global__ void k_vof_ring(VofArgs a) {
  const VMesh m{a.D, a.dx, a.dy};
  const int nx = a.D.nx, ny = a.D.ny;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  int i, j;
  if (t < ny) { i = 0; j = t + 1; }
  else if (t < 2 * ny) { i = nx + 1; j = t - ny + 1; }
  else if (t < 2 * ny + nx + 2) { i = t - 2 * ny; j = 0; }
  else if (t < 2 * ny + 2 * (nx + 2)) { i = t - 2 * ny - (nx + 2); j = ny + 1; }
  else return;
  const int k = a.D.id(i, j);
  const double c = a.C[k];
  if (!(c > 1.0e-6 && c < 1.0 - 1.0e-6)) return;
  const int si = i < 1 ? 1 : (i > nx ? nx : i);
  const int sj = j < 1 ? 1 : (j > ny ? ny : j);
  const int ks = a.D.id(si, sj);
  double snx = a.seg[3 * ks], sny = a.seg[3 * ks + 1];
  const double nr = fhypot(snx, sny);
  if (nr > 1.0e-12) {
    snx = snx / nr; sny = sny / nr;
    put_seg(a.seg, k, snx, sny, compute_alpha(m.xf(i), m.xf(i + 1), m.yf(j), m.yf(j + 1), snx, sny, c));
  }
}

// Donor-region flux through one face (src/module_interface_vof.f90:1204-1222
// for x, :1252-1270 for y).
__device__ __forceinline__ double x_flux(const VMesh& m, const double* __restrict__ seg,
                                         const double* __restrict__ u, double dt, int i, int j) {
  const double uf = u[m.D.id(i, j)];
  const double d = fabs(uf) * dt;
  if (d <= 1.0e-14) return 0.0;
  const double xp = m.xf(i);
  if (uf > 0.0) {
    const int ks = m.D.id(i - 1, j);
    return cut_box_area(xp - d, xp, m.yf(j), m.yf(j + 1), seg[3 * ks], seg[3 * ks + 1], seg[3 * ks + 2]);
  }
  const int ks = m.D.id(i, j);
  return -cut_box_area(xp, xp + d, m.yf(j), m.yf(j + 1), seg[3 * ks], seg[3 * ks + 1], seg[3 * ks + 2]);
}
__device__ __forceinline__ double y_flux(const VMesh& m, const double* __restrict__ seg,
                                         const double* __restrict__ v, double dt, int i, int j) {
  const double vf = v[m.D.id(i, j)];
  const double d = fabs(vf) * dt;
  if (d <= 1.0e-14) return 0.0;
  const double yp = m.yf(j);
  if (vf > 0.0) {
    const int ks = m.D.id(i, j - 1);
    return cut_box_area(m.xf(i), m.xf(i + 1), yp - d, yp, seg[3 * ks], seg[3 * ks + 1], seg[3 * ks + 2]);
  }
  const int ks = m.D.id(i, j);
  return -cut_box_area(m.xf(i), m.xf(i + 1), yp, yp + d, seg[3 * ks], seg[3 * ks + 1], seg[3 * ks + 2]);
}

// One Weymouth-Yue direction pass (src/module_interface_vof.f90:1199-1285):
// interior cells get C - div(flux)/dV + c_d dt/dh du; ghost cells copy Cin.
// c_d = [C^n >= 0.5] is read from Cn (frozen at time n, :1189-1197).
__global__ void k_vof_pass(VofArgs a, int dir, int clamp, const double* __restrict__ Cin,
                           double* __restrict__ Cout) {
  const VMesh m{a.D, a.dx, a.dy};
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.D.nx, ny = a.D.ny;
  if (i > nx + 1 || j > ny + 1) return;
  const int k = a.D.id(i, j);
  if (i < 1 || i > nx || j < 1 || j > ny) { Cout[k] = Cin[k]; return; }
  const double area = a.dx * a.dy;
  const double cd = a.Cn[k] >= 0.5 ? 1.0 : 0.0;
  double c;
  if (dir == 0) {
    const double fw = x_flux(m, a.seg, a.u, a.dt, i, j);
    const double fe = x_flux(m, a.seg, a.u, a.dt, i + 1, j);
    c = Cin[k] - (fe - fw) / area + cd * (a.dt / a.dx) * (a.u[k + 1] - a.u[k]);
  } else {
    const double fs = y_flux(m, a.seg, a.v, a.dt, i, j);
    const double fn = y_flux(m, a.seg, a.v, a.dt, i, j + 1);
    c = Cin[k] - (fn - fs) / area + cd * (a.dt / a.dy) * (a.v[k + a.D.P] - a.v[k]);
  }
  if (clamp) c = fmax(0.0, fmin(1.0, c));
  Cout[k] = c;
}

// src/module_mpi_comm.f90:636-683 apply_vof_bc (np = 1): zero-gradient
// edge ghosts, corners untouched.
__global__ void k_vof_bc(Dims D, double* __restrict__ C) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nx = D.nx, ny = D.ny;
  if (t < ny) {
    const int j = t + 1;
    C[D.id(0, j)] = C[D.id(1, j)];
    C[D.id(nx + 1, j)] = C[D.id(nx, j)];
  } else if (t < ny + nx) {
    const int i = t - ny + 1;
    C[D.id(i, 0)] = C[D.id(i, 1)];
    C[D.id(i, ny + 1)] = C[D.id(i, ny)];
  }
}

// src/module_interface_vof.f90:530-560: physical corners of C, then rho and
// mu at every cell; mu's corners equal the interior corner values.
__global__ void k_props_cells(PropsArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.D.nx, ny = a.D.ny;
  if (i > nx + 1 || j > ny + 1) return;
  const int k = a.D.id(i, j);
  if (!a.two_phase) {
    a.rho[k] = a.rho1; a.rho_u[k] = a.rho1; a.rho_v[k] = a.rho1;
    a.mu[k] = a.mu1; a.mu_node[k] = a.mu1;
    return;
  }
  const bool corner = (i == 0 || i == nx + 1) && (j == 0 || j == ny + 1);
  double cv;
  if (corner) {
    const int ki = a.D.id(i == 0 ? 1 : nx, j == 0 ? 1 : ny);
    cv = a.C[ki];
    a.C[k] = cv;
  } else {
    cv = a.C[k];
  }
  const double c = fmax(0.0, fmin(1.0, cv));
  a.rho[k] = c * a.rho1 + (1.0 - c) * a.rho2;
  a.mu[k] = c * a.mu1 + (1.0 - c) * a.mu2;
}

// src/module_interface_vof.f90:575-615: face densities (arithmetic) and node
// viscosity (harmonic).
__global__ void k_props_faces(PropsArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int nx = a.D.nx, ny = a.D.ny;
  if (!a.two_phase || i > nx + 1 || j > ny + 1) return;
  const int k = a.D.id(i, j);
  if (j <= ny) a.rho_u[k] = 0.5 * (a.rho[k - 1] + a.rho[k]);
  if (i <= nx) a.rho_v[k] = 0.5 * (a.rho[k - a.D.P] + a.rho[k]);
  const double sw = a.mu[k - a.D.P - 1], se = a.mu[k - a.D.P];
  const double nw = a.mu[k - 1], ne = a.mu[k];
  a.mu_node[k] = 4.0 / (1.0 / sw + 1.0 / se + 1.0 / nw + 1.0 / ne);
}

// src/module_interface_vof.f90:663-686: unit normal of grad C at interior cells.
__global__ void k_csf_normals(CsfArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > a.D.nx || j > a.D.ny) return;
  const int k = a.D.id(i, j);
  const double dcx = (a.C[k + 1] - a.C[k - 1]) / (2.0 * a.dx);
  const double dcy = (a.C[k + a.D.P] - a.C[k - a.D.P]) / (2.0 * a.dy);
  const double gm = sqrt(dcx * dcx + dcy * dcy);
  double nxv = 0.0, nyv = 0.0;
  if (gm > 1.0e-3 / a.dx) { nxv = dcx / gm; nyv = dcy / gm; }
  a.nxv[k] = nxv; a.nyv[k] = nyv;
}

// src/module_interface_vof.f90:694-704: kappa = -div n (ghost ring stays 0).
__global__ void k_csf_kappa(CsfArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > a.D.nx || j > a.D.ny) return;
  const int k = a.D.id(i, j);
  double kap = 0.0;
  if (a.nxv[k] != 0.0 || a.nyv[k] != 0.0)
    kap = -((a.nxv[k + 1] - a.nxv[k - 1]) / (2.0 * a.dx) + (a.nyv[k + a.D.P] - a.nyv[k - a.D.P]) / (2.0 * a.dy));
  a.kappa[k] = kap;
}

// src/module_interface_vof.f90:721-787: face forces sigma * kappa_face * dC/dn.
__global__ void k_csf_force(CsfArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.D.nx, ny = a.D.ny;
  if (i > nx + 1 || j > ny + 1) return;
  const int k = a.D.id(i, j);
  a.curv[k] = a.kappa[k];
  if (i >= 1 && j >= 1 && j <= ny) {
    const double ka = 0.5 * (a.kappa[k - 1] + a.kappa[k]);
    const double gc = (a.C[k] - a.C[k - 1]) / a.dx;
    a.fx[k] = a.sigma * ka * gc;
  }
  if (i >= 1 && i <= nx && j >= 1) {
    const double ka = 0.5 * (a.kappa[k - a.D.P] + a.kappa[k]);
    const double gc = (a.C[k] - a.C[k - a.D.P]) / a.dy;
    a.fy[k] = a.sigma * ka * gc;
  }
}

}  // namespace covof
