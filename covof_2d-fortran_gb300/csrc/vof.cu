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
// Pure cells (C <= 1e-6 or >= 1-1e-6) short-circuit, so the reconstruction
// cost concentrates on interface cells, which get one warp each (below).
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

__device__ __forceinline__ void put_seg(double* seg, int k, double a, double b, double c) {
  seg[3 * k] = a; seg[3 * k + 1] = b; seg[3 * k + 2] = c;
}

// ---------------------------------------------------------------------------
// Reconstruction, src/module_interface_reconstruction.f90:283-343 (PLIC),
// :346-457 (ELVIRA) and :580-683 (reconstruct_interface).  Interface cells
// are few, and each costs hundreds of FP64 polygon clips (ELVIRA: 7
// candidates x (45 bisection steps + 8 neighbour clips)) -- FP64 issue is
// the scarce unit of a GB300 SM -- so one thread per cell would leave a
// handful of warps issuing long serial chains while the rest of the GPU
// idles.  Instead:
//   k_vof_classify  writes pure cells and appends interface cells to a list;
//   k_vof_mixed     gives every listed cell one warp;
//   k_vof_ring_warp does the ghost ring (normal of the nearest interior
//                   cell, fresh line constant) the same way.
// Every value is bit-identical to the serial evaluation.

// compute_alpha (src/module_interface_reconstruction.f90:105-147: bisection
// on the clipped area, 45 levels) with the levels replayed D per round by
// a group of 2^D lanes (lanes gbase .. gbase + 2^D - 1 of the warp): lane
// gbase + n evaluates node n (heap numbering, n = 1 .. 2^D - 1) of the
// round's decision tree, whose interval it derives from the round's (lo, hi)
// with the same midpoint formula along the node's path, so every midpoint
// equals the serial one bit for bit; a ballot then walks the tree exactly as
// the serial loop would.  Every lane of the warp must call this together.
template <int D>
__device__ double tree_alpha(int sub, int gbase, double xmin, double xmax, double ymin, double ymax,
                             double nx, double ny, double c_target) {
  const double total = (xmax - xmin) * (ymax - ymin);
  const double target = fmax(0.0, fmin(1.0, c_target)) * total;
  const double v1 = nx * xmin + ny * ymin;
  const double v2 = nx * xmax + ny * ymin;
  const double v3 = nx * xmax + ny * ymax;
  const double v4 = nx * xmin + ny * ymax;
  const double mn = fmin(v1, fmin(v2, fmin(v3, v4)));
  const double mx = fmax(v1, fmax(v2, fmax(v3, v4)));
  double lo = -mx - 1.0e-12;
  double hi = -mn + 1.0e-12;
  for (int left = 45; left > 0;) {
    const int L = left < D ? left : D;
    bool below = false;
    if (sub >= 1 && sub < (1 << L)) {
      double l = lo, h = hi;
      const int depth = 31 - __clz(sub);
      for (int b = depth - 1; b >= 0; --b) {
        const double mid = 0.5 * (l + h);
        if ((sub >> b) & 1) l = mid; else h = mid;
      }
      const double mid = 0.5 * (l + h);
      below = cut_box_area(xmin, xmax, ymin, ymax, nx, ny, mid) < target;
    }
    const unsigned gb = __ballot_sync(0xffffffffu, below) >> gbase;
    int n = 1;
    for (int lev = 0; lev < L; ++lev) {
      const double mid = 0.5 * (lo + hi);
      const bool bl = (gb >> n) & 1u;
      if (bl) hi = mid; else lo = mid;
      n = 2 * n + (bl ? 0 : 1);
    }
    left -= L;
  }
  if (c_target <= 1.0e-7) return 1.0e9;
  if (c_target >= 1.0 - 1.0e-7) return -1.0e9;
  return 0.5 * (lo + hi);
}

// Pure cells of (0:nx+1, 0:ny+1) get their segment; interface cells are
// appended to list (one atomic per warp).  The list order does not matter:
// every entry is reconstructed independently.
__global__ void k_vof_classify(VofArgs a, int* __restrict__ list, int* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const bool in = i <= a.D.nx + 1 && j <= a.D.ny + 1;
  bool mixed = false;
  int k = 0;
  if (in) {
    k = a.D.id(i, j);
    const double c = a.C[k];
    if (c <= 1.0e-6) put_seg(a.seg, k, 1.0, 0.0, 1.0e9);
    else if (c >= 1.0 - 1.0e-6) put_seg(a.seg, k, 1.0, 0.0, -1.0e9);
    else mixed = true;
  }
  const unsigned lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31u;
  const unsigned bal = __ballot_sync(0xffffffffu, mixed);
  if (!bal) return;
  const int leader = __ffs(bal) - 1;
  int base = 0;
  if ((int)lane == leader) base = atomicAdd(count, __popc(bal));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (mixed) list[base + __popc(bal & ((1u << lane) - 1u))] = k;
}

// One warp per listed cell, for lists of min_count .. max_count - 1 cells
// (the block and thread forms below take the shorter and the longer ones).
// ELVIRA (inner cells):
// candidate q on lanes 4q .. 4q+3 (lanes 28-31 repeat candidate 6 and are
// ignored); its bisection runs 2 levels per round, its 8 neighbour clips 2
// per lane, and the error is summed and the candidate chosen in the
// reference order.  PLIC, and ELVIRA on ghost cells: one normal, 5 levels
// per round.
__global__ void __launch_bounds__(128) k_vof_mixed(VofArgs a, const int* __restrict__ list,
                                                    const int* __restrict__ count, int min_count, int max_count) {
  const VMesh m{a.D, a.dx, a.dy};
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int n = *count;
  if (n < min_count || n >= max_count) return;
  const int nx = a.D.nx, ny = a.D.ny;
  const double* __restrict__ C = a.C;
  const double dx = a.dx, dy = a.dy;
  for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n; e += nwarps) {
    const int k = list[e];
    const int j = k / a.D.P, i = k - j * a.D.P;
    const double c = C[k];
    const double xmin = m.xf(i), xmax = m.xf(i + 1), ymin = m.yf(j), ymax = m.yf(j + 1);
    const bool inner = (i >= 1 && i <= nx && j >= 1 && j <= ny);
    // checked builds: an inner cell reads its 3 x 3 neighbourhood (ghost
    // cells of the list read only themselves)
    if (inner && a.D.nbhd(k, 22) != k) continue;
    auto Cq = [&](int p, int q) { return C[a.D.id(p, q)]; };
    if (a.method != COVOF_RECON_ELVIRA || !inner) {
      double pnx = 1.0, pny = 0.0;
      if (a.method != COVOF_RECON_ELVIRA && inner) {
        const double cmm = Cq(i - 1, j - 1), c0m = Cq(i, j - 1), cpm = Cq(i + 1, j - 1);
        const double cm0 = Cq(i - 1, j), cp0 = Cq(i + 1, j);
        const double cmp = Cq(i - 1, j + 1), c0p = Cq(i, j + 1), cpp = Cq(i + 1, j + 1);
        const double mxv = -((cpp + 2.0 * cp0 + cpm) - (cmp + 2.0 * cm0 + cmm)) / (8.0 * dx);
        const double myv = -((cpp + 2.0 * c0p + cmp) - (cpm + 2.0 * c0m + cmm)) / (8.0 * dy);
        const double nrm = fhypot(mxv, myv);
        if (nrm > 1.0e-12) { pnx = mxv / nrm; pny = myv / nrm; }
      } else if (a.method != COVOF_RECON_ELVIRA) {
        const double nrm = fhypot(1.0, 0.0);
        pnx = 1.0 / nrm; pny = 0.0 / nrm;
      }
      const double al = tree_alpha<5>(lane, 0, xmin, xmax, ymin, ymax, pnx, pny, c);
      if (lane == 0) put_seg(a.seg, k, pnx, pny, al);
      continue;
    }
    const int q = (lane >> 2) < 7 ? (lane >> 2) : 6, sub = lane & 3, gbase = lane & ~3;
    const double Hm1 = (Cq(i - 1, j - 1) + Cq(i - 1, j) + Cq(i - 1, j + 1)) * dy;
    const double H0 = (Cq(i, j - 1) + Cq(i, j) + Cq(i, j + 1)) * dy;
    const double Hp1 = (Cq(i + 1, j - 1) + Cq(i + 1, j) + Cq(i + 1, j + 1)) * dy;
    const double Wm1 = (Cq(i - 1, j - 1) + Cq(i, j - 1) + Cq(i + 1, j - 1)) * dx;
    const double W0 = (Cq(i - 1, j) + Cq(i, j) + Cq(i + 1, j)) * dx;
    const double Wp1 = (Cq(i - 1, j + 1) + Cq(i, j + 1) + Cq(i + 1, j + 1)) * dx;
    const double sgy = (Cq(i, j + 1) < Cq(i, j - 1)) ? 1.0 : -1.0;
    const double sgx = (Cq(i + 1, j) < Cq(i - 1, j)) ? 1.0 : -1.0;
    double cnx, cny;
    switch (q) {
      case 0: cnx = -sgy * (Hp1 - Hm1) / (2.0 * dx); cny = sgy * 1.0; break;
      case 1: cnx = -sgy * (Hp1 - H0) / (dx); cny = sgy * 1.0; break;
      case 2: cnx = -sgy * (H0 - Hm1) / (dx); cny = sgy * 1.0; break;
      case 3: cnx = sgx * 1.0; cny = -sgx * (Wp1 - Wm1) / (2.0 * dy); break;
      case 4: cnx = sgx * 1.0; cny = -sgx * (Wp1 - W0) / (dy); break;
      case 5: cnx = sgx * 1.0; cny = -sgx * (W0 - Wm1) / (dy); break;
      default:
        cnx = -((Cq(i + 1, j + 1) + 2.0 * Cq(i + 1, j) + Cq(i + 1, j - 1)) -
                (Cq(i - 1, j + 1) + 2.0 * Cq(i - 1, j) + Cq(i - 1, j - 1))) / (8.0 * dx);
        cny = -((Cq(i + 1, j + 1) + 2.0 * Cq(i, j + 1) + Cq(i - 1, j + 1)) -
                (Cq(i + 1, j - 1) + 2.0 * Cq(i, j - 1) + Cq(i - 1, j - 1))) / (8.0 * dy);
        break;
    }
    const double cn = fhypot(cnx, cny);
    const bool valid = !(cn < 1.0e-12);
    const double ux = valid ? cnx / cn : 1.0, uy = valid ? cny / cn : 0.0;
    const double ca = tree_alpha<2>(sub, gbase, xmin, xmax, ymin, ymax, ux, uy, c);
    // neighbour s (reference order: dj = -1..1, di = -1..1, centre skipped)
    // on lane sub (s = sub) and sub + 4
    double sq[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int s = sub + 4 * h;
      const int t = s < 4 ? s : s + 1;
      const int di = t % 3 - 1, dj = t / 3 - 1;
      const double vt = Cq(i + di, j + dj) * dx * dy;
      const double vr = cut_box_area(m.xf(i + di), m.xf(i + di + 1), m.yf(j + dj), m.yf(j + dj + 1), ux, uy, ca);
      const double df = vr - vt;
      sq[h] = df * df;
    }
    double err = 0.0;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      const double v = __shfl_sync(0xffffffffu, s < 4 ? sq[0] : sq[1], gbase + (s & 3));
      err = err + v;
    }
    double best_err = 1.0e30, bnx = 1.0, bny = 0.0, ba = 0.0;
#pragma unroll
    for (int qq = 0; qq < 7; ++qq) {
      const double eq = __shfl_sync(0xffffffffu, err, 4 * qq);
      const int vq = __shfl_sync(0xffffffffu, valid ? 1 : 0, 4 * qq);
      const double xq = __shfl_sync(0xffffffffu, ux, 4 * qq);
      const double yq = __shfl_sync(0xffffffffu, uy, 4 * qq);
      const double aq = __shfl_sync(0xffffffffu, ca, 4 * qq);
      if (vq && eq < best_err) { best_err = eq; bnx = xq; bny = yq; ba = aq; }
    }
    if (lane == 0) put_seg(a.seg, k, bnx, bny, ba);
  }
}

// ELVIRA with one 128-thread block per listed cell, for lists shorter than
// max_count (about one wave of blocks): the latency form.  Candidate q on
// the 16 lanes 16q .. 16q+15 (lanes 112-127 repeat candidate 6 and are
// ignored), so its bisection runs 4 levels per round (12 rounds against the
// warp form's 23) and its 8 neighbour clips one per lane; the candidates
// meet in shared memory and thread 0 chooses in the reference order.  Ghost
// cells of the list (one normal) go to the first warp, 5 levels per round.
// Bit-identical to the warp and thread forms.
__global__ void __launch_bounds__(128) k_vof_elvira_block(VofArgs a, const int* __restrict__ list,
                                                          const int* __restrict__ count, int max_count) {
  __shared__ double s_err[7], s_ux[7], s_uy[7], s_ca[7];
  __shared__ int s_valid[7];
  const VMesh m{a.D, a.dx, a.dy};
  const int n = *count;
  if (n >= max_count) return;
  const int lane = threadIdx.x & 31;
  const int q = (threadIdx.x >> 4) < 7 ? (int)(threadIdx.x >> 4) : 6;
  const int sub = lane & 15, gbase = lane & 16;
  const int nx = a.D.nx, ny = a.D.ny;
  const double* __restrict__ C = a.C;
  const double dx = a.dx, dy = a.dy;
  for (int e = blockIdx.x; e < n; e += gridDim.x) {
    const int k = list[e];
    const int j = k / a.D.P, i = k - j * a.D.P;
    const double c = C[k];
    const double xmin = m.xf(i), xmax = m.xf(i + 1), ymin = m.yf(j), ymax = m.yf(j + 1);
    const bool inner = (i >= 1 && i <= nx && j >= 1 && j <= ny);
    if (inner && a.D.nbhd(k, 24) != k) continue;
    auto Cq = [&](int p, int qq) { return C[a.D.id(p, qq)]; };
    if (!inner) {
      // a ghost cell: the (1, 0) normal and a fresh line constant
      if (threadIdx.x < 32) {
        const double al = tree_alpha<5>(lane, 0, xmin, xmax, ymin, ymax, 1.0, 0.0, c);
        if (lane == 0) put_seg(a.seg, k, 1.0, 0.0, al);
      }
      continue;
    }
    const double Hm1 = (Cq(i - 1, j - 1) + Cq(i - 1, j) + Cq(i - 1, j + 1)) * dy;
    const double H0 = (Cq(i, j - 1) + Cq(i, j) + Cq(i, j + 1)) * dy;
    const double Hp1 = (Cq(i + 1, j - 1) + Cq(i + 1, j) + Cq(i + 1, j + 1)) * dy;
    const double Wm1 = (Cq(i - 1, j - 1) + Cq(i, j - 1) + Cq(i + 1, j - 1)) * dx;
    const double W0 = (Cq(i - 1, j) + Cq(i, j) + Cq(i + 1, j)) * dx;
    const double Wp1 = (Cq(i - 1, j + 1) + Cq(i, j + 1) + Cq(i + 1, j + 1)) * dx;
    const double sgy = (Cq(i, j + 1) < Cq(i, j - 1)) ? 1.0 : -1.0;
    const double sgx = (Cq(i + 1, j) < Cq(i - 1, j)) ? 1.0 : -1.0;
    double cnx, cny;
    switch (q) {
      case 0: cnx = -sgy * (Hp1 - Hm1) / (2.0 * dx); cny = sgy * 1.0; break;
      case 1: cnx = -sgy * (Hp1 - H0) / (dx); cny = sgy * 1.0; break;
      case 2: cnx = -sgy * (H0 - Hm1) / (dx); cny = sgy * 1.0; break;
      case 3: cnx = sgx * 1.0; cny = -sgx * (Wp1 - Wm1) / (2.0 * dy); break;
      case 4: cnx = sgx * 1.0; cny = -sgx * (Wp1 - W0) / (dy); break;
      case 5: cnx = sgx * 1.0; cny = -sgx * (W0 - Wm1) / (dy); break;
      default:
        cnx = -((Cq(i + 1, j + 1) + 2.0 * Cq(i + 1, j) + Cq(i + 1, j - 1)) -
                (Cq(i - 1, j + 1) + 2.0 * Cq(i - 1, j) + Cq(i - 1, j - 1))) / (8.0 * dx);
        cny = -((Cq(i + 1, j + 1) + 2.0 * Cq(i, j + 1) + Cq(i - 1, j + 1)) -
                (Cq(i + 1, j - 1) + 2.0 * Cq(i, j - 1) + Cq(i - 1, j - 1))) / (8.0 * dy);
        break;
    }
    const double cn = fhypot(cnx, cny);
    const bool valid = !(cn < 1.0e-12);
    const double ux = valid ? cnx / cn : 1.0, uy = valid ? cny / cn : 0.0;
    const double ca = tree_alpha<4>(sub, gbase, xmin, xmax, ymin, ymax, ux, uy, c);
    // neighbour s (reference order: dj = -1..1, di = -1..1, centre skipped) on lane sub = s
    double sq = 0.0;
    if (sub < 8) {
      const int t = sub < 4 ? sub : sub + 1;
      const int di = t % 3 - 1, dj = t / 3 - 1;
      const double vt = Cq(i + di, j + dj) * dx * dy;
      const double vr = cut_box_area(m.xf(i + di), m.xf(i + di + 1), m.yf(j + dj), m.yf(j + dj + 1), ux, uy, ca);
      const double df = vr - vt;
      sq = df * df;
    }
    double err = 0.0;
#pragma unroll
    for (int s = 0; s < 8; ++s) err = err + __shfl_sync(0xffffffffu, sq, gbase + s);
    if (sub == 0 && (threadIdx.x >> 4) < 7) {
      s_err[q] = err; s_valid[q] = valid ? 1 : 0; s_ux[q] = ux; s_uy[q] = uy; s_ca[q] = ca;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double best_err = 1.0e30, bnx = 1.0, bny = 0.0, ba = 0.0;
      for (int qq = 0; qq < 7; ++qq)
        if (s_valid[qq] && s_err[qq] < best_err) { best_err = s_err[qq]; bnx = s_ux[qq]; bny = s_uy[qq]; ba = s_ca[qq]; }
      put_seg(a.seg, k, bnx, bny, ba);
    }
    __syncthreads();
  }
}

// compute_alpha (src/module_interface_reconstruction.f90:105-147) as the
// serial 45-step bisection, one thread.
__device__ double serial_alpha(double xmin, double xmax, double ymin, double ymax, double nx, double ny,
                               double c_target) {
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
    if (cut_box_area(xmin, xmax, ymin, ymax, nx, ny, mid) < target) hi = mid;
    else lo = mid;
  }
  return 0.5 * (lo + hi);
}

// One thread per listed cell, for lists of at least min_count cells.  A
// warp instruction on the FP64 pipe costs the same whatever its active
// lanes, and the warp form spends lanes on idle tree nodes and on 1.5
// clips per bisection level; once the interface cells fill every warp slot
// of the GPU, the serial form (32 cells per warp, one clip per level) does
// the same work in fewer FP64 warp instructions.  Same arithmetic, same
// order: bit-identical to the warp form and to the serial reference.
__global__ void __launch_bounds__(128) k_vof_mixed_cell(VofArgs a, const int* __restrict__ list,
                                                        const int* __restrict__ count, int min_count) {
  const VMesh m{a.D, a.dx, a.dy};
  const int n = *count;
  if (n < min_count) return;
  const int nx = a.D.nx, ny = a.D.ny;
  const double* __restrict__ C = a.C;
  const double dx = a.dx, dy = a.dy;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int k = list[e];
    const int j = k / a.D.P, i = k - j * a.D.P;
    const double c = C[k];
    const double xmin = m.xf(i), xmax = m.xf(i + 1), ymin = m.yf(j), ymax = m.yf(j + 1);
    const bool inner = (i >= 1 && i <= nx && j >= 1 && j <= ny);
    if (inner && a.D.nbhd(k, 23) != k) continue;
    auto Cq = [&](int p, int q) { return C[a.D.id(p, q)]; };
    if (a.method != COVOF_RECON_ELVIRA || !inner) {
      double pnx = 1.0, pny = 0.0;
      if (a.method != COVOF_RECON_ELVIRA && inner) {
        const double cmm = Cq(i - 1, j - 1), c0m = Cq(i, j - 1), cpm = Cq(i + 1, j - 1);
        const double cm0 = Cq(i - 1, j), cp0 = Cq(i + 1, j);
        const double cmp = Cq(i - 1, j + 1), c0p = Cq(i, j + 1), cpp = Cq(i + 1, j + 1);
        const double mxv = -((cpp + 2.0 * cp0 + cpm) - (cmp + 2.0 * cm0 + cmm)) / (8.0 * dx);
        const double myv = -((cpp + 2.0 * c0p + cmp) - (cpm + 2.0 * c0m + cmm)) / (8.0 * dy);
        const double nrm = fhypot(mxv, myv);
        if (nrm > 1.0e-12) { pnx = mxv / nrm; pny = myv / nrm; }
      } else if (a.method != COVOF_RECON_ELVIRA) {
        const double nrm = fhypot(1.0, 0.0);
        pnx = 1.0 / nrm; pny = 0.0 / nrm;
      }
      put_seg(a.seg, k, pnx, pny, serial_alpha(xmin, xmax, ymin, ymax, pnx, pny, c));
      continue;
    }
    const double Hm1 = (Cq(i - 1, j - 1) + Cq(i - 1, j) + Cq(i - 1, j + 1)) * dy;
    const double H0 = (Cq(i, j - 1) + Cq(i, j) + Cq(i, j + 1)) * dy;
    const double Hp1 = (Cq(i + 1, j - 1) + Cq(i + 1, j) + Cq(i + 1, j + 1)) * dy;
    const double Wm1 = (Cq(i - 1, j - 1) + Cq(i, j - 1) + Cq(i + 1, j - 1)) * dx;
    const double W0 = (Cq(i - 1, j) + Cq(i, j) + Cq(i + 1, j)) * dx;
    const double Wp1 = (Cq(i - 1, j + 1) + Cq(i, j + 1) + Cq(i + 1, j + 1)) * dx;
    const double sgy = (Cq(i, j + 1) < Cq(i, j - 1)) ? 1.0 : -1.0;
    const double sgx = (Cq(i + 1, j) < Cq(i - 1, j)) ? 1.0 : -1.0;
    double best_err = 1.0e30, bnx = 1.0, bny = 0.0, ba = 0.0;
    for (int q = 0; q < 7; ++q) {
      double cnx, cny;
      switch (q) {
        case 0: cnx = -sgy * (Hp1 - Hm1) / (2.0 * dx); cny = sgy * 1.0; break;
        case 1: cnx = -sgy * (Hp1 - H0) / (dx); cny = sgy * 1.0; break;
        case 2: cnx = -sgy * (H0 - Hm1) / (dx); cny = sgy * 1.0; break;
        case 3: cnx = sgx * 1.0; cny = -sgx * (Wp1 - Wm1) / (2.0 * dy); break;
        case 4: cnx = sgx * 1.0; cny = -sgx * (Wp1 - W0) / (dy); break;
        case 5: cnx = sgx * 1.0; cny = -sgx * (W0 - Wm1) / (dy); break;
        default:
          cnx = -((Cq(i + 1, j + 1) + 2.0 * Cq(i + 1, j) + Cq(i + 1, j - 1)) -
                  (Cq(i - 1, j + 1) + 2.0 * Cq(i - 1, j) + Cq(i - 1, j - 1))) / (8.0 * dx);
          cny = -((Cq(i + 1, j + 1) + 2.0 * Cq(i, j + 1) + Cq(i - 1, j + 1)) -
                  (Cq(i + 1, j - 1) + 2.0 * Cq(i, j - 1) + Cq(i - 1, j - 1))) / (8.0 * dy);
          break;
      }
      const double cn = fhypot(cnx, cny);
      if (cn < 1.0e-12) continue;
      const double ux = cnx / cn, uy = cny / cn;
      const double ca = serial_alpha(xmin, xmax, ymin, ymax, ux, uy, c);
      double err = 0.0;
      for (int dj = -1; dj <= 1; ++dj)
        for (int di = -1; di <= 1; ++di) {
          if (di == 0 && dj == 0) continue;
          const double vt = Cq(i + di, j + dj) * dx * dy;
          const double vr = cut_box_area(m.xf(i + di), m.xf(i + di + 1), m.yf(j + dj), m.yf(j + dj + 1), ux, uy, ca);
          const double df = vr - vt;
          err = err + df * df;
        }
      if (err < best_err) { best_err = err; bnx = ux; bny = uy; ba = ca; }
    }
    put_seg(a.seg, k, bnx, bny, ba);
  }
}

// Ghost ring (src/module_interface_reconstruction.f90:602-681), one warp per
// ring cell: the normal of the nearest interior cell, a fresh line constant.
__global__ void __launch_bounds__(128) k_vof_ring_warp(VofArgs a) {
  const VMesh m{a.D, a.dx, a.dy};
  const int nx = a.D.nx, ny = a.D.ny;
  const int lane = threadIdx.x & 31;
  const int nring = 2 * ny + 2 * (nx + 2);
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nring; t += nwarps) {
    int i, j;
    if (t < ny) { i = 0; j = t + 1; }
    else if (t < 2 * ny) { i = nx + 1; j = t - ny + 1; }
    else if (t < 2 * ny + nx + 2) { i = t - 2 * ny; j = 0; }
    else { i = t - 2 * ny - (nx + 2); j = ny + 1; }
    const int k = a.D.id(i, j);
    const double c = a.C[k];
    if (!(c > 1.0e-6 && c < 1.0 - 1.0e-6)) continue;
    // the normal of the nearest interior cell, or of the wrapped one in a
    // periodic direction (:606-627: the normals' halo exchange, then the
    // copies on the non-periodic sides).  With x closed and y periodic the
    // y wrap of the corners happens before the x copies fill column 0 / nx+1,
    // so the reference's corner normal is zero and no segment is formed.
    if (!a.D.perx && a.D.pery && (i == 0 || i == nx + 1) && (j == 0 || j == ny + 1)) continue;
    const int si = a.D.perx ? a.D.wrap_i(i) : (i < 1 ? 1 : (i > nx ? nx : i));
    const int sj = a.D.pery ? a.D.wrap_j(j) : (j < 1 ? 1 : (j > ny ? ny : j));
    const int ks = a.D.id(si, sj);
    double snx = a.seg[3 * ks], sny = a.seg[3 * ks + 1];
    const double nr = fhypot(snx, sny);
    if (!(nr > 1.0e-12)) continue;
    snx = snx / nr; sny = sny / nr;
    const double al = tree_alpha<5>(lane, 0, m.xf(i), m.xf(i + 1), m.yf(j), m.yf(j + 1), snx, sny, c);
    if (lane == 0) put_seg(a.seg, k, snx, sny, al);
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

// The flux of face i (x) / j (y) with the periodic sync of
// src/module_interface_vof.f90:1223-1231, 1268-1276: the two images of the
// periodic face (1 and nx+1) carry the flux computed at the one the velocity
// of face 1 comes from.
__device__ __forceinline__ double x_flux_p(const VMesh& m, const double* __restrict__ seg,
                                           const double* __restrict__ u, double dt, int i, int j) {
  if (m.D.perx && (i == 1 || i == m.D.nx + 1))
    return x_flux(m, seg, u, dt, u[m.D.id(1, j)] >= 0.0 ? m.D.nx + 1 : 1, j);
  return x_flux(m, seg, u, dt, i, j);
}
__device__ __forceinline__ double y_flux_p(const VMesh& m, const double* __restrict__ seg,
                                           const double* __restrict__ v, double dt, int i, int j) {
  if (m.D.pery && (j == 1 || j == m.D.ny + 1))
    return y_flux(m, seg, v, dt, i, v[m.D.id(i, 1)] >= 0.0 ? m.D.ny + 1 : 1);
  return y_flux(m, seg, v, dt, i, j);
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
  if (a.D.nbhd(k, 20) != k) return;  // checked builds: a neighbourhood outside the array
  const double area = a.dx * a.dy;
  const double cd = a.Cn[k] >= 0.5 ? 1.0 : 0.0;
  double c;
  if (dir == 0) {
    const double fw = x_flux_p(m, a.seg, a.u, a.dt, i, j);
    const double fe = x_flux_p(m, a.seg, a.u, a.dt, i + 1, j);
    c = Cin[k] - (fe - fw) / area + cd * (a.dt / a.dx) * (a.u[k + 1] - a.u[k]);
  } else {
    const double fs = y_flux_p(m, a.seg, a.v, a.dt, i, j);
    const double fn = y_flux_p(m, a.seg, a.v, a.dt, i, j + 1);
    c = Cin[k] - (fn - fs) / area + cd * (a.dt / a.dy) * (a.v[k + a.D.P] - a.v[k]);
  }
  if (clamp) c = fmax(0.0, fmin(1.0, c));
  Cout[k] = c;
}

// One CIAM direction pass (src/module_interface_vof.f90:963-1073): the
// Weymouth-Yue donor flux volumes, then the Lagrangian remap
// (C dh - dF / dh') / (dh - dt du) (plain divergence where the remapped width
// would vanish), clamped; ghost cells copy Cin.
__global__ void k_ciam_pass(VofArgs a, int dir, const double* __restrict__ Cin, double* __restrict__ Cout) {
  const VMesh m{a.D, a.dx, a.dy};
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.D.nx, ny = a.D.ny;
  if (i > nx + 1 || j > ny + 1) return;
  const int k = a.D.id(i, j);
  if (i < 1 || i > nx || j < 1 || j > ny) { Cout[k] = Cin[k]; return; }
  if (a.D.nbhd(k, 20) != k) return;  // checked builds: a neighbourhood outside the array
  double c;
  if (dir == 0) {
    const double fw = x_flux(m, a.seg, a.u, a.dt, i, j);
    const double fe = x_flux(m, a.seg, a.u, a.dt, i + 1, j);
    const double denom = a.dx - a.dt * (a.u[k + 1] - a.u[k]);
    const double df = fe - fw;
    c = denom > 1.0e-12 ? (Cin[k] * a.dx - df / a.dy) / denom : Cin[k] - df / (a.dx * a.dy);
  } else {
    const double fs = y_flux(m, a.seg, a.v, a.dt, i, j);
    const double fn = y_flux(m, a.seg, a.v, a.dt, i, j + 1);
    const double denom = a.dy - a.dt * (a.v[k + a.D.P] - a.v[k]);
    const double df = fn - fs;
    c = denom > 1.0e-12 ? (Cin[k] * a.dy - df / a.dx) / denom : Cin[k] - df / (a.dx * a.dy);
  }
  Cout[k] = fmax(0.0, fmin(1.0, c));
}

// src/module_interface_reconstruction.f90:686-725 evaluate_limiter
__device__ __forceinline__ double tvd_limiter(int lim, double r, double cd, double cu, double ca) {
  switch (lim) {
    case COVOF_LIMITER_VAN_LEER:
      return r > 0.0 ? 2.0 * r / (1.0 + r) : 0.0;
    case COVOF_LIMITER_MUSCL:
      return fmax(0.0, fmin(2.0 * r, fmin(0.5 * (1.0 + r), 2.0)));
    case COVOF_LIMITER_HRIC: {
      const double denom = ca - cu;
      if (fabs(denom) < 1.0e-12) return 0.0;
      const double ctD = (cd - cu) / denom;
      double ctf = ctD;
      if (ctD >= 0.0 && ctD <= 1.0) ctf = ctD < 0.5 ? 2.0 * ctD : 1.0;
      if (fabs(1.0 - ctD) > 1.0e-12) {
        const double phi = 2.0 * (ctf - ctD) / (1.0 - ctD);
        return fmax(0.0, fmin(2.0, phi));
      }
      return 1.0;
    }
    default:
      return fmax(0.0, fmax(fmin(2.0 * r, 1.0), fmin(r, 2.0)));
  }
}

// Limited upwind flux through x face i (between cells i-1 and i), or y face j
// (src/module_interface_vof.f90:853-913); `o` is the stride along the face
// normal, lo / hi the first and last ghost index along it.
__device__ __forceinline__ double tvd_face_flux(int lim, double uf, double dt, double dh, const double* C, int k,
                                                int o, int idx, int hi) {
  const double cl = C[k - o], cr = C[k];
  const double cfl = 1.0 - fmin(1.0, fabs(uf) * dt / dh);
  if (uf >= 0.0) {
    const double cu = C[k - (idx - 2 >= 0 ? 2 : idx) * o];
    const double dup = cl - cu, dloc = cr - cl;
    const double r = fabs(dloc) > 1.0e-12 ? dup / dloc : 0.0;
    const double phi = tvd_limiter(lim, r, cl, cu, cr);
    return uf * (cl + 0.5 * phi * cfl * dloc);
  }
  const double cu = C[k + (idx + 1 <= hi ? 1 : 0) * o];
  const double dup = cu - cr, dloc = cr - cl;
  const double r = fabs(dloc) > 1.0e-12 ? dup / dloc : 0.0;
  const double phi = tvd_limiter(lim, r, cr, cu, cl);
  return uf * (cr - 0.5 * phi * cfl * dloc);
}

// src/module_interface_vof.f90:828-935 advect_vof_tvd: one conservative
// update from the four face fluxes of C^n, clamped; ghost cells copy Cin.
__global__ void k_tvd_advect(VofArgs a, int lim, const double* __restrict__ Cin, double* __restrict__ Cout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.D.nx, ny = a.D.ny, P = a.D.P;
  if (i > nx + 1 || j > ny + 1) return;
  const int k = a.D.id(i, j);
  if (i < 1 || i > nx || j < 1 || j > ny) { Cout[k] = Cin[k]; return; }
  if (a.D.nbhd(k, 20) != k) return;  // checked builds: a neighbourhood outside the array
  const double fw = tvd_face_flux(lim, a.u[k], a.dt, a.dx, Cin, k, 1, i, nx + 1);
  const double fe = tvd_face_flux(lim, a.u[k + 1], a.dt, a.dx, Cin, k + 1, 1, i + 1, nx + 1);
  const double fs = tvd_face_flux(lim, a.v[k], a.dt, a.dy, Cin, k, P, j, ny + 1);
  const double fn = tvd_face_flux(lim, a.v[k + P], a.dt, a.dy, Cin, k + P, P, j + 1, ny + 1);
  const double c = Cin[k] - (a.dt / a.dx) * (fe - fw) - (a.dt / a.dy) * (fn - fs);
  Cout[k] = fmax(0.0, fmin(1.0, c));
}

// exchange_halos_scalar then apply_vof_bc on a periodic domain (np = 1,
// src/module_mpi_comm.f90:25-56, 636-683), one block: the wrap in x (rows
// 0..ny+1), then in y (columns 0..nx+1), then the apply_vof_bc edges
// (periodic rows / columns 1..n again, zero gradient on the other
// direction's sides).  halo = 0: apply_vof_bc alone.
__global__ void k_vof_halo_bc(Dims D, double* __restrict__ C, int halo) {
  const int nx = D.nx, ny = D.ny;
  if (halo && D.perx)
    for (int j = (int)threadIdx.x; j <= ny + 1; j += blockDim.x) {
      C[D.id(0, j)] = C[D.id(nx, j)];
      C[D.id(nx + 1, j)] = C[D.id(1, j)];
    }
  __syncthreads();
  if (halo && D.pery)
    for (int i = (int)threadIdx.x; i <= nx + 1; i += blockDim.x) {
      C[D.id(i, 0)] = C[D.id(i, ny)];
      C[D.id(i, ny + 1)] = C[D.id(i, 1)];
    }
  __syncthreads();
  for (int j = 1 + (int)threadIdx.x; j <= ny; j += blockDim.x) {
    C[D.id(0, j)] = C[D.id(D.perx ? nx : 1, j)];
    C[D.id(nx + 1, j)] = C[D.id(D.perx ? 1 : nx, j)];
  }
  for (int i = 1 + (int)threadIdx.x; i <= nx; i += blockDim.x) {
    C[D.id(i, 0)] = C[D.id(i, D.pery ? ny : 1)];
    C[D.id(i, ny + 1)] = C[D.id(i, D.pery ? 1 : ny)];
  }
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
  // C's corners are rewritten at physical corners only (:532-535); mu's
  // corners always equal the interior corner's (:553-556)
  double cv = a.C[k], cm = cv;
  if (corner) {
    const int ki = a.D.id(i == 0 ? 1 : nx, j == 0 ? 1 : ny);
    cm = a.C[ki];
    if (!a.D.perx && !a.D.pery) {
      cv = cm;
      a.C[k] = cv;
    }
  }
  // SVOF: the properties follow the smoothed indicator (:541-545)
  const double c = fmax(0.0, fmin(1.0, a.Cs ? a.Cs[k] : cv));
  const double c_mu = fmax(0.0, fmin(1.0, a.Cs ? a.Cs[k] : cm));
  a.rho[k] = c * a.rho1 + (1.0 - c) * a.rho2;
  a.mu[k] = c_mu * a.mu1 + (1.0 - c_mu) * a.mu2;
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
  if (a.Cs) {
    // SVOF (:596-601): harmonic blend at the node of the smoothed indicator
    double cn = 0.25 * (a.Cs[k - a.D.P - 1] + a.Cs[k - a.D.P] + a.Cs[k - 1] + a.Cs[k]);
    cn = fmax(0.0, fmin(1.0, cn));
    const double denom = a.mu2 * cn + a.mu1 * (1.0 - cn);
    a.mu_node[k] = (a.mu1 * a.mu2) / fmax(1.0e-30, denom);
    return;
  }
  const double sw = a.mu[k - a.D.P - 1], se = a.mu[k - a.D.P];
  const double nw = a.mu[k - 1], ne = a.mu[k];
  a.mu_node[k] = 4.0 / (1.0 / sw + 1.0 / se + 1.0 / nw + 1.0 / ne);
}

// src/module_interface_vof.f90:663-686: unit normal of the gradient of C
// (or of C_s / C_tilde with smoothing) at interior cells.
__global__ void k_csf_normals(CsfArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > a.D.nx || j > a.D.ny) return;
  const int k = a.D.id(i, j);
  if (a.D.nbhd(k, 21) != k) return;  // checked builds
  const double dcx = (a.N[k + 1] - a.N[k - 1]) / (2.0 * a.dx);
  const double dcy = (a.N[k + a.D.P] - a.N[k - a.D.P]) / (2.0 * a.dy);
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
  if (a.D.nbhd(k, 21) != k) return;  // checked builds
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

COVOF_UNIT_HOOKS(vof)
