// poisson.cu -- variable-density pressure Poisson of the STANDARD_PROJECTION
// step on one GB300.
//
// Operator (src/module_simulation.f90:2483-2533, 2668-2707):
//   (A x)_ij = aP x_ij - aW x_i-1 - aE x_i+1 - aS x_j-1 - aN x_j+1,
//   aW(i) = aE(i-1) = dt*dy/(rho_u*dx) on the shared u-face (0 on walls),
//   aP = aW + aE + aS + aN + 1e-12*dvol.
// Storage: one coefficient per face (ax: west face of cell i, ay: south face
// of cell j) plus aP, all in the (0:nx+1, 0:ny+1) layout; vectors keep a
// zero ghost ring so the stencil needs no boundary branches (a wall face
// has a zero coefficient; an outflow face multiplies a zero ghost, which is
// what the reference's skipped term means).
//
// Solver: one cooperative persistent kernel per solve runs every PCG
// iteration with device-side convergence tests; blocks meet at a bounded
// grid barrier, dot products are warp-shuffle + block partials + one fixed
// order FP64 combine (deterministic).  The mixed path runs FP32 PCG inner
// solves (FP32 coefficients and vectors, FP32 partial sums, FP64 combine)
// inside FP64 iterative refinement on the true FP64 residual.
#include "common.cuh"
#include "poisson.cuh"

namespace covof {

// ---------------------------------------------------------------------------
// Assembly.  One thread per interior cell; writes ax(i,j), ay(i,j), aP(i,j),
// b(i,j), plus the east column ax(nx+1,j) and north row ay(i,ny+1).
__global__ void k_poisson_assemble(Dims D, double dt, double dx, double dy, int4 wall,
                                   const double* __restrict__ rho_u,
                                   const double* __restrict__ rho_v,
                                   const double* __restrict__ u, const double* __restrict__ v,
                                   const double* __restrict__ b_in, int pinned,
                                   double* __restrict__ ax, double* __restrict__ ay,
                                   double* __restrict__ aP, double* __restrict__ b,
                                   double* __restrict__ isd, double* __restrict__ invD) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > D.nx || j > D.ny) return;
  const int k = D.id(i, j);
  const double dvol = __dmul_rn(dx, dy);
  const double cx = __dmul_rn(dt, dy), cy = __dmul_rn(dt, dx);
  double aW = 0.0, aE = 0.0, aS = 0.0, aN = 0.0;
  if (!(i == 1 && wall.x)) {
    double r = rho_u[k]; if (r < 1.0e-12) r = 1.0;
    aW = __ddiv_rn(cx, __dmul_rn(r, dx));
  }
  if (!(i == D.nx && wall.y)) {
    double r = rho_u[k + 1]; if (r < 1.0e-12) r = 1.0;
    aE = __ddiv_rn(cx, __dmul_rn(r, dx));
  }
  if (!(j == 1 && wall.z)) {
    double r = rho_v[k]; if (r < 1.0e-12) r = 1.0;
    aS = __ddiv_rn(cy, __dmul_rn(r, dy));
  }
  if (!(j == D.ny && wall.w)) {
    double r = rho_v[k + D.P]; if (r < 1.0e-12) r = 1.0;
    aN = __ddiv_rn(cy, __dmul_rn(r, dy));
  }
  double ap = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(aW, aE), aS), aN), __dmul_rn(1.0e-12, dvol));
  ax[k] = aW; ay[k] = aS; aP[k] = ap;
  if (i == D.nx) ax[k + 1] = aE;
  if (j == D.ny) ay[k + D.P] = aN;
  double bb;
  if (b_in) {
    bb = b_in[k];
  } else {
    // b = -[(u_{i+1}-u_i) dy + (v_{j+1}-v_j) dx]  (src/module_simulation.f90:2484-2487)
    double div = __dadd_rn(__dmul_rn(__dsub_rn(u[k + 1], u[k]), dy),
                           __dmul_rn(__dsub_rn(v[k + D.P], v[k]), dx));
    bb = -div;
  }
  if (pinned && i == 1 && j == 1) bb = 0.0;
  b[k] = bb;
  if (isd) isd[k] = 1.0 / sqrt(ap);
  if (invD) invD[k] = 1.0 / ap;
}

// FP32 copy of the symmetrically scaled operator D^-1/2 A D^-1/2 (unit
// diagonal) for the mixed path: a face coefficient becomes
// a_f / sqrt(aP_left aP_right).  Ghost entries of isd are zero, so an
// outflow face (which only multiplies a zero ghost) gets a zero coefficient.
__global__ void k_poisson_scale32(Dims D, const double* __restrict__ ax, const double* __restrict__ ay,
                                  const double* __restrict__ isd, float* __restrict__ ax32,
                                  float* __restrict__ ay32, float* __restrict__ aP32) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > D.nx + 1 || j > D.ny + 1) return;
  const int k = D.id(i, j);
  if (j <= D.ny) ax32[k] = (float)(ax[k] * isd[k - 1] * (i <= D.nx ? isd[k] : 0.0));
  if (i <= D.nx) ay32[k] = (float)(ay[k] * isd[k - D.P] * (j <= D.ny ? isd[k] : 0.0));
  if (i <= D.nx && j <= D.ny) aP32[k] = 1.0f;
}

// Interior copy between a caller field and a solver vector (ghosts of dst untouched).
__global__ void k_copy_interior(Dims D, const double* __restrict__ src, double* __restrict__ dst,
                                int zero_pin) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > D.nx || j > D.ny) return;
  int k = D.id(i, j);
  dst[k] = (zero_pin && i == 1 && j == 1) ? 0.0 : src[k];
}

// ---------------------------------------------------------------------------
// Exact operator (reference term order, no contraction): used by the
// operator-apply entry point, whose result is compared bit for bit.
__device__ __forceinline__ double stencil_exact(const Dims& D, int k, const double* __restrict__ x,
                                                const double* __restrict__ ax,
                                                const double* __restrict__ ay,
                                                const double* __restrict__ aP) {
  double val = __dmul_rn(aP[k], x[k]);
  val = __dsub_rn(val, __dmul_rn(ax[k], x[k - 1]));
  val = __dsub_rn(val, __dmul_rn(ax[k + 1], x[k + 1]));
  val = __dsub_rn(val, __dmul_rn(ay[k], x[k - D.P]));
  val = __dsub_rn(val, __dmul_rn(ay[k + D.P], x[k + D.P]));
  return val;
}

__device__ __forceinline__ double fmad_(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fmad_(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// ---------------------------------------------------------------------------
// Tiled persistent PCG.  The interior is cut into TX x TY tiles (TX*TY =
// 1024 = blockDim.x, one cell per thread); tile t belongs to block t % G for
// the whole solve, so a cell is read and written by the same thread in every
// phase.  Vectors written by other blocks (r, the old direction) are read
// through L2 (__ldcg) after a grid barrier, into a shared-memory halo tile.
//
// One iteration = 2 grid barriers:
//   phase S: d_new = z + beta d_old on the tile and its halo (from r, d_old),
//            Ad = A d_new on the tile; write d_new, Ad; partial <d,Ad>
//   phase U: alpha; x += alpha d; r -= alpha Ad; partials <r,r>, <r,z>
// d is double-buffered (phase S of iteration k writes buffer k&1 and reads
// buffer (k+1)&1), so no block overwrites a direction another block reads.
__host__ __device__ Tiles make_tiles(const Dims& D) {
  Tiles t;
  t.TX = D.nx <= 32 ? 32 : (D.nx <= 64 ? 64 : 128);
  t.TY = 1024 / t.TX;
  t.ntx = (D.nx + t.TX - 1) / t.TX;
  t.nty = (D.ny + t.TY - 1) / t.TY;
  t.ntiles = t.ntx * t.nty;
  return t;
}

constexpr int kHalo = 130 * 10;  // max (TX+2)*(TY+2) over TX in {32, 64, 128}

template <typename T>
struct Sys {
  T* x; const T* b; T* r; T* d0; T* d1; T* Ad;
  const T* ax; const T* ay; const T* aP; const T* invD;  // aP, invD unused when unit diagonal
};

template <typename T, bool UNIT>
__device__ __forceinline__ T precond(const Sys<T>& S, int k, T rv) {
  return UNIT ? rv : rv * S.invD[k];
}

// Grid reduction of NV values: each thread accumulates its own cells in T
// (FP32 on the mixed path), the block and grid combines run in FP64.
template <typename T, int NV>
__device__ __forceinline__ bool reduce(GridReducer& R, T (&acc)[NV], double (&out)[NV]) {
  double v[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = (double)acc[q];
  bool ok = R.sum(v);
#pragma unroll
  for (int q = 0; q < NV; ++q) out[q] = v[q];
  return ok;
}

// Phase S on one tile.  Returns this thread's <d,Ad> contribution.
template <typename T, bool UNIT>
__device__ __forceinline__ T phase_stencil(const Dims& D, const Tiles& tl, int tile, const Sys<T>& S,
                                           const T* __restrict__ dold, T* __restrict__ dnew, T beta,
                                           bool first, int pinned_k, T* sd) {
  const int tx0 = (tile % tl.ntx) * tl.TX, ty0 = (tile / tl.ntx) * tl.TY;  // 0-based interior origin
  const int HX = tl.TX + 2, HY = tl.TY + 2;
  // d_new on tile + halo into shared memory (zero outside the ghost ring)
  for (int e = threadIdx.x; e < HX * HY; e += blockDim.x) {
    const int lx = e % HX, ly = e / HX;
    const int i = tx0 + lx, j = ty0 + ly;  // global index incl. ghost (i = 0 .. nx+1)
    T v = T(0);
    if (i <= D.nx + 1 && j <= D.ny + 1) {
      const int k = D.id(i, j);
      const bool interior = i >= 1 && i <= D.nx && j >= 1 && j <= D.ny;
      if (interior && k != pinned_k) {
        const T z = precond<T, UNIT>(S, k, __ldcg(S.r + k));
        v = first ? z : fmad_(beta, __ldcg(dold + k), z);
      }
    }
    sd[e] = v;
  }
  __syncthreads();
  const int lx = threadIdx.x % tl.TX, ly = threadIdx.x / tl.TX;
  const int i = tx0 + lx + 1, j = ty0 + ly + 1;
  T contrib = T(0);
  if (i <= D.nx && j <= D.ny) {
    const int k = D.id(i, j);
    const int c = (ly + 1) * HX + (lx + 1);
    const T dc = sd[c];
    T v = UNIT ? dc : S.aP[k] * dc;
    v = fmad_(-S.ax[k], sd[c - 1], v);
    v = fmad_(-S.ax[k + 1], sd[c + 1], v);
    v = fmad_(-S.ay[k], sd[c - HX], v);
    v = fmad_(-S.ay[k + D.P], sd[c + HX], v);
    if (k == pinned_k) v = T(0);
    dnew[k] = dc;
    S.Ad[k] = v;
    contrib = dc * v;
  }
  __syncthreads();
  return contrib;
}

struct PcgOut {
  int iters, status;
  double r_norm, b_norm;
  bool ok;
};

// Jacobi-PCG on S.x (in/out).  x_zero: S.x is known to be zero (skip A x).
template <typename T, bool UNIT>
__device__ PcgOut pcg_tiled(const Dims& D, const Tiles& tl, GridReducer& R, const Sys<T>& S,
                            int pinned, double rel, int max_iter, bool x_zero, T* sd) {
  const int pinned_k = pinned ? D.P + 1 : -1;
  PcgOut o{0, COVOF_OK, 0.0, 1.0, true};
  // r = b - A x ; <b,b>, <r,r>, <r,z>
  {
    T acc[3] = {T(0), T(0), T(0)};
    for (int tile = blockIdx.x; tile < tl.ntiles; tile += gridDim.x) {
      const int i = (tile % tl.ntx) * tl.TX + (int)(threadIdx.x % tl.TX) + 1;
      const int j = (tile / tl.ntx) * tl.TY + (int)(threadIdx.x / tl.TX) + 1;
      if (i <= D.nx && j <= D.ny) {
        const int k = D.id(i, j);
        T rv = S.b[k];
        if (!x_zero) {
          const T xc = __ldcg(S.x + k);
          T v = UNIT ? xc : S.aP[k] * xc;
          v = fmad_(-S.ax[k], __ldcg(S.x + k - 1), v);
          v = fmad_(-S.ax[k + 1], __ldcg(S.x + k + 1), v);
          v = fmad_(-S.ay[k], __ldcg(S.x + k - D.P), v);
          v = fmad_(-S.ay[k + D.P], __ldcg(S.x + k + D.P), v);
          rv = rv - v;
        }
        if (k == pinned_k) rv = T(0);
        S.r[k] = rv;
        const T z = (k == pinned_k) ? T(0) : precond<T, UNIT>(S, k, rv);
        acc[0] = fmad_(S.b[k], S.b[k], acc[0]);
        acc[1] = fmad_(rv, rv, acc[1]);
        acc[2] = fmad_(rv, z, acc[2]);
      }
    }
    double tot[3];
    o.ok = reduce<T, 3>(R, acc, tot);
    o.b_norm = sqrt(tot[0]);
    if (o.b_norm < 1.0e-30) o.b_norm = 1.0;
    o.r_norm = sqrt(tot[1]);
    if (!o.ok || !(o.r_norm / o.b_norm > rel)) {
      if (!o.ok) o.status = COVOF_TIMEOUT;
      return o;
    }
    double rz_old = tot[2];
    double beta = 0.0;
    bool converged = false;
    while (o.iters < max_iter) {
      const int it = o.iters;
      o.iters++;
      T* dnew = (it & 1) ? S.d1 : S.d0;
      const T* dold = (it & 1) ? S.d0 : S.d1;
      // phase S
      T a1[1] = {T(0)};
      for (int tile = blockIdx.x; tile < tl.ntiles; tile += gridDim.x)
        a1[0] += phase_stencil<T, UNIT>(D, tl, tile, S, dold, dnew, (T)beta, it == 0, pinned_k, sd);
      double dAd[1];
      if (!reduce<T, 1>(R, a1, dAd)) { o.ok = false; break; }
      if (fabs(dAd[0]) < 1.0e-35) { o.status = COVOF_BREAKDOWN; break; }
      const double alpha = rz_old / dAd[0];
      const T al = (T)alpha;
      // phase U
      T a2[2] = {T(0), T(0)};
      for (int tile = blockIdx.x; tile < tl.ntiles; tile += gridDim.x) {
        const int i = (tile % tl.ntx) * tl.TX + (int)(threadIdx.x % tl.TX) + 1;
        const int j = (tile / tl.ntx) * tl.TY + (int)(threadIdx.x / tl.TX) + 1;
        if (i <= D.nx && j <= D.ny) {
          const int k = D.id(i, j);
          S.x[k] = fmad_(al, dnew[k], S.x[k]);
          const T rv = fmad_(-al, S.Ad[k], S.r[k]);
          S.r[k] = rv;
          const T z = (k == pinned_k) ? T(0) : precond<T, UNIT>(S, k, rv);
          a2[0] = fmad_(rv, rv, a2[0]);
          a2[1] = fmad_(rv, z, a2[1]);
        }
      }
      double t2[2];
      if (!reduce<T, 2>(R, a2, t2)) { o.ok = false; break; }
      o.r_norm = sqrt(t2[0]);
      if (isnan(o.r_norm)) { o.status = COVOF_NAN; break; }
      if (o.r_norm / o.b_norm <= rel) { converged = true; break; }
      if (fabs(rz_old) < 1.0e-35) { o.status = COVOF_BREAKDOWN; break; }
      beta = t2[1] / rz_old;
      rz_old = t2[1];
    }
    if (o.ok && o.status == COVOF_OK && !converged) o.status = COVOF_MAXITER;
    if (!o.ok) o.status = COVOF_TIMEOUT;
  }
  return o;
}

// Mean removal (reference gauge, src/module_simulation.f90:2579-2582).
__device__ bool remove_mean(const Dims& D, const Tiles& tl, GridReducer& R, double* x) {
  double acc[1] = {0.0};
  for (int tile = blockIdx.x; tile < tl.ntiles; tile += gridDim.x) {
    const int i = (tile % tl.ntx) * tl.TX + (int)(threadIdx.x % tl.TX) + 1;
    const int j = (tile / tl.ntx) * tl.TY + (int)(threadIdx.x / tl.TX) + 1;
    if (i <= D.nx && j <= D.ny) acc[0] += x[D.id(i, j)];
  }
  double tot[1];
  if (!reduce<double, 1>(R, acc, tot)) return false;
  const double mean = tot[0] / (double)((long long)D.nx * D.ny);
  for (int tile = blockIdx.x; tile < tl.ntiles; tile += gridDim.x) {
    const int i = (tile % tl.ntx) * tl.TX + (int)(threadIdx.x % tl.TX) + 1;
    const int j = (tile / tl.ntx) * tl.TY + (int)(threadIdx.x / tl.TX) + 1;
    if (i <= D.nx && j <= D.ny) { const int k = D.id(i, j); x[k] = x[k] - mean; }
  }
  return true;
}

// Plain FP64 Jacobi-PCG solve.
__global__ void __launch_bounds__(1024, 1) k_pcg_fp64(PoissonArgs a) {
  __shared__ double sd[kHalo];
  const Dims D = a.D;
  const Tiles tl = make_tiles(D);
  GridReducer R{a.part, a.bar, a.err, gridDim.x, 0};
  Sys<double> S{a.x, a.b, a.r, a.d, a.d2, a.Ad, a.ax, a.ay, a.aP, a.invD};
  PcgOut o = pcg_tiled<double, false>(D, tl, R, S, a.pinned, a.tol, a.max_iter, false, sd);
  bool ok = o.ok;
  if (ok && !a.pinned) ok = remove_mean(D, tl, R, a.x);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.res->iters = o.iters;
    a.res->relres = o.r_norm / o.b_norm;
    a.res->status = ok ? o.status : COVOF_TIMEOUT;
    a.res->outer = 0;
  }
}

// Mixed: FP32 PCG inner solves on S A S (unit diagonal) inside FP64
// iterative refinement on the true FP64 residual.
__global__ void __launch_bounds__(1024, 1) k_pcg_mixed(PoissonArgs a) {
  __shared__ float sd[kHalo];
  const Dims D = a.D;
  const Tiles tl = make_tiles(D);
  GridReducer R{a.part, a.bar, a.err, gridDim.x, 0};
  const int pinned_k = a.pinned ? D.P + 1 : -1;
  Sys<float> S{a.e32, a.r32b, a.r32, a.d32, a.d32b, a.Ad32, a.ax32, a.ay32, nullptr, nullptr};
  bool ok = true;
  int total_inner = 0, outer = 0, status = COVOF_OK;
  double b_norm = 1.0, r_norm = 0.0;
  for (;;) {
    // FP64 residual r = b - A x (FMA form), ||b||, ||r||, sum(r), sum(aP)
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int tile = blockIdx.x; tile < tl.ntiles; tile += gridDim.x) {
      const int i = (tile % tl.ntx) * tl.TX + (int)(threadIdx.x % tl.TX) + 1;
      const int j = (tile / tl.ntx) * tl.TY + (int)(threadIdx.x / tl.TX) + 1;
      if (i <= D.nx && j <= D.ny) {
        const int k = D.id(i, j);
        double v = a.aP[k] * __ldcg(a.x + k);
        v = fma(-a.ax[k], __ldcg(a.x + k - 1), v);
        v = fma(-a.ax[k + 1], __ldcg(a.x + k + 1), v);
        v = fma(-a.ay[k], __ldcg(a.x + k - D.P), v);
        v = fma(-a.ay[k + D.P], __ldcg(a.x + k + D.P), v);
        double rr = a.b[k] - v;
        if (k == pinned_k) rr = 0.0;
        a.r[k] = rr;
        acc[0] = fma(a.b[k], a.b[k], acc[0]);
        acc[1] = fma(rr, rr, acc[1]);
        acc[2] += rr;
        acc[3] += a.aP[k];
      }
    }
    double tot[4];
    if (!reduce<double, 4>(R, acc, tot)) { ok = false; break; }
    b_norm = sqrt(tot[0]);
    if (b_norm < 1.0e-30) b_norm = 1.0;
    r_norm = sqrt(tot[1]);
    if (isnan(r_norm)) { status = COVOF_NAN; break; }
    if (r_norm / b_norm <= a.tol) break;
    if (outer >= a.max_refine || total_inner >= a.max_iter) { status = COVOF_MAXITER; break; }
    // Inner problem on the scaled operator S A S, S = D^-1/2 (unit diagonal,
    // O(1) entries, so FP32 rounding follows the Jacobi-scaled condition
    // number, not the density contrast):
    //   (S A S) y = S (r - c aP) / ||r||,   x += ||r|| S y.
    // Reference gauge: A is a Neumann operator plus a 1e-12*dvol shift FP32
    // cannot represent; c = sum(r)/sum(aP) removes the right-hand side's
    // (rounding-level) component along the scaled null vector S^-1 1.  The
    // outer test is always the true FP64 residual.
    const double cdef = a.pinned ? 0.0 : tot[2] / tot[3];
    const double scale = 1.0 / r_norm;
    for (int tile = blockIdx.x; tile < tl.ntiles; tile += gridDim.x) {
      const int i = (tile % tl.ntx) * tl.TX + (int)(threadIdx.x % tl.TX) + 1;
      const int j = (tile / tl.ntx) * tl.TY + (int)(threadIdx.x / tl.TX) + 1;
      if (i <= D.nx && j <= D.ny) {
        const int k = D.id(i, j);
        a.r32b[k] = (k == pinned_k) ? 0.0f : (float)((a.r[k] - cdef * a.aP[k]) * a.isd[k] * scale);
        a.e32[k] = 0.0f;
      }
    }
    // (pcg_tiled's first pass reads only own cells when x_zero)
    int budget = a.max_iter - total_inner;
    if (budget > a.inner_max_iter) budget = a.inner_max_iter;
    PcgOut o = pcg_tiled<float, true>(D, tl, R, S, a.pinned, a.inner_tol, budget, true, sd);
    total_inner += o.iters;
    outer++;
    if (!o.ok) { ok = false; break; }
    if (o.status == COVOF_NAN) { status = COVOF_NAN; break; }
    // x += ||r|| S y on own cells; the next residual pass reads neighbours'
    // x, hence the barrier.
    for (int tile = blockIdx.x; tile < tl.ntiles; tile += gridDim.x) {
      const int i = (tile % tl.ntx) * tl.TX + (int)(threadIdx.x % tl.TX) + 1;
      const int j = (tile / tl.ntx) * tl.TY + (int)(threadIdx.x / tl.TX) + 1;
      if (i <= D.nx && j <= D.ny) {
        const int k = D.id(i, j);
        a.x[k] = fma(r_norm * a.isd[k], (double)a.e32[k], a.x[k]);
      }
    }
    if (!grid_barrier(a.bar, gridDim.x, a.err)) { ok = false; break; }
    if (o.iters == 0) { status = COVOF_BREAKDOWN; break; }
  }
  if (ok && !a.pinned) ok = remove_mean(D, tl, R, a.x);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.res->iters = total_inner;
    a.res->relres = r_norm / b_norm;
    a.res->status = ok ? status : COVOF_TIMEOUT;
    a.res->outer = outer;
  }
}

// Velocity correction u -= dt/rho_u (p_e - p_w)/dx, v likewise
// (src/module_simulation.f90:2586-2654); wall faces untouched.
__global__ void k_project_correct(Dims D, double dt, double dx, double dy, int4 wall,
                                  double* __restrict__ u, double* __restrict__ v,
                                  const double* __restrict__ p, const double* __restrict__ rho_u,
                                  const double* __restrict__ rho_v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int nx = D.nx, ny = D.ny;
  if (i <= nx + 1 && j <= ny) {
    bool w = (i == 1 && wall.x) || (i == nx + 1 && wall.y);
    if (!w) {
      int k = D.id(i, j);
      double r = rho_u[k]; if (r < 1.0e-12) r = 1.0;
      double pw = (i > 1) ? p[k - 1] : p[D.id(1, j)];
      double pe = (i <= nx) ? p[k] : p[D.id(nx, j)];
      double g = __ddiv_rn(__dsub_rn(pe, pw), dx);
      u[k] = __dsub_rn(u[k], __dmul_rn(__ddiv_rn(dt, r), g));
    }
  }
  if (i <= nx && j <= ny + 1) {
    bool w = (j == 1 && wall.z) || (j == ny + 1 && wall.w);
    if (!w) {
      int k = D.id(i, j);
      double r = rho_v[k]; if (r < 1.0e-12) r = 1.0;
      double ps = (j > 1) ? p[k - D.P] : p[D.id(i, 1)];
      double pn = (j <= ny) ? p[k] : p[D.id(i, ny)];
      double g = __ddiv_rn(__dsub_rn(pn, ps), dy);
      v[k] = __dsub_rn(v[k], __dmul_rn(__ddiv_rn(dt, r), g));
    }
  }
}

// Standalone operator application for tests: y = A x (interior of y).
__global__ void k_poisson_apply(Dims D, const double* __restrict__ x, double* __restrict__ y,
                                const double* __restrict__ ax, const double* __restrict__ ay,
                                const double* __restrict__ aP) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > D.nx || j > D.ny) return;
  int k = D.id(i, j);
  y[k] = stencil_exact(D, k, x, ax, ay, aP);
}

}  // namespace covof
