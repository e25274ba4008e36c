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
                                   float* __restrict__ ax32, float* __restrict__ ay32,
                                   float* __restrict__ aP32) {
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
  if (ax32) {
    ax32[k] = (float)aW; ay32[k] = (float)aS; aP32[k] = (float)ap;
    if (i == D.nx) ax32[k + 1] = (float)aE;
    if (j == D.ny) ay32[k + D.P] = (float)aN;
  }
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
// Arithmetic helpers with explicit rounding (no contraction), per type.
template <typename T> struct Ar;
template <> struct Ar<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};
template <> struct Ar<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};

// y = A x at (i,j), reference term order.  x is read through L2 (__ldcg):
// other blocks wrote it earlier in this kernel.
template <typename T>
__device__ __forceinline__ T stencil(const Dims& D, int k, const T* __restrict__ x,
                                     const T* __restrict__ ax, const T* __restrict__ ay,
                                     const T* __restrict__ aP) {
  using A = Ar<T>;
  T val = A::mul(aP[k], __ldcg(x + k));
  val = A::sub(val, A::mul(ax[k], __ldcg(x + k - 1)));
  val = A::sub(val, A::mul(ax[k + 1], __ldcg(x + k + 1)));
  val = A::sub(val, A::mul(ay[k], __ldcg(x + k - D.P)));
  val = A::sub(val, A::mul(ay[k + D.P], __ldcg(x + k + D.P)));
  return val;
}

// Static cell ownership: warp w of the grid walks 32-wide row segments
// s = w, w + nwarps, ...; a thread owns the same cells in every phase.
struct Walker {
  int nsx, nseg, gw, nw, lane;
  __device__ Walker(const Dims& D) {
    nsx = (D.nx + 31) >> 5;
    nseg = nsx * D.ny;
    lane = threadIdx.x & 31;
    gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    nw = (gridDim.x * blockDim.x) >> 5;
  }
};
#define FOR_OWNED_CELLS(D, W, i, j, k)                                   \
  for (int s_ = (W).gw; s_ < (W).nseg; s_ += (W).nw)                      \
    for (int j = s_ / (W).nsx + 1, i = (s_ - (j - 1) * (W).nsx) * 32 + (W).lane + 1, k = (D).id(i, j); \
         i <= (D).nx; i = (D).nx + 1)

struct Ctl {
  unsigned int* bar;
  int* err;
  double* part;  // nblocks * 4
  unsigned int nblocks;
};

// ---------------------------------------------------------------------------
// One PCG solve on (x, b) in precision T (Jacobi preconditioner z = r / aP).
// Returns the number of iterations; *rnorm_out / *bnorm_out are the final
// recursive residual norm and ||b||; *st_out the loop status.  `rel` is the
// stopping ratio on ||r||/||b||.  r, d, Ad are scratch vectors.
template <typename T>
__device__ int pcg_core(const Dims& D, const Ctl& C, const Walker& W, T* x, const T* b, T* r, T* d,
                        T* Ad, const T* ax, const T* ay, const T* aP, int pinned, double rel,
                        int max_iter, int* st_out, double* rnorm_out, double* bnorm_out,
                        bool* ok_out) {
  using A = Ar<T>;
  const int bid = blockIdx.x;
  bool ok = true;
  // r = b - A x ; partials <b,b>, <r,r>
  {
    T acc[2] = {T(0), T(0)};
    FOR_OWNED_CELLS(D, W, i, j, k) {
      T y = stencil<T>(D, k, x, ax, ay, aP);
      T rr = A::sub(b[k], y);
      if (pinned && k == D.P + 1) rr = T(0);
      r[k] = rr;
      acc[0] = A::add(acc[0], A::mul(b[k], b[k]));
      acc[1] = A::add(acc[1], A::mul(rr, rr));
    }
    block_sum<T, 2>(acc);
    if (threadIdx.x == 0) { C.part[bid * 4 + 0] = (double)acc[0]; C.part[bid * 4 + 1] = (double)acc[1]; }
  }
  ok = grid_barrier(C.bar, C.nblocks, C.err);
  double tot[4];
  {
    double t2[2];
    // combine with stride 4 layout
    __shared__ double sh2[2];
    if (threadIdx.x < 32) {
      double a0 = 0.0, a1 = 0.0;
      for (int q = threadIdx.x; q < (int)C.nblocks; q += 32) {
        a0 += __ldcg(C.part + q * 4 + 0);
        a1 += __ldcg(C.part + q * 4 + 1);
      }
      a0 = warp_sum(a0); a1 = warp_sum(a1);
      if (threadIdx.x == 0) { sh2[0] = a0; sh2[1] = a1; }
    }
    __syncthreads();
    t2[0] = sh2[0]; t2[1] = sh2[1];
    __syncthreads();
    tot[0] = t2[0]; tot[1] = t2[1];
  }
  double b_norm = sqrt(tot[0]);
  if (b_norm < 1.0e-30) b_norm = 1.0;
  double r_norm = sqrt(tot[1]);
  int iters = 0, status = COVOF_OK;
  if (ok && r_norm / b_norm > rel) {
    // d = z = r / aP ; <r,z>
    T acc[1] = {T(0)};
    FOR_OWNED_CELLS(D, W, i, j, k) {
      T z = A::div(r[k], aP[k]);
      if (pinned && k == D.P + 1) z = T(0);
      d[k] = z;
      acc[0] = A::add(acc[0], A::mul(r[k], z));
    }
    block_sum<T, 1>(acc);
    // reuse slot 2 so the previous slots stay readable until everyone passed
    if (threadIdx.x == 0) C.part[bid * 4 + 2] = (double)acc[0];
    ok = grid_barrier(C.bar, C.nblocks, C.err);
    double rz_old;
    {
      __shared__ double sh1;
      if (threadIdx.x < 32) {
        double a0 = 0.0;
        for (int q = threadIdx.x; q < (int)C.nblocks; q += 32) a0 += __ldcg(C.part + q * 4 + 2);
        a0 = warp_sum(a0);
        if (threadIdx.x == 0) sh1 = a0;
      }
      __syncthreads();
      rz_old = sh1;
      __syncthreads();
    }
    bool converged = false;
    int slot = 0;  // alternate partial slots {0,1} / {2,3} between reductions
    while (ok && iters < max_iter) {
      iters++;
      // Ad = A d ; <d,Ad>
      {
        T acc1[1] = {T(0)};
        FOR_OWNED_CELLS(D, W, i, j, k) {
          T y = stencil<T>(D, k, d, ax, ay, aP);
          if (pinned && k == D.P + 1) y = T(0);
          Ad[k] = y;
          acc1[0] = A::add(acc1[0], A::mul(d[k], y));
        }
        block_sum<T, 1>(acc1);
        if (threadIdx.x == 0) C.part[bid * 4 + slot] = (double)acc1[0];
      }
      ok = grid_barrier(C.bar, C.nblocks, C.err);
      if (!ok) break;
      double dAd;
      {
        __shared__ double sh1;
        if (threadIdx.x < 32) {
          double a0 = 0.0;
          for (int q = threadIdx.x; q < (int)C.nblocks; q += 32) a0 += __ldcg(C.part + q * 4 + slot);
          a0 = warp_sum(a0);
          if (threadIdx.x == 0) sh1 = a0;
        }
        __syncthreads();
        dAd = sh1;
        __syncthreads();
      }
      slot ^= 2;
      if (fabs(dAd) < 1.0e-35) { status = COVOF_BREAKDOWN; break; }
      const double alpha = rz_old / dAd;
      const T al = (T)alpha;
      // x += alpha d ; r -= alpha Ad ; <r,r>, <r,z>
      {
        T acc2[2] = {T(0), T(0)};
        FOR_OWNED_CELLS(D, W, i, j, k) {
          T xv = A::add(x[k], A::mul(al, d[k]));
          T rv = A::sub(r[k], A::mul(al, Ad[k]));
          x[k] = xv; r[k] = rv;
          T z = A::div(rv, aP[k]);
          if (pinned && k == D.P + 1) z = T(0);
          acc2[0] = A::add(acc2[0], A::mul(rv, rv));
          acc2[1] = A::add(acc2[1], A::mul(rv, z));
        }
        block_sum<T, 2>(acc2);
        if (threadIdx.x == 0) { C.part[bid * 4 + slot] = (double)acc2[0]; C.part[bid * 4 + slot + 1] = (double)acc2[1]; }
      }
      ok = grid_barrier(C.bar, C.nblocks, C.err);
      if (!ok) break;
      double rr, rz_new;
      {
        __shared__ double sh2[2];
        if (threadIdx.x < 32) {
          double a0 = 0.0, a1 = 0.0;
          for (int q = threadIdx.x; q < (int)C.nblocks; q += 32) {
            a0 += __ldcg(C.part + q * 4 + slot);
            a1 += __ldcg(C.part + q * 4 + slot + 1);
          }
          a0 = warp_sum(a0); a1 = warp_sum(a1);
          if (threadIdx.x == 0) { sh2[0] = a0; sh2[1] = a1; }
        }
        __syncthreads();
        rr = sh2[0]; rz_new = sh2[1];
        __syncthreads();
      }
      slot ^= 2;
      r_norm = sqrt(rr);
      if (isnan(r_norm)) { status = COVOF_NAN; break; }
      if (r_norm / b_norm <= rel) { converged = true; break; }
      if (fabs(rz_old) < 1.0e-35) { status = COVOF_BREAKDOWN; break; }
      const double beta = rz_new / rz_old;
      rz_old = rz_new;
      const T be = (T)beta;
      // d = z + beta d
      FOR_OWNED_CELLS(D, W, i, j, k) {
        T z = A::div(r[k], aP[k]);
        if (pinned && k == D.P + 1) z = T(0);
        d[k] = A::add(z, A::mul(be, d[k]));
      }
      ok = grid_barrier(C.bar, C.nblocks, C.err);
    }
    if (ok && status == COVOF_OK && !converged) status = COVOF_MAXITER;
  }
  if (!ok) status = COVOF_TIMEOUT;
  *st_out = status;
  *rnorm_out = r_norm;
  *bnorm_out = b_norm;
  *ok_out = ok;
  return iters;
}

// Mean removal (reference gauge, src/module_simulation.f90:2579-2582).
__device__ bool remove_mean(const Dims& D, const Ctl& C, const Walker& W, double* x) {
  double acc[1] = {0.0};
  FOR_OWNED_CELLS(D, W, i, j, k) acc[0] += x[k];
  block_sum<double, 1>(acc);
  // A region of its own: the PCG loop may have exited right after a combine
  // that other blocks are still reading.
  double* mpart = C.part + 4 * C.nblocks;
  if (threadIdx.x == 0) mpart[blockIdx.x] = acc[0];
  bool ok = grid_barrier(C.bar, C.nblocks, C.err);
  if (!ok) return false;
  __shared__ double shm;
  if (threadIdx.x < 32) {
    double a0 = 0.0;
    for (int q = threadIdx.x; q < (int)C.nblocks; q += 32) a0 += __ldcg(mpart + q);
    a0 = warp_sum(a0);
    if (threadIdx.x == 0) shm = a0;
  }
  __syncthreads();
  const double mean = shm / (double)((long long)D.nx * D.ny);
  FOR_OWNED_CELLS(D, W, i, j, k) x[k] = x[k] - mean;
  return true;
}

// Plain FP64 PCG solve.
__global__ void __launch_bounds__(256) k_pcg_fp64(PoissonArgs a) {
  const Dims D = a.D;
  Ctl C{a.bar, a.err, a.part, gridDim.x};
  Walker W(D);
  int st; double rn, bn; bool ok;
  int it = pcg_core<double>(D, C, W, a.x, a.b, a.r, a.d, a.Ad, a.ax, a.ay, a.aP, a.pinned, a.tol,
                            a.max_iter, &st, &rn, &bn, &ok);
  if (ok && !a.pinned) ok = remove_mean(D, C, W, a.x);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.res->iters = it;
    a.res->relres = rn / bn;
    a.res->status = ok ? st : COVOF_TIMEOUT;
    a.res->outer = 0;
  }
}

// Mixed: FP32 PCG inner solves inside FP64 iterative refinement.
__global__ void __launch_bounds__(256) k_pcg_mixed(PoissonArgs a) {
  const Dims D = a.D;
  Ctl C{a.bar, a.err, a.part, gridDim.x};
  Walker W(D);
  const int bid = blockIdx.x;
  bool ok = true;
  int total_inner = 0, outer = 0, status = COVOF_OK;
  double b_norm = 1.0, r_norm = 0.0;
  for (;;) {
    // FP64 residual r = b - A x, ||b||, ||r||
    {
      double acc[2] = {0.0, 0.0};
      FOR_OWNED_CELLS(D, W, i, j, k) {
        double y = stencil<double>(D, k, a.x, a.ax, a.ay, a.aP);
        double rr = __dsub_rn(a.b[k], y);
        if (a.pinned && k == D.P + 1) rr = 0.0;
        a.r[k] = rr;
        acc[0] += a.b[k] * a.b[k];
        acc[1] += rr * rr;
      }
      block_sum<double, 2>(acc);
      if (threadIdx.x == 0) { a.part[bid * 4 + 0] = acc[0]; a.part[bid * 4 + 1] = acc[1]; }
    }
    ok = grid_barrier(a.bar, gridDim.x, a.err);
    if (!ok) break;
    {
      __shared__ double sh2[2];
      if (threadIdx.x < 32) {
        double a0 = 0.0, a1 = 0.0;
        for (int q = threadIdx.x; q < (int)gridDim.x; q += 32) {
          a0 += __ldcg(a.part + q * 4 + 0);
          a1 += __ldcg(a.part + q * 4 + 1);
        }
        a0 = warp_sum(a0); a1 = warp_sum(a1);
        if (threadIdx.x == 0) { sh2[0] = a0; sh2[1] = a1; }
      }
      __syncthreads();
      b_norm = sqrt(sh2[0]);
      r_norm = sqrt(sh2[1]);
      __syncthreads();
    }
    if (b_norm < 1.0e-30) b_norm = 1.0;
    if (isnan(r_norm)) { status = COVOF_NAN; break; }
    if (r_norm / b_norm <= a.tol) break;
    if (outer >= a.max_refine || total_inner >= a.max_iter) { status = COVOF_MAXITER; break; }
    // inner right-hand side r32 = r / ||r||, e = 0
    const double scale = 1.0 / r_norm;
    FOR_OWNED_CELLS(D, W, i, j, k) {
      a.r32b[k] = (float)(a.r[k] * scale);
      a.e32[k] = 0.0f;
    }
    // pcg_core starts with a residual pass that reads e through the stencil;
    // every block must have cleared its cells first.
    ok = grid_barrier(a.bar, gridDim.x, a.err);
    if (!ok) break;
    int st; double rn, bn; bool iok;
    int budget = a.max_iter - total_inner;
    if (budget > a.inner_max_iter) budget = a.inner_max_iter;
    int it = pcg_core<float>(D, C, W, a.e32, a.r32b, a.r32, a.d32, a.Ad32, a.ax32, a.ay32, a.aP32,
                             a.pinned, a.inner_tol, budget, &st, &rn, &bn, &iok);
    total_inner += it;
    outer++;
    if (!iok) { ok = false; break; }
    if (st == COVOF_NAN) { status = COVOF_NAN; break; }
    // x += ||r|| e  (own cells; the next residual pass reads x after a barrier)
    FOR_OWNED_CELLS(D, W, i, j, k) a.x[k] = __dadd_rn(a.x[k], __dmul_rn(r_norm, (double)a.e32[k]));
    ok = grid_barrier(a.bar, gridDim.x, a.err);
    if (!ok) break;
    if (it == 0) { status = COVOF_BREAKDOWN; break; }
  }
  if (ok && !a.pinned) ok = remove_mean(D, C, W, a.x);
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
  y[k] = stencil<double>(D, k, x, ax, ay, aP);
}

}  // namespace covof
