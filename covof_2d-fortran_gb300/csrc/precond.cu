// precond.cu -- the sequential preconditioners of the momentum / coupled
// Krylov solves: SSOR and BLOCK_TRIANGULAR (src/module_linear_solvers.f90:
// 137-278), built from lexicographic SSOR solves (:1278-1401).
//
// A lexicographic Gauss-Seidel sweep is a chain: cell (i, j) needs the new
// values of (i-1, j) and (i, j-1).  It runs as a wavefront (one warp per band
// of 32 rows, lane r on row r, lane r at column t - r on step t; the band
// below publishes its progress in chunks of 32 columns), so every cell sees
// the operands of the serial loop and the sweeps reproduce the reference's
// values bit for bit.  Independent solves (the u, v and pressure blocks of
// SSOR; u and v of BLOCK_TRIANGULAR) run side by side in one launch.
//
// The Krylov iterations that apply these preconditioners run from the host:
// the sweeps are launches of their own, each dot product a reduction read
// back (the same recurrences as the persistent kernels of momentum.cu, which
// serve the JACOBI / ILU0 / no-preconditioner cases).
#include "handle.cuh"
#include "precond.cuh"

namespace covof {

namespace {

constexpr int kSsorAhead = 4;

__device__ __forceinline__ bool nz(double a) { return (__double_as_longlong(a) << 1) != 0; }

struct SsorOps {
  double z, e, n, c, W, E, S, N, P, y;
};

// One sweep of band b of job J (forward when s is even).  Returns false when
// a wait gave up.  Prefetched operands are still old at prefetch time: the
// cell itself and the one ahead along its row are written later by this
// lane; the next row by lane r+1 one step after this lane; the neighbouring
// band's edge row only after this band publishes the chunk that holds it.
__device__ bool ssor_band(const SsorArgs& A, const SsorJob& J, int s, int b) {
  const Dims& D = A.D;
  const int P = D.P, ni = J.ni, nj = J.nj;
  const int lane = threadIdx.x & 31;
  const int nb = (nj + 31) >> 5;
  const unsigned int nch = (unsigned int)((ni + 31) >> 5);
  const unsigned int base = (unsigned int)s * nch;
  const bool fwd = (s & 1) == 0;
  const int j = fwd ? 32 * b + lane + 1 : 32 * b + 32 - lane;
  const bool valid = j <= nj;
  const int dep = fwd ? b - 1 : b + 1;
  const bool has_dep = fwd ? b > 0 : b < nb - 1;
  const int along = fwd ? 1 : -1;
  const int ahead_row = fwd ? P : -P;
  const bool edge_ahead_row = fwd ? (j == nj) : (j == 1);
  const bool edge_back_row = fwd ? (j == 1) : (j == nj);
  const double omega = J.omega, om1 = 1.0 - J.omega;
  auto fetch = [&](int t, SsorOps& o) {
    const int c = t - lane;
    o = SsorOps{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 1.0};
    if (valid && c >= 0 && c < ni) {
      const int i = fwd ? c + 1 : ni - c;
      const int k = D.id(i, j);
      const bool edge_along = fwd ? (i == ni) : (i == 1);
      o.z = __ldcg(J.z + k);
      o.c = __ldcg(J.r + k);
      if (!edge_along) o.e = __ldcg(J.r + k + along);
      if (!edge_ahead_row) o.n = __ldcg(J.r + k + ahead_row);
      o.W = __ldg(J.st.W + k); o.E = __ldg(J.st.E + k);
      o.S = __ldg(J.st.S + k); o.N = __ldg(J.st.N + k);
      o.P = __ldg(J.st.P + k); o.y = __ldg(J.st.rP + k);
    }
  };
  SsorOps ring[kSsorAhead];
#pragma unroll
  for (int q = 0; q < kSsorAhead; ++q) fetch(q, ring[q]);
  double prev = 0.0;
  // the neighbouring band's edge row for lane 0, one chunk at a time: lane q
  // holds column t0 + q, loaded together right after the chunk's wait, so
  // lane 0's step reads a register (a shuffle) instead of waiting on L2
  double edge = 0.0;
  const int j0 = fwd ? 32 * b + 1 : 32 * b + 32;  // lane 0's row
  const int T = ni + 31;
  for (int tt = 0; tt < T; tt += kSsorAhead) {
#pragma unroll
    for (int q = 0; q < kSsorAhead; ++q) {
      const int t = tt + q;
      if (t >= T) break;  // uniform across the warp
      if ((t & 31) == 0 && t < ni && has_dep) {
        if (!warp_wait_ge(J.prog + 32 * dep, base + (unsigned int)(t >> 5) + 1u, A.err)) return false;
        const int cq = t + lane;
        edge = 0.0;
        if (cq < ni) {
          const int iq = fwd ? cq + 1 : ni - cq;
          edge = __ldcg(J.r + D.id(iq, j0) - ahead_row);
        }
      }
      const double edge0 = __shfl_sync(0xffffffffu, edge, t & 31);
      const double across = __shfl_up_sync(0xffffffffu, prev, 1);
      const int c = t - lane;
      if (valid && c >= 0 && c < ni) {
        const SsorOps& o = ring[q];
        const int i = fwd ? c + 1 : ni - c;
        const int k = D.id(i, j);
        const bool edge_back = fwd ? (i == 1) : (i == ni);
        // across a domain edge the neighbour is a ghost entry, zero
        const double back = edge_back ? 0.0 : prev;
        const double back_row = edge_back_row ? 0.0 : (lane == 0 ? edge0 : across);
        double vW, vE, vS, vN;
        if (fwd) { vW = back; vE = o.e; vS = back_row; vN = o.n; }
        else     { vE = back; vW = o.e; vN = back_row; vS = o.n; }
        double v;
        if (J.kind == 0) {
          // "coefficient /= 0" tested on the bit patterns (integer pipe; +0
          // and -0 both read as zero), the FP64 pipe being the scarce one
          double val = o.z;
          if (nz(o.W)) val = val + o.W * vW;
          if (nz(o.E)) val = val + o.E * vE;
          if (nz(o.S)) val = val + o.S * vS;
          if (nz(o.N)) val = val + o.N * vN;
          // o.P is the centre as the sweeps read it (1 where |aP| < 1e-30)
          v = om1 * o.c + omega * div_rcp(val, o.P, o.y);
        } else {
          double val;
          if (fwd) {
            val = o.z;
            if (i > 1) val = val + o.W * vW;
            if (j > 1) val = val + o.S * vS;
          } else {
            val = o.P * o.c;
            if (i < ni) val = val + o.E * vE;
            if (j < nj) val = val + o.N * vN;
          }
          v = div_rcp(val, o.P, o.y);
          if (J.pin && i == 1 && j == 1) v = 0.0;
        }
        __stcg(J.r + k, v);
        prev = v;
      }
      fetch(t + kSsorAhead, ring[q]);
      const int c31 = t - 31;
      if (c31 >= 0 && ((c31 & 31) == 31 || c31 == ni - 1)) {
        __syncwarp();
        if (lane == 31) {
          __threadfence();
          st_release_u32(J.prog + 32 * b, base + (unsigned int)(c31 >> 5) + 1u);
        }
      }
    }
  }
  return true;
}

__device__ __forceinline__ int job_of(const SsorArgs& a, int g) {
  int q = 0;
  while (q + 1 < a.njob && g >= a.band0[q + 1]) ++q;
  return q;
}

}  // namespace

// Bands of all jobs are numbered consecutively; block x owns bands x,
// x + gridDim, ... and runs them in increasing order in forward sweeps and in
// decreasing order in backward ones, so every wait is on a band its owner
// reaches first (the launch is cooperative: every block is resident).
__global__ void __launch_bounds__(32) k_ssor(SsorArgs a) {
  const int total = a.band0[a.njob];
  if ((int)blockIdx.x >= total) return;
  int smax = 0;
  for (int q = 0; q < a.njob; ++q) smax = max(smax, 2 * a.job[q].sweeps);
  for (int s = 0; s < smax; ++s) {
    if ((s & 1) == 0) {
      for (int g = blockIdx.x; g < total; g += gridDim.x) {
        const int q = job_of(a, g);
        if (s < 2 * a.job[q].sweeps && !ssor_band(a, a.job[q], s, g - a.band0[q])) return;
      }
    } else {
      const int last = blockIdx.x + ((total - 1 - (int)blockIdx.x) / (int)gridDim.x) * (int)gridDim.x;
      for (int g = last; g >= 0; g -= gridDim.x) {
        const int q = job_of(a, g);
        if (s < 2 * a.job[q].sweeps && !ssor_band(a, a.job[q], s, g - a.band0[q])) return;
      }
    }
  }
}

namespace {

// Flat vector operations of the Krylov recurrences over whole packed vectors
// (ghost entries are zero in every operand and stay zero).
enum VecOp {
  kSub,       // y = x0 - x1
  kAxpy,      // y = y + c0 x0
  kXmby,      // y = x0 - c0 y
  kXpby,      // y = x0 + c0 y
  kBicgP,     // y = x0 + c0 (y - c1 x1)             (p = r + beta (p - omega v))
  kAxpy2,     // y = y + c0 x0 + c1 x1                (x += alpha p + omega s)
  kSubC,      // y = x0 - c0 x1                       (s = r - alpha v)
  kMul,       // y = x0 x1                            (Jacobi: src times the inverse diagonal)
  kCopy       // y = x0
};

// (an output may alias an input: every entry is read before it is written)
__global__ void k_vop(int op, size_t n, double* y, const double* x0, const double* x1, double c0, double c1) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    switch (op) {
      case kSub: y[q] = x0[q] - x1[q]; break;
      case kAxpy: y[q] = y[q] + c0 * x0[q]; break;
      case kXmby: y[q] = x0[q] - c0 * y[q]; break;
      case kXpby: y[q] = x0[q] + c0 * y[q]; break;
      case kBicgP: y[q] = x0[q] + c0 * (y[q] - c1 * x1[q]); break;
      case kAxpy2: y[q] = y[q] + c0 * x0[q] + c1 * x1[q]; break;
      case kSubC: y[q] = x0[q] - c0 * x1[q]; break;
      case kMul: y[q] = x0[q] * x1[q]; break;
      default: y[q] = x0[q]; break;
    }
  }
}

// BiCGSTAB(2)'s closing update (src/module_linear_solvers.f90:361-579):
// x += g1 r0 + g2 r1, r0 -= g1 r1 + g2 r2, u0 -= g1 u1 + g2 u2.
__global__ void k_bicg2_close(size_t n, double g1, double g2, double* __restrict__ x, double* __restrict__ r0,
                              const double* __restrict__ r1, const double* __restrict__ r2,
                              double* __restrict__ u0, const double* __restrict__ u1,
                              const double* __restrict__ u2) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const double a0 = r0[q], a1 = r1[q];
    x[q] = x[q] + g1 * a0 + g2 * a1;
    r0[q] = a0 - (g1 * a1 + g2 * r2[q]);
    u0[q] = u0[q] - (g1 * u1[q] + g2 * u2[q]);
  }
}

constexpr int kDotMax = 5;
constexpr int kDotThreads = 256;

struct DotSet {
  const double* x[kDotMax];
  const double* y[kDotMax];  // nullptr: the sum of x
  int np;
};

// Block partials of up to five dot products, grid-strided in a fixed order.
__global__ void __launch_bounds__(kDotThreads) k_dots(size_t n, DotSet d, double* __restrict__ part) {
  double acc[kDotMax] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int p = 0; p < kDotMax; ++p)
      if (p < d.np) acc[p] += d.y[p] ? d.x[p][q] * d.y[p][q] : d.x[p][q];
  }
  block_sum<double, kDotMax>(acc);
  if (threadIdx.x == 0)
    for (int p = 0; p < kDotMax; ++p) part[blockIdx.x * kDotMax + p] = acc[p];
}

// Totals from the block partials (one block, fixed order).
__global__ void __launch_bounds__(kDotThreads) k_dots_final(int nparts, const double* __restrict__ part,
                                                            double* __restrict__ out) {
  double acc[kDotMax] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nparts; b += blockDim.x)
#pragma unroll
    for (int p = 0; p < kDotMax; ++p) acc[p] += part[b * kDotMax + p];
  block_sum<double, kDotMax>(acc);
  if (threadIdx.x == 0)
    for (int p = 0; p < kDotMax; ++p) out[p] = acc[p];
}

// Zero the ghost ring of a field-layout array (so flat reductions over it
// see the cells only).
__global__ void k_zero_ghosts(Dims D, double* __restrict__ a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int W = D.nx + 2, H = D.ny + 2;
  if (t < W) { a[D.id(t, 0)] = 0.0; a[D.id(t, H - 1)] = 0.0; }
  if (t < H) { a[D.id(0, t)] = 0.0; a[D.id(W - 1, t)] = 0.0; }
}

// BLOCK_TRIANGULAR, after the Schur solve: r_p -= mean(r_p) over the cells
// (sum: the block's total, its ghost entries are zero).
__global__ void k_bt_center(Dims D, double* __restrict__ rp, const double* __restrict__ sum) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > D.nx || j > D.ny) return;
  const double mean = *sum / (double)((long long)D.nx * D.ny);
  const int k = D.id(i, j);
  rp[k] = rp[k] - mean;
}

// BLOCK_TRIANGULAR right-hand sides of the velocity solves: z - B^T r_p
// (src/module_linear_solvers.f90:202-246); wall DOFs keep z.
__global__ void k_bt_rhs(MomArgs a, const double* __restrict__ z, const double* __restrict__ rp,
                         double* __restrict__ h) {
  const Dims& D = a.D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int g = D.P * (D.ny + 2);
  if (i <= D.nx + 1 && j <= D.ny) {
    const int k = D.id(i, j);
    h[k] = (i == 1 || i == D.nx + 1) ? z[k] : z[k] - (rp[k] - rp[k - 1]) * a.dy;
  }
  if (i <= D.nx && j <= D.ny + 1) {
    const int k = D.id(i, j);
    const bool wall = (j == 1 && (a.bc[2] == COVOF_BC_DIRICHLET || a.bc[2] == COVOF_BC_FREESLIP)) ||
                      (j == D.ny + 1 && (a.bc[3] == COVOF_BC_DIRICHLET || a.bc[3] == COVOF_BC_FREESLIP));
    h[g + k] = wall ? z[g + k] : z[g + k] - (rp[k] - rp[k - D.P]) * a.dx;
  }
}

}  // namespace

namespace host {

bool uses_sweeps(const covof_params& P) {
  return P.use_precond && (P.precond == COVOF_PRECOND_SSOR || P.precond == COVOF_PRECOND_BLOCK_TRIANGULAR);
}

int ensure_sweeps(covof_handle* h) {
  SweepKit& K = h->sweep;
  if (K.ready) return COVOF_OK;
  const size_t g = h->g;
  const int nblk = h->prm.solver_type == COVOF_SOLVER_MONOLITHIC ? 3 : 2;
  K.n = (size_t)nblk * g;
  CS(dalloc(&K.coef, 18 * g));
  Stencil* st[3] = {&K.blk.u, &K.blk.v, &K.blk.s};
  for (int b = 0; b < 3; ++b) {
    double* c = K.coef + 6 * g * b;
    *st[b] = Stencil{c, c + g, c + 2 * g, c + 3 * g, c + 4 * g, c + 5 * g};
  }
  for (int q = 0; q < 3; ++q) CS(dalloc(&K.t[q], K.n));
  K.max_bands = (h->D.ny + 1 + 31) / 32;
  CS(dalloc(&K.prog, (size_t)kSsorMaxJobs * 32 * K.max_bands));
  int per_sm = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_ssor, 32, 0));
  K.cap = per_sm * h->sm_count;
  if (K.cap < 1) return COVOF_CUDA_ERROR;
  K.dot_blocks = 2 * h->sm_count;
  CS(dalloc(&K.part, (size_t)kDotMax * K.dot_blocks));
  CS(dalloc(&K.dsum, kDotMax));
  if (cudaMallocHost(&K.hdot, 8 * sizeof(double)) != cudaSuccess) return COVOF_CUDA_ERROR;
  K.ready = true;
  return COVOF_OK;
}

void sweep_free(covof_handle* h) {
  SweepKit& K = h->sweep;
  dfree(K.coef);
  for (int q = 0; q < 3; ++q) dfree(K.t[q]);
  dfree(K.prog); dfree(K.part); dfree(K.dsum);
  if (K.hdot) cudaFreeHost(K.hdot);
  K.hdot = nullptr;
  K.ready = false;
}

namespace {

int launch_ssor(covof_handle* h, SsorJob* jobs, int njob) {
  SweepKit& K = h->sweep;
  SsorArgs a;
  a.D = h->D;
  a.njob = njob;
  a.err = h->err;
  a.band0[0] = 0;
  for (int q = 0; q < njob; ++q) {
    a.job[q] = jobs[q];
    a.job[q].prog = K.prog + (size_t)q * 32 * K.max_bands;
    a.band0[q + 1] = a.band0[q] + (jobs[q].nj + 31) / 32;
  }
  CK(cudaMemsetAsync(K.prog, 0, (size_t)kSsorMaxJobs * 32 * K.max_bands * sizeof(unsigned int), h->stream));
  const int nb = a.band0[njob] < K.cap ? a.band0[njob] : K.cap;
  void* args[] = {&a};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nb);
  cfg.blockDim = dim3(32);
  cfg.stream = h->stream;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  CK(cudaLaunchKernelExC(&cfg, (const void*)k_ssor, args));
  return COVOF_OK;
}

SsorJob job(const Stencil& st, const double* z, double* r, int ni, int nj, int sweeps, double omega) {
  SsorJob j;
  j.st = st; j.z = z; j.r = r; j.ni = ni; j.nj = nj; j.sweeps = sweeps; j.omega = omega; j.prog = nullptr;
  j.kind = 0; j.pin = 0;
  return j;
}

}  // namespace

// dst = M^-1 src for SSOR / BLOCK_TRIANGULAR (src/module_linear_solvers.f90:
// 137-278); the stencils are the handle's (prec_blocks_dev).
int sweep_precond(covof_handle* h, const MomArgs& a, const double* src, double* dst) {
  SweepKit& K = h->sweep;
  const size_t g = h->g;
  const int nx = h->D.nx, ny = h->D.ny;
  const bool mono = a.mono != 0;
  const bool bt = h->prm.precond == COVOF_PRECOND_BLOCK_TRIANGULAR && mono;
  CK(cudaMemsetAsync(dst, 0, K.n * sizeof(double), h->stream));
  if (!bt) {
    SsorJob jobs[3] = {job(K.blk.u, src, dst, nx + 1, ny, 2, 1.0), job(K.blk.v, src + g, dst + g, nx, ny + 1, 2, 1.0),
                       job(K.blk.s, src + 2 * g, dst + 2 * g, nx, ny, 2, 1.0)};
    return launch_ssor(h, jobs, mono ? 3 : 2);
  }
  // Schur complement: 12 pairs, omega 1.25, then its mean removed
  SsorJob js = job(K.blk.s, src + 2 * g, dst + 2 * g, nx, ny, 12, 1.25);
  CS(launch_ssor(h, &js, 1));
  DotSet d{};
  d.x[0] = dst + 2 * g; d.y[0] = nullptr; d.np = 1;
  k_dots<<<K.dot_blocks, kDotThreads, 0, h->stream>>>(g, d, K.part);
  k_dots_final<<<1, kDotThreads, 0, h->stream>>>(K.dot_blocks, K.part, K.dsum);
  const dim3 blk(32, 8);
  const dim3 gc((nx + 31) / 32, (ny + 7) / 8), gf((nx + 1 + 31) / 32, (ny + 1 + 7) / 8);
  k_bt_center<<<gc, blk, 0, h->stream>>>(h->D, dst + 2 * g, K.dsum);
  double* hz = K.t[1];
  k_bt_rhs<<<gf, blk, 0, h->stream>>>(a, src, dst + 2 * g, hz);
  CK(cudaGetLastError());
  SsorJob jobs[2] = {job(K.blk.u, hz, dst, nx + 1, ny, 4, 1.0), job(K.blk.v, hz + g, dst + g, nx, ny + 1, 4, 1.0)};
  return launch_ssor(h, jobs, 2);
}

namespace {

// Up to five dot products over n flat entries (y = nullptr: the plain sum
// of x), read back to the host; also reads the kernels' error flag.
int read_dots(covof_handle* h, size_t n, std::initializer_list<std::pair<const double*, const double*>> prs,
              double* out) {
  SweepKit& K = h->sweep;
  DotSet d{};
  d.np = 0;
  for (auto& p : prs) { d.x[d.np] = p.first; d.y[d.np] = p.second; ++d.np; }
  k_dots<<<K.dot_blocks, kDotThreads, 0, h->stream>>>(n, d, K.part);
  k_dots_final<<<1, kDotThreads, 0, h->stream>>>(K.dot_blocks, K.part, K.dsum);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(K.hdot, K.dsum, kDotMax * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  int e = 0;
  CK(cudaMemcpyAsync(&e, h->err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CS(sync(h));
  if (e != 0) return COVOF_TIMEOUT;
  for (int p = 0; p < d.np; ++p) out[p] = K.hdot[p];
  return COVOF_OK;
}

// The host-driven Krylov state: the persistent kernels' vectors (a.x, a.v*)
// plus the handle's sweep scratch.
struct HostKrylov {
  covof_handle* h;
  const MomArgs& a;
  size_t n;
  int grid;
  int status_err = COVOF_OK;
  HostKrylov(covof_handle* hh, const MomArgs& aa) : h(hh), a(aa), n(hh->sweep.n) {
    grid = 4 * hh->sm_count;
  }
  void vop(int op, double* y, const double* x0, const double* x1 = nullptr, double c0 = 0.0, double c1 = 0.0) {
    k_vop<<<grid, 256, 0, h->stream>>>(op, n, y, x0, x1, c0, c1);
  }
  int A(const double* x, double* y) {
    k_mom_matvec<<<grid, 256, 0, h->stream>>>(a, x, y);
    CK(cudaGetLastError());
    return COVOF_OK;
  }
  int M(const double* src, double* dst) { return sweep_precond(h, a, src, dst); }
  int PA(const double* x, double* y) {
    CS(A(x, h->sweep.t[0]));
    return M(h->sweep.t[0], y);
  }
  // up to five dot products (y = nullptr: plain sum), read back; also reads
  // the kernels' error flag
  int dots(std::initializer_list<std::pair<const double*, const double*>> prs, double* out) {
    return read_dots(h, n, prs, out);
  }
};

// src/module_linear_solvers.f90:361-579 solve_bicgstab2 (left preconditioned)
int bicgstab2_host(HostKrylov& K, int* iters) {
  const MomArgs& a = K.a;
  double *x = a.x, *rt = a.v0, *r0 = a.v1, *r1 = a.v2, *r2 = a.v3, *u0 = a.v4, *u1 = a.v5, *u2 = a.v6;
  double* bh = K.h->sweep.t[2];
  const double tol = a.tol;
  const int max_iter = a.max_iter;
  *iters = 0;
  CS(K.M(a.rhs, bh));
  CS(K.PA(x, r0));
  K.vop(kSub, r0, bh, r0);
  for (double* v : {u0, u1, u2, r1, r2}) CK(cudaMemsetAsync(v, 0, K.n * sizeof(double), K.h->stream));
  double t[5];
  CS(K.dots({{r0, r0}}, t));
  const double r0n = sqrt(t[0]);
  if (r0n < 1.0e-12) return COVOF_OK;
  K.vop(kCopy, rt, r0);
  double rho0 = 1.0, alpha = 0.0, omega = 1.0;
  int iter = 0;
  int status = COVOF_MAXITER;
  while (iter < max_iter) {
    iter = iter + 2;
    rho0 = -omega * rho0;
    CS(K.dots({{rt, r0}}, t));
    double rho1 = t[0];
    if (fabs(rho0) < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    double beta = alpha * (rho1 / rho0);
    rho0 = rho1;
    K.vop(kXmby, u0, r0, nullptr, beta);
    CS(K.PA(u0, u1));
    CS(K.dots({{rt, u1}}, t));
    double gamma = t[0];
    if (fabs(gamma) < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    alpha = rho0 / gamma;
    K.vop(kAxpy, r0, u1, nullptr, -alpha);
    K.vop(kAxpy, x, u0, nullptr, alpha);
    CS(K.PA(r0, r1));
    CS(K.dots({{rt, r1}}, t));
    rho1 = t[0];
    if (fabs(rho0) < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    beta = alpha * (rho1 / rho0);
    rho0 = rho1;
    K.vop(kXmby, u0, r0, nullptr, beta);
    K.vop(kXmby, u1, r1, nullptr, beta);
    CS(K.PA(u1, u2));
    CS(K.dots({{rt, u2}}, t));
    gamma = t[0];
    if (fabs(gamma) < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    alpha = rho0 / gamma;
    K.vop(kAxpy, x, u0, nullptr, alpha);
    K.vop(kAxpy, r0, u1, nullptr, -alpha);
    K.vop(kAxpy, r1, u2, nullptr, -alpha);
    CS(K.PA(r1, r2));
    CS(K.dots({{r1, r1}, {r2, r1}, {r2, r2}, {r0, r1}, {r0, r2}}, t));
    const double s11 = t[0], s12 = t[1], s22 = t[2], rhs1 = t[3], rhs2 = t[4];
    const double rn1 = sqrt(s11), rn2 = sqrt(s22);
    double g1, g2;
    if (rn1 < 1.0e-300) { status = COVOF_BREAKDOWN; break; }
    else if (rn2 < 1.0e-300) { g2 = 0.0; g1 = rhs1 / s11; }
    else {
      const double i1 = 1.0 / rn1, i2 = 1.0 / rn2;
      const double c12 = s12 * i1 * i2;
      const double b1 = rhs1 * i1, b2 = rhs2 * i2;
      const double det = 1.0 - c12 * c12;
      if (fabs(det) < 1.0e-14) { g2 = 0.0; g1 = b1 * i1; }
      else { g1 = (b1 - c12 * b2) / (det * rn1); g2 = (b2 - c12 * b1) / (det * rn2); }
    }
    k_bicg2_close<<<K.grid, 256, 0, K.h->stream>>>(K.n, g1, g2, x, r0, r1, r2, u0, u1, u2);
    if (g2 != 0.0) omega = g2;
    else if (fabs(g1) > 1.0e-300) omega = g1;
    else omega = 1.0;
    CS(K.dots({{r0, r0}}, t));
    const double rn = sqrt(t[0]);
    if (rn != rn || rn > 1.0e30) { status = COVOF_NAN; break; }
    if (rn / r0n < tol || rn < 1.0e-12) { *iters = iter; return COVOF_OK; }
  }
  *iters = iter;
  return status;
}

// src/module_linear_solvers.f90:584-730 solve_bicgstab (left preconditioned)
int bicgstab_host(HostKrylov& K, int* iters) {
  const MomArgs& a = K.a;
  double *x = a.x, *bh = a.v0, *r = a.v1, *rt = a.v2, *p = a.v3, *v = a.v4, *s = a.v5, *tt = a.v6;
  const double tol = a.tol;
  const int max_iter = a.max_iter;
  *iters = max_iter;
  CS(K.M(a.rhs, bh));
  CS(K.PA(x, r));
  K.vop(kSub, r, bh, r);
  double t[5];
  CS(K.dots({{r, r}}, t));
  const double r0 = sqrt(t[0]);
  if (r0 < 1.0e-12) { *iters = 0; return COVOF_OK; }
  K.vop(kCopy, rt, r);
  double rho_old = 1.0, alpha = 1.0, omega = 1.0;
  for (int it = 1; it <= max_iter; ++it) {
    CS(K.dots({{rt, r}}, t));
    const double rho = t[0];
    if (fabs(rho) < 1.0e-30) return COVOF_BREAKDOWN;
    if (it == 1) K.vop(kCopy, p, r);
    else K.vop(kBicgP, p, r, v, (rho / rho_old) * (alpha / omega), omega);
    CS(K.PA(p, v));
    CS(K.dots({{rt, v}}, t));
    if (fabs(t[0]) < 1.0e-30) return COVOF_BREAKDOWN;
    alpha = rho / t[0];
    K.vop(kSubC, s, r, v, alpha);
    CS(K.dots({{s, s}}, t));
    const double sn = sqrt(t[0]);
    if (sn != sn || sn > 1.0e30) return COVOF_NAN;
    if (sn / r0 < tol || sn < 1.0e-12) {
      K.vop(kAxpy, x, p, nullptr, alpha);
      *iters = it;
      return COVOF_OK;
    }
    CS(K.PA(s, tt));
    CS(K.dots({{tt, tt}, {tt, s}}, t));
    omega = t[0] > 1.0e-30 ? t[1] / t[0] : 0.0;
    K.vop(kAxpy2, x, p, s, alpha, omega);
    K.vop(kSubC, r, s, tt, omega);
    rho_old = rho;
    CS(K.dots({{r, r}}, t));
    const double rn = sqrt(t[0]);
    if (rn != rn || rn > 1.0e30) return COVOF_NAN;
    if (rn / r0 < tol || rn < 1.0e-12) { *iters = it; return COVOF_OK; }
    if (fabs(omega) < 1.0e-30) return COVOF_BREAKDOWN;
  }
  return COVOF_MAXITER;
}

// src/module_linear_solvers.f90:735-838 solve_cg (operator unpreconditioned,
// the preconditioner applied to the residual)
int cg_host(HostKrylov& K, int* iters) {
  const MomArgs& a = K.a;
  double *x = a.x, *r = a.v1, *z = a.v2, *p = a.v3, *Ap = a.v4;
  const double tol = a.tol;
  const int max_iter = a.max_iter;
  *iters = max_iter;
  CS(K.A(x, Ap));
  K.vop(kSub, r, a.rhs, Ap);
  double t[5];
  CS(K.dots({{r, r}}, t));
  const double r0 = sqrt(t[0]);
  if (r0 < 1.0e-12) { *iters = 0; return COVOF_OK; }
  CS(K.M(r, z));
  K.vop(kCopy, p, z);
  CS(K.dots({{r, z}}, t));
  double rz_old = t[0];
  for (int it = 1; it <= max_iter; ++it) {
    CS(K.A(p, Ap));
    CS(K.dots({{p, Ap}}, t));
    if (fabs(t[0]) < 1.0e-30) return COVOF_BREAKDOWN;
    const double alpha = rz_old / t[0];
    K.vop(kAxpy, x, p, nullptr, alpha);
    K.vop(kAxpy, r, Ap, nullptr, -alpha);
    CS(K.dots({{r, r}}, t));
    const double rn = sqrt(t[0]);
    if (rn / r0 < tol || rn < 1.0e-13) { *iters = it; return COVOF_OK; }
    CS(K.M(r, z));
    CS(K.dots({{r, z}}, t));
    const double beta = t[0] / rz_old;
    rz_old = t[0];
    K.vop(kXpby, p, z, nullptr, beta);
  }
  return COVOF_MAXITER;
}

}  // namespace

// The stencils of the sweep preconditioners from a's fields (after
// k_mom_diag; the Schur stencil for MONOLITHIC).
int prec_blocks_dev(covof_handle* h, const MomArgs& a) {
  CS(ensure_sweeps(h));
  const dim3 blk(32, 8);
  const dim3 gf((h->D.nx + 1 + 31) / 32, (h->D.ny + 1 + 7) / 8), gc((h->D.nx + 31) / 32, (h->D.ny + 7) / 8);
  k_prec_blocks<<<gf, blk, 0, h->stream>>>(a, h->sweep.blk);
  if (a.mono) k_prec_schur<<<gc, blk, 0, h->stream>>>(a, h->sweep.blk);
  CK(cudaGetLastError());
  return COVOF_OK;
}

// dst = M^-1 src for the configured preconditioner, from a's fields after
// k_mom_diag / k_mono_diag / k_mom_assemble (the inverse Jacobi diagonal).
int precond_apply_dev(covof_handle* h, const MomArgs& a, const double* src, double* dst) {
  if (uses_sweeps(h->prm)) {
    CS(prec_blocks_dev(h, a));
    return sweep_precond(h, a, src, dst);
  }
  const size_t n = (a.mono ? 3 : 2) * h->g;
  k_vop<<<4 * h->sm_count, 256, 0, h->stream>>>(a.precond_on ? kMul : kCopy, n, dst, src, a.idiag, 0.0, 0.0);
  CK(cudaGetLastError());
  return COVOF_OK;
}

// The Krylov solve of a (assembled rows, packed right-hand side and start
// vector in place) with a sweep preconditioner, iterated from the host; the
// result record is written to the device like the persistent kernels'.
int sweep_solve(covof_handle* h, const MomArgs& a) {
  CK(cudaMemsetAsync(h->err, 0, sizeof(int), h->stream));
  HostKrylov K(h, a);
  int it = 0, st;
  switch (h->prm.linear_solver) {
    case COVOF_LINEAR_BICGSTAB: st = bicgstab_host(K, &it); break;
    case COVOF_LINEAR_CG: st = cg_host(K, &it); break;
    default: st = bicgstab2_host(K, &it); break;
  }
  if (st == COVOF_CUDA_ERROR || st == COVOF_TIMEOUT) return st;
  *h->h_kres = KrylovResult{it, st};
  CK(cudaMemcpyAsync(h->d_kres, h->h_kres, sizeof(KrylovResult), cudaMemcpyHostToDevice, h->stream));
  return sync(h);
}

// The pressure Poisson's PCG with the symmetric Gauss-Seidel preconditioner
// (p_precond SSOR; src/module_simulation.f90:2587-2758), FP64, iterated
// from the host around the wavefront sweep pair: the recurrences, stopping
// test and gauge handling of the Jacobi-PCG kernel (pinned cell held at
// zero; otherwise the mean removed at the end).  Writes the result record to
// the device.
int pcg_sgs(covof_handle* h, const PoissonArgs& a) {
  CS(ensure_sweeps(h));
  const Dims D = h->D;
  const size_t g = h->g;
  const int nx = D.nx, ny = D.ny;
  const int pin = a.pinned ? D.id(1, 1) : -1;
  double *x = a.x, *r = a.r, *z = a.z, *d = a.d, *Ad = a.Ad;
  const double* b = a.b;
  CK(cudaMemsetAsync(h->err, 0, sizeof(int), h->stream));
  const int zg = (nx + 2 > ny + 2 ? nx + 2 : ny + 2);
  k_zero_ghosts<<<(zg + 255) / 256, 256, 0, h->stream>>>(D, x);
  for (double* v : {r, z, d, Ad}) CK(cudaMemsetAsync(v, 0, g * sizeof(double), h->stream));
  const int grid = 4 * h->sm_count;
  const dim3 blk(32, 8), gc((nx + 31) / 32, (ny + 7) / 8);
  auto matvec = [&](const double* in, double* out) -> int {
    k_poisson_apply<<<gc, blk, 0, h->stream>>>(D, in, out, a.ax, a.ay, a.aP);
    if (pin >= 0) CK(cudaMemsetAsync(out + pin, 0, sizeof(double), h->stream));
    CK(cudaGetLastError());
    return COVOF_OK;
  };
  SsorJob J = job(Stencil{const_cast<double*>(a.ax), const_cast<double*>(a.ax) + 1, const_cast<double*>(a.ay),
                          const_cast<double*>(a.ay) + D.P, const_cast<double*>(a.aP), const_cast<double*>(a.invD)},
                  r, z, nx, ny, 1, 1.0);
  J.kind = 1;
  J.pin = a.pinned;
  auto vop = [&](int op, double* y, const double* x0, const double* x1, double c0) {
    k_vop<<<grid, 256, 0, h->stream>>>(op, g, y, x0, x1, c0, 0.0);
  };
  CS(matvec(x, Ad));
  vop(kSub, r, b, Ad, 0.0);
  double t[5];
  CS(read_dots(h, g, {{b, b}, {r, r}}, t));
  double b_norm = sqrt(t[0]);
  if (b_norm < 1.0e-30) b_norm = 1.0;
  double r_norm = sqrt(t[1]);
  int iters = 0, status = COVOF_OK;
  bool converged = false;
  if (r_norm != r_norm) {
    status = COVOF_NAN;  // a NaN in b or x
  } else if (r_norm / b_norm > a.tol) {
    CS(launch_ssor(h, &J, 1));
    vop(kCopy, d, z, nullptr, 0.0);
    CS(read_dots(h, g, {{r, z}}, t));
    double rz_old = t[0];
    for (int it = 1; it <= a.max_iter; ++it) {
      iters = iters + 1;
      CS(matvec(d, Ad));
      CS(read_dots(h, g, {{d, Ad}}, t));
      if (fabs(t[0]) < 1.0e-35) { status = COVOF_BREAKDOWN; break; }
      const double alpha = rz_old / t[0];
      vop(kAxpy, x, d, nullptr, alpha);
      vop(kAxpy, r, Ad, nullptr, -alpha);
      CS(read_dots(h, g, {{r, r}}, t));
      r_norm = sqrt(t[0]);
      if (r_norm != r_norm) { status = COVOF_NAN; break; }
      if (r_norm / b_norm <= a.tol) { converged = true; break; }
      CS(launch_ssor(h, &J, 1));
      CS(read_dots(h, g, {{r, z}}, t));
      if (fabs(rz_old) < 1.0e-35) { status = COVOF_BREAKDOWN; break; }
      const double beta = t[0] / rz_old;
      rz_old = t[0];
      vop(kXpby, d, z, nullptr, beta);
    }
    if (status == COVOF_OK && !converged) status = COVOF_MAXITER;
  }
  if (!a.pinned) {
    CS(read_dots(h, g, {{x, nullptr}}, t));
    CK(cudaMemcpyAsync(h->sweep.dsum, &t[0], sizeof(double), cudaMemcpyHostToDevice, h->stream));
    k_bt_center<<<gc, blk, 0, h->stream>>>(D, x, h->sweep.dsum);
    CK(cudaGetLastError());
  }
  *h->h_pres = PcgResult{iters, status, 0, 0, r_norm / b_norm};
  CK(cudaMemcpyAsync(h->d_pres, h->h_pres, sizeof(PcgResult), cudaMemcpyHostToDevice, h->stream));
  return sync(h);
}

}  // namespace host
}  // namespace covof

COVOF_UNIT_HOOKS(precond)
