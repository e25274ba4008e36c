// svof.cu -- interface smoothing on the device.
//
// SVOF (src/module_interface_vof.f90:387-476): 25 pairs of lexicographic
// Gauss-Seidel sweeps, forward then backward, of (I - D lap) C_s = C with
// homogeneous Neumann walls, then the clamp to [0, 1] and the ghost ring.  A
// Gauss-Seidel sweep is a chain: cell (i, j) needs the new values of (i-1, j)
// and (i, j-1) (forward).  Cells of one anti-diagonal are independent, so the
// sweep runs as a wavefront and every cell sees exactly the operands of the
// serial loop -- the result is the reference's bit for bit.
//
// Mapping: one warp per band of 32 rows, lane r on row r of the band; at step
// t lane r updates column t - r, so the new south value comes from lane r-1
// by a shuffle and the new west value is the lane's own previous result.  The
// band's bottom row reads the band below, which publishes its top row's
// progress in chunks of 32 columns (a release store of a per-band counter;
// the band above polls it with acquire loads, bounded).  Backward sweeps
// mirror everything (lane 0 on the top row, columns right to left, waiting on
// the band above).  A warp that owns several bands runs them lowest first in
// forward sweeps and highest first in backward ones, so every wait is on work
// that its owner reaches first; the launch is cooperative, so every warp is
// resident.  FP64 issue per SM is the scarce resource: one warp per block,
// one block per band, spread over the SMs.
//
// Diffusion smoothing (:1416-1461): explicit steps, one thread per cell,
// ping-pong buffers, ghost-aware reads.
#include "vof.cuh"

namespace covof {

namespace {

// One sweep of one band.  Forward: lane r on row 32 b + r + 1, columns left
// to right.  Backward: lane r on row 32 b + 32 - r, columns right to left.
// Returns false when a wait gave up.
//
// The operands that are still old when the step runs (C, the value along the
// sweep direction ahead, the value across in the row the sweep reaches next)
// are loaded kSvofAhead steps early into a register ring, so a step waits on
// the shuffle and the FP64 chain only, not on an L2 round trip.  They are
// still old at prefetch time: the lane's own row ahead is written by itself
// later; the next row's cell is written by lane r+1 one step after this
// lane's step; the neighbouring band's edge row is written only after this
// band publishes the chunk holding that column, which follows this lane's
// step.
constexpr int kSvofAhead = 8;

__device__ bool svof_band(const SvofArgs& a, int s, int b) {
  const Dims& D = a.D;
  const int nx = D.nx, ny = D.ny, P = D.P;
  const int lane = threadIdx.x & 31;
  const int nb = (ny + 31) >> 5;
  const unsigned int nch = (unsigned int)((nx + 31) >> 5);
  const unsigned int base = (unsigned int)s * nch;
  const bool fwd = (s & 1) == 0;
  const int j = fwd ? 32 * b + lane + 1 : 32 * b + 32 - lane;
  const bool valid = j <= ny;
  // the band whose edge row this band's lane 0 reads
  const int dep = fwd ? b - 1 : b + 1;
  const bool has_dep = fwd ? b > 0 : b < nb - 1;
  const double wx = a.wx, wy = a.wy;
  // neighbour offsets: along = ahead in the sweep direction (old),
  // ahead_row = the row the sweep reaches next (old), back_row = the row
  // already swept (new: shuffle, or the band edge for lane 0)
  const int along = fwd ? 1 : -1;
  const int ahead_row = fwd ? P : -P;
  const bool edge_ahead_row = fwd ? (j == ny) : (j == 1);
  const bool edge_back_row = fwd ? (j == 1) : (j == ny);
  // operands of step t: C, old along, old ahead-row
  auto fetch = [&](int t, double& xc, double& xa, double& xr) {
    const int c = t - lane;
    xc = 0.0; xa = 0.0; xr = 0.0;
    if (valid && c >= 0 && c < nx) {
      const int i = fwd ? c + 1 : nx - c;
      const int k = D.id(i, j);
      const bool edge_along = fwd ? (i == nx) : (i == 1);
      xc = __ldg(a.C + k);
      if (!edge_along) xa = __ldcg(a.Cs + k + along);
      if (!edge_ahead_row) xr = __ldcg(a.Cs + k + ahead_row);
    }
  };
  double rc[kSvofAhead], ra[kSvofAhead], rr[kSvofAhead];
#pragma unroll
  for (int q = 0; q < kSvofAhead; ++q) fetch(q, rc[q], ra[q], rr[q]);
  double prev = 0.0;  // this lane's value of the previous step
  // the neighbouring band's edge row for lane 0, one chunk at a time: lane q
  // holds column t0 + q, loaded together right after the chunk's wait, so
  // lane 0's step reads a register (a shuffle) instead of waiting on L2
  double edge = 0.0;
  const int j0 = fwd ? 32 * b + 1 : 32 * b + 32;  // lane 0's row
  const int T = nx + 31;
  for (int tt = 0; tt < T; tt += kSvofAhead) {
#pragma unroll
    for (int q = 0; q < kSvofAhead; ++q) {
      const int t = tt + q;
      if (t >= T) break;  // uniform across the warp
      // lane 0 starts a chunk of columns (t < nx: past the last column no
      // chunk is left to wait for)
      if ((t & 31) == 0 && t < nx && has_dep) {
        if (!warp_wait_ge(a.prog + 32 * dep, base + (unsigned int)(t >> 5) + 1u, a.err)) return false;
        const int cq = t + lane;
        edge = 0.0;
        if (cq < nx) {
          const int iq = fwd ? cq + 1 : nx - cq;
          edge = __ldcg(a.Cs + D.id(iq, j0) - ahead_row);
        }
      }
      const double edge0 = __shfl_sync(0xffffffffu, edge, t & 31);
      // lane r-1's previous value: the new neighbour across the band's rows
      const double across = __shfl_up_sync(0xffffffffu, prev, 1);
      const int c = t - lane;
      if (valid && c >= 0 && c < nx) {
        const int i = fwd ? c + 1 : nx - c;
        const int k = D.id(i, j);
        const bool edge_back = fwd ? (i == 1) : (i == nx);
        const double aE = (i == nx) ? 0.0 : wx;
        const double aW = (i == 1) ? 0.0 : wx;
        const double aN = (j == ny) ? 0.0 : wy;
        const double aS = (j == 1) ? 0.0 : wy;
        // 1 + aE + aW + aN + aS and its reciprocal, per wall pattern (host)
        const int wf = (i == nx ? 1 : 0) | (i == 1 ? 2 : 0) | (j == ny ? 4 : 0) | (j == 1 ? 8 : 0);
        const double aP = a.aP[wf], yP = a.rP[wf];
        // neighbours across a wall enter with a zero coefficient; they are
        // read as 0 (the reference multiplies its Neumann ghost copy by 0)
        const double back = edge_back ? 0.0 : prev;  // new, this lane's previous step
        const double back_row = edge_back_row ? 0.0 : (lane == 0 ? edge0 : across);  // new
        double vE, vW, vN, vS;
        if (fwd) { vE = ra[q]; vW = back; vN = rr[q]; vS = back_row; }
        else     { vW = ra[q]; vE = back; vS = rr[q]; vN = back_row; }
        const double sum = aE * vE + aW * vW + aN * vN + aS * vS;
        const double v = div_rcp(rc[q] + sum, aP, yP);
        __stcg(a.Cs + k, v);
        prev = v;
      }
      // refill this slot for step t + kSvofAhead
      fetch(t + kSvofAhead, rc[q], ra[q], rr[q]);
      // lane 31 (the band's edge row towards the waiting band) finished a
      // chunk of 32 columns: publish it
      const int c31 = t - 31;
      if (c31 >= 0 && ((c31 & 31) == 31 || c31 == nx - 1)) {
        __syncwarp();
        if (lane == 31) {
          __threadfence();
          st_release_u32(a.prog + 32 * b, base + (unsigned int)(c31 >> 5) + 1u);
        }
      }
    }
  }
  return true;
}

}  // namespace

__global__ void __launch_bounds__(32) k_svof_sgs(SvofArgs a) {
  const int nb = (a.D.ny + 31) >> 5;
  if ((int)blockIdx.x >= nb) return;  // the host launches at most nb blocks
  for (int s = 0; s < 2 * kSvofIters; ++s) {
    if ((s & 1) == 0) {
      for (int b = blockIdx.x; b < nb; b += gridDim.x)
        if (!svof_band(a, s, b)) return;
    } else {
      const int last = blockIdx.x + ((nb - 1 - (int)blockIdx.x) / (int)gridDim.x) * (int)gridDim.x;
      for (int b = last; b >= 0; b -= gridDim.x)
        if (!svof_band(a, s, b)) return;
    }
  }
}

// Clamp to [0, 1] and the Neumann ghost ring with its corners (:455-474).
__global__ void k_svof_finish(Dims D, double* __restrict__ Cs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = D.nx, ny = D.ny;
  if (i > nx + 1 || j > ny + 1) return;
  // ghost-ring entries copy their interior neighbour's clamped value
  // (corners: the diagonal interior cell); interior entries clamp in place.
  // A ghost may read its interior cell before or after that cell's own
  // clamp: the clamp is idempotent, so both give the same value.
  const int ii = i < 1 ? 1 : (i > nx ? nx : i);
  const int jj = j < 1 ? 1 : (j > ny ? ny : j);
  const double c = Cs[D.id(ii, jj)];
  Cs[D.id(i, j)] = fmax(0.0, fmin(1.0, c));
}

// One explicit diffusion step (:1445-1452): dst = src + dtau lap(src) on the
// interior, src's ghosts read as their Neumann copies (:1439-1442).
__global__ void k_diffusion_step(Dims D, double dtau, double dx2, double dy2, const double* __restrict__ src,
                                 double* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int nx = D.nx, ny = D.ny;
  if (i > nx || j > ny) return;
  const int k = D.id(i, j);
  const double c = src[k];
  const double e = src[D.id(i < nx ? i + 1 : nx, j)];
  const double w = src[D.id(i > 1 ? i - 1 : 1, j)];
  const double n = src[D.id(i, j < ny ? j + 1 : ny)];
  const double s = src[D.id(i, j > 1 ? j - 1 : 1)];
  const double lx = (e - 2.0 * c + w) / dx2;
  const double ly = (n - 2.0 * c + s) / dy2;
  dst[k] = c + dtau * (lx + ly);
}

// Final ghost ring of C_tilde (:1456-1459): west / east from the interior,
// then south / north rows including the corners.
__global__ void k_diffusion_ghosts(Dims D, double* __restrict__ Ct) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = D.nx, ny = D.ny;
  if (i > nx + 1 || j > ny + 1) return;
  if (i >= 1 && i <= nx && j >= 1 && j <= ny) return;
  const int ii = i < 1 ? 1 : (i > nx ? nx : i);
  const int jj = j < 1 ? 1 : (j > ny ? ny : j);
  Ct[D.id(i, j)] = Ct[D.id(ii, jj)];
}

}  // namespace covof

COVOF_UNIT_HOOKS(svof)
