// poisson.cuh -- argument blocks shared by poisson.cu and the C ABI layer.
#pragma once
#include "common.cuh"

namespace covof {

struct PcgResult {
  int iters;      // PCG iterations (mixed: total FP32 inner iterations)
  int status;     // COVOF_*
  int outer;      // mixed: FP64 refinement steps
  int pad;
  double relres;  // ||r||/||b|| at exit (mixed: true FP64 residual)
};

// Geometric multigrid hierarchy of the flexible CG's inner V-cycle (levels
// 1 .. nl-1; level 0 is the fine operator itself).  Level l owns 7 arrays of
// (nx+2)*(ny+2) elements at pool + off (elements of the V-cycle's arithmetic:
// float on the mixed path, double for COVOF_PREC_FP64_MG): two solution
// buffers, right-hand side, west / south face coefficients, diagonal, and
// omega / diagonal (the sweeps multiply instead of dividing); level 0's
// omega / diagonal is at pool + wd0_off.
constexpr int kMgMaxLevels = 16;
constexpr long long kMgTailSmem = 200 * 1024;  // cap on the shared-memory tail (plus ~6 KB static)
constexpr long long kMgWarpCoarse = 256;        // coarsest levels this small run in one warp
constexpr int kMgTailDepth = 6;                 // tail levels cycled with gamma > 1 (deeper ones: V)
constexpr long long kMgWCells = 512LL * 512;    // meshes from this size on run the tail as a W-cycle
struct MgLevel {
  int nx, ny;
  int fx, fy;  // coarsening factors from the next finer level (level 0: 1, 1)
  long long off;
};
struct MgHier {
  MgLevel lv[kMgMaxLevels];
  int nl;      // levels including level 0
  int tail;    // first level run by block 0 alone out of shared memory, nl if none
  void* pool;  // float or double elements, by the V-cycle's arithmetic
  long long wd0_off;  // level 0's omega / diagonal, (nx+2)*(ny+2) elements
  float omega; // Jacobi weight
  float cw;    // coarse-correction weight
  int nu, nuc; // sweeps before / after each coarse correction; sweeps on the coarsest level
  int gamma;   // coarse corrections per tail level (1: V-cycle, 2: W-cycle)
  int semi;    // some level is semi-coarsened (2 x 1 or 1 x 2 aggregates)
  int tail_smem;     // bytes of block 0's shared memory holding the tail levels
  // exact != 0: the coarsest level (at most 64 cells, in the tail) is solved
  // by a dense inverse formed once per solve, 64 x 64 elements at element
  // offset inv_off of the tail's shared memory, instead of nuc sweeps
  int exact, inv_off;
};

struct PoissonArgs {
  Dims D;
  // FP64 system
  double* x; const double* b; double* r; double* d; double* d2; double* Ad;
  const double* ax; const double* ay; const double* aP; const double* invD;
  const double* isd;  // 1/sqrt(aP) (mixed path scaling), zero ghost ring
  double* z; double* w; double* p; double* q;  // FP64 flexible-CG vectors (mixed)
  float* xb;  // boundary-row exchange of the shared-memory inner solvers
  unsigned int* flags;  // per-block publish counters (Chebyshev inner solver)
  double cheb_lo;
  // FP32 inner system (mixed)
  float* e32; float* r32b; float* r32; float* d32; float* d32b; float* Ad32;
  const float* ax32; const float* ay32; const float* aP32;
  MgHier mg;  // COVOF_INNER_MG
  // control
  unsigned int* bar; int* err; double* part;  // part: 16 * nblocks doubles
  PcgResult* res;
  const int* redo;  // non-null: the launch runs only if *redo != 0 (the pinned fallback)
  int bskip;        // cell left out of ||b|| (the pinned cell on the reference-gauge route), else -1
  double tol, inner_tol;
  int max_iter, inner_max_iter, max_refine, pinned;
};

__global__ void k_poisson_assemble(Dims D, double dt, double dx, double dy, int4 wall,
                                   const double* __restrict__ rho_u,
                                   const double* __restrict__ rho_v,
                                   const double* __restrict__ u, const double* __restrict__ v,
                                   const double* __restrict__ b_in, int pinned,
                                   double* __restrict__ ax, double* __restrict__ ay,
                                   double* __restrict__ aP, double* __restrict__ b,
                                   double* __restrict__ isd, double* __restrict__ invD);
__global__ void k_poisson_scale32(Dims D, const double* __restrict__ ax, const double* __restrict__ ay,
                                  const double* __restrict__ isd, float* __restrict__ ax32,
                                  float* __restrict__ ay32, float* __restrict__ aP32,
                                  const double* __restrict__ aP, int unscaled);
__global__ void k_copy_interior(Dims D, const double* __restrict__ src, double* __restrict__ dst,
                                int zero_pin);
__global__ void k_wrap_ghosts(Dims D, double* __restrict__ x);
struct Tiles {
  int TX, TY, ntx, nty, ntiles;
};
__host__ __device__ Tiles make_tiles(const Dims& D, int threads = 1024);
__global__ void k_pcg_fp64(PoissonArgs a);
// The pinned gauge through the reference gauge (mixed multigrid).  The
// pinned system (rows k != (1,1), x(1,1) = 0) and the reference-gauge one
// share the operator A, whose rows sum to e = A 1 (the 1e-12 dvol shift).
// With kappa = -mean(x0) of the initial guess, the right-hand side
// F_k = b_k + kappa e_k (k != (1,1)), F(1,1) = -sum of the others, is
// consistent, and if x0 solves the pinned system, x0 + kappa 1 solves this
// one; a reference-gauge solution x of F, shifted by -x(1,1), leaves the
// pinned residual (x(1,1) - kappa) e + (its own residual).  That residual is
// checked and the pinned solve rerun from the shifted x if the check fails;
// after a failure the next kPinRetry solves go to the pinned solve directly.
// ctl (ints): [0] rerun the pinned solve, [1] direct solves left, [2] the
// reference-gauge route runs in this solve.  lvl (doubles): [0] x(1,1),
// [1] kappa, [2] F(1,1).
constexpr int kPinBlocks = 256;
constexpr int kPinRetry = 8;
__global__ void k_pin_sum(Dims D, const double* __restrict__ b, const double* __restrict__ x,
                          const double* __restrict__ ax, const double* __restrict__ ay,
                          const double* __restrict__ aP, double* __restrict__ part, const int* __restrict__ ctl);
__global__ void k_pin_rhs(Dims D, const double* __restrict__ part, double* __restrict__ lvl, int* __restrict__ ctl);
__global__ void k_pin_form(Dims D, const double* __restrict__ b, const double* __restrict__ ax,
                           const double* __restrict__ ay, const double* __restrict__ aP, double* __restrict__ F,
                           const double* __restrict__ lvl, const int* __restrict__ ctl);
__global__ void k_pin_level(Dims D, const double* __restrict__ x, double* __restrict__ lvl, const int* __restrict__ ctl);
__global__ void k_pin_shift(Dims D, double* __restrict__ x, const double* __restrict__ lvl, const int* __restrict__ ctl);
__global__ void k_pin_resid(Dims D, const double* __restrict__ b, const double* __restrict__ x,
                            const double* __restrict__ ax, const double* __restrict__ ay,
                            const double* __restrict__ aP, double* __restrict__ part, const int* __restrict__ ctl);
__global__ void k_pin_final(Dims D, const double* __restrict__ part, double tol, PcgResult* res, int* ctl);
__global__ void k_pcg_mixed(PoissonArgs a);
__global__ void k_pcg_mixed_smem(PoissonArgs a);
__global__ void k_pcg_mixed_cheb(PoissonArgs a);
__global__ void k_pcg_mixed_stream(PoissonArgs a);
__global__ void k_pcg_mixed_cluster(PoissonArgs a);
__global__ void k_pcg_mixed_mg(PoissonArgs a);
__global__ void k_pcg_fp64_mg(PoissonArgs a);
__global__ void k_pcg_mixed_mg_semi(PoissonArgs a);
__global__ void k_pcg_fp64_mg_semi(PoissonArgs a);
__global__ void k_pcg_fp64_batch(const PoissonArgs* __restrict__ cases, BatchTeams bt);
__global__ void k_pcg_mixed_mg_batch(const PoissonArgs* __restrict__ cases, BatchTeams bt);
__global__ void k_pcg_fp64_mg_batch(const PoissonArgs* __restrict__ cases, BatchTeams bt);
__global__ void k_pcg_mixed_mg_batch_semi(const PoissonArgs* __restrict__ cases, BatchTeams bt);
__global__ void k_pcg_fp64_mg_batch_semi(const PoissonArgs* __restrict__ cases, BatchTeams bt);
__global__ void k_pcg_mixed_batch(const PoissonArgs* __restrict__ cases, BatchTeams bt);
__global__ void k_pcg_mixed_smem_batch(const PoissonArgs* __restrict__ cases, BatchTeams bt);
// Shared-memory bytes of k_pcg_mixed_cheb for a strip of R rows of nx cells.
inline size_t smem_cheb_bytes(int nx, int R) { return (size_t)(6 * R + 5) * (size_t)(nx + 2) * sizeof(float); }
// Shared-memory bytes of k_pcg_mixed_smem for a strip of R rows of nx cells.
inline size_t smem_strip_bytes(int nx, int R) { return (size_t)(6 * R + 7) * (size_t)(nx + 2) * sizeof(float); }
__global__ void k_project_correct(Dims D, double dt, double dx, double dy, int4 wall,
                                  double* __restrict__ u, double* __restrict__ v,
                                  const double* __restrict__ p, const double* __restrict__ rho_u,
                                  const double* __restrict__ rho_v);
__global__ void k_poisson_apply(Dims D, const double* __restrict__ x, double* __restrict__ y,
                                const double* __restrict__ ax, const double* __restrict__ ay,
                                const double* __restrict__ aP);

}  // namespace covof
