// capi.cu -- the extern "C" boundary (include/covof_gpu.h): handle life
// cycle, device mirrors for host-pointer calls, scratch management and the
// launch sequences of every entry point.  No exception crosses the boundary;
// every CUDA error becomes COVOF_CUDA_ERROR.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "handle.cuh"

using namespace covof;

namespace covof {
namespace host {

// One thread: fold this step's predictor and Poisson result records in.
__global__ void k_step_log(const KrylovResult* kr, const PcgResult* pr, RunStats* s) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int step = s->step;
  s->mom_iters += kr->iters;
  s->poisson_iters += pr->iters;
  s->refine_steps += pr->outer;
  s->last_relres = pr->relres;
  if (!(pr->relres <= s->max_relres)) s->max_relres = pr->relres;  // also takes a NaN
  if (s->first_bad_step < 0) {
    const int bad = kr->status != COVOF_OK ? kr->status : pr->status;
    if (bad != COVOF_OK) {
      s->first_bad_step = step;
      s->first_bad_status = bad;
    }
  }
  s->step = step + 1;
}


int check_params(const covof_params* p) {
  if (!p) return COVOF_INVALID;
  if (p->nx < 2 || p->ny < 2 || !(p->dx > 0.0) || !(p->dy > 0.0)) return COVOF_INVALID;
  if ((long long)(p->nx + 2) * (p->ny + 2) > (1LL << 30)) return COVOF_INVALID;
  for (int s = 0; s < 4; ++s) {
    const int t = p->bc_type[s];
    if (t == COVOF_BC_NEUMANN) return COVOF_UNSUPPORTED;
    // a periodic direction names both of its sides (left / right, bottom / top)
    if (t == COVOF_BC_PERIODIC) {
      if (p->bc_type[s ^ 1] != COVOF_BC_PERIODIC) return COVOF_INVALID;
      continue;
    }
    if (t != COVOF_BC_DIRICHLET && t != COVOF_BC_FREESLIP) return COVOF_INVALID;
  }
  if (p->advection_method < COVOF_ADVECT_WEYMOUTH_YUE || p->advection_method > COVOF_ADVECT_TVD) return COVOF_INVALID;
  if (p->p_precision < COVOF_PREC_FP64 || p->p_precision > COVOF_PREC_FP64_MG) return COVOF_INVALID;
  if (p->tvd_limiter < COVOF_LIMITER_SUPERBEE || p->tvd_limiter > COVOF_LIMITER_HRIC) return COVOF_INVALID;
  return COVOF_OK;
}

bool periodic(const covof_params& p) {
  return p.bc_type[0] == COVOF_BC_PERIODIC || p.bc_type[2] == COVOF_BC_PERIODIC;
}

// The periodic branches on the GPU: the Poisson operator in the plain FP64
// Jacobi-PCG, the projection correction, the velocity and VOF ghosts and the
// Weymouth-Yue step (src/module_simulation.f90:2679-2701, 2602-2654;
// src/module_mpi_comm.f90:25-56, 332-351, 636-683; src/module_interface_vof.f90:
// 1223-1231, 1268-1276).  The momentum predictor (its velocity DOFs change
// with periodicity), the multigrid and sweep Poisson solvers, CIAM / TVD and
// the smoothing filters refuse periodic boundaries.
int check_periodic_vof(const covof_params& p) {
  if (!periodic(p)) return COVOF_OK;
  if (p.advection_method != COVOF_ADVECT_WEYMOUTH_YUE || p.enable_svof_smoothing || p.enable_diffusion_smoothing)
    return COVOF_UNSUPPORTED;
  return COVOF_OK;
}

// The flexible CG with the multigrid V-cycle: MIXED with COVOF_INNER_MG (FP32
// V-cycle) or FP64_MG (FP64 V-cycle).
bool mg_path(const covof_params& p) {
  return (p.p_precision == COVOF_PREC_MIXED && p.p_inner_kind == COVOF_INNER_MG) ||
         p.p_precision == COVOF_PREC_FP64_MG;
}

int4 wall_flags(const covof_params& p) {
  auto w = [&](int s) { return (p.bc_type[s] == COVOF_BC_DIRICHLET || p.bc_type[s] == COVOF_BC_FREESLIP) ? 1 : 0; };
  return make_int4(w(0), w(1), w(2), w(3));
}

dim3 grid2(int ni, int nj, dim3 b) { return dim3((ni + b.x - 1) / b.x, (nj + b.y - 1) / b.y); }

int ensure_fields(covof_handle* h) {
  if (h->have_fields) return COVOF_OK;
  const size_t g = h->g;
  CS(dalloc(&h->f_u, g)); CS(dalloc(&h->f_v, g)); CS(dalloc(&h->f_p, g));
  CS(dalloc(&h->f_rho_u, g)); CS(dalloc(&h->f_rho_v, g)); CS(dalloc(&h->f_mu, g));
  CS(dalloc(&h->f_mu_node, g)); CS(dalloc(&h->f_fx, g)); CS(dalloc(&h->f_fy, g));
  CS(dalloc(&h->f_u_old, g)); CS(dalloc(&h->f_v_old, g)); CS(dalloc(&h->f_C, g));
  CS(dalloc(&h->f_u_nm1, g)); CS(dalloc(&h->f_v_nm1, g));
  CS(dalloc(&h->f_Cs, g)); CS(dalloc(&h->f_Ct, g));
  CS(dalloc(&h->f_rho, g)); CS(dalloc(&h->f_curv, g)); CS(dalloc(&h->f_b, g));
  CS(dalloc(&h->f_x2, 2 * g)); CS(dalloc(&h->f_seg, 3 * g));
  h->have_fields = true;
  return COVOF_OK;
}

int ensure_poisson(covof_handle* h) {
  if (h->have_poisson) return COVOF_OK;
  const size_t g = h->g;
  CS(dalloc(&h->px, g)); CS(dalloc(&h->pb, g)); CS(dalloc(&h->pr, g)); CS(dalloc(&h->pd, g));
  CS(dalloc(&h->pAd, g)); CS(dalloc(&h->pax, g)); CS(dalloc(&h->pay, g)); CS(dalloc(&h->paP, g));
  CS(dalloc(&h->pisd, g)); CS(dalloc(&h->pinvD, g)); CS(dalloc(&h->pd2, g)); CS(dalloc(&h->d32b, g));
  CS(dalloc(&h->pz, g)); CS(dalloc(&h->pw, g)); CS(dalloc(&h->pp, g)); CS(dalloc(&h->pq, g));
  CS(dalloc(&h->pxb, (size_t)8 * h->sm_count * (size_t)(h->D.nx + 2)));
  CS(dalloc(&h->e32, g)); CS(dalloc(&h->r32b, g)); CS(dalloc(&h->r32, g)); CS(dalloc(&h->d32, g));
  CS(dalloc(&h->Ad32, g)); CS(dalloc(&h->ax32, g)); CS(dalloc(&h->ay32, g)); CS(dalloc(&h->aP32, g));
  CS(dalloc(&h->pin_part, (size_t)4 * kPinBlocks + 4)); CS(dalloc(&h->pin_ctl, 4));
  CS(dalloc(&h->pin_b, g));
  // multigrid levels: halve each dimension down to about 64 cells; es =
  // bytes per element of the V-cycle's arithmetic
  const long long es = h->prm.p_precision == COVOF_PREC_FP64_MG ? 8 : 4;
  MgHier& H = h->mg;
  H.nl = 1;
  H.lv[0].nx = h->D.nx; H.lv[0].ny = h->D.ny; H.lv[0].off = 0;
  H.lv[0].fx = H.lv[0].fy = 1;
  H.semi = 0;
  long long pool = 0;
  // cell sides of the level being coarsened: on anisotropic cells the
  // couplings across the short side are the strong ones, and only that
  // direction is halved (semi-coarsening) until the cells are within a
  // factor 2 of square; aggregation across the weak direction leaves the
  // smooth error of the strong one to a point smoother that cannot reduce it
  double hx = h->prm.dx, hy = h->prm.dy;
  while (H.nl < kMgMaxLevels && (long long)H.lv[H.nl - 1].nx * H.lv[H.nl - 1].ny > 64 &&
         (H.lv[H.nl - 1].nx > 1 || H.lv[H.nl - 1].ny > 1)) {
    const MgLevel& f = H.lv[H.nl - 1];
    int fx = 2, fy = 2;
    if (hy >= 2.0 * hx) fy = 1;
    else if (hx >= 2.0 * hy) fx = 1;
    // a direction already one cell wide: the other one only
    if (f.nx < 2) { fx = 1; fy = 2; }
    if (f.ny < 2) { fy = 1; fx = 2; }
    MgLevel& c = H.lv[H.nl];
    c.fx = fx; c.fy = fy;
    c.nx = (f.nx + fx - 1) / fx;
    c.ny = (f.ny + fy - 1) / fy;
    hx *= fx; hy *= fy;
    if (fx != 2 || fy != 2) H.semi = 1;
    c.off = pool;
    pool += 7LL * (c.nx + 2) * (c.ny + 2);
    H.nl += 1;
  }
  H.wd0_off = pool;
  pool += (long long)g;
  // the tail: from the first level of at most p_mg_tail cells whose levels
  // down to the coarsest (eight fields each) fit in kMgTailSmem bytes of
  // shared memory
  const long long tail_cells = h->prm.p_mg_tail > 0 ? h->prm.p_mg_tail : 2048;
  H.tail = H.nl;
  H.tail_smem = 0;
  for (int l = 1; l < H.nl; ++l) {
    long long bytes = 0;
    for (int q = l; q < H.nl; ++q) bytes += 8LL * es * (H.lv[q].nx + 2) * (H.lv[q].ny + 2);
    if ((long long)H.lv[l].nx * H.lv[l].ny <= tail_cells && bytes <= kMgTailSmem) {
      H.tail = l;
      H.tail_smem = (int)bytes;
      break;
    }
  }
  H.omega = 0.8f;
  // the block-local tail levels run a W-cycle (two coarse corrections per
  // level) on meshes of at least kMgWCells cells: at 1024^2 it cuts the outer
  // iterations by a tenth for a few us more tail work; on small meshes the
  // tail is most of the cycle and a W-cycle there costs more than it saves
  H.gamma = (long long)h->D.nx * h->D.ny >= kMgWCells ? 2 : 1;
  H.nu = h->prm.p_mg_nu < 1 ? 1 : (h->prm.p_mg_nu > 8 ? 8 : h->prm.p_mg_nu);
  H.cw = (float)(h->prm.p_mg_cw > 0.0 && h->prm.p_mg_cw <= 4.0 ? h->prm.p_mg_cw : 1.0);
  // an even count leaves the coarsest correction in its first buffer
  const int nuc = h->prm.p_mg_nuc > 0 ? (h->prm.p_mg_nuc > 1024 ? 1024 : h->prm.p_mg_nuc) : 64;
  H.nuc = (nuc + 1) & ~1;
  // p_mg_nuc < 0: the coarsest level solved exactly (a dense inverse in the
  // tail's shared memory) when it is in the tail and has at most 64 cells
  H.exact = 0;
  H.inv_off = 0;
  const long long ncoarse = (long long)H.lv[H.nl - 1].nx * H.lv[H.nl - 1].ny;
  if (h->prm.p_mg_nuc < 0 && H.tail < H.nl && ncoarse <= 64 && H.tail_smem + 64 * 64 * es <= kMgTailSmem) {
    H.exact = 1;
    H.inv_off = (int)(H.tail_smem / es);
    H.tail_smem += (int)(64 * 64 * es);
    H.nuc = 0;
  }
  if (pool > 0) {
    unsigned char* raw = nullptr;
    CS(dalloc(&raw, (size_t)(pool * es)));
    H.pool = raw;
  }
  h->have_poisson = true;
  return COVOF_OK;
}

int ensure_mom(covof_handle* h) {
  if (h->have_mom) return COVOF_OK;
  const size_t g2 = 2 * h->g;
  // Krylov vectors: u and v blocks, and the pressure block for MONOLITHIC
  // (zero-filled, so the pressure block's ghost entries read as zero)
  const size_t gk = (h->prm.solver_type == COVOF_SOLVER_MONOLITHIC ? 3 : 2) * h->g;
  CS(dalloc(&h->mx, gk)); CS(dalloc(&h->mrhs, gk)); CS(dalloc(&h->mdiag, gk));
  CS(dalloc(&h->mcoef, 9 * g2)); CS(dalloc(&h->midiag, gk));
  CS(dalloc(&h->al_r, h->g)); CS(dalloc(&h->al_max, 4));
  for (int q = 0; q < 7; ++q) CS(dalloc(&h->mv[q], gk));
  h->have_mom = true;
  return COVOF_OK;
}

// interface cells from which the reconstruction runs one thread per cell
int vof_cell_min(const covof_handle* h) {
  return h->launch.vof_cell_min > 0 ? h->launch.vof_cell_min : kVofCellMin;
}

int ensure_vof(covof_handle* h) {
  if (h->have_vof) return COVOF_OK;
  const size_t g = h->g;
  CS(dalloc(&h->cs, g)); CS(dalloc(&h->seg, 3 * g));
  CS(dalloc(&h->cnx, g)); CS(dalloc(&h->cny, g)); CS(dalloc(&h->ckap, g));
  CS(dalloc(&h->vlist, g)); CS(dalloc(&h->vcount, 1));
  CS(dalloc(&h->dscr, g));
  const int nb = (h->D.ny + 31) / 32;
  CS(dalloc(&h->svof_prog, (size_t)32 * nb));
  // the SVOF wavefront: one 32-thread block per band of 32 rows, all resident
  int per_sm = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_svof_sgs, 32, 0));
  const int cap = per_sm * h->sm_count;
  if (cap < 1) return COVOF_CUDA_ERROR;
  h->svof_nb = nb < cap ? nb : cap;
  // the thread-per-cell reconstruction: every block resident, grid-stride
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_vof_mixed_cell, 128, 0));
  h->vof_cell_nb = (per_sm < 1 ? 1 : per_sm) * h->sm_count;
  h->have_vof = true;
  return COVOF_OK;
}

int ensure_adj(covof_handle* h) {
  if (h->have_adj) return COVOF_OK;
  const size_t g = h->g;
  CS(dalloc(&h->arhs, g)); CS(dalloc(&h->apsi, g)); CS(dalloc(&h->apart, 1024)); CS(dalloc(&h->asum, 1));
  h->have_adj = true;
  return COVOF_OK;
}

int ensure_adj_host(covof_handle* h) {
  if (h->f_gu) return COVOF_OK;
  const size_t g = h->g;
  CS(dalloc(&h->f_gu, g)); CS(dalloc(&h->f_gv, g)); CS(dalloc(&h->f_gp, g));
  CS(dalloc(&h->f_gbu, g)); CS(dalloc(&h->f_gbv, g)); CS(dalloc(&h->f_ou, g)); CS(dalloc(&h->f_ov, g));
  return COVOF_OK;
}

// Block count of a persistent cooperative kernel: per_sm_max blocks on
// every SM (one by default: fewer arrivals per grid barrier, and the
// 1024-thread Poisson blocks fill an SM anyway), fewer when the kernel's
// registers or shared memory allow fewer co-resident blocks or there are
// fewer work units, never more than the partials array's slots.
int coop_blocks(covof_handle* h, const void* fn, int threads, long long units, size_t smem = 0,
                int per_sm_max = 1) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem) != cudaSuccess || per_sm < 1)
    return -1;
  if (per_sm > per_sm_max) per_sm = per_sm_max;
  long long nb = (long long)per_sm * h->sm_count;
  if (units < nb) nb = units < 1 ? 1 : units;
  if (nb > h->part_blocks) nb = h->part_blocks;
  return (int)nb;
}

int launch_coop(covof_handle* h, const void* fn, int nblocks, int threads, void** args, bool timed,
                size_t smem = 0) {
  CK(cudaMemsetAsync(h->bar, 0, (size_t)(64 + h->sm_count) * sizeof(unsigned int), h->stream));
  CK(cudaMemsetAsync(h->err, 0, sizeof(int), h->stream));
  if (timed) CK(cudaEventRecord(h->ev0, h->stream));
  // cooperative launch through the extensible API: the same co-residency
  // guarantee as cudaLaunchCooperativeKernel, and a stream capture records it
  // as a cooperative kernel node
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblocks);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = h->stream;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  CK(cudaLaunchKernelExC(&cfg, fn, args));
  if (timed) CK(cudaEventRecord(h->ev1, h->stream));
  return COVOF_OK;
}

// One thread-block cluster of nblocks CTAs (all co-scheduled by the hardware).
int launch_cluster(covof_handle* h, const void* fn, int nblocks, int threads, void** args, bool timed,
                   size_t smem) {
  CK(cudaMemsetAsync(h->bar, 0, (size_t)(64 + h->sm_count) * sizeof(unsigned int), h->stream));
  CK(cudaMemsetAsync(h->err, 0, sizeof(int), h->stream));
  if (timed) CK(cudaEventRecord(h->ev0, h->stream));
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = nblocks;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblocks);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = h->stream;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  CK(cudaLaunchKernelExC(&cfg, fn, args));
  if (timed) CK(cudaEventRecord(h->ev1, h->stream));
  return COVOF_OK;
}

int h2d(covof_handle* h, double* d, const double* s, size_t n) {
  if (!s) return COVOF_INVALID;
  CK(cudaMemcpyAsync(d, s, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  return COVOF_OK;
}
int d2h(covof_handle* h, double* s, const double* d, size_t n) {
  if (!s) return COVOF_INVALID;
  CK(cudaMemcpyAsync(s, d, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return COVOF_OK;
}
int sync(covof_handle* h) {
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaGetLastError());
  return COVOF_OK;
}

// ---------------------------------------------------------------------------
// Poisson
//
// Launch plan: the plain FP64 path runs k_pcg_fp64 over 1024-cell tiles; the
// mixed path runs the shared-memory-resident inner solver (Chebyshev or CG,
// one row strip per block) when a strip fits the opt-in shared memory, else
// the tiled kernel.
// Block size of the plain FP64 PCG: 1024-cell tiles when there are at least
// two per SM; otherwise the size that puts the fewest cells on the busiest
// block, so that a small mesh spreads over every SM (the FP64 issue rate of
// an SM, not bandwidth, bounds this kernel on GB300).
int fp64_threads(const covof_handle* h) {
  const long long G = h->sm_count;
  if (make_tiles(h->D, 1024).ntiles >= 2 * G) return 1024;
  int best = 1024;
  long long best_cells = -1;
  for (int t : {1024, 512, 256, 128}) {
    const long long nt = make_tiles(h->D, t).ntiles;
    const long long cells = ((nt + G - 1) / G) * t;  // cells of the busiest block
    if (best_cells < 0 || cells < best_cells) { best_cells = cells; best = t; }
  }
  return best;
}

// Block size of the multigrid kernel: 1024-cell tiles when there is one
// for every SM; on smaller meshes the largest of 512 and 256 that still
// gives every SM a tile, else 256 -- the outer FP64 passes are bound by the
// FP64 issue of the SMs that hold tiles, so a small mesh spreads over more
// SMs (the 128 x 256 bubble step: 2.06 -> 1.83 ms with 256-thread blocks)
int mg_threads(const covof_handle* h) {
  const long long G = h->sm_count;
  for (int t : {1024, 512})
    if (make_tiles(h->D, t).ntiles >= G) return t;
  return 256;
}

int poisson_plan(covof_handle* h) {
  if (h->have_pplan) return COVOF_OK;
  CS(ensure_poisson(h));  // the multigrid plan sizes its shared memory from the hierarchy
  const covof_params& P = h->prm;
  const bool mixed = P.p_precision == COVOF_PREC_MIXED;
  const covof_launch& L = h->launch;
  const void* fn = mixed ? (const void*)k_pcg_mixed : (const void*)k_pcg_fp64;
  const int threads = mixed ? kPoissonThreads : (L.p_threads ? L.p_threads : fp64_threads(h));
  long long units = (long long)make_tiles(h->D, threads).ntiles;
  size_t smem = 0;
  h->p_cluster = false;
  if (mg_path(P)) {
    // multigrid inner: one persistent block per SM, tile-owned outer
    const bool semi = h->mg.semi != 0;
    const void* mfn = P.p_precision == COVOF_PREC_FP64_MG
                          ? (semi ? (const void*)k_pcg_fp64_mg_semi : (const void*)k_pcg_fp64_mg)
                          : (semi ? (const void*)k_pcg_mixed_mg_semi : (const void*)k_pcg_mixed_mg);
    long long units = h->sm_count;
    if (L.p_blocks > 0 && L.p_blocks < units) units = L.p_blocks;
    const size_t tail = (size_t)h->mg.tail_smem;
    // opt in whatever the size: the kernel's static shared memory counts
    // against the 48 KB a launch gets without it
    if (cudaFuncSetAttribute(mfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tail) != cudaSuccess)
      return COVOF_CUDA_ERROR;
    const int mthreads = L.p_threads ? L.p_threads : mg_threads(h);
    const long long mtiles = make_tiles(h->D, mthreads).ntiles;
    if (mtiles < units) units = mtiles;
    const int nb = coop_blocks(h, mfn, mthreads, units, tail);
    if (nb < 1) return COVOF_CUDA_ERROR;
    h->p_fn = mfn;
    h->p_smem = tail;
    h->p_nb = nb;
    h->p_threads = mthreads;
    h->have_pplan = true;
    return COVOF_OK;
  }
  if (mixed && P.p_inner_kind == COVOF_INNER_CHEBYSHEV && L.p_inner_form == 3) {
    // the whole inner state in one thread-block cluster (asked for by the
    // launch override: measured no faster than strips on every SM for the
    // meshes that fit, so the rules do not pick it)
    int G = L.p_blocks > 0 ? L.p_blocks : 16;
    if (G > P.ny) G = P.ny;
    const int Rmax = (P.ny + G - 1) / G;
    const size_t bytes = smem_cheb_bytes(P.nx, Rmax);
    const void* cfn = (const void*)k_pcg_mixed_cluster;
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
    cudaFuncAttributes fa;
    bool fits = G >= 1 && G <= 16 && cudaFuncGetAttributes(&fa, cfn) == cudaSuccess &&
                bytes + fa.sharedSizeBytes <= (size_t)optin &&
                cudaFuncSetAttribute(cfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess &&
                (G <= 8 || cudaFuncSetAttribute(cfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess);
    if (fits) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = G; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3(G); cfg.blockDim = dim3(kPoissonThreads); cfg.dynamicSmemBytes = bytes;
      cfg.attrs = at; cfg.numAttrs = 1;
      int nclusters = 0;
      fits = cudaOccupancyMaxActiveClusters(&nclusters, cfn, &cfg) == cudaSuccess && nclusters >= 1 &&
             G <= h->part_blocks;
    }
    cudaGetLastError();
    if (fits) {
      h->p_fn = cfn;
      h->p_smem = bytes;
      h->p_nb = G;
      h->p_threads = kPoissonThreads;
      h->p_cluster = true;
      h->have_pplan = true;
      return COVOF_OK;
    }
    return COVOF_UNSUPPORTED;  // the cluster asked for does not fit
  }
  if (mixed) {
    // one row strip per block, at most one block per SM
    int G = P.ny < h->sm_count ? P.ny : h->sm_count;
    if (L.p_blocks > 0 && L.p_blocks < G) G = L.p_blocks;
    const int Rmax = (P.ny + G - 1) / G;
    const bool cheb = P.p_inner_kind != COVOF_INNER_CG;
    const void* sfn = cheb ? (const void*)k_pcg_mixed_cheb : (const void*)k_pcg_mixed_smem;
    const size_t bytes = cheb ? smem_cheb_bytes(P.nx, Rmax) : smem_strip_bytes(P.nx, Rmax);
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
    cudaFuncAttributes fa;
    const bool stream = P.p_inner_kind == COVOF_INNER_CHEBYSHEV_STREAM || (cheb && L.p_inner_form == 2);
    if (!stream && cudaFuncGetAttributes(&fa, sfn) == cudaSuccess && bytes + fa.sharedSizeBytes <= (size_t)optin &&
        cudaFuncSetAttribute(sfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess) {
      fn = sfn;
      smem = bytes;
      units = G;
    } else if (cheb) {
      cudaGetLastError();
      if (L.p_inner_form == 1) return COVOF_UNSUPPORTED;  // strips asked for do not fit
      fn = (const void*)k_pcg_mixed_stream;  // strips stream through L2 / HBM
      units = G;
    }
    cudaGetLastError();
  } else if (L.p_blocks > 0 && L.p_blocks < units) {
    units = L.p_blocks;  // fewer blocks than tiles: each block walks several tiles
  }
  const int nb = coop_blocks(h, fn, threads, units, smem);
  if (nb < 1) return COVOF_CUDA_ERROR;
  if (mixed && fn != (const void*)k_pcg_mixed && nb != (int)units)
    return COVOF_CUDA_ERROR;  // strips are sized for exactly G blocks
  h->p_fn = fn;
  h->p_smem = smem;
  h->p_nb = nb;
  h->p_threads = threads;
  h->have_pplan = true;
  return COVOF_OK;
}

// Assembly on the handle's stream and the argument block of the solve.
int pois_pre(covof_handle* h, double dt, const double* u, const double* v, const double* b,
             const double* rho_u, const double* rho_v, double* p, PoissonArgs* out) {
  const covof_params& P = h->prm;
  if (!rho_u || !rho_v || !p || (!b && (!u || !v))) return COVOF_INVALID;
  const bool mixed = P.p_precision == COVOF_PREC_MIXED;
  // the symmetric Gauss-Seidel preconditioner belongs to the plain FP64 PCG
  if (P.p_precond == COVOF_PRECOND_SSOR && P.p_precision != COVOF_PREC_FP64) return COVOF_UNSUPPORTED;
  // periodic boundaries: the plain FP64 Jacobi-PCG
  if (periodic(P) && (P.p_precision != COVOF_PREC_FP64 || P.p_precond == COVOF_PRECOND_SSOR))
    return COVOF_UNSUPPORTED;
  CS(ensure_poisson(h));
  CS(poisson_plan(h));
  const int pinned = P.p_gauge == COVOF_GAUGE_PINNED;
  const dim3 blk(32, 8), grd = grid2(P.nx, P.ny, blk);
  k_poisson_assemble<<<grd, blk, 0, h->stream>>>(h->D, dt, P.dx, P.dy, wall_flags(P), rho_u, rho_v, u, v,
                                                  b, pinned, h->pax, h->pay, h->paP, h->pb,
                                                  mixed ? h->pisd : nullptr,
                                                  P.p_precision == COVOF_PREC_FP64 ? h->pinvD : nullptr);
  if (mixed)
    k_poisson_scale32<<<grid2(P.nx + 1, P.ny + 1, blk), blk, 0, h->stream>>>(
        h->D, h->pax, h->pay, h->pisd, h->ax32, h->ay32, h->aP32, h->paP, P.p_inner_kind == COVOF_INNER_MG ? 1 : 0);
  k_copy_interior<<<grd, blk, 0, h->stream>>>(h->D, p, h->px, pinned);
  // periodic: the initial guess's ghost ring carries the wrapped interior
  // (the first residual's stencil reads it)
  if (periodic(P)) k_wrap_ghosts<<<1, 1024, 0, h->stream>>>(h->D, h->px);
  CK(cudaGetLastError());
  PoissonArgs& a = *out;
  std::memset(&a, 0, sizeof(a));
  a.D = h->D;
  a.x = h->px; a.b = h->pb; a.r = h->pr; a.d = h->pd; a.d2 = h->pd2; a.Ad = h->pAd;
  a.ax = h->pax; a.ay = h->pay; a.aP = h->paP; a.invD = h->pinvD; a.isd = h->pisd;
  a.z = h->pz; a.w = h->pw; a.p = h->pp; a.q = h->pq; a.xb = h->pxb;
  a.flags = h->bar + 64; a.cheb_lo = P.p_cheb_lo;
  a.e32 = h->e32; a.r32b = h->r32b; a.r32 = h->r32; a.d32 = h->d32; a.d32b = h->d32b; a.Ad32 = h->Ad32;
  a.ax32 = h->ax32; a.ay32 = h->ay32; a.aP32 = h->aP32;
  a.bar = h->bar; a.err = h->err; a.part = h->part; a.res = h->d_pres;
  a.tol = P.p_tol; a.inner_tol = P.p_inner_tol;
  a.max_iter = P.p_max_iter; a.inner_max_iter = P.p_inner_max_iter;
  a.max_refine = P.p_max_refine; a.pinned = pinned;
  a.bskip = -1;
  a.mg = h->mg;
  return COVOF_OK;
}

// Solution back into the caller's field.
int pois_post(covof_handle* h, double* p) {
  const dim3 blk(32, 8), grd = grid2(h->prm.nx, h->prm.ny, blk);
  k_copy_interior<<<grd, blk, 0, h->stream>>>(h->D, h->px, p, 0);
  CK(cudaGetLastError());
  return COVOF_OK;
}

// Assembly, solve and copy-back on the handle's stream; the result record
// stays on the device (h->d_pres).  Nothing here synchronises.
int poisson_enqueue(covof_handle* h, double dt, const double* u, const double* v, const double* b,
                    const double* rho_u, const double* rho_v, double* p, bool timed) {
  PoissonArgs a;
  CS(pois_pre(h, dt, u, v, b, rho_u, rho_v, p, &a));
  const covof_params& P = h->prm;
  if (mg_path(P) && a.pinned &&
      (h->p_fn == (const void*)k_pcg_mixed_mg || h->p_fn == (const void*)k_pcg_fp64_mg ||
       h->p_fn == (const void*)k_pcg_mixed_mg_semi || h->p_fn == (const void*)k_pcg_fp64_mg_semi)) {
    // The pinned system solved through the reference gauge, whose
    // deflation handles the constant mode exactly (35 against 41 outer
    // iterations at 1024^2); the pinned residual is checked after the shift
    // and the pinned solve rerun only if the check fails (see poisson.cuh).
    const Dims& D = h->D;
    double* part = h->pin_part;
    double* lvl = h->pin_part + 4 * kPinBlocks;
    int* ctl = h->pin_ctl;
    const dim3 blk(32, 8), grd = grid2(P.nx, P.ny, blk);
    if (timed) CK(cudaEventRecord(h->ev0, h->stream));
    k_pin_sum<<<kPinBlocks, 256, 0, h->stream>>>(D, h->pb, h->px, h->pax, h->pay, h->paP, part, ctl);
    k_pin_rhs<<<1, 256, 0, h->stream>>>(D, part, lvl, ctl);
    k_pin_form<<<grd, blk, 0, h->stream>>>(D, h->pb, h->pax, h->pay, h->paP, h->pin_b, lvl, ctl);
    CK(cudaGetLastError());
    PoissonArgs ar = a;
    ar.pinned = 0;
    ar.b = h->pin_b;
    ar.bskip = D.P + 1;
    ar.redo = ctl + 2;
    void* args_r[] = {&ar};
    CS(launch_coop(h, h->p_fn, h->p_nb, h->p_threads, args_r, false, h->p_smem));
    k_pin_level<<<1, 32, 0, h->stream>>>(D, h->px, lvl, ctl);
    k_pin_shift<<<grd, blk, 0, h->stream>>>(D, h->px, lvl, ctl);
    k_pin_resid<<<kPinBlocks, 256, 0, h->stream>>>(D, h->pb, h->px, h->pax, h->pay, h->paP, part, ctl);
    k_pin_final<<<1, 256, 0, h->stream>>>(D, part, P.p_tol, h->d_pres, ctl);
    CK(cudaGetLastError());
    PoissonArgs af = a;
    af.redo = ctl;
    void* args_f[] = {&af};
    CS(launch_coop(h, h->p_fn, h->p_nb, h->p_threads, args_f, false, h->p_smem));
    if (timed) CK(cudaEventRecord(h->ev1, h->stream));
    return pois_post(h, p);
  }
  if (h->prm.p_precond == COVOF_PRECOND_SSOR) {
    // FP64 PCG with the Gauss-Seidel sweep pair, iterated from the host
    if (timed) CK(cudaEventRecord(h->ev0, h->stream));
    CS(pcg_sgs(h, a));
    if (timed) CK(cudaEventRecord(h->ev1, h->stream));
    return pois_post(h, p);
  }
  void* args[] = {&a};
  if (h->p_cluster) CS(launch_cluster(h, h->p_fn, h->p_nb, h->p_threads, args, timed, h->p_smem));
  else CS(launch_coop(h, h->p_fn, h->p_nb, h->p_threads, args, timed, h->p_smem));
  return pois_post(h, p);
}

// Reads the result record back (one small copy + stream synchronisation).
int poisson_finish(covof_handle* h, int* iters, double* relres) {
  CK(cudaMemcpyAsync(h->h_pres, h->d_pres, sizeof(PcgResult), cudaMemcpyDeviceToHost, h->stream));
  CS(sync(h));
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, h->ev0, h->ev1) == cudaSuccess) h->last_solve_ms = ms;
  cudaGetLastError();
  h->last_refine = h->h_pres->outer;
  if (iters) *iters = h->h_pres->iters;
  if (relres) *relres = h->h_pres->relres;
  return h->h_pres->status;
}

int poisson_dev(covof_handle* h, double dt, const double* u, const double* v, const double* b,
                const double* rho_u, const double* rho_v, double* p, int* iters, double* relres) {
  CS(poisson_enqueue(h, dt, u, v, b, rho_u, rho_v, p, true));
  return poisson_finish(h, iters, relres);
}

int correct_dev(covof_handle* h, double dt, double* u, double* v, const double* p,
                const double* rho_u, const double* rho_v) {
  const covof_params& P = h->prm;
  const dim3 blk(32, 8), grd = grid2(P.nx + 1, P.ny + 1, blk);
  k_project_correct<<<grd, blk, 0, h->stream>>>(h->D, dt, P.dx, P.dy, wall_flags(P), u, v, p, rho_u, rho_v);
  CK(cudaGetLastError());
  return COVOF_OK;
}

BcArgs bc_args(const covof_handle* h) {
  BcArgs b;
  b.D = h->D;
  for (int s = 0; s < 4; ++s) { b.bc[s] = h->prm.bc_type[s]; b.bcu[s] = h->prm.bc_u[s]; b.bcv[s] = h->prm.bc_v[s]; }
  return b;
}

int velocity_bc_dev(covof_handle* h, double* u, double* v) {
  const BcArgs b = bc_args(h);
  if (periodic(h->prm)) k_vbc_periodic<<<1, 1024, 0, h->stream>>>(b, u, v);
  k_vbc_we<<<(h->D.ny + 127) / 128, 128, 0, h->stream>>>(b, u, v);
  k_vbc_sn<<<(h->D.nx + 127) / 128, 128, 0, h->stream>>>(b, u, v);
  k_vbc_corners<<<1, 32, 0, h->stream>>>(b, u, v);
  CK(cudaGetLastError());
  return COVOF_OK;
}

// ---------------------------------------------------------------------------
// Projection and its adjoint
int projection_dev(covof_handle* h, double dt, const double* us, const double* vs, const double* rho_u,
                   const double* rho_v, double* p, double* u, double* v, int* iters, double* relres) {
  if (!us || !vs || !u || !v) return COVOF_INVALID;
  int st = poisson_dev(h, dt, us, vs, nullptr, rho_u, rho_v, p, iters, relres);
  if (st == COVOF_CUDA_ERROR || st == COVOF_INVALID || st == COVOF_UNSUPPORTED || st == COVOF_TIMEOUT) return st;
  if (u != us) CK(cudaMemcpyAsync(u, us, h->g * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  if (v != vs) CK(cudaMemcpyAsync(v, vs, h->g * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CS(correct_dev(h, dt, u, v, p, rho_u, rho_v));
  CS(sync(h));
  return st;
}

int vjp_dev(covof_handle* h, double dt, const double* rho_u, const double* rho_v, const double* p,
            const double* gu, const double* gv, const double* gp, double* grad_u, double* grad_v,
            double* grad_bu, double* grad_bv, int* iters, double* relres) {
  const covof_params& P = h->prm;
  if (!rho_u || !rho_v || !p || !gu || !gv || !grad_u || !grad_v || !grad_bu || !grad_bv) return COVOF_INVALID;
  if (periodic(P)) return COVOF_UNSUPPORTED;  // the adjoint's face kernels assume walls
  CS(ensure_adj(h));
  double gp_mean = 0.0;
  if (gp && P.p_gauge == COVOF_GAUGE_REFERENCE) {
    // p has its mean removed: only the mean-free part of gp reaches A^-1
    k_sum_interior<<<256, 256, 0, h->stream>>>(h->D, gp, h->apart);
    k_sum_final<<<1, 256, 0, h->stream>>>(h->apart, 256, h->asum);
    double s = 0.0;
    CK(cudaMemcpyAsync(&s, h->asum, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CS(sync(h));
    gp_mean = s / (double)((long long)P.nx * P.ny);
  }
  AdjArgs a;
  a.D = h->D; a.dx = P.dx; a.dy = P.dy; a.dt = dt; a.wall = wall_flags(P);
  a.rho_u = rho_u; a.rho_v = rho_v; a.p = p; a.gu = gu; a.gv = gv; a.gp = gp;
  a.rhs = h->arhs; a.psi = h->apsi;
  a.grad_u = grad_u; a.grad_v = grad_v; a.grad_bu = grad_bu; a.grad_bv = grad_bv;
  const dim3 blk(32, 8);
  k_adj_rhs<<<grid2(P.nx, P.ny, blk), blk, 0, h->stream>>>(a, gp_mean);
  CK(cudaMemsetAsync(h->apsi, 0, h->g * sizeof(double), h->stream));
  CK(cudaGetLastError());
  int st = poisson_dev(h, dt, nullptr, nullptr, h->arhs, rho_u, rho_v, h->apsi, iters, relres);
  if (st == COVOF_CUDA_ERROR || st == COVOF_INVALID || st == COVOF_UNSUPPORTED || st == COVOF_TIMEOUT) return st;
  k_adj_grad<<<grid2(P.nx + 1, P.ny + 1, blk), blk, 0, h->stream>>>(a);
  CK(cudaGetLastError());
  CS(sync(h));
  return st;
}

// ---------------------------------------------------------------------------
// Momentum predictor
MomArgs mom_args(covof_handle* h, double dt, const double* u_n, const double* v_n,
                 const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                 const double* fx, const double* fy, const double* u_old, const double* v_old) {
  const covof_params& P = h->prm;
  MomArgs a;
  a.D = h->D; a.dx = P.dx; a.dy = P.dy; a.dt = dt; a.gx = P.gx; a.gy = P.gy;
  for (int s = 0; s < 4; ++s) { a.bc[s] = P.bc_type[s]; a.bcu[s] = P.bc_u[s]; a.bcv[s] = P.bc_v[s]; }
  a.conv = P.enable_convection; a.scheme = P.convective_scheme;
  // history: the handle's u_nm1 / v_nm1 fields once has_nm1 is set
  // (src/module_simulation.f90:508-520)
  const bool gear = P.time_scheme == COVOF_TIME_GEAR && h->has_nm1;
  a.alpha = gear ? 1.5 : 1.0;
  a.gear_rhs = gear ? 1 : 0;
  a.ab2 = P.convective_linearization == COVOF_CONV_LIN_AB2 ? 1 : 0;
  a.ab2_ext = (a.ab2 && h->has_nm1) ? 1 : 0;
  a.u_nm1 = h->f_u_nm1; a.v_nm1 = h->f_v_nm1;
  a.r_al = nullptr; a.p_al = nullptr;  // set by al_enqueue
  a.mono = 0; a.pm = nullptr;           // set by mono_enqueue
  a.u_n = u_n; a.v_n = v_n; a.rho_u = rho_u; a.rho_v = rho_v; a.mu = mu; a.mu_node = mu_node;
  a.fx = fx; a.fy = fy; a.u_old = u_old; a.v_old = v_old;
  a.x = h->mx; a.rhs = h->mrhs; a.diag = h->mdiag; a.coef = h->mcoef; a.idiag = h->midiag;
  a.v0 = h->mv[0]; a.v1 = h->mv[1]; a.v2 = h->mv[2]; a.v3 = h->mv[3];
  a.v4 = h->mv[4]; a.v5 = h->mv[5]; a.v6 = h->mv[6];
  a.precond_on = P.use_precond && (P.precond == COVOF_PRECOND_JACOBI || P.precond == COVOF_PRECOND_ILU0);
  a.max_iter = P.max_iter; a.tol = P.tol; a.method = P.linear_solver;
  a.bar = h->bar; a.err = h->err; a.part = h->part; a.res = h->d_kres;
  return a;
}

int check_mom_params(const covof_params& P) {
  if (periodic(P)) return COVOF_UNSUPPORTED;
  if (P.convective_scheme != COVOF_CONV_UPWIND && P.convective_scheme != COVOF_CONV_CENTERED &&
      P.convective_scheme != COVOF_CONV_TVD_SUPERBEE)
    return COVOF_UNSUPPORTED;
  if (P.time_scheme != 0 && P.time_scheme != COVOF_TIME_EULER && P.time_scheme != COVOF_TIME_GEAR)
    return COVOF_UNSUPPORTED;
  if (P.convective_linearization != 0 && P.convective_linearization != COVOF_CONV_LIN_PICARD &&
      P.convective_linearization != COVOF_CONV_LIN_AB2)
    return COVOF_UNSUPPORTED;
  if (P.linear_solver != COVOF_LINEAR_BICGSTAB && P.linear_solver != COVOF_LINEAR_BICGSTAB2 &&
      P.linear_solver != COVOF_LINEAR_CG)
    return COVOF_UNSUPPORTED;
  if (P.use_precond && P.precond != COVOF_PRECOND_NONE && P.precond != COVOF_PRECOND_JACOBI &&
      P.precond != COVOF_PRECOND_ILU0 && !uses_sweeps(P))
    return COVOF_INVALID;
  if (P.max_iter < 0) return COVOF_INVALID;
  return COVOF_OK;
}

int predictor_plan(covof_handle* h) {
  if (h->have_mplan) return COVOF_OK;
  const covof_params& P = h->prm;
  const void* fn = P.linear_solver == COVOF_LINEAR_BICGSTAB ? (const void*)k_bicgstab
                 : P.linear_solver == COVOF_LINEAR_CG ? (const void*)k_cg
                 : (const void*)k_bicgstab2;
  long long nseg = (long long)((P.nx + 1 + 31) / 32) * P.ny + (long long)((P.nx + 31) / 32) * (P.ny + 1);
  if (P.solver_type == COVOF_SOLVER_MONOLITHIC) nseg += (long long)((P.nx + 31) / 32) * P.ny;
  // two 512-thread blocks per SM where the registers allow: the Krylov
  // loops stream their vectors and coefficients from HBM, and a second
  // block doubles the loads in flight
  const int nb = coop_blocks(h, fn, kKrylovThreads, (nseg + kKrylovThreads / 32 - 1) / (kKrylovThreads / 32), 0,
                             kKrylovBlocksPerSm);
  if (nb < 1) return COVOF_CUDA_ERROR;
  h->m_fn = fn;
  h->m_nb = nb;
  h->have_mplan = true;
  return COVOF_OK;
}

// Predictor assembly (Jacobi diagonal, right-hand side, packed initial
// guess) on the handle's stream and the argument block of the Krylov solve.
int mom_pre(covof_handle* h, double dt, double* u, double* v, const double* rho_u, const double* rho_v,
            const double* mu, const double* mu_node, const double* fx, const double* fy, const double* u_old,
            const double* v_old, MomArgs* out) {
  const covof_params& P = h->prm;
  if (!u || !v || !rho_u || !rho_v || !mu || !mu_node || !fx || !fy || !u_old || !v_old) return COVOF_INVALID;
  CS(check_mom_params(P));
  CS(ensure_mom(h));
  CS(predictor_plan(h));
  // fields_old of the operator is the current field: the Krylov kernel only
  // writes its own vectors, u and v are overwritten after the solve.
  MomArgs& a = *out;
  a = mom_args(h, dt, u, v, rho_u, rho_v, mu, mu_node, fx, fy, u_old, v_old);
  const dim3 blk(32, 8), grd = grid2(P.nx + 1, P.ny + 1, blk);
  k_mom_diag<<<grd, blk, 0, h->stream>>>(a);
  k_mom_rhs<<<grd, blk, 0, h->stream>>>(a);
  k_mom_assemble<<<grd, blk, 0, h->stream>>>(a);
  k_mom_pack<<<grd, blk, 0, h->stream>>>(a, u, v);
  CK(cudaGetLastError());
  return COVOF_OK;
}

// The Krylov solve of a prepared argument block: the persistent kernel of
// the configured method, or with SSOR / BLOCK_TRIANGULAR the host-driven
// iterations over the sweep stencils (assembled here from a's fields).
int krylov_run(covof_handle* h, MomArgs& a) {
  if (uses_sweeps(h->prm)) {
    CS(prec_blocks_dev(h, a));
    return sweep_solve(h, a);
  }
  void* args[] = {&a};
  return launch_coop(h, h->m_fn, h->m_nb, kKrylovThreads, args, false);
}

// Solved velocities back into u, v, then the velocity boundary conditions.
int mom_post(covof_handle* h, const MomArgs& a, double* u, double* v) {
  const dim3 blk(32, 8), grd = grid2(h->prm.nx + 1, h->prm.ny + 1, blk);
  k_mom_unpack<<<grd, blk, 0, h->stream>>>(a, u, v);
  CK(cudaGetLastError());
  return velocity_bc_dev(h, u, v);
}

// ---------------------------------------------------------------------------
// Augmented Lagrangian coupling (solver_type AUGMENTED_LAGRANGIAN / AAL)
bool is_al(const covof_params& P) {
  return P.solver_type == COVOF_SOLVER_AUGMENTED_LAGRANGIAN || P.solver_type == COVOF_SOLVER_AAL;
}

int check_coupling(const covof_params& P) {
  if (P.solver_type == 0 || P.solver_type == COVOF_SOLVER_STANDARD_PROJECTION || is_al(P) ||
      P.solver_type == COVOF_SOLVER_MONOLITHIC)
    return COVOF_OK;
  if (P.solver_type == COVOF_SOLVER_CAAL) return COVOF_UNSUPPORTED;
  return COVOF_INVALID;
}

AlArgs al_args(covof_handle* h, double dt, const double* u, const double* v, double* p, const double* rho,
               const double* mu) {
  const covof_params& P = h->prm;
  AlArgs a;
  a.D = h->D; a.dx = P.dx; a.dy = P.dy; a.dt = dt;
  a.u = u; a.v = v; a.rho = rho; a.mu = mu; a.p = p; a.r = h->al_r; a.maxv = h->al_max;
  a.adaptive = P.adaptative_al ? 1 : 0;
  a.r_al = P.r_al; a.k_aal = P.k_aal;
  // src/module_navier_stokes.f90:1137-1147 (the domain lengths are nx dx, ny dy)
  const double lx = P.nx * P.dx, ly = P.ny * P.dy;
  if (P.l0_ref > 0.0) a.L0 = P.l0_ref;
  else if (P.enable_two_phase && P.ic_radius > 0.0) a.L0 = 2.0 * P.ic_radius;
  else a.L0 = fmin(lx, ly);
  a.t0 = P.t0_ref > 0.0 ? P.t0_ref : dt;
  a.g_norm = sqrt(P.gx * P.gx + P.gy * P.gy);
  a.sigma = P.enable_two_phase ? P.sigma : 0.0;
  a.alpha_time = (P.time_scheme == COVOF_TIME_GEAR && h->has_nm1) ? 1.5 : 1.0;
  a.u0_ref = P.u0_ref; a.p0_ref = P.p0_ref;
  a.mu_max = fmax(P.mu1, P.mu2);
  return a;
}

// src/module_simulation.f90:546-607: the penalty field, the preconditioner
// diagonal once (from the fields at the start of the coupling), then Uzawa
// iterations of rhs (with -grad p), assembly (linearised about the current
// u), pack, the Krylov solve, unpack + velocity BC and p -= r div u.  The
// max |div u| exit test (uzawa_iter > 1, uzawa_tol > 0) reads one scalar
// back per iteration (host_check); without it nothing waits for the host.
int al_enqueue(covof_handle* h, double dt, double* u, double* v, double* p, const double* rho,
               const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
               const double* fx, const double* fy, const double* u_old, const double* v_old, bool host_check,
               int* total_iters, int* uzawa_done) {
  const covof_params& P = h->prm;
  if (!u || !v || !p || !rho || !rho_u || !rho_v || !mu || !mu_node || !fx || !fy || !u_old || !v_old)
    return COVOF_INVALID;
  CS(check_mom_params(P));
  CS(ensure_mom(h));
  CS(predictor_plan(h));
  const dim3 blk(32, 8);
  const dim3 gc = grid2(P.nx, P.ny, blk), gg = grid2(P.nx + 2, P.ny + 2, blk), gf = grid2(P.nx + 1, P.ny + 1, blk);
  AlArgs al = al_args(h, dt, u, v, p, rho, mu);
  if (al.adaptive) {
    CK(cudaMemsetAsync(h->al_max, 0, 2 * sizeof(unsigned long long), h->stream));
    k_al_maxima<<<gc, blk, 0, h->stream>>>(al);
  }
  k_al_penalty<<<gg, blk, 0, h->stream>>>(al);
  MomArgs a = mom_args(h, dt, u, v, rho_u, rho_v, mu, mu_node, fx, fy, u_old, v_old);
  a.r_al = h->al_r;
  a.p_al = p;
  k_mom_diag<<<gf, blk, 0, h->stream>>>(a);
  CK(cudaGetLastError());
  // the preconditioner blocks once, from the fields at the coupling's start
  const bool sweeps = uses_sweeps(P);
  if (sweeps) CS(prec_blocks_dev(h, a));
  const int umax = P.uzawa_iter > 0 ? P.uzawa_iter : 1;
  int total = 0, done = 0, status = COVOF_OK;
  for (int m = 1; m <= umax; ++m) {
    done = m;
    k_mom_rhs<<<gf, blk, 0, h->stream>>>(a);
    k_mom_assemble<<<gf, blk, 0, h->stream>>>(a);
    k_mom_pack<<<gf, blk, 0, h->stream>>>(a, u, v);
    CK(cudaGetLastError());
    if (sweeps) {
      CS(sweep_solve(h, a));
    } else {
      void* args[] = {&a};
      CS(launch_coop(h, h->m_fn, h->m_nb, kKrylovThreads, args, false));
    }
    CS(mom_post(h, a, u, v));
    k_al_pressure<<<gc, blk, 0, h->stream>>>(al);
    CK(cudaGetLastError());
    if (host_check || total_iters) {
      CK(cudaMemcpyAsync(h->h_kres, h->d_kres, sizeof(KrylovResult), cudaMemcpyDeviceToHost, h->stream));
      unsigned long long dm = 0;
      if (host_check) {
        CK(cudaMemsetAsync(h->al_max + 2, 0, sizeof(unsigned long long), h->stream));
        k_al_divmax<<<gc, blk, 0, h->stream>>>(al);
        CK(cudaMemcpyAsync(&dm, h->al_max + 2, sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
      }
      CS(sync(h));
      total += h->h_kres->iters;
      if (h->h_kres->status != COVOF_OK) status = h->h_kres->status;
      if (status == COVOF_NAN || status == COVOF_TIMEOUT) break;
      double dmax;
      std::memcpy(&dmax, &dm, sizeof(double));
      if (host_check && umax > 1 && P.uzawa_tol > 0.0 && dmax <= P.uzawa_tol) break;
    }
  }
  if (total_iters) *total_iters = total;
  if (uzawa_done) *uzawa_done = done;
  return status;
}

// MONOLITHIC coupling, src/module_simulation.f90:552-583: the
// preconditioner blocks (momentum diagonals, then the Schur diagonal of the
// pressure block), the right-hand side (momentum without a pressure term,
// zero continuity block, src/module_navier_stokes.f90:1079-1100), assembly
// (linearised about the current u), pack (u, v, p), one Krylov solve of the
// coupled system, unpack (u, v, p) and the velocity boundary conditions.
// The Krylov result record is left on the device.
int mono_enqueue(covof_handle* h, double dt, double* u, double* v, double* p, const double* rho_u,
                 const double* rho_v, const double* mu, const double* mu_node, const double* fx, const double* fy,
                 const double* u_old, const double* v_old) {
  const covof_params& P = h->prm;
  if (!u || !v || !p || !rho_u || !rho_v || !mu || !mu_node || !fx || !fy || !u_old || !v_old)
    return COVOF_INVALID;
  if (P.solver_type != COVOF_SOLVER_MONOLITHIC) return COVOF_INVALID;
  CS(check_mom_params(P));
  CS(ensure_mom(h));
  CS(predictor_plan(h));
  const dim3 blk(32, 8);
  const dim3 gc = grid2(P.nx, P.ny, blk), gf = grid2(P.nx + 1, P.ny + 1, blk);
  MomArgs a = mom_args(h, dt, u, v, rho_u, rho_v, mu, mu_node, fx, fy, u_old, v_old);
  a.mono = 1;
  a.pm = p;
  k_mom_diag<<<gf, blk, 0, h->stream>>>(a);
  k_mono_diag<<<gc, blk, 0, h->stream>>>(a);
  k_mom_rhs<<<gf, blk, 0, h->stream>>>(a);
  CK(cudaMemsetAsync(a.rhs + 2 * h->g, 0, h->g * sizeof(double), h->stream));
  k_mom_assemble<<<gf, blk, 0, h->stream>>>(a);
  k_mom_pack<<<gf, blk, 0, h->stream>>>(a, u, v);
  CK(cudaGetLastError());
  CS(krylov_run(h, a));
  return mom_post(h, a, u, v);
}

// Predictor on the handle's stream, result record left on the device.
int predictor_enqueue(covof_handle* h, double dt, double* u, double* v, const double* rho_u,
                      const double* rho_v, const double* mu, const double* mu_node, const double* fx,
                      const double* fy, const double* u_old, const double* v_old) {
  MomArgs a;
  CS(mom_pre(h, dt, u, v, rho_u, rho_v, mu, mu_node, fx, fy, u_old, v_old, &a));
  CS(krylov_run(h, a));
  return mom_post(h, a, u, v);
}

int predictor_dev(covof_handle* h, double dt, double* u, double* v, const double* rho_u,
                  const double* rho_v, const double* mu, const double* mu_node, const double* fx,
                  const double* fy, const double* u_old, const double* v_old, int* iters) {
  CS(predictor_enqueue(h, dt, u, v, rho_u, rho_v, mu, mu_node, fx, fy, u_old, v_old));
  CK(cudaMemcpyAsync(h->h_kres, h->d_kres, sizeof(KrylovResult), cudaMemcpyDeviceToHost, h->stream));
  CS(sync(h));
  if (iters) *iters = h->h_kres->iters;
  return h->h_kres->status;
}

// ---------------------------------------------------------------------------
// VOF
VofArgs vof_args(covof_handle* h, double dt, const double* C, const double* Cn, const double* u,
                 const double* v) {
  VofArgs a;
  a.D = h->D; a.dx = h->prm.dx; a.dy = h->prm.dy; a.dt = dt; a.method = h->prm.recon;
  a.C = C; a.seg = h->seg; a.Cn = Cn; a.u = u; a.v = v;
  return a;
}

// Pure cells directly, interface cells by one of three forms chosen on the
// device-side count (the list is built on the device, so nothing here
// waits for the host; the forms that do not match return at once): ELVIRA
// lists of at most one wave of 128-thread blocks, one block per cell (the
// latency form); one warp per cell; from vof_cell_min(h) cells on, one
// thread per cell.  Then the ghost ring.
int reconstruct_dev(covof_handle* h, const double* C, double* seg_out) {
  CS(check_periodic_vof(h->prm));
  CS(ensure_vof(h));
  VofArgs a = vof_args(h, 0.0, C, C, nullptr, nullptr);
  if (seg_out) a.seg = seg_out;
  const dim3 blk(32, 4), grd = grid2(h->D.nx + 2, h->D.ny + 2, blk);
  CK(cudaMemsetAsync(h->vcount, 0, sizeof(int), h->stream));
  k_vof_classify<<<grd, blk, 0, h->stream>>>(a, h->vlist, h->vcount);
  const int cmin = vof_cell_min(h);
  const int bmax = h->prm.recon == COVOF_RECON_ELVIRA && h->vof_block_form
                       ? (cmin < 4 * h->sm_count ? cmin : 4 * h->sm_count) : 0;
  if (bmax > 0) k_vof_elvira_block<<<4 * h->sm_count, 128, 0, h->stream>>>(a, h->vlist, h->vcount, bmax);
  k_vof_mixed<<<4 * h->sm_count, 128, 0, h->stream>>>(a, h->vlist, h->vcount, bmax, cmin);
  k_vof_mixed_cell<<<h->vof_cell_nb, 128, 0, h->stream>>>(a, h->vlist, h->vcount, cmin);
  const int nring = 2 * h->D.ny + 2 * (h->D.nx + 2);
  k_vof_ring_warp<<<(nring + 3) / 4, 128, 0, h->stream>>>(a);
  CK(cudaGetLastError());
  return COVOF_OK;
}

// exchange_halos_scalar + apply_vof_bc (src/module_interface_vof.f90:809-810,
// 1238-1242): the exchange is the periodic wrap, nothing on a closed domain
int vof_bc_dev(covof_handle* h, double* C) {
  if (periodic(h->prm)) k_vof_halo_bc<<<1, 1024, 0, h->stream>>>(h->D, C, 1);
  else k_vof_bc<<<(h->D.nx + h->D.ny + 127) / 128, 128, 0, h->stream>>>(h->D, C);
  CK(cudaGetLastError());
  return COVOF_OK;
}

// src/module_interface_vof.f90:1162-1377
// The configured transport (src/module_interface_vof.f90:801-808): the
// geometric schemes reconstruct, pass, apply the VOF BC, reconstruct, pass;
// TVD is one explicit update.
int wy_step_dev(covof_handle* h, double dt, int x_first, const double* u, const double* v, double* C) {
  CS(check_periodic_vof(h->prm));
  CS(ensure_vof(h));
  const dim3 blk(32, 4), grd = grid2(h->D.nx + 2, h->D.ny + 2, blk);
  const int method = h->prm.advection_method;
  VofArgs a = vof_args(h, dt, C, C, u, v);
  if (method == COVOF_ADVECT_TVD) {
    CK(cudaMemcpyAsync(h->cs, C, h->g * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    k_tvd_advect<<<grd, blk, 0, h->stream>>>(a, h->prm.tvd_limiter, h->cs, C);
    CK(cudaGetLastError());
    return COVOF_OK;
  }
  const bool ciam = method == COVOF_ADVECT_CIAM;
  const int d1 = x_first ? 0 : 1, d2 = x_first ? 1 : 0;
  CS(reconstruct_dev(h, C, nullptr));
  if (ciam) k_ciam_pass<<<grd, blk, 0, h->stream>>>(a, d1, C, h->cs);
  else k_vof_pass<<<grd, blk, 0, h->stream>>>(a, d1, 0, C, h->cs);
  CK(cudaGetLastError());
  CS(vof_bc_dev(h, h->cs));
  CS(reconstruct_dev(h, h->cs, nullptr));
  a.C = h->cs;
  if (ciam) k_ciam_pass<<<grd, blk, 0, h->stream>>>(a, d2, h->cs, C);
  else k_vof_pass<<<grd, blk, 0, h->stream>>>(a, d2, 1, h->cs, C);
  CK(cudaGetLastError());
  return COVOF_OK;
}

int props_dev(covof_handle* h, double* C, double* rho, double* rho_u, double* rho_v, double* mu,
              double* mu_node, const double* Cs) {
  const covof_params& P = h->prm;
  PropsArgs a;
  a.D = h->D; a.two_phase = P.enable_two_phase;
  a.rho1 = P.rho1; a.rho2 = P.rho2; a.mu1 = P.mu1; a.mu2 = P.mu2;
  a.C = C; a.rho = rho; a.rho_u = rho_u; a.rho_v = rho_v; a.mu = mu; a.mu_node = mu_node;
  a.Cs = P.enable_svof_smoothing ? Cs : nullptr;
  const dim3 blk(32, 8);
  k_props_cells<<<grid2(h->D.nx + 2, h->D.ny + 2, blk), blk, 0, h->stream>>>(a);
  k_props_faces<<<grid2(h->D.nx + 1, h->D.ny + 1, blk), blk, 0, h->stream>>>(a);
  CK(cudaGetLastError());
  return COVOF_OK;
}

int csf_dev(covof_handle* h, const double* C, double* fx, double* fy, double* curv, const double* Cs,
            const double* Ct) {
  const covof_params& P = h->prm;
  if (!P.enable_surface_tension || P.sigma <= 0.0) {
    CK(cudaMemsetAsync(fx, 0, h->g * sizeof(double), h->stream));
    CK(cudaMemsetAsync(fy, 0, h->g * sizeof(double), h->stream));
    CK(cudaMemsetAsync(curv, 0, h->g * sizeof(double), h->stream));
    return COVOF_OK;
  }
  CS(ensure_vof(h));
  CsfArgs a;
  a.D = h->D; a.dx = P.dx; a.dy = P.dy; a.sigma = P.sigma;
  a.C = C; a.nxv = h->cnx; a.nyv = h->cny; a.kappa = h->ckap; a.fx = fx; a.fy = fy; a.curv = curv;
  // normals from C_tilde (diffusion smoothing), else C_s (SVOF), else C
  // (src/module_interface_vof.f90:682-690)
  a.N = (P.enable_diffusion_smoothing && Ct) ? Ct : (P.enable_svof_smoothing && Cs) ? Cs : C;
  const dim3 blk(32, 8);
  k_csf_normals<<<grid2(h->D.nx, h->D.ny, blk), blk, 0, h->stream>>>(a);
  k_csf_kappa<<<grid2(h->D.nx, h->D.ny, blk), blk, 0, h->stream>>>(a);
  k_csf_force<<<grid2(h->D.nx + 2, h->D.ny + 2, blk), blk, 0, h->stream>>>(a);
  CK(cudaGetLastError());
  return COVOF_OK;
}

// src/module_interface_vof.f90:387-476 smooth_svof_helmholtz: C_s = C, the
// wavefront Gauss-Seidel sweeps (svof.cu), then the clamp and ghost ring.
int svof_dev(covof_handle* h, const double* C, double* Cs) {
  if (periodic(h->prm)) return COVOF_UNSUPPORTED;
  CS(ensure_vof(h));
  const covof_params& P = h->prm;
  double kw = P.svof_filter_width;
  if (kw <= 0.0) kw = 1.0;
  const double Dw = kw * P.dx * P.dy;
  SvofArgs a;
  a.D = h->D; a.wx = Dw / (P.dx * P.dx); a.wy = Dw / (P.dy * P.dy);
  for (int f = 0; f < 16; ++f) {
    const double aE = (f & 1) ? 0.0 : a.wx, aW = (f & 2) ? 0.0 : a.wx;
    const double aN = (f & 4) ? 0.0 : a.wy, aS = (f & 8) ? 0.0 : a.wy;
    a.aP[f] = 1.0 + aE + aW + aN + aS;
    a.rP[f] = 1.0 / a.aP[f];
  }
  a.C = C; a.Cs = Cs; a.prog = h->svof_prog; a.err = h->err;
  const int nb = (h->D.ny + 31) / 32;
  CK(cudaMemcpyAsync(Cs, C, h->g * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemsetAsync(h->svof_prog, 0, (size_t)32 * nb * sizeof(unsigned int), h->stream));
  void* args[] = {&a};
  CS(launch_coop(h, (const void*)k_svof_sgs, h->svof_nb, 32, args, false));
  const dim3 blk(32, 8);
  k_svof_finish<<<grid2(h->D.nx + 2, h->D.ny + 2, blk), blk, 0, h->stream>>>(h->D, Cs);
  CK(cudaGetLastError());
  return COVOF_OK;
}

// src/module_interface_vof.f90:1416-1461 vof_smooth_diffusion: C -> C_tilde
int diffusion_dev(covof_handle* h, const double* C, double* Ct) {
  if (periodic(h->prm)) return COVOF_UNSUPPORTED;
  CS(ensure_vof(h));
  const covof_params& P = h->prm;
  int steps = P.diffusion_smoothing_steps;
  if (steps < 1) steps = 3;
  const double dtau = 0.2 * fmin(P.dx * P.dx, P.dy * P.dy);
  const dim3 blk(32, 8);
  // ping-pong so that the last step writes Ct; the interior of the first
  // source is C itself (ghost reads map to the interior)
  const double* src = C;
  for (int s = 0; s < steps; ++s) {
    double* dst = ((steps - 1 - s) % 2 == 0) ? Ct : h->dscr;
    k_diffusion_step<<<grid2(h->D.nx, h->D.ny, blk), blk, 0, h->stream>>>(h->D, dtau, P.dx * P.dx, P.dy * P.dy,
                                                                          src, dst);
    src = dst;
  }
  k_diffusion_ghosts<<<grid2(h->D.nx + 2, h->D.ny + 2, blk), blk, 0, h->stream>>>(h->D, Ct);
  CK(cudaGetLastError());
  return COVOF_OK;
}

// The interface-derived fields of the resident state after a VOF step
// (src/module_interface_vof.f90:811-824): C_s (SVOF, when svof_now),
// properties, C_tilde (diffusion smoothing), curvature + CSF.
int smooth_props_csf(covof_handle* h, bool svof_now) {
  const covof_params& P = h->prm;
  if (svof_now && P.enable_svof_smoothing) CS(svof_dev(h, h->f_C, h->f_Cs));
  CS(props_dev(h, h->f_C, h->f_rho, h->f_rho_u, h->f_rho_v, h->f_mu, h->f_mu_node, h->f_Cs));
  if (P.enable_diffusion_smoothing) CS(diffusion_dev(h, h->f_C, h->f_Ct));
  return csf_dev(h, h->f_C, h->f_fx, h->f_fy, h->f_curv, h->f_Cs, h->f_Ct);
}

int vof_advect_dev(covof_handle* h, double dt, const double* u, const double* v, double* C,
                   double* rho, double* rho_u, double* rho_v, double* mu, double* mu_node,
                   double* fx, double* fy, double* curv) {
  if (!u || !v || !C || !rho || !rho_u || !rho_v || !mu || !mu_node || !fx || !fy || !curv)
    return COVOF_INVALID;
  CS(ensure_fields(h));
  const covof_params& P = h->prm;
  CS(wy_step_dev(h, dt, (h->vof_step_count % 2) == 0, u, v, C));
  h->vof_step_count += 1;
  CS(vof_bc_dev(h, C));
  // the smoothed indicators are the handle's resident C_s / C_tilde
  if (P.enable_svof_smoothing) CS(svof_dev(h, C, h->f_Cs));
  CS(props_dev(h, C, rho, rho_u, rho_v, mu, mu_node, h->f_Cs));
  if (P.enable_diffusion_smoothing) CS(diffusion_dev(h, C, h->f_Ct));
  CS(csf_dev(h, C, fx, fy, curv, h->f_Cs, h->f_Ct));
  return COVOF_OK;
}

// ---------------------------------------------------------------------------
// Resident time stepping
double** field_slot(covof_handle* h, int f) {
  switch (f) {
    case COVOF_FIELD_U: return &h->f_u;
    case COVOF_FIELD_V: return &h->f_v;
    case COVOF_FIELD_P: return &h->f_p;
    case COVOF_FIELD_C: return &h->f_C;
    case COVOF_FIELD_RHO: return &h->f_rho;
    case COVOF_FIELD_RHO_U: return &h->f_rho_u;
    case COVOF_FIELD_RHO_V: return &h->f_rho_v;
    case COVOF_FIELD_MU: return &h->f_mu;
    case COVOF_FIELD_MU_NODE: return &h->f_mu_node;
    case COVOF_FIELD_FX_SIGMA: return &h->f_fx;
    case COVOF_FIELD_FY_SIGMA: return &h->f_fy;
    case COVOF_FIELD_CURVATURE: return &h->f_curv;
    case COVOF_FIELD_U_OLD: return &h->f_u_old;
    case COVOF_FIELD_V_OLD: return &h->f_v_old;
    case COVOF_FIELD_U_NM1: return &h->f_u_nm1;
    case COVOF_FIELD_V_NM1: return &h->f_v_nm1;
    case COVOF_FIELD_C_S: return &h->f_Cs;
    case COVOF_FIELD_C_TILDE: return &h->f_Ct;
    default: return nullptr;
  }
}

// Gear / BDF2 and Adams-Bashforth read the velocity of step n-1.
bool needs_history(const covof_params& P) {
  return P.time_scheme == COVOF_TIME_GEAR || P.convective_linearization == COVOF_CONV_LIN_AB2;
}

// u_nm1 = u_old (or u on a first step), src/module_simulation.f90:508-520;
// enqueued before u_old = u.
int rotate_history(covof_handle* h) {
  if (!needs_history(h->prm)) return COVOF_OK;
  const size_t bytes = h->g * sizeof(double);
  CK(cudaMemcpyAsync(h->f_u_nm1, h->has_nm1 ? h->f_u_old : h->f_u, bytes, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(h->f_v_nm1, h->has_nm1 ? h->f_v_old : h->f_v, bytes, cudaMemcpyDeviceToDevice, h->stream));
  return COVOF_OK;
}

// Everything a step launches, in stream order, with no host synchronisation
// (src/module_simulation.f90:492-559 for STANDARD_PROJECTION).
int enqueue_step(covof_handle* h, double dt, bool x_first) {
  const size_t bytes = h->g * sizeof(double);
  CS(rotate_history(h));
  CK(cudaMemcpyAsync(h->f_u_old, h->f_u, bytes, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(h->f_v_old, h->f_v, bytes, cudaMemcpyDeviceToDevice, h->stream));
  if (h->prm.enable_two_phase) {
    // advect_vof: Weymouth-Yue step, VOF BC, properties, curvature + CSF
    CS(wy_step_dev(h, dt, x_first ? 1 : 0, h->f_u, h->f_v, h->f_C));
    CS(vof_bc_dev(h, h->f_C));
    CS(smooth_props_csf(h, true));
    CS(velocity_bc_dev(h, h->f_u, h->f_v));
  }
  if (is_al(h->prm)) {
    CS(al_enqueue(h, dt, h->f_u, h->f_v, h->f_p, h->f_rho, h->f_rho_u, h->f_rho_v, h->f_mu, h->f_mu_node,
                  h->f_fx, h->f_fy, h->f_u_old, h->f_v_old, h->al_check, nullptr, nullptr));
    // no Poisson solve in this coupling: its record reads COVOF_OK, 0 iterations
    CK(cudaMemsetAsync(h->d_pres, 0, sizeof(PcgResult), h->stream));
  } else if (h->prm.solver_type == COVOF_SOLVER_MONOLITHIC) {
    CS(mono_enqueue(h, dt, h->f_u, h->f_v, h->f_p, h->f_rho_u, h->f_rho_v, h->f_mu, h->f_mu_node, h->f_fx,
                    h->f_fy, h->f_u_old, h->f_v_old));
    CK(cudaMemsetAsync(h->d_pres, 0, sizeof(PcgResult), h->stream));
  } else {
    CS(predictor_enqueue(h, dt, h->f_u, h->f_v, h->f_rho_u, h->f_rho_v, h->f_mu, h->f_mu_node, h->f_fx,
                         h->f_fy, h->f_u_old, h->f_v_old));
    CS(poisson_enqueue(h, dt, h->f_u, h->f_v, nullptr, h->f_rho_u, h->f_rho_v, h->f_p, false));
    CS(correct_dev(h, dt, h->f_u, h->f_v, h->f_p, h->f_rho_u, h->f_rho_v));
    CS(velocity_bc_dev(h, h->f_u, h->f_v));
  }
  k_step_log<<<1, 32, 0, h->stream>>>(h->d_kres, h->d_pres, h->d_run);
  CK(cudaGetLastError());
  return COVOF_OK;
}

void drop_graphs(covof_handle* h) {
  for (cudaGraphExec_t& g : h->step_graph) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
}

// Capture one step per Weymouth-Yue pass order.  Capture runs on a
// non-blocking stream of its own, so that no legacy-stream work of another
// library joins it.  COVOF_UNSUPPORTED: the driver refused the capture.
int capture_steps(covof_handle* h, double dt) {
  drop_graphs(h);
  for (int q = 0; q < 2; ++q) {
    cudaStream_t keep = h->stream;
    h->stream = h->cap_stream;
    cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
    int st = e == cudaSuccess ? enqueue_step(h, dt, q == 0) : COVOF_OK;
    cudaGraph_t g = nullptr;
    if (e == cudaSuccess) e = cudaStreamEndCapture(h->stream, &g);
    h->stream = keep;
    if (st == COVOF_OK && e == cudaSuccess && g) e = cudaGraphInstantiate(&h->step_graph[q], g, 0ULL);
    if (g) cudaGraphDestroy(g);
    if (st != COVOF_OK || e != cudaSuccess || !h->step_graph[q]) {
      cudaGetLastError();
      drop_graphs(h);
      return (st != COVOF_OK && st != COVOF_CUDA_ERROR) ? st : COVOF_UNSUPPORTED;
    }
  }
  h->graph_dt = dt;
  return COVOF_OK;
}

int run_steps(covof_handle* h, double dt, int nsteps, int flags, covof_run_stats* out) {
  if (nsteps < 0 || !(dt > 0.0)) return COVOF_INVALID;
  const covof_params& P = h->prm;
  if (P.p_precond == COVOF_PRECOND_SSOR && P.p_precision != COVOF_PREC_FP64) return COVOF_UNSUPPORTED;
  CS(check_mom_params(P));
  CS(check_coupling(P));
  // the Uzawa exit test reads a scalar back per iteration: eager steps
  h->al_check = is_al(P) && P.uzawa_iter > 1 && P.uzawa_tol > 0.0;
  if (h->al_check) flags &= ~COVOF_RUN_GRAPH;
  // the sweep preconditioners' Krylov iterations are driven from the host
  if (uses_sweeps(P) || P.p_precond == COVOF_PRECOND_SSOR) flags &= ~COVOF_RUN_GRAPH;
  // every buffer and launch plan exists before a capture starts
  CS(ensure_fields(h));
  CS(ensure_poisson(h));
  CS(poisson_plan(h));
  CS(ensure_mom(h));
  CS(predictor_plan(h));
  CS(ensure_vof(h));
  *h->h_run = RunStats{0, 0, 0, 0.0, 0.0, 0, -1, COVOF_OK, 0};
  CK(cudaMemcpyAsync(h->d_run, h->h_run, sizeof(RunStats), cudaMemcpyHostToDevice, h->stream));
  bool graph = (flags & COVOF_RUN_GRAPH) != 0 && !h->graph_refused;
  // A step without history (the first of a Gear / Adams-Bashforth run)
  // differs from the later ones: it runs eagerly, and the graphs are
  // captured with has_nm1 set.
  const bool first_plain = needs_history(P) && !h->has_nm1 && nsteps > 0;
  auto ensure_graphs = [&]() -> int {
    if (graph && (!h->step_graph[0] || h->graph_dt != dt)) {
      const int st = capture_steps(h, dt);
      if (st == COVOF_UNSUPPORTED) {
        h->graph_refused = true;
        graph = false;
      } else if (st != COVOF_OK) {
        return st;
      }
    }
    return COVOF_OK;
  };
  if (!first_plain) CS(ensure_graphs());
  CK(cudaEventRecord(h->ev2, h->stream));
  for (int k = 0; k < nsteps; ++k) {
    const bool x_first = (h->vof_step_count % 2) == 0;
    if (graph && !(first_plain && k == 0)) CK(cudaGraphLaunch(h->step_graph[x_first ? 0 : 1], h->stream));
    else CS(enqueue_step(h, dt, x_first));
    if (P.enable_two_phase) h->vof_step_count += 1;
    if (!h->has_nm1) {
      h->has_nm1 = true;
      if (first_plain) {
        drop_graphs(h);
        CS(ensure_graphs());
      }
    }
  }
  CK(cudaEventRecord(h->ev3, h->stream));
  CK(cudaMemcpyAsync(h->h_run, h->d_run, sizeof(RunStats), cudaMemcpyDeviceToHost, h->stream));
  CS(sync(h));
  const RunStats& r = *h->h_run;
  if (out) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev2, h->ev3);
    cudaGetLastError();
    out->steps = r.step;
    out->first_bad_step = r.first_bad_step;
    out->first_bad_status = r.first_bad_status;
    out->graph = graph ? 1 : 0;
    out->mom_iters = r.mom_iters;
    out->poisson_iters = r.poisson_iters;
    out->refine_steps = r.refine_steps;
    out->last_relres = r.last_relres;
    out->max_relres = r.max_relres;
    out->ms = ms;
  }
  return r.first_bad_step < 0 ? COVOF_OK : r.first_bad_status;
}

}  // namespace host
}  // namespace covof

using namespace covof::host;

// ===========================================================================
extern "C" {

void covof_params_default(covof_params* p, int nx, int ny, double lx, double ly) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->nx = nx; p->ny = ny;
  p->dx = nx > 0 ? lx / (double)nx : 0.0;
  p->dy = ny > 0 ? ly / (double)ny : 0.0;
  for (int s = 0; s < 4; ++s) { p->bc_type[s] = COVOF_BC_DIRICHLET; p->bc_u[s] = 0.0; p->bc_v[s] = 0.0; }
  p->linear_solver = COVOF_LINEAR_BICGSTAB2;
  p->precond = COVOF_PRECOND_JACOBI;
  p->use_precond = 1;
  p->max_iter = 300;
  p->tol = 1.0e-5;
  p->enable_convection = 1;
  p->convective_scheme = COVOF_CONV_UPWIND;
  p->p_precond = COVOF_PRECOND_JACOBI;
  p->p_max_iter = 1000;
  p->p_gauge = COVOF_GAUGE_REFERENCE;
  p->p_precision = COVOF_PREC_FP64;
  p->p_tol = 1.0e-7;
  p->p_inner_tol = 1.0e-4;
  p->p_inner_max_iter = 32;
  p->p_max_refine = 1000000;
  p->enable_two_phase = 0;
  p->enable_surface_tension = 0;
  p->rho1 = 1.0; p->rho2 = 1.0; p->mu1 = 1.0e-3; p->mu2 = 1.0e-3;
  p->sigma = 0.0; p->gx = 0.0; p->gy = 0.0;
  p->recon = COVOF_RECON_PLIC;
  p->p_inner_kind = COVOF_INNER_MG;
  p->p_cheb_lo = 1.0e-3;
  p->p_mg_nu = 2;
  p->p_mg_cw = 2.0;
  p->p_mg_tail = 2048;
  p->time_scheme = COVOF_TIME_EULER;
  p->convective_linearization = COVOF_CONV_LIN_PICARD;
  p->enable_svof_smoothing = 0;
  p->svof_filter_width = 1.0;
  p->enable_diffusion_smoothing = 0;
  p->diffusion_smoothing_steps = 3;
  p->advection_method = COVOF_ADVECT_WEYMOUTH_YUE;
  p->tvd_limiter = COVOF_LIMITER_SUPERBEE;
  p->solver_type = COVOF_SOLVER_STANDARD_PROJECTION;
  p->r_al = 100.0;
  p->adaptative_al = 0;
  p->k_aal = 100.0;
  p->l0_ref = p->t0_ref = p->u0_ref = p->p0_ref = 0.0;
  p->ic_radius = 0.25;
  p->uzawa_iter = 1;
  p->uzawa_tol = 1.0e-12;
  p->p_mg_nuc = -1;
}

int covof_abi_version(void) { return COVOF_ABI_VERSION; }

int covof_bounds_check(long long* bad, long long* first) {
  if (!bad || !first) return COVOF_INVALID;
  int (*const get[])(unsigned long long*, unsigned long long*) = {
      bounds_check_poisson, bounds_check_momentum, bounds_check_vof, bounds_check_svof,
      bounds_check_adjoint, bounds_check_output, bounds_check_precond, bounds_check_peak,
      bounds_check_batch, bounds_check_capi, bounds_check_static_scratch};
  *bad = 0;
  *first = 0;
  for (auto f : get) {
    unsigned long long c = 0, w = 0;
    const int st = f(&c, &w);
    if (st != COVOF_OK) return st;  // COVOF_UNSUPPORTED: not a checked build
    if (c && !*first) *first = (long long)w;
    *bad += (long long)c;
  }
  return COVOF_OK;
}

int covof_set_wait_budget(long long polls) {
  if (polls < 0) return COVOF_INVALID;
  const long long v = polls == 0 ? kSpinLimit : polls;
  int (*const set[])(long long) = {set_wait_budget_poisson, set_wait_budget_momentum, set_wait_budget_vof,
                                    set_wait_budget_svof, set_wait_budget_adjoint, set_wait_budget_output,
                                    set_wait_budget_precond, set_wait_budget_peak, set_wait_budget_batch,
                                    set_wait_budget_capi, set_wait_budget_static_scratch};
  for (auto f : set) CS(f(v));
  return COVOF_OK;
}

const char* covof_strerror(int s) {
  switch (s) {
    case COVOF_OK: return "ok";
    case COVOF_MAXITER: return "iteration cap reached before the tolerance";
    case COVOF_BREAKDOWN: return "Krylov breakdown";
    case COVOF_NAN: return "NaN or divergence in the residual";
    case COVOF_TIMEOUT: return "a bounded device-side wait gave up";
    case COVOF_UNSUPPORTED: return "option not implemented on this path";
    case COVOF_CUDA_ERROR: return "CUDA error";
    case COVOF_INVALID: return "invalid argument";
    case COVOF_TOO_LARGE: return "mesh larger than the fixed scratch of the allocation-free entry point";
    default: return "unknown status";
  }
}

int covof_create(const covof_params* params, covof_handle** out) {
  if (!out) return COVOF_INVALID;
  *out = nullptr;
  int st = check_params(params);
  if (st != COVOF_OK) return st;
  covof_handle* h = new (std::nothrow) covof_handle();
  if (!h) return COVOF_INVALID;
  h->prm = *params;
  h->D = Dims{params->nx, params->ny, params->nx + 2};
  h->D.perx = params->bc_type[0] == COVOF_BC_PERIODIC ? 1 : 0;
  h->D.pery = params->bc_type[2] == COVOF_BC_PERIODIC ? 1 : 0;
  h->g = (size_t)(params->nx + 2) * (size_t)(params->ny + 2);
  auto fail = [&](int code) { covof_destroy(h); return code; };
  if (cudaGetDevice(&h->device) != cudaSuccess) return fail(COVOF_CUDA_ERROR);
  if (cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess)
    return fail(COVOF_CUDA_ERROR);
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->device);
  if (!coop) return fail(COVOF_UNSUPPORTED);
  if (cudaStreamCreate(&h->stream) != cudaSuccess) return fail(COVOF_CUDA_ERROR);
  if (cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(COVOF_CUDA_ERROR);
  if (cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess ||
      cudaEventCreate(&h->ev2) != cudaSuccess || cudaEventCreate(&h->ev3) != cudaSuccess)
    return fail(COVOF_CUDA_ERROR);
  h->part_blocks = kKrylovBlocksPerSm * h->sm_count;  // most blocks of a persistent launch
  if (dalloc(&h->bar, (size_t)64 + h->sm_count) || dalloc(&h->err, 1) ||
      dalloc(&h->part, (size_t)kMaxPartRegions * h->part_blocks) ||
      dalloc(&h->d_pres, 1) || dalloc(&h->d_kres, 1) || dalloc(&h->d_run, 1))
    return fail(COVOF_CUDA_ERROR);
  if (cudaMallocHost(&h->h_pres, sizeof(PcgResult)) != cudaSuccess ||
      cudaMallocHost(&h->h_kres, sizeof(KrylovResult)) != cudaSuccess ||
      cudaMallocHost(&h->h_run, sizeof(RunStats)) != cudaSuccess)
    return fail(COVOF_CUDA_ERROR);
  *out = h;
  return COVOF_OK;
}

int covof_destroy(covof_handle* h) {
  if (!h) return COVOF_INVALID;
  writer_destroy(h);
  if (h->stream) cudaStreamSynchronize(h->stream);
  sweep_free(h);
  double** fl[] = {&h->f_u, &h->f_v, &h->f_p, &h->f_rho_u, &h->f_rho_v, &h->f_mu, &h->f_mu_node,
                   &h->f_fx, &h->f_fy, &h->f_u_old, &h->f_v_old, &h->f_u_nm1, &h->f_v_nm1, &h->f_Cs, &h->f_Ct, &h->dscr, &h->al_r,
                   &h->f_C, &h->f_rho, &h->f_curv,
                   &h->f_b, &h->f_x2, &h->f_seg, &h->px, &h->pb, &h->pr, &h->pd, &h->pAd,
                   &h->pax, &h->pay, &h->paP, &h->pisd, &h->pinvD, &h->pd2, &h->pz, &h->pw, &h->pp, &h->pq, &h->mx, &h->mrhs, &h->mdiag, &h->cs, &h->seg, &h->mcoef, &h->midiag,
                   &h->cnx, &h->cny, &h->ckap, &h->part, &h->arhs, &h->apsi, &h->apart, &h->asum,
                   &h->f_gu, &h->f_gv, &h->f_gp, &h->f_gbu, &h->f_gbv, &h->f_ou, &h->f_ov};
  for (double** q : fl) dfree(*q);
  for (int q = 0; q < 7; ++q) dfree(h->mv[q]);
  float** ff[] = {&h->pxb, &h->e32, &h->r32b, &h->r32, &h->d32, &h->d32b, &h->Ad32, &h->ax32, &h->ay32, &h->aP32};
  for (float** q : ff) dfree(*q);
  drop_graphs(h);
  dfree(h->bar); dfree(h->err); dfree(h->d_pres); dfree(h->d_kres); dfree(h->d_run);
  dfree(h->vlist); dfree(h->vcount); dfree(h->mg.pool); dfree(h->pin_part); dfree(h->pin_ctl); dfree(h->pin_b);
  if (h->h_pres) cudaFreeHost(h->h_pres);
  if (h->h_kres) cudaFreeHost(h->h_kres);
  if (h->h_run) cudaFreeHost(h->h_run);
  for (cudaEvent_t e : {h->ev0, h->ev1, h->ev2, h->ev3})
    if (e) cudaEventDestroy(e);
  if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return COVOF_OK;
}

int covof_device_info(const covof_handle* h, int* device, int* sm_count) {
  if (!h) return COVOF_INVALID;
  if (device) *device = h->device;
  if (sm_count) *sm_count = h->sm_count;
  return COVOF_OK;
}

int covof_get_stream(const covof_handle* h, void** stream) {
  if (!h || !stream) return COVOF_INVALID;
  *stream = (void*)h->stream;
  return COVOF_OK;
}

int covof_last_solve_ms(const covof_handle* h, double* ms) {
  if (!h || !ms) return COVOF_INVALID;
  *ms = h->last_solve_ms;
  return COVOF_OK;
}

int covof_last_refine_steps(const covof_handle* h, int* steps) {
  if (!h || !steps) return COVOF_INVALID;
  *steps = h->last_refine;
  return COVOF_OK;
}

int covof_get_vof_step_count(const covof_handle* h, int* count) {
  if (!h || !count) return COVOF_INVALID;
  *count = h->vof_step_count;
  return COVOF_OK;
}
int covof_set_vof_step_count(covof_handle* h, int count) {
  if (!h || count < 0) return COVOF_INVALID;
  h->vof_step_count = count;
  return COVOF_OK;
}

// ---- Poisson ---------------------------------------------------------------
int covof_poisson_solve_dev(covof_handle* h, double dt, const double* u_star, const double* v_star,
                            const double* rho_u, const double* rho_v, double* p, int* iters,
                            double* relres) {
  if (!h) return COVOF_INVALID;
  return poisson_dev(h, dt, u_star, v_star, nullptr, rho_u, rho_v, p, iters, relres);
}

int covof_poisson_solve_rhs_dev(covof_handle* h, double dt, const double* b, const double* rho_u,
                                const double* rho_v, double* p, int* iters, double* relres) {
  if (!h || !b) return COVOF_INVALID;
  return poisson_dev(h, dt, nullptr, nullptr, b, rho_u, rho_v, p, iters, relres);
}

int covof_poisson_solve(covof_handle* h, double dt, const double* u_star, const double* v_star,
                        const double* rho_u, const double* rho_v, double* p, int* iters,
                        double* relres) {
  if (!h) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_u, u_star, g)); CS(h2d(h, h->f_v, v_star, g));
  CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g)); CS(h2d(h, h->f_p, p, g));
  int st = poisson_dev(h, dt, h->f_u, h->f_v, nullptr, h->f_rho_u, h->f_rho_v, h->f_p, iters, relres);
  if (st == COVOF_CUDA_ERROR || st == COVOF_INVALID || st == COVOF_UNSUPPORTED) return st;
  CS(d2h(h, p, h->f_p, g));
  CS(sync(h));
  return st;
}

int covof_poisson_solve_rhs(covof_handle* h, double dt, const double* b, const double* rho_u,
                            const double* rho_v, double* p, int* iters, double* relres) {
  if (!h) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_b, b, g));
  CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g)); CS(h2d(h, h->f_p, p, g));
  int st = poisson_dev(h, dt, nullptr, nullptr, h->f_b, h->f_rho_u, h->f_rho_v, h->f_p, iters, relres);
  if (st == COVOF_CUDA_ERROR || st == COVOF_INVALID || st == COVOF_UNSUPPORTED) return st;
  CS(d2h(h, p, h->f_p, g));
  CS(sync(h));
  return st;
}

// y = A x on device arrays: assembly from rho_u, rho_v, the operand's
// interior into a solver vector with a zero ghost ring (as inside the
// solvers), then the stencil; y's interior written.
int poisson_apply_enqueue(covof_handle* h, double dt, const double* rho_u, const double* rho_v, const double* x,
                          double* y) {
  CS(ensure_poisson(h));
  const covof_params& P = h->prm;
  const size_t g = h->g;
  const dim3 blk(32, 8), grd = grid2(P.nx, P.ny, blk);
  // only the coefficients are used: the right-hand side slot reads y
  k_poisson_assemble<<<grd, blk, 0, h->stream>>>(h->D, dt, P.dx, P.dy, wall_flags(P), rho_u, rho_v,
                                                  nullptr, nullptr, y, 0, h->pax, h->pay, h->paP,
                                                  h->pb, nullptr, nullptr);
  CK(cudaMemsetAsync(h->px, 0, g * sizeof(double), h->stream));
  k_copy_interior<<<grd, blk, 0, h->stream>>>(h->D, x, h->px, 0);
  if (periodic(P)) k_wrap_ghosts<<<1, 1024, 0, h->stream>>>(h->D, h->px);
  k_poisson_apply<<<grd, blk, 0, h->stream>>>(h->D, h->px, y, h->pax, h->pay, h->paP);
  CK(cudaGetLastError());
  return COVOF_OK;
}

int covof_poisson_apply(covof_handle* h, double dt, const double* rho_u, const double* rho_v,
                        const double* x, double* y) {
  if (!h || !rho_u || !rho_v || !x || !y) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g));
  CS(h2d(h, h->f_p, x, g)); CS(h2d(h, h->f_b, y, g));
  CS(poisson_apply_enqueue(h, dt, h->f_rho_u, h->f_rho_v, h->f_p, h->f_b));
  CS(d2h(h, y, h->f_b, g));
  CS(sync(h));
  return COVOF_OK;
}

int covof_poisson_apply_dev(covof_handle* h, double dt, const double* rho_u, const double* rho_v,
                            const double* x, double* y) {
  if (!h || !rho_u || !rho_v || !x || !y) return COVOF_INVALID;
  CS(poisson_apply_enqueue(h, dt, rho_u, rho_v, x, y));
  CS(sync(h));
  return COVOF_OK;
}

int covof_project_correct(covof_handle* h, double dt, double* u, double* v, const double* p,
                          const double* rho_u, const double* rho_v) {
  if (!h) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_u, u, g)); CS(h2d(h, h->f_v, v, g)); CS(h2d(h, h->f_p, p, g));
  CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g));
  CS(correct_dev(h, dt, h->f_u, h->f_v, h->f_p, h->f_rho_u, h->f_rho_v));
  CS(d2h(h, u, h->f_u, g)); CS(d2h(h, v, h->f_v, g));
  return sync(h);
}

// ---- projection adjoint ------------------------------------------------------
int covof_projection_dev(covof_handle* h, double dt, const double* u_star, const double* v_star,
                         const double* rho_u, const double* rho_v, double* p, double* u, double* v,
                         int* iters, double* relres) {
  if (!h) return COVOF_INVALID;
  return projection_dev(h, dt, u_star, v_star, rho_u, rho_v, p, u, v, iters, relres);
}

int covof_projection(covof_handle* h, double dt, const double* u_star, const double* v_star,
                     const double* rho_u, const double* rho_v, double* p, double* u, double* v,
                     int* iters, double* relres) {
  if (!h) return COVOF_INVALID;
  CS(ensure_fields(h));
  CS(ensure_adj_host(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_u, u_star, g)); CS(h2d(h, h->f_v, v_star, g));
  CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g)); CS(h2d(h, h->f_p, p, g));
  CS(h2d(h, h->f_ou, u, g)); CS(h2d(h, h->f_ov, v, g));
  int st = projection_dev(h, dt, h->f_u, h->f_v, h->f_rho_u, h->f_rho_v, h->f_p, h->f_ou, h->f_ov, iters, relres);
  if (st == COVOF_CUDA_ERROR || st == COVOF_INVALID || st == COVOF_UNSUPPORTED || st == COVOF_TIMEOUT) return st;
  CS(d2h(h, p, h->f_p, g)); CS(d2h(h, u, h->f_ou, g)); CS(d2h(h, v, h->f_ov, g));
  CS(sync(h));
  return st;
}

int covof_projection_vjp_dev(covof_handle* h, double dt, const double* rho_u, const double* rho_v,
                             const double* p, const double* gu, const double* gv, const double* gp,
                             double* grad_u, double* grad_v, double* grad_bu, double* grad_bv,
                             int* iters, double* relres) {
  if (!h) return COVOF_INVALID;
  return vjp_dev(h, dt, rho_u, rho_v, p, gu, gv, gp, grad_u, grad_v, grad_bu, grad_bv, iters, relres);
}

int covof_projection_vjp(covof_handle* h, double dt, const double* rho_u, const double* rho_v,
                         const double* p, const double* gu, const double* gv, const double* gp,
                         double* grad_u, double* grad_v, double* grad_bu, double* grad_bv,
                         int* iters, double* relres) {
  if (!h) return COVOF_INVALID;
  CS(ensure_fields(h));
  CS(ensure_adj_host(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g)); CS(h2d(h, h->f_p, p, g));
  CS(h2d(h, h->f_gu, gu, g)); CS(h2d(h, h->f_gv, gv, g));
  if (gp) CS(h2d(h, h->f_gp, gp, g));
  CS(h2d(h, h->f_ou, grad_u, g)); CS(h2d(h, h->f_ov, grad_v, g));
  CS(h2d(h, h->f_gbu, grad_bu, g)); CS(h2d(h, h->f_gbv, grad_bv, g));
  int st = vjp_dev(h, dt, h->f_rho_u, h->f_rho_v, h->f_p, h->f_gu, h->f_gv, gp ? h->f_gp : nullptr,
                   h->f_ou, h->f_ov, h->f_gbu, h->f_gbv, iters, relres);
  if (st == COVOF_CUDA_ERROR || st == COVOF_INVALID || st == COVOF_UNSUPPORTED || st == COVOF_TIMEOUT) return st;
  CS(d2h(h, grad_u, h->f_ou, g)); CS(d2h(h, grad_v, h->f_ov, g));
  CS(d2h(h, grad_bu, h->f_gbu, g)); CS(d2h(h, grad_bv, h->f_gbv, g));
  CS(sync(h));
  return st;
}

// ---- momentum --------------------------------------------------------------
int covof_predictor_dev(covof_handle* h, double dt, double* u, double* v, const double* rho_u,
                        const double* rho_v, const double* mu, const double* mu_node,
                        const double* fx_sigma, const double* fy_sigma, const double* u_old,
                        const double* v_old, int* iters) {
  if (!h) return COVOF_INVALID;
  return predictor_dev(h, dt, u, v, rho_u, rho_v, mu, mu_node, fx_sigma, fy_sigma, u_old, v_old, iters);
}

int covof_predictor(covof_handle* h, double dt, double* u, double* v, const double* rho_u,
                    const double* rho_v, const double* mu, const double* mu_node,
                    const double* fx_sigma, const double* fy_sigma, const double* u_old,
                    const double* v_old, int* iters) {
  if (!h) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_u, u, g)); CS(h2d(h, h->f_v, v, g));
  CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g));
  CS(h2d(h, h->f_mu, mu, g)); CS(h2d(h, h->f_mu_node, mu_node, g));
  CS(h2d(h, h->f_fx, fx_sigma, g)); CS(h2d(h, h->f_fy, fy_sigma, g));
  CS(h2d(h, h->f_u_old, u_old, g)); CS(h2d(h, h->f_v_old, v_old, g));
  int st = predictor_dev(h, dt, h->f_u, h->f_v, h->f_rho_u, h->f_rho_v, h->f_mu, h->f_mu_node,
                         h->f_fx, h->f_fy, h->f_u_old, h->f_v_old, iters);
  if (st == COVOF_CUDA_ERROR || st == COVOF_INVALID || st == COVOF_UNSUPPORTED) return st;
  CS(d2h(h, u, h->f_u, g)); CS(d2h(h, v, h->f_v, g));
  CS(sync(h));
  return st;
}

int covof_momentum_apply(covof_handle* h, double dt, const double* xu, const double* xv,
                         double* yu, double* yv, const double* u_n, const double* v_n,
                         const double* rho_u, const double* rho_v, const double* mu,
                         const double* mu_node) {
  if (!h || !xu || !xv || !yu || !yv) return COVOF_INVALID;
  CS(check_mom_params(h->prm));
  CS(ensure_fields(h));
  CS(ensure_mom(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_u, u_n, g)); CS(h2d(h, h->f_v, v_n, g));
  CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g));
  CS(h2d(h, h->f_mu, mu, g)); CS(h2d(h, h->f_mu_node, mu_node, g));
  CS(h2d(h, h->f_x2, xu, g)); CS(h2d(h, h->f_x2 + g, xv, g));
  double* y = h->mv[0];  // 2g doubles
  CS(h2d(h, y, yu, g)); CS(h2d(h, y + g, yv, g));
  // u_old / v_old / u_nm1 / v_nm1 (Adams-Bashforth, Gear) are the resident fields
  MomArgs a = mom_args(h, dt, h->f_u, h->f_v, h->f_rho_u, h->f_rho_v, h->f_mu, h->f_mu_node,
                       nullptr, nullptr, h->f_u_old, h->f_v_old);
  const dim3 blk(32, 8), grd = grid2(h->prm.nx + 1, h->prm.ny + 1, blk);
  k_mom_apply<<<grd, blk, 0, h->stream>>>(a, h->f_x2, h->f_x2 + g, y, y + g);
  CK(cudaGetLastError());
  CS(d2h(h, yu, y, g)); CS(d2h(h, yv, y + g, g));
  return sync(h);
}

int covof_precond_apply(covof_handle* h, double dt, const double* zu, const double* zv, const double* zp,
                        double* yu, double* yv, double* yp, const double* u_n, const double* v_n,
                        const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                        const double* r_al) {
  const bool mono = h && h->prm.solver_type == COVOF_SOLVER_MONOLITHIC;
  if (!h || !zu || !zv || !yu || !yv || (mono && (!zp || !yp))) return COVOF_INVALID;
  CS(check_mom_params(h->prm));
  CS(ensure_fields(h));
  CS(ensure_mom(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_u, u_n, g)); CS(h2d(h, h->f_v, v_n, g));
  CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g));
  CS(h2d(h, h->f_mu, mu, g)); CS(h2d(h, h->f_mu_node, mu_node, g));
  double* z = h->mv[0];
  double* y = h->mv[1];
  CK(cudaMemsetAsync(z, 0, (mono ? 3 : 2) * g * sizeof(double), h->stream));
  CS(h2d(h, z, zu, g)); CS(h2d(h, z + g, zv, g));
  if (mono) CS(h2d(h, z + 2 * g, zp, g));
  MomArgs a = mom_args(h, dt, h->f_u, h->f_v, h->f_rho_u, h->f_rho_v, h->f_mu, h->f_mu_node, nullptr, nullptr,
                       h->f_u_old, h->f_v_old);
  a.mono = mono ? 1 : 0;
  if (is_al(h->prm) && r_al) {
    CS(h2d(h, h->al_r, r_al, g));
    a.r_al = h->al_r;
  }
  const dim3 blk(32, 8), gf = grid2(h->prm.nx + 1, h->prm.ny + 1, blk), gc = grid2(h->prm.nx, h->prm.ny, blk);
  k_mom_diag<<<gf, blk, 0, h->stream>>>(a);
  if (mono) k_mono_diag<<<gc, blk, 0, h->stream>>>(a);
  k_mom_assemble<<<gf, blk, 0, h->stream>>>(a);
  CK(cudaGetLastError());
  CK(cudaMemsetAsync(h->err, 0, sizeof(int), h->stream));
  CS(precond_apply_dev(h, a, z, y));
  CS(d2h(h, yu, y, g)); CS(d2h(h, yv, y + g, g));
  if (mono) CS(d2h(h, yp, y + 2 * g, g));
  int e = 0;
  CK(cudaMemcpyAsync(&e, h->err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CS(sync(h));
  return e != 0 ? COVOF_TIMEOUT : COVOF_OK;
}

// ---- SP step -----------------------------------------------------------------
int covof_sp_step_dev(covof_handle* h, double dt, double* u, double* v, double* p,
                      const double* rho_u, const double* rho_v, const double* mu,
                      const double* mu_node, const double* fx_sigma, const double* fy_sigma,
                      const double* u_old, const double* v_old, int* total_iters,
                      double* final_relres) {
  if (!h || !p) return COVOF_INVALID;
  int iu = 0, ip = 0;
  double rr = 0.0;
  int s1 = predictor_dev(h, dt, u, v, rho_u, rho_v, mu, mu_node, fx_sigma, fy_sigma, u_old, v_old, &iu);
  if (s1 == COVOF_CUDA_ERROR || s1 == COVOF_INVALID || s1 == COVOF_UNSUPPORTED || s1 == COVOF_TIMEOUT ||
      s1 == COVOF_NAN)
    return s1;
  int s2 = poisson_dev(h, dt, u, v, nullptr, rho_u, rho_v, p, &ip, &rr);
  if (s2 == COVOF_CUDA_ERROR || s2 == COVOF_INVALID || s2 == COVOF_UNSUPPORTED || s2 == COVOF_TIMEOUT)
    return s2;
  CS(correct_dev(h, dt, u, v, p, rho_u, rho_v));
  CS(velocity_bc_dev(h, u, v));
  CS(sync(h));
  if (total_iters) *total_iters = iu + ip;
  if (final_relres) *final_relres = rr;
  return s2 != COVOF_OK ? s2 : s1;
}

int covof_sp_step(covof_handle* h, double dt, double* u, double* v, double* p,
                  const double* rho_u, const double* rho_v, const double* mu,
                  const double* mu_node, const double* fx_sigma, const double* fy_sigma,
                  const double* u_old, const double* v_old, int* total_iters,
                  double* final_relres) {
  if (!h) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_u, u, g)); CS(h2d(h, h->f_v, v, g)); CS(h2d(h, h->f_p, p, g));
  CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g));
  CS(h2d(h, h->f_mu, mu, g)); CS(h2d(h, h->f_mu_node, mu_node, g));
  CS(h2d(h, h->f_fx, fx_sigma, g)); CS(h2d(h, h->f_fy, fy_sigma, g));
  CS(h2d(h, h->f_u_old, u_old, g)); CS(h2d(h, h->f_v_old, v_old, g));
  int st = covof_sp_step_dev(h, dt, h->f_u, h->f_v, h->f_p, h->f_rho_u, h->f_rho_v, h->f_mu,
                             h->f_mu_node, h->f_fx, h->f_fy, h->f_u_old, h->f_v_old, total_iters,
                             final_relres);
  if (st == COVOF_CUDA_ERROR || st == COVOF_INVALID || st == COVOF_UNSUPPORTED || st == COVOF_TIMEOUT)
    return st;
  CS(d2h(h, u, h->f_u, g)); CS(d2h(h, v, h->f_v, g)); CS(d2h(h, p, h->f_p, g));
  CS(sync(h));
  return st;
}

// ---- augmented Lagrangian step -------------------------------------------------
int covof_al_step(covof_handle* h, double dt, double* u, double* v, double* p, const double* rho,
                  const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
                  const double* fx_sigma, const double* fy_sigma, const double* u_old, const double* v_old,
                  int* total_iters, int* uzawa_done) {
  if (!h) return COVOF_INVALID;
  if (!is_al(h->prm)) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_u, u, g)); CS(h2d(h, h->f_v, v, g)); CS(h2d(h, h->f_p, p, g));
  CS(h2d(h, h->f_rho, rho, g)); CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g));
  CS(h2d(h, h->f_mu, mu, g)); CS(h2d(h, h->f_mu_node, mu_node, g));
  CS(h2d(h, h->f_fx, fx_sigma, g)); CS(h2d(h, h->f_fy, fy_sigma, g));
  CS(h2d(h, h->f_u_old, u_old, g)); CS(h2d(h, h->f_v_old, v_old, g));
  int it = 0, ud = 0;
  const int st = al_enqueue(h, dt, h->f_u, h->f_v, h->f_p, h->f_rho, h->f_rho_u, h->f_rho_v, h->f_mu,
                            h->f_mu_node, h->f_fx, h->f_fy, h->f_u_old, h->f_v_old, true, &it, &ud);
  if (st == COVOF_CUDA_ERROR || st == COVOF_INVALID || st == COVOF_UNSUPPORTED || st == COVOF_TIMEOUT) return st;
  CS(d2h(h, u, h->f_u, g)); CS(d2h(h, v, h->f_v, g)); CS(d2h(h, p, h->f_p, g));
  CS(sync(h));
  if (total_iters) *total_iters = it;
  if (uzawa_done) *uzawa_done = ud;
  return st;
}

// ---- MONOLITHIC step ------------------------------------------------------------
int covof_monolithic_step(covof_handle* h, double dt, double* u, double* v, double* p, const double* rho_u,
                          const double* rho_v, const double* mu, const double* mu_node, const double* fx_sigma,
                          const double* fy_sigma, const double* u_old, const double* v_old, int* iters) {
  if (!h) return COVOF_INVALID;
  if (h->prm.solver_type != COVOF_SOLVER_MONOLITHIC) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_u, u, g)); CS(h2d(h, h->f_v, v, g)); CS(h2d(h, h->f_p, p, g));
  CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g));
  CS(h2d(h, h->f_mu, mu, g)); CS(h2d(h, h->f_mu_node, mu_node, g));
  CS(h2d(h, h->f_fx, fx_sigma, g)); CS(h2d(h, h->f_fy, fy_sigma, g));
  CS(h2d(h, h->f_u_old, u_old, g)); CS(h2d(h, h->f_v_old, v_old, g));
  CS(mono_enqueue(h, dt, h->f_u, h->f_v, h->f_p, h->f_rho_u, h->f_rho_v, h->f_mu, h->f_mu_node, h->f_fx,
                  h->f_fy, h->f_u_old, h->f_v_old));
  CK(cudaMemcpyAsync(h->h_kres, h->d_kres, sizeof(KrylovResult), cudaMemcpyDeviceToHost, h->stream));
  CS(d2h(h, u, h->f_u, g)); CS(d2h(h, v, h->f_v, g)); CS(d2h(h, p, h->f_p, g));
  CS(sync(h));
  if (iters) *iters = h->h_kres->iters;
  return h->h_kres->status;
}

// ---- VOF -----------------------------------------------------------------------
int covof_vof_reconstruct_dev(covof_handle* h, const double* C, double* seg) {
  if (!h || !C || !seg) return COVOF_INVALID;
  CS(reconstruct_dev(h, C, seg));
  return sync(h);
}

int covof_vof_reconstruct(covof_handle* h, const double* C, double* seg) {
  if (!h) return COVOF_INVALID;
  CS(ensure_fields(h));
  CS(h2d(h, h->f_C, C, h->g));
  CS(reconstruct_dev(h, h->f_C, h->f_seg));
  CS(d2h(h, seg, h->f_seg, 3 * h->g));
  return sync(h);
}

int covof_vof_wy_step_dev(covof_handle* h, double dt, int x_first, const double* u,
                          const double* v, double* C) {
  if (!h || !u || !v || !C) return COVOF_INVALID;
  CS(wy_step_dev(h, dt, x_first, u, v, C));
  return sync(h);
}

int covof_vof_wy_step(covof_handle* h, double dt, int x_first, const double* u, const double* v,
                      double* C) {
  if (!h) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_u, u, g)); CS(h2d(h, h->f_v, v, g)); CS(h2d(h, h->f_C, C, g));
  CS(wy_step_dev(h, dt, x_first, h->f_u, h->f_v, h->f_C));
  CS(d2h(h, C, h->f_C, g));
  return sync(h);
}

int covof_vof_advect_dev(covof_handle* h, double dt, const double* u, const double* v, double* C,
                         double* rho, double* rho_u, double* rho_v, double* mu, double* mu_node,
                         double* fx_sigma, double* fy_sigma, double* curvature) {
  if (!h) return COVOF_INVALID;
  CS(vof_advect_dev(h, dt, u, v, C, rho, rho_u, rho_v, mu, mu_node, fx_sigma, fy_sigma, curvature));
  return sync(h);
}

int covof_vof_advect(covof_handle* h, double dt, const double* u, const double* v, double* C,
                     double* rho, double* rho_u, double* rho_v, double* mu, double* mu_node,
                     double* fx_sigma, double* fy_sigma, double* curvature) {
  if (!h) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  // in/out arrays keep the caller's values wherever the reference leaves them
  CS(h2d(h, h->f_u, u, g)); CS(h2d(h, h->f_v, v, g)); CS(h2d(h, h->f_C, C, g));
  CS(h2d(h, h->f_rho, rho, g)); CS(h2d(h, h->f_rho_u, rho_u, g)); CS(h2d(h, h->f_rho_v, rho_v, g));
  CS(h2d(h, h->f_mu, mu, g)); CS(h2d(h, h->f_mu_node, mu_node, g));
  CS(h2d(h, h->f_fx, fx_sigma, g)); CS(h2d(h, h->f_fy, fy_sigma, g)); CS(h2d(h, h->f_curv, curvature, g));
  CS(vof_advect_dev(h, dt, h->f_u, h->f_v, h->f_C, h->f_rho, h->f_rho_u, h->f_rho_v, h->f_mu,
                    h->f_mu_node, h->f_fx, h->f_fy, h->f_curv));
  CS(d2h(h, C, h->f_C, g)); CS(d2h(h, rho, h->f_rho, g)); CS(d2h(h, rho_u, h->f_rho_u, g));
  CS(d2h(h, rho_v, h->f_rho_v, g)); CS(d2h(h, mu, h->f_mu, g)); CS(d2h(h, mu_node, h->f_mu_node, g));
  CS(d2h(h, fx_sigma, h->f_fx, g)); CS(d2h(h, fy_sigma, h->f_fy, g)); CS(d2h(h, curvature, h->f_curv, g));
  return sync(h);
}

int covof_svof_smooth(covof_handle* h, const double* C, double* C_s) {
  if (!h || !C) return COVOF_INVALID;
  CS(ensure_fields(h));
  CS(h2d(h, h->f_C, C, h->g));
  CS(svof_dev(h, h->f_C, h->f_Cs));
  if (C_s) CS(d2h(h, C_s, h->f_Cs, h->g));
  int err = 0;
  CK(cudaMemcpyAsync(&err, h->err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CS(sync(h));
  return err != 0 ? err : COVOF_OK;  // a wavefront wait that gave up: COVOF_TIMEOUT
}

int covof_diffusion_smooth(covof_handle* h, const double* C, double* C_tilde) {
  if (!h || !C) return COVOF_INVALID;
  CS(ensure_fields(h));
  CS(h2d(h, h->f_C, C, h->g));
  CS(diffusion_dev(h, h->f_C, h->f_Ct));
  if (C_tilde) CS(d2h(h, C_tilde, h->f_Ct, h->g));
  return sync(h);
}

int covof_update_physical_properties(covof_handle* h, double* C, double* rho, double* rho_u,
                                     double* rho_v, double* mu, double* mu_node) {
  if (!h) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_C, C, g)); CS(h2d(h, h->f_rho, rho, g)); CS(h2d(h, h->f_rho_u, rho_u, g));
  CS(h2d(h, h->f_rho_v, rho_v, g)); CS(h2d(h, h->f_mu, mu, g)); CS(h2d(h, h->f_mu_node, mu_node, g));
  // with SVOF the properties follow the resident C_s (covof_svof_smooth)
  CS(props_dev(h, h->f_C, h->f_rho, h->f_rho_u, h->f_rho_v, h->f_mu, h->f_mu_node, h->f_Cs));
  CS(d2h(h, C, h->f_C, g)); CS(d2h(h, rho, h->f_rho, g)); CS(d2h(h, rho_u, h->f_rho_u, g));
  CS(d2h(h, rho_v, h->f_rho_v, g)); CS(d2h(h, mu, h->f_mu, g)); CS(d2h(h, mu_node, h->f_mu_node, g));
  return sync(h);
}

int covof_apply_velocity_bc(covof_handle* h, double* u, double* v) {
  if (!h || !u || !v) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_u, u, g)); CS(h2d(h, h->f_v, v, g));
  CS(velocity_bc_dev(h, h->f_u, h->f_v));
  CS(d2h(h, u, h->f_u, g)); CS(d2h(h, v, h->f_v, g));
  return sync(h);
}

int covof_apply_vof_bc(covof_handle* h, double* C) {
  if (!h || !C) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_C, C, g));
  if (periodic(h->prm)) k_vof_halo_bc<<<1, 1024, 0, h->stream>>>(h->D, h->f_C, 0);
  else k_vof_bc<<<(h->D.nx + h->D.ny + 127) / 128, 128, 0, h->stream>>>(h->D, h->f_C);
  CK(cudaGetLastError());
  CS(d2h(h, C, h->f_C, g));
  return sync(h);
}

int covof_compute_curvature_and_csf(covof_handle* h, const double* C, double* fx_sigma,
                                    double* fy_sigma, double* curvature) {
  if (!h) return COVOF_INVALID;
  CS(ensure_fields(h));
  const size_t g = h->g;
  CS(h2d(h, h->f_C, C, g)); CS(h2d(h, h->f_fx, fx_sigma, g)); CS(h2d(h, h->f_fy, fy_sigma, g));
  CS(h2d(h, h->f_curv, curvature, g));
  // normals from the resident C_tilde / C_s when smoothing is on
  CS(csf_dev(h, h->f_C, h->f_fx, h->f_fy, h->f_curv, h->f_Cs, h->f_Ct));
  CS(d2h(h, fx_sigma, h->f_fx, g)); CS(d2h(h, fy_sigma, h->f_fy, g)); CS(d2h(h, curvature, h->f_curv, g));
  return sync(h);
}

// ---- launch shapes ------------------------------------------------------------
int covof_set_launch(covof_handle* h, const covof_launch* launch) {
  if (!h || !launch) return COVOF_INVALID;
  const covof_launch& L = *launch;
  if (L.p_threads != 0 && L.p_threads != 128 && L.p_threads != 256 && L.p_threads != 512 && L.p_threads != 1024)
    return COVOF_INVALID;
  if (L.p_blocks < 0 || L.p_blocks > h->sm_count || L.p_inner_form < 0 || L.p_inner_form > 3 ||
      (L.p_inner_form == 3 && L.p_blocks > 16) || L.vof_cell_min < 0)
    return COVOF_INVALID;
  if (h->stream) cudaStreamSynchronize(h->stream);
  const covof_launch keep = h->launch;
  h->launch = L;
  h->have_pplan = false;
  drop_graphs(h);
  const int st = poisson_plan(h);
  if (st != COVOF_OK) {
    h->launch = keep;
    h->have_pplan = false;
    return st;
  }
  return COVOF_OK;
}

int covof_get_launch(covof_handle* h, covof_launch* launch) {
  if (!h || !launch) return COVOF_INVALID;
  CS(poisson_plan(h));
  launch->p_threads = h->p_threads;
  launch->p_blocks = h->p_nb;
  launch->p_inner_form = h->p_fn == (const void*)k_pcg_mixed_cheb ? 1
                       : h->p_fn == (const void*)k_pcg_mixed_stream ? 2
                       : h->p_fn == (const void*)k_pcg_mixed_cluster ? 3 : 0;
  launch->vof_cell_min = vof_cell_min(h);
  return COVOF_OK;
}

// ---- resident time stepping -------------------------------------------------
int covof_state_set(covof_handle* h, int field, const double* host) {
  if (!h || !host) return COVOF_INVALID;
  CS(ensure_fields(h));
  double** slot = field_slot(h, field);
  if (!slot) return COVOF_INVALID;
  CS(h2d(h, *slot, host, h->g));
  return sync(h);
}

int covof_state_get(covof_handle* h, int field, double* host) {
  if (!h || !host) return COVOF_INVALID;
  CS(ensure_fields(h));
  double** slot = field_slot(h, field);
  if (!slot) return COVOF_INVALID;
  CS(d2h(h, host, *slot, h->g));
  return sync(h);
}

int covof_set_has_nm1(covof_handle* h, int has_nm1) {
  if (!h) return COVOF_INVALID;
  if (h->has_nm1 != (has_nm1 != 0)) {
    if (h->stream) cudaStreamSynchronize(h->stream);
    drop_graphs(h);  // the captured steps bake the flag in
  }
  h->has_nm1 = has_nm1 != 0;
  return COVOF_OK;
}

int covof_get_has_nm1(const covof_handle* h, int* has_nm1) {
  if (!h || !has_nm1) return COVOF_INVALID;
  *has_nm1 = h->has_nm1 ? 1 : 0;
  return COVOF_OK;
}

int covof_state_field_dev(covof_handle* h, int field, double** dev) {
  if (!h || !dev) return COVOF_INVALID;
  CS(ensure_fields(h));
  double** slot = field_slot(h, field);
  if (!slot) return COVOF_INVALID;
  *dev = *slot;
  return COVOF_OK;
}

int covof_run_steps(covof_handle* h, double dt, int nsteps, int flags, covof_run_stats* stats) {
  if (!h) return COVOF_INVALID;
  return run_steps(h, dt, nsteps, flags, stats);
}

}  // extern "C"

COVOF_UNIT_HOOKS(capi)
