// batch.cu -- many independent cases stepped together (covof_batch_* in
// include/covof_gpu.h).
//
// Every case keeps a handle of its own (fields, solver scratch); one time
// step of the whole batch is, in stream order:
//   1. per case, in parallel branches: u_old = u, v_old = v; the VOF step
//      (two-phase cases) and the velocity BC; predictor assembly;
//   2. ONE persistent cooperative launch: the predictor Krylov solves of all
//      cases (k_mom_krylov_batch, or k_mom_bicgstab_batch / k_mom_cg_batch
//      when every case uses that method);
//   3. per case: unpack + velocity BC; Poisson assembly;
//   4. ONE persistent cooperative launch: the Poisson solves of all cases
//      (k_pcg_mixed_mg_batch / k_pcg_mixed_smem_batch / k_pcg_mixed_batch,
//      k_pcg_fp64_mg_batch for the FP64 multigrid form, or k_pcg_fp64_batch
//      for plain FP64 batches);
//   5. per case: copy-back, velocity correction, velocity BC, status log.
// The grid of a batched solve is cut into teams (contiguous block ranges,
// common.cuh: BatchTeams); a team solves its cases one after another with
// barriers, reductions and neighbour counters of its own, so small cases do
// not wait on grid-wide barriers and the GPU stays full however uneven the
// case sizes are.  With COVOF_RUN_GRAPH each step is one CUDA-graph launch.
#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "handle.cuh"

using namespace covof;
using namespace covof::host;

namespace {

constexpr int kForks = 8;  // parallel branches for the per-case stages

struct Plan {
  int threads = 0, nblocks = 0, nteams = 0;
  std::vector<int> block_team;
  std::vector<int4> team;
  std::vector<int> case_list;
  // device copies and team-scoped synchronisation words
  int* d_block_team = nullptr;
  int4* d_team = nullptr;
  int* d_case_list = nullptr;
  unsigned int* d_bar = nullptr;
  unsigned int* d_flags = nullptr;
  int* d_err = nullptr;
  double* d_part = nullptr;
  float* d_xb = nullptr;  // boundary rows of the shared-memory inner form
  int xbw = 0;
  size_t smem = 0;        // dynamic shared memory per block of the launch
  BatchTeams dev() const {
    return BatchTeams{d_block_team, d_team, d_case_list, d_bar, d_flags, d_err, d_part, d_xb, xbw};
  }
};

}  // namespace

struct covof_batch {
  int ncases = 0, device = 0, sm_count = 0;
  bool mixed = false;
  std::vector<covof_handle*> h;
  cudaStream_t stream = nullptr, cap = nullptr;
  cudaStream_t fork[kForks] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[kForks] = {};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  Plan pplan, mplan;
  PoissonArgs* h_pargs = nullptr;  // pinned: argument blocks of the batched solves
  MomArgs* h_margs = nullptr;
  PoissonArgs* d_pargs = nullptr;
  MomArgs* d_margs = nullptr;
  const void* pfn = nullptr;  // the batched Poisson kernel
  const void* mfn = nullptr;  // the batched momentum Krylov kernel
  cudaGraphExec_t graph[2] = {};
  std::vector<double> graph_dt;
  bool graph_refused = false;
  int step_count = 0;
};

namespace {

int next_pow2(long long v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

// Teams for a batched solve over at most max_blocks co-resident blocks.
// The makespan is the busiest block's load, so a case gets about as many
// blocks as its share of the batch's work (work ~ cells x the longer side,
// the growth of the iteration count), rounded up to a power of two, at most
// 16 and never more blocks than rows.  Blocks are then shared among the
// size classes in proportion to their work, and the cases of a class go to
// its teams longest first.
// min_team (optional): a lower bound on the team size of each case (the
// shared-memory form needs enough blocks for the strips to fit).
int make_plan(Plan& pl, const std::vector<covof_handle*>& hs, int max_blocks, int threads,
              const std::vector<int>* min_team = nullptr) {
  const int n = (int)hs.size();
  std::vector<long long> work(n), cls(n);
  long long wtot = 0;
  for (int c = 0; c < n; ++c) {
    const long long cells = (long long)hs[c]->prm.nx * hs[c]->prm.ny;
    work[c] = cells * std::max(hs[c]->prm.nx, hs[c]->prm.ny);
    wtot += work[c];
  }
  for (int c = 0; c < n; ++c) {
    const double share = (double)work[c] * max_blocks / (double)wtot;
    int t = next_pow2((long long)std::ceil(share));
    t = std::min(t, 16);
    while (t > 1 && t > hs[c]->prm.ny) t >>= 1;
    if (min_team) t = std::max(t, (*min_team)[c]);
    cls[c] = t;
  }
  // blocks per class
  std::vector<int> sizes;
  for (int c = 0; c < n; ++c)
    if (std::find(sizes.begin(), sizes.end(), (int)cls[c]) == sizes.end()) sizes.push_back((int)cls[c]);
  std::sort(sizes.begin(), sizes.end());
  std::vector<int> nteams(sizes.size());
  int used = 0;
  for (size_t s = 0; s < sizes.size(); ++s) {
    long long w = 0, cnt = 0;
    for (int c = 0; c < n; ++c)
      if (cls[c] == sizes[s]) { w += work[c]; ++cnt; }
    int nt = (int)std::floor((double)max_blocks * (double)w / (double)wtot / sizes[s]);
    nt = (int)std::max(1LL, std::min((long long)nt, cnt));
    nteams[s] = nt;
    used += nt * sizes[s];
  }
  // hand leftover blocks to the class with the most work per block, while
  // it has more cases than teams
  std::vector<long long> wcls(sizes.size(), 0), ncls(sizes.size(), 0);
  for (size_t s = 0; s < sizes.size(); ++s)
    for (int c = 0; c < n; ++c)
      if (cls[c] == sizes[s]) { wcls[s] += work[c]; ++ncls[s]; }
  for (;;) {
    int best = -1;
    double best_load = -1.0;
    for (size_t s = 0; s < sizes.size(); ++s) {
      if (nteams[s] >= ncls[s] || used + sizes[s] > max_blocks) continue;
      const double load = (double)wcls[s] / ((double)nteams[s] * sizes[s]);
      if (load > best_load) { best_load = load; best = (int)s; }
    }
    if (best < 0) break;
    nteams[best] += 1;
    used += sizes[best];
  }
  // shrink the largest classes until the teams fit
  while (used > max_blocks) {
    int best = -1;
    for (size_t s = 0; s < sizes.size(); ++s)
      if (nteams[s] > 1 && (best < 0 || sizes[s] * nteams[s] > sizes[best] * nteams[best])) best = (int)s;
    if (best < 0) return COVOF_UNSUPPORTED;  // one team per class does not fit
    nteams[best] -= 1;
    used -= sizes[best];
  }
  // LPT within each class
  pl.threads = threads;
  pl.block_team.clear();
  pl.team.clear();
  pl.case_list.clear();
  int first = 0;
  for (size_t s = 0; s < sizes.size(); ++s) {
    std::vector<int> cs;
    for (int c = 0; c < n; ++c)
      if (cls[c] == sizes[s]) cs.push_back(c);
    std::sort(cs.begin(), cs.end(), [&](int a, int b) { return work[a] > work[b] || (work[a] == work[b] && a < b); });
    const int nt = nteams[s];
    std::vector<long long> load(nt, 0);
    std::vector<std::vector<int>> lists(nt);
    for (int c : cs) {
      int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      load[k] += work[c];
      lists[k].push_back(c);
    }
    for (int k = 0; k < nt; ++k) {
      const int t = (int)pl.team.size();
      const int begin = (int)pl.case_list.size();
      for (int c : lists[k]) pl.case_list.push_back(c);
      pl.team.push_back(make_int4(first, sizes[s], begin, (int)pl.case_list.size()));
      for (int b = 0; b < sizes[s]; ++b) pl.block_team.push_back(t);
      first += sizes[s];
    }
  }
  pl.nblocks = first;
  pl.nteams = (int)pl.team.size();
  CS(dalloc(&pl.d_block_team, pl.block_team.size()));
  CS(dalloc(&pl.d_team, pl.team.size()));
  CS(dalloc(&pl.d_case_list, pl.case_list.size()));
  CS(dalloc(&pl.d_bar, (size_t)32 * pl.nteams));
  CS(dalloc(&pl.d_flags, (size_t)pl.nblocks));
  CS(dalloc(&pl.d_err, (size_t)pl.nteams));
  CS(dalloc(&pl.d_part, (size_t)16 * pl.nblocks));
  CK(cudaMemcpy(pl.d_block_team, pl.block_team.data(), pl.block_team.size() * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(pl.d_team, pl.team.data(), pl.team.size() * sizeof(int4), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(pl.d_case_list, pl.case_list.data(), pl.case_list.size() * sizeof(int), cudaMemcpyHostToDevice));
  return COVOF_OK;
}

void free_plan(Plan& pl) {
  dfree(pl.d_block_team); dfree(pl.d_team); dfree(pl.d_case_list);
  dfree(pl.d_bar); dfree(pl.d_flags); dfree(pl.d_err); dfree(pl.d_part); dfree(pl.d_xb);
}

// Shared-memory form of the mixed batch: the smallest power-of-two team per
// case whose row strips fit one block's shared memory (at most 32 blocks,
// never more blocks than rows).  Returns false when some case does not fit.
bool smem_teams(const std::vector<covof_handle*>& hs, size_t budget, std::vector<int>& tmin, size_t& bytes) {
  bytes = 0;
  tmin.assign(hs.size(), 1);
  for (size_t c = 0; c < hs.size(); ++c) {
    const int nx = hs[c]->prm.nx, ny = hs[c]->prm.ny;
    int t = 1;
    while (t <= 32 && t <= ny && smem_cheb_bytes(nx, (ny + t - 1) / t) > budget) t <<= 1;
    if (t > 32 || t > ny) return false;
    tmin[c] = t;
  }
  return true;
}

int max_coresident(const covof_batch* b, const void* fn, int threads) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess || per_sm < 1) return -1;
  return per_sm * b->sm_count;
}

int launch_batch(covof_batch* b, const Plan& pl, const void* fn, const void* cases) {
  // (pl.smem: dynamic shared memory of the shared-memory inner form)
  CK(cudaMemsetAsync(pl.d_bar, 0, (size_t)32 * pl.nteams * sizeof(unsigned int), b->stream));
  CK(cudaMemsetAsync(pl.d_flags, 0, (size_t)pl.nblocks * sizeof(unsigned int), b->stream));
  CK(cudaMemsetAsync(pl.d_err, 0, (size_t)pl.nteams * sizeof(int), b->stream));
  BatchTeams bt = pl.dev();
  void* args[] = {(void*)&cases, &bt};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(pl.nblocks);
  cfg.blockDim = dim3(pl.threads);
  cfg.dynamicSmemBytes = pl.smem;
  cfg.stream = b->stream;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  CK(cudaLaunchKernelExC(&cfg, fn, args));
  return COVOF_OK;
}

// Per-case work in kForks parallel branches of b->stream: handle c runs on
// fork stream c % kForks while f(c) enqueues.
template <class F>
int per_case(covof_batch* b, F f) {
  CK(cudaEventRecord(b->ev_fork, b->stream));
  for (int k = 0; k < kForks; ++k) CK(cudaStreamWaitEvent(b->fork[k], b->ev_fork, 0));
  int st = COVOF_OK;
  for (int c = 0; c < b->ncases && st == COVOF_OK; ++c) {
    covof_handle* h = b->h[c];
    cudaStream_t keep = h->stream;
    h->stream = b->fork[c % kForks];
    st = f(c, h);
    h->stream = keep;
  }
  for (int k = 0; k < kForks; ++k) {
    CK(cudaEventRecord(b->ev_join[k], b->fork[k]));
    CK(cudaStreamWaitEvent(b->stream, b->ev_join[k], 0));
  }
  return st;
}

// One time step of every case on b->stream (src/module_simulation.f90:492-559
// per case, as covof_run_steps).
int enqueue_batch_step(covof_batch* b, const double* dt, bool x_first) {
  CS(per_case(b, [&](int c, covof_handle* h) -> int {
    const size_t bytes = h->g * sizeof(double);
    CS(rotate_history(h));
    CK(cudaMemcpyAsync(h->f_u_old, h->f_u, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->f_v_old, h->f_v, bytes, cudaMemcpyDeviceToDevice, h->stream));
    if (h->prm.enable_two_phase) {
      CS(wy_step_dev(h, dt[c], x_first ? 1 : 0, h->f_u, h->f_v, h->f_C));
      CS(vof_bc_dev(h, h->f_C));
    }
    return COVOF_OK;
  }));
  // SVOF's cooperative wavefront launches run one case at a time on the
  // batch stream (one spinning cooperative grid on the device at a time)
  for (covof_handle* h : b->h) {
    if (!h->prm.enable_two_phase || !h->prm.enable_svof_smoothing) continue;
    cudaStream_t keep = h->stream;
    h->stream = b->stream;
    const int st = svof_dev(h, h->f_C, h->f_Cs);
    h->stream = keep;
    CS(st);
  }
  CS(per_case(b, [&](int c, covof_handle* h) -> int {
    if (h->prm.enable_two_phase) {
      CS(smooth_props_csf(h, false));
      CS(velocity_bc_dev(h, h->f_u, h->f_v));
    }
    return mom_pre(h, dt[c], h->f_u, h->f_v, h->f_rho_u, h->f_rho_v, h->f_mu, h->f_mu_node, h->f_fx,
                   h->f_fy, h->f_u_old, h->f_v_old, &b->h_margs[c]);
  }));
  CK(cudaMemcpyAsync(b->d_margs, b->h_margs, sizeof(MomArgs) * b->ncases, cudaMemcpyHostToDevice, b->stream));
  CS(launch_batch(b, b->mplan, b->mfn, b->d_margs));
  CS(per_case(b, [&](int c, covof_handle* h) -> int {
    CS(mom_post(h, b->h_margs[c], h->f_u, h->f_v));
    return pois_pre(h, dt[c], h->f_u, h->f_v, nullptr, h->f_rho_u, h->f_rho_v, h->f_p, &b->h_pargs[c]);
  }));
  CK(cudaMemcpyAsync(b->d_pargs, b->h_pargs, sizeof(PoissonArgs) * b->ncases, cudaMemcpyHostToDevice,
                     b->stream));
  CS(launch_batch(b, b->pplan, b->pfn, b->d_pargs));
  CS(per_case(b, [&](int c, covof_handle* h) -> int {
    CS(pois_post(h, h->f_p));
    CS(correct_dev(h, dt[c], h->f_u, h->f_v, h->f_p, h->f_rho_u, h->f_rho_v));
    CS(velocity_bc_dev(h, h->f_u, h->f_v));
    k_step_log<<<1, 32, 0, h->stream>>>(h->d_kres, h->d_pres, h->d_run);
    CK(cudaGetLastError());
    return COVOF_OK;
  }));
  return COVOF_OK;
}

void drop_graphs(covof_batch* b) {
  for (cudaGraphExec_t& g : b->graph) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
}

int capture(covof_batch* b, const double* dt) {
  drop_graphs(b);
  for (int q = 0; q < 2; ++q) {
    cudaStream_t keep = b->stream;
    b->stream = b->cap;
    cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    int st = e == cudaSuccess ? enqueue_batch_step(b, dt, q == 0) : COVOF_OK;
    cudaGraph_t g = nullptr;
    if (e == cudaSuccess) e = cudaStreamEndCapture(b->stream, &g);
    b->stream = keep;
    if (st == COVOF_OK && e == cudaSuccess && g) e = cudaGraphInstantiate(&b->graph[q], g, 0ULL);
    if (g) cudaGraphDestroy(g);
    if (st != COVOF_OK || e != cudaSuccess || !b->graph[q]) {
      cudaGetLastError();
      drop_graphs(b);
      return (st != COVOF_OK && st != COVOF_CUDA_ERROR) ? st : COVOF_UNSUPPORTED;
    }
  }
  b->graph_dt.assign(dt, dt + b->ncases);
  return COVOF_OK;
}

}  // namespace

extern "C" {

int covof_batch_destroy(covof_batch* b) {
  if (!b) return COVOF_INVALID;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  for (covof_handle* h : b->h)
    if (h) covof_destroy(h);
  free_plan(b->pplan);
  free_plan(b->mplan);
  dfree(b->d_pargs);
  dfree(b->d_margs);
  if (b->h_pargs) cudaFreeHost(b->h_pargs);
  if (b->h_margs) cudaFreeHost(b->h_margs);
  for (int k = 0; k < kForks; ++k) {
    if (b->fork[k]) cudaStreamDestroy(b->fork[k]);
    if (b->ev_join[k]) cudaEventDestroy(b->ev_join[k]);
  }
  for (cudaEvent_t e : {b->ev_fork, b->ev0, b->ev1})
    if (e) cudaEventDestroy(e);
  if (b->cap) cudaStreamDestroy(b->cap);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return COVOF_OK;
}

int covof_batch_create(const covof_params* cases, int ncases, covof_batch** out) {
  if (!out || !cases || ncases < 1) return COVOF_INVALID;
  *out = nullptr;
  covof_batch* b = new (std::nothrow) covof_batch();
  if (!b) return COVOF_INVALID;
  auto fail = [&](int code) { covof_batch_destroy(b); return code; };
  b->ncases = ncases;
  b->mixed = cases[0].p_precision == COVOF_PREC_MIXED;
  const bool mg = mg_path(cases[0]);
  for (int c = 0; c < ncases; ++c) {
    // one arithmetic per batch; a mixed batch runs either the multigrid inner
    // iteration for every case or Chebyshev for every case
    if (cases[c].p_precision != cases[0].p_precision) return fail(COVOF_INVALID);
    if (b->mixed && (cases[c].p_inner_kind == COVOF_INNER_MG) != mg) return fail(COVOF_UNSUPPORTED);
    if (b->mixed && cases[c].p_inner_kind == COVOF_INNER_CG) return fail(COVOF_UNSUPPORTED);
    if (cases[c].p_precond == COVOF_PRECOND_SSOR) return fail(COVOF_UNSUPPORTED);
    // the batch's Krylov kernels are the persistent ones (no sweep preconditioners)
    if (uses_sweeps(cases[c])) return fail(COVOF_UNSUPPORTED);
    // the batch runs the projection coupling
    if (check_coupling(cases[c]) != COVOF_OK ||
        (cases[c].solver_type != 0 && cases[c].solver_type != COVOF_SOLVER_STANDARD_PROJECTION))
      return fail(COVOF_UNSUPPORTED);
    const int s = check_mom_params(cases[c]);
    if (s != COVOF_OK) return fail(s);
  }
  b->h.assign(ncases, nullptr);
  for (int c = 0; c < ncases; ++c) {
    const int s = covof_create(&cases[c], &b->h[c]);
    if (s != COVOF_OK) return fail(s);
    covof_handle* h = b->h[c];
    h->vof_block_form = false;  // the cases' VOF stages run side by side
    if (ensure_fields(h) || ensure_poisson(h) || ensure_mom(h) || ensure_vof(h) || poisson_plan(h) ||
        predictor_plan(h))
      return fail(COVOF_CUDA_ERROR);
  }
  b->device = b->h[0]->device;
  b->sm_count = b->h[0]->sm_count;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess)
    return fail(COVOF_CUDA_ERROR);
  for (int k = 0; k < kForks; ++k)
    if (cudaStreamCreateWithFlags(&b->fork[k], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_join[k], cudaEventDisableTiming) != cudaSuccess)
      return fail(COVOF_CUDA_ERROR);
  if (cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess)
    return fail(COVOF_CUDA_ERROR);
  // Poisson: a multigrid batch runs k_pcg_mixed_mg_batch; a Chebyshev batch
  // keeps each case's inner state in shared-memory row strips when every
  // case fits a team of at most 32 blocks, else it streams the inner state
  // through L2 / HBM
  b->pfn = b->mixed ? (const void*)k_pcg_mixed_batch : (const void*)k_pcg_fp64_batch;
  std::vector<int> tmin;
  bool smem_form = false;
  bool want_stream = false;
  for (int c = 0; c < ncases; ++c) want_stream |= cases[c].p_inner_kind == COVOF_INNER_CHEBYSHEV_STREAM;
  if (mg) {
    // the semi-coarsening kernel when some case has anisotropic cells
    bool semi = false;
    for (covof_handle* h : b->h) semi = semi || h->mg.semi != 0;
    if (cases[0].p_precision == COVOF_PREC_FP64_MG)
      b->pfn = semi ? (const void*)k_pcg_fp64_mg_batch_semi : (const void*)k_pcg_fp64_mg_batch;
    else
      b->pfn = semi ? (const void*)k_pcg_mixed_mg_batch_semi : (const void*)k_pcg_mixed_mg_batch;
  }
  if (b->mixed && !want_stream && !mg) {
    int optin = 0;
    cudaFuncAttributes fa;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
    if (cudaFuncGetAttributes(&fa, (const void*)k_pcg_mixed_smem_batch) == cudaSuccess &&
        optin > (int)fa.sharedSizeBytes &&
        smem_teams(b->h, (size_t)optin - fa.sharedSizeBytes, tmin, b->pplan.smem)) {
      smem_form = true;
      b->pfn = (const void*)k_pcg_mixed_smem_batch;
    }
    cudaGetLastError();
  }
  int pmax = 0;
  if (smem_form) {
    // the launch's shared memory: the largest strip over the cases, with
    // teams no smaller than tmin (larger teams only shorten strips)
    size_t bytes = 0;
    for (int c = 0; c < ncases; ++c) {
      const int nx = b->h[c]->prm.nx, ny = b->h[c]->prm.ny;
      bytes = std::max(bytes, smem_cheb_bytes(nx, (ny + tmin[c] - 1) / tmin[c]));
    }
    b->pplan.smem = bytes;
    if (cudaFuncSetAttribute(b->pfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
      return fail(COVOF_CUDA_ERROR);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, b->pfn, 1024, bytes) != cudaSuccess || per_sm < 1)
      return fail(COVOF_CUDA_ERROR);
    pmax = per_sm * b->sm_count;
  } else if (mg) {
    // the largest multigrid tail of the batch in every block
    size_t bytes = 0;
    for (covof_handle* h : b->h) bytes = std::max(bytes, (size_t)h->mg.tail_smem);
    b->pplan.smem = bytes;
    // opt in whatever the size: the kernel's static shared memory counts
    // against the 48 KB a launch gets without it
    if (cudaFuncSetAttribute(b->pfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
      return fail(COVOF_CUDA_ERROR);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, b->pfn, 1024, bytes) != cudaSuccess || per_sm < 1)
      return fail(COVOF_CUDA_ERROR);
    pmax = per_sm * b->sm_count;
  } else {
    pmax = max_coresident(b, b->pfn, 1024);
  }
  // one method across the batch: its own kernel (two blocks per SM)
  b->mfn = (const void*)k_mom_krylov_batch;
  {
    bool same = true;
    for (covof_handle* h : b->h) same = same && h->prm.linear_solver == b->h[0]->prm.linear_solver;
    const int m = b->h[0]->prm.linear_solver;
    if (same && m == COVOF_LINEAR_BICGSTAB) b->mfn = (const void*)k_mom_bicgstab_batch;
    if (same && m == COVOF_LINEAR_CG) b->mfn = (const void*)k_mom_cg_batch;
  }
  const int mmax = max_coresident(b, b->mfn, 512);
  if (pmax < 1 || mmax < 1) return fail(COVOF_CUDA_ERROR);
  int s = make_plan(b->pplan, b->h, pmax, 1024, smem_form ? &tmin : nullptr);
  if (s != COVOF_OK) return fail(s);
  if (smem_form) {
    int wmax = 0;
    for (covof_handle* h : b->h) wmax = std::max(wmax, h->prm.nx + 2);
    b->pplan.xbw = wmax;
    if (dalloc(&b->pplan.d_xb, (size_t)4 * b->pplan.nblocks * wmax)) return fail(COVOF_CUDA_ERROR);
  }
  s = make_plan(b->mplan, b->h, mmax, 512);
  if (s != COVOF_OK) return fail(s);
  if (dalloc(&b->d_pargs, (size_t)ncases) || dalloc(&b->d_margs, (size_t)ncases) ||
      cudaMallocHost(&b->h_pargs, sizeof(PoissonArgs) * ncases) != cudaSuccess ||
      cudaMallocHost(&b->h_margs, sizeof(MomArgs) * ncases) != cudaSuccess)
    return fail(COVOF_CUDA_ERROR);
  *out = b;
  return COVOF_OK;
}

int covof_batch_set_has_nm1(covof_batch* b, int has_nm1) {
  if (!b) return COVOF_INVALID;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  for (covof_handle* h : b->h) CS(covof_set_has_nm1(h, has_nm1));
  return COVOF_OK;
}

int covof_batch_state_set(covof_batch* b, int icase, int field, const double* host) {
  if (!b || icase < 0 || icase >= b->ncases) return COVOF_INVALID;
  return covof_state_set(b->h[icase], field, host);
}

int covof_batch_state_get(covof_batch* b, int icase, int field, double* host) {
  if (!b || icase < 0 || icase >= b->ncases) return COVOF_INVALID;
  if (b->stream) cudaStreamSynchronize(b->stream);
  return covof_state_get(b->h[icase], field, host);
}

int covof_batch_info(const covof_batch* b, int* poisson_teams, int* poisson_blocks, int* predictor_teams,
                     int* predictor_blocks) {
  if (!b) return COVOF_INVALID;
  if (poisson_teams) *poisson_teams = b->pplan.nteams;
  if (poisson_blocks) *poisson_blocks = b->pplan.nblocks;
  if (predictor_teams) *predictor_teams = b->mplan.nteams;
  if (predictor_blocks) *predictor_blocks = b->mplan.nblocks;
  return COVOF_OK;
}

int covof_batch_run_steps(covof_batch* b, const double* dt, int nsteps, int flags, covof_run_stats* stats,
                          double* ms) {
  if (!b || !dt || nsteps < 0) return COVOF_INVALID;
  for (int c = 0; c < b->ncases; ++c)
    if (!(dt[c] > 0.0)) return COVOF_INVALID;
  for (covof_handle* h : b->h) {
    *h->h_run = RunStats{0, 0, 0, 0.0, 0.0, 0, -1, COVOF_OK, 0};
    CK(cudaMemcpyAsync(h->d_run, h->h_run, sizeof(RunStats), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  bool graph = (flags & COVOF_RUN_GRAPH) != 0 && !b->graph_refused;
  // the first step of a case with Gear / Adams-Bashforth and no history yet
  // runs eagerly; the graphs are captured with every has_nm1 set
  bool first_plain = false;
  for (covof_handle* h : b->h) first_plain |= needs_history(h->prm) && !h->has_nm1;
  first_plain = first_plain && nsteps > 0;
  auto ensure_graphs = [&]() -> int {
    if (!graph) return COVOF_OK;
    bool same = b->graph[0] && b->graph_dt.size() == (size_t)b->ncases;
    for (int c = 0; same && c < b->ncases; ++c) same = b->graph_dt[c] == dt[c];
    if (!same) {
      const int st = capture(b, dt);
      if (st == COVOF_UNSUPPORTED) {
        b->graph_refused = true;
        graph = false;
      } else if (st != COVOF_OK) {
        return st;
      }
    }
    return COVOF_OK;
  };
  if (!first_plain) CS(ensure_graphs());
  CK(cudaEventRecord(b->ev0, b->stream));
  for (int k = 0; k < nsteps; ++k) {
    const bool x_first = (b->step_count % 2) == 0;
    if (graph && !(first_plain && k == 0)) CK(cudaGraphLaunch(b->graph[x_first ? 0 : 1], b->stream));
    else CS(enqueue_batch_step(b, dt, x_first));
    b->step_count += 1;
    if (k == 0) {
      for (covof_handle* h : b->h) h->has_nm1 = true;
      if (first_plain) {
        // the fork streams are idle before they join a capture
        CK(cudaStreamSynchronize(b->stream));
        drop_graphs(b);
        CS(ensure_graphs());
      }
    }
  }
  CK(cudaEventRecord(b->ev1, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  CK(cudaGetLastError());
  float el = 0.f;
  cudaEventElapsedTime(&el, b->ev0, b->ev1);
  if (ms) *ms = el;
  int status = COVOF_OK;
  for (int c = 0; c < b->ncases; ++c) {
    covof_handle* h = b->h[c];
    if (h->prm.enable_two_phase) h->vof_step_count += nsteps;
    CK(cudaMemcpy(h->h_run, h->d_run, sizeof(RunStats), cudaMemcpyDeviceToHost));
    const RunStats& r = *h->h_run;
    if (stats) {
      covof_run_stats& o = stats[c];
      o.steps = r.step;
      o.first_bad_step = r.first_bad_step;
      o.first_bad_status = r.first_bad_status;
      o.graph = graph ? 1 : 0;
      o.mom_iters = r.mom_iters;
      o.poisson_iters = r.poisson_iters;
      o.refine_steps = r.refine_steps;
      o.last_relres = r.last_relres;
      o.max_relres = r.max_relres;
      o.ms = el;
    }
    if (status == COVOF_OK && r.first_bad_step >= 0) status = r.first_bad_status;
  }
  return status;
}

}  // extern "C"

COVOF_UNIT_HOOKS(batch)
