// handle.cuh -- internal: the handle behind covof_handle* and the enqueue
// helpers of capi.cu that the batch engine (batch.cu) reuses.  Not part of
// the C ABI.
#pragma once
#include <cstring>

#include "common.cuh"
#include "momentum.cuh"
#include "poisson.cuh"
#include "vof.cuh"
#include "adjoint.cuh"

namespace covof {
// the bounded waits' poll budget of each translation unit (common.cuh)
int set_wait_budget_poisson(long long);
int set_wait_budget_momentum(long long);
int set_wait_budget_vof(long long);
int set_wait_budget_svof(long long);
int set_wait_budget_adjoint(long long);
int set_wait_budget_output(long long);
int set_wait_budget_precond(long long);
int set_wait_budget_peak(long long);
int set_wait_budget_batch(long long);
int set_wait_budget_capi(long long);
int set_wait_budget_static_scratch(long long);
// the bounds-check record of each translation unit (common.cuh)
int bounds_check_poisson(unsigned long long*, unsigned long long*);
int bounds_check_momentum(unsigned long long*, unsigned long long*);
int bounds_check_vof(unsigned long long*, unsigned long long*);
int bounds_check_svof(unsigned long long*, unsigned long long*);
int bounds_check_adjoint(unsigned long long*, unsigned long long*);
int bounds_check_output(unsigned long long*, unsigned long long*);
int bounds_check_precond(unsigned long long*, unsigned long long*);
int bounds_check_peak(unsigned long long*, unsigned long long*);
int bounds_check_batch(unsigned long long*, unsigned long long*);
int bounds_check_capi(unsigned long long*, unsigned long long*);
int bounds_check_static_scratch(unsigned long long*, unsigned long long*);

namespace host {

constexpr int kPoissonThreads = 1024;  // one cell per thread per 1024-cell tile
constexpr int kKrylovThreads = 512;    // momentum Krylov kernels (64 registers)
constexpr int kKrylovBlocksPerSm = 2;  // co-resident momentum Krylov blocks per SM
constexpr int kVofCellMin = 16384;   // interface cells from which reconstruction runs a thread per cell
constexpr int kMaxPartRegions = 16;  // doubles per block in the partials array

template <typename T>
inline int dalloc(T** p, size_t n) {
  if (cudaMalloc((void**)p, n * sizeof(T)) != cudaSuccess) { *p = nullptr; return COVOF_CUDA_ERROR; }
  if (cudaMemset(*p, 0, n * sizeof(T)) != cudaSuccess) return COVOF_CUDA_ERROR;
  return COVOF_OK;
}
template <typename T>
inline void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

#define CK(call)                                      \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return COVOF_CUDA_ERROR;   \
  } while (0)
#define CS(call)                          \
  do {                                    \
    int s_ = (call);                      \
    if (s_ != COVOF_OK) return s_;        \
  } while (0)

// Device-side statistics of a resident run, folded in by k_step_log after
// every step so that the host reads them once at the end.
struct RunStats {
  long long mom_iters, poisson_iters, refine_steps;
  double last_relres, max_relres;
  int step, first_bad_step, first_bad_status, pad;
};

// One thread: fold this step's predictor and Poisson result records in.
__global__ void k_step_log(const KrylovResult* kr, const PcgResult* pr, RunStats* s);

// Buffers of the sweep preconditioners (SSOR, BLOCK_TRIANGULAR; precond.cu),
// allocated on first use.
struct SweepKit {
  bool ready = false;
  size_t n = 0;                 // entries of a packed Krylov vector
  double* coef = nullptr;       // 18 arrays of (nx+2)*(ny+2): the u, v, Schur stencils
  PBlk blk{};
  double* t[3] = {};            // scratch vectors: A x, the block-triangular rhs, M^-1 b
  unsigned int* prog = nullptr; // wavefront progress, per job and band
  int max_bands = 0, cap = 0, dot_blocks = 0;
  double *part = nullptr, *dsum = nullptr, *hdot = nullptr;  // dot products (hdot pinned)
};

}  // namespace host
}  // namespace covof

struct covof_handle {
  using Dims = covof::Dims;
  using PcgResult = covof::PcgResult;
  using KrylovResult = covof::KrylovResult;
  covof_params prm;
  int device = 0, sm_count = 0;
  cudaStream_t stream = nullptr;
  Dims D{};
  size_t g = 0;
  int vof_step_count = 0;
  bool has_nm1 = false;  // u_nm1 / v_nm1 hold step n-1 (fields%has_nm1)
  double* al_r = nullptr;                // augmented Lagrangian penalty field r_aal
  unsigned long long* al_max = nullptr;  // maxima of the penalty scales and of |div u|
  bool al_check = false;                // resident steps test the Uzawa exit on the host
  void* writer = nullptr;               // snapshot output state (output.cu)
  unsigned int* svof_prog = nullptr;  // SVOF band progress (32 words per band)
  int svof_nb = 0;                    // blocks of the SVOF launch (planned by ensure_vof)
  int vof_cell_nb = 0;                // blocks of the thread-per-cell reconstruction (ensure_vof)
  // ELVIRA's block-per-cell latency form for short interface lists: on for
  // a case that has the GPU to itself, off in a batch (many cases at once:
  // there throughput counts, and the block form does 2.5x the clips per cell)
  bool vof_block_form = true;
  // caller-field mirrors (host-pointer entry points)
  bool have_fields = false;
  double *f_u = nullptr, *f_v = nullptr, *f_p = nullptr, *f_rho_u = nullptr, *f_rho_v = nullptr,
         *f_mu = nullptr, *f_mu_node = nullptr, *f_fx = nullptr, *f_fy = nullptr,
         *f_u_old = nullptr, *f_v_old = nullptr, *f_u_nm1 = nullptr, *f_v_nm1 = nullptr,
         *f_Cs = nullptr, *f_Ct = nullptr, *dscr = nullptr,
         *f_C = nullptr, *f_rho = nullptr,
         *f_curv = nullptr, *f_b = nullptr, *f_x2 = nullptr, *f_seg = nullptr;
  // Poisson scratch
  bool have_poisson = false;
  double *px = nullptr, *pb = nullptr, *pr = nullptr, *pd = nullptr, *pAd = nullptr,
         *pax = nullptr, *pay = nullptr, *paP = nullptr, *pisd = nullptr, *pinvD = nullptr,
         *pd2 = nullptr, *pz = nullptr, *pw = nullptr, *pp = nullptr, *pq = nullptr;
  float* pxb = nullptr;  // boundary-row exchange of the shared-memory inner solver
  float *e32 = nullptr, *r32b = nullptr, *r32 = nullptr, *d32 = nullptr, *d32b = nullptr, *Ad32 = nullptr,
        *ax32 = nullptr, *ay32 = nullptr, *aP32 = nullptr;
  covof::MgHier mg{};  // multigrid hierarchy of the FP32 inner operator (pool: levels >= 1)
  // pinned gauge through the reference gauge: partial sums and levels, the
  // control ints, the consistent right-hand side
  double* pin_part = nullptr;
  int* pin_ctl = nullptr;
  double* pin_b = nullptr;
  // momentum scratch (each 2g)
  bool have_mom = false;
  double *mx = nullptr, *mrhs = nullptr, *mdiag = nullptr, *mv[7] = {};
  double *mcoef = nullptr, *midiag = nullptr;  // assembled operator rows, inverse diagonal
  covof::host::SweepKit sweep;                   // SSOR / BLOCK_TRIANGULAR preconditioners
  // VOF scratch
  bool have_vof = false;
  double *cs = nullptr, *seg = nullptr, *cnx = nullptr, *cny = nullptr, *ckap = nullptr;
  int *vlist = nullptr, *vcount = nullptr;  // interface-cell list of the reconstruction
  // adjoint scratch
  bool have_adj = false;
  double *arhs = nullptr, *apsi = nullptr, *apart = nullptr, *asum = nullptr;
  double *f_gu = nullptr, *f_gv = nullptr, *f_gp = nullptr, *f_gbu = nullptr, *f_gbv = nullptr,
         *f_ou = nullptr, *f_ov = nullptr;
  // control
  unsigned int* bar = nullptr;  // [0] grid barrier counter, [64..) per-block publish counters
  int* err = nullptr;
  double* part = nullptr;
  int part_blocks = 0;
  PcgResult* d_pres = nullptr;
  KrylovResult* d_kres = nullptr;
  PcgResult* h_pres = nullptr;
  KrylovResult* h_kres = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_solve_ms = 0.0;
  int last_refine = 0;
  // launch plans, fixed for the handle's mesh and parameters (computed once,
  // so that a stream capture records launches only)
  bool have_pplan = false;
  covof_launch launch{};   // overrides of the planning rules (zero: rule)
  const void* p_fn = nullptr;
  size_t p_smem = 0;
  int p_nb = 0, p_threads = 0;
  bool p_cluster = false;  // the plan is one thread-block cluster (k_pcg_mixed_cluster)
  bool have_mplan = false;
  const void* m_fn = nullptr;
  int m_nb = 0;
  // resident time stepping
  cudaStream_t cap_stream = nullptr;       // non-blocking stream used only while capturing
  cudaGraphExec_t step_graph[2] = {};      // [0]: x-first Weymouth-Yue order, [1]: y-first
  double graph_dt = 0.0;
  bool graph_refused = false;
  covof::host::RunStats* d_run = nullptr;
  covof::host::RunStats* h_run = nullptr;
  cudaEvent_t ev2 = nullptr, ev3 = nullptr;
};

namespace covof {
namespace host {

// Helpers of capi.cu shared with the batch engine (batch.cu).
int ensure_fields(covof_handle* h);
int ensure_poisson(covof_handle* h);
int ensure_mom(covof_handle* h);
int ensure_vof(covof_handle* h);
int check_mom_params(const covof_params& P);
int poisson_plan(covof_handle* h);
int predictor_plan(covof_handle* h);
int4 wall_flags(const covof_params& p);
bool mg_path(const covof_params& p);
bool periodic(const covof_params& p);
int check_periodic_vof(const covof_params& p);
dim3 grid2(int ni, int nj, dim3 b);
int sync(covof_handle* h);
int pois_pre(covof_handle* h, double dt, const double* u, const double* v, const double* b,
             const double* rho_u, const double* rho_v, double* p, PoissonArgs* out);
int pois_post(covof_handle* h, double* p);
int mom_pre(covof_handle* h, double dt, double* u, double* v, const double* rho_u, const double* rho_v,
            const double* mu, const double* mu_node, const double* fx, const double* fy, const double* u_old,
            const double* v_old, MomArgs* out);
int mom_post(covof_handle* h, const MomArgs& a, double* u, double* v);
int wy_step_dev(covof_handle* h, double dt, int x_first, const double* u, const double* v, double* C);
bool needs_history(const covof_params& P);
void writer_destroy(covof_handle* h);
bool is_al(const covof_params& P);
int check_coupling(const covof_params& P);
int al_enqueue(covof_handle* h, double dt, double* u, double* v, double* p, const double* rho,
               const double* rho_u, const double* rho_v, const double* mu, const double* mu_node,
               const double* fx, const double* fy, const double* u_old, const double* v_old, bool host_check,
               int* total_iters, int* uzawa_done);
int rotate_history(covof_handle* h);
void drop_graphs(covof_handle* h);
int vof_bc_dev(covof_handle* h, double* C);
int props_dev(covof_handle* h, double* C, double* rho, double* rho_u, double* rho_v, double* mu,
              double* mu_node, const double* Cs = nullptr);
int csf_dev(covof_handle* h, const double* C, double* fx, double* fy, double* curv,
            const double* Cs = nullptr, const double* Ct = nullptr);
int svof_dev(covof_handle* h, const double* C, double* Cs);
int diffusion_dev(covof_handle* h, const double* C, double* Ct);
int smooth_props_csf(covof_handle* h, bool svof_now);
int velocity_bc_dev(covof_handle* h, double* u, double* v);
int correct_dev(covof_handle* h, double dt, double* u, double* v, const double* p, const double* rho_u,
                const double* rho_v);
double** field_slot(covof_handle* h, int f);
// precond.cu
bool uses_sweeps(const covof_params& P);
int ensure_sweeps(covof_handle* h);
void sweep_free(covof_handle* h);
int prec_blocks_dev(covof_handle* h, const MomArgs& a);
int sweep_precond(covof_handle* h, const MomArgs& a, const double* src, double* dst);
int sweep_solve(covof_handle* h, const MomArgs& a);
int precond_apply_dev(covof_handle* h, const MomArgs& a, const double* src, double* dst);
int pcg_sgs(covof_handle* h, const PoissonArgs& a);

}  // namespace host
}  // namespace covof
