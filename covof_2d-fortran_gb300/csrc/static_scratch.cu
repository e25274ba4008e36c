// static_scratch.cu -- allocation-free variant of the plain FP64 Poisson
// solve (covof_poisson_solve_rhs_static_dev).
//
// Some callers cannot allocate device memory when they call the solver: a
// host code whose device memory is handed out by its own pool allocator that
// reserved the whole GPU at start-up, or a driver loop that must not pay the
// implicit device-wide synchronisation of cudaMalloc/cudaFree between time
// steps.  This entry point takes no handle and allocates nothing: its scratch
// (solver vectors, coefficients, reduction partials, barrier words, result)
// lives in the file-scope array below, which every GPU that loads the library
// holds until the process exits.
#include <cstring>

#include "common.cuh"
#include "poisson.cuh"

using namespace covof;

namespace {

// Largest mesh served: (nx+2)*(ny+2) <= kMaxGhosted, e.g. 256 x 256 cells.
constexpr size_t kMaxGhosted = (size_t)258 * 258;
constexpr int kVectors = 10;            // x, b, r, d0, d1, Ad, ax, ay, aP, invD
constexpr size_t kMaxBlocks = 1024;     // partials for up to 1024 blocks
constexpr size_t kCtlWords = 1024;      // barrier counter + spare words
constexpr size_t kScratchBytes =
    kVectors * kMaxGhosted * sizeof(double) +   // 5.3 MB of vectors
    16 * kMaxBlocks * sizeof(double) +          // reduction partials
    kCtlWords * sizeof(unsigned int) +          // barrier / error words
    256;                                        // result record

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// The device address of g_scratch on the current device.  The host-side
// name g_scratch is only a stand-in; the kernels need the address, which is
// looked up on every call (cheap once the module is loaded; a first call on
// a device loads it, and a cudaDeviceReset can move the array, so no
// address is kept between calls).
int scratch_base(unsigned char** base) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return COVOF_CUDA_ERROR;
  *base = static_cast<unsigned char*>(p);
  return COVOF_OK;
}

int4 walls(const covof_params& p) {
  auto w = [&](int s) { return (p.bc_type[s] == COVOF_BC_DIRICHLET || p.bc_type[s] == COVOF_BC_FREESLIP) ? 1 : 0; };
  return make_int4(w(0), w(1), w(2), w(3));
}

}  // namespace

extern "C" int covof_poisson_solve_rhs_static_dev(const covof_params* prm, double dt, const double* b,
                                                  const double* rho_u, const double* rho_v, double* p,
                                                  int* iters, double* relres) {
  if (!prm || !b || !rho_u || !rho_v || !p) return COVOF_INVALID;
  const covof_params& P = *prm;
  if (P.nx < 2 || P.ny < 2 || !(P.dx > 0.0) || !(P.dy > 0.0)) return COVOF_INVALID;
  // this entry runs the plain FP64 Jacobi-PCG only
  if (P.p_precision != COVOF_PREC_FP64 || P.p_precond == COVOF_PRECOND_SSOR) return COVOF_UNSUPPORTED;
  for (int s = 0; s < 4; ++s)
    if (P.bc_type[s] != COVOF_BC_DIRICHLET && P.bc_type[s] != COVOF_BC_FREESLIP) return COVOF_UNSUPPORTED;
  const size_t g = (size_t)(P.nx + 2) * (size_t)(P.ny + 2);
  if (g > kMaxGhosted) return COVOF_TOO_LARGE;

  // an error left by the caller's earlier asynchronous work is reported as
  // such before the shared array is touched, not taken for this call's
  if (cudaGetLastError() != cudaSuccess) return COVOF_CUDA_ERROR;
  int dev = 0, sms = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return COVOF_CUDA_ERROR;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return COVOF_CUDA_ERROR;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
    return COVOF_UNSUPPORTED;
  unsigned char* base = nullptr;
  int st = scratch_base(&base);
  if (st != COVOF_OK) return st;

  // carve the array (every vector keeps a zero ghost ring)
  double* v = reinterpret_cast<double*>(base);
  double *x = v, *bb = v + g, *r = v + 2 * g, *d0 = v + 3 * g, *d1 = v + 4 * g, *Ad = v + 5 * g;
  double *ax = v + 6 * g, *ay = v + 7 * g, *aP = v + 8 * g, *invD = v + 9 * g;
  double* part = v + kVectors * kMaxGhosted;
  unsigned int* ctl = reinterpret_cast<unsigned int*>(part + 16 * kMaxBlocks);
  PcgResult* res = reinterpret_cast<PcgResult*>(ctl + kCtlWords);
  int* err = reinterpret_cast<int*>(ctl + 1);

  cudaStream_t s0 = 0;  // legacy default stream
  // The array keeps the previous call's contents, possibly for another mesh
  // size: clear every vector this call uses, and the control words.
  if (cudaMemsetAsync(v, 0, (size_t)kVectors * g * sizeof(double), s0) != cudaSuccess) return COVOF_CUDA_ERROR;
  if (cudaMemsetAsync(ctl, 0, kCtlWords * sizeof(unsigned int), s0) != cudaSuccess) return COVOF_CUDA_ERROR;

  const Dims D{P.nx, P.ny, P.nx + 2};
  const int pinned = P.p_gauge == COVOF_GAUGE_PINNED;
  const dim3 blk(32, 8), grd((P.nx + 31) / 32, (P.ny + 7) / 8);
  k_poisson_assemble<<<grd, blk, 0, s0>>>(D, dt, P.dx, P.dy, walls(P), rho_u, rho_v, nullptr, nullptr, b,
                                          pinned, ax, ay, aP, bb, nullptr, invD);
  k_copy_interior<<<grd, blk, 0, s0>>>(D, p, x, pinned);
  if (cudaGetLastError() != cudaSuccess) return COVOF_CUDA_ERROR;

  PoissonArgs a;
  std::memset(&a, 0, sizeof(a));
  a.D = D;
  a.x = x; a.b = bb; a.r = r; a.d = d0; a.d2 = d1; a.Ad = Ad;
  a.ax = ax; a.ay = ay; a.aP = aP; a.invD = invD;
  a.bar = ctl; a.err = err; a.part = part; a.res = res;
  a.tol = P.p_tol; a.max_iter = P.p_max_iter; a.pinned = pinned;
  const void* fn = (const void*)k_pcg_fp64;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 1024, 0) != cudaSuccess || per_sm < 1)
    return COVOF_CUDA_ERROR;
  long long nb = sms;
  const long long ntiles = make_tiles(D).ntiles;
  if (ntiles < nb) nb = ntiles;
  if (nb > (long long)per_sm * sms) nb = (long long)per_sm * sms;
  if (nb > (long long)kMaxBlocks) nb = kMaxBlocks;
  void* args[] = {&a};
  if (cudaLaunchCooperativeKernel(fn, dim3((unsigned)nb), dim3(1024), args, 0, s0) != cudaSuccess)
    return COVOF_CUDA_ERROR;
  k_copy_interior<<<grd, blk, 0, s0>>>(D, x, p, 0);
  PcgResult h;
  if (cudaMemcpyAsync(&h, res, sizeof(h), cudaMemcpyDeviceToHost, s0) != cudaSuccess) return COVOF_CUDA_ERROR;
  if (cudaStreamSynchronize(s0) != cudaSuccess || cudaGetLastError() != cudaSuccess) return COVOF_CUDA_ERROR;
  if (iters) *iters = h.iters;
  if (relres) *relres = h.relres;
  return h.status;
}

COVOF_UNIT_HOOKS(static_scratch)
