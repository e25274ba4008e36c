// common.cuh -- shared device helpers for the COVOF GB300 kernels.
//
// Field layout: the reference's (0:nx+1, 0:ny+1) Fortran arrays, i fastest,
// pitch nx+2 (src/module_fields.f90:129-169).  Device mirrors keep exactly
// that layout so host<->device copies are single contiguous memcpys.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "../../include/covof_gpu.h"

#define COVOF_WARP 32

namespace covof {

// Error word written by device code.  A bounded wait that gives up stores
// COVOF_TIMEOUT; the first writer wins.
__device__ __forceinline__ void set_error(int* err, int code) { atomicCAS(err, 0, code); }

// ---------------------------------------------------------------------------
// Bounds-check build (-DCOVOF_CHECKED): every cell index formed on the device
// through Dims::id and every stencil centre of the operators is checked
// against the (nx+2) x (ny+2) ghosted extents.  A bad index is counted, the
// first one recorded (site << 40 | index + 2^39), and the access redirected to
// a valid element instead of leaving the array; covof_bounds_check reads and
// clears the record.  One record per translation unit (no relocatable device
// code); COVOF_UNIT_HOOKS gives each unit its reader.  The normal build
// compiles every check away.
#ifdef COVOF_CHECKED
static __device__ unsigned long long g_oob_count = 0;
static __device__ unsigned long long g_oob_first = 0;
static __device__ __noinline__ void oob_record(int site, long long index) {
  if (atomicAdd(&g_oob_count, 1ULL) == 0ULL)
    g_oob_first = ((unsigned long long)site << 40) | (unsigned long long)(index + (1LL << 39));
}
#endif

struct Dims {
  int nx, ny, P;  // P = nx + 2
  // periodic directions (one rank: the ghost ring holds the wrapped
  // interior, src/module_mpi_comm.f90:46-56)
  int perx = 0, pery = 0;
  // the interior cell whose value a ghost cell (i, j) carries in a periodic
  // direction (i, j themselves otherwise)
  __host__ __device__ __forceinline__ int wrap_i(int i) const { return perx ? (i == 0 ? nx : (i == nx + 1 ? 1 : i)) : i; }
  __host__ __device__ __forceinline__ int wrap_j(int j) const { return pery ? (j == 0 ? ny : (j == ny + 1 ? 1 : j)) : j; }
  __host__ __device__ __forceinline__ int id(int i, int j) const {
#if defined(COVOF_CHECKED) && defined(__CUDA_ARCH__)
    if (i < 0 || i > nx + 1 || j < 0 || j > ny + 1) {
      oob_record(1, (long long)j * P + i);
      return 0;
    }
#endif
    return j * P + i;
  }
  // the 3 x 3 neighbourhood of cell k lies inside the ghosted array (checked
  // builds: else recorded under site and an interior cell returned)
  __device__ __forceinline__ int nbhd(int k, int site) const {
#ifdef COVOF_CHECKED
    if (k - P - 1 < 0 || (long long)k + P + 1 >= (long long)P * (ny + 2)) {
      oob_record(site, k);
      return P + 1;
    }
#else
    (void)site;
#endif
    return k;
  }
};

// ---------------------------------------------------------------------------
// Grid-wide barrier for kernels launched with cudaLaunchCooperativeKernel
// (co-residency of all blocks is guaranteed by that launch).  Counting form:
// thread 0 of every block adds 1 with release semantics to one counter and
// polls it with acquire loads until it reaches (epoch+1) * nblocks; no reset
// and no second word, so the critical path is one atomic and one poll.
// Every spin is bounded: after g_spin_limit polls (kSpinLimit, ~1-2 s,
// unless covof_set_wait_budget lowered it) the block records COVOF_TIMEOUT and
// returns false, and every caller leaves its loop; a block that left never
// arrives again, so every other block times out at its next barrier and no
// block can wait forever.  The counter must be zero at launch.
constexpr long long kSpinLimit = 1LL << 21;
// One copy per translation unit (the library is built without relocatable
// device code); COVOF_UNIT_HOOKS gives each unit its setter, and
// covof_set_wait_budget calls them all.
static __device__ long long g_spin_limit = kSpinLimit;
#ifdef COVOF_CHECKED
#define COVOF_BOUNDS_READER(unit)                                                                   \
  int bounds_check_##unit(unsigned long long* count, unsigned long long* first) {                   \
    const unsigned long long zero = 0;                                                             \
    if (cudaMemcpyFromSymbol(count, g_oob_count, sizeof(*count)) != cudaSuccess ||                 \
        cudaMemcpyFromSymbol(first, g_oob_first, sizeof(*first)) != cudaSuccess ||                 \
        cudaMemcpyToSymbol(g_oob_count, &zero, sizeof(zero)) != cudaSuccess ||                     \
        cudaMemcpyToSymbol(g_oob_first, &zero, sizeof(zero)) != cudaSuccess)                       \
      return 6;                                                                                    \
    return 0;                                                                                      \
  }
#else
#define COVOF_BOUNDS_READER(unit)                                                      \
  int bounds_check_##unit(unsigned long long* count, unsigned long long* first) {      \
    *count = 0;                                                                       \
    *first = 0;                                                                       \
    return 5;                                                                         \
  }
#endif
// Per-unit hooks: the wait budget setter and the bounds record reader.
#define COVOF_UNIT_HOOKS(unit)                                                            \
  namespace covof {                                                                      \
  int set_wait_budget_##unit(long long polls) {                                          \
    return cudaMemcpyToSymbol(g_spin_limit, &polls, sizeof(polls)) == cudaSuccess ? 0 : 6; \
  }                                                                                      \
  COVOF_BOUNDS_READER(unit)                                                              \
  }

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_add_release_u32(unsigned int* p, unsigned int v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release_u32(unsigned int* p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// lane 0 waits until *p >= need (bounded); the warp learns the outcome
__device__ __forceinline__ bool warp_wait_ge(const unsigned int* p, unsigned int need, int* err) {
  int ok = 1;
  if ((threadIdx.x & 31) == 0) {
    long long spins = 0;
    while ((int)(ld_acquire_u32(p) - need) < 0) {
      if (++spins > g_spin_limit) { set_error(err, COVOF_TIMEOUT); ok = 0; break; }
    }
  }
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

// x / b, correctly rounded, from yb = RN(1 / b): q0 = RN(x yb) is within one
// ulp of x / b, the remainder x - b q0 is exact in one FMA, and one FMA
// correction step q0 + r yb rounds to the correctly rounded quotient
// (P. Markstein, "IA-64 and Elementary Functions", 2000, Theorem 8.10; x, b
// normal, x / b in range).  Three dependent FP64 operations instead of a
// full division.
__device__ __forceinline__ double div_rcp(double x, double b, double yb) {
  const double q0 = __dmul_rn(x, yb);
  const double r = __fma_rn(-b, q0, x);
  return __fma_rn(r, yb, q0);
}

struct GridSync {
  unsigned int* count;
  int* err;
  unsigned int nblocks;
  unsigned int epoch;
  __device__ bool sync() {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
      int ok = 1;
      red_add_release_u32(count, 1u);
      const unsigned int target = (epoch + 1u) * nblocks;
      long long spins = 0;
      while ((int)(ld_acquire_u32(count) - target) < 0) {
        if (++spins > g_spin_limit) { set_error(err, COVOF_TIMEOUT); ok = 0; break; }
      }
      s_ok = ok;
    }
    epoch++;
    __syncthreads();
    return s_ok != 0;
  }
};

// ---------------------------------------------------------------------------
// Deterministic reductions.  Block partials are combined by every block in
// the same fixed order, so all blocks obtain bit-identical totals and take
// identical convergence decisions.
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum NV values per thread across the block; result valid in thread 0.
template <typename T, int NV>
__device__ __forceinline__ void block_sum(T (&v)[NV]) {
  __shared__ T sh[NV][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k][wid] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      T t = lane < nw ? sh[k][lane] : T(0);
      v[k] = warp_sum(t);
    }
  }
  __syncthreads();
}

// Fused hypot: sqrt(x^2+y^2) with an FMA-based residual correction (after
// C. F. Borges, "An improved algorithm for hypot(a,b)", ACM TOMS 2021).  Each
// operation is an explicit IEEE round-to-nearest intrinsic so the result is
// identical to the host implementation bit for bit.
__device__ __forceinline__ double fhypot(double x, double y) {
  double ax = fabs(x), ay = fabs(y);
  if (isinf(ax) || isinf(ay)) return __longlong_as_double(0x7ff0000000000000LL);
  if (isnan(ax) || isnan(ay)) return __dadd_rn(ax, ay);
  if (ax < ay) { double t = ax; ax = ay; ay = t; }
  if (ay == 0.0) return ax;
  if (ay < __dmul_rn(ax, 0x1p-30)) return ax;
  double scale = 1.0;
  if (ax > 0x1p+500) { ax = __dmul_rn(ax, 0x1p-600); ay = __dmul_rn(ay, 0x1p-600); scale = 0x1p+600; }
  else if (ax < 0x1p-450) { ax = __dmul_rn(ax, 0x1p+600); ay = __dmul_rn(ay, 0x1p+600); scale = 0x1p-600; }
  double h = __dsqrt_rn(__fma_rn(ax, ax, __dmul_rn(ay, ay)));
  double h_sq = __dmul_rn(h, h), h_lo = __fma_rn(h, h, -h_sq);
  double x_sq = __dmul_rn(ax, ax), x_lo = __fma_rn(ax, ax, -x_sq);
  double y_sq = __dmul_rn(ay, ay), y_lo = __fma_rn(ay, ay, -y_sq);
  double r = __dadd_rn(__dadd_rn(__dsub_rn(x_sq, h_sq), y_sq), __dadd_rn(__dsub_rn(x_lo, h_lo), y_lo));
  h = __dadd_rn(h, __ddiv_rn(r, __dmul_rn(2.0, h)));
  return __dmul_rn(h, scale);
}

}  // namespace covof

namespace covof {

// Grid-wide sum of up to 8 FP64 values per thread, deterministic: block
// partials are written to one of two regions, the grid meets at the
// barrier, then every block combines all partials in the same fixed order
// (warp 0: strided partial sums, then a shuffle tree), so all blocks obtain
// bit-identical totals.  Consecutive reductions alternate regions, so a
// region is rewritten only after every block has passed the barrier that
// follows its last read.  part must hold 2 * 8 * nblocks doubles (nblocks =
// the team size).
// A team: the blocks of one cooperative launch that work on one case (all
// of the grid for a single-case solve; a slice of it when many cases share
// one persistent launch).  rank in [0, size); barriers, reductions and work
// distribution are over the team only.
struct Team {
  int rank, size;
};
__device__ __forceinline__ Team grid_team() { return Team{(int)blockIdx.x, (int)gridDim.x}; }

// Many cases in one persistent cooperative launch: the grid is cut into
// teams (contiguous block ranges); each team solves its list of cases one
// after another with barriers, reductions and publish counters of its own.
struct BatchTeams {
  const int* block_team;   // [nblocks] team of each block
  const int4* team;        // [nteams] first block, size, [begin, end) in case_list
  const int* case_list;    // case indices, grouped by team
  unsigned int* bar;       // [32 * nteams] barrier counter per team (one 128-byte line each)
  unsigned int* flags;     // [nblocks] publish counters (Chebyshev neighbour exchange)
  int* err;                // [nteams] error words
  double* part;            // [16 * nblocks] reduction partials (2 regions x 8 per block)
  float* xb;               // [4 * nblocks * xbw] boundary-row exchange (shared-memory inner form)
  int xbw;                 // row length of xb: largest nx + 2 of the batch
};

// This block's team, its reducer (partials, barrier and error word of the team).
__device__ __forceinline__ Team batch_team(const BatchTeams& bt, int4& T) {
  T = bt.team[bt.block_team[blockIdx.x]];
  return Team{(int)blockIdx.x - T.x, T.y};
}

struct GridReducer {
  double* part;
  GridSync gs;
  int region;
  int rank;  // this block's partials slot (its team rank)
  template <int NV>
  __device__ bool sum(double (&v)[NV]) {
    return sum_map<NV, NV>(v, v, [](const double* w, double* o) {
#pragma unroll
      for (int q = 0; q < NV; ++q) o[q] = w[q];
    });
  }

  // As sum(), but thread 0 maps the NV totals to NO scalars before the
  // broadcast.  FP64 issue is the scarce resource of a GB300 SM: a division
  // or square root evaluated by every warp of a 1024-thread block costs as
  // much as a whole stencil sweep, so scalar recurrences (step lengths,
  // norms, convergence flags) run once per block, in thread 0, which may
  // also keep private state (e.g. the previous <r,z>) across calls.
  template <int NV, int NO, class F>
  __device__ bool sum_map(double (&v)[NV], double (&out)[NO], F f) {
    static_assert(NV <= 8 && NO <= 8, "at most 8 values");
    block_sum<double, NV>(v);
    double* base = part + (size_t)region * gs.nblocks * 8;
    if (threadIdx.x == 0) {
#pragma unroll
      for (int q = 0; q < NV; ++q) base[rank * 8 + q] = v[q];
    }
    const bool ok = gs.sync();
    __shared__ double sh[8];
    // the fixed-order combine runs in warp 0 only
    if (threadIdx.x < 32) {
      double w[NV];
#pragma unroll
      for (int q = 0; q < NV; ++q) w[q] = 0.0;
      for (int b = threadIdx.x; b < (int)gs.nblocks; b += 32) {
#pragma unroll
        for (int q = 0; q < NV; ++q) w[q] += __ldcg(base + b * 8 + q);
      }
#pragma unroll
      for (int q = 0; q < NV; ++q) w[q] = warp_sum(w[q]);
      if (threadIdx.x == 0) {
        double o[NO];
        f(w, o);
#pragma unroll
        for (int q = 0; q < NO; ++q) sh[q] = o[q];
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NO; ++q) out[q] = sh[q];
    __syncthreads();
    region ^= 1;
    return ok;
  }
};

}  // namespace covof
