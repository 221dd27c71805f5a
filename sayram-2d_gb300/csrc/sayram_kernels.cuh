// sayram_kernels.cuh -- sm_103a kernels of the Sayram-2D per-step hot path.
//
// Storage (all instances of a batch share one flat, padded, system-ordered layout):
//   instance b, cell (i, j) lives at index base_b + j*pitch_b + i, with pitch_b = nx_b rounded up
//   to a multiple of 4 and one zero row above (j = -1) and below (j = ny) every instance. The
//   reference's system order K = j*nx + i (Mesh.h:66-68) is kept inside each row. Every array
//   is zero in the padding and the pad rows and no kernel ever writes there, so the 5-point
//   stencil needs no bounds tests: out-of-domain neighbours contribute 0 * 0.
//
// Linear system (Jacobi-scaled, column form): with D = diag(M) the solver works on y = D f and
//   A~ = M D^{-1}, which has a unit diagonal.  Row L stores the four off-diagonal magnitudes
//   cw[L] = A_{W->L}/D_W (the west neighbour's outflow fraction through the face it shares with
//   L), ce, cs, cn likewise, so (A~ y)_L = y_L - (cw y_W + ce y_E + cs y_S + cn y_N).  Column K of
//   A~ holds -A_{K,sigma}/D_K, the fractions of K's outflow; they are >= 0 and sum to < 1 (M is a
//   column-diagonally-dominant M-matrix), which keeps FP32 storage well scaled and makes the
//   positivity polish y' = R + (I - A~) max(y, 0) a 1-norm contraction.
//
// Reductions are deterministic: every chunk (1024, 2048 or 4096 cells, chosen per batch) writes
// its partial sums, and the last block to finish an instance's chunks (counted with one atomic
// per chunk) adds them in chunk order and updates that instance's Krylov scalars.  No kernel waits on another block.
#pragma once

#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

namespace sg {

constexpr int kThreads = 256;  // threads per block of the streaming kernels
constexpr int kTX = 32;        // assembly tile width (alpha0, contiguous)
constexpr int kTY = 16;        // assembly tile height (log E)
constexpr int kAsmThreads = 256;
constexpr int kAsmGridPerSm = 96;  // k_assemble blocks launched per SM (grid-stride over tiles)
constexpr int kFieldThreads = 256;  // threads per block of the layout transforms
constexpr double kEps = DBL_EPSILON;  // gEPS, source/common.h:38

enum { XMIN = 0, XMAX = 1, YMIN = 2, YMAX = 3 };
enum { DIRICHLET = 0, ZEROFLUX = 1 };
enum { ST_OK = 0, ST_NOT_CONVERGED = 3, ST_NEGATIVE = 4 };
enum { PH_K1 = 0, PH_K2 = 1, PH_K3 = 2, PH_RESID = 3, PH_POLISH = 4, PH_COUNT = 8 };

// Per-instance constants.
struct InstDev {
  int nx, ny, pitch, enabled;
  int bc[4];
  long long base;  // index of cell (0,0) in the padded storage
  long long hoff;  // offset of the instance in the packed alpha-major host layout
  int chunk0, nchunks;
  int tile0, ntx, nty, pad0;
  int xe, ye;     // offsets into the per-vertex-column / per-vertex-row arrays (nx+1 / ny+1)
  int dir[4];     // offsets into the Dirichlet vertex value array (-1 for zero-flux sides)
  double dt;
};

// Per-instance solver state (mutable, device resident).
struct InstState {
  double rho, alpha, omega, beta;
  double rr, rr_target, bb, rr64;
  double rel, mass_drift, min_f, pad_d;
  long long clamped, steps;
  long long cum_iters, cum_refines;  // totals since creation (work accounting)
  int ycur, pcur, outer_active, inner_active;
  int restart, fresh, has_x, iters;
  int iters_total, refines, status;
  int nhist;               // earlier states held in the history buffers (extrapolated start)
  int hslot;               // history buffer holding f^(n-1); f^(n-2), ... are in the ones before it
  unsigned int rmax_bits;  // bits of max |R| over the instance (non-negative float; atomicMax order)
  unsigned int cnt[PH_COUNT];
};

// Batch-wide control words.
struct Ctl {
  int n_outer;   // instances still refining in this step
  int n_inner;   // instances inside an inner Krylov solve
  unsigned long long launches;  // kernel launches (block 0 of every kernel adds one)
  unsigned int kdone[8];        // blocks finished per kernel (graph-conditional updates)
  unsigned int outer_loops;     // residual evaluations run by the device-side loop this step
  unsigned int inner_loops;     // Krylov iterations run by the device-side loop this solve
  int go_outer, go_inner;       // the loop decisions of the cooperative solve (k_solve_coop)
};

template <typename T>
struct Q4 {
  T a[4];
};

__device__ __forceinline__ Q4<float> ld4(const float* p) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  return Q4<float>{{v.x, v.y, v.z, v.w}};
}
__device__ __forceinline__ Q4<double> ld4(const double* p) {
  const double2 u = reinterpret_cast<const double2*>(p)[0];
  const double2 w = reinterpret_cast<const double2*>(p)[1];
  return Q4<double>{{u.x, u.y, w.x, w.y}};
}
__device__ __forceinline__ void st4(float* p, const Q4<float>& q) {
  *reinterpret_cast<float4*>(p) = make_float4(q.a[0], q.a[1], q.a[2], q.a[3]);
}
__device__ __forceinline__ void st4(double* p, const Q4<double>& q) {
  reinterpret_cast<double2*>(p)[0] = make_double2(q.a[0], q.a[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(q.a[2], q.a[3]);
}

// Element i of a small pointer array inside a kernel parameter, chosen by selects: indexing the
// array with a run-time value makes every thread of every block copy the whole parameter to
// local memory first (with a grid of ~14,000 assembly blocks, ~300 MB of local stores a launch).
template <typename P>
__device__ __forceinline__ P sel2(P const (&a)[2], int i) {
  return i ? a[1] : a[0];
}
template <typename P>
__device__ __forceinline__ P sel3(P const (&a)[3], int i) {
  return i == 0 ? a[0] : (i == 1 ? a[1] : a[2]);
}

__device__ __forceinline__ void count_launch(Ctl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctl->launches, 1ull);
}

// Sum of NQ values over the block (result valid in thread 0). T is the warp-level type.
template <int NQ, typename T>
__device__ __forceinline__ void block_sum(T (&v)[NQ], double (&out)[NQ]) {
  __shared__ double sm[NQ][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    T x = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sm[q][warp] = (double)x;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double x = lane < nw ? sm[q][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      out[q] = x;
    }
  }
  __syncthreads();
}

// Sum over the block of per-warp totals held in lane 0 of each warp (result in thread 0).
template <int NQ>
__device__ __forceinline__ void block_sum_lane0(const double (&w)[NQ], double (&out)[NQ]) {
  __shared__ double sm0[NQ][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; ++q) sm0[q][warp] = w[q];
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double x = lane < nw ? sm0[q][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      out[q] = x;
    }
  }
  __syncthreads();
}

// Chunk-partial bookkeeping: thread 0 stores this chunk's partials, then the block learns whether
// it is the last of the instance's chunks for this phase. If so, totals (in chunk order) are
// returned in tot (valid in thread 0) and the phase counter is reset.
template <int NQ>
__device__ __forceinline__ bool chunk_finish(InstState& st, int phase, int chunk0, int nchunks,
                                             int chunk, double* part, const double (&mine)[NQ],
                                             double (&tot)[NQ]) {
  __shared__ int s_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) part[(size_t)chunk * 4 + q] = mine[q];
    __threadfence();
    const unsigned prev = atomicAdd(&st.cnt[phase], 1u);
    s_last = (prev == (unsigned)(nchunks - 1));
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  double acc[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) acc[q] = 0.0;
  for (int k = threadIdx.x; k < nchunks; k += blockDim.x)
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] += __ldcg(&part[(size_t)(chunk0 + k) * 4 + q]);
  block_sum<NQ, double>(acc, tot);
  if (threadIdx.x == 0) st.cnt[phase] = 0;
  return true;
}

}  // namespace sg
