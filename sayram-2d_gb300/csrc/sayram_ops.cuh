// sayram_ops.cuh -- the kernels of one backward-Euler step (see sayram_kernels.cuh for layout).
//
//   k_setup      once per instance: coefficients -> per-cell face factors, UKK, loss diagonal
//   k_dtable     on demand: D fields interpolated from a D table -> the face factors again
//   k_begin      per step: resets the per-instance solver state
//   k_assemble   fused vertex interpolation + PPFV face fluxes + diagonal/RHS + Jacobi scaling
//   k_resid      outer residual r = R - A~ y (adds the last Krylov correction first)
//   k_bicg1/2/3  one BiCGSTAB iteration in T precision (FP64 or FP32) with fused SpMV + dots
//   k_polish     positivity polish y' = R + (I - A~) y+, f = y'/D, min / clamp / mass checks
//   k_field_*    alpha-major FP64 <-> padded system order transposes for the host-buffer step
//
// The assembly, residual, polish and state are written once over an arithmetic policy A:
//   F64A  IEEE binary64 (the FP64 drop-in and the FP32 + FP64-residual mode)
//   DWA   double-word pairs of FP32 (dword.cuh): FP64-class accuracy on the FP32 pipes
// Per-cell "wide" arrays (f, 1/D, R, column sums, y, the face factors, the weights and Dirichlet
// values) hold 8 bytes per entry in both: one double, or one (hi, lo) float pair.
#pragma once

#include <cooperative_groups.h>

#include "dword.cuh"
#include "sayram_kernels.cuh"

namespace sg {

// ------------------------------------------------------------------------------ arguments
struct Geo {  // per-cell face factors (time independent while the coefficients are)
  double *aAx, *aBx, *Sx, *aAy, *aBy, *Sy, *ukk, *sdiag;
  double* G;  // G per cell, FP64 (kept so that new D fields can re-derive the face factors)
  double* decay;  // 1 / (1 + dt/tau): one step of pure loss (extrapolated start); null: 1
};

struct Common {
  const InstDev* inst;
  InstState* st;
  Ctl* ctl;
  const int* chunk_inst;
  int nchunks;
  const int* tile_inst;
  int ntiles;
  int ninst;
  const double* wx;    // per vertex column: (wL, wR) bilinear weights (Solver.cc:333-336)
  const double* wy;    // per vertex row: (wB, wT)
  const double* dirv;  // Dirichlet vertex values
  double* part;        // 4 doubles per chunk
  // when set, [nchunks, ntiles, ninst] are read from device memory (lists that change between
  // steps, as in the server) instead of the by-value counts above
  const int* dyn;
  int pmax;  // largest row pitch of any instance (shared-memory halo of the SpMV kernels)
  // device-side loops of the per-step CUDA graph (use_cond = 0: the host drives the loops; 1: the
  // graph's WHILE nodes; 2: the cooperative solve kernel)
  unsigned long long h_outer, h_inner;  // cudaGraphConditionalHandle of the two WHILE nodes
  int use_cond;
  int guard_refine, guard_iters;  // hard caps on loop trips, whatever the bookkeeping says
  int hist_cap;  // history depth used for the starting point (kHist; 1 when the buffers alias)
  int precond;   // 1: the inner Krylov solve is preconditioned on the left by the alpha-line blocks
};

__device__ __forceinline__ int n_chunks(const Common& cm) { return cm.dyn ? cm.dyn[0] : cm.nchunks; }
__device__ __forceinline__ int n_tiles(const Common& cm) { return cm.dyn ? cm.dyn[1] : cm.ntiles; }
__device__ __forceinline__ int n_inst(const Common& cm) { return cm.dyn ? cm.dyn[2] : cm.ninst; }

// The last block of a loop-deciding kernel sets the graph's WHILE conditions from the number of
// instances still active. The trip counters make both loops terminate after guard_refine
// residual evaluations and guard_iters Krylov iterations even if the counts were inconsistent.
// which = 0: after the residual (decides both loops); which = 1: after a Krylov iteration.
__device__ __forceinline__ void loop_epilogue(const Common& cm, int which) {
  if (!cm.use_cond) return;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(&cm.ctl->kdone[which], 1u);
    if (prev == gridDim.x - 1) {
      __threadfence();
      const int nout = atomicAdd(&cm.ctl->n_outer, 0);
      const int nin = atomicAdd(&cm.ctl->n_inner, 0);
      unsigned go_o = 0u, go_i;
      if (which == 0) {
        const unsigned lo = atomicAdd(&cm.ctl->outer_loops, 1u) + 1u;
        atomicExch(&cm.ctl->inner_loops, 0u);
        go_o = (nout > 0 && lo < (unsigned)cm.guard_refine) ? 1u : 0u;
        go_i = (nin > 0 && lo < (unsigned)cm.guard_refine) ? 1u : 0u;
      } else {
        const unsigned li = atomicAdd(&cm.ctl->inner_loops, 1u) + 1u;
        go_i = (nin > 0 && li < (unsigned)cm.guard_iters) ? 1u : 0u;
      }
      if (cm.use_cond == 1) {
        if (which == 0) cudaGraphSetConditional(cm.h_outer, go_o);
        cudaGraphSetConditional(cm.h_inner, go_i);
      } else {  // read by every block of the cooperative solve after its next grid barrier
        if (which == 0) atomicExch(&cm.ctl->go_outer, (int)go_o);
        atomicExch(&cm.ctl->go_inner, (int)go_i);
      }
      atomicExch(&cm.ctl->kdone[which], 0u);
    }
  }
}

template <typename C>
struct Coef {  // row-oriented scaled off-diagonal magnitudes (hi parts when split)
  C *cw, *ce, *cs, *cn;
  float *lw, *le, *ls, *ln;  // low parts for the FP32-split storage (null for FP64)
};

constexpr int kOrder = 4;  // earlier states the extrapolated start of each solve goes back
constexpr int kHist = 3;   // history buffers: with f^n (the state the polish replaces) they hold kOrder

struct Fields {
  double* f;       // state, padded system order
  double* fh[kHist];  // earlier states f^(n-1) .. f^(n-3), rotated per instance (InstState::hslot)
  const double* decay;  // 1 / (1 + dt/tau) per cell (the extrapolated start); null: 1
  double* invD;    // 1 / diag(M)
  double* R;       // right-hand side
  double* colsum;  // 1^T M per column (conservation check)
  double* y64[2];  // scaled solution y = D f (ping-pong)
};

template <typename T>
struct Kry {
  T *r, *rh, *t, *x;
  T *p[2], *v[2];
};

// ------------------------------------------------------------------------------ arithmetic
struct F64A {
  using V = double;
  static constexpr int kAsmBlocks = 4;  // k_assemble: resident blocks (64 registers)
  template <typename Ix>
  __device__ static V ld(const double* p, Ix i) { return p[i]; }
  template <typename Ix>
  __device__ static void st(double* p, Ix i, V v) { p[i] = v; }
  __device__ static Q4<V> ld4(const double* p) { return sg::ld4(p); }
  __device__ static void st4(double* p, const Q4<V>& q) { sg::st4(p, q); }
  __device__ static V add(V a, V b) { return a + b; }
  __device__ static V sub(V a, V b) { return a - b; }
  __device__ static V mul(V a, V b) { return a * b; }
  __device__ static V fma(V a, V b, V c) { return a * b + c; }
  // a*x + b*y and a*x - b*y (the same expression trees as fma(a, x, mul(b, y)) and
  // sub(mul(a, x), mul(b, y)))
  __device__ static V dot2(V a, V x, V b, V y) { return a * x + b * y; }
  __device__ static V fma0(V a, V b) { return a * b; }  // fma(a, b, 0)
  __device__ static V dot2s(V a, V x, V b, V y) { return a * x - b * y; }
  // sums whose terms all have the same sign (cheaper in double-word form)
  __device__ static V addp(V a, V b) { return a + b; }
  __device__ static V fmap(V a, V b, V c) { return a * b + c; }
  __device__ static V addf(V a, float b) { return a + (double)b; }
  __device__ static V rcp(V a) { return 1.0 / a; }
  __device__ static V div(V a, V b) { return a / b; }
  __device__ static V abs(V a) { return fabs(a); }
  __device__ static V neg(V a) { return -a; }
  // g, the polynomial extrapolation in time through f and n earlier states h1..h4 (n = 1..4) of
  // the loss-compensated sequence c_k = h_k r^k (r = 1/(1 + dt/tau), one step of pure loss), times
  // r: g = r (c0 + d1), r (c0 + 2 d1 - d2), r (c0 + 3 (d1 - d2) + d3),
  // r (c0 + 4 (d1 + d3) - 6 d2 - d4) with d_m = c_(m-1) - c_m, c0 = f. Exact for pure loss;
  // r = 1 gives the plain polynomial. The next solve starts from y0 = D g.
  __device__ static V extrap(V f, V h1, V h2, V h3, V h4, int n, V r) {
    const double c1 = h1 * r;
    const double d1 = f - c1;
    double c = d1;
    if (n >= 2) {
      const double r2 = r * r, c2 = h2 * r2;
      const double d2 = c1 - c2;
      if (n == 2) {
        c = 2.0 * d1 - d2;
      } else {
        const double r3 = r2 * r, c3 = h3 * r3;
        const double d3 = c2 - c3;
        c = n == 3 ? 3.0 * (d1 - d2) + d3 : 4.0 * (d1 + d3) - 6.0 * d2 - (c3 - h4 * (r3 * r));
      }
    }
    return r * (f + c);
  }
  __device__ static V rsub1(V a) { return 1.0 - a; }
  __device__ static V max0(V a) { return fmax(a, 0.0); }
  __device__ static V k(double c) { return c; }
  __device__ static bool lt0(V a) { return a < 0.0; }
  __device__ static bool gt0(V a) { return a > 0.0; }
  __device__ static float f32(V a) { return (float)a; }
  __device__ static float sq32(V a) { return (float)(a * a); }
  __device__ static double to_d(V a) { return a; }
  __device__ static V from_d(double a) { return a; }
  // the conversions of the layout transforms (none here)
  __device__ static double to_d_io(V a) { return a; }
  __device__ static V from_d_io(double a) { return a; }
  __device__ static void split(V a, float& hi, float& lo) {
    hi = __double2float_rn(a);
    lo = __double2float_rn(a - (double)hi);
  }
  __device__ static V hilo(float hi, float lo) { return (double)hi + (double)lo; }
  // r * s for a power-of-two s, in the Krylov precision T
  template <typename T>
  __device__ static T scaled(V a, float s) { return (T)(a * (double)s); }
  // y + x*s for the FP32/FP64 Krylov correction x in scaled units
  template <typename T>
  __device__ static V add_scaled(V y, T x, float s) { return y + (double)x * (double)s; }
  using Acc = double;  // per-thread accumulator of scaled squares
  __device__ static Acc sq_scaled(V a, float s) { const double t = a * (double)s; return t * t; }
  __device__ static double warp_total(Acc a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    return a;
  }
  __device__ static double warp_total_v(V a) { return warp_total(a); }
};

struct DWA {
  using V = dw;
  // k_assemble: 6 resident blocks (40 registers, no spill); measured on the 4096-instance batch
  // with 64 launched blocks per SM: 4 blocks 5.72 ms, 5 blocks (48 registers) 5.27 ms, 6 blocks
  // 5.16 ms per launch (with 96 launched per SM: 5.09 ms)
  static constexpr int kAsmBlocks = 6;
  template <typename Ix>
  __device__ static V ld(const double* p, Ix i) {
    const float2 q = reinterpret_cast<const float2*>(p)[i];
    return dw{q.x, q.y};
  }
  template <typename Ix>
  __device__ static void st(double* p, Ix i, V v) { reinterpret_cast<float2*>(p)[i] = make_float2(v.hi, v.lo); }
  __device__ static Q4<V> ld4(const double* p) {
    const float4 a = reinterpret_cast<const float4*>(p)[0];
    const float4 b = reinterpret_cast<const float4*>(p)[1];
    return Q4<V>{{dw{a.x, a.y}, dw{a.z, a.w}, dw{b.x, b.y}, dw{b.z, b.w}}};
  }
  __device__ static void st4(double* p, const Q4<V>& q) {
    reinterpret_cast<float4*>(p)[0] = make_float4(q.a[0].hi, q.a[0].lo, q.a[1].hi, q.a[1].lo);
    reinterpret_cast<float4*>(p)[1] = make_float4(q.a[2].hi, q.a[2].lo, q.a[3].hi, q.a[3].lo);
  }
  // Sums and multiply-adds are accurate to a few u^2 of their operands' magnitudes (SloppyDWPlusDW,
  // dw_fma), which is the accuracy every use needs: matrix entries against their forward-error
  // scale, residuals against |R|, increments against |f|.
  __device__ static V add(V a, V b) { return dw_add_same(a, b); }
  __device__ static V sub(V a, V b) { return dw_add_same(a, dw_neg(b)); }
  __device__ static V mul(V a, V b) { return dw_mul(a, b); }
  __device__ static V fma(V a, V b, V c) { return dw_fma(a, b, c); }
  __device__ static V dot2(V a, V x, V b, V y) { return dw_dot2(a, x, b, y); }
  __device__ static V fma0(V a, V b) { return dw_fma0(a, b); }  // fma(a, b, 0)
  __device__ static V dot2s(V a, V x, V b, V y) { return dw_dot2(a, x, dw_neg(b), y); }
  __device__ static V addp(V a, V b) { return dw_add_same(a, b); }
  __device__ static V fmap(V a, V b, V c) { return dw_fma(a, b, c); }
  __device__ static V addf(V a, float b) { return dw_add_f(a, b); }
  __device__ static V rcp(V a) { return dw_rcp(a); }
  __device__ static V div(V a, V b) { return dw_div(a, b); }
  __device__ static V abs(V a) { return dw_abs(a); }
  __device__ static V neg(V a) { return dw_neg(a); }
  // as F64A::extrap, in double-word: with loss rates up to 10 per day an increment is ~10 % of f,
  // so FP32 increments would leave ~1e-8 of f in the start, above what the extrapolation achieves; the
  // starting point only steers the iteration, the converged answer does not depend on it
  __device__ static V extrap(V f, V h1, V h2, V h3, V h4, int n, V r) {
    const dw c1 = dw_mul(h1, r);
    const dw d1 = sub(f, c1);
    dw c = d1;
    if (n >= 2) {
      const dw r2 = dw_mul(r, r), c2 = dw_mul(h2, r2);
      const dw d2 = sub(c1, c2);
      if (n == 2) {
        c = sub(dw{2.0f * d1.hi, 2.0f * d1.lo}, d2);
      } else {
        const dw r3 = dw_mul(r2, r), c3 = dw_mul(h3, r3);
        const dw d3 = sub(c2, c3);
        c = n == 3 ? add(dw_mul_f(sub(d1, d2), 3.0f), d3)
                   : sub(sub(dw_mul_f(add(d1, d3), 4.0f), dw_mul_f(d2, 6.0f)), sub(c3, dw_mul(h4, dw_mul(r3, r))));
      }
    }
    return dw_mul(r, add(f, c));
  }
  __device__ static V rsub1(V a) { return dw_add_f(dw_neg(a), 1.0f); }  // 1 - a (DWPlusFP)
  __device__ static V max0(V a) { return dw_max0(a); }
  __device__ static V k(double c) { return dw_from_double(c); }
  __device__ static bool lt0(V a) { return a.hi < 0.0f; }
  __device__ static bool gt0(V a) { return a.hi > 0.0f; }
  __device__ static float f32(V a) { return a.hi; }
  __device__ static float sq32(V a) { return a.hi * a.hi; }
  __device__ static double to_d(V a) { return dw_to_double(a); }
  __device__ static V from_d(double a) { return dw_from_double(a); }
  // the same bits with integer rounding (the layout transforms convert every cell per call)
  __device__ static double to_d_io(V a) { return dw_to_double_int(a); }
  __device__ static V from_d_io(double a) { return dw_from_double_int(a); }
  __device__ static void split(V a, float& hi, float& lo) {
    hi = a.hi;
    lo = a.lo;
  }
  __device__ static V hilo(float hi, float lo) { return dw{hi, lo}; }
  template <typename T>
  __device__ static T scaled(V a, float s) { return (T)(a.hi * s); }
  template <typename T>
  __device__ static V add_scaled(V y, T x, float s) { return dw_add_f(y, (float)x * s); }
  using Acc = float;
  __device__ static Acc sq_scaled(V a, float s) { const float t = a.hi * s; return t * t; }
  __device__ static double warp_total(Acc a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    return (double)a;
  }
  __device__ static double warp_total_v(V a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const dw b{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
      a = dw_add(a, b);
    }
    return dw_to_double(a);
  }
};

// Power-of-two scale of an instance's refinement system: 2^-e with max|R| = m * 2^e, m in
// [0.5, 1). Residuals are handed to the Krylov solver as r * scale, so its vectors and dot
// products stay O(1) or below whatever the magnitude of f (no FP32 underflow).
__device__ __forceinline__ float rhs_scale(unsigned int rmax_bits) {
  const float m = __uint_as_float(rmax_bits);
  if (!(m > 0.0f) || !isfinite(m)) return 1.0f;
  int e;
  frexpf(m, &e);
  return ldexpf(1.0f, -e);
}

// ------------------------------------------------------------------------------ setup
// Face factors of cell (i,j) from the reference's general formula (Solver.cc:68-97) evaluated on
// the XNEG and YNEG edges (Mesh.cc:80-151); the XPOS/YPOS edges of a rectangular cell give the
// same pair. Uses non-contracting intrinsics so the values match the CPU evaluation.
__device__ __forceinline__ void face_pair(double Kx, double Ky, double Ax, double Ay, double Bx,
                                          double By, double n0, double n1, const double L[4],
                                          double* aa, double* ab) {
  const double ex = __dadd_rn(Bx, -Ax), ey = __dadd_rn(By, -Ay);
  const double length = __dsqrt_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)));
  const double vkb0 = __dadd_rn(Bx, -Kx), vkb1 = __dadd_rn(By, -Ky);
  const double vka0 = __dadd_rn(Ax, -Kx), vka1 = __dadd_rn(Ay, -Ky);
  const double rvkb0 = vkb1, rvkb1 = -vkb0, rvka0 = vka1, rvka1 = -vka0;
  const double t0 = __dadd_rn(__dmul_rn(n0, L[0]), __dmul_rn(n1, L[2]));
  const double t1 = __dadd_rn(__dmul_rn(n0, L[1]), __dmul_rn(n1, L[3]));
  *aa = __ddiv_rn(__dmul_rn(length, __dadd_rn(__dmul_rn(t0, rvkb0), __dmul_rn(t1, rvkb1))),
                  __dadd_rn(__dmul_rn(vka0, rvkb0), __dmul_rn(vka1, rvkb1)));
  *ab = __ddiv_rn(__dmul_rn(length, __dadd_rn(__dmul_rn(t0, rvka0), __dmul_rn(t1, rvka1))),
                  __dadd_rn(__dmul_rn(vkb0, rvka0), __dmul_rn(vkb1, rvka1)));
}

// Face factors of cell K from G and D (Solver::update_Lambda, Solver.cc:57-65, then the general
// a_sigma formula on the XNEG and YNEG edges), stored in the policy's wide format.
template <typename A>
__device__ __forceinline__ void setup_faces(const Geo& geo, long long K, double xl, double xr, double yb,
                                            double yt, double g, double dxx, double dxy, double dyy) {
  const double Kx = __dmul_rn(0.5, __dadd_rn(xl, xr)), Ky = __dmul_rn(0.5, __dadd_rn(yb, yt));
  const double L[4] = {__dmul_rn(dxx, g), __dmul_rn(dxy, g), __dmul_rn(dxy, g), __dmul_rn(dyy, g)};
  double aa, ab;
  face_pair(Kx, Ky, xl, yt, xl, yb, -1.0, 0.0, L, &aa, &ab);  // XNEG: A=(i,j+1) B=(i,j)
  A::st(geo.aAx, K, A::from_d(aa));
  A::st(geo.aBx, K, A::from_d(ab));
  A::st(geo.Sx, K, A::from_d(__dadd_rn(aa, ab)));
  face_pair(Kx, Ky, xl, yb, xr, yb, 0.0, -1.0, L, &aa, &ab);  // YNEG: A=(i,j) B=(i+1,j)
  A::st(geo.aAy, K, A::from_d(aa));
  A::st(geo.aBy, K, A::from_d(ab));
  A::st(geo.Sy, K, A::from_d(__dadd_rn(aa, ab)));
}

// Every time-independent per-cell value of cell K from its edges, dt, G, D and 1/tau: the face
// factors (setup_faces), G (when kept), UKK = G * (dx*dy/dt), the diagonal term UKK*(1 + dt/tau)
// (Solver.cc:190-199, Mesh.h:61-63) and the one-step loss factor 1/(1 + dt/tau) (when kept). The
// one definition k_setup and the allocation-free entry point's set-up both call.
template <typename A>
__device__ __forceinline__ void setup_cell(const Geo& geo, long long K, double xl, double xr, double yb,
                                           double yt, double dt, double g, double dxx, double dxy, double dyy,
                                           double itau) {
  const double dx = __dadd_rn(xr, -xl), dy = __dadd_rn(yt, -yb);
  setup_faces<A>(geo, K, xl, xr, yb, yt, g, dxx, dxy, dyy);
  if (geo.G) geo.G[K] = g;
  const double ukk = __dmul_rn(g, __ddiv_rn(__dmul_rn(dx, dy), dt));
  A::st(geo.ukk, K, A::from_d(ukk));
  const double lossd = __dadd_rn(1.0, __dmul_rn(dt, itau));
  A::st(geo.sdiag, K, A::from_d(__dmul_rn(ukk, lossd)));
  if (geo.decay) A::st(geo.decay, K, A::from_d(__ddiv_rn(1.0, lossd)));
}

// One instance: stage holds alpha-major G, Dxx, Dxy, Dyy, inv_tau, f0 (each nx*ny). mask bits
// 0-4 select the coefficient sections (all five together), bit 5 the initial state. Values are
// computed in FP64 and stored in the policy's wide format.
template <typename A>
__global__ void k_setup(Common cm, Geo geo, double* f, const double* stage, const double* xe,
                        const double* ye, int b, int mask) {
  const InstDev I = cm.inst[b];
  const long long ncell = (long long)I.nx * I.ny;
  const double* G = stage;
  const double* Dxx = stage + ncell;
  const double* Dxy = stage + 2 * ncell;
  const double* Dyy = stage + 3 * ncell;
  const double* itau = stage + 4 * ncell;
  const double* f0 = stage + 5 * ncell;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
       c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c / I.ny), j = (int)(c % I.ny);
    const long long K = I.base + (long long)j * I.pitch + i;
    if (mask & 31)
      setup_cell<A>(geo, K, xe[I.xe + i], xe[I.xe + i + 1], ye[I.ye + j], ye[I.ye + j + 1], I.dt, G[c], Dxx[c],
                    Dxy[c], Dyy[c], itau[c]);
    if (mask & 32) A::st(f, K, A::from_d(f0[c]));
  }
}

// A diffusion-coefficient table on the device and the host-side values it is read with (see
// k_dtable). Row factors are per E row of each instance, at the instance's y-edge offset.
struct DTab {
  int na, ne;
  double xmin, xmax;      // alpha0 of the first and last node (radians)
  double lymin, lymax;    // log E of the first and last node
  double denorm;          // gME^2 gC^2
  const double *Daa, *Dap, *Dpp;        // (na, ne) row-major
  const double *rp, *rdl, *rdl2;        // per row: p, dlogE/dp, (dlogE/dp)^2
};

// calWeight (utils.h:44-58): weight of the lower node; past the last node, the last node with
// weight 1 (i = n-1, w = 0). Below the first node the reference converts a negative floor() to
// size_t (undefined in C++); its own i < 0 branch (first node, weight 1) is what is done here.
__device__ __forceinline__ void cal_weight(long long* i, double* w, long long n, double pos) {
  if (pos < 0.0) {
    *i = 0;
    *w = 1.0;
  } else if (*i < n) {
    *w = __dadd_rn(1.0, -__dadd_rn(pos, -(double)*i));
  } else {
    *i = n - 1;
    *w = 0.0;
  }
}

// D fields of Albert_Young(_LC)::constructD (Albert_Young.cc:112-134) at the cell centres, then
// the face factors of those cells. locate (Albert_Young.cc:94-110) places a centre in the table
// from its end points (uniform in alpha0 and log E); interp2D (utils.h:24-41) is bilinear. The
// transcendental row factors p = e2p(exp(log E)), dlogE/dp and its square (utils.h:12-20), the
// logs of the table's energy bounds and the unit factor come from the host's libm, so every
// operation here is a separately rounded IEEE add, multiply or divide in the reference's order.
// Tiles [t0, t1) of the tile list.
template <typename A>
__global__ void k_dtable(Common cm, Geo geo, DTab t, const double* xe, const double* ye, int t0, int t1) {
  const double s2d = 86400.0;  // 3600 * 24
  for (int tl = t0 + blockIdx.x; tl < t1; tl += gridDim.x) {
    const int b = cm.tile_inst[tl];
    const InstDev I = cm.inst[b];
    if (!I.enabled) continue;
    const int lt = tl - I.tile0, i0t = (lt % I.ntx) * kTX, j0t = (lt / I.ntx) * kTY;
    for (int q = threadIdx.x; q < kTX * kTY; q += blockDim.x) {
      const int i = i0t + (q % kTX), j = j0t + (q / kTX);
      if (i >= I.nx || j >= I.ny) continue;
      const long long K = I.base + (long long)j * I.pitch + i;
      const double xl = xe[I.xe + i], xr = xe[I.xe + i + 1];
      const double yb = ye[I.ye + j], yt = ye[I.ye + j + 1];
      const double alpha0 = __dmul_rn(0.5, __dadd_rn(xl, xr)), logE = __dmul_rn(0.5, __dadd_rn(yb, yt));
      const double px = __dmul_rn(__ddiv_rn(__dadd_rn(alpha0, -t.xmin), __dadd_rn(t.xmax, -t.xmin)), (double)(t.na - 1));
      const double py = __dmul_rn(__ddiv_rn(__dadd_rn(logE, -t.lymin), __dadd_rn(t.lymax, -t.lymin)), (double)(t.ne - 1));
      long long ia = px >= 0.0 ? (long long)floor(px) : 0, je = py >= 0.0 ? (long long)floor(py) : 0;
      double wi, wj;
      cal_weight(&ia, &wi, t.na - 1, px);
      cal_weight(&je, &wj, t.ne - 1, py);
      const double ui = __dadd_rn(1.0, -wi), uj = __dadd_rn(1.0, -wj);
      const long long r00 = ia * t.ne + je, r10 = r00 + t.ne;
      const double* raw[3] = {t.Daa, t.Dap, t.Dpp};
      double v[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double* r = raw[k];
        const double s1 = __dmul_rn(__dmul_rn(r[r00], wi), wj);
        const double s2 = __dmul_rn(__dmul_rn(r[r10], ui), wj);
        const double s3 = __dmul_rn(__dmul_rn(r[r10 + 1], ui), uj);
        const double s4 = __dmul_rn(__dmul_rn(r[r00 + 1], wi), uj);
        v[k] = __dadd_rn(__dadd_rn(__dadd_rn(s1, s2), s3), s4);
      }
      const double p = t.rp[I.ye + j], dl = t.rdl[I.ye + j], dl2 = t.rdl2[I.ye + j];
      const double dxx = __ddiv_rn(__dmul_rn(__dmul_rn(v[0], t.denorm), s2d), __dmul_rn(p, p));
      const double dxy = __ddiv_rn(__dmul_rn(__dmul_rn(__dmul_rn(v[1], t.denorm), s2d), dl), p);
      const double dyy = __dmul_rn(__dmul_rn(__dmul_rn(v[2], t.denorm), s2d), dl2);
      setup_faces<A>(geo, K, xl, xr, yb, yt, geo.G[K], dxx, dxy, dyy);
    }
  }
}

// alpha-major FP64 (packed at hoff) -> padded system order in the wide format, for tiles
// [t0, t1) of the tile list (t1 < 0: all), one 32x16 tile at a time: read along j (contiguous on the host side), transposed through shared memory,
// written along i (contiguous on the device side).
// When `restart` is set, a cell given back exactly the double it would be read out as keeps its
// stored value (in the double-word format that value can carry low bits a double does not), and
// an instance with any other cell loses its history of earlier states (the extrapolated start
// restarts from the new state). An instance given back its own state is left exactly as it was.
template <typename A>
__global__ void __launch_bounds__(kFieldThreads) k_field_in(Common cm, double* dst, const double* src, int restart,
                                                             int t0, int t1) {
  using V = typename A::V;
  count_launch(cm.ctl);
  constexpr int kItems = kTX * kTY / kFieldThreads;
  static_assert(kItems * kFieldThreads == kTX * kTY, "a tile splits evenly over the block");
  __shared__ double tile[kTY][kTX + 1];
  if (t1 < 0) t1 = n_tiles(cm);
  for (int t = t0 + blockIdx.x; t < t1; t += gridDim.x) {
    const int b = cm.tile_inst[t];
    const InstDev I = cm.inst[b];
    if (!I.enabled) continue;
    const int lt = t - I.tile0, i0 = (lt % I.ntx) * kTX, j0 = (lt / I.ntx) * kTY;
    // the stored values of this thread's cells of the second pass, loaded ahead of the barrier so
    // that their latency overlaps the host-order loads
    V old[kItems] = {};
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      const int q = threadIdx.x + k * kFieldThreads;
      const int i = i0 + (q % kTX), j = j0 + (q / kTX);  // i fastest
      if (restart && i < I.nx && j < I.ny) old[k] = A::ld(dst, I.base + (long long)j * I.pitch + i);
    }
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      const int q = threadIdx.x + k * kFieldThreads;
      const int i = i0 + (q / kTY), j = j0 + (q % kTY);  // j fastest
      if (i < I.nx && j < I.ny) tile[j - j0][i - i0] = src[I.hoff + (long long)i * I.ny + j];
    }
    __syncthreads();
    int changed = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      const int q = threadIdx.x + k * kFieldThreads;
      const int i = i0 + (q % kTX), j = j0 + (q / kTX);  // i fastest
      if (i < I.nx && j < I.ny) {
        const double v = tile[j - j0][i - i0];
        if (restart && __double_as_longlong(A::to_d_io(old[k])) == __double_as_longlong(v)) continue;
        changed = 1;
        A::st(dst, I.base + (long long)j * I.pitch + i, A::from_d_io(v));
      }
    }
    if (__syncthreads_or(restart && changed) && threadIdx.x == 0) cm.st[b].nhist = 0;
  }
}

// padded system order in the wide format -> alpha-major FP64, transposed like k_field_in (tiles
// [t0, t1) of the tile list; t1 < 0: all)
template <typename A>
__global__ void k_field_out(Common cm, double* dst, const double* src, int t0, int t1) {
  count_launch(cm.ctl);
  __shared__ double tile[kTY][kTX + 1];
  if (t1 < 0) t1 = n_tiles(cm);
  for (int t = t0 + blockIdx.x; t < t1; t += gridDim.x) {
    const int b = cm.tile_inst[t];
    const InstDev I = cm.inst[b];
    if (!I.enabled) continue;
    const int lt = t - I.tile0, i0 = (lt % I.ntx) * kTX, j0 = (lt / I.ntx) * kTY;
    for (int q = threadIdx.x; q < kTX * kTY; q += blockDim.x) {
      const int i = i0 + (q % kTX), j = j0 + (q / kTX);  // i fastest
      if (i < I.nx && j < I.ny) tile[j - j0][i - i0] = A::to_d_io(A::ld(src, I.base + (long long)j * I.pitch + i));
    }
    __syncthreads();
    for (int q = threadIdx.x; q < kTX * kTY; q += blockDim.x) {
      const int i = i0 + (q / kTY), j = j0 + (q % kTY);  // j fastest
      if (i < I.nx && j < I.ny) dst[I.hoff + (long long)i * I.ny + j] = tile[j - j0][i - i0];
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------ step control
__global__ void k_begin(Common cm) {
  count_launch(cm.ctl);
  for (int b = blockIdx.x * blockDim.x + threadIdx.x, ni_ = n_inst(cm); b < ni_; b += gridDim.x * blockDim.x) {
    InstState& s = cm.st[b];
    const bool on = cm.inst[b].enabled != 0;
    s.outer_active = on ? 1 : 0;
    s.inner_active = 0;
    s.restart = 0;
    s.fresh = 0;
    s.has_x = 0;
    s.iters = 0;
    s.iters_total = 0;
    s.refines = 0;
    s.clamped = 0;
    s.rmax_bits = 0u;
    if (on) atomicAdd(&cm.ctl->n_outer, 1);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cm.ctl->outer_loops = 0u;
    cm.ctl->inner_loops = 0u;
    cm.ctl->kdone[0] = 0u;
    cm.ctl->kdone[1] = 0u;
  }
}

// ------------------------------------------------------------------------------ assembly
template <typename C, typename A>
struct AsmOut;
template <typename A>
struct AsmOut<double, A> {
  template <typename Ix>
  __device__ static void put(const Coef<double>& c, int which, Ix idx, typename A::V v) {
    double* a = which == 0 ? c.cw : which == 1 ? c.ce : which == 2 ? c.cs : c.cn;
    a[idx] = A::to_d(v);
  }
};
template <typename A>
struct AsmOut<float, A> {
  template <typename Ix>
  __device__ static void put(const Coef<float>& c, int which, Ix idx, typename A::V v) {
    float hi, lo;
    A::split(v, hi, lo);
    float* a = which == 0 ? c.cw : which == 1 ? c.ce : which == 2 ? c.cs : c.cn;
    float* l = which == 0 ? c.lw : which == 1 ? c.le : which == 2 ? c.ls : c.ln;
    a[idx] = hi;
    l[idx] = lo;
  }
};

// Inner face (Solver.cc:99-141, calculate_mu Solver.h:63-67). K and L one-sided data:
// a_sigma = aA*fA + aB*fB, S = aA + aB, inv = 1/(f + eps).
template <typename A>
__device__ __forceinline__ void inner_face(typename A::V aK, typename A::V SK, typename A::V invK,
                                           typename A::V aL, typename A::V SL, typename A::V invL,
                                           typename A::V* AK, typename A::V* AL) {
  using V = typename A::V;
  const V absK = A::abs(aK), absL = A::abs(aL);
  const V denom = A::addp(A::addp(absK, absL), A::k(2 * kEps));
  const V muK = A::div(A::addp(absL, A::k(kEps)), denom);
  const V muL = A::rsub1(muK);
  const V B = A::dot2s(muL, aL, muK, aK);
  // B+ = (|B| + B)/2 goes to K's coefficient, B- = (|B| - B)/2 to L's; at most one is nonzero,
  // so only that one is multiplied by its 1/(f + eps) and added (all terms >= 0)
  const V mK = A::mul(muK, SK), mL = A::mul(muL, SL);
  const bool pos = A::gt0(B);
  const V T = A::mul(pos ? B : A::max0(A::neg(B)), pos ? invK : invL);
  const V X = A::addp(pos ? mK : mL, T);
  *AK = pos ? X : mK;
  *AL = pos ? mL : X;
}

// Dirichlet face (Solver.cc:143-164): B = -a_sigma; A = S + B+/(f+eps); R += B-.
template <typename A>
__device__ __forceinline__ void dirichlet_face(typename A::V aK, typename A::V SK, typename A::V invK,
                                               typename A::V* Aout, typename A::V* Bm) {
  *Aout = A::fmap(A::max0(A::neg(aK)), invK, SK);
  *Bm = A::max0(aK);
}

// One tile of kTX x kTY cells per iteration; vertices and faces are computed once per tile
// (plus a one-cell halo), in shared memory.
// Tiles [t0, t1) of the tile list (t1 < 0: all of them).
template <typename C, typename A>
__global__ void __launch_bounds__(kAsmThreads, A::kAsmBlocks) k_assemble(Common cm, Geo geo, Fields fl, Coef<C> co,
                                                                       int t0, int t1) {
  using V = typename A::V;
  count_launch(cm.ctl);
  constexpr int HX = kTX + 2, HY = kTY + 2, VX = kTX + 1, VY = kTY + 1;
  __shared__ V fS[HY][HX];
  __shared__ V iS[HY][HX];
  __shared__ V vS[VY][VX];
  // x-faces: outflow to the left / right cell; y-faces: to the cell below / above. On a Dirichlet
  // side the slot of the missing outside cell holds the face's RHS part instead.
  __shared__ V xLR[2][kTY][VX];
  V(*const xL)[VX] = xLR[0];
  V(*const xR)[VX] = xLR[1];
  __shared__ V yB[VY][kTX], yT[VY][kTX];
  __shared__ V hS[VY][2];  // the tile's vertex rows: bilinear weights (wB, wT), Solver.cc:333-336
  // f interpolated along each halo row at each vertex column (steps 1-2 only: shares the face
  // arrays' storage, which step 3 fills after a barrier)
  static_assert(HY * VX <= 2 * kTY * VX, "row interpolations must fit in the x-face arrays");
  V(*const rS)[VX] = reinterpret_cast<V(*)[VX]>(&xLR[0][0][0]);
  // step 1's thread layout: kRowT threads own one vertex column each and walk its halo rows,
  // kRowS rows apart
  constexpr int kRowS = 7, kRowT = VX * kRowS;
  static_assert(kRowT < kAsmThreads && 3 * kRowS >= HY, "step 1 layout");
  const V zero = A::k(0.0);
  const int nt_ = t1 < 0 ? n_tiles(cm) : t1;
  for (int t = t0 + blockIdx.x; t < nt_; t += gridDim.x) {
    const int b = cm.tile_inst[t];
    const InstDev I = cm.inst[b];
    if (!I.enabled) continue;  // uniform in the block
    const int lt = t - I.tile0;
    const int i0 = (lt % I.ntx) * kTX, j0 = (lt / I.ntx) * kTY;
    const int nx = I.nx, ny = I.ny, P = I.pitch;
    // 32-bit cell indices: every batch holds fewer than 2^31 cells (checked at allocation), and an
    // int index makes each address one wide multiply-add
    const int base = (int)I.base;
    // the extrapolated start g the last polish left in the idle y buffer (none before the first
    // step or after the state was replaced: then y0 = D f)
    const bool has_g = cm.st[b].nhist > 0;
    const int yc = cm.st[b].ycur;
    const double* gp = sel2(fl.y64, yc ^ 1);
    // the per-cell data of step 4 is only needed after three barriers: start its trip to L2 now
#pragma unroll
    for (int q = threadIdx.x; q < kTX * kTY; q += kAsmThreads) {
      const int i = i0 + (q % kTX), j = j0 + (q / kTX);
      if (i < nx && j < ny) {
        const int K = base + j * P + i;
        asm volatile("prefetch.global.L2 [%0];" ::"l"(geo.sdiag + K));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(geo.ukk + K));
        if (has_g) asm volatile("prefetch.global.L2 [%0];" ::"l"(gp + K));
      }
    }
    // 1) per vertex column Iv (threads below kRowT) and halo row j: f and 1/(f+eps) of the cell left
    //    of the column, and r = wL f_left + wR f_right, f interpolated along the row at the column
    //    (Solver.cc:333-336; a boundary column takes its adjacent cell's f). The remaining threads
    //    take the right halo column and the vertex-row weights.
    if (threadIdx.x < kRowT) {
      const int vx = threadIdx.x % VX, Iv = i0 + vx;
      const bool xin = Iv > 0 && Iv < nx;
      const V wL = xin ? A::ld(cm.wx, 2 * (I.xe + Iv)) : zero;
      const V wR = xin ? A::ld(cm.wx, 2 * (I.xe + Iv) + 1) : zero;
      for (int hy = threadIdx.x / VX; hy < HY; hy += kRowS) {
        const int j = j0 + hy - 1;
        V fa = zero, ia = zero, r = zero;
        if (j >= 0 && j < ny && Iv <= nx) {
          const int K = base + j * P + Iv;  // the cell right of the column
          V fb = zero;
          if (Iv > 0) {
            fa = A::ld(fl.f, K - 1);
            ia = A::rcp(A::addp(fa, A::k(kEps)));
          }
          if (Iv < nx) fb = A::ld(fl.f, K);
          r = xin ? A::fmap(wL, fa, A::mul(wR, fb)) : (Iv == 0 ? fb : fa);
        }
        fS[hy][vx] = fa;
        iS[hy][vx] = ia;
        rS[hy][vx] = r;
      }
    } else {
      for (int q = threadIdx.x - kRowT; q < HY + VY; q += kAsmThreads - kRowT) {
        if (q < HY) {
          const int i = i0 + kTX, j = j0 + q - 1;
          V fv = zero, iv = zero;
          if (i < nx && j >= 0 && j < ny) {
            fv = A::ld(fl.f, base + j * P + i);
            iv = A::rcp(A::addp(fv, A::k(kEps)));
          }
          fS[q][HX - 1] = fv;
          iS[q][HX - 1] = iv;
        } else {
          const int vy = q - HY, Jv = j0 + vy;
          const bool in = Jv > 0 && Jv < ny;
          hS[vy][0] = in ? A::ld(cm.wy, 2 * (I.ye + Jv)) : zero;
          hS[vy][1] = in ? A::ld(cm.wy, 2 * (I.ye + Jv) + 1) : zero;
        }
      }
    }
    __syncthreads();
    // 2) vertex values (Solver.cc:299-422): corners copy, interior bilinear, boundary edges
    //    linear, then Dirichlet overrides with XMIN < XMAX < YMIN < YMAX precedence. The bilinear
    //    value wB (wL f00 + wR f10) + wT (wL f01 + wR f11) is formed from the two row
    //    interpolations of step 1 with the same operations in the same order.
    for (int q = threadIdx.x; q < VX * VY; q += blockDim.x) {
      const int vx = q % VX, vy = q / VX;
      const int Iv = i0 + vx, Jv = j0 + vy;
      if (Iv > nx || Jv > ny) continue;
      V val;
      if (Jv == ny && I.bc[YMAX] == DIRICHLET) val = A::ld(cm.dirv, I.dir[YMAX] + Iv);
      else if (Jv == 0 && I.bc[YMIN] == DIRICHLET) val = A::ld(cm.dirv, I.dir[YMIN] + Iv);
      else if (Iv == nx && I.bc[XMAX] == DIRICHLET) val = A::ld(cm.dirv, I.dir[XMAX] + Jv);
      else if (Iv == 0 && I.bc[XMIN] == DIRICHLET) val = A::ld(cm.dirv, I.dir[XMIN] + Jv);
      else {
        // cell rows below / above vertex row Jv, clamped to the domain at the edges
        const int cj0 = Jv > 0 ? Jv - 1 : 0, cj1 = Jv < ny ? Jv : ny - 1;
        const V r0 = rS[cj0 - j0 + 1][vx];
        if (Jv > 0 && Jv < ny) {  // interior and vertical boundary edges: linear in y
          const V r1 = rS[cj1 - j0 + 1][vx];
          val = A::fmap(hS[vy][0], r0, A::mul(hS[vy][1], r1));
        } else {
          val = r0;  // horizontal boundary edges (linear in x) and corners
        }
      }
      vS[vy][vx] = val;
    }
    __syncthreads();
    // 3a) x-faces (vertex column Iv between cells Iv-1 and Iv)
    for (int q = threadIdx.x; q < kTY * VX; q += blockDim.x) {
      const int vx = q % VX, ry = q / VX;
      const int Iv = i0 + vx, j = j0 + ry;
      V aL = zero, aR = zero, bm = zero;
      if (j < ny && Iv <= nx) {
        const V vLo = vS[ry][vx], vHi = vS[ry + 1][vx];  // vertices (Iv, j), (Iv, j+1)
        if (Iv > 0 && Iv < nx) {
          const int K = base + j * P + Iv, L = K - 1;
          // K's XNEG edge: A=(Iv, j+1), B=(Iv, j); L's XPOS edge: A=(Iv, j), B=(Iv, j+1)
          const V aK = A::dot2(A::ld(geo.aAx, K), vHi, A::ld(geo.aBx, K), vLo);
          const V aLs = A::dot2(A::ld(geo.aAx, L), vLo, A::ld(geo.aBx, L), vHi);
          inner_face<A>(aK, A::ld(geo.Sx, K), iS[ry + 1][vx + 1], aLs, A::ld(geo.Sx, L), iS[ry + 1][vx], &aR, &aL);
        } else if (Iv == 0 && I.bc[XMIN] == DIRICHLET) {
          const int K = base + j * P;
          dirichlet_face<A>(A::dot2(A::ld(geo.aAx, K), vHi, A::ld(geo.aBx, K), vLo), A::ld(geo.Sx, K),
                            iS[ry + 1][vx + 1], &aR, &bm);
        } else if (Iv == nx && I.bc[XMAX] == DIRICHLET) {
          const int K = base + j * P + nx - 1;  // XPOS edge: A=(nx, j), B=(nx, j+1)
          dirichlet_face<A>(A::dot2(A::ld(geo.aAx, K), vLo, A::ld(geo.aBx, K), vHi), A::ld(geo.Sx, K),
                            iS[ry + 1][vx], &aL, &bm);
        }
      }
      xL[ry][vx] = Iv == 0 ? bm : aL;
      xR[ry][vx] = Iv == nx ? bm : aR;
    }
    // 3b) y-faces (vertex row Jv between cells Jv-1 and Jv)
    for (int q = threadIdx.x; q < VY * kTX; q += blockDim.x) {
      const int cx = q % kTX, vy = q / kTX;
      const int i = i0 + cx, Jv = j0 + vy;
      V aB = zero, aT = zero, bm = zero;
      if (i < nx && Jv <= ny) {
        const V vLe = vS[vy][cx], vRi = vS[vy][cx + 1];  // vertices (i, Jv), (i+1, Jv)
        if (Jv > 0 && Jv < ny) {
          const int K = base + Jv * P + i, L = K - P;
          // K's YNEG edge: A=(i, Jv), B=(i+1, Jv); L's YPOS edge: A=(i+1, Jv), B=(i, Jv)
          const V aK = A::dot2(A::ld(geo.aAy, K), vLe, A::ld(geo.aBy, K), vRi);
          const V aLs = A::dot2(A::ld(geo.aAy, L), vRi, A::ld(geo.aBy, L), vLe);
          inner_face<A>(aK, A::ld(geo.Sy, K), iS[vy + 1][cx + 1], aLs, A::ld(geo.Sy, L), iS[vy][cx + 1], &aT, &aB);
        } else if (Jv == 0 && I.bc[YMIN] == DIRICHLET) {
          const int K = base + i;
          dirichlet_face<A>(A::dot2(A::ld(geo.aAy, K), vLe, A::ld(geo.aBy, K), vRi), A::ld(geo.Sy, K),
                            iS[vy + 1][cx + 1], &aT, &bm);
        } else if (Jv == ny && I.bc[YMAX] == DIRICHLET) {
          const int K = base + (ny - 1) * P + i;  // YPOS edge: A=(i+1,ny), B=(i,ny)
          dirichlet_face<A>(A::dot2(A::ld(geo.aAy, K), vRi, A::ld(geo.aBy, K), vLe), A::ld(geo.Sy, K),
                            iS[vy][cx + 1], &aB, &bm);
        }
      }
      yB[vy][cx] = Jv == 0 ? bm : aB;
      yT[vy][cx] = Jv == ny ? bm : aT;
    }
    __syncthreads();
    // 4) per cell: diagonal in the reference's triplet order, RHS, scaling, scatter
    float rmax = 0.0f;
#pragma unroll
    for (int q = threadIdx.x; q < kTX * kTY; q += kAsmThreads) {
      const int cx = q % kTX, cy = q / kTX;
      const int i = i0 + cx, j = j0 + cy;
      if (i >= nx || j >= ny) continue;
      const int K = base + j * P + i;
      const V Aw = xR[cy][cx], Ae = xL[cy][cx + 1], As = yT[cy][cx], An = yB[cy + 1][cx];
      const bool wIn = i > 0, eIn = i < nx - 1, sIn = j > 0, nIn = j < ny - 1;
      // every term below is >= 0; a sum that is still zero takes its first term as it is (0 + x
      // = x), which spares an interior cell three double-word additions
      V D = wIn ? Aw : zero, Rv = zero, dir = zero;
      bool has_dir = false;
      if (eIn) D = A::addp(D, Ae);
      if (sIn) D = A::addp(D, As);
      if (nIn) D = A::addp(D, An);
      if (!wIn && I.bc[XMIN] == DIRICHLET) { D = A::addp(D, Aw); dir = A::addp(dir, Aw); Rv = A::addp(Rv, xL[cy][cx]); has_dir = true; }
      if (!eIn && I.bc[XMAX] == DIRICHLET) { D = A::addp(D, Ae); dir = A::addp(dir, Ae); Rv = A::addp(Rv, xR[cy][cx + 1]); has_dir = true; }
      if (!sIn && I.bc[YMIN] == DIRICHLET) { D = A::addp(D, As); dir = A::addp(dir, As); Rv = A::addp(Rv, yB[cy][cx]); has_dir = true; }
      if (!nIn && I.bc[YMAX] == DIRICHLET) { D = A::addp(D, An); dir = A::addp(dir, An); Rv = A::addp(Rv, yT[cy + 1][cx]); has_dir = true; }
      const V sd = A::ld(geo.sdiag, K);
      D = A::addp(D, sd);
      const V fK = fS[cy + 1][cx + 1];
      const V ukk = A::ld(geo.ukk, K);
      Rv = has_dir ? A::fmap(ukk, fK, Rv) : A::fma0(ukk, fK);
      rmax = fmaxf(rmax, fabsf(A::f32(Rv)));
      const V inv = A::rcp(D);
      A::st(fl.invD, K, inv);
      A::st(fl.R, K, Rv);
      A::st(fl.colsum, K, has_dir ? A::addp(sd, dir) : sd);
      // start the solve from D g, g the loss-compensated polynomial extrapolation in time the
      // last polish formed (only the starting point of the iteration; the converged answer does
      // not depend on it)
      A::st(sel2(fl.y64, yc), K, A::mul(D, has_g ? A::ld(gp, K) : fK));
      if (wIn) AsmOut<C, A>::put(co, 1, K - 1, A::mul(Aw, inv));  // row K-1, east entry
      if (eIn) AsmOut<C, A>::put(co, 0, K + 1, A::mul(Ae, inv));  // row K+1, west entry
      if (sIn) AsmOut<C, A>::put(co, 3, K - P, A::mul(As, inv));  // row K-P, north entry
      if (nIn) AsmOut<C, A>::put(co, 2, K + P, A::mul(An, inv));  // row K+P, south entry
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    if ((threadIdx.x & 31) == 0 && rmax > 0.0f) atomicMax(&cm.st[b].rmax_bits, __float_as_uint(rmax));
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------ streaming helpers
// Resident blocks per SM the Krylov kernels are compiled for: in FP32, 6 (registers capped at
// 40; their shared memory allows 6, and the extra blocks in flight raised their bandwidth by
// 8-14 %); in FP64, 4 (a cap of 40 registers spills).
template <typename T>
constexpr int krylov_blocks() { return sizeof(T) == 4 ? 6 : 4; }

// Locates 4-cell group g (0 .. CH/(4*kThreads) - 1) of this thread in chunk c (CH cells) of
// instance I.
struct Slot {
  long long K;
  bool valid;
};
template <int CH>
__device__ __forceinline__ long long chunk_start(int c, const InstDev& I) {
  return I.base + (long long)(c - I.chunk0) * CH;
}
__device__ __forceinline__ long long inst_end(const InstDev& I) { return I.base + (long long)I.ny * I.pitch; }
template <int CH>
__device__ __forceinline__ Slot slot_of(int c, const InstDev& I, int g) {
  Slot s;
  s.K = chunk_start<CH>(c, I) + 4 * (threadIdx.x + g * kThreads);
  s.valid = s.K < inst_end(I);
  return s;
}

// Runs body(c) for every chunk c of this block (c = blockIdx.x + k*gridDim.x) whose instance
// passes want(instance). The instance checks run in parallel, one chunk per thread, and the
// passing chunks are compacted in shared memory: a launch in which most instances have finished
// costs one round of checks per block instead of two dependent loads per chunk. Chunks are
// independent, so the order in which a block takes them does not change any result.
// Chunks [c0, c1) of the list only (c1 < 0: to the end).
template <typename W, typename Body>
__device__ __forceinline__ void for_active_chunks(const Common& cm, W&& want, Body&& body, int c0 = 0, int c1 = -1) {
  __shared__ int s_list[kThreads];
  __shared__ int s_cnt;
  const int nc = (c1 < 0 ? n_chunks(cm) : c1) - c0;
  const int per = (int)blockIdx.x < nc ? (nc - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  for (int r0 = 0; r0 < per; r0 += kThreads) {
    if (threadIdx.x == 0) s_cnt = 0;
    __syncthreads();
    const int k = r0 + (int)threadIdx.x;
    if (k < per) {
      const int c = c0 + (int)blockIdx.x + k * (int)gridDim.x;
      if (want(cm.chunk_inst[c])) s_list[atomicAdd(&s_cnt, 1)] = c;
    }
    __syncthreads();
    const int m = s_cnt;
    for (int q = 0; q < m; ++q) body(s_list[q]);
    __syncthreads();
  }
}

// Fills smem[0 .. n) with a 4-aligned stretch [e0, e0 + n) of a vector computed cell-wise by
// f(k) -> Q4<T> (k a multiple of 4): the chunk plus one row above and below, so that the stencil
// of every cell in the chunk reads shared memory only.
template <typename T, typename F>
__device__ __forceinline__ void stage_rows(T* sm, long long e0, long long n, F&& f) {
#pragma unroll 2
  for (long long q = 4LL * threadIdx.x; q < n; q += 4LL * blockDim.x) {
    const Q4<T> v = f(e0 + q);
    *reinterpret_cast<Q4<T>*>(sm + q) = v;
  }
}

// A~ x over a 4-cell group from a staged vector (sm holds x at global index e0 + offset)
template <typename T>
__device__ __forceinline__ Q4<T> stencil_sm(const T* sm, long long o, int P, const Q4<T>& cw,
                                            const Q4<T>& ce, const Q4<T>& cs, const Q4<T>& cn) {
  const Q4<T> c = *reinterpret_cast<const Q4<T>*>(sm + o);
  const Q4<T> d = *reinterpret_cast<const Q4<T>*>(sm + o - P);
  const Q4<T> u = *reinterpret_cast<const Q4<T>*>(sm + o + P);
  const T w0 = sm[o - 1], e3 = sm[o + 4];
  Q4<T> r;
  const T wv[4] = {w0, c.a[0], c.a[1], c.a[2]};
  const T ev[4] = {c.a[1], c.a[2], c.a[3], e3};
#pragma unroll
  for (int k = 0; k < 4; ++k) r.a[k] = c.a[k] - (cw.a[k] * wv[k] + ce.a[k] * ev[k] + cs.a[k] * d.a[k] + cn.a[k] * u.a[k]);
  return r;
}

// ------------------------------------------------------------------------------ preconditioner
// Alpha-line block preconditioner. Every 4-cell group of the padded layout lies inside one row
// (rows start at multiples of 4), and B is the tridiagonal of the group's own west/east couplings
// -- unit diagonal, -cw below, -ce above -- with the couplings to the neighbouring groups dropped:
// block Jacobi with 4-cell alpha-line blocks, the direction in which the scaled systems are
// stiffest (Dxx/dalpha^2 against Dyy/dlogE^2). line4 returns B^-1 q by Thomas elimination
// without pivoting (B is a column-diagonally-dominant M-matrix: every column of the outflow
// fractions sums to < 1, so each pivot stays in (0, 1]). The factors are formed in FP32 with
// separately rounded intrinsics whatever the vector precision, so every kernel that applies
// B^-1 applies the same linear map; padding cells (q = cw = ce = 0) stay 0.
__device__ __forceinline__ float fmaT(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmaT(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mulT(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mulT(double a, double b) { return __dmul_rn(a, b); }

template <typename T, typename CT>
__device__ __forceinline__ Q4<T> line4(const Q4<T>& q, const Q4<CT>& cw, const Q4<CT>& ce) {
  const float w1 = (float)cw.a[1], w2 = (float)cw.a[2], w3 = (float)cw.a[3];
  const float c0 = (float)ce.a[0];
  const float i1 = __frcp_rn(__fmaf_rn(-w1, c0, 1.0f));
  const float c1 = __fmul_rn((float)ce.a[1], i1);
  const float i2 = __frcp_rn(__fmaf_rn(-w2, c1, 1.0f));
  const float c2 = __fmul_rn((float)ce.a[2], i2);
  const float i3 = __frcp_rn(__fmaf_rn(-w3, c2, 1.0f));
  // forward: d_j = (q_j + w_j d_(j-1)) / pivot_j; backward: z_j = d_j + c_j z_(j+1)
  const T d0 = q.a[0];
  const T d1 = mulT(fmaT((T)w1, d0, q.a[1]), (T)i1);
  const T d2 = mulT(fmaT((T)w2, d1, q.a[2]), (T)i2);
  const T d3 = mulT(fmaT((T)w3, d2, q.a[3]), (T)i3);
  Q4<T> z;
  z.a[3] = d3;
  z.a[2] = fmaT((T)c2, d3, d2);
  z.a[1] = fmaT((T)c1, z.a[2], d1);
  z.a[0] = fmaT((T)c0, z.a[1], d0);
  return z;
}

// Coefficients of a row in the wide arithmetic: from the FP64 arrays or the (hi, lo) split
template <typename C, typename A>
struct CoefW;
template <typename A>
struct CoefW<double, A> {
  __device__ static Q4<typename A::V> row(const Coef<double>& c, int which, long long K) {
    const double* a = which == 0 ? c.cw : which == 1 ? c.ce : which == 2 ? c.cs : c.cn;
    const Q4<double> q = ld4(a + K);
    Q4<typename A::V> o;
#pragma unroll
    for (int k = 0; k < 4; ++k) o.a[k] = A::from_d(q.a[k]);
    return o;
  }
};
template <typename A>
struct CoefW<float, A> {
  __device__ static Q4<typename A::V> row(const Coef<float>& c, int which, long long K) {
    const float* a = which == 0 ? c.cw : which == 1 ? c.ce : which == 2 ? c.cs : c.cn;
    const float* l = which == 0 ? c.lw : which == 1 ? c.le : which == 2 ? c.ls : c.ln;
    const Q4<float> h = ld4(a + K), lo = ld4(l + K);
    Q4<typename A::V> o;
#pragma unroll
    for (int k = 0; k < 4; ++k) o.a[k] = A::hilo(h.a[k], lo.a[k]);
    return o;
  }
};

// y = A~ x for a 4-cell group given the centre values, the west value of cell 0, the east value
// of cell 3 and the rows below/above.
template <typename T, typename CT>
__device__ __forceinline__ Q4<T> stencil(const Q4<T>& c, T w0, T e3, const Q4<T>& dn, const Q4<T>& up,
                                         const Q4<CT>& cw, const Q4<CT>& ce, const Q4<CT>& cs,
                                         const Q4<CT>& cn) {
  Q4<T> o;
  const T wv[4] = {w0, c.a[0], c.a[1], c.a[2]};
  const T ev[4] = {c.a[1], c.a[2], c.a[3], e3};
#pragma unroll
  for (int k = 0; k < 4; ++k)
    o.a[k] = c.a[k] - ((T)cw.a[k] * wv[k] + (T)ce.a[k] * ev[k] + (T)cs.a[k] * dn.a[k] + (T)cn.a[k] * up.a[k]);
  return o;
}

// The same stencil in the wide arithmetic: A~ y = y - sum_nbr c * y_nbr
template <typename A>
__device__ __forceinline__ Q4<typename A::V> stencilW(const Q4<typename A::V>& c, typename A::V w0,
                                                      typename A::V e3, const Q4<typename A::V>& dn,
                                                      const Q4<typename A::V>& up,
                                                      const Q4<typename A::V>& cw, const Q4<typename A::V>& ce,
                                                      const Q4<typename A::V>& cs, const Q4<typename A::V>& cn) {
  using V = typename A::V;
  Q4<V> o;
  const V wv[4] = {w0, c.a[0], c.a[1], c.a[2]};
  const V ev[4] = {c.a[1], c.a[2], c.a[3], e3};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const V s = A::fma(cn.a[k], up.a[k], A::fma(cs.a[k], dn.a[k], A::fma(ce.a[k], ev[k], A::mul(cw.a[k], wv[k]))));
    o.a[k] = A::sub(c.a[k], s);
  }
  return o;
}

// ------------------------------------------------------------------------------ outer residual
// r = R - A~ (y + x) in the wide arithmetic; writes y + x to the other y buffer and the Krylov's
// right-hand side B^-1 r (T precision, scaled). Partials: ||r||^2, ||R||^2, ||B^-1 r||^2.
template <typename T, typename C, typename A, int CH>
__device__ __forceinline__ void resid_body(Common cm, Fields fl, Coef<C> co, Kry<T> kr, double tol, double inner_tol,
                                           int max_refine) {
  using V = typename A::V;
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = reinterpret_cast<V*>(smraw);
  for_active_chunks(cm, [&](int b_) { return cm.st[b_].outer_active != 0; }, [&](int c) {
    const int b = cm.chunk_inst[c];
    InstState& st = cm.st[b];
    const InstDev I = cm.inst[b];
    const double* yin = sel2(fl.y64, st.ycur);
    double* yout = sel2(fl.y64, st.ycur ^ 1);
    const bool hx = st.has_x != 0;
    const float sc = rhs_scale(st.rmax_bits);  // r is handed over as r * sc
    const float isc = 1.0f / sc;                // exact: sc is a power of two
    const int P = I.pitch;
    const long long c0 = chunk_start<CH>(c, I);
    const long long c1 = min(c0 + (long long)CH, inst_end(I));
    const long long e0 = c0 - P;
    // y + x (the last Krylov correction, in scaled units) over the chunk and one row each side
    stage_rows<V>(sm, e0, (c1 - c0) + 2LL * P, [&](long long k) {
      Q4<V> y = A::ld4(yin + k);
      if (hx) {
        const Q4<T> x = ld4(kr.x + k);
#pragma unroll
        for (int m = 0; m < 4; ++m) y.a[m] = A::template add_scaled<T>(y.a[m], x.a[m], isc);
      }
      return y;
    });
    __syncthreads();
    typename A::Acc q0 = 0, q1 = 0;
    T q2 = (T)0;
#pragma unroll 1
    for (int g = 0; g < CH / (4 * kThreads); ++g) {
      const long long K = c0 + 4 * (threadIdx.x + g * kThreads);
      if (K < c1) {
        const long long o = K - e0;
        const Q4<V> cw = CoefW<C, A>::row(co, 0, K), ce = CoefW<C, A>::row(co, 1, K);
        const Q4<V> cs = CoefW<C, A>::row(co, 2, K), cn = CoefW<C, A>::row(co, 3, K);
        const Q4<V> R = A::ld4(fl.R + K);
        Q4<T> r;
        Q4<V> yc;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          const V yv = sm[o + m];
          const V s1 = A::fma(cn.a[m], sm[o + m + P], A::fma(cs.a[m], sm[o + m - P],
                              A::fma(ce.a[m], sm[o + m + 1], A::mul(cw.a[m], sm[o + m - 1]))));
          const V rv = A::sub(R.a[m], A::sub(yv, s1));
          yc.a[m] = yv;
          r.a[m] = A::template scaled<T>(rv, sc);
          q0 += A::sq_scaled(rv, sc);
          q1 += A::sq_scaled(R.a[m], sc);
        }
        if (cm.precond) {  // the Krylov matrix's couplings (the hi parts in the FP32 modes)
          r = line4<T, C>(r, ld4(co.cw + K), ld4(co.ce + K));
#pragma unroll
          for (int m = 0; m < 4; ++m) q2 += r.a[m] * r.a[m];
        }
        A::st4(yout + K, yc);
        st4(kr.r + K, r);
      }
    }
    double w3 = (double)q2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w3 += __shfl_xor_sync(0xffffffffu, w3, o);
    const double w[3] = {A::warp_total(q0), A::warp_total(q1), w3};
    double tot[3], mine[3];
    block_sum_lane0<3>(w, mine);
    if (chunk_finish<3>(st, PH_RESID, I.chunk0, I.nchunks, c, cm.part, mine, tot) && threadIdx.x == 0) {
      // tot holds ||r*sc||^2, ||R*sc||^2 and ||B^-1 r*sc||^2
      st.ycur ^= 1;
      st.has_x = 0;
      if (st.refines == 0) st.bb = tot[1];
      st.refines += 1;
      st.cum_refines += 1;
      st.rr64 = tot[0];
      st.rel = st.bb > 0 ? sqrt(tot[0] / st.bb) : 0.0;
      if (!(st.rel > tol)) {
        st.outer_active = 0;
        st.status = ST_OK;
        atomicSub(&cm.ctl->n_outer, 1);
      } else if (st.refines >= max_refine) {
        st.outer_active = 0;
        st.status = ST_NOT_CONVERGED;
        atomicSub(&cm.ctl->n_outer, 1);
      } else {
        st.inner_active = 1;
        st.fresh = 1;
        st.restart = 1;
        st.iters = 0;
        // the Krylov's residual is B^-1 r: its target is the relative reduction asked, or the
        // final tolerance carried into preconditioned units by this pass's norm ratio
        const double rrk = cm.precond ? tot[2] : tot[0];
        st.rr = rrk;
        const double a = inner_tol * inner_tol * rrk;
        const double bnd = 0.0625 * tol * tol * st.bb * (cm.precond && tot[0] > 0.0 ? rrk / tot[0] : 1.0);
        st.rr_target = a > bnd ? a : bnd;
        atomicAdd(&cm.ctl->n_inner, 1);
      }
    }
  });
}
template <typename T, typename C, typename A, int CH>
__global__ void __launch_bounds__(kThreads, 4) k_resid(Common cm, Fields fl, Coef<C> co, Kry<T> kr,
                                                        double tol, double inner_tol, int max_refine) {
  count_launch(cm.ctl);
  resid_body<T, C, A, CH>(cm, fl, co, kr, tol, inner_tol, max_refine);
  loop_epilogue(cm, 0);
}

// ------------------------------------------------------------------------------ BiCGSTAB
// Left-preconditioned BiCGSTAB on B^-1 A~ x = B^-1 r (B = I without the preconditioner; the
// residual r the kernels carry is the preconditioned one, and x is the correction itself).
// k1: p = r + beta (p_old - omega v_old)  (p = r on a restart, which also sets r^ = r);
//     v = B^-1 A~ p;  partial (r^, v). p is computed once per cell into shared memory (chunk plus
//     one row above and below) and the stencil reads it there.
template <typename T, int CH>
__device__ __forceinline__ void bicg1_body(Common cm, Coef<T> co, Kry<T> kr) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  for_active_chunks(cm, [&](int b_) { return cm.st[b_].inner_active != 0; }, [&](int c) {
    const int b = cm.chunk_inst[c];
    InstState& st = cm.st[b];
    const InstDev I = cm.inst[b];
    const int pc = st.pcur;
    const bool rs = st.restart != 0;
    const T beta = (T)st.beta, omega = (T)st.omega;
    const T* __restrict__ r = kr.r;
    const T* __restrict__ po = sel2(kr.p, pc);
    const T* __restrict__ vo = sel2(kr.v, pc);
    T* __restrict__ pn = sel2(kr.p, pc ^ 1);
    T* __restrict__ vn = sel2(kr.v, pc ^ 1);
    const int P = I.pitch;
    const long long c0 = chunk_start<CH>(c, I);
    const long long c1 = min(c0 + (long long)CH, inst_end(I));
    const long long e0 = c0 - P;
    stage_rows<T>(sm, e0, (c1 - c0) + 2LL * P, [&](long long k) {
      Q4<T> x = ld4(r + k);
      if (!rs) {
        const Q4<T> a = ld4(po + k), v = ld4(vo + k);
#pragma unroll
        for (int m = 0; m < 4; ++m) x.a[m] = x.a[m] + beta * (a.a[m] - omega * v.a[m]);
      }
      return x;
    });
    __syncthreads();
    T q[1] = {(T)0};
#pragma unroll 2
    for (int g = 0; g < CH / (4 * kThreads); ++g) {
      const long long K = c0 + 4 * (threadIdx.x + g * kThreads);
      if (K < c1) {
        const long long o = K - e0;
        const Q4<T> pcv = *reinterpret_cast<const Q4<T>*>(sm + o);
        const Q4<T> cwq = ld4(co.cw + K), ceq = ld4(co.ce + K);
        Q4<T> v = stencil_sm<T>(sm, o, P, cwq, ceq, ld4(co.cs + K), ld4(co.cn + K));
        if (cm.precond) v = line4<T, T>(v, cwq, ceq);  // v = B^-1 A~ p
        st4(pn + K, pcv);
        st4(vn + K, v);
        Q4<T> rh;
        if (rs) {
          rh = ld4(r + K);
          st4(kr.rh + K, rh);
        } else {
          rh = ld4(kr.rh + K);
        }
#pragma unroll
        for (int m = 0; m < 4; ++m) q[0] += rh.a[m] * v.a[m];
      }
    }
    double tot[1], mine[1];
    block_sum<1, T>(q, mine);
    if (chunk_finish<1>(st, PH_K1, I.chunk0, I.nchunks, c, cm.part, mine, tot) && threadIdx.x == 0) {
      if (st.restart) {
        st.rho = st.rr;  // (r^, r) with r^ = r
        st.restart = 0;
      }
      st.pcur ^= 1;
      const double den = tot[0];
      if (den != 0.0 && isfinite(den) && st.rho != 0.0) {
        st.alpha = st.rho / den;
      } else {
        st.alpha = 0.0;  // breakdown: this iteration degenerates to a minimal-residual step
        st.restart = 1;
      }
    }
  });
}
template <typename T, int CH>
__global__ void __launch_bounds__(kThreads, krylov_blocks<T>()) k_bicg1(Common cm, Coef<T> co, Kry<T> kr) {
  count_launch(cm.ctl);
  bicg1_body<T, CH>(cm, co, kr);
}

// k2: s = r - alpha v;  t = B^-1 A~ s;  partials (t, s), (t, t). s is staged like p in k1.
template <typename T, int CH>
__device__ __forceinline__ void bicg2_body(Common cm, Coef<T> co, Kry<T> kr) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  for_active_chunks(cm, [&](int b_) { return cm.st[b_].inner_active != 0; }, [&](int c) {
    const int b = cm.chunk_inst[c];
    InstState& st = cm.st[b];
    const InstDev I = cm.inst[b];
    const T alpha = (T)st.alpha;
    const T* __restrict__ r = kr.r;
    const T* __restrict__ vv = sel2(kr.v, st.pcur);
    const int P = I.pitch;
    const long long c0 = chunk_start<CH>(c, I);
    const long long c1 = min(c0 + (long long)CH, inst_end(I));
    const long long e0 = c0 - P;
    stage_rows<T>(sm, e0, (c1 - c0) + 2LL * P, [&](long long k) {
      Q4<T> x = ld4(r + k);
      const Q4<T> v = ld4(vv + k);
#pragma unroll
      for (int m = 0; m < 4; ++m) x.a[m] -= alpha * v.a[m];
      return x;
    });
    __syncthreads();
    T q[2] = {(T)0, (T)0};
#pragma unroll 2
    for (int g = 0; g < CH / (4 * kThreads); ++g) {
      const long long K = c0 + 4 * (threadIdx.x + g * kThreads);
      if (K < c1) {
        const long long o = K - e0;
        const Q4<T> sc = *reinterpret_cast<const Q4<T>*>(sm + o);
        const Q4<T> cwq = ld4(co.cw + K), ceq = ld4(co.ce + K);
        Q4<T> t = stencil_sm<T>(sm, o, P, cwq, ceq, ld4(co.cs + K), ld4(co.cn + K));
        if (cm.precond) t = line4<T, T>(t, cwq, ceq);  // t = B^-1 A~ s
        st4(kr.t + K, t);
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          q[0] += t.a[m] * sc.a[m];
          q[1] += t.a[m] * t.a[m];
        }
      }
    }
    double tot[2], mine[2];
    block_sum<2, T>(q, mine);
    if (chunk_finish<2>(st, PH_K2, I.chunk0, I.nchunks, c, cm.part, mine, tot) && threadIdx.x == 0) {
      if (tot[1] > 0.0 && isfinite(tot[0])) {
        st.omega = tot[0] / tot[1];
      } else {
        st.omega = 0.0;
      }
      if (st.omega == 0.0) st.restart = 1;
    }
  });
}
template <typename T, int CH>
__global__ void __launch_bounds__(kThreads, krylov_blocks<T>()) k_bicg2(Common cm, Coef<T> co, Kry<T> kr) {
  count_launch(cm.ctl);
  bicg2_body<T, CH>(cm, co, kr);
}

// k3: x += alpha p + omega s (x starts at 0 on the first iteration of a solve);
//     r = s - omega t;  partials (r^, r), (r, r); convergence test.
template <typename T, int CH>
__device__ __forceinline__ void bicg3_body(Common cm, Kry<T> kr, int max_iters) {
  for_active_chunks(cm, [&](int b_) { return cm.st[b_].inner_active != 0; }, [&](int c) {
    const int b = cm.chunk_inst[c];
    InstState& st = cm.st[b];
    const InstDev I = cm.inst[b];
    const T alpha = (T)st.alpha, omega = (T)st.omega;
    const bool fresh = st.fresh != 0;
    const T* pp = sel2(kr.p, st.pcur);
    const T* vv = sel2(kr.v, st.pcur);
    T q[2] = {(T)0, (T)0};
#pragma unroll 2
    for (int g = 0; g < CH / (4 * kThreads); ++g) {
    const Slot s = slot_of<CH>(c, I, g);
    if (s.valid) {
      const long long K = s.K;
      const Q4<T> r = ld4(kr.r + K), v = ld4(vv + K), p = ld4(pp + K), t = ld4(kr.t + K);
      const Q4<T> rh = ld4(kr.rh + K);
      Q4<T> x = fresh ? Q4<T>{{(T)0, (T)0, (T)0, (T)0}} : ld4(kr.x + K);
      Q4<T> rn;
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const T sv = r.a[m] - alpha * v.a[m];
        x.a[m] += alpha * p.a[m] + omega * sv;
        rn.a[m] = sv - omega * t.a[m];
        q[0] += rh.a[m] * rn.a[m];
        q[1] += rn.a[m] * rn.a[m];
      }
      st4(kr.x + K, x);
      st4(kr.r + K, rn);
    }
    }
    double tot[2], mine[2];
    block_sum<2, T>(q, mine);
    if (chunk_finish<2>(st, PH_K3, I.chunk0, I.nchunks, c, cm.part, mine, tot) && threadIdx.x == 0) {
      st.fresh = 0;
      st.has_x = 1;
      st.iters += 1;
      st.iters_total += 1;
      st.cum_iters += 1;
      const double rhoN = tot[0];
      st.rr = tot[1];
      if (!(tot[1] > st.rr_target) || st.iters >= max_iters || !isfinite(tot[1])) {
        st.inner_active = 0;
        atomicSub(&cm.ctl->n_inner, 1);
      } else {
        const double beta = (rhoN / st.rho) * (st.alpha / st.omega);
        st.rho = rhoN;
        if (!isfinite(beta) || rhoN == 0.0) {
          st.restart = 1;
          st.beta = 0.0;
        } else {
          st.beta = beta;
        }
      }
    }
  });
}
template <typename T, int CH>
__global__ void __launch_bounds__(kThreads, krylov_blocks<T>()) k_bicg3(Common cm, Kry<T> kr, int max_iters) {
  count_launch(cm.ctl);
  bicg3_body<T, CH>(cm, kr, max_iters);
  loop_epilogue(cm, 1);
}

// The refinement loop of one step in one cooperative launch, for batches whose chunks fit in
// one wave of co-resident blocks (one large instance: there the launch and ramp of each kernel
// of the graph's loops cost more than its pass over the cells). The same chunk bodies as the
// kernels above, separated by grid-wide barriers. The loop decisions are the graph's: the last
// block of each deciding pass writes them (loop_epilogue, use_cond = 2) before the barrier,
// every block reads them after it, and nothing rewrites them before every block has finished
// the next pass -- so every block runs the same sequence of barriers, and the guards bound it.
// Launch only cooperatively (cudaLaunchAttributeCooperative), with at most one block per chunk.
// MINB resident blocks per SM: 2 (124 registers, no spill) when the chunks fit in 2 per SM,
// else 4 (64 registers, some spilled); on one 1024 x 1024 instance in double-word mode the first
// took 0.84 ms per step, the second 0.90, the separate kernels 0.98.
template <typename T, typename C, typename A, int CH, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_solve_coop(Common cm, Fields fl, Coef<C> cfull, Coef<T> ck,
                                                                Kry<T> kr, double tol, double inner_tol,
                                                                int max_refine, int max_iters) {
  count_launch(cm.ctl);
  cooperative_groups::grid_group grid = cooperative_groups::this_grid();
  const volatile int* go_outer = &cm.ctl->go_outer;
  const volatile int* go_inner = &cm.ctl->go_inner;
  // the trip counts are capped here as well (the same in every block), so the loops end even if
  // the decisions were never written
  for (int o = 0; o < cm.guard_refine; ++o) {
    resid_body<T, C, A, CH>(cm, fl, cfull, kr, tol, inner_tol, max_refine);
    loop_epilogue(cm, 0);
    grid.sync();
    const bool more = *go_outer != 0;
    bool inner = *go_inner != 0;
    for (int it = 0; inner && it < cm.guard_iters; ++it) {
      bicg1_body<T, CH>(cm, ck, kr);
      grid.sync();
      bicg2_body<T, CH>(cm, ck, kr);
      grid.sync();
      bicg3_body<T, CH>(cm, kr, max_iters);
      loop_epilogue(cm, 1);
      grid.sync();
      inner = *go_inner != 0;
    }
    if (!more) break;
  }
}

// ------------------------------------------------------------------------------ polish + checks
// y' = R + (I - A~) max(y, 0) >= 0 (R >= 0, fractions >= 0), f = y' / D; partials: sum colsum*f,
// sum R, clamped count; the chunk minimum of f travels in part slot 3. Chunks [c0, c1) of the
// list (c1 < 0: all); a range must hold whole instances.
// It also forms the next solve's start g (extrap over the new f, f^n and up to kOrder - 1 earlier
// states from the history) into the idle y buffer, and moves f^n into the oldest history slot.
// 4 resident blocks per SM (64 registers; measured on the 4096-instance batch: 2.55 ms per
// launch against 2.81 ms with 3 blocks and 80 registers)
template <typename C, typename A, int CH>
__global__ void __launch_bounds__(kThreads, 4) k_polish(Common cm, Fields fl, Coef<C> co, int c0, int c1) {
  using V = typename A::V;
  count_launch(cm.ctl);
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = reinterpret_cast<V*>(smraw);
  __shared__ float smin[kThreads / 32];
  for_active_chunks(cm, [&](int b_) { return cm.inst[b_].enabled != 0; }, [&](int c) {
    const int b = cm.chunk_inst[c];
    InstState& st = cm.st[b];
    const InstDev I = cm.inst[b];
    const double* y = sel2(fl.y64, st.ycur);
    double* gout = sel2(fl.y64, st.ycur ^ 1);
    // earlier states for the next start: f^n (the current f) and up to kOrder - 1 from the history
    const int nh = min(min(st.nhist + 1, kOrder), cm.hist_cap), hs = st.hslot;
    const double* h2p = sel3(fl.fh, hs);
    const double* h3p = sel3(fl.fh, (hs + 2) % kHist);
    const double* h4p = sel3(fl.fh, (hs + 1) % kHist);
    double* hw = sel3(fl.fh, (hs + 1) % kHist);  // the oldest slot (f^(n-3)) takes f^n
    const int P = I.pitch;
    const long long c0 = chunk_start<CH>(c, I);
    const long long c1 = min(c0 + (long long)CH, inst_end(I));
    const long long e0 = c0 - P;
    stage_rows<V>(sm, e0, (c1 - c0) + 2LL * P, [&](long long k) {
      Q4<V> v = A::ld4(y + k);
#pragma unroll
      for (int m = 0; m < 4; ++m) v.a[m] = A::max0(v.a[m]);
      return v;
    });
    __syncthreads();
    V mass = A::k(0.0), rsum = A::k(0.0);
    float clamp = 0.0f;
    float mn = 3.0e38f;
#pragma unroll 1
    for (int g = 0; g < CH / (4 * kThreads); ++g) {
      const long long K = c0 + 4 * (threadIdx.x + g * kThreads);
      if (K < c1) {
        const long long o = K - e0;
        // y' = R + sum over the neighbours of the outflow fraction times max(y, 0): every term is
        // >= 0, accumulated one direction at a time so that one coefficient row is live at once
        const Q4<V> R = A::ld4(fl.R + K);
        Q4<V> yp = R;
#pragma unroll
        for (int dir = 0; dir < 4; ++dir) {
          const Q4<V> c = CoefW<C, A>::row(co, dir, K);
          const long long on = o + (dir == 0 ? -1 : dir == 1 ? 1 : dir == 2 ? -P : P);
#pragma unroll
          for (int m = 0; m < 4; ++m) yp.a[m] = A::fmap(c.a[m], sm[on + m], yp.a[m]);
        }
        const Q4<V> inv = A::ld4(fl.invD + K), cols = A::ld4(fl.colsum + K);
        const int row_i0 = (int)((K - I.base) % I.pitch);
        Q4<V> fo;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          const V fv = A::mul(yp.a[m], inv.a[m]);
          fo.a[m] = fv;
          mass = A::fmap(cols.a[m], fv, mass);
          rsum = A::addp(rsum, R.a[m]);
          if (row_i0 + m < I.nx) {
            clamp += A::lt0(A::ld(y, K + m)) ? 1.0f : 0.0f;
            mn = fminf(mn, A::f32(fv));
          }
        }
        const Q4<V> fn = A::ld4(fl.f + K);
        Q4<V> g;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          // the states read here (the oldest one included) are read before the slot is replaced
          const V h2 = nh >= 2 ? A::ld(h2p, K + m) : fn.a[m];
          const V h3 = nh >= 3 ? A::ld(h3p, K + m) : h2;
          const V h4 = nh >= 4 ? A::ld(h4p, K + m) : h3;
          g.a[m] = A::extrap(fo.a[m], fn.a[m], h2, h3, h4, nh, fl.decay ? A::ld(fl.decay, K + m) : A::k(1.0));
        }
        A::st4(gout + K, g);
        A::st4(hw + K, fn);  // f^n into the oldest slot
        A::st4(fl.f + K, fo);
      }
    }
    // block minimum (separate from the sums)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = mn;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w) mn = fminf(mn, smin[w]);
      smin[0] = mn;
    }
    __syncthreads();
    float cl = clamp;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cl += __shfl_xor_sync(0xffffffffu, cl, o);
    const double w[3] = {A::warp_total_v(mass), A::warp_total_v(rsum), (double)cl};
    double tot[3], mine[3];
    block_sum_lane0<3>(w, mine);
    if (threadIdx.x == 0) cm.part[(size_t)c * 4 + 3] = (double)smin[0];
    if (chunk_finish<3>(st, PH_POLISH, I.chunk0, I.nchunks, c, cm.part, mine, tot)) {
      // the last block of the instance: minimum over its chunks, by the whole block
      __shared__ double s_min[kThreads / 32];
      double m = 1.0e300;
      for (int k = threadIdx.x; k < I.nchunks; k += blockDim.x) m = fmin(m, __ldcg(&cm.part[(size_t)(I.chunk0 + k) * 4 + 3]));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
      if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = m;
      __syncthreads();
      if (threadIdx.x == 0) {
        double gmin = s_min[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) gmin = fmin(gmin, s_min[w]);
        st.min_f = gmin;
        st.clamped = (long long)tot[2];
        st.mass_drift = tot[1] != 0.0 ? fabs(tot[0] - tot[1]) / fabs(tot[1]) : 0.0;
        st.steps += 1;
        st.hslot = (st.hslot + 1) % kHist;
        st.nhist = min(st.nhist + 1, kOrder);
        if (!(gmin >= 0.0)) st.status = ST_NEGATIVE;
      }
    }
    __syncthreads();
  }, c0, c1);
}

}  // namespace sg
