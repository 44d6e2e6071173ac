// nlgb_core.cuh -- device-side building blocks of the Jacobi-PCG solvers.
//
// The reference's hot loop is OpenNL's nlSolveSystemIterative(NL_CG) with a
// Jacobi preconditioner (called from src/lib/OGF/scene_graph/NL/matrix.cpp:
// 364,390-393 and, through nlSolve, from plugins/OGF/WarpDrive/commands/
// voxel_grob_transport_commands.cpp:281).  Per iteration it does one CRS SpMV
// (nlMultMatrixVector), two dot products and three axpy-like vector updates.
//
// Here every system is cut into fixed "tiles" of `tile_rows` consecutive rows.
// A tile is always processed by one 256-thread CTA with one fixed thread
// mapping, and every scalar (p.q, r.z, r.r) is the canonical reduction of the
// per-tile partials.  Because the summation order depends only on the system
// (its n, tile_rows and threads-per-row), the plain one-kernel-per-phase
// solver, the batched persistent kernel and the server all produce
// bit-identical iterates for the same system, whatever else is in the batch.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "nlgb_df.cuh"

namespace nlgb {

constexpr int kCTA = 256;            // threads per CTA for every solver kernel
constexpr int kWarps = kCTA / 32;
constexpr int kParts = 8;            // partial-sum slots per tile
// Slots used by each phase.  Consecutive phases use disjoint slots, so in the
// persistent kernel a CTA may start writing the next phase's partials while
// a slower CTA of its team is still reducing the previous phase's.
constexpr int kSlotPQ = 0;           // p.q                  (1 value)
constexpr int kSlotXR = 1;           // r.z, r.r             (2 values)
constexpr int kSlotFinal = 3;        // ||b - A x||^2        (1 value)
constexpr int kSlotInit = 4;         // b.b, r.z, r.r / mixed outer: 4 values

enum : int {
  ST_RUNNING = 0,
  ST_CONVERGED = 1,
  ST_MAX_ITER = 2,
  ST_BREAKDOWN = 3,
  ST_STAGNATION = 4,
  ST_DEVICE_ERR = 5,
  ST_BAD_INPUT = 6,
  ST_ABORTED = 7,
  ST_TRUE_STALLED = 8,   // recursive residual met eps, the true one did not after kMaxTrueChecks continuations
};

// FP64 / double-float solves stop on the recursive residual (OpenNL's rule)
// and then recompute the true one: at most this many times the iteration is
// continued with a lower recursive threshold before ST_TRUE_STALLED.
constexpr int kMaxTrueChecks = 4;

// Device-resident scalar state of one system (one per system, in HBM).
struct __align__(16) SysState {
  double rho, alpha, beta;     // CG scalars (FP64 in both precisions)
  double bnorm2;               // ||b||^2
  double thresh2;              // eps^2 (outer / plain)
  double rr;                   // last ||r||^2 (recursive residual)
  double rr_true;              // ||b - A x||^2 recomputed in FP64 at the end
  double rr64_prev;            // mixed: previous outer true residual^2
  double in_rr0;               // mixed: ||r||^2 at the start of the inner solve
  double in_thresh2;           // mixed: inner eps^2
  long long iter;              // CG iterations performed (inner ones, mixed)
  long long max_iter;
  long long guard;             // body passes executed (termination guard)
  long long guard_cap;
  int status;                  // ST_*
  int mode;                    // mixed: 0 = an outer step is due, 1 = inner PCG
  int outer, max_outer;        // mixed refinement steps
  int in_iter, in_max;         // mixed inner iterations in this outer step
  int zero_rhs;                // b == 0: the solution is x = 0
  int stall;                   // mixed: outer steps in a row without progress
  unsigned int cnt[4];         // last-CTA counters of the phase kernels
  int stage;                   // 0 start, 1 iterating, 2 final residual due, 3 done, 4 continuation
                               // due (the p update after a failed true-residual check is pending)
  int precision;               // batched: 0 FP64, 1 mixed
  int fell_back;               // mixed system continued in FP64 (FP32 could not track it)
  int checks;                  // FP64 / double-float: continuations after a failed true-residual check
  long long iter_at_fallback;  // FP32 iterations done before the FP64 fallback
  long long iter_stop;         // > 0: a graph chunk pauses (status unchanged) at this iteration
  long long coop_epoch;        // single-kernel iterations run in this solve (grid-barrier targets)
  double rthresh2;             // FP64 / double-float: threshold^2 of the recursive residual (starts at thresh2)
  int cont_ok;                 // beta / rho of the last iteration are valid (the iteration can be continued)
  int pad_;
  // Two-level election of the x / r update (FP64, double-float) and of the
  // mixed c / r update (index 1; index 0 is not used): arrivals per group of
  // tiles, groups done, and each group's warp-level sums (canonical order,
  // see elect2 in nlgb_solver.cu).
  unsigned int gcnt[2][8];
  unsigned int tcnt[2];
  unsigned int pad2_[2];
  double wsum[2][8][2];
};

// Algorithmic HBM bytes of one solve (n rows, z nonzeros), from its final
// state: per FP64 PCG iteration 12z + 108n (CRS values + int32 columns, row
// pointers, x gather, q; x/p/r/q/D^-1 vector passes); per FP32 iteration
// 8z + 56n; per FP64 reliable update 12z + 52n; plus the initial residual
// (12z + 36n) and the final true residual (12z + 16n).
inline __host__ __device__ double algo_bytes(long long n, long long z, const SysState& h) {
  const bool mixed_used = h.outer > 0;
  const double it32 = mixed_used ? double(h.fell_back ? h.iter_at_fallback : h.iter) : 0.0;
  const double it64 = double(h.iter) - it32;
  const double N = double(n), Z = double(z);
  double b = (12.0 * Z + 36.0 * N) + (12.0 * Z + 16.0 * N);
  b += it64 * (12.0 * Z + 108.0 * N) + it32 * (8.0 * Z + 56.0 * N);
  b += double(h.outer) * (12.0 * Z + 52.0 * N);
  if (h.fell_back) b += 12.0 * Z + 36.0 * N;   // FP64 restart residual
  // each failed true-residual check: that residual pass and the p update
  // that resumes the iteration
  b += double(h.checks) * (12.0 * Z + 48.0 * N);
  return b;
}

// Tiles per CTA in the vector phases of the graph solver: tiles of fewer
// than 512 rows are grouped so that a CTA covers about 512 rows.
inline __host__ __device__ int vec_tiles_for(int tile_rows) {
  return tile_rows >= 512 ? 1 : 512 / tile_rows;
}

// Everything a tile procedure needs about one system.
struct SysView {
  int n;                 // rows (== columns)
  int tile_rows;         // rows per tile (even; the autotuner uses multiples of 128)
  int n_tiles;
  int tpr;               // threads per row used by the SpMV (1..32)
  int df;                // 1: double-float iteration (x, r, p, q hold float2 pairs)
  const int* rp;         // CRS row pointers (n+1)
  const int* ci;         // CRS column indices
  const double* va;      // FP64 values
  const float* va32;     // FP32 values (mixed), may be null
  const float2* vadf;    // double-float values, may be null
  const double* dinv;    // Jacobi: 1/diag (1 where diag == 0)
  const float* dinv32;
  const float2* dinvdf;
  const double* b;
  double* x;
  double* r;
  double* p;
  double* q;
  float* r32;
  float* p32;
  float* q32;
  float* c32;            // mixed: correction accumulated by the inner PCG
  double* part;          // n_tiles * kParts tile partials
  SysState* st;
  const volatile int* abort_flag;   // host-mapped; nonzero -> stop
  long long budget;      // persistent kernel: iterations in this launch (> 0; else the launch's own)
};

// ---------------------------------------------------------------------------
// Reductions with a fixed order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block sum of up to 4 values at once, valid in thread 0 (every caller
// uses it there).  Each value goes through the tree of warp_sum (the lane
// butterfly, levels 16, 8, 4, 2, 1), then the eight warp totals are added in
// order.  The first two levels of several values share one FP64 addition
// per lane: at level 16 the lanes of one half-warp keep value a and receive
// the partner half's a while the other half-warp does the same for value b;
// at level 8 the quarter-warps split the pairs (a, b) and (c, d) the same
// way.  Floating-point addition is commutative, so each value's chain of
// additions is the butterfly's bit for bit, while GB300's narrow FP64 pipe
// issues 5 (K <= 2) or 6 (K <= 4) warp additions instead of 5 K, and the
// final sum of the warp totals runs in one thread instead of 256.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K]) {
  static_assert(K >= 1 && K <= 4, "block_sum: 1 to 4 values");
  __shared__ double red[K][kWarps];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  constexpr unsigned kAll = 0xffffffffu;
  double tot[4];
  if constexpr (K == 1) {
    tot[0] = warp_sum(v[0]);
  } else {
    const bool h16 = (l & 16) != 0;
    // level 16, values (0, 1): lanes 0-15 carry v0, lanes 16-31 v1
    double u = (h16 ? v[1] : v[0]) + __shfl_xor_sync(kAll, h16 ? v[0] : v[1], 16);
    if constexpr (K == 2) {
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) u += __shfl_xor_sync(kAll, u, o);
      tot[0] = u;                               // lanes 0-15
      tot[1] = __shfl_sync(kAll, u, 16);        // lanes 16-31
    } else {
      // level 16, values (2, 3) (a zero stands in for a missing fourth)
      const double v3 = K == 4 ? v[K - 1] : 0.0;
      const double u2 = (h16 ? v3 : v[2]) + __shfl_xor_sync(kAll, h16 ? v[2] : v3, 16);
      // level 8: quarter-warps 0 / 2 carry (v0, v1), quarter-warps 1 / 3 (v2, v3)
      const bool h8 = (l & 8) != 0;
      double t = (h8 ? u2 : u) + __shfl_xor_sync(kAll, h8 ? u : u2, 8);
#pragma unroll
      for (int o = 4; o > 0; o >>= 1) t += __shfl_xor_sync(kAll, t, o);
      tot[0] = t;                               // lanes 0-7
      tot[2] = __shfl_sync(kAll, t, 8);         // lanes 8-15
      tot[1] = __shfl_sync(kAll, t, 16);        // lanes 16-23
      tot[3] = __shfl_sync(kAll, t, 24);        // lanes 24-31
    }
  }
  __syncthreads();   // protect red[] from a previous use
  if (l == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) red[k][w] = tot[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < kWarps; ++i) s += red[k][i];
      v[k] = s;
    }
  }
}

// Canonical reduction of component `comp` of the tile partials (strided by
// kParts): thread t sums tiles t, t+256, ... in order, then block_sum (the
// result is valid in thread 0).
template <int K>
__device__ __forceinline__ void canon_reduce(const double* part, int n_tiles,
                                             const int (&comp)[K], double (&out)[K]) {
#pragma unroll
  for (int k = 0; k < K; ++k) out[k] = 0.0;
  // unrolled so the loads of one thread are in flight together (the sum
  // order stays tile t, t+256, t+512, ...)
#pragma unroll 8
  for (int t = threadIdx.x; t < n_tiles; t += kCTA) {
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] += __ldcg(part + (size_t)t * kParts + comp[k]);
  }
  block_sum<K>(out);
}

// Sub-warp sum over T lanes (butterfly: every lane ends with the same value).
template <int T, typename A>
__device__ __forceinline__ A subwarp_sum(A v) {
#pragma unroll
  for (int o = T / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Row dot product a_row . x with T threads per row.  All 32 lanes of the warp
// must call it (the shuffles use the full mask); `valid` masks the loads.
// kCoh: gather x through L2 only (needed when x was written earlier in the
// same kernel by another CTA, i.e. in the persistent batched kernel; the
// read-only path may return stale data there.  L1-cached gathers after the
// team barrier's acquire measured the same on GB300.)
// ---------------------------------------------------------------------------
template <int T, typename VT, typename XT, typename A, bool kCoh = false>
__device__ __forceinline__ A row_dot(const int* __restrict__ rp, const int* __restrict__ ci,
                                     const VT* __restrict__ va, const XT* __restrict__ x,
                                     int row, bool valid, int lane) {
  A sum = A(0);
  if (valid) {
    const int k0 = __ldg(rp + row), k1 = __ldg(rp + row + 1);
#pragma unroll 2
    for (int k = k0 + lane; k < k1; k += T) {
      const int c = __ldg(ci + k);
      const XT xc = kCoh ? __ldcg(x + c) : __ldg(x + c);
      sum = fma(A(__ldg(va + k)), A(xc), sum);
    }
  }
  return subwarp_sum<T, A>(sum);
}

// Rows [lo, hi) of a tile with T threads per row, one pass of kCTA/T rows at
// a time; epi(row, sum) is called by the row's lane 0.  Measured on GB300 and
// not kept: two rows per sub-warp in flight (2.96 vs 5.25 TB/s on the
// 7-nonzero Laplacian SpMV) and a "stream" layout staging each tile's
// nonzeros in shared memory (3.3 vs 5.2 TB/s there, 2.6 vs 4.4 on the
// 14-nonzero LSCM normal matrix).
template <int T, typename VT, typename XT, typename A, bool kCoh, typename Epi>
__device__ __forceinline__ void tile_rows_dot(const int* __restrict__ rp, const int* __restrict__ ci,
                                              const VT* __restrict__ va, const XT* __restrict__ x,
                                              int lo, int hi, Epi&& epi) {
  const int sub = threadIdx.x / T, lane = threadIdx.x % T;
  constexpr int RPP = kCTA / T;
  for (int base = lo; base < hi; base += RPP) {
    const int row = base + sub;
    const bool valid = row < hi;
    const A v = row_dot<T, VT, XT, A, kCoh>(rp, ci, va, x, row, valid, lane);
    if (valid && lane == 0) epi(row, v);
  }
}

__device__ __forceinline__ int tile_lo(const SysView& s, int tile) { return tile * s.tile_rows; }
__device__ __forceinline__ int tile_hi(const SysView& s, int tile) {
  const int h = (tile + 1) * s.tile_rows;
  return h < s.n ? h : s.n;
}

// ---------------------------------------------------------------------------
// FP64 tile procedures (plain form).
// ---------------------------------------------------------------------------

// q = A p on the tile; returns (block-wide) sum_i p_i q_i.
template <int T, bool kCoh = false>
__device__ double tile_spmv_pq(const SysView& s, int tile) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  double acc[1] = {0.0};
  tile_rows_dot<T, double, double, double, kCoh>(s.rp, s.ci, s.va, s.p, lo, hi,
    [&](int row, double qv) {
      s.q[row] = qv;
      acc[0] = fma(__ldcg(s.p + row), qv, acc[0]);
    });
  block_sum<1>(acc);
  return acc[0];
}

// r = b - A x, p = D^-1 r on the tile; returns (b.b, r.D^-1 r, r.r).
template <int T, bool kCoh = false>
__device__ void tile_residual(const SysView& s, int tile, double (&out)[3]) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  out[0] = out[1] = out[2] = 0.0;
  tile_rows_dot<T, double, double, double, kCoh>(s.rp, s.ci, s.va, s.x, lo, hi,
    [&](int row, double ax) {
      const double bi = s.b[row];
      const double ri = bi - ax;
      const double zi = s.dinv[row] * ri;
      s.r[row] = ri;
      s.p[row] = zi;
      out[0] = fma(bi, bi, out[0]);
      out[1] = fma(zi, ri, out[1]);
      out[2] = fma(ri, ri, out[2]);
    });
  block_sum<3>(out);
}

// Vector-phase loop helper: pairs of rows with 16-byte loads.  Row pairs
// [lo, hi) with lo even; an odd tail row is handled by thread 0 last.
template <typename F2, typename F1>
__device__ __forceinline__ void pair_loop(int lo, int hi, F2&& body2, F1&& body1) {
  const int p0 = lo >> 1, p1 = hi >> 1;
  for (int i2 = p0 + threadIdx.x; i2 < p1; i2 += kCTA) body2(i2);
  if ((hi & 1) && threadIdx.x == 0) body1(hi - 1);
}

// x += a p, r -= a q, z = D^-1 r; returns (r.z, r.r).  z is stored over q
// (A p is dead once r is updated, and the next SpMV rewrites q), so the p
// update reads z instead of computing D^-1 r again: one FP64 product per
// row fewer on GB300's narrow FP64 pipe, the same bytes (z written here,
// r and D^-1 no longer read there) and the same bits.
__device__ __forceinline__ void tile_update_xr(const SysView& s, int tile, double alpha,
                                               double (&out)[2]) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  double rz = 0.0, rr = 0.0;
  double2* x2 = reinterpret_cast<double2*>(s.x);
  double2* r2 = reinterpret_cast<double2*>(s.r);
  const double2* p2 = reinterpret_cast<const double2*>(s.p);
  double2* q2 = reinterpret_cast<double2*>(s.q);
  const double2* d2 = reinterpret_cast<const double2*>(s.dinv);
  pair_loop(lo, hi,
    [&](int i2) {
      double2 xv = __ldcg(x2 + i2), rv = __ldcg(r2 + i2);
      const double2 pv = __ldcg(p2 + i2), qv = __ldcg(q2 + i2), dv = __ldg(d2 + i2);
      xv.x = fma(alpha, pv.x, xv.x); xv.y = fma(alpha, pv.y, xv.y);
      rv.x = fma(-alpha, qv.x, rv.x); rv.y = fma(-alpha, qv.y, rv.y);
      x2[i2] = xv; r2[i2] = rv;
      const double zx = dv.x * rv.x, zy = dv.y * rv.y;
      q2[i2] = make_double2(zx, zy);
      rz = fma(zx, rv.x, rz); rz = fma(zy, rv.y, rz);
      rr = fma(rv.x, rv.x, rr); rr = fma(rv.y, rv.y, rr);
    },
    [&](int i) {
      s.x[i] = fma(alpha, __ldcg(s.p + i), __ldcg(s.x + i));
      const double ri = fma(-alpha, __ldcg(s.q + i), __ldcg(s.r + i));
      s.r[i] = ri;
      const double zi = s.dinv[i] * ri;
      s.q[i] = zi;
      rz = fma(zi, ri, rz);
      rr = fma(ri, ri, rr);
    });
  out[0] = rz; out[1] = rr;
  block_sum<2>(out);
}

// p = z + beta p, z = D^-1 r as tile_update_xr left it in q (every
// executor runs this right after tile_update_xr of the same iteration, or,
// after a true-residual check, as the pending update of the iteration that
// stopped: q still holds that iteration's z).
__device__ __forceinline__ void tile_update_p(const SysView& s, int tile, double beta) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  double2* p2 = reinterpret_cast<double2*>(s.p);
  const double2* z2 = reinterpret_cast<const double2*>(s.q);
  pair_loop(lo, hi,
    [&](int i2) {
      const double2 zv = __ldcg(z2 + i2);
      double2 pv = __ldcg(p2 + i2);
      pv.x = fma(beta, pv.x, zv.x);
      pv.y = fma(beta, pv.y, zv.y);
      p2[i2] = pv;
    },
    [&](int i) {
      s.p[i] = fma(beta, __ldcg(s.p + i), __ldcg(s.q + i));
    });
}

// Zero x on the tile (used when b == 0).
__device__ __forceinline__ void tile_zero_x(const SysView& s, int tile) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  for (int i = lo + threadIdx.x; i < hi; i += kCTA) s.x[i] = 0.0;
}

// ||b - A x||^2 on the tile, without writing anything.
template <int T, bool kCoh = false>
__device__ double tile_true_rr(const SysView& s, int tile) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  double acc[1] = {0.0};
  tile_rows_dot<T, double, double, double, kCoh>(s.rp, s.ci, s.va, s.x, lo, hi,
    [&](int row, double ax) {
      const double ri = s.b[row] - ax;
      acc[0] = fma(ri, ri, acc[0]);
    });
  block_sum<1>(acc);
  return acc[0];
}

// ---------------------------------------------------------------------------
// Double-float tile procedures: the FP64 iteration above (same phases, slots,
// scalar steps and canonical reductions) with r, p, q and x holding (hi, lo)
// float pairs in their 8-byte slots and the matrix and D^-1 read from
// double-float copies, so that the iteration runs on the FP32 pipe.  The
// initial and final residuals are FP64 (x converted on the fly).  A thread's
// partial dot products are double-float; the CTA reduces them in
// double-float (warp butterflies, then the eight warps in order) and hands
// one double per value to the canonical tile reduction.
// ---------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void df_block_sum(float2 (&v)[K], double (&out)[K]) {
  __shared__ float2 red[K][kWarps];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < K; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      float2 t;
      t.x = __shfl_xor_sync(0xffffffffu, v[k].x, o);
      t.y = __shfl_xor_sync(0xffffffffu, v[k].y, o);
      v[k] = df::dadd(v[k], t);   // commutative: every lane ends with the same value
    }
  }
  __syncthreads();   // protect red[] from a previous use
  if (l == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) red[k][w] = v[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float2 s = red[k][0];
#pragma unroll
    for (int i = 1; i < kWarps; ++i) s = df::dadd(s, red[k][i]);
    out[k] = df::to_double(s);
  }
}

// a_row . x in double-float with T threads per row (all 32 lanes call it).
// The lane's products are summed unnormalised: the heads through TwoSum,
// every error term into one float tail, normalised once at the end.  The
// dependency chain per nonzero is then one addition deep, and the loop is
// unrolled four times, so that more gathers are in flight (the FP32
// arithmetic is far from any limit; the loop is bound by memory latency).
template <int T, bool kCoh>
__device__ __forceinline__ float2 row_dot_df(const int* __restrict__ rp, const int* __restrict__ ci,
                                             const float2* __restrict__ va, const float2* __restrict__ x,
                                             int row, bool valid, int lane) {
  float hs = 0.f, tl = 0.f;
  if (valid) {
    const int k0 = __ldg(rp + row), k1 = __ldg(rp + row + 1);
#pragma unroll 4
    for (int k = k0 + lane; k < k1; k += T) {
      const int c = __ldg(ci + k);
      const float2 xc = kCoh ? __ldcg(x + c) : __ldg(x + c);
      const float2 a = __ldg(va + k);
      const float p = df::mul(a.x, xc.x);
      float e = df::fma(a.x, xc.x, -p);
      e = df::fma(a.x, xc.y, e);
      e = df::fma(a.y, xc.x, e);
      const float2 t = df::two_sum(hs, p);
      hs = t.x;
      tl = df::add(tl, df::add(t.y, e));
    }
  }
  float2 sum = df::fast_two_sum(hs, tl);
#pragma unroll
  for (int o = T / 2; o > 0; o >>= 1) {
    float2 t;
    t.x = __shfl_xor_sync(0xffffffffu, sum.x, o);
    t.y = __shfl_xor_sync(0xffffffffu, sum.y, o);
    sum = df::dadd(sum, t);
  }
  return sum;
}

// a_row . x in FP64 with x held as double-float (initial / final residual).
template <int T, bool kCoh>
__device__ __forceinline__ double row_dot_xdf(const int* __restrict__ rp, const int* __restrict__ ci,
                                              const double* __restrict__ va, const float2* __restrict__ x,
                                              int row, bool valid, int lane) {
  double sum = 0.0;
  if (valid) {
    const int k0 = __ldg(rp + row), k1 = __ldg(rp + row + 1);
    for (int k = k0 + lane; k < k1; k += T) {
      const int c = __ldg(ci + k);
      const float2 xc = kCoh ? __ldcg(x + c) : __ldg(x + c);
      sum = fma(__ldg(va + k), df::to_double(xc), sum);
    }
  }
  return subwarp_sum<T, double>(sum);
}

// r = b - A x (FP64, rounded to double-float), p = D^-1 r; returns
// (b.b, r.D^-1 r, r.r).
template <int T, bool kCoh = false>
__device__ void tile_df_residual(const SysView& s, int tile, double (&out)[3]) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  const float2* x2 = reinterpret_cast<const float2*>(s.x);
  float2* r2 = reinterpret_cast<float2*>(s.r);
  float2* p2 = reinterpret_cast<float2*>(s.p);
  const int sub = threadIdx.x / T, lane = threadIdx.x % T;
  constexpr int RPP = kCTA / T;
  double bb[1] = {0.0};
  float2 v[2] = {df::make(0.f, 0.f), df::make(0.f, 0.f)};
  for (int base = lo; base < hi; base += RPP) {
    const int row = base + sub;
    const bool valid = row < hi;
    const double ax = row_dot_xdf<T, kCoh>(s.rp, s.ci, s.va, x2, row, valid, lane);
    if (valid && lane == 0) {
      const double bi = s.b[row];
      const float2 ri = df::from_double(bi - ax);
      const float2 zi = df::dmul(__ldg(s.dinvdf + row), ri);
      r2[row] = ri;
      p2[row] = zi;
      bb[0] = fma(bi, bi, bb[0]);
      v[0] = df::mac(v[0], zi, ri);
      v[1] = df::mac(v[1], ri, ri);
    }
  }
  double o[2];
  df_block_sum<2>(v, o);
  block_sum<1>(bb);
  out[0] = bb[0]; out[1] = o[0]; out[2] = o[1];
}

// q = A p on the tile; returns sum_i p_i q_i.
template <int T, bool kCoh = false>
__device__ double tile_df_spmv_pq(const SysView& s, int tile) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  const float2* p2 = reinterpret_cast<const float2*>(s.p);
  float2* q2 = reinterpret_cast<float2*>(s.q);
  const int sub = threadIdx.x / T, lane = threadIdx.x % T;
  constexpr int RPP = kCTA / T;
  float2 acc[1] = {df::make(0.f, 0.f)};
  for (int base = lo; base < hi; base += RPP) {
    const int row = base + sub;
    const bool valid = row < hi;
    const float2 qv = row_dot_df<T, kCoh>(s.rp, s.ci, s.vadf, p2, row, valid, lane);
    if (valid && lane == 0) {
      q2[row] = qv;
      acc[0] = df::mac(acc[0], __ldcg(p2 + row), qv);
    }
  }
  double o[1];
  df_block_sum<1>(acc, o);
  return o[0];
}

// x += a p, r -= a q; returns (r.D^-1 r, r.r).
__device__ __forceinline__ void tile_df_update_xr(const SysView& s, int tile, double alpha,
                                                  double (&out)[2]) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  const float2 a = df::from_double(alpha), na = df::neg(a);
  float4* x4 = reinterpret_cast<float4*>(s.x);
  float4* r4 = reinterpret_cast<float4*>(s.r);
  const float4* p4 = reinterpret_cast<const float4*>(s.p);
  const float4* q4 = reinterpret_cast<const float4*>(s.q);
  const float4* d4 = reinterpret_cast<const float4*>(s.dinvdf);
  float2 v[2] = {df::make(0.f, 0.f), df::make(0.f, 0.f)};
  pair_loop(lo, hi,
    [&](int i2) {
      const float4 xv = __ldcg(x4 + i2), rv = __ldcg(r4 + i2);
      const float4 pv = __ldcg(p4 + i2), qv = __ldcg(q4 + i2), dv = __ldg(d4 + i2);
      const float2 x0 = df::mac(df::make(xv.x, xv.y), a, df::make(pv.x, pv.y));
      const float2 x1 = df::mac(df::make(xv.z, xv.w), a, df::make(pv.z, pv.w));
      const float2 r0 = df::mac(df::make(rv.x, rv.y), na, df::make(qv.x, qv.y));
      const float2 r1 = df::mac(df::make(rv.z, rv.w), na, df::make(qv.z, qv.w));
      x4[i2] = make_float4(x0.x, x0.y, x1.x, x1.y);
      r4[i2] = make_float4(r0.x, r0.y, r1.x, r1.y);
      const float2 z0 = df::dmul(df::make(dv.x, dv.y), r0);
      const float2 z1 = df::dmul(df::make(dv.z, dv.w), r1);
      v[0] = df::mac(v[0], z0, r0); v[0] = df::mac(v[0], z1, r1);
      v[1] = df::mac(v[1], r0, r0); v[1] = df::mac(v[1], r1, r1);
    },
    [&](int i) {
      float2* x2 = reinterpret_cast<float2*>(s.x);
      float2* r2 = reinterpret_cast<float2*>(s.r);
      x2[i] = df::mac(__ldcg(x2 + i), a, __ldcg(reinterpret_cast<const float2*>(s.p) + i));
      const float2 ri = df::mac(__ldcg(r2 + i), na, __ldcg(reinterpret_cast<const float2*>(s.q) + i));
      r2[i] = ri;
      const float2 zi = df::dmul(__ldg(s.dinvdf + i), ri);
      v[0] = df::mac(v[0], zi, ri);
      v[1] = df::mac(v[1], ri, ri);
    });
  df_block_sum<2>(v, out);
}

// p = D^-1 r + beta p.
__device__ __forceinline__ void tile_df_update_p(const SysView& s, int tile, double beta) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  const float2 bt = df::from_double(beta);
  float4* p4 = reinterpret_cast<float4*>(s.p);
  const float4* r4 = reinterpret_cast<const float4*>(s.r);
  const float4* d4 = reinterpret_cast<const float4*>(s.dinvdf);
  pair_loop(lo, hi,
    [&](int i2) {
      const float4 rv = __ldcg(r4 + i2), dv = __ldg(d4 + i2), pv = __ldcg(p4 + i2);
      const float2 p0 = df::mac(df::dmul(df::make(dv.x, dv.y), df::make(rv.x, rv.y)), bt,
                                df::make(pv.x, pv.y));
      const float2 p1 = df::mac(df::dmul(df::make(dv.z, dv.w), df::make(rv.z, rv.w)), bt,
                                df::make(pv.z, pv.w));
      p4[i2] = make_float4(p0.x, p0.y, p1.x, p1.y);
    },
    [&](int i) {
      float2* p2 = reinterpret_cast<float2*>(s.p);
      const float2 zi = df::dmul(__ldg(s.dinvdf + i), __ldcg(reinterpret_cast<const float2*>(s.r) + i));
      p2[i] = df::mac(zi, bt, __ldcg(p2 + i));
    });
}

// ||b - A x||^2 on the tile (FP64, x held as double-float).
template <int T, bool kCoh = false>
__device__ double tile_df_true_rr(const SysView& s, int tile) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  const float2* x2 = reinterpret_cast<const float2*>(s.x);
  const int sub = threadIdx.x / T, lane = threadIdx.x % T;
  constexpr int RPP = kCTA / T;
  double acc[1] = {0.0};
  for (int base = lo; base < hi; base += RPP) {
    const int row = base + sub;
    const bool valid = row < hi;
    const double ax = row_dot_xdf<T, kCoh>(s.rp, s.ci, s.va, x2, row, valid, lane);
    if (valid && lane == 0) {
      const double ri = s.b[row] - ax;
      acc[0] = fma(ri, ri, acc[0]);
    }
  }
  block_sum<1>(acc);
  return acc[0];
}

// Compile-time selection between the FP64 (D = false) and double-float
// (D = true) procedures of the same phase.
template <bool D, int T, bool kCoh = false>
__device__ __forceinline__ void phase_residual(const SysView& s, int tile, double (&out)[3]) {
  if constexpr (D) tile_df_residual<T, kCoh>(s, tile, out);
  else tile_residual<T, kCoh>(s, tile, out);
}
template <bool D, int T, bool kCoh = false>
__device__ __forceinline__ double phase_spmv_pq(const SysView& s, int tile) {
  if constexpr (D) return tile_df_spmv_pq<T, kCoh>(s, tile);
  else return tile_spmv_pq<T, kCoh>(s, tile);
}
template <bool D>
__device__ __forceinline__ void phase_update_xr(const SysView& s, int tile, double alpha, double (&out)[2]) {
  if constexpr (D) tile_df_update_xr(s, tile, alpha, out);
  else tile_update_xr(s, tile, alpha, out);
}
template <bool D>
__device__ __forceinline__ void phase_update_p(const SysView& s, int tile, double beta) {
  if constexpr (D) tile_df_update_p(s, tile, beta);
  else tile_update_p(s, tile, beta);
}
template <bool D, int T, bool kCoh = false>
__device__ __forceinline__ double phase_true_rr(const SysView& s, int tile) {
  if constexpr (D) return tile_df_true_rr<T, kCoh>(s, tile);
  else return tile_true_rr<T, kCoh>(s, tile);
}

// ---------------------------------------------------------------------------
// Mixed-precision tile procedures: FP32 matrix values and Krylov vectors,
// FP64 for the outer residual, the solution update and the accumulation of
// every dot product that feeds alpha / beta.
// ---------------------------------------------------------------------------

// x += c (FP64 update from the FP32 correction), c = 0.
__device__ __forceinline__ void tile_mx_apply(const SysView& s, int tile) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  double2* x2 = reinterpret_cast<double2*>(s.x);
  float2* c2 = reinterpret_cast<float2*>(s.c32);
  pair_loop(lo, hi,
    [&](int i2) {
      double2 xv = __ldcg(x2 + i2);
      const float2 cv = __ldcg(c2 + i2);
      xv.x += double(cv.x); xv.y += double(cv.y);
      x2[i2] = xv;
      c2[i2] = make_float2(0.f, 0.f);
    },
    [&](int i) {
      s.x[i] = __ldcg(s.x + i) + double(__ldcg(s.c32 + i));
      s.c32[i] = 0.f;
    });
}

// Reliable update: r64 = b - A64 x (FP64), r32 = float(r64).  The search
// direction p32 is kept (the Krylov recurrence continues on the corrected
// residual).  Returns (b.b, ||r64||^2, r32.z32, ||r32||^2), all accumulated
// in FP64.
template <int T, bool kCoh = false>
__device__ void tile_mx_outer(const SysView& s, int tile, double (&out)[4]) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  out[0] = out[1] = out[2] = out[3] = 0.0;
  tile_rows_dot<T, double, double, double, kCoh>(s.rp, s.ci, s.va, s.x, lo, hi,
    [&](int row, double ax) {
      const double bi = s.b[row];
      const double ri = bi - ax;
      const float r32 = float(ri);
      const float z32 = s.dinv32[row] * r32;
      s.r32[row] = r32;
      out[0] = fma(bi, bi, out[0]);
      out[1] = fma(ri, ri, out[1]);
      out[2] = fma(double(z32), double(r32), out[2]);
      out[3] = fma(double(r32), double(r32), out[3]);
    });
  block_sum<4>(out);
}

// q32 = A32 p32 (FP32 row sums); returns sum p.q accumulated in FP64.
template <int T, bool kCoh = false>
__device__ double tile_mx_spmv_pq(const SysView& s, int tile) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  double acc[1] = {0.0};
  tile_rows_dot<T, float, float, float, kCoh>(s.rp, s.ci, s.va32, s.p32, lo, hi,
    [&](int row, float qv) {
      s.q32[row] = qv;
      acc[0] += double(__ldcg(s.p32 + row) * qv);   // FP32 product, FP64 accumulation
    });
  block_sum<1>(acc);
  return acc[0];
}

// c32 += a p32, r32 -= a q32 (FP32 arithmetic, alpha from FP64);
// returns (r.D^-1 r, r.r) accumulated in FP64.
__device__ __forceinline__ void tile_mx_update_cr(const SysView& s, int tile, double alpha,
                                                  double (&out)[2]) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  const float a = float(alpha);
  // A thread owns at most a row pair of the tile (tiles are <= 2 * kCTA
  // rows): its products are summed in FP32 (at most two terms, error of the
  // order of the FP32 storage of r and z themselves), converted once, and
  // everything across threads, tiles and the vector is accumulated in FP64.
  // This keeps the GB300's small FP64 pipe (1/56 of FP32) off the hot loop.
  float rz32 = 0.f, rr32 = 0.f;
  float2* c2 = reinterpret_cast<float2*>(s.c32);
  float2* r2 = reinterpret_cast<float2*>(s.r32);
  const float2* p2 = reinterpret_cast<const float2*>(s.p32);
  const float2* q2 = reinterpret_cast<const float2*>(s.q32);
  const float2* d2 = reinterpret_cast<const float2*>(s.dinv32);
  double rz = 0.0, rr = 0.0;
  pair_loop(lo, hi,
    [&](int i2) {
      float2 cv = __ldcg(c2 + i2), rv = __ldcg(r2 + i2);
      const float2 pv = __ldcg(p2 + i2), qv = __ldcg(q2 + i2), dv = __ldg(d2 + i2);
      cv.x = fmaf(a, pv.x, cv.x); cv.y = fmaf(a, pv.y, cv.y);
      rv.x = fmaf(-a, qv.x, rv.x); rv.y = fmaf(-a, qv.y, rv.y);
      c2[i2] = cv; r2[i2] = rv;
      const float zx = dv.x * rv.x, zy = dv.y * rv.y;
      rz32 = fmaf(zy, rv.y, zx * rv.x);
      rr32 = fmaf(rv.y, rv.y, rv.x * rv.x);
      rz += double(rz32);
      rr += double(rr32);
    },
    [&](int i) {
      s.c32[i] = fmaf(a, __ldcg(s.p32 + i), __ldcg(s.c32 + i));
      const float ri = fmaf(-a, __ldcg(s.q32 + i), __ldcg(s.r32 + i));
      s.r32[i] = ri;
      const float zi = s.dinv32[i] * ri;
      rz += double(zi * ri);
      rr += double(ri * ri);
    });
  out[0] = rz; out[1] = rr;
  block_sum<2>(out);
}

// p32 = D^-1 r32 + beta p32.
__device__ __forceinline__ void tile_mx_update_p(const SysView& s, int tile, double beta) {
  const int lo = tile_lo(s, tile), hi = tile_hi(s, tile);
  const float bt = float(beta);
  float2* p2 = reinterpret_cast<float2*>(s.p32);
  const float2* r2 = reinterpret_cast<const float2*>(s.r32);
  const float2* d2 = reinterpret_cast<const float2*>(s.dinv32);
  pair_loop(lo, hi,
    [&](int i2) {
      const float2 rv = __ldcg(r2 + i2), dv = __ldg(d2 + i2);
      float2 pv = __ldcg(p2 + i2);
      pv.x = fmaf(bt, pv.x, dv.x * rv.x);
      pv.y = fmaf(bt, pv.y, dv.y * rv.y);
      p2[i2] = pv;
    },
    [&](int i) {
      s.p32[i] = fmaf(bt, __ldcg(s.p32 + i), s.dinv32[i] * __ldcg(s.r32 + i));
    });
}

// ---------------------------------------------------------------------------
// Scalar steps (run by one thread once all tile partials of a phase are in).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool finite_pos(double v) { return v > 0.0 && v < 1.0e300; }

// After the initial residual: decide whether any iteration is needed.
__device__ __forceinline__ void scalar_after_init(SysState* st, double bb, double rz, double rr) {
  st->bnorm2 = bb;
  st->rthresh2 = st->thresh2;
  st->checks = 0;
  st->cont_ok = 0;
  st->rho = rz;
  st->rr = rr;
  if (!st->fell_back) st->iter = 0;   // a fallback keeps counting the FP32 iterations
  if (!(bb > 0.0)) {             // b == 0 (or NaN): x = 0 is the solution
    st->zero_rhs = (bb == 0.0);
    st->status = (bb == 0.0) ? ST_CONVERGED : ST_BREAKDOWN;
    return;
  }
  if (!(rr <= 1.0e300)) { st->status = ST_BREAKDOWN; return; }
  if (rr <= st->thresh2 * bb) { st->status = ST_CONVERGED; return; }
  if (st->max_iter <= 0) { st->status = ST_MAX_ITER; return; }
  if (!finite_pos(rz)) { st->status = ST_BREAKDOWN; return; }
}

__device__ __forceinline__ void scalar_after_pq(SysState* st, double pq) {
  if (!finite_pos(pq)) { st->status = ST_BREAKDOWN; return; }
  st->alpha = st->rho / pq;
}

// beta and rho are advanced before the stopping test, so that an iteration
// stopped on the recursive residual can be continued (scalar_after_check).
__device__ __forceinline__ void scalar_after_xr(SysState* st, double rz, double rr) {
  st->iter += 1;
  st->rr = rr;
  if (!(rr <= 1.0e300)) { st->status = ST_BREAKDOWN; return; }
  const bool rz_ok = finite_pos(rz);
  st->cont_ok = rz_ok ? 1 : 0;
  if (rz_ok) {
    st->beta = rz / st->rho;
    st->rho = rz;
  }
  if (rr <= st->rthresh2 * st->bnorm2) { st->status = ST_CONVERGED; return; }
  if (st->iter >= st->max_iter) { st->status = ST_MAX_ITER; return; }
  if (!rz_ok) { st->status = ST_BREAKDOWN; return; }
}

// After the final true residual ||b - A x||^2 (rr_true) of an FP64 or
// double-float solve.  The iteration stopped when its recursively updated
// residual met eps (OpenNL's rule); in finite precision that residual drifts
// away from the true one, so the true one may still miss eps.  Then the
// recursive threshold is lowered by the observed ratio (with a 0.9 margin in
// norm) and the same recurrence continues (status back to ST_RUNNING,
// returns true; the caller applies the pending p update first).  After
// kMaxTrueChecks continuations, or when the gap is too large to close by
// iterating (the recursive residual would have to go 1e4x below eps: the
// attainable accuracy of the recurrence is reached), the solve ends with
// ST_TRUE_STALLED.  Mixed-precision systems stop on the true residual
// already and are left alone.
__host__ __device__ __forceinline__ bool scalar_after_check(SysState* st) {
  if (st->status != ST_CONVERGED || st->zero_rhs || st->precision == 1) return false;
  if (st->rr_true <= st->thresh2 * st->bnorm2) return false;
  const double next = st->thresh2 * (st->rr / st->rr_true) * 0.81;
  if (!st->cont_ok || st->checks >= kMaxTrueChecks || st->iter >= st->max_iter || !(st->rr > 0.0) ||
      !(next >= st->thresh2 * 1.0e-8)) {
    st->status = ST_TRUE_STALLED;
    return false;
  }
  st->rthresh2 = next;
  st->checks += 1;
  st->status = ST_RUNNING;
  return true;
}

// Mixed precision = FP32 PCG with FP64 reliable updates (defect correction
// that keeps the Krylov direction): the inner iteration runs on FP32 values
// and vectors; whenever its FP32 residual has dropped by in_thresh since the
// last update (or claims convergence), the FP32 correction is added to the
// FP64 solution, the true residual b - A x is recomputed in FP64 and replaces
// the FP32 residual, and the iteration continues with the same p.  Restarted
// refinement (a fresh inner PCG per outer step) loses the Krylov space each
// time and stagnates on the ill-conditioned LSCM normal equations; the
// continued recurrence keeps FP64-like iteration counts.
//
// After a reliable update (FP64 residual rr64, new FP32 residual's r.z and
// r.r).  The first call (outer == 0) is the initial residual.
__device__ __forceinline__ void scalar_after_outer(SysState* st, double bb, double rr64,
                                                   double rz32, double rr32) {
  if (st->outer == 0) st->bnorm2 = bb;
  const double bb0 = st->bnorm2;
  st->rr = rr64;
  if (!(bb0 > 0.0)) {
    st->zero_rhs = (bb0 == 0.0);
    st->status = (bb0 == 0.0) ? ST_CONVERGED : ST_BREAKDOWN;
    return;
  }
  if (!(rr64 <= 1.0e300)) { st->status = ST_BREAKDOWN; return; }
  if (rr64 <= st->thresh2 * bb0) { st->status = ST_CONVERGED; return; }
  if (st->iter >= st->max_iter) { st->status = ST_MAX_ITER; return; }
  if (st->outer >= st->max_outer) { st->status = ST_STAGNATION; return; }
  // FP32 not tracking the FP64 system: an update is due after the FP32
  // residual fell by in_thresh (0.1 by default), so a healthy update shrinks
  // the true residual by about as much.  Two updates in a row that shrink it
  // by less than 2x mean the FP32-rounded matrix is too far from the FP64
  // one (kappa * u32 ~ 1, e.g. LSCM normal equations): report STAGNATION so
  // the caller continues this system in FP64 from the current x.
  if (st->outer > 0) {
    if (rr64 > 0.25 * st->rr64_prev) st->stall += 1;
    else st->stall = 0;
  }
  st->rr64_prev = rr64;
  if (st->stall >= 2) { st->status = ST_STAGNATION; return; }
  if (!finite_pos(rz32) || !finite_pos(rr32)) { st->status = ST_BREAKDOWN; return; }
  st->beta = (st->outer == 0) ? 0.0 : rz32 / st->rho;
  st->rho = rz32;
  st->in_rr0 = rr32;     // FP32 residual^2 right after this update
  st->in_iter = 0;
  st->outer += 1;
  st->mode = 1;
}

// After the FP32 vector update: either continue (beta from the FP32
// residual) or request a reliable update (mode -> 0).
__device__ __forceinline__ void scalar_after_mx_cr(SysState* st, double rz, double rr) {
  st->iter += 1;
  st->in_iter += 1;
  if (!(rr <= 1.0e300)) { st->status = ST_BREAKDOWN; return; }
  if (rr <= st->in_thresh2 * st->in_rr0 || rr <= st->thresh2 * st->bnorm2 ||
      st->in_iter >= st->in_max || st->iter >= st->max_iter || !finite_pos(rz)) {
    st->mode = 0;
    return;
  }
  st->beta = rz / st->rho;
  st->rho = rz;
}

}  // namespace nlgb
