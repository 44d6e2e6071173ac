// nlgb_solver.cu -- plain FP64 and mixed FP32/FP64 Jacobi-PCG on one GPU.
//
// Replaces the iteration of OpenNL's nlSolveSystemIterative(NL_CG, Jacobi)
// (call sites: src/lib/OGF/scene_graph/NL/matrix.cpp:364,390-393; nlSolve at
// plugins/OGF/WarpDrive/commands/voxel_grob_transport_commands.cpp:281).
//
// One PCG iteration = three kernels (SpMV + p.q; x/r update + r.z, r.r;
// p update).  Each kernel's last CTA reduces the tile partials in a fixed
// order and advances the scalar state in HBM, so the host never reads a
// scalar during the solve: the loop is a CUDA-graph while-node whose
// condition is cleared from the device.  A guard kernel counts body passes
// and clears the condition after a hard cap, so the loop always ends.
#include "nlgb_batch.h"
#include "nlgb_core.cuh"
#include "nlgb_internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>

namespace nlgb {

// ---------------------------------------------------------------------------
// Last-CTA election: thread 0 publishes this tile's partials; returns true in
// every thread of the CTA that arrived last.
// ---------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ bool publish_elect(const SysView& s, int tile, const double (&v)[K], int slot,
                                              unsigned int* counter) {
  __shared__ int am_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) __stcg(s.part + (size_t)tile * kParts + slot + k, v[k]);
    __threadfence();
    const unsigned int prev = atomicAdd(counter, 1u);
    am_last = (prev == (unsigned int)s.n_tiles - 1u);
    if (am_last) *counter = 0u;   // next use is in a later kernel
  }
  __syncthreads();
  if (am_last) __threadfence();
  return am_last != 0;
}

// ---------------------------------------------------------------------------
// Two-level last-CTA election with the canonical reduction (the tails of
// k_update_xr and of the mixed iteration's c / r update).  The canonical
// order (canon_reduce) sums tile t into thread (t mod 256)'s running sum,
// then each warp's 32 running sums by a butterfly, then the 8 warp totals in
// order.  Here the tiles of warp g's running sums -- those with (t mod 256)
// / 32 == g -- form group g: the CTAs of a group arrive on the group's
// counter, the last one computes the group's warp total (one warp, the same
// loads, adds and butterfly), and the last of the groups adds the 8 totals
// in order.  Same result bit for bit as one CTA reducing every partial, but
// the partials are read by eight CTAs in parallel as their groups complete,
// and no counter takes more than 1/8 of the arrivals.  Each CTA covers vec
// consecutive tiles starting at tile0 (vec divides 32, so they lie in one
// group).  Returns true in every thread of the CTA that finishes; thread 0
// then holds the K sums in out.
// ---------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ bool elect2(const SysView& s, int tile0, int vec, int slot, int phase,
                                       double (&out)[K]) {
  __shared__ int flag;
  SysState* st = s.st;
  const int g = (tile0 & 255) >> 5;
  const int ngroups = min(8, (s.n_tiles + 31) >> 5);
  if (threadIdx.x == 0) {
    const int per_grp = 32 / vec, per_cyc = 256 / vec;
    const int G = (int)gridDim.x;
    const int size = (G / per_cyc) * per_grp + min(max(G % per_cyc - g * per_grp, 0), per_grp);
    __threadfence();
    const unsigned int prev = atomicAdd(&st->gcnt[phase][g], 1u);
    flag = (prev == (unsigned int)size - 1u);
    if (flag) st->gcnt[phase][g] = 0u;   // next use is in a later kernel
  }
  __syncthreads();
  if (!flag) return false;
  __threadfence();
  if (threadIdx.x < 32) {
    double v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = 0.0;
#pragma unroll 8
    for (int t = (g << 5) + (int)threadIdx.x; t < s.n_tiles; t += kCTA) {
#pragma unroll
      for (int k = 0; k < K; ++k) v[k] += __ldcg(s.part + (size_t)t * kParts + slot + k);
    }
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < K; ++k) __stcg(&st->wsum[phase][g][k], v[k]);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int prev = atomicAdd(&st->tcnt[phase], 1u);
    flag = (prev == (unsigned int)ngroups - 1u);
    if (flag) st->tcnt[phase] = 0u;
  }
  __syncthreads();
  if (!flag) return false;
  __threadfence();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double sum = 0.0;
      for (int w = 0; w < 8; ++w) sum += (w < ngroups) ? __ldcg(&st->wsum[phase][w][k]) : 0.0;
      out[k] = sum;
    }
  }
  return true;
}

__device__ __forceinline__ int ld_status(const SysState* st) { return __ldcg(&st->status); }
__device__ __forceinline__ int ld_mode(const SysState* st) { return __ldcg(&st->mode); }

// ---------------------------------------------------------------------------
// Plain FP64 kernels.
// ---------------------------------------------------------------------------
// D: double-float iteration (the same kernels on float pairs).
template <int T, bool D>
__global__ void __launch_bounds__(kCTA) k_init(SysView s) {
  double v[3];
  phase_residual<D, T>(s, blockIdx.x, v);
  if (publish_elect<3>(s, blockIdx.x, v, kSlotInit, &s.st->cnt[0])) {
    const int comp[3] = {kSlotInit, kSlotInit + 1, kSlotInit + 2};
    double o[3];
    canon_reduce<3>(s.part, s.n_tiles, comp, o);
    if (threadIdx.x == 0) scalar_after_init(s.st, o[0], o[1], o[2]);
  }
}

// The SpMV hands p.q on without a reduction tail: k_spmv_pq stores its
// tiles' p.q partials and ends, and every CTA of k_update_xr reduces those
// partials itself in the canonical order and applies the scalar step
// (alpha) to its own shared copy of the state.  The serial tail of a
// last-CTA reduction (fence, arrival, partial loads, fence, scalar step)
// left the SMs idle for several microseconds after the SpMV.  k_update_xr
// keeps its tail: its r.z and r.r feed beta and the stopping test, and
// having every CTA of k_update_p reduce them instead cost more than the tail
// (measured on the 1.3M-unknown LSCM iteration: the SpMV 76.4 -> 69.8 us,
// k_update_p 11.0 -> 23.1 us, with 1,134 CTAs re-reading the same partials
// before their short tile work).  Same sums, same scalar steps: the
// iterates are those of the other executors bit for bit.

// Every thread's copy of the system state into shared memory (16-byte
// words; the state was written by an earlier kernel).
__device__ __forceinline__ void load_state(SysState& dst, const SysState* src) {
  constexpr int kWords = (int)(sizeof(SysState) / 16);
  static_assert(sizeof(SysState) % 16 == 0, "SysState is 16-byte aligned");
  const int4* sp = reinterpret_cast<const int4*>(src);
  int4* dp = reinterpret_cast<int4*>(&dst);
  for (int i = threadIdx.x; i < kWords; i += blockDim.x) dp[i] = __ldcg(sp + i);
  __syncthreads();
}

// Eight CTAs per SM (32 registers): the tile autotuner sizes one wave of
// CTAs on that residency.
template <int T, bool D>
__global__ void __launch_bounds__(kCTA, 8) k_spmv_pq(SysView s) {
  if (ld_status(s.st) != ST_RUNNING) return;
  const double v = phase_spmv_pq<D, T>(s, blockIdx.x);
  if (threadIdx.x == 0) __stcg(s.part + (size_t)blockIdx.x * kParts + kSlotPQ, v);
}

// Vector phases: each CTA handles vec_tiles_for(tile_rows) consecutive tiles
// (the partial of every tile is still computed and stored on its own, so the
// canonical reduction is unchanged): small tiles are grouped into fuller CTAs.
__device__ __forceinline__ int vec_t0(const SysView& s) { return blockIdx.x * vec_tiles_for(s.tile_rows); }
__device__ __forceinline__ int vec_t1(const SysView& s) {
  return min(s.n_tiles, (int)(blockIdx.x + 1) * vec_tiles_for(s.tile_rows));
}

template <int K>
__device__ __forceinline__ void store_parts(const SysView& s, int tile, const double (&v)[K], int slot) {
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) __stcg(s.part + (size_t)tile * kParts + slot + k, v[k]);
  }
}

// alpha = rho / p.q from the SpMV's partials (every CTA), then x, r and
// z = D^-1 r; the last CTA of the two-level election writes alpha back and
// takes the step after r.z and r.r (beta, stopping test).
template <bool D>
__global__ void __launch_bounds__(kCTA, 8) k_update_xr(SysView s) {
  __shared__ SysState sst;
  load_state(sst, s.st);
  if (sst.status != ST_RUNNING) return;
  {
    const int comp[1] = {kSlotPQ};
    double o[1];
    canon_reduce<1>(s.part, s.n_tiles, comp, o);
    if (threadIdx.x == 0) scalar_after_pq(&sst, o[0]);
    __syncthreads();
  }
  if (sst.status == ST_RUNNING) {
    const double alpha = sst.alpha;
    for (int t = vec_t0(s), t1 = vec_t1(s); t < t1; ++t) {
      double v[2];
      phase_update_xr<D>(s, t, alpha, v);
      store_parts<2>(s, t, v, kSlotXR);
    }
  }
  double o[2];
  if (elect2<2>(s, vec_t0(s), vec_tiles_for(s.tile_rows), kSlotXR, 1, o) && threadIdx.x == 0) {
    s.st->alpha = sst.alpha;
    s.st->status = sst.status;
    if (sst.status == ST_RUNNING) scalar_after_xr(s.st, o[0], o[1]);
  }
}

template <bool D>
__global__ void __launch_bounds__(kCTA, 8) k_update_p(SysView s) {
  if (ld_status(s.st) != ST_RUNNING) return;
  const double beta = __ldcg(&s.st->beta);
  for (int t = vec_t0(s), t1 = vec_t1(s); t < t1; ++t) phase_update_p<D>(s, t, beta);
}

// ---------------------------------------------------------------------------
// One whole FP64 PCG iteration in one cooperative kernel (small and mid-size
// systems, all tiles in one resident wave): SpMV + p.q, grid barrier, x / r
// update, grid barrier, p update; the kernel boundary orders the next
// iteration's SpMV after this p update.  Every CTA reduces the tile partials
// in the canonical order and applies the same scalar steps to its own copy
// of the state (identical results), so the phases need no extra barrier for
// the scalars; CTA 0 writes the state back.  The tile procedures, reductions
// and scalar steps are those of the three-kernel iteration: the iterates are
// bit-identical.  Replaces three kernel boundaries and three last-CTA
// reduction tails per iteration by two barriers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long coop_atom_add(unsigned long long* p) {
  unsigned long long old;
  asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], 1;" : "=l"(old) : "l"(p) : "memory");
  return old;
}
__device__ __forceinline__ unsigned long long coop_ld_acquire(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long coop_clock_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid barrier on a monotonic counter (one arrival per CTA per barrier):
// returns false in every thread if the wait exceeded 4 s.
__device__ bool coop_grid_sync(unsigned long long* bar, unsigned long long target) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    coop_atom_add(bar);
    const unsigned long long t0 = coop_clock_ns();
    unsigned int spins = 0;
    while (coop_ld_acquire(bar) < target) {
      if ((++spins & 63u) == 0u && coop_clock_ns() - t0 > 4000000000ULL) { ok = 0; break; }
    }
  }
  __syncthreads();
  return ok != 0;
}

template <int T, bool D>
__global__ void __launch_bounds__(kCTA) k_iter(SysView s, unsigned long long* bar) {
  __shared__ SysState sst;
  if (threadIdx.x == 0) sst = *s.st;      // written by the previous kernel
  __syncthreads();
  if (sst.status != ST_RUNNING) return;
  const int G = gridDim.x;
  const unsigned long long base = (unsigned long long)sst.coop_epoch * 2ULL * (unsigned long long)G;
  for (int t = blockIdx.x; t < s.n_tiles; t += G) {
    const double v = phase_spmv_pq<D, T>(s, t);
    if (threadIdx.x == 0) __stcg(s.part + (size_t)t * kParts + kSlotPQ, v);
  }
  bool ok = coop_grid_sync(bar, base + G);
  if (ok) {
    const int comp[1] = {kSlotPQ};
    double o[1];
    canon_reduce<1>(s.part, s.n_tiles, comp, o);
    if (threadIdx.x == 0) scalar_after_pq(&sst, o[0]);
    __syncthreads();
    if (sst.status == ST_RUNNING) {
      const double alpha = sst.alpha;
      for (int t = blockIdx.x; t < s.n_tiles; t += G) {
        double v[2];
        phase_update_xr<D>(s, t, alpha, v);
        if (threadIdx.x == 0) {
          __stcg(s.part + (size_t)t * kParts + kSlotXR, v[0]);
          __stcg(s.part + (size_t)t * kParts + kSlotXR + 1, v[1]);
        }
      }
    }
    // every CTA takes the second barrier (the epoch arithmetic counts both)
    ok = coop_grid_sync(bar, base + 2ULL * G);
    if (ok && sst.status == ST_RUNNING) {
      const int comp2[2] = {kSlotXR, kSlotXR + 1};
      double o2[2];
      canon_reduce<2>(s.part, s.n_tiles, comp2, o2);
      if (threadIdx.x == 0) scalar_after_xr(&sst, o2[0], o2[1]);
      __syncthreads();
      if (sst.status == ST_RUNNING) {
        const double beta = sst.beta;
        for (int t = blockIdx.x; t < s.n_tiles; t += G) phase_update_p<D>(s, t, beta);
      }
    }
  }
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    if (!ok) sst.status = ST_DEVICE_ERR;
    sst.coop_epoch += 1;
    *s.st = sst;
  }
}

// Termination guard of a while-node body (single thread).  use_handle == 0:
// launched outside a graph (eager mode), the host reads the status instead.
__global__ void k_guard(SysView s, cudaGraphConditionalHandle h, int need_mode, int use_handle) {
  SysState* st = s.st;
  st->guard += 1;
  bool stop = st->status != ST_RUNNING;
  if (!stop && s.abort_flag != nullptr && *s.abort_flag != 0) {
    st->status = ST_ABORTED;
    stop = true;
  }
  if (!stop && st->guard >= st->guard_cap) {
    st->status = ST_MAX_ITER;
    stop = true;
  }
  if (!stop && need_mode >= 0 && st->mode != need_mode) stop = true;
  // pause of a resumable chunk: the system stays ST_RUNNING
  if (!stop && st->iter_stop > 0 && st->iter >= st->iter_stop) stop = true;
  if (stop && use_handle) cudaGraphSetConditional(h, 0u);
}

// Before a resumable chunk of at most `iters` iterations: pause point and a
// matching cap on while-body passes.
__global__ void k_chunk_start(SysState* st, long long iters, int unroll) {
  st->iter_stop = st->iter + iters;
  st->guard_cap = st->guard + iters / unroll + 4;
}

// After a chunk: a system that stopped (converged or failed) is done; its
// true residual was computed by the final kernel of the graph.  A system
// whose true-residual check asked for more iterations keeps stage 4.
__global__ void k_chunk_end(SysState* st) {
  if (st->status != ST_RUNNING) st->stage = 3;
}

__device__ __forceinline__ unsigned long long chunk_clock_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Mirrored chunks (ChunkMirror): the budget comes from host-mapped memory
// written before the launch; the start time is kept there for the end.
__global__ void k_chunk_start_m(SysState* st, ChunkMirror* m, int unroll) {
  const long long budget = *reinterpret_cast<volatile long long*>(&m->budget);
  const long long iters = budget > 0 ? budget : 1;
  st->iter_stop = st->iter + iters;
  st->guard_cap = st->guard + iters / unroll + 4;
  *reinterpret_cast<volatile unsigned long long*>(&m->t_start) = chunk_clock_ns();
}

// End of a mirrored chunk (one warp): the k_chunk_end rule, then the state
// copied to the mirror, the duration, a system-scope fence by every lane,
// and last the sequence number the host polls.
__global__ void k_chunk_end_m(SysState* st, ChunkMirror* m) {
  if (threadIdx.x == 0 && st->status != ST_RUNNING) st->stage = 3;
  __syncwarp();
  static_assert(sizeof(SysState) % 8 == 0, "SysState is copied in 8-byte words");
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(st);
  volatile unsigned long long* dst = reinterpret_cast<volatile unsigned long long*>(&m->st);
  for (int i = (int)threadIdx.x; i < (int)(sizeof(SysState) / 8); i += (int)blockDim.x) dst[i] = __ldcg(src + i);
  if (threadIdx.x == 0) {
    const unsigned long long t0 = *reinterpret_cast<volatile unsigned long long*>(&m->t_start);
    *reinterpret_cast<volatile unsigned long long*>(&m->t_ns) = chunk_clock_ns() - t0;
  }
  __threadfence_system();
  __syncwarp();
  if (threadIdx.x == 0) {
    volatile unsigned int* seq = &m->seq;
    *seq = *seq + 1u;
  }
}

// After the final residual: the true-residual check (single thread).  A
// continuation sets the status back to running and stage 4.
__global__ void k_check(SysState* st) {
  if (scalar_after_check(st)) st->stage = 4;
}

// Start of a continuation (stage 4): the p update the stopped iteration did
// not do, p = D^-1 r + beta p (vector-phase grid); no-op otherwise.
template <bool D>
__global__ void __launch_bounds__(kCTA) k_resume_p(SysView s) {
  if (ld_status(s.st) != ST_RUNNING || __ldcg(&s.st->stage) != 4) return;
  const double beta = __ldcg(&s.st->beta);
  for (int t = vec_t0(s), t1 = vec_t1(s); t < t1; ++t) phase_update_p<D>(s, t, beta);
}

// After k_resume_p: iterating again (single thread).
__global__ void k_resume_mark(SysState* st) {
  if (st->stage == 4) st->stage = 1;
}

// ||b - A x||^2 of the final iterate; zeroes x when b == 0.
template <int T, bool D>
__global__ void __launch_bounds__(kCTA) k_final(SysView s) {
  double v[1] = {0.0};
  if (__ldcg(&s.st->zero_rhs)) {
    tile_zero_x(s, blockIdx.x);   // all-zero bits: 0.0 in either representation
  } else {
    v[0] = phase_true_rr<D, T>(s, blockIdx.x);
  }
  if (publish_elect<1>(s, blockIdx.x, v, kSlotFinal, &s.st->cnt[3])) {
    const int comp[1] = {kSlotFinal};
    double o[1];
    canon_reduce<1>(s.part, s.n_tiles, comp, o);
    if (threadIdx.x == 0) s.st->rr_true = o[0];
  }
}

// Chunk forms (resumable executor, ViewGraph): the initial residual only for
// a fresh system (stage 0; the last CTA moves it to stage 1, or 2 when no
// iteration is needed), and the final residual only for a system that
// stopped (a paused chunk leaves it running).  Every CTA reads stage /
// status before it arrives on the election, so all of them take the same
// branch.
template <int T, bool D>
__global__ void __launch_bounds__(kCTA) k_init_chunk(SysView s) {
  if (__ldcg(&s.st->stage) != 0 || ld_status(s.st) != ST_RUNNING) return;
  double v[3];
  phase_residual<D, T>(s, blockIdx.x, v);
  if (publish_elect<3>(s, blockIdx.x, v, kSlotInit, &s.st->cnt[0])) {
    const int comp[3] = {kSlotInit, kSlotInit + 1, kSlotInit + 2};
    double o[3];
    canon_reduce<3>(s.part, s.n_tiles, comp, o);
    if (threadIdx.x == 0) {
      scalar_after_init(s.st, o[0], o[1], o[2]);
      s.st->stage = s.st->status == ST_RUNNING ? 1 : 2;
    }
  }
}

template <int T, bool D>
__global__ void __launch_bounds__(kCTA) k_final_if(SysView s) {
  if (ld_status(s.st) == ST_RUNNING) return;
  double v[1] = {0.0};
  if (__ldcg(&s.st->zero_rhs)) {
    tile_zero_x(s, blockIdx.x);
  } else {
    v[0] = phase_true_rr<D, T>(s, blockIdx.x);
  }
  if (publish_elect<1>(s, blockIdx.x, v, kSlotFinal, &s.st->cnt[3])) {
    const int comp[1] = {kSlotFinal};
    double o[1];
    canon_reduce<1>(s.part, s.n_tiles, comp, o);
    if (threadIdx.x == 0) s.st->rr_true = o[0];
  }
}

// Mixed chunk, after its (possibly skipped) initial FP64 residual.
__global__ void k_mark_started(SysState* st) {
  if (st->stage == 0) st->stage = st->status == ST_RUNNING ? 1 : 2;
}

// A mixed system whose FP32 iteration cannot track it (STAGNATION before any
// fallback) continues as FP64 PCG from its current x, keeping its iteration
// count -- the same transition as the persistent kernel's and the graph
// solver's.
__global__ void k_fallback_fp64(SysState* st) {
  if (st->status != ST_STAGNATION || st->fell_back || st->precision != 1) return;
  st->status = ST_RUNNING;
  st->precision = 0;
  st->fell_back = 1;
  st->stage = 0;
  st->mode = 0;
  st->iter_at_fallback = st->iter;
}

// ---------------------------------------------------------------------------
// Mixed-precision kernels.
// ---------------------------------------------------------------------------
// Reliable update, part 1: x += c, c = 0 (only when an update is due).
__global__ void __launch_bounds__(kCTA) k_mx_apply(SysView s) {
  if (ld_status(s.st) != ST_RUNNING || ld_mode(s.st) != 0) return;
  for (int t = vec_t0(s), t1 = vec_t1(s); t < t1; ++t) tile_mx_apply(s, t);
}

// Reliable update, part 2: FP64 true residual, FP32 residual replaced.
template <int T>
__global__ void __launch_bounds__(kCTA) k_mx_outer(SysView s) {
  if (ld_status(s.st) != ST_RUNNING || ld_mode(s.st) != 0) return;
  double v[4];
  tile_mx_outer<T>(s, blockIdx.x, v);
  if (publish_elect<4>(s, blockIdx.x, v, kSlotInit, &s.st->cnt[0])) {
    const int comp[4] = {kSlotInit, kSlotInit + 1, kSlotInit + 2, kSlotInit + 3};
    double o[4];
    canon_reduce<4>(s.part, s.n_tiles, comp, o);
    if (threadIdx.x == 0) scalar_after_outer(s.st, o[0], o[1], o[2], o[3]);
  }
}

// q32 = A32 p32; stores the tiles' p.q partials (alpha is taken by every CTA
// of k_mx_update_cr, as in the FP64 iteration).
template <int T>
__global__ void __launch_bounds__(kCTA) k_mx_spmv_pq(SysView s) {
  if (ld_status(s.st) != ST_RUNNING || ld_mode(s.st) != 1) return;
  const double v = tile_mx_spmv_pq<T>(s, blockIdx.x);
  if (threadIdx.x == 0) __stcg(s.part + (size_t)blockIdx.x * kParts + kSlotPQ, v);
}

// alpha from the SpMV's partials (every CTA), then c += a p, r -= a q; the
// last CTA writes alpha back, decides whether a reliable update is due and
// sets the condition of the IF node that runs it (use_handle == 0: eager
// mode, the update kernels are launched anyway and check the mode).
__global__ void __launch_bounds__(kCTA) k_mx_update_cr(SysView s, cudaGraphConditionalHandle h_upd,
                                                       int use_handle) {
  __shared__ SysState sst;
  load_state(sst, s.st);
  if (sst.status != ST_RUNNING || sst.mode != 1) return;
  {
    const int comp[1] = {kSlotPQ};
    double o[1];
    canon_reduce<1>(s.part, s.n_tiles, comp, o);
    if (threadIdx.x == 0) scalar_after_pq(&sst, o[0]);
    __syncthreads();
  }
  if (sst.status == ST_RUNNING) {
    const double alpha = sst.alpha;
    for (int t = vec_t0(s), t1 = vec_t1(s); t < t1; ++t) {
      double v[2];
      tile_mx_update_cr(s, t, alpha, v);
      store_parts<2>(s, t, v, kSlotXR);
    }
  }
  double o[2];
  if (elect2<2>(s, vec_t0(s), vec_tiles_for(s.tile_rows), kSlotXR, 1, o) && threadIdx.x == 0) {
    s.st->alpha = sst.alpha;
    s.st->status = sst.status;
    if (sst.status == ST_RUNNING) scalar_after_mx_cr(s.st, o[0], o[1]);
    const bool upd = s.st->status == ST_RUNNING && s.st->mode == 0;
    if (use_handle) cudaGraphSetConditional(h_upd, upd ? 1u : 0u);
  }
}

__global__ void __launch_bounds__(kCTA) k_mx_update_p(SysView s) {
  if (ld_status(s.st) != ST_RUNNING || ld_mode(s.st) != 1) return;
  const double beta = __ldcg(&s.st->beta);
  for (int t = vec_t0(s), t1 = vec_t1(s); t < t1; ++t) tile_mx_update_p(s, t, beta);
}

// ---------------------------------------------------------------------------
// Standalone SpMV (nlMultMatrixVector) and helpers.
// ---------------------------------------------------------------------------
template <int T, typename V, typename X>
__global__ void __launch_bounds__(kCTA) k_spmv(int n, int tile_rows, const int* __restrict__ rp,
                                               const int* __restrict__ ci, const V* __restrict__ va,
                                               const X* __restrict__ x, X* __restrict__ y) {
  const int lo = blockIdx.x * tile_rows;
  const int hi = min(lo + tile_rows, n);
  tile_rows_dot<T, V, X, X, false>(rp, ci, va, x, lo, hi, [&](int row, X v) { y[row] = v; });
}

// dinv[i] = 1 / a_ii (1 when the diagonal is missing or zero); fp32 copies.
__global__ void k_jacobi(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                         const double* __restrict__ va, double* dinv, float* dinv32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = 0.0;
  for (int k = rp[i]; k < rp[i + 1]; ++k)
    if (ci[k] == i) d += va[k];
  const double inv = (d != 0.0) ? 1.0 / d : 1.0;
  dinv[i] = inv;
  if (dinv32) dinv32[i] = float(inv);
}

__global__ void k_to_f32(long long n, const double* __restrict__ a, float* __restrict__ b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = float(a[i]);
}

__global__ void k_to_df(long long n, const double* __restrict__ a, float2* __restrict__ b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = df::from_double(a[i]);
}

// In place, element by element: a double becomes its (hi, lo) float pair in
// the same 8 bytes, and back.
__global__ void k_df_pack(long long n, double* x) {
  float2* x2 = reinterpret_cast<float2*>(x);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = x[i];
    x2[i] = df::from_double(v);
  }
}
__global__ void k_df_unpack(long long n, double* x) {
  float2* x2 = reinterpret_cast<float2*>(x);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float2 v = x2[i];
    x[i] = df::to_double(v);
  }
}

// Largest biased FP64 exponent of a[0..n) (2047 for Inf/NaN) and smallest
// one among its nonzero entries (0 for subnormals): out[0] max, out[1] min.
__global__ void k_exp_range(long long n, const double* __restrict__ a, int* out) {
  int mx = 0, mn = 4096;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(a[i]);
    if ((bits << 1) == 0ULL) continue;   // +-0
    const int e = (int)((bits >> 52) & 0x7ffULL);
    mx = max(mx, e);
    mn = min(mn, e);
  }
  mx = __reduce_max_sync(0xffffffffu, mx);
  mn = __reduce_min_sync(0xffffffffu, mn);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, mx);
    atomicMin(out + 1, mn);
  }
}

// Histogram of row lengths: bins 0..31 exact, bin 32 = longer; max length.
__global__ void k_row_hist(int n, const int* __restrict__ rp, int* hist33, int* maxlen) {
  __shared__ int h[33];
  __shared__ int mx;
  if (threadIdx.x < 33) h[threadIdx.x] = 0;
  if (threadIdx.x == 0) mx = 0;
  __syncthreads();
  int local_max = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int len = rp[i + 1] - rp[i];
    atomicAdd(&h[len < 32 ? len : 32], 1);
    local_max = max(local_max, len);
  }
  atomicMax(&mx, local_max);
  __syncthreads();
  if (threadIdx.x < 33 && h[threadIdx.x]) atomicAdd(&hist33[threadIdx.x], h[threadIdx.x]);
  if (threadIdx.x == 0) atomicMax(maxlen, mx);
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
static int grid_for(long long n, int threads) {
  long long g = (n + threads - 1) / threads;
  return (int)std::max(1LL, std::min(g, 152LL * 32));
}

// 256-thread phase CTAs resident on the device at once (eight per SM: the
// phase kernels use at most 32 registers per thread).
static long long resident_slots() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
    cudaGetLastError();
    sms = 152;
  }
  return 8LL * sms;
}
long long phase_resident_slots() { return resident_slots(); }

// CTAs of the single-kernel iteration k_iter<T> resident at once (0 if the
// occupancy cannot be queried).
// Above ~640 CTAs the single-counter barrier and the per-CTA canonical
// reductions (CTAs x tiles partial reads) cost more than the two kernel
// boundaries they replace (measured on GB300: 512 CTAs 30 vs 38 us per
// iteration, 834-1,024 CTAs 47-64 vs 39-50 us).
constexpr long long kCoopMaxCtas = 640;

template <bool D>
static const void* iter_kernel(int tpr) {
  switch (tpr) {
    case 1: return (const void*)k_iter<1, D>;
    case 2: return (const void*)k_iter<2, D>;
    case 4: return (const void*)k_iter<4, D>;
    case 8: return (const void*)k_iter<8, D>;
    case 16: return (const void*)k_iter<16, D>;
    default: return (const void*)k_iter<32, D>;
  }
}

// Resident CTAs per SM of the single-kernel iteration: the smaller of its
// FP64 and double-float forms, so that a matrix's layout and executor do not
// depend on the precision it is solved in (0 if it cannot be queried).
static int coop_per_sm(int tpr) {
  int a = 0, b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, iter_kernel<false>(tpr), kCTA, 0) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, iter_kernel<true>(tpr), kCTA, 0) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return std::min(a, b);
}

static long long coop_wave(int tpr) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  const int per_sm = coop_per_sm(tpr);
  return std::min<long long>((long long)per_sm * sms, kCoopMaxCtas);
}

TuneChoice autotune(int n, long long nnz, int max_row, const int* hist33) {
  // Threads per row: the smallest power of two with at most ~8 nonzeros per
  // lane for the typical row (measured on GB300 with the 7-nonzero cotangent
  // Laplacian: 1 thread/row 5.25 TB/s, 2 -> 4.4, 4 -> 2.7, 8 -> 1.4; with the
  // 14-nonzero LSCM normal matrix 2 threads/row is best), raised when long
  // rows dominate.
  long long cnt = 0, acc = 0;
  for (int b = 0; b < 33; ++b) { cnt += hist33 ? hist33[b] : 0; acc += hist33 ? (long long)hist33[b] * b : 0; }
  const double mean = n > 0 ? double(nnz) / double(n) : 0.0;
  // 90th percentile of the clipped histogram.
  int p90 = 0;
  if (hist33 && cnt > 0) {
    long long c = 0;
    for (int b = 0; b < 33; ++b) { c += hist33[b]; if (c * 10 >= cnt * 9) { p90 = b; break; } }
  } else {
    p90 = (int)std::ceil(mean);
  }
  const double typical = std::max(mean, 0.75 * double(p90 == 32 ? std::max(32, max_row) : p90));
  int tpr = 1;
  while (tpr < 32 && tpr * 8 < typical) tpr *= 2;
  // Tile rows.  Every phase kernel runs one CTA per tile (the vector phases
  // one per tile group), eight 256-thread CTAs resident per SM.  A second,
  // nearly empty wave of CTAs costs as much as a full one (measured on GB300
  // with the 1.3M-row LSCM matrix: 1,276 tiles of 1,024 rows left the SMs
  // idle 27 % of the SpMV), so the tile size minimises the rows of the
  // busiest CTA slot, ceil(tiles / slots) x tile_rows, over multiples of 128
  // rows with at most 4,096 tiles; among equal costs the fewest tiles (each
  // scalar is a reduction over the tiles, so three waves of 384-row tiles
  // are slower than one wave of 1,152).  Small systems keep 128-row tiles:
  // one wave of CTAs as small as they go; systems just above one resident
  // wave of the single-kernel iteration (k_iter) at 128 rows take 256-row
  // tiles, so that they still fit that wave (one tile per CTA).
  const long long slots = resident_slots();
  const long long cw = coop_wave(tpr);
  int tile = 128;
  if (cw > 0 && (long long)n > 128 * cw && (long long)n <= 256 * cw) {
    tile = 256;
  } else if ((long long)n > slots * 128) {
    long long best_cost = -1;
    for (int t = 128; t <= 16384; t += 128) {
      const long long nt = ((long long)n + t - 1) / t;
      if (nt > 4096) continue;
      const long long cost = ((nt + slots - 1) / slots) * (long long)t;
      if (best_cost < 0 || cost <= best_cost) { best_cost = cost; tile = t; }
    }
  }
  (void)acc;
  return TuneChoice{tpr, tile};
}

cudaError_t row_histogram(const DeviceCRS& A, int* hist33_host, int* max_row, cudaStream_t s) {
  int* d = nullptr;
  NLGB_CUDA_TRY(cudaMallocAsync(&d, 34 * sizeof(int), s));
  NLGB_CUDA_TRY(cudaMemsetAsync(d, 0, 34 * sizeof(int), s));
  if (A.n > 0) {
    k_row_hist<<<grid_for(A.n, 256), 256, 0, s>>>(A.n, A.rp, d, d + 33);
    count_launches(1);
  }
  NLGB_CUDA_TRY(cudaGetLastError());
  int h[34];
  NLGB_CUDA_TRY(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
  NLGB_CUDA_TRY(cudaStreamSynchronize(s));
  NLGB_CUDA_TRY(cudaFreeAsync(d, s));
  std::memcpy(hist33_host, h, 33 * sizeof(int));
  *max_row = h[33];
  return cudaSuccess;
}

cudaError_t crs_upload(DeviceCRS& A, int n, int m, const int* rp, const int* ci,
                       const double* va, cudaStream_t s) {
  crs_free(A);
  const long long nnz = rp[n];
  A.n = n; A.m = m; A.nnz = nnz;
  NLGB_CUDA_TRY(cudaMallocAsync(&A.rp, (size_t)(n + 1) * sizeof(int), s));
  NLGB_CUDA_TRY(cudaMallocAsync(&A.ci, (size_t)std::max(1LL, nnz) * sizeof(int), s));
  NLGB_CUDA_TRY(cudaMallocAsync(&A.va, (size_t)std::max(1LL, nnz) * sizeof(double), s));
  NLGB_CUDA_TRY(cudaMemcpyAsync(A.rp, rp, (size_t)(n + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
  if (nnz > 0) {
    NLGB_CUDA_TRY(cudaMemcpyAsync(A.ci, ci, (size_t)nnz * sizeof(int), cudaMemcpyHostToDevice, s));
    NLGB_CUDA_TRY(cudaMemcpyAsync(A.va, va, (size_t)nnz * sizeof(double), cudaMemcpyHostToDevice, s));
  }
  return cudaSuccess;
}

cudaError_t crs_adopt_device(DeviceCRS& A, int n, int m, long long nnz, int* rp, int* ci,
                             double* va, cudaStream_t) {
  crs_free(A);
  A.n = n; A.m = m; A.nnz = nnz; A.rp = rp; A.ci = ci; A.va = va;
  return cudaSuccess;
}

void crs_free(DeviceCRS& A) {
  if (!A.owns) { A = DeviceCRS(); return; }
  cudaFree(A.rp); cudaFree(A.ci); cudaFree(A.va); cudaFree(A.va32);
  cudaFree(A.dinv); cudaFree(A.dinv32);
  cudaFree(A.vadf); cudaFree(A.dinvdf);
  A = DeviceCRS();
}

void crs_free_async(DeviceCRS& A, cudaStream_t s) {
  if (!A.owns) { A = DeviceCRS(); return; }
  for (void* p : {(void*)A.rp, (void*)A.ci, (void*)A.va, (void*)A.va32, (void*)A.dinv, (void*)A.dinv32,
                  (void*)A.vadf, (void*)A.dinvdf})
    if (p) cudaFreeAsync(p, s);
  A = DeviceCRS();
}

long long device_bytes(const DeviceCRS& A) {
  long long b = (long long)(A.n + 1) * 4 + A.nnz * 12;
  if (A.va32) b += A.nnz * 4;
  if (A.dinv) b += (long long)A.n * 8;
  if (A.dinv32) b += (long long)A.n * 4;
  if (A.vadf) b += A.nnz * 8;
  if (A.dinvdf) b += (long long)A.n * 8;
  return b;
}

cudaError_t crs_prepare(DeviceCRS& A, bool need_fp32, cudaStream_t s) {
  if (A.tpr == 0) {
    int hist[33];
    int mx = 0;
    NLGB_CUDA_TRY(row_histogram(A, hist, &mx, s));
    A.max_row = mx;
    const TuneChoice c = autotune(A.n, A.nnz, mx, hist);
    A.tpr = c.tpr;
    A.tile_rows = c.tile_rows;
  }
  if (!A.dinv) {
    NLGB_CUDA_TRY(cudaMallocAsync(&A.dinv, (size_t)std::max(1, A.n) * sizeof(double), s));
    NLGB_CUDA_TRY(cudaMallocAsync(&A.dinv32, (size_t)std::max(1, A.n) * sizeof(float), s));
    if (A.n > 0) {
      k_jacobi<<<(A.n + 255) / 256, 256, 0, s>>>(A.n, A.rp, A.ci, A.va, A.dinv, A.dinv32);
      count_launches(1);
    }
    NLGB_CUDA_TRY(cudaGetLastError());
  }
  if (need_fp32 && !A.va32) {
    NLGB_CUDA_TRY(cudaMallocAsync(&A.va32, (size_t)std::max(1LL, A.nnz) * sizeof(float), s));
    if (A.nnz > 0) {
      k_to_f32<<<grid_for(A.nnz, 256), 256, 0, s>>>(A.nnz, A.va, A.va32);
      count_launches(1);
    }
    NLGB_CUDA_TRY(cudaGetLastError());
  }
  return cudaSuccess;
}

// Exponent range [2^-100, 2^100] for the double-float copies: the low
// halves (2^-24 of the high ones) stay normal floats, and products and sums
// of a few such values stay finite.
constexpr int kDfMinExp = 1023 - 100, kDfMaxExp = 1023 + 100;

static cudaError_t exp_range(long long n, const double* a, int* host2, cudaStream_t s) {
  host2[0] = 0; host2[1] = 4096;
  if (n <= 0) return cudaSuccess;
  int* d = nullptr;
  NLGB_CUDA_TRY(cudaMallocAsync(&d, 2 * sizeof(int), s));
  NLGB_CUDA_TRY(cudaMemcpyAsync(d, host2, 2 * sizeof(int), cudaMemcpyHostToDevice, s));
  k_exp_range<<<grid_for(n, 256), 256, 0, s>>>(n, a, d);
  count_launches(1);
  NLGB_CUDA_TRY(cudaGetLastError());
  NLGB_CUDA_TRY(cudaMemcpyAsync(host2, d, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  NLGB_CUDA_TRY(cudaStreamSynchronize(s));
  NLGB_CUDA_TRY(cudaFreeAsync(d, s));
  return cudaSuccess;
}

cudaError_t crs_prepare_df(DeviceCRS& A, bool* usable, cudaStream_t s) {
  NLGB_CUDA_TRY(crs_prepare(A, false, s));
  if (A.df_state == 0) {
    int rv[2], rd[2];
    NLGB_CUDA_TRY(exp_range(A.nnz, A.va, rv, s));
    NLGB_CUDA_TRY(exp_range(A.n, A.dinv, rd, s));
    const bool ok = rv[0] <= kDfMaxExp && rd[0] <= kDfMaxExp &&
                    (A.nnz == 0 || rv[1] >= kDfMinExp) && (A.n == 0 || rd[1] >= kDfMinExp);
    A.df_state = ok ? 1 : -1;
  }
  if (A.df_state > 0 && !A.vadf) {
    NLGB_CUDA_TRY(cudaMallocAsync(&A.vadf, (size_t)std::max(1LL, A.nnz) * sizeof(float2), s));
    NLGB_CUDA_TRY(cudaMallocAsync(&A.dinvdf, (size_t)std::max(1, A.n) * sizeof(float2), s));
    if (A.nnz > 0) {
      k_to_df<<<grid_for(A.nnz, 256), 256, 0, s>>>(A.nnz, A.va, A.vadf);
      count_launches(1);
    }
    if (A.n > 0) {
      k_to_df<<<grid_for(A.n, 256), 256, 0, s>>>(A.n, A.dinv, A.dinvdf);
      count_launches(1);
    }
    NLGB_CUDA_TRY(cudaGetLastError());
  }
  *usable = A.df_state > 0;
  return cudaSuccess;
}

cudaError_t df_pack(double* x, long long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_df_pack<<<grid_for(n, 256), 256, 0, s>>>(n, x);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t df_unpack(double* x, long long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_df_unpack<<<grid_for(n, 256), 256, 0, s>>>(n, x);
  count_launches(1);
  return cudaGetLastError();
}

template <typename V, typename X>
static cudaError_t spmv_dispatch(const DeviceCRS& A, const V* va, const X* x, X* y, cudaStream_t s) {
  if (A.n == 0) return cudaSuccess;
  const int tile = A.tile_rows > 0 ? A.tile_rows : 512;
  const int grid = (A.n + tile - 1) / tile;
  switch (A.tpr > 0 ? A.tpr : 4) {
    case 1: k_spmv<1, V, X><<<grid, kCTA, 0, s>>>(A.n, tile, A.rp, A.ci, va, x, y); break;
    case 2: k_spmv<2, V, X><<<grid, kCTA, 0, s>>>(A.n, tile, A.rp, A.ci, va, x, y); break;
    case 4: k_spmv<4, V, X><<<grid, kCTA, 0, s>>>(A.n, tile, A.rp, A.ci, va, x, y); break;
    case 8: k_spmv<8, V, X><<<grid, kCTA, 0, s>>>(A.n, tile, A.rp, A.ci, va, x, y); break;
    case 16: k_spmv<16, V, X><<<grid, kCTA, 0, s>>>(A.n, tile, A.rp, A.ci, va, x, y); break;
    default: k_spmv<32, V, X><<<grid, kCTA, 0, s>>>(A.n, tile, A.rp, A.ci, va, x, y); break;
  }
  count_launches(1);

  return cudaGetLastError();
}

cudaError_t spmv64(const DeviceCRS& A, const double* x, double* y, cudaStream_t s) {
  NLGB_CUDA_TRY((spmv_dispatch<double, double>(A, A.va, x, y, s)));
  return cudaSuccess;
}
cudaError_t spmv32(const DeviceCRS& A, const float* x, float* y, cudaStream_t s) {
  NLGB_CUDA_TRY((spmv_dispatch<float, float>(A, A.va32, x, y, s)));
  return cudaSuccess;
}

// --- graph construction helpers ---
// `dep` may be null (no dependency) or a node the new one runs after.
static cudaError_t add_kernel(cudaGraph_t g, cudaGraphNode_t* node, cudaGraphNode_t dep,
                              const void* fn, int grid, int block, void** args) {
  cudaKernelNodeParams kp;
  std::memset(&kp, 0, sizeof(kp));
  kp.func = const_cast<void*>(fn);
  kp.gridDim = dim3((unsigned)std::max(1, grid));
  kp.blockDim = dim3((unsigned)block);
  kp.sharedMemBytes = 0;
  kp.kernelParams = args;
  return cudaGraphAddKernelNode(node, g, dep ? &dep : nullptr, dep ? 1 : 0, &kp);
}

static cudaError_t add_cond(cudaGraph_t g, cudaGraphNode_t* node, cudaGraphNode_t dep,
                            cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                            cudaGraph_t* body) {
  alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)];
  std::memset(raw, 0, sizeof(raw));
  cudaGraphNodeParams* cp = reinterpret_cast<cudaGraphNodeParams*>(raw);
  cp->type = cudaGraphNodeTypeConditional;
  cp->conditional.handle = h;
  cp->conditional.type = type;
  cp->conditional.size = 1;
  cudaError_t e = cudaGraphAddNode(node, g, dep ? &dep : nullptr, nullptr, dep ? 1 : 0, cp);
  if (e != cudaSuccess) return e;
  *body = cp->conditional.phGraph_out[0];
  return cudaSuccess;
}

static cudaError_t add_while(cudaGraph_t g, cudaGraphNode_t* node, cudaGraphNode_t dep,
                             cudaGraphConditionalHandle h, cudaGraph_t* body) {
  return add_cond(g, node, dep, h, cudaGraphCondTypeWhile, body);
}

// The kernels of one threads-per-row variant; df selects the double-float
// form of the plain iteration (init, SpMV, vector updates, final residual).
struct KernelSet {
  const void *init, *spmv, *fin, *mx_outer, *mx_spmv, *iter, *update_xr, *update_p, *resume_p,
      *init_chunk, *fin_if;
};
template <int T, bool D>
static KernelSet kernel_set() {
  return {(const void*)k_init<T, D>, (const void*)k_spmv_pq<T, D>, (const void*)k_final<T, D>,
          (const void*)k_mx_outer<T>, (const void*)k_mx_spmv_pq<T>, (const void*)k_iter<T, D>,
          (const void*)k_update_xr<D>, (const void*)k_update_p<D>, (const void*)k_resume_p<D>,
          (const void*)k_init_chunk<T, D>, (const void*)k_final_if<T, D>};
}
template <bool D>
static KernelSet kernels_for_t(int tpr) {
  switch (tpr) {
    case 1: return kernel_set<1, D>();
    case 2: return kernel_set<2, D>();
    case 4: return kernel_set<4, D>();
    case 8: return kernel_set<8, D>();
    case 16: return kernel_set<16, D>();
    default: return kernel_set<32, D>();
  }
}
static KernelSet kernels_for(int tpr, bool df) {
  return df ? kernels_for_t<true>(tpr) : kernels_for_t<false>(tpr);
}

constexpr int kUnrollPlain = 4;   // CG iterations per while-body pass
constexpr int kCoopTilesPerCta = 1;   // measured: two tiles per CTA lose to three kernels
constexpr int kUnrollInner = 4;
constexpr long long kMaxItersBetweenUpdates = 1000;   // mixed: forced reliable update

PcgSolver::~PcgSolver() { release(); }

void PcgSolver::release() {
  if (plain_exec_) cudaGraphExecDestroy(plain_exec_);
  if (mixed_exec_) cudaGraphExecDestroy(mixed_exec_);
  if (df_exec_) cudaGraphExecDestroy(df_exec_);
  if (cont_exec_) cudaGraphExecDestroy(cont_exec_);
  if (cont_df_exec_) cudaGraphExecDestroy(cont_df_exec_);
  plain_exec_ = mixed_exec_ = df_exec_ = cont_exec_ = cont_df_exec_ = nullptr;
  cudaFree(b_); cudaFree(x_); cudaFree(r_); cudaFree(p_); cudaFree(q_); cudaFree(part_);
  cudaFree(coop_bar_);
  coop_bar_ = nullptr;
  cudaFree(r32_); cudaFree(p32_); cudaFree(q32_); cudaFree(c32_); cudaFree(st_);
  if (st_host_) cudaFreeHost(st_host_);
  if (ev0_) cudaEventDestroy(ev0_);
  if (ev1_) cudaEventDestroy(ev1_);
  b_ = x_ = r_ = p_ = q_ = part_ = nullptr;
  r32_ = p32_ = q32_ = c32_ = nullptr;
  st_ = st_host_ = nullptr;
  ev0_ = ev1_ = nullptr;
  mixed_alloc_ = false;
}

cudaError_t PcgSolver::bind(DeviceCRS* A, cudaStream_t stream) {
  release();
  A_ = A;
  stream_ = stream;
  n_ = A->n;
  tpr_ = A->tpr;
  tile_rows_ = A->tile_rows;
  n_tiles_ = std::max(1, (n_ + tile_rows_ - 1) / tile_rows_);
  // One cooperative kernel per iteration when the tiles fit in one resident
  // wave of it at no more than kCoopTilesPerCta tiles per CTA (latency-bound
  // sizes); larger systems keep one kernel per phase at full occupancy.
  int dev = 0, sms = 0, per_sm = 0;
  use_coop_ = false;
  if (cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
      (per_sm = coop_per_sm(tpr_)) > 0) {
    const long long wave = std::min<long long>((long long)per_sm * sms, kCoopMaxCtas);
    use_coop_ = n_tiles_ <= kCoopTilesPerCta * wave;
    coop_grid_ = (int)std::min<long long>(n_tiles_, wave);
  }
  cudaGetLastError();
  return alloc(false);
}

cudaError_t PcgSolver::alloc(bool mixed) {
  const size_t n8 = (size_t)std::max(2, n_ + 2) * sizeof(double);
  if (!x_) {
    NLGB_CUDA_TRY(cudaMalloc(&b_, n8));
    NLGB_CUDA_TRY(cudaMalloc(&x_, n8));
    NLGB_CUDA_TRY(cudaMalloc(&r_, n8));
    NLGB_CUDA_TRY(cudaMalloc(&p_, n8));
    NLGB_CUDA_TRY(cudaMalloc(&q_, n8));
    NLGB_CUDA_TRY(cudaMalloc(&part_, (size_t)n_tiles_ * kParts * sizeof(double)));
    NLGB_CUDA_TRY(cudaMalloc(&st_, sizeof(SysState)));
    NLGB_CUDA_TRY(cudaMallocHost(&st_host_, sizeof(SysState)));
    NLGB_CUDA_TRY(cudaEventCreate(&ev0_));
    NLGB_CUDA_TRY(cudaEventCreate(&ev1_));
    NLGB_CUDA_TRY(cudaMalloc(&coop_bar_, 256));
  }
  if (mixed && !mixed_alloc_) {
    const size_t n4 = (size_t)std::max(4, n_ + 4) * sizeof(float);
    NLGB_CUDA_TRY(cudaMalloc(&r32_, n4));
    NLGB_CUDA_TRY(cudaMalloc(&p32_, n4));
    NLGB_CUDA_TRY(cudaMalloc(&q32_, n4));
    NLGB_CUDA_TRY(cudaMalloc(&c32_, n4));
    mixed_alloc_ = true;
  }
  return cudaSuccess;
}

static SysView make_view(DeviceCRS* A, int tile_rows, int n_tiles, double* b, double* x, double* r,
                         double* p, double* q, float* r32, float* p32, float* q32, float* c32,
                         double* part, void* st, const volatile int* abort_flag, bool df = false) {
  SysView v;
  std::memset(&v, 0, sizeof(v));
  v.n = A->n; v.tile_rows = tile_rows; v.n_tiles = n_tiles; v.tpr = A->tpr;
  v.df = df ? 1 : 0;
  v.rp = A->rp; v.ci = A->ci; v.va = A->va; v.va32 = A->va32; v.vadf = A->vadf;
  v.dinv = A->dinv; v.dinv32 = A->dinv32; v.dinvdf = A->dinvdf;
  v.b = b; v.x = x; v.r = r; v.p = p; v.q = q;
  v.r32 = r32; v.p32 = p32; v.q32 = q32; v.c32 = c32;
  v.part = part; v.st = (SysState*)st; v.abort_flag = abort_flag;
  return v;
}

// The while loop of the plain (FP64 or double-float) iteration, after
// `dep`: kUnrollPlain iterations per pass (one cooperative kernel each, or
// three phase kernels), then the guard.
cudaError_t PcgSolver::add_plain_loop(cudaGraph_t g, cudaGraphNode_t dep, SysView* v, bool df,
                                      cudaGraphNode_t* loop_out) {
  const KernelSet ks = kernels_for(tpr_, df);
  cudaGraphConditionalHandle h;
  NLGB_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault));
  void* a1[] = {v};
  cudaGraph_t body;
  NLGB_CUDA_TRY(add_while(g, loop_out, dep, h, &body));
  cudaGraphNode_t prev = nullptr;
  unsigned long long* bar = coop_bar_;
  void* a_it[] = {v, &bar};
  for (int u = 0; u < kUnrollPlain; ++u) {
    if (use_coop_) {
      cudaGraphNode_t n1;
      NLGB_CUDA_TRY(add_kernel(body, &n1, prev, ks.iter, coop_grid_, kCTA, a_it));
      cudaKernelNodeAttrValue coop;
      std::memset(&coop, 0, sizeof(coop));
      coop.cooperative = 1;
      NLGB_CUDA_TRY(cudaGraphKernelNodeSetAttribute(n1, cudaKernelNodeAttributeCooperative, &coop));
      prev = n1;
      continue;
    }
    cudaGraphNode_t n1, n2, n3;
    NLGB_CUDA_TRY(add_kernel(body, &n1, prev, ks.spmv, n_tiles_, kCTA, a1));
    const int vg = (n_tiles_ + vec_tiles_for(tile_rows_) - 1) / vec_tiles_for(tile_rows_);
    NLGB_CUDA_TRY(add_kernel(body, &n2, n1, ks.update_xr, vg, kCTA, a1));
    NLGB_CUDA_TRY(add_kernel(body, &n3, n2, ks.update_p, vg, kCTA, a1));
    prev = n3;
  }
  int need_mode = -1, use_handle = 1;
  void* ag[] = {v, &h, &need_mode, &use_handle};
  cudaGraphNode_t n_g;
  NLGB_CUDA_TRY(add_kernel(body, &n_g, prev, (const void*)k_guard, 1, 1, ag));
  return cudaSuccess;
}

// init -> while { iterations ; guard } -> final residual -> true-residual
// check.  cont == true: the continuation after a failed check instead,
// resume p update -> mark -> while { ... } -> final residual -> check.
cudaError_t PcgSolver::build_plain_graph(bool df, bool cont) {
  SysView v = make_view(A_, tile_rows_, n_tiles_, b_, x_, r_, p_, q_, nullptr, nullptr, nullptr,
                        nullptr, part_, st_, abort_flag_, df);
  const KernelSet ks = kernels_for(tpr_, df);
  cudaGraph_t g;
  NLGB_CUDA_TRY(cudaGraphCreate(&g, 0));
  void* a1[] = {&v};
  SysState* st = (SysState*)st_;
  void* ast[] = {&st};
  const int vg = (n_tiles_ + vec_tiles_for(tile_rows_) - 1) / vec_tiles_for(tile_rows_);
  cudaGraphNode_t n_first, n_loop, n_fin, n_chk;
  if (cont) {
    cudaGraphNode_t n_res;
    NLGB_CUDA_TRY(add_kernel(g, &n_res, nullptr, ks.resume_p, vg, kCTA, a1));
    NLGB_CUDA_TRY(add_kernel(g, &n_first, n_res, (const void*)k_resume_mark, 1, 1, ast));
  } else {
    NLGB_CUDA_TRY(add_kernel(g, &n_first, nullptr, ks.init, n_tiles_, kCTA, a1));
  }
  cudaError_t e = add_plain_loop(g, n_first, &v, df, &n_loop);
  if (e == cudaSuccess) e = add_kernel(g, &n_fin, n_loop, ks.fin, n_tiles_, kCTA, a1);
  if (e == cudaSuccess) e = add_kernel(g, &n_chk, n_fin, (const void*)k_check, 1, 1, ast);
  cudaGraphExec_t* out = cont ? (df ? &cont_df_exec_ : &cont_exec_) : (df ? &df_exec_ : &plain_exec_);
  if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  NLGB_CUDA_TRY(e);
  return cudaSuccess;
}

cudaError_t PcgSolver::build_mixed_graph() {
  SysView v = make_view(A_, tile_rows_, n_tiles_, b_, x_, r_, p_, q_, r32_, p32_, q32_, c32_,
                        part_, st_, abort_flag_);
  const KernelSet ks = kernels_for(tpr_, false);
  // [initial FP64 residual] -> while { ( p update ; q = A32 p, p.q ;
  //   c/r update -> IF(update due) { x += c ; FP64 residual } ) x U ; guard }
  // -> final FP64 residual.
  cudaGraph_t g;
  NLGB_CUDA_TRY(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle h_loop;
  NLGB_CUDA_TRY(cudaGraphConditionalHandleCreate(&h_loop, g, 1u, cudaGraphCondAssignDefault));
  void* a1[] = {&v};
  cudaGraphNode_t n_first, n_loop, n_fin;
  NLGB_CUDA_TRY(add_kernel(g, &n_first, nullptr, ks.mx_outer, n_tiles_, kCTA, a1));
  cudaGraph_t body;
  NLGB_CUDA_TRY(add_while(g, &n_loop, n_first, h_loop, &body));
  cudaGraphNode_t prev = nullptr;
  cudaGraphConditionalHandle h_upd[kUnrollInner];
  for (int u = 0; u < kUnrollInner; ++u) {
    NLGB_CUDA_TRY(cudaGraphConditionalHandleCreate(&h_upd[u], body, 0u, cudaGraphCondAssignDefault));
    cudaGraphNode_t n1, n2, n3, n_if, n4, n5;
    const int vg = (n_tiles_ + vec_tiles_for(tile_rows_) - 1) / vec_tiles_for(tile_rows_);
    NLGB_CUDA_TRY(add_kernel(body, &n1, prev, (const void*)k_mx_update_p, vg, kCTA, a1));
    NLGB_CUDA_TRY(add_kernel(body, &n2, n1, ks.mx_spmv, n_tiles_, kCTA, a1));
    int use_handle = 1;
    void* acr[] = {&v, &h_upd[u], &use_handle};
    NLGB_CUDA_TRY(add_kernel(body, &n3, n2, (const void*)k_mx_update_cr, vg, kCTA, acr));
    cudaGraph_t ubody;
    NLGB_CUDA_TRY(add_cond(body, &n_if, n3, h_upd[u], cudaGraphCondTypeIf, &ubody));
    NLGB_CUDA_TRY(add_kernel(ubody, &n4, nullptr, (const void*)k_mx_apply, vg, kCTA, a1));
    NLGB_CUDA_TRY(add_kernel(ubody, &n5, n4, ks.mx_outer, n_tiles_, kCTA, a1));
    prev = n_if;
  }
  int need_any = -1, use_handle = 1;
  void* ag[] = {&v, &h_loop, &need_any, &use_handle};
  cudaGraphNode_t n_g;
  NLGB_CUDA_TRY(add_kernel(body, &n_g, prev, (const void*)k_guard, 1, 1, ag));
  NLGB_CUDA_TRY(add_kernel(g, &n_fin, n_loop, ks.fin, n_tiles_, kCTA, a1));
  cudaError_t e = cudaGraphInstantiate(&mixed_exec_, g, 0);
  cudaGraphDestroy(g);
  NLGB_CUDA_TRY(e);
  return cudaSuccess;
}

static bool eager_mode();

// ---------------------------------------------------------------------------
// ViewGraph: resumable PCG chunks of a system whose buffers and state live
// elsewhere (a SystemSlot of the server or of the persistent solver).  The
// kernels and their order are those of the single-system graphs, so a
// system's iterates do not depend on where a chunk ends, on other systems
// running concurrently on other streams, or on switching between this
// executor and the persistent kernel:
//   FP64 / double-float:  initial residual (stage 0 only) -> resume p update
//     (stage 4 only) -> while { (q = A p, p.q ; x, r ; p) x 4 ; guard } ->
//     final residual (if the system stopped) -> true-residual check -> end;
//   mixed:  initial FP64 residual (fresh system only) -> mark started ->
//     while { (p ; q = A32 p, p.q ; c, r -> IF(update due) { x += c ; FP64
//     residual }) x 4 ; guard } -> final residual (if stopped) -> end.
// A chunk pauses on whole passes of 4 iterations (guard), the system stays
// running; the server continues it with another chunk later.
// ---------------------------------------------------------------------------
ViewGraph::~ViewGraph() {
  if (exec_) cudaGraphExecDestroy(exec_);
  if (e0_) cudaEventDestroy(e0_);
  if (e1_) cudaEventDestroy(e1_);
}

cudaError_t ViewGraph::build(const SysView& v, bool mixed) {
  if (exec_) cudaGraphExecDestroy(exec_);
  exec_ = nullptr;
  if (!e0_) NLGB_CUDA_TRY(cudaEventCreate(&e0_));
  if (!e1_) NLGB_CUDA_TRY(cudaEventCreate(&e1_));
  view_ = v;
  mixed_ = mixed;
  const KernelSet ks = kernels_for(v.tpr, !mixed && v.df != 0);
  cudaGraph_t g;
  NLGB_CUDA_TRY(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle h;
  NLGB_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault));
  void* a1[] = {&view_};
  SysState* st = v.st;
  void* ae[] = {&st};
  const int vg = (v.n_tiles + vec_tiles_for(v.tile_rows) - 1) / vec_tiles_for(v.tile_rows);
  cudaGraphNode_t n_start, n_loop, n_fin, n_end, prev = nullptr, n_first = nullptr;
  cudaGraph_t body;
  ChunkMirror* mirror = mirror_;
  int unroll = kUnrollPlain;
  void* am[] = {&st, &mirror, &unroll};
  if (mirror_) NLGB_CUDA_TRY(add_kernel(g, &n_first, nullptr, (const void*)k_chunk_start_m, 1, 1, am));
  if (!mixed) {
    cudaGraphNode_t n_init, n_res;
    NLGB_CUDA_TRY(add_kernel(g, &n_init, n_first, ks.init_chunk, v.n_tiles, kCTA, a1));
    NLGB_CUDA_TRY(add_kernel(g, &n_res, n_init, ks.resume_p, vg, kCTA, a1));
    NLGB_CUDA_TRY(add_kernel(g, &n_start, n_res, (const void*)k_resume_mark, 1, 1, ae));
    NLGB_CUDA_TRY(add_while(g, &n_loop, n_start, h, &body));
    for (int u = 0; u < kUnrollPlain; ++u) {
      cudaGraphNode_t n1, n2, n3;
      NLGB_CUDA_TRY(add_kernel(body, &n1, prev, ks.spmv, v.n_tiles, kCTA, a1));
      NLGB_CUDA_TRY(add_kernel(body, &n2, n1, ks.update_xr, vg, kCTA, a1));
      NLGB_CUDA_TRY(add_kernel(body, &n3, n2, ks.update_p, vg, kCTA, a1));
      prev = n3;
    }
  } else {
    cudaGraphNode_t n_outer;
    NLGB_CUDA_TRY(add_kernel(g, &n_outer, n_first, ks.mx_outer, v.n_tiles, kCTA, a1));
    NLGB_CUDA_TRY(add_kernel(g, &n_start, n_outer, (const void*)k_mark_started, 1, 1, ae));
    NLGB_CUDA_TRY(add_while(g, &n_loop, n_start, h, &body));
    for (int u = 0; u < kUnrollInner; ++u) {
      cudaGraphConditionalHandle h_upd;
      NLGB_CUDA_TRY(cudaGraphConditionalHandleCreate(&h_upd, body, 0u, cudaGraphCondAssignDefault));
      cudaGraphNode_t n1, n2, n3, n_if, n4, n5;
      NLGB_CUDA_TRY(add_kernel(body, &n1, prev, (const void*)k_mx_update_p, vg, kCTA, a1));
      NLGB_CUDA_TRY(add_kernel(body, &n2, n1, ks.mx_spmv, v.n_tiles, kCTA, a1));
      int use_handle = 1;
      void* acr[] = {&view_, &h_upd, &use_handle};
      NLGB_CUDA_TRY(add_kernel(body, &n3, n2, (const void*)k_mx_update_cr, vg, kCTA, acr));
      cudaGraph_t ubody;
      NLGB_CUDA_TRY(add_cond(body, &n_if, n3, h_upd, cudaGraphCondTypeIf, &ubody));
      NLGB_CUDA_TRY(add_kernel(ubody, &n4, nullptr, (const void*)k_mx_apply, vg, kCTA, a1));
      NLGB_CUDA_TRY(add_kernel(ubody, &n5, n4, ks.mx_outer, v.n_tiles, kCTA, a1));
      prev = n_if;
    }
  }
  int need_mode = -1, use_handle = 1;
  void* ag[] = {&view_, &h, &need_mode, &use_handle};
  cudaGraphNode_t n_g;
  NLGB_CUDA_TRY(add_kernel(body, &n_g, prev, (const void*)k_guard, 1, 1, ag));
  NLGB_CUDA_TRY(add_kernel(g, &n_fin, n_loop, ks.fin_if, v.n_tiles, kCTA, a1));
  if (!mixed) {
    cudaGraphNode_t n_chk;
    NLGB_CUDA_TRY(add_kernel(g, &n_chk, n_fin, (const void*)k_check, 1, 1, ae));
    n_fin = n_chk;
  }
  if (mirror_) {
    void* aem[] = {&st, &mirror};
    NLGB_CUDA_TRY(add_kernel(g, &n_end, n_fin, (const void*)k_chunk_end_m, 1, 32, aem));
  } else {
    NLGB_CUDA_TRY(add_kernel(g, &n_end, n_fin, (const void*)k_chunk_end, 1, 1, ae));
  }
  cudaError_t e = cudaGraphInstantiate(&exec_, g, 0);
  cudaGraphDestroy(g);
  NLGB_CUDA_TRY(e);
  return cudaSuccess;
}

// Everything the graph embeds: a slot freed and reallocated from the
// stream-ordered pool may return the same state and vector addresses for a
// different matrix, so every pointer and size is compared.
static bool same_view(const SysView& a, const SysView& b) {
  return a.n == b.n && a.tile_rows == b.tile_rows && a.n_tiles == b.n_tiles && a.tpr == b.tpr &&
         a.df == b.df && a.vadf == b.vadf && a.dinvdf == b.dinvdf &&
         a.rp == b.rp && a.ci == b.ci && a.va == b.va && a.dinv == b.dinv && a.b == b.b &&
         a.x == b.x && a.r == b.r && a.p == b.p && a.q == b.q && a.part == b.part && a.st == b.st &&
         a.va32 == b.va32 && a.dinv32 == b.dinv32 && a.r32 == b.r32 && a.p32 == b.p32 &&
         a.q32 == b.q32 && a.c32 == b.c32 && a.abort_flag == b.abort_flag;
}

cudaError_t ViewGraph::prepare(const SysView& v, bool mixed) { return prepare(v, mixed, nullptr); }

cudaError_t ViewGraph::prepare(const SysView& v, bool mixed, ChunkMirror* m, cudaStream_t upload) {
  if (!exec_ || mixed != mixed_ || m != mirror_ || !same_view(v, view_)) {
    mirror_ = m;
    NLGB_CUDA_TRY(build(v, mixed));
    if (upload) NLGB_CUDA_TRY(cudaGraphUpload(exec_, upload));
  }
  return cudaSuccess;
}

cudaError_t ViewGraph::launch(cudaStream_t s) {
  if (!mirror_) return cudaErrorInvalidValue;
  if (eager_mode()) {
    k_chunk_start_m<<<1, 1, 0, s>>>(view_.st, mirror_, kUnrollPlain);
    NLGB_CUDA_TRY(cudaGetLastError());
    const long long budget = *reinterpret_cast<volatile long long*>(&mirror_->budget);
    return run_eager(s, budget > 0 ? budget : 1);
  }
  if (!exec_) return cudaErrorInvalidValue;
  return cudaGraphLaunch(exec_, s);
}

void ViewGraph::account(long long iters_before, long long iters_after) {
  if (eager_counted_) {   // run_eager counted its launches (plus the chunk start)
    eager_counted_ = false;
    count_launches(1);
    return;
  }
  const long long passes = (std::max(0LL, iters_after - iters_before) + kUnrollPlain - 1) / kUnrollPlain;
  count_launches((mixed_ ? 5 : 7) + std::max(1LL, passes) * (3LL * kUnrollPlain + 1));
}

cudaError_t ViewGraph::run(const SysView& v, long long iters, cudaStream_t s, float* ms, bool mixed) {
  if (!eager_mode()) NLGB_CUDA_TRY(prepare(v, mixed));
  else { view_ = v; mixed_ = mixed; }
  if (!e0_) NLGB_CUDA_TRY(cudaEventCreate(&e0_));
  if (!e1_) NLGB_CUDA_TRY(cudaEventCreate(&e1_));
  NLGB_CUDA_TRY(cudaEventRecord(e0_, s));
  k_chunk_start<<<1, 1, 0, s>>>(v.st, std::max(1LL, iters), kUnrollPlain);
  NLGB_CUDA_TRY(cudaGetLastError());
  if (eager_mode()) {
    NLGB_CUDA_TRY(run_eager(s, iters));
  } else {
    NLGB_CUDA_TRY(cudaGraphLaunch(exec_, s));
  }
  NLGB_CUDA_TRY(cudaEventRecord(e1_, s));
  pending_ = true;
  ms_ = ms;
  return cudaSuccess;
}

cudaError_t chunk_fallback_fp64(SysState* st, cudaStream_t s) {
  k_fallback_fp64<<<1, 1, 0, s>>>(st);
  count_launches(1);
  return cudaGetLastError();
}

bool ViewGraph::done() const {
  if (!pending_) return true;
  return cudaEventQuery(e1_) != cudaErrorNotReady;
}

// Eager mode: the chunk's kernels launched one by one (profiling only).
cudaError_t ViewGraph::run_eager(cudaStream_t s, long long iters) {
  const KernelSet ks = kernels_for(view_.tpr, !mixed_ && view_.df != 0);
  const int vg = (view_.n_tiles + vec_tiles_for(view_.tile_rows) - 1) / vec_tiles_for(view_.tile_rows);
  const cudaGraphConditionalHandle none = 0;
  const int need = -1, no_handle = 0;
  void* a1[] = {&view_};
  void* ag[] = {&view_, const_cast<cudaGraphConditionalHandle*>(&none), const_cast<int*>(&need),
                const_cast<int*>(&no_handle)};
  void* acr[] = {&view_, const_cast<cudaGraphConditionalHandle*>(&none), const_cast<int*>(&no_handle)};
  SysState* st = view_.st;
  void* ae[] = {&st};
  int status = ST_RUNNING;
  long long launched = 0;
  auto go = [&](const void* fn, int grid, int block, void** args) {
    ++launched;
    return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, 0, s);
  };
  if (!mixed_) {
    NLGB_CUDA_TRY(go(ks.init_chunk, view_.n_tiles, kCTA, a1));
    NLGB_CUDA_TRY(go(ks.resume_p, vg, kCTA, a1));
    NLGB_CUDA_TRY(go((const void*)k_resume_mark, 1, 1, ae));
  } else {
    NLGB_CUDA_TRY(go(ks.mx_outer, view_.n_tiles, kCTA, a1));
    NLGB_CUDA_TRY(go((const void*)k_mark_started, 1, 1, ae));
  }
  NLGB_CUDA_TRY(cudaMemcpyAsync(&status, &st->status, sizeof(int), cudaMemcpyDeviceToHost, s));
  NLGB_CUDA_TRY(cudaStreamSynchronize(s));
  for (long long pass = 0; pass * kUnrollPlain < std::max(1LL, iters) && status == ST_RUNNING; ++pass) {
    for (int u = 0; u < kUnrollPlain; ++u) {
      if (!mixed_) {
        NLGB_CUDA_TRY(go(ks.spmv, view_.n_tiles, kCTA, a1));
        NLGB_CUDA_TRY(go(ks.update_xr, vg, kCTA, a1));
        NLGB_CUDA_TRY(go(ks.update_p, vg, kCTA, a1));
      } else {
        NLGB_CUDA_TRY(go((const void*)k_mx_update_p, vg, kCTA, a1));
        NLGB_CUDA_TRY(go(ks.mx_spmv, view_.n_tiles, kCTA, a1));
        NLGB_CUDA_TRY(go((const void*)k_mx_update_cr, vg, kCTA, acr));
        NLGB_CUDA_TRY(go((const void*)k_mx_apply, vg, kCTA, a1));   // return unless an update is due
        NLGB_CUDA_TRY(go(ks.mx_outer, view_.n_tiles, kCTA, a1));
      }
    }
    NLGB_CUDA_TRY(go((const void*)k_guard, 1, 1, ag));
    NLGB_CUDA_TRY(cudaMemcpyAsync(&status, &st->status, sizeof(int), cudaMemcpyDeviceToHost, s));
    NLGB_CUDA_TRY(cudaStreamSynchronize(s));
  }
  NLGB_CUDA_TRY(go(ks.fin_if, view_.n_tiles, kCTA, a1));
  if (!mixed_) NLGB_CUDA_TRY(go((const void*)k_check, 1, 1, ae));
  if (mirror_) {
    ChunkMirror* mirror = mirror_;
    void* aem[] = {&st, &mirror};
    NLGB_CUDA_TRY(go((const void*)k_chunk_end_m, 1, 32, aem));
  } else {
    NLGB_CUDA_TRY(go((const void*)k_chunk_end, 1, 1, ae));
  }
  count_launches(launched);
  eager_counted_ = true;
  return cudaSuccess;
}

cudaError_t ViewGraph::finish(long long iters_before, long long iters_after) {
  if (!pending_) return cudaSuccess;
  pending_ = false;
  NLGB_CUDA_TRY(cudaEventSynchronize(e1_));
  if (ms_) NLGB_CUDA_TRY(cudaEventElapsedTime(ms_, e0_, e1_));
  // kernels executed: chunk start and end, the fixed nodes before and after
  // the loop, and per while-body pass 3 kernels per unrolled iteration + the
  // guard (mixed: + 2 per reliable update, counted as passes x 1 here)
  account(iters_before, iters_after);
  return cudaSuccess;
}

// Eager mode (environment NLGB_EAGER_SOLVE=1, read at every solve): the
// same kernels as the graphs, launched one by one from a host loop that
// reads the status after every unrolled pass.  Slower (one host round trip
// per pass); it exists so that profilers and launch lists, which do not
// descend into conditional graph nodes, see every kernel of an iteration.
static bool eager_mode() {
  const char* e = std::getenv("NLGB_EAGER_SOLVE");
  return e != nullptr && e[0] == '1';
}

cudaError_t PcgSolver::run_eager(bool mixed, bool df, SysState* h, bool cont) {
  SysView v = make_view(A_, tile_rows_, n_tiles_, b_, x_, r_, p_, q_, r32_, p32_, q32_, c32_,
                        part_, st_, abort_flag_, df && !mixed);
  const KernelSet ks = kernels_for(tpr_, df && !mixed);
  const int vg = (n_tiles_ + vec_tiles_for(tile_rows_) - 1) / vec_tiles_for(tile_rows_);
  const cudaGraphConditionalHandle none = 0;
  const int need = -1, no_handle = 0;
  long long launched = 0;
  auto go = [&](const void* fn, int grid, int block, void** args) {
    ++launched;
    return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, 0, stream_);
  };
  void* a1[] = {&v};
  void* ag[] = {&v, const_cast<cudaGraphConditionalHandle*>(&none), const_cast<int*>(&need),
                const_cast<int*>(&no_handle)};
  void* acr[] = {&v, const_cast<cudaGraphConditionalHandle*>(&none), const_cast<int*>(&no_handle)};
  SysState* st = (SysState*)st_;
  void* ast[] = {&st};
  if (cont) {
    NLGB_CUDA_TRY(go(ks.resume_p, vg, kCTA, a1));
    NLGB_CUDA_TRY(go((const void*)k_resume_mark, 1, 1, ast));
  } else {
    NLGB_CUDA_TRY(go(mixed ? ks.mx_outer : ks.init, n_tiles_, kCTA, a1));
  }
  while (true) {
    for (int u = 0; u < (mixed ? kUnrollInner : kUnrollPlain); ++u) {
      if (mixed) {
        NLGB_CUDA_TRY(go((const void*)k_mx_update_p, vg, kCTA, a1));
        NLGB_CUDA_TRY(go(ks.mx_spmv, n_tiles_, kCTA, a1));
        NLGB_CUDA_TRY(go((const void*)k_mx_update_cr, vg, kCTA, acr));
        NLGB_CUDA_TRY(go((const void*)k_mx_apply, vg, kCTA, a1));   // return unless an update is due
        NLGB_CUDA_TRY(go(ks.mx_outer, n_tiles_, kCTA, a1));
      } else {
        NLGB_CUDA_TRY(go(ks.spmv, n_tiles_, kCTA, a1));
        NLGB_CUDA_TRY(go(ks.update_xr, vg, kCTA, a1));
        NLGB_CUDA_TRY(go(ks.update_p, vg, kCTA, a1));
      }
    }
    NLGB_CUDA_TRY(go((const void*)k_guard, 1, 1, ag));
    NLGB_CUDA_TRY(cudaMemcpyAsync(h, st_, sizeof(SysState), cudaMemcpyDeviceToHost, stream_));
    NLGB_CUDA_TRY(cudaStreamSynchronize(stream_));
    if (h->status != ST_RUNNING) break;
  }
  NLGB_CUDA_TRY(go(ks.fin, n_tiles_, kCTA, a1));
  if (!mixed) NLGB_CUDA_TRY(go((const void*)k_check, 1, 1, ast));
  count_launches(launched);
  return cudaSuccess;
}

cudaError_t PcgSolver::run_cont(bool df, float* ms) {
  cudaGraphExec_t* ex = df ? &cont_df_exec_ : &cont_exec_;
  if (!eager_mode() && !*ex) NLGB_CUDA_TRY(build_plain_graph(df, true));
  SysState* h = (SysState*)st_host_;
  const long long guard0 = h->guard;
  NLGB_CUDA_TRY(cudaEventRecord(ev0_, stream_));
  if (eager_mode()) {
    NLGB_CUDA_TRY(run_eager(false, df, h, true));
  } else {
    NLGB_CUDA_TRY(cudaGraphLaunch(*ex, stream_));
  }
  NLGB_CUDA_TRY(cudaEventRecord(ev1_, stream_));
  NLGB_CUDA_TRY(cudaMemcpyAsync(h, st_, sizeof(SysState), cudaMemcpyDeviceToHost, stream_));
  NLGB_CUDA_TRY(cudaStreamSynchronize(stream_));
  NLGB_CUDA_TRY(cudaEventElapsedTime(ms, ev0_, ev1_));
  if (eager_mode()) return cudaSuccess;   // run_eager counted its launches
  ++graph_launches_;
  // resume p update, mark, final residual, check + every while-body pass
  const long long per_iter = use_coop_ ? 1 : 3;
  count_launches(4 + (h->guard - guard0) * (per_iter * kUnrollPlain + 1));
  return cudaSuccess;
}

// Runs one graph (mixed, plain FP64 or plain double-float: df) on the
// internal b_ / x_ (x_ already packed as double-float for df); `done` > 0
// continues a mixed solve that fell back to FP64 after `done` iterations.
// Leaves the final state in st_host_.
cudaError_t PcgSolver::run_graph(bool mixed, bool df, const SolveParams& prm, long long max_iter,
                                 long long done, int outer, float* ms) {
  if (mixed) df = false;
  cudaGraphExec_t* plain = df ? &df_exec_ : &plain_exec_;
  if (mixed && !mixed_exec_) NLGB_CUDA_TRY(build_mixed_graph());
  if (!mixed && !*plain) {
    cudaError_t e = build_plain_graph(df);
    if (e != cudaSuccess && use_coop_) {
      // cooperative kernel nodes refused here: one kernel per phase instead
      // (both plain graphs are rebuilt so that they keep one executor)
      cudaGetLastError();
      use_coop_ = false;
      if (plain_exec_) cudaGraphExecDestroy(plain_exec_);
      if (df_exec_) cudaGraphExecDestroy(df_exec_);
      if (cont_exec_) cudaGraphExecDestroy(cont_exec_);
      if (cont_df_exec_) cudaGraphExecDestroy(cont_df_exec_);
      plain_exec_ = df_exec_ = cont_exec_ = cont_df_exec_ = nullptr;
      e = build_plain_graph(df);
    }
    NLGB_CUDA_TRY(e);
  }
  SysState* h = (SysState*)st_host_;
  std::memset(h, 0, sizeof(SysState));
  h->thresh2 = prm.eps * prm.eps;
  h->max_iter = max_iter;
  h->status = ST_RUNNING;
  h->mode = 0;
  h->max_outer = std::max(1, prm.max_outer);
  h->in_thresh2 = prm.inner_eps * prm.inner_eps;
  // a reliable update at least every kMaxItersBetweenUpdates iterations
  h->in_max = (int)std::max(1LL, std::min<long long>(max_iter, kMaxItersBetweenUpdates));
  h->precision = mixed ? 1 : 0;
  h->iter = done;
  h->outer = outer;
  h->fell_back = done > 0 || outer > 0 ? 1 : 0;
  h->iter_at_fallback = done;
  // Hard cap on while-body passes: enough for max_iter iterations plus the
  // outer steps; reached only if the scalar logic failed to stop the loop.
  const int unroll = mixed ? kUnrollInner : kUnrollPlain;
  h->guard_cap = std::max(0LL, max_iter - done) / unroll + 2LL * (h->max_outer + 2) + 4;
  NLGB_CUDA_TRY(cudaMemcpyAsync(st_, h, sizeof(SysState), cudaMemcpyHostToDevice, stream_));
  NLGB_CUDA_TRY(cudaMemsetAsync(coop_bar_, 0, sizeof(unsigned long long), stream_));   // coop_epoch = 0 too
  if (mixed) {
    NLGB_CUDA_TRY(cudaMemsetAsync(c32_, 0, (size_t)n_ * sizeof(float), stream_));
    NLGB_CUDA_TRY(cudaMemsetAsync(p32_, 0, (size_t)n_ * sizeof(float), stream_));
  }
  NLGB_CUDA_TRY(cudaEventRecord(ev0_, stream_));
  if (eager_mode()) {
    NLGB_CUDA_TRY(run_eager(mixed, df, h));
  } else {
    NLGB_CUDA_TRY(cudaGraphLaunch(mixed ? mixed_exec_ : *plain, stream_));
  }
  NLGB_CUDA_TRY(cudaEventRecord(ev1_, stream_));
  NLGB_CUDA_TRY(cudaMemcpyAsync(h, st_, sizeof(SysState), cudaMemcpyDeviceToHost, stream_));
  NLGB_CUDA_TRY(cudaStreamSynchronize(stream_));
  NLGB_CUDA_TRY(cudaEventElapsedTime(ms, ev0_, ev1_));
  if (eager_mode()) return cudaSuccess;   // run_eager counted its launches
  ++graph_launches_;
  // Kernel nodes executed: every while-body pass runs all of its kernels
  // (3 per unrolled iteration + the guard); the mixed graph adds 2 kernels
  // per reliable update after the first; plus the first and final kernels
  // (and the true-residual check of the plain graph).
  const long long passes = h->guard;
  const long long per_iter = (!mixed && use_coop_) ? 1 : 3;
  long long k = (mixed ? 2 : 3) + passes * (per_iter * unroll + 1);
  if (mixed) k += 2LL * std::max(0, h->outer - outer - 1);
  count_launches(k);
  return cudaSuccess;
}

cudaError_t PcgSolver::solve(const double* b, double* x, const SolveParams& prm, SolveResult* res) {
  const bool mixed = prm.precision == 1;
  bool df = false;
  if (mixed) {
    NLGB_CUDA_TRY(crs_prepare(*A_, true, stream_));
    NLGB_CUDA_TRY(alloc(true));
  } else if (prm.precision == 3) {
    NLGB_CUDA_TRY(crs_prepare_df(*A_, &df, stream_));   // false: out of range, FP64 runs
  }
  const long long max_iter = prm.max_iter >= 0 ? prm.max_iter : 5LL * n_;
  NLGB_CUDA_TRY(cudaMemcpyAsync(b_, b, (size_t)n_ * sizeof(double), cudaMemcpyDeviceToDevice, stream_));
  NLGB_CUDA_TRY(cudaMemcpyAsync(x_, x, (size_t)n_ * sizeof(double), cudaMemcpyDeviceToDevice, stream_));
  if (df) NLGB_CUDA_TRY(df_pack(x_, n_, stream_));
  float ms = 0.f;
  SysState* h = (SysState*)st_host_;
  // An FP64 / double-float stop whose true residual missed eps leaves the
  // state running (k_check): continue the recurrence until it passes or
  // stalls (at most kMaxTrueChecks continuations).
  auto continue_checks = [&](bool dfc) -> cudaError_t {
    for (int c = 0; c <= kMaxTrueChecks && h->status == ST_RUNNING; ++c) {
      float m = 0.f;
      NLGB_CUDA_TRY(run_cont(dfc, &m));
      ms += m;
    }
    return cudaSuccess;
  };
  NLGB_CUDA_TRY(run_graph(mixed, df, prm, max_iter, 0, 0, &ms));
  if (!mixed) NLGB_CUDA_TRY(continue_checks(df));
  if (df) NLGB_CUDA_TRY(df_unpack(x_, n_, stream_));
  if (mixed && h->status == ST_STAGNATION && !h->fell_back) {
    // FP32 cannot track this system (kappa * u32 ~ 1): continue it with the
    // FP64 PCG from the current x, keeping the iteration count.
    const long long done = h->iter;
    const int outer = h->outer;
    float ms2 = 0.f;
    NLGB_CUDA_TRY(run_graph(false, false, prm, max_iter, done, outer, &ms2));
    ms += ms2;
    NLGB_CUDA_TRY(continue_checks(false));
  }
  NLGB_CUDA_TRY(cudaMemcpyAsync(x, x_, (size_t)n_ * sizeof(double), cudaMemcpyDeviceToDevice, stream_));
  NLGB_CUDA_TRY(cudaStreamSynchronize(stream_));
  if (res) {
    res->status = h->status;
    res->iterations = h->iter;
    res->outer_steps = h->outer;
    const double bb = h->bnorm2;
    res->rel_residual = bb > 0 ? std::sqrt(h->rr / bb) : 0.0;
    res->true_rel_residual = bb > 0 ? std::sqrt(h->rr_true / bb) : 0.0;
    res->seconds = ms * 1e-3;
    res->algo_bytes = algo_bytes(n_, A_->nnz, *h);
    res->precision = mixed ? 1 : (df ? 3 : 0);
  }
  return cudaSuccess;
}

}  // namespace nlgb
