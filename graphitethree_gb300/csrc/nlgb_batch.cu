// nlgb_batch.cu -- many independent Jacobi-PCG systems in one persistent
// kernel launch (plain FP64 or mixed FP32/FP64 per system).
//
// Reference context: geogram's mesh_make_atlas solves one LSCM system per
// chart, one after another, each through nlSolve (called from
// src/lib/OGF/mesh/commands/mesh_grob_surface_commands.cpp:724); a GPU that
// runs them one at a time is launch- and latency-bound on the small charts.
//
// Layout of one launch (grid = every co-resident CTA, cooperative launch):
//   * large systems are run by "teams" of k CTAs; a team synchronises its
//     phases with a global-memory barrier (bounded spin, then an error flag),
//     runs the system it was planned for, then draws further large systems
//     from a shared team queue (largest first) until it is empty;
//   * every other CTA is a queue worker: it pops the next small system from
//     an atomic queue and runs it alone (phases separated by __syncthreads).
// Each system's iteration is the same sequence of tile procedures and scalar
// steps as the single-system solver (nlgb_solver.cu), with the same tiles
// and the same canonical reductions, so a system's iterates do not depend on
// the team size, on the other systems in the launch or on where an epoch
// boundary falls: a result is bit-identical alone and in any mix.
// Every CTA of a team computes the scalars redundantly from the tile
// partials; rank 0 stores the system state back to HBM.
#include "nlgb_batch.h"
#include "nlgb_core.cuh"
#include "nlgb_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>

namespace nlgb {

namespace {

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}


// Barriers this CTA has completed in the current launch (set to 0 at kernel
// start; every CTA of a team passes the same sequence of barriers).
__shared__ unsigned long long s_bar_epoch;
// Limit of one barrier wait (BatchArgs::barrier_timeout_ns, 4 s by default),
// after which the CTA sets the launch's error flag and returns.
__shared__ unsigned long long s_bar_timeout_ns;
// Time box: the CTA's deadline on the GPU clock (0: none) and the stop
// decision of the current iteration of its system.
__shared__ unsigned long long s_deadline;
__shared__ int s_stop;

// Start of an iteration: the team's rank 0 decides whether the time box is
// used up and publishes the answer before the iteration's first barrier (a
// single CTA keeps it in shared memory).
__device__ __forceinline__ void stop_probe(TeamBar* bar, int k, int r) {
  if (s_deadline == 0ULL || r != 0 || threadIdx.x != 0) return;
  const int late = globaltimer_ns() > s_deadline ? 1 : 0;
  if (k > 1) *((volatile unsigned long long*)&bar->stop.count) = (unsigned long long)late;
  else s_stop = late;
}
// Thread 0, after the iteration's first barrier: every CTA of the team reads
// rank 0's decision (the writer passes the barrier's release before any
// reader's acquire; the next write comes after the iteration's last barrier,
// which every reader passes after reading).
__device__ __forceinline__ void stop_read(TeamBar* bar, int k) {
  if (s_deadline != 0ULL && k > 1) s_stop = (int)*((volatile unsigned long long*)&bar->stop.count);
}

__device__ __forceinline__ unsigned long long atom_add_acq_rel(unsigned long long* p, unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
  return old;
}

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Team barrier.  k == 1: a CTA barrier.  Returns false (in every thread) if
// the wait timed out or another CTA already flagged an error.  r: rank of
// this CTA in the team.  The __syncthreads before the arrival orders the
// CTA's writes before thread 0's release; thread 0's acquire and the
// __syncthreads after the wait order the other CTAs' writes before this
// CTA's next reads (which go through L2: __ldcg).
__device__ __noinline__ bool team_sync(TeamBar* bar, int k, int r, int* err) {
  if (k == 1) {
    __syncthreads();
    return true;
  }
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    const unsigned long long e = s_bar_epoch + 1;
    s_bar_epoch = e;
    unsigned long long target;
    if (k <= kBarFlat) {
      atom_add_acq_rel(&bar->top.count, 1ULL);
      target = e * (unsigned long long)k;
    } else {
      const int g = r / kBarGroup;
      const int n_groups = (k + kBarGroup - 1) / kBarGroup;
      const unsigned long long g_size = (unsigned long long)min(kBarGroup, k - g * kBarGroup);
      if (atom_add_acq_rel(&bar->grp[g].count, 1ULL) + 1ULL == e * g_size)
        atom_add_acq_rel(&bar->top.count, 1ULL);
      target = e * (unsigned long long)n_groups;
    }
    if (ld_acquire(&bar->top.count) < target) {
      const unsigned long long t0 = globaltimer_ns();
      unsigned int spins = 0;
      while (ld_acquire(&bar->top.count) < target) {
        if ((++spins & 31u) == 0u) {
          if (*((volatile int*)err) != 0) { ok = 0; break; }
          if (globaltimer_ns() - t0 > s_bar_timeout_ns) {
            atomicExch(err, 1);
            ok = 0;
            break;
          }
        }
        __nanosleep(8);
      }
    }
  }
  __syncthreads();
  return ok != 0;
}

// Runtime dispatch of the SpMV tile procedures on the system's threads-per-row
// (coherent gathers: x and p were written earlier in this kernel).
#define NLGB_TPR_SWITCH(...)                                            \
  switch (s.tpr) {                                                      \
    case 1: { constexpr int T = 1; __VA_ARGS__; } break;                \
    case 2: { constexpr int T = 2; __VA_ARGS__; } break;                \
    case 4: { constexpr int T = 4; __VA_ARGS__; } break;                \
    case 8: { constexpr int T = 8; __VA_ARGS__; } break;                \
    case 16: { constexpr int T = 16; __VA_ARGS__; } break;              \
    default: { constexpr int T = 32; __VA_ARGS__; } break;              \
  }

__device__ void put_parts(const SysView& s, int tile, int slot, const double* v, int K) {
  if (threadIdx.x == 0)
    for (int k = 0; k < K; ++k) __stcg(s.part + (size_t)tile * kParts + slot + k, v[k]);
}

template <int K>
__device__ void get_sums(const SysView& s, int slot, double (&o)[K]) {
  int comp[K];
#pragma unroll
  for (int k = 0; k < K; ++k) comp[k] = slot + k;
  canon_reduce<K>(s.part, s.n_tiles, comp, o);
}

// Thread 0 applies a scalar step to the CTA's shared copy of the state; the
// barrier after it publishes the result to the other threads.
#define NLGB_SCALAR(stmt)        \
  if (threadIdx.x == 0) { stmt; } \
  __syncthreads();

// Phase procedures: the tile loop of one phase for this CTA's tiles (t = r,
// r + k, ...), partials stored for the canonical reduction.  Kept out of line
// so that each is register-allocated on its own: inlined into the one
// persistent kernel (six threads-per-row variants of each) they forced the
// kernel to spill inside the SpMV loops.  NLGB_HOT_PHASE marks the three
// phases of the FP64 iteration.
#ifndef NLGB_HOT_PHASE
#define NLGB_HOT_PHASE __noinline__
#endif
template <bool D>
__device__ __noinline__ void ph_residual(const SysView& s, int r, int k) {
  for (int t = r; t < s.n_tiles; t += k) {
    double v[3];
    NLGB_TPR_SWITCH((phase_residual<D, T, true>(s, t, v)));
    put_parts(s, t, kSlotInit, v, 3);
  }
}
__device__ __noinline__ void ph_mx_outer(const SysView& s, int r, int k) {
  for (int t = r; t < s.n_tiles; t += k) {
    double v[4];
    NLGB_TPR_SWITCH(tile_mx_outer<T, true>(s, t, v));
    put_parts(s, t, kSlotInit, v, 4);
  }
}
template <bool D>
__device__ NLGB_HOT_PHASE void ph_spmv_pq(const SysView& s, int r, int k) {
  for (int t = r; t < s.n_tiles; t += k) {
    double v[1];
    NLGB_TPR_SWITCH((v[0] = phase_spmv_pq<D, T, true>(s, t)));
    put_parts(s, t, kSlotPQ, v, 1);
  }
}
template <bool D>
__device__ NLGB_HOT_PHASE void ph_update_xr(const SysView& s, int r, int k, double alpha) {
  for (int t = r; t < s.n_tiles; t += k) {
    double v[2];
    phase_update_xr<D>(s, t, alpha, v);
    put_parts(s, t, kSlotXR, v, 2);
  }
}
template <bool D>
__device__ NLGB_HOT_PHASE void ph_update_p(const SysView& s, int r, int k, double beta) {
  for (int t = r; t < s.n_tiles; t += k) phase_update_p<D>(s, t, beta);
}
__device__ __noinline__ void ph_mx_update_p(const SysView& s, int r, int k, double beta) {
  for (int t = r; t < s.n_tiles; t += k) tile_mx_update_p(s, t, beta);
}
__device__ __noinline__ void ph_mx_spmv_pq(const SysView& s, int r, int k) {
  for (int t = r; t < s.n_tiles; t += k) {
    double v[1];
    NLGB_TPR_SWITCH(v[0] = tile_mx_spmv_pq<T, true>(s, t));
    put_parts(s, t, kSlotPQ, v, 1);
  }
}
__device__ __noinline__ void ph_mx_update_cr(const SysView& s, int r, int k, double alpha) {
  for (int t = r; t < s.n_tiles; t += k) {
    double v[2];
    tile_mx_update_cr(s, t, alpha, v);
    put_parts(s, t, kSlotXR, v, 2);
  }
}
__device__ __noinline__ void ph_mx_apply(const SysView& s, int r, int k) {
  for (int t = r; t < s.n_tiles; t += k) tile_mx_apply(s, t);
}
template <bool D>
__device__ __noinline__ void ph_final(const SysView& s, int r, int k, bool zero_rhs) {
  for (int t = r; t < s.n_tiles; t += k) {
    double v[1] = {0.0};
    if (zero_rhs) {
      tile_zero_x(s, t);
    } else {
      NLGB_TPR_SWITCH((v[0] = phase_true_rr<D, T, true>(s, t)));
    }
    put_parts(s, t, kSlotFinal, v, 1);
  }
}

// Canonical sums of K consecutive partial slots (out of line, as above).
struct Sums4 { double v[4]; };
__device__ __noinline__ Sums4 sums_of(const SysView& s, int slot, int K) {
  Sums4 o = {{0.0, 0.0, 0.0, 0.0}};
  switch (K) {
    case 1: { double a[1]; get_sums<1>(s, slot, a); o.v[0] = a[0]; } break;
    case 2: { double a[2]; get_sums<2>(s, slot, a); o.v[0] = a[0]; o.v[1] = a[1]; } break;
    case 3: { double a[3]; get_sums<3>(s, slot, a); for (int i = 0; i < 3; ++i) o.v[i] = a[i]; } break;
    default: { double a[4]; get_sums<4>(s, slot, a); for (int i = 0; i < 4; ++i) o.v[i] = a[i]; } break;
  }
  return o;
}

// One system, run by a team (rank r of k CTAs) for at most `budget`
// iterations.  st: the CTA's shared-memory copy of the system state.
__device__ void run_system_once(const SysView& s, SysState* st, int r, int k, TeamBar* bar, int* err,
                                long long budget) {
  const bool mixed = st->precision == 1;
  long long done_iters = 0;
  if (st->stage == 0) {
    if (!mixed) {
      if (s.df) ph_residual<true>(s, r, k);
      else ph_residual<false>(s, r, k);
      if (!team_sync(bar, k, r, err)) { NLGB_SCALAR(st->status = ST_DEVICE_ERR; st->stage = 3); return; }
      const Sums4 o = sums_of(s, kSlotInit, 3);
      NLGB_SCALAR(scalar_after_init(st, o.v[0], o.v[1], o.v[2]); st->stage = st->status == ST_RUNNING ? 1 : 2);
    } else {
      // initial FP64 residual (first "reliable update"; c = 0, p = 0)
      ph_mx_outer(s, r, k);
      if (!team_sync(bar, k, r, err)) { NLGB_SCALAR(st->status = ST_DEVICE_ERR; st->stage = 3); return; }
      const Sums4 o = sums_of(s, kSlotInit, 4);
      NLGB_SCALAR(st->mode = 0; scalar_after_outer(st, o.v[0], o.v[1], o.v[2], o.v[3]);
                  st->stage = st->status == ST_RUNNING ? 1 : 2);
    }
  }
  for (;;) {
    if (st->stage == 4) {
      // continuation after a failed true-residual check (possibly left by
      // another executor): the pending p update, then more iterations
      if (s.df) ph_update_p<true>(s, r, k, st->beta);
      else ph_update_p<false>(s, r, k, st->beta);
      if (!team_sync(bar, k, r, err)) { NLGB_SCALAR(st->status = ST_DEVICE_ERR; st->stage = 3); return; }
      NLGB_SCALAR(st->stage = 1);
    }
    while (st->stage == 1 && (budget <= 0 || done_iters < budget)) {
      stop_probe(bar, k, r);
      if (!mixed) {
        // q = A p, p.q
        if (s.df) ph_spmv_pq<true>(s, r, k);
        else ph_spmv_pq<false>(s, r, k);
        if (!team_sync(bar, k, r, err)) break;
        {
          const Sums4 o = sums_of(s, kSlotPQ, 1);
          NLGB_SCALAR(scalar_after_pq(st, o.v[0]); stop_read(bar, k));
        }
        if (st->status != ST_RUNNING) { NLGB_SCALAR(st->stage = 2); break; }
        if (s.df) ph_update_xr<true>(s, r, k, st->alpha);
        else ph_update_xr<false>(s, r, k, st->alpha);
        if (!team_sync(bar, k, r, err)) break;
        {
          const Sums4 o = sums_of(s, kSlotXR, 2);
          NLGB_SCALAR(scalar_after_xr(st, o.v[0], o.v[1]));
        }
        ++done_iters;
        if (st->status != ST_RUNNING) { NLGB_SCALAR(st->stage = 2); break; }
        if (s.df) ph_update_p<true>(s, r, k, st->beta);
        else ph_update_p<false>(s, r, k, st->beta);
        if (!team_sync(bar, k, r, err)) break;
        if (s_stop) break;   // time box used up: the system resumes next epoch
      } else {
        // FP32 PCG iteration with FP64 reliable updates; same phase order as
        // the graph solver: p update, SpMV + p.q, c/r update, [update].
        ph_mx_update_p(s, r, k, st->beta);
        if (!team_sync(bar, k, r, err)) break;
        ph_mx_spmv_pq(s, r, k);
        if (!team_sync(bar, k, r, err)) break;
        {
          const Sums4 o = sums_of(s, kSlotPQ, 1);
          NLGB_SCALAR(scalar_after_pq(st, o.v[0]); stop_read(bar, k));
        }
        if (st->status != ST_RUNNING) { NLGB_SCALAR(st->stage = 2); break; }
        ph_mx_update_cr(s, r, k, st->alpha);
        if (!team_sync(bar, k, r, err)) break;
        {
          const Sums4 o = sums_of(s, kSlotXR, 2);
          NLGB_SCALAR(scalar_after_mx_cr(st, o.v[0], o.v[1]));
        }
        ++done_iters;
        if (st->status != ST_RUNNING) { NLGB_SCALAR(st->stage = 2); break; }
        if (st->mode == 0) {
          // reliable update: x += c, r = b - A x in FP64, FP32 residual replaced
          ph_mx_apply(s, r, k);
          if (!team_sync(bar, k, r, err)) break;
          ph_mx_outer(s, r, k);
          if (!team_sync(bar, k, r, err)) break;
          const Sums4 o = sums_of(s, kSlotInit, 4);
          NLGB_SCALAR(scalar_after_outer(st, o.v[0], o.v[1], o.v[2], o.v[3]);
                      // FP32 cannot track this system: continue it in FP64
                      // from the current x (same rule as the graph solver).
                      if (st->status == ST_STAGNATION && !st->fell_back) {
                        st->status = ST_RUNNING; st->precision = 0; st->fell_back = 1;
                        st->stage = 0; st->mode = 0; st->iter_at_fallback = st->iter;
                      });
          if (st->stage == 0) break;
          if (st->status != ST_RUNNING) { NLGB_SCALAR(st->stage = 2); break; }
        }
        if (s_stop) break;   // time box used up: the system resumes next epoch
      }
    }
    if (*((volatile int*)err) != 0 && st->stage != 3) {
      NLGB_SCALAR(st->status = ST_DEVICE_ERR; st->stage = 3);
      return;
    }
    if (st->stage == 2) {
      // final true residual (FP64) of the returned x; x = 0 when b == 0
      if (s.df) ph_final<true>(s, r, k, st->zero_rhs != 0);
      else ph_final<false>(s, r, k, st->zero_rhs != 0);
      if (!team_sync(bar, k, r, err)) { NLGB_SCALAR(st->status = ST_DEVICE_ERR; st->stage = 3); return; }
      const Sums4 o = sums_of(s, kSlotFinal, 1);
      NLGB_SCALAR(st->rr_true = o.v[0]; st->stage = scalar_after_check(st) ? 4 : 3);
      if (st->stage == 4) continue;
    }
    return;
  }
}

// One system; a mixed system that falls back to FP64 restarts here at stage
// 0 with precision 0 (its FP32 iterations stay counted).
__device__ void run_system(const SysView& s, SysState* st, int r, int k, TeamBar* bar, int* err,
                           long long budget) {
  run_system_once(s, st, r, k, bar, err, budget);
  if (st->stage == 0 && st->fell_back && st->precision == 0)
    run_system_once(s, st, r, k, bar, err, budget);
}

// Four CTAs per SM (64 registers): stating the bound lets ptxas plan for it,
// with far fewer spills than its own choice of the same 64 registers.
__global__ void __launch_bounds__(kCTA, 4) k_batch(BatchArgs a) {
  __shared__ SysView sv;
  __shared__ SysState sst;
  __shared__ int pick;
  const int cta = blockIdx.x;
  if (threadIdx.x == 0) {
    s_bar_epoch = 0ULL;
    s_bar_timeout_ns = a.barrier_timeout_ns;
    s_deadline = a.epoch_ns > 0ULL ? globaltimer_ns() + a.epoch_ns : 0ULL;
    s_stop = 0;
  }
  if (a.times && cta == 0 && threadIdx.x == 0) a.times[0] = globaltimer_ns();
  __syncthreads();
  auto load = [&](int sys) {
    if (threadIdx.x == 0) {
      sv = a.views[sys];
      sst = *sv.st;
      s_stop = 0;
    }
    __syncthreads();
  };
  auto past_deadline = [&]() { return s_deadline != 0ULL && globaltimer_ns() > s_deadline; };
  auto store = [&](bool rank0) {
    __syncthreads();
    if (rank0 && threadIdx.x == 0) {
      *sv.st = sst;
      __threadfence();
    }
    __syncthreads();
  };
  if (cta < a.team_ctas) {
    const int team = a.cta_team[cta];
    const TeamDesc td = a.teams[team];
    const int r = cta - td.cta_begin;
    TeamBar* bar = a.bars + team;
    for (int j = td.sys_begin; j < td.sys_end; ++j) {
      load(a.team_sys[j]);
      if (sst.stage != 3) run_system(sv, &sst, r, td.k, bar, a.err, sv.budget > 0 ? sv.budget : a.budget);
      store(r == 0);
    }
    // Then the shared team queue: rank 0 draws the next system and publishes
    // it through the team barrier; a second barrier keeps the next draw from
    // overwriting `pick` before every CTA of the team has read it.
    while (a.n_tqueue > 0) {
      // past the time box, rank 0 draws nothing (publishes the end of the queue)
      if (r == 0 && threadIdx.x == 0)
        *((volatile unsigned long long*)&bar->pick.count) =
            past_deadline() ? (unsigned long long)a.n_tqueue : atomicAdd(a.tqueue_head, 1u);
      if (!team_sync(bar, td.k, r, a.err)) break;
      if (threadIdx.x == 0) pick = (int)*((volatile unsigned long long*)&bar->pick.count);
      __syncthreads();
      const int q = pick;
      if (!team_sync(bar, td.k, r, a.err)) break;
      if (q >= a.n_tqueue) break;
      load(a.tqueue[q]);
      if (sst.stage != 3) run_system(sv, &sst, r, td.k, bar, a.err, sv.budget > 0 ? sv.budget : a.budget);
      store(r == 0);
    }
    if (a.times && r == 0 && threadIdx.x == 0) a.times[2 + team] = globaltimer_ns();
  } else {
    while (true) {
      if (threadIdx.x == 0) pick = past_deadline() ? a.n_queue : (int)atomicAdd(a.queue_head, 1u);
      __syncthreads();
      const int q = pick;
      __syncthreads();
      if (q >= a.n_queue) break;
      load(a.queue[q]);
      if (sst.stage != 3) run_system(sv, &sst, 0, 1, nullptr, a.err, sv.budget > 0 ? sv.budget : a.budget);
      store(true);
    }
    if (a.times && threadIdx.x == 0) atomicMax(&a.times[1], globaltimer_ns());
  }
}

__global__ void k_gather_states(const SysView* views, int n, SysState* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = *views[i].st;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
BatchRunner::~BatchRunner() {
  cudaFree(d_views_); cudaFree(d_teams_); cudaFree(d_cta_team_); cudaFree(d_team_sys_);
  cudaFree(d_queue_); cudaFree(d_tqueue_); cudaFree(d_bars_); cudaFree(d_ctl_); cudaFree(d_times_);
  if (h_err_) cudaFreeHost(h_err_);
  cudaFree(d_states_);
  if (ev0_) cudaEventDestroy(ev0_);
  if (ev1_) cudaEventDestroy(ev1_);
}

cudaError_t BatchRunner::init(cudaStream_t s) {
  stream_ = s;
  int dev = 0;
  NLGB_CUDA_TRY(cudaGetDevice(&dev));
  NLGB_CUDA_TRY(cudaDeviceGetAttribute(&n_sm_, cudaDevAttrMultiProcessorCount, dev));
  int per_sm = 0;
  NLGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, kCTA, 0));
  per_sm_ = std::max(1, per_sm);
  grid_ = n_sm_ * per_sm_;
  NLGB_CUDA_TRY(cudaMalloc(&d_ctl_, 3 * sizeof(int)));
  NLGB_CUDA_TRY(cudaMallocHost(&h_err_, sizeof(int)));
  *h_err_ = 0;
  NLGB_CUDA_TRY(cudaEventCreate(&ev0_));
  NLGB_CUDA_TRY(cudaEventCreate(&ev1_));
  // Test hooks for the barrier's failure path (read once per runner): a
  // shorter wait limit, and a first team told to wait for one CTA more than
  // it is given, so that its first barrier runs out -- the kernel must then
  // flag the error, return, and leave the GPU usable.
  if (const char* e = std::getenv("NLGB_BARRIER_TIMEOUT_MS")) {
    const double ms = std::atof(e);
    if (ms > 0.0) barrier_timeout_ns_ = (unsigned long long)(ms * 1e6);
  }
  if (const char* e = std::getenv("NLGB_TEST_TEAM_SHORTFALL")) test_shortfall_ = e[0] == '1';
  return cudaSuccess;
}

template <typename T>
static cudaError_t ensure(T*& p, size_t& cap, size_t n) {
  if (n <= cap && p) return cudaSuccess;
  cudaFree(p);
  p = nullptr;
  cap = std::max<size_t>(n, 16);
  return cudaMalloc(&p, cap * sizeof(T));
}

// Schedule for one launch.  Small systems (fewer than kLargeTiles tiles) go to
// the single-CTA queue, whose workers get a share of the grid proportional to
// the small systems' work (at least one, at most one per system).  The large
// ones, largest first, get teams sized by their share of the remaining CTAs
// (at least 2, at most one CTA per tile) until the CTAs run out; the rest
// wait in the team queue, from which every team draws (largest first) once
// its own system is done -- list scheduling, so one mis-estimated system
// does not leave the other teams idle.
void BatchRunner::plan(const std::vector<SysView>& views, const std::vector<long long>& work) {
  teams_.clear(); cta_team_.clear(); team_sys_.clear(); queue_.clear(); tqueue_.clear();
  const int n = (int)views.size();
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
  std::vector<int> large;
  double w_large = 0.0, w_small = 0.0;
  for (int i : order) {
    const double w = (double)std::max(1LL, work[i]);
    if (views[i].n_tiles >= kLargeTiles) { large.push_back(i); w_large += w; }
    else { queue_.push_back(i); w_small += w; }
  }
  if (large.empty()) return;
  int reserve = 0;
  if (!queue_.empty()) {
    reserve = (int)std::ceil((double)grid_ * w_small / (w_small + w_large));
    reserve = std::max(1, std::min(reserve, std::min((int)queue_.size(), grid_ / 2)));
  }
  const int avail = grid_ - reserve_ - reserve;
  if (avail < 2) {   // no room for a team: everything goes to the queue workers
    queue_.insert(queue_.begin(), large.begin(), large.end());
    return;
  }
  const double per_cta = w_large / (double)avail;
  int cta = 0;
  for (int i : large) {
    const double w = (double)std::max(1LL, work[i]);
    const int cap = std::min(kBarGroup * kBarMaxGroups, std::max(2, views[i].n_tiles));
    int k = (int)std::min<double>((double)cap, std::max(2.0, std::floor(w / per_cta)));
    if (cta + k > avail) k = avail - cta;     // the last team takes what is left
    if (k < 2) { tqueue_.push_back(i); continue; }
    // Balanced: the fewest CTAs with the same tiles on the busiest CTA (1,023
    // tiles on 604 CTAs are 2 on the busiest, as on 512; the other 92 CTAs
    // would only add barrier and reduction traffic).
    const int per = (views[i].n_tiles + k - 1) / k;
    k = std::max(2, (views[i].n_tiles + per - 1) / per);
    TeamDesc td;
    td.cta_begin = cta;
    td.k = k;
    td.sys_begin = (int)team_sys_.size();
    team_sys_.push_back(i);
    td.sys_end = (int)team_sys_.size();
    for (int c = 0; c < k; ++c) cta_team_.push_back((int)teams_.size());
    teams_.push_back(td);
    cta += k;
  }
}

constexpr int kPrioTilesPerCta = 4;

void BatchRunner::plan_priority(const std::vector<SysView>& views) {
  teams_.clear(); cta_team_.clear(); team_sys_.clear(); queue_.clear(); tqueue_.clear();
  const int n = (int)views.size();
  const int avail_all = std::max(1, grid_ - reserve_);
  int n_small = 0;
  for (int i = 0; i < n; ++i) n_small += views[i].n_tiles < kLargeTiles ? 1 : 0;
  // queue workers: one per small system, at most half the grid
  const int workers = n_small == 0 ? 0 : std::max(1, std::min(n_small, avail_all / 2));
  const int avail = avail_all - workers;
  int cta = 0;
  for (int i = 0; i < n; ++i) {
    if (views[i].n_tiles < kLargeTiles) { queue_.push_back(i); continue; }
    const int room = avail - cta;
    if (room < 2) { tqueue_.push_back(i); continue; }
    // about kPrioTilesPerCta tiles per CTA: enough CTAs to finish the
    // system soon, few enough that each CTA's tile work outweighs the
    // team's barriers and that the next systems get teams too
    int k = std::min({(views[i].n_tiles + kPrioTilesPerCta - 1) / kPrioTilesPerCta, kBarGroup * kBarMaxGroups,
                      room});
    k = std::max(2, k);
    // balanced: the fewest CTAs with the same tiles on the busiest CTA
    const int per = (views[i].n_tiles + k - 1) / k;
    k = std::max(2, (views[i].n_tiles + per - 1) / per);
    TeamDesc td;
    td.cta_begin = cta;
    td.k = k;
    td.sys_begin = (int)team_sys_.size();
    team_sys_.push_back(i);
    td.sys_end = (int)team_sys_.size();
    for (int c = 0; c < k; ++c) cta_team_.push_back((int)teams_.size());
    teams_.push_back(td);
    cta += k;
  }
  // without any team, large systems left over go to the queue workers too
  if (teams_.empty() && !tqueue_.empty()) {
    queue_.insert(queue_.end(), tqueue_.begin(), tqueue_.end());
    tqueue_.clear();
  }
}

cudaError_t BatchRunner::run(const std::vector<SysView>& views, const std::vector<long long>& work,
                             long long budget, BatchLaunchStats* stats) {
  NLGB_CUDA_TRY(launch(views, work, budget));
  return finish(stats);
}

cudaError_t BatchRunner::launch(const std::vector<SysView>& views, const std::vector<long long>& work,
                                long long budget) {
  pending_ = false;
  if (views.empty()) return cudaSuccess;
  if (priority_plan_) plan_priority(views);
  else plan(views, work);
  NLGB_CUDA_TRY(ensure(d_views_, cap_views_, views.size()));
  NLGB_CUDA_TRY(ensure(d_teams_, cap_teams_, teams_.size()));
  NLGB_CUDA_TRY(ensure(d_cta_team_, cap_cta_team_, cta_team_.size()));
  NLGB_CUDA_TRY(ensure(d_team_sys_, cap_team_sys_, team_sys_.size()));
  NLGB_CUDA_TRY(ensure(d_queue_, cap_queue_, queue_.size()));
  NLGB_CUDA_TRY(ensure(d_tqueue_, cap_tqueue_, tqueue_.size()));
  NLGB_CUDA_TRY(ensure(d_bars_, cap_bars_, teams_.size()));
  cudaStream_t s = stream_;
  NLGB_CUDA_TRY(cudaMemcpyAsync(d_views_, views.data(), views.size() * sizeof(SysView), cudaMemcpyHostToDevice, s));
  if (!teams_.empty()) {
    if (test_shortfall_ && teams_[0].k < kBarFlat) {
      std::vector<TeamDesc> t = teams_;
      t[0].k += 1;   // no CTA is mapped to the extra rank: the team's barrier cannot complete
      NLGB_CUDA_TRY(cudaMemcpy(d_teams_, t.data(), t.size() * sizeof(TeamDesc), cudaMemcpyHostToDevice));
    } else {
      NLGB_CUDA_TRY(cudaMemcpyAsync(d_teams_, teams_.data(), teams_.size() * sizeof(TeamDesc),
                                    cudaMemcpyHostToDevice, s));
    }
    NLGB_CUDA_TRY(cudaMemcpyAsync(d_cta_team_, cta_team_.data(), cta_team_.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    NLGB_CUDA_TRY(cudaMemcpyAsync(d_team_sys_, team_sys_.data(), team_sys_.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    NLGB_CUDA_TRY(cudaMemsetAsync(d_bars_, 0, teams_.size() * sizeof(TeamBar), s));
  }
  if (!queue_.empty())
    NLGB_CUDA_TRY(cudaMemcpyAsync(d_queue_, queue_.data(), queue_.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  if (!tqueue_.empty())
    NLGB_CUDA_TRY(cudaMemcpyAsync(d_tqueue_, tqueue_.data(), tqueue_.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  NLGB_CUDA_TRY(cudaMemsetAsync(d_ctl_, 0, 3 * sizeof(int), s));
  BatchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.views = d_views_;
  a.teams = d_teams_;
  a.cta_team = d_cta_team_;
  a.team_sys = d_team_sys_;
  a.queue = d_queue_;
  a.tqueue = d_tqueue_;
  a.bars = d_bars_;
  a.err = d_ctl_;
  a.queue_head = reinterpret_cast<unsigned int*>(d_ctl_ + 1);
  a.tqueue_head = reinterpret_cast<unsigned int*>(d_ctl_ + 2);
  a.team_ctas = (int)cta_team_.size();
  a.n_queue = (int)queue_.size();
  a.n_tqueue = teams_.empty() ? 0 : (int)tqueue_.size();
  a.budget = budget;
  a.times = nullptr;
  a.barrier_timeout_ns = barrier_timeout_ns_;
  a.epoch_ns = epoch_ns_;
  if (timing_) {
    NLGB_CUDA_TRY(ensure(d_times_, cap_times_, teams_.size() + 2));
    NLGB_CUDA_TRY(cudaMemsetAsync(d_times_, 0, (teams_.size() + 2) * sizeof(unsigned long long), s));
    a.times = d_times_;
  }
  // Grid: every team CTA plus queue workers, never more than can be resident
  // (less the reserve).
  const int workers = queue_.empty() ? 0 : std::max(1, std::min(std::max(1, grid_ - reserve_) - a.team_ctas,
                                                                (int)queue_.size()));
  const int grid = a.team_ctas + std::max(0, workers);
  void* args[] = {&a};
  NLGB_CUDA_TRY(cudaEventRecord(ev0_, s));
  NLGB_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_batch, dim3(grid), dim3(kCTA), args, 0, s));
  NLGB_CUDA_TRY(cudaEventRecord(ev1_, s));
  NLGB_CUDA_TRY(cudaMemcpyAsync(h_err_, d_ctl_, sizeof(int), cudaMemcpyDeviceToHost, s));
  last_grid_ = grid;
  last_workers_ = workers;
  pending_ = true;
  return cudaSuccess;
}

cudaError_t BatchRunner::finish(BatchLaunchStats* stats) {
  if (!pending_) {
    if (stats) *stats = BatchLaunchStats();
    return cudaSuccess;
  }
  pending_ = false;
  NLGB_CUDA_TRY(cudaStreamSynchronize(stream_));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev0_, ev1_);
  if (timing_) {
    h_times_.assign(teams_.size() + 2, 0ULL);
    NLGB_CUDA_TRY(cudaMemcpy(h_times_.data(), d_times_, h_times_.size() * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost));
  }
  const int err = *h_err_;
  if (stats) {
    stats->ms = ms;
    stats->n_teams = (int)teams_.size();
    stats->team_ctas = (int)cta_team_.size();
    stats->queue_ctas = last_workers_;
    stats->error = err;
    stats->grid = last_grid_;
  }
  if (err) {
    set_error("batched solve: a team barrier timed out");
    return cudaErrorLaunchTimeout;
  }
  return cudaSuccess;
}

cudaError_t BatchRunner::gather_states(SysState* out, int n) {
  if (n <= 0) return cudaSuccess;
  NLGB_CUDA_TRY(ensure(d_states_, cap_states_, (size_t)n));
  k_gather_states<<<(n + 127) / 128, 128, 0, stream_>>>(d_views_, n, d_states_);
  count_launches(1);
  NLGB_CUDA_TRY(cudaGetLastError());
  NLGB_CUDA_TRY(cudaMemcpyAsync(out, d_states_, sizeof(SysState) * n, cudaMemcpyDeviceToHost, stream_));
  NLGB_CUDA_TRY(cudaStreamSynchronize(stream_));
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Per-system device slot.
// ---------------------------------------------------------------------------
static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

size_t SystemSlot::bytes_for(int n, int tile_rows, bool mixed) {
  const size_t n8 = align256((size_t)std::max(2, n + 2) * sizeof(double));
  const size_t n4 = align256((size_t)std::max(4, n + 4) * sizeof(float));
  const int n_tiles = std::max(1, (n + tile_rows - 1) / tile_rows);
  const size_t parts = align256((size_t)n_tiles * kParts * sizeof(double));
  const size_t st = align256(sizeof(SysState));
  // mixed systems also carry the FP64 r, p, q of a possible FP64 fallback
  return mixed ? (5 * n8 + 4 * n4 + parts + st) : (5 * n8 + parts + st);
}

cudaError_t SystemSlot::alloc(DeviceCRS* Am, bool mx, cudaStream_t s, bool dfl) {
  A = Am;
  mixed = mx;
  df = dfl && !mx && Am->vadf != nullptr && Am->dinvdf != nullptr;
  const int n = A->n;
  bytes = bytes_for(n, A->tile_rows, mixed);
  NLGB_CUDA_TRY(cudaMallocAsync(&block, bytes, s));
  char* p = static_cast<char*>(block);
  const size_t n8 = align256((size_t)std::max(2, n + 2) * sizeof(double));
  const size_t n4 = align256((size_t)std::max(4, n + 4) * sizeof(float));
  std::memset(&view, 0, sizeof(view));
  view.n = n;
  view.tile_rows = A->tile_rows;
  view.n_tiles = std::max(1, (n + A->tile_rows - 1) / A->tile_rows);
  view.tpr = A->tpr;
  view.rp = A->rp; view.ci = A->ci; view.va = A->va; view.va32 = A->va32;
  view.dinv = A->dinv; view.dinv32 = A->dinv32;
  if (df) {
    view.df = 1;
    view.vadf = A->vadf;
    view.dinvdf = A->dinvdf;
  }
  view.b = reinterpret_cast<double*>(p); p += n8;
  view.x = reinterpret_cast<double*>(p); p += n8;
  view.r = reinterpret_cast<double*>(p); p += n8;
  view.p = reinterpret_cast<double*>(p); p += n8;
  view.q = reinterpret_cast<double*>(p); p += n8;
  if (mixed) {
    view.r32 = reinterpret_cast<float*>(p); p += n4;
    view.p32 = reinterpret_cast<float*>(p); p += n4;
    view.q32 = reinterpret_cast<float*>(p); p += n4;
    view.c32 = reinterpret_cast<float*>(p); p += n4;
  }
  view.part = reinterpret_cast<double*>(p);
  p += align256((size_t)view.n_tiles * kParts * sizeof(double));
  view.st = reinterpret_cast<SysState*>(p);
  return cudaSuccess;
}

cudaError_t SystemSlot::start(const double* b, const double* x0, const SolveParams& prm,
                              cudaStream_t s) {
  const size_t n = (size_t)view.n;
  NLGB_CUDA_TRY(cudaMemcpyAsync(const_cast<double*>(view.b), b, n * sizeof(double), cudaMemcpyDefault, s));
  if (x0) NLGB_CUDA_TRY(cudaMemcpyAsync(view.x, x0, n * sizeof(double), cudaMemcpyDefault, s));
  else NLGB_CUDA_TRY(cudaMemsetAsync(view.x, 0, n * sizeof(double), s));   // 0.0 in either form
  if (df && x0) NLGB_CUDA_TRY(df_pack(view.x, (long long)n, s));
  if (mixed) {
    NLGB_CUDA_TRY(cudaMemsetAsync(view.p32, 0, n * sizeof(float), s));
    NLGB_CUDA_TRY(cudaMemsetAsync(view.c32, 0, n * sizeof(float), s));
  }
  SysState h;
  std::memset(&h, 0, sizeof(h));
  const long long max_iter = prm.max_iter >= 0 ? prm.max_iter : 5LL * view.n;
  h.thresh2 = prm.eps * prm.eps;
  h.max_iter = max_iter;
  h.status = ST_RUNNING;
  h.max_outer = std::max(1, prm.max_outer);
  h.in_thresh2 = prm.inner_eps * prm.inner_eps;
  h.in_max = (int)std::max(1LL, std::min<long long>(max_iter, 1000));
  h.precision = mixed ? 1 : 0;
  h.stage = 0;
  // cudaMemcpyAsync from pageable memory is staged synchronously, so the
  // stack copy may go out of scope after the call.
  NLGB_CUDA_TRY(cudaMemcpyAsync(view.st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  return cudaSuccess;
}

void SystemSlot::release(cudaStream_t s) {
  if (block) cudaFreeAsync(block, s);
  block = nullptr;
}

}  // namespace nlgb
