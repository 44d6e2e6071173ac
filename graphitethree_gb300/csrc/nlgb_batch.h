// nlgb_batch.h -- host/device interface of the persistent batched solver.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "nlgb_core.cuh"

namespace nlgb {

// Systems with at least this many tiles are run by multi-CTA teams; smaller
// ones are popped from the queue by single CTAs.
constexpr int kLargeTiles = 16;
// When only large systems are left in the server (at least kGraphMinTiles
// tiles each, at most kMaxGraphSystems of them), each continues on its own
// graph executor, one after the other in an epoch (measured on GB300: from
// ~500 tiles the graph path is faster per iteration than the persistent
// kernel).
constexpr int kGraphMinTiles = 384;
constexpr size_t kMaxGraphSystems = 4;

// Team barrier on monotonic 64-bit arrival counters (never reset within a
// launch): barrier number e of a team is complete when its counter reaches
// e x (arrivals per barrier).  Teams of up to kBarFlat CTAs arrive on one
// counter; larger teams arrive on the counter of their group of kBarGroup,
// and the last of each group on the top counter, so at most kBarGroup
// atomics in a row hit one address.  Each counter has its own 128-byte line.
constexpr int kBarFlat = 64;
constexpr int kBarGroup = 32;
constexpr int kBarMaxGroups = 32;   // teams of up to 1024 CTAs
struct __align__(128) BarLine {
  unsigned long long count;
  unsigned long long pad_[15];
};
struct TeamBar {
  BarLine top;
  BarLine grp[kBarMaxGroups];
  BarLine pick;   // .count: team-queue entry drawn by the team's rank 0
  BarLine stop;   // .count: 1 when rank 0 found the epoch's time box used up
};

struct TeamDesc {
  int cta_begin;
  int k;          // CTAs in the team
  int sys_begin;  // range in team_sys
  int sys_end;
};

struct BatchArgs {
  const SysView* views;
  const TeamDesc* teams;
  const int* cta_team;       // team of each team CTA
  const int* team_sys;       // system indices handled by teams, grouped by team
  const int* queue;          // system indices handled by queue workers
  const int* tqueue;         // large systems drawn by any free team, largest first
  TeamBar* bars;
  int* err;                  // nonzero: a barrier timed out
  unsigned int* queue_head;
  unsigned int* tqueue_head;
  int team_ctas;
  int n_queue;
  int n_tqueue;
  long long budget;          // iterations per system in this launch (<= 0: no limit)
  // Optional timing (null: off), %globaltimer ns: [0] kernel start, [1] last
  // queue worker done, [2 + t] team t done.
  unsigned long long* times;
  unsigned long long barrier_timeout_ns;   // limit of one team-barrier wait
  // Time box of the launch (0: none): a system stops at the first iteration
  // boundary after it (its team's rank 0 reads the clock at the start of
  // each iteration and tells the team through the iteration's first
  // barrier), and no further system is started.
  unsigned long long epoch_ns;
};

struct BatchLaunchStats {
  double ms = 0;
  int n_teams = 0;
  int team_ctas = 0;
  int queue_ctas = 0;
  int grid = 0;
  int error = 0;
};

// Device storage of one system's Krylov state: a single stream-ordered
// allocation (cudaMallocAsync, pooled) carved into 256-byte aligned arrays.
// FP64 plain: b, x, r, p, q; mixed: b, x, r32, p32, q32, c32; plus the tile
// partials and the SysState.
struct SolveParams;
struct DeviceCRS;
struct SystemSlot {
  DeviceCRS* A = nullptr;
  void* block = nullptr;
  size_t bytes = 0;
  bool mixed = false;
  bool df = false;     // double-float iteration: x holds float pairs until df_unpack
  SysView view{};
  static size_t bytes_for(int n, int tile_rows, bool mixed);
  // df: A must have its double-float copies (crs_prepare_df said usable).
  cudaError_t alloc(DeviceCRS* A, bool mixed, cudaStream_t s, bool df = false);
  // b, x0: host or device vectors of n doubles (x0 may be null: zero start);
  // a double-float slot packs x after the upload.
  cudaError_t start(const double* b, const double* x0, const SolveParams& prm, cudaStream_t s);
  void release(cudaStream_t s);
};

// Resumable PCG chunks (FP64, double-float or mixed precision) of a system
// whose buffers and device state belong to a SystemSlot, as CUDA graphs (see
// nlgb_solver.cu).
// Host-mapped record of one system's chunks (pinned host memory, written by
// the device over the C2C link): the host sets the next chunk's budget
// before launching it; the chunk's last kernel copies the system's state
// here, stores the chunk's device duration and then bumps `seq`, so that a
// host thread sees the end of a chunk by reading memory, without a CUDA call.
struct ChunkMirror {
  SysState st;                   // the system's state after the last chunk
  long long budget;              // host: iterations of the next chunk
  unsigned long long t_start;    // device: %globaltimer at the chunk's start
  unsigned long long t_ns;       // device: the chunk's duration
  unsigned int seq;              // device: +1 after st and t_ns of a chunk are written
  unsigned int pad_;
};

class ViewGraph {
 public:
  ViewGraph() = default;
  ~ViewGraph();
  ViewGraph(const ViewGraph&) = delete;
  ViewGraph& operator=(const ViewGraph&) = delete;
  // Build (or keep) the chunk graph of this system (mixed: the
  // mixed-precision iteration); run() does it too, prepare() lets a caller
  // pay the instantiation ahead of time.
  cudaError_t prepare(const SysView& v, bool mixed);
  // Queue a chunk of at most `iters` iterations (whole passes of 4) of the
  // system on stream s; finish() waits for it and stores its time in *ms;
  // done() tells, without blocking, whether it has finished.
  cudaError_t run(const SysView& v, long long iters, cudaStream_t s, float* ms, bool mixed = false);
  bool done() const;
  cudaError_t finish(long long iters_before, long long iters_after);
  // Mirrored chunks: the graph reads its budget from `m` (host-mapped) and
  // ends by writing the state there (ChunkMirror).  launch() is then the
  // only CUDA call of a chunk: the caller writes m->budget, launches and
  // polls m->seq; account() counts the chunk's kernels afterwards.
  // A graph (re)built here is uploaded on `upload` when given, so that its
  // first launch does not pay for it.
  cudaError_t prepare(const SysView& v, bool mixed, ChunkMirror* m, cudaStream_t upload = nullptr);
  cudaError_t launch(cudaStream_t s);
  void account(long long iters_before, long long iters_after);

 private:
  cudaError_t build(const SysView& v, bool mixed);
  cudaError_t run_eager(cudaStream_t s, long long iters);
  SysView view_{};
  ChunkMirror* mirror_ = nullptr;
  bool mixed_ = false;
  cudaGraphExec_t exec_ = nullptr;
  cudaEvent_t e0_ = nullptr, e1_ = nullptr;
  float* ms_ = nullptr;
  bool pending_ = false;
  bool eager_counted_ = false;
};

// A mixed system whose state says STAGNATION (FP32 cannot track it) is
// switched to FP64 PCG from its current x (stage 0, iteration count kept);
// stream-ordered, before the system's next chunk.
cudaError_t chunk_fallback_fp64(SysState* st, cudaStream_t s);

// Launches the persistent kernel over a set of resident systems.  Each
// system's SysState (device) must be initialised by the caller (status
// ST_RUNNING, stage 0, thresholds, max_iter, precision); the state is read
// at the start and written back at the end of every launch, so a system can
// be advanced over several launches (epochs) with identical results.
class BatchRunner {
 public:
  BatchRunner() = default;
  ~BatchRunner();
  BatchRunner(const BatchRunner&) = delete;
  BatchRunner& operator=(const BatchRunner&) = delete;

  cudaError_t init(cudaStream_t s);
  // work[i]: relative cost estimate of system i (bytes per iteration x
  // expected iterations).
  // run() = launch() + finish().  Between the two the host may queue other
  // work (uploads of new requests) on other streams.
  cudaError_t run(const std::vector<SysView>& views, const std::vector<long long>& work,
                  long long budget, BatchLaunchStats* stats);
  cudaError_t launch(const std::vector<SysView>& views, const std::vector<long long>& work,
                     long long budget);
  cudaError_t finish(BatchLaunchStats* stats);
  // Copy the SysState of every system of the last launch into `out`
  // (host, pinned or pageable; views.size() entries), one transfer.
  cudaError_t gather_states(SysState* out, int n);
  int max_grid() const { return grid_; }
  // Per-team completion times of the next launches (tracing): after
  // finish(), last_times() holds [kernel start, queue workers done, team
  // 0 done, ...] in ns of the GPU clock.
  void set_timing(bool on) { timing_ = on; }
  // Time box of the next launches (0: none, every system runs its budget).
  void set_epoch_ns(unsigned long long ns) { epoch_ns_ = ns; }
  // Priority plan: the views are given in priority order; teams (one CTA
  // per tile at most) go to the large systems in that order until the grid
  // is used, the rest wait in the team queue in that order, small systems go
  // to the queue workers in that order.  Otherwise: the work-proportional
  // plan (plan()).
  void set_priority_plan(bool on) { priority_plan_ = on; }
  // CTAs of the co-resident capacity left unused (room for kernels of other
  // streams, e.g. system builds, while an epoch runs).
  void set_reserve(int ctas) { reserve_ = ctas; }
  const std::vector<unsigned long long>& last_times() const { return h_times_; }

 private:
  void plan(const std::vector<SysView>& views, const std::vector<long long>& work);
  void plan_priority(const std::vector<SysView>& views);

  cudaStream_t stream_ = nullptr;
  int n_sm_ = 0, per_sm_ = 0, grid_ = 0;
  std::vector<TeamDesc> teams_;
  std::vector<int> cta_team_, team_sys_, queue_, tqueue_;
  SysView* d_views_ = nullptr;
  TeamDesc* d_teams_ = nullptr;
  int *d_cta_team_ = nullptr, *d_team_sys_ = nullptr, *d_queue_ = nullptr, *d_tqueue_ = nullptr;
  int* d_ctl_ = nullptr;           // error flag, queue head, team-queue head
  TeamBar* d_bars_ = nullptr;
  size_t cap_views_ = 0, cap_teams_ = 0, cap_cta_team_ = 0, cap_team_sys_ = 0, cap_queue_ = 0,
         cap_tqueue_ = 0, cap_bars_ = 0;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  int* h_err_ = nullptr;           // pinned
  SysState* d_states_ = nullptr;
  size_t cap_states_ = 0;
  int last_grid_ = 0, last_workers_ = 0;
  bool pending_ = false;
  bool timing_ = false;
  bool priority_plan_ = false;
  int reserve_ = 0;
  unsigned long long epoch_ns_ = 0;
  unsigned long long barrier_timeout_ns_ = 4000000000ULL;
  bool test_shortfall_ = false;
  unsigned long long* d_times_ = nullptr;
  size_t cap_times_ = 0;
  std::vector<unsigned long long> h_times_;
};

}  // namespace nlgb
