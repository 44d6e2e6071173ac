// nlgb_server.cpp -- solve server with HBM-budget admission and continuous
// batching (include/nl_gb300.h, nlgb_server_*).
//
// In the reference every solve is a synchronous nlSolve under Graphite's
// global command lock (src/lib/OGF/scene_graph/commands/commands.cpp:
// 99-117), and an atlas is parameterised chart after chart
// (mesh_grob_surface_commands.cpp:724).  Here one host thread owns the GPU:
//   * requests become eligible at their arrival time (server clock);
//   * admission is first-fit against the HBM budget (device footprint of
//     the matrix, its FP32 copy, the Jacobi diagonal and every right-hand
//     side's Krylov state), so large requests do not block small ones;
//   * every epoch is one launch of the persistent batched kernel over all
//     active systems for at most epoch_iters iterations each; while it runs,
//     newly eligible requests are uploaded (and least-squares rows
//     assembled) on a second stream; they join the next epoch;
//   * after each epoch the states of all systems are gathered in one copy;
//     finished requests are copied back to the caller's buffer and their
//     device memory is released.
// SERIAL mode is the baseline: one request at a time, each system solved by
// the graph-captured single-system PCG.
#include "../../include/nl.h"
#include "../../include/nl_gb300.h"
#include "nlgb_batch.h"
#include "nlgb_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

using namespace nlgb;
using Clock = std::chrono::steady_clock;

namespace {

enum ReqState { R_FUTURE, R_PENDING, R_ACTIVE, R_DONE, R_FAILED };

struct Req {
  long long id = 0;
  int kind = 0;                 // 0: CRS, 1: row stream, 2: mesh (built on the GPU)
  int least_squares = 1;
  int n = 0;                    // unknowns per system
  int n_rhs = 1;
  // inputs (host copies, released once uploaded)
  std::vector<int> rp, ci;
  std::vector<double> va, b, x0;
  long long n_rows = 0;
  std::vector<long long> row_ptr;
  std::vector<int> col;
  std::vector<double> val, rhs, weight, xl;
  int n_vars = 0;
  bool has_weight = false, has_rhs = false, has_xl = false;
  // mesh requests
  int mesh_kind = 0;            // NLGB_MESH_LSCM / NLGB_MESH_FAIRING
  int n_verts = 0, n_tris = 0;
  std::vector<double> xyz;
  std::vector<int> tris;
  int pins[2] = {0, 0};
  double pin_uv[4] = {0.0, 0.0, 1.0, 1.0};
  double lambda = 0.0;
  double* x_out = nullptr;
  double arrival = 0.0;
  // runtime
  ReqState state = R_FUTURE;
  size_t bytes = 0;
  DeviceCRS A;
  double* d_rhs = nullptr;      // assembled right-hand sides (row streams)
  std::vector<SystemSlot> slots;
  std::vector<int> sys_done;
  std::vector<int> sys_stage;   // SysState::stage after the last epoch
  std::vector<long long> sys_iter;
  // SRPT bookkeeping per system: residual at the first and at the previous
  // epoch boundary, and the estimated iterations left (< 0: not estimated)
  std::vector<double> rr_first, rr_prev, est_left;
  std::vector<long long> it_prev;
  double iter_cost = 0.0;            // bytes-equivalent of one iteration of one system
  // SRPT stream executor: per system, its chunk graphs, whether a chunk is
  // in flight, whether it runs the mixed iteration now, a pending switch to
  // FP64, and the measured time per iteration (ms; < 0 unknown)
  std::vector<std::unique_ptr<ViewGraph>> graphs;
  std::vector<int> mirror_idx;       // per system, its ChunkMirror in the server's pool
  std::vector<int> running, mixed_now, need_fallback;
  std::vector<double> ms_per_iter;
  std::vector<nlgb_result> res;
  double t_done = 0.0;
  double t_built = 0.0, t_prepared = 0.0;   // admission phases (server clock, tracing)
  int status = NL_GB300_STATUS_NONE;
  std::string error;
};

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = q * (double)(v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - (double)i;
  return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

size_t estimate_bytes(const Req& r, int precision) {
  const bool mixed = precision == NL_GB300_PRECISION_MIXED;
  const bool dfl = precision == NL_GB300_PRECISION_DOUBLE_FLOAT;
  const size_t slot = SystemSlot::bytes_for(r.n, 128, mixed);
  size_t nnz = 0, upload = 0;
  if (r.kind == 0) {
    nnz = (size_t)r.rp[r.n];
  } else if (r.kind == 2) {
    // LSCM normal matrix ~14 nonzeros per row, Laplacian ~7; the device row
    // stream of the build (12 B per coefficient + weights) is counted too
    const bool lscm = r.mesh_kind == NLGB_MESH_LSCM;
    nnz = (size_t)r.n * (lscm ? 16 : 8);
    const size_t coefs = lscm ? 12 * (size_t)r.n_tris : 6 * (size_t)r.n_tris + (size_t)r.n_verts;
    upload = (size_t)r.n_verts * 24 + (size_t)r.n_tris * 12 + coefs * 12 + coefs * 8 +
             (size_t)r.n * 8 * r.n_rhs;
  } else {
    // normal-matrix nonzeros: about half the row-merge candidates
    double cand = 0.0;
    for (long long i = 0; i < r.n_rows; ++i) {
      const double k = double(r.row_ptr[i + 1] - r.row_ptr[i]);
      cand += k * k;
    }
    nnz = r.least_squares ? (size_t)(0.5 * cand) : (size_t)r.row_ptr[r.n_rows];
    upload = (size_t)r.row_ptr[r.n_rows] * 24 + (size_t)r.n_rows * (16 + 8 * r.n_rhs) +
             (size_t)r.n_vars * 8 * r.n_rhs + (size_t)r.n * 8 * r.n_rhs;
  }
  const size_t mat = (size_t)(r.n + 1) * 4 + nnz * (12 + (mixed ? 4 : 0) + (dfl ? 8 : 0)) +
                     (size_t)r.n * (12 + (dfl ? 8 : 0));
  return mat + upload + (size_t)r.n_rhs * slot;
}

}  // namespace

struct nlgb_server_s {
  nlgb_server_config cfg;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::thread th;
  bool stop = false;
  bool aborting = false;
  Clock::time_point origin = Clock::now();
  long long next_id = 0;
  std::map<long long, std::unique_ptr<Req>> reqs;
  std::deque<Req*> incoming;
  // BATCHED: future / pending belong to the admission thread, active to the
  // worker; admitted requests pass from one to the other through `admitted`
  // (guarded by mu).  SERIAL: one thread owns them all.
  std::vector<Req*> future, pending, active;
  std::deque<Req*> admitted;
  std::condition_variable cv_admit;   // wakes the admission thread
  std::vector<std::thread> adm_th;
  int admitters_live = 0;
  bool admitter_done = false;         // every admission thread has exited
  long long sys_in_flight = 0;        // systems admitted or being admitted (guarded by mu)
  size_t used = 0;
  // statistics (guarded by mu)
  nlgb_server_stats st{};
  std::vector<double> latencies;
  double first_arrival = -1.0, last_done = 0.0;
  double t_used = 0.0;           // server time of the last change of `used`
  std::string fatal;
  int device = 0;                // the creator's current device (the worker uses it too)
  // Abort flag in pinned, mapped host memory: the guard kernel of a graph
  // executor polls it once per while-loop pass.
  volatile int* abort_host = nullptr;
  int* abort_dev = nullptr;
  // SRPT stream executor: one ChunkMirror per admitted system (pinned,
  // mapped; max_systems of them) and the free indices (guarded by mu)
  ChunkMirror* mirrors = nullptr;
  std::vector<int> mirror_free;
  // Requests whose systems are all done, handed by the worker to the
  // completion threads (result download, release; guarded by mu)
  std::deque<Req*> finished;
  std::condition_variable cv_complete;
  std::vector<std::thread> cmp_th;
  bool worker_done = false;
  // Chunk graphs of released requests.  Destroying an executable graph
  // waits for the device to be idle, which would stall every thread's CUDA
  // calls behind the chunks in flight; they are destroyed by the completion
  // threads when no chunk runs (or, past kGraveyardCap, the oldest ones
  // regardless).  Guarded by mu; lanes_busy is the worker's count of
  // chunks in flight.
  std::vector<std::unique_ptr<ViewGraph>> graveyard;
  std::atomic<int> lanes_busy{0};
  // Tracing (environment NLGB_SERVER_TRACE = path): CSV lines per epoch of
  // the persistent kernel ("E"), per chunk ("C"), per admission ("A"), per
  // completion ("D", "R") and one summary of the stream worker's host time
  // ("W"); the file starts with the column names.
  FILE* trace = nullptr;

  double now() const { return std::chrono::duration<double>(Clock::now() - origin).count(); }
};

namespace {

// Least-squares request: a row stream assembled into normal equations, or an
// LSCM mesh.
bool req_least_squares(const Req& r) {
  return (r.kind == 1 && r.least_squares) || (r.kind == 2 && r.mesh_kind == NLGB_MESH_LSCM);
}

// Precision of one request: NL_GB300_PRECISION_AUTO runs square systems in
// mixed precision and least-squares row submissions (normal equations,
// kappa(A^T A) = kappa(A)^2, too ill-conditioned for FP32 values on meshes)
// in FP64 from the start, instead of spending an FP32 phase before the
// fallback.  (Double-float is not chosen automatically: on the LSCM normal
// equations of large meshes it needs ~12 % more iterations than FP64 and
// ends with a true residual a few times above the threshold.)
int req_precision(const nlgb_server_s* S, const Req& r) {
  if (S->cfg.precision == NL_GB300_PRECISION_AUTO) {
    return req_least_squares(r) ? NL_GB300_PRECISION_DOUBLE : NL_GB300_PRECISION_MIXED;
  }
  return S->cfg.precision;
}
bool req_mixed(const nlgb_server_s* S, const Req& r) {
  return req_precision(S, r) == NL_GB300_PRECISION_MIXED;
}

// Device footprint admitted by the server: every change goes through here,
// so that the peak and the time integral stay exact.  add_used_locked: with
// S->mu held.
void add_used_locked(nlgb_server_s* S, long long delta) {
  const double t = S->now();
  S->st.byte_seconds += double(S->used) * std::max(0.0, t - S->t_used);
  S->t_used = t;
  if (delta < 0) S->used -= std::min<size_t>(S->used, (size_t)(-delta));
  else S->used += (size_t)delta;
  S->st.used_bytes = S->used;
  S->st.peak_bytes = std::max(S->st.peak_bytes, S->used);
}
void add_used(nlgb_server_s* S, long long delta) {
  std::lock_guard<std::mutex> lk(S->mu);
  add_used_locked(S, delta);
}

// Cost of one iteration of one system of r (bytes-equivalent): its
// algorithmic bytes, at least what a latency-bound iteration occupies (one
// CTA slot of the persistent kernel for ~15 us, at the HBM rate shared by
// ~608 slots: ~160 kB).
constexpr double kServiceFloorBytes = 1.6e5;
constexpr long long kProbeIters = 16;      // SRPT: first epoch of a new system
constexpr int kReserveCtas = 16;           // persistent-kernel slots left to system builds
constexpr long long kUnrollPlainIters = 4;  // a chunk pauses on whole passes of 4 iterations
constexpr int kAdmitters = 4;               // admission threads of the batched server
constexpr int kCompleters = 2;              // completion threads of the SRPT stream executor
constexpr size_t kGraveyardCap = 1024;      // chunk graphs kept for destruction at an idle moment
double iteration_cost(const Req& r, bool mixed) {
  const double n = double(r.A.n), z = double(r.A.nnz);
  const double b = mixed ? 8.0 * z + 56.0 * n : 12.0 * z + 108.0 * n;
  return std::max(b, kServiceFloorBytes);
}

SolveParams params_of(const nlgb_server_s* S, const Req& r, int precision) {
  SolveParams p;
  p.eps = (req_least_squares(r) && S->cfg.eps_least_squares > 0.0) ? S->cfg.eps_least_squares : S->cfg.eps;
  p.max_iter = S->cfg.max_iter;
  p.precision = precision;
  p.inner_eps = S->cfg.inner_eps;
  p.max_outer = 100000;
  return p;
}

// Upload / assemble a request on stream `s` and start its systems.
// df_slots: the slots run the double-float iteration in the persistent
// kernel (x packed as float pairs); the serial worker keeps FP64 slots and
// lets the single-system solver convert.
bool admit(nlgb_server_s* S, Req* r, cudaStream_t s, bool df_slots) {
  const int prec = req_precision(S, *r);
  const bool mixed = prec == NL_GB300_PRECISION_MIXED;
  cudaError_t e = cudaSuccess;
  if (r->kind == 0) {
    e = crs_upload(r->A, r->n, r->n, r->rp.data(), r->ci.data(), r->va.data(), s);
  } else if (r->kind == 2) {
    // build the system from the mesh on the GPU (right-hand sides: LSCM's
    // from the pins, fairing's given by the caller)
    bool bad = false;
    e = cudaMallocAsync((void**)&r->d_rhs, sizeof(double) * std::max<size_t>(1, (size_t)r->n_rhs * r->n), s);
    if (e == cudaSuccess && r->mesh_kind == NLGB_MESH_LSCM) {
      // (triangle indices were checked on the host at submission)
      e = build_lscm_system(r->n_verts, r->xyz.data(), r->n_tris, r->tris.data(), r->pins, r->pin_uv,
                            r->A, r->d_rhs, s, &bad, false);
    } else if (e == cudaSuccess) {
      e = build_fairing_system(r->n_verts, r->xyz.data(), r->n_tris, r->tris.data(), r->lambda, r->A, s,
                               &bad, false);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(r->d_rhs, r->b.data(), sizeof(double) * (size_t)r->n_rhs * r->n,
                            cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess && bad) {
      set_error("nlgb_server_submit_mesh: triangle index out of range");
      e = cudaErrorInvalidValue;
    }
  } else {
    long long* drp = nullptr; int* dcol = nullptr;
    double *dval = nullptr, *drhs = nullptr, *dw = nullptr, *dxl = nullptr;
    const long long nc = r->row_ptr[r->n_rows];
    auto up = [&](void** dst, const void* src, size_t bytes) {
      if (e != cudaSuccess) return;
      e = cudaMalloc(dst, std::max<size_t>(bytes, 8));
      if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, s);
    };
    up((void**)&drp, r->row_ptr.data(), sizeof(long long) * (r->n_rows + 1));
    up((void**)&dcol, r->col.data(), sizeof(int) * nc);
    up((void**)&dval, r->val.data(), sizeof(double) * nc);
    if (r->has_rhs) up((void**)&drhs, r->rhs.data(), sizeof(double) * r->rhs.size());
    if (r->has_weight) up((void**)&dw, r->weight.data(), sizeof(double) * r->weight.size());
    if (r->has_xl) up((void**)&dxl, r->xl.data(), sizeof(double) * r->xl.size());
    else up((void**)&dxl, nullptr, 0);
    if (e == cudaSuccess)
      e = cudaMallocAsync((void**)&r->d_rhs, sizeof(double) * std::max<size_t>(1, (size_t)r->n_rhs * r->n), s);
    if (e == cudaSuccess) {
      LSRowsDevice R;
      R.n_rows = r->n_rows; R.n_coefs = nc; R.n_free = r->n; R.n_vars = r->n_vars;
      R.n_systems = r->n_rhs; R.row_ptr = drp; R.col = dcol; R.val = dval;
      R.rhs = r->has_rhs ? drhs : nullptr; R.weight = r->has_weight ? dw : nullptr; R.xl = dxl;
      e = r->least_squares ? assemble_normal_equations(R, r->A, r->d_rhs, s)
                           : assemble_square(R, r->A, r->d_rhs, s);
    }
    cudaStreamSynchronize(s);
    cudaFree(drp); cudaFree(dcol); cudaFree(dval); cudaFree(drhs); cudaFree(dw); cudaFree(dxl);
  }
  r->t_built = S->now();
  if (e == cudaSuccess) e = crs_prepare(r->A, mixed, s);
  // throughput tiling of the batched server (config.min_tile_rows): set
  // before any slot, graph or plan reads the layout
  if (e == cudaSuccess && S->cfg.mode == NLGB_SERVER_BATCHED && S->cfg.min_tile_rows > r->A.tile_rows)
    r->A.tile_rows = S->cfg.min_tile_rows;
  r->t_prepared = S->now();
  bool dfl = false;   // false also when the matrix is outside double-float's range: FP64 runs
  if (e == cudaSuccess && prec == NL_GB300_PRECISION_DOUBLE_FLOAT) e = crs_prepare_df(r->A, &dfl, s);
  if (e == cudaSuccess) {
    // true footprint now known
    const size_t actual = (size_t)device_bytes(r->A) + (size_t)r->n_rhs * SystemSlot::bytes_for(r->n, r->A.tile_rows, mixed);
    add_used(S, (long long)actual - (long long)r->bytes);
    r->bytes = actual;
    r->iter_cost = iteration_cost(*r, mixed);
    r->slots.resize((size_t)r->n_rhs);
    const SolveParams prm = params_of(S, *r, prec);
    for (int k = 0; k < r->n_rhs && e == cudaSuccess; ++k) {
      e = r->slots[k].alloc(&r->A, mixed, s, dfl && df_slots);
      if (e != cudaSuccess) break;
      r->slots[k].view.abort_flag = S->abort_dev;
      const double* bk = r->kind == 0 ? r->b.data() + (size_t)k * r->n : r->d_rhs + (size_t)k * r->n;
      const double* xk = r->x0.empty() ? nullptr : r->x0.data() + (size_t)k * r->n;
      e = r->slots[k].start(bk, xk, prm, s);
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  // host inputs are no longer needed
  std::vector<int>().swap(r->rp); std::vector<int>().swap(r->ci); std::vector<double>().swap(r->va);
  std::vector<double>().swap(r->b); std::vector<double>().swap(r->x0);
  std::vector<long long>().swap(r->row_ptr); std::vector<int>().swap(r->col);
  std::vector<double>().swap(r->val); std::vector<double>().swap(r->rhs);
  std::vector<double>().swap(r->weight); std::vector<double>().swap(r->xl);
  std::vector<double>().swap(r->xyz); std::vector<int>().swap(r->tris);
  if (e != cudaSuccess) {
    r->error = std::string("admission failed: ") + last_error();
    return false;
  }
  r->sys_done.assign((size_t)r->n_rhs, 0);
  r->sys_stage.assign((size_t)r->n_rhs, 0);
  r->sys_iter.assign((size_t)r->n_rhs, 0);
  r->rr_first.assign((size_t)r->n_rhs, 0.0);
  r->rr_prev.assign((size_t)r->n_rhs, 0.0);
  r->est_left.assign((size_t)r->n_rhs, -1.0);
  r->it_prev.assign((size_t)r->n_rhs, 0);
  r->running.assign((size_t)r->n_rhs, 0);
  r->need_fallback.assign((size_t)r->n_rhs, 0);
  r->ms_per_iter.assign((size_t)r->n_rhs, -1.0);
  r->mixed_now.assign((size_t)r->n_rhs, 0);
  for (int k = 0; k < r->n_rhs; ++k) r->mixed_now[k] = r->slots[k].mixed ? 1 : 0;
  r->res.assign((size_t)r->n_rhs, nlgb_result{});
  return true;
}

// Stream-ordered release of a request's device memory (no device-wide
// synchronisation: the solver's other streams keep running).
void release(nlgb_server_s* S, Req* r, cudaStream_t s) {
  const double t0 = S->trace ? S->now() : 0.0;
  for (auto& sl : r->slots) sl.release(s);
  r->slots.clear();
  const double t1 = S->trace ? S->now() : 0.0;
  if (!r->graphs.empty()) {
    std::lock_guard<std::mutex> lk(S->mu);
    for (auto& g : r->graphs)
      if (g) S->graveyard.push_back(std::move(g));
  }
  r->graphs.clear();
  if (S->trace) std::fprintf(S->trace, "R,%.6f,%lld,%.6f,%.6f\n", S->now(), r->id, t1 - t0, S->now() - t1);
  if (!r->mirror_idx.empty()) {
    std::lock_guard<std::mutex> lk(S->mu);
    for (int i : r->mirror_idx) S->mirror_free.push_back(i);
    r->mirror_idx.clear();
  }
  crs_free_async(r->A, s);
  if (r->d_rhs) cudaFreeAsync(r->d_rhs, s);
  r->d_rhs = nullptr;
  add_used(S, -(long long)r->bytes);
  r->bytes = 0;
}

void finish_request(nlgb_server_s* S, Req* r, bool ok) {
  if (r->status == NL_GB300_STATUS_ABORTED) {
    ok = false;
    if (r->error.empty()) r->error = "aborted by nlgb_server_abort";
  }
  std::lock_guard<std::mutex> lk(S->mu);
  r->t_done = S->now();
  r->state = ok ? R_DONE : R_FAILED;
  if (ok) {
    S->st.completed += 1;
    S->latencies.push_back(r->t_done - r->arrival);
    S->last_done = std::max(S->last_done, r->t_done);
    for (auto& x : r->res) {
      S->st.iterations += x.iterations;
      S->st.algo_bytes += x.algo_bytes;
    }
  } else {
    S->st.failed += 1;
  }
  S->cv_done.notify_all();
}

void fill_result(nlgb_result& o, const SysState& h, double secs, long long n, long long nnz,
                 int precision) {
  o.algo_bytes = algo_bytes(n, nnz, h);
  o.precision = precision;
  o.status = h.status;
  o.iterations = h.iter;
  o.refinement_steps = h.outer;
  o.rel_residual = h.bnorm2 > 0 ? std::sqrt(h.rr / h.bnorm2) : 0.0;
  o.true_rel_residual = h.bnorm2 > 0 ? std::sqrt(h.rr_true / h.bnorm2) : 0.0;
  o.seconds = secs;
}

// Move submissions into the worker's lists and arrived requests to pending.
// Returns false when the server is stopping and has nothing left.
bool intake(nlgb_server_s* S, bool block_if_idle) {
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    while (!S->incoming.empty()) {
      S->future.push_back(S->incoming.front());
      S->incoming.pop_front();
    }
    const double t = S->now();
    std::stable_sort(S->future.begin(), S->future.end(),
                     [](const Req* a, const Req* b) { return a->arrival < b->arrival; });
    size_t k = 0;
    while (k < S->future.size() && S->future[k]->arrival <= t) {
      S->future[k]->state = R_PENDING;
      S->pending.push_back(S->future[k]);
      ++k;
    }
    S->future.erase(S->future.begin(), S->future.begin() + (long)k);
    const bool idle = S->active.empty() && S->pending.empty();
    // aborting: hand back control so queued requests are failed at once
    if (S->aborting && !S->future.empty()) return true;
    if (!idle || !block_if_idle) return true;
    if (S->future.empty()) {
      if (S->stop) return false;
      // nothing queued: sleep until a submission or shutdown
      S->cv_work.wait(lk, [&] { return S->stop || !S->incoming.empty(); });
    } else {
      const double wait_s = std::max(0.0, S->future.front()->arrival - S->now());
      S->cv_work.wait_for(lk, std::chrono::duration<double>(wait_s),
                          [&] { return S->stop || S->aborting || !S->incoming.empty(); });
    }
  }
}

void fail_all_waiting(nlgb_server_s* S, const char* why) {
  std::vector<Req*> drop;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    for (Req* r : S->pending) drop.push_back(r);
    for (Req* r : S->future) drop.push_back(r);
    for (Req* r : S->incoming) drop.push_back(r);
    S->pending.clear(); S->future.clear(); S->incoming.clear();
  }
  for (Req* r : drop) {
    r->error = why;
    r->status = NL_GB300_STATUS_ABORTED;
    finish_request(S, r, false);
  }
}

// Copy a finished request's solutions to the caller's buffer, release its
// device memory and report it.
void complete_request(nlgb_server_s* S, Req* r, cudaStream_t su) {
  bool ok = true;
  const double t0 = S->trace ? S->now() : 0.0;
  for (int k = 0; k < r->n_rhs; ++k) {
    if (r->res[k].status == NL_GB300_STATUS_ABORTED) continue;   // nothing to return
    if (r->slots[k].df && df_unpack(r->slots[k].view.x, r->n, su) != cudaSuccess) ok = false;
    if (cudaMemcpyAsync(r->x_out + (size_t)k * r->n, r->slots[k].view.x, sizeof(double) * r->n,
                        cudaMemcpyDeviceToHost, su) != cudaSuccess) ok = false;
  }
  for (int k = 0; k < r->n_rhs; ++k)
    if (r->res[k].status != NL_GB300_STATUS_CONVERGED && r->status != NL_GB300_STATUS_ABORTED)
      r->status = r->res[k].status;
  cudaStreamSynchronize(su);
  if (r->status == NL_GB300_STATUS_NONE) r->status = NL_GB300_STATUS_CONVERGED;
  const double t1 = S->trace ? S->now() : 0.0;
  release(S, r, su);
  if (S->trace)
    std::fprintf(S->trace, "D,%.6f,%lld,%d,%.6f,%.6f\n", S->now(), r->id, r->n, t1 - t0, S->now() - t1);
  finish_request(S, r, ok);
}

// Iterations a system still needs, from its residual history: the slower
// of the average reduction rate since the start and the rate over the last
// epoch, extrapolated to the threshold (CG's residual is not monotone; the
// slower rate errs on the side of more work).
double estimate_left(Req* r, int k, const SysState& h) {
  if (h.bnorm2 <= 0.0 || h.iter <= 0) return -1.0;
  if (r->rr_first[k] <= 0.0) r->rr_first[k] = h.bnorm2;   // zero initial guess: ||r0|| = ||b||
  const double rr = std::max(h.rr, 1e-300);
  const double target = std::max((h.precision == 1 ? h.thresh2 : h.rthresh2) * h.bnorm2, 1e-300);
  const double left_max = double(std::max(1LL, h.max_iter - h.iter));
  double rate = std::log(rr / r->rr_first[k]) / double(h.iter);
  const long long dk = h.iter - r->it_prev[k];
  if (r->it_prev[k] > 0 && dk >= 8 && r->rr_prev[k] > 0.0)
    rate = std::max(rate, std::log(rr / r->rr_prev[k]) / double(dk));
  r->it_prev[k] = h.iter;
  r->rr_prev[k] = rr;
  if (rr <= target) return 1.0;
  if (!(rate < -1e-9)) return left_max;
  return std::min(left_max, std::max(1.0, std::log(target / rr) / rate));
}

// Admission thread of the BATCHED server: arrived requests are admitted in
// arrival order, first fit against the HBM budget, each uploaded and built
// (or assembled) on this thread's stream while the worker's epochs run (the
// persistent kernel leaves kReserveCtas slots for these kernels); admitted
// requests join the next epoch.
void admitter(nlgb_server_s* S) {
  cudaSetDevice(S->device);
  // Builds run at the highest stream priority: their kernels are short and
  // the solver's streams keep the GPU busy; at the default priority every
  // host synchronisation of a build would wait behind queued solver work.
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  cudaStream_t su = nullptr;
  cudaStreamCreateWithPriority(&su, cudaStreamNonBlocking, greatest);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    while (!S->incoming.empty()) {
      S->future.push_back(S->incoming.front());
      S->incoming.pop_front();
    }
    if (S->aborting || !S->fatal.empty()) {
      std::vector<Req*> drop(S->pending.begin(), S->pending.end());
      drop.insert(drop.end(), S->future.begin(), S->future.end());
      S->pending.clear();
      S->future.clear();
      lk.unlock();
      for (Req* r : drop) {
        r->error = S->fatal.empty() ? "server aborted" : S->fatal;
        r->status = NL_GB300_STATUS_ABORTED;
        finish_request(S, r, false);
      }
      lk.lock();
      if (S->stop) break;
      S->cv_admit.wait_for(lk, std::chrono::milliseconds(50));
      continue;
    }
    const double t = S->now();
    std::stable_sort(S->future.begin(), S->future.end(),
                     [](const Req* a, const Req* b) { return a->arrival < b->arrival; });
    size_t j = 0;
    while (j < S->future.size() && S->future[j]->arrival <= t) {
      S->future[j]->state = R_PENDING;
      S->pending.push_back(S->future[j]);
      ++j;
    }
    S->future.erase(S->future.begin(), S->future.begin() + (long)j);
    // SRPT schedule: of the arrived requests that fit the HBM budget, the
    // one with the least estimated work (its footprint, which scales with
    // the bytes of an iteration, times sqrt(n) for the O(sqrt(n)) Jacobi-CG
    // iterations of a 2D mesh operator); under overload the budget then
    // holds the requests that can finish soonest instead of the oldest.
    // ALL schedule: first fit in arrival order.
    const bool shortest = S->cfg.schedule == NLGB_SCHEDULE_SRPT;
    Req* pick = nullptr;
    size_t pick_i = 0;
    double pick_key = 0.0;
    for (size_t i = 0; i < S->pending.size(); ++i) {
      Req* r = S->pending[i];
      if (S->used + r->bytes > S->cfg.hbm_budget_bytes || S->sys_in_flight + r->n_rhs > S->cfg.max_systems)
        continue;
      const double key = double(r->bytes) * std::sqrt(double(std::max(1, r->n)));
      if (!pick || (shortest && key < pick_key)) {
        pick = r;
        pick_i = i;
        pick_key = key;
        if (!shortest) break;
      }
    }
    if (pick) S->pending.erase(S->pending.begin() + (long)pick_i);
    if (pick) {
      add_used_locked(S, (long long)pick->bytes);
      S->sys_in_flight += pick->n_rhs;
      lk.unlock();
      const double ta = S->now();
      bool ok = admit(S, pick, su, true);
      const double tg = S->now();
      if (ok && S->cfg.schedule == NLGB_SCHEDULE_SRPT) {
        // instantiate the chunk graphs here, off the worker's path; each
        // system reports its chunks through its own mirror (the pool holds
        // max_systems, and sys_in_flight counted this request's systems)
        {
          std::lock_guard<std::mutex> g(S->mu);
          for (int k = 0; k < pick->n_rhs && !S->mirror_free.empty(); ++k) {
            pick->mirror_idx.push_back(S->mirror_free.back());
            S->mirror_free.pop_back();
          }
        }
        ok = (int)pick->mirror_idx.size() == pick->n_rhs;
        pick->graphs.resize((size_t)pick->n_rhs);
        for (int k = 0; k < pick->n_rhs && ok; ++k) {
          ChunkMirror* m = &S->mirrors[pick->mirror_idx[k]];
          m->budget = 0;
          pick->graphs[k].reset(new ViewGraph());
          ok = pick->graphs[k]->prepare(pick->slots[k].view, pick->slots[k].mixed, m, su) == cudaSuccess;
        }
        if (ok) ok = cudaStreamSynchronize(su) == cudaSuccess;
        if (!ok) pick->error = std::string("admission failed: ") + last_error();
      }
      const double tb = S->now();
      if (S->trace)
        std::fprintf(S->trace, "A,%.6f,%lld,%d,%d,%.6f,%zu,%.6f,%.6f,%.6f,%.6f\n", ta, pick->id,
                     pick->kind == 2 ? pick->mesh_kind : -1, pick->n, tb - ta, pick->bytes, pick->arrival, tb - tg,
                     pick->t_built - ta, pick->t_prepared - pick->t_built);
      if (!ok) {
        release(S, pick, su);
        {
          std::lock_guard<std::mutex> g(S->mu);
          S->sys_in_flight -= pick->n_rhs;
        }
        finish_request(S, pick, false);
      }
      lk.lock();
      if (ok) {
        pick->state = R_ACTIVE;
        S->admitted.push_back(pick);
        S->cv_work.notify_all();
      }
      continue;
    }
    if (S->stop && S->future.empty() && S->pending.empty() && S->incoming.empty()) break;
    // nothing admissible: wait for a submission, an arrival, freed memory or shutdown
    double wait_s = 0.05;
    if (!S->future.empty()) wait_s = std::min(wait_s, std::max(0.0, S->future.front()->arrival - S->now()));
    S->cv_admit.wait_for(lk, std::chrono::duration<double>(wait_s));
  }
  if (--S->admitters_live == 0) S->admitter_done = true;
  S->cv_work.notify_all();
  S->cv_admit.notify_all();
  lk.unlock();
  cudaStreamSynchronize(su);
  cudaStreamDestroy(su);
}

void worker_batched(nlgb_server_s* S) {
  cudaSetDevice(S->device);
  cudaStream_t sc = nullptr, su = nullptr;
  cudaStreamCreateWithFlags(&sc, cudaStreamNonBlocking);
  cudaStreamCreateWithFlags(&su, cudaStreamNonBlocking);
  BatchRunner runner;
  if (runner.init(sc) != cudaSuccess) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->fatal = last_error();
    S->cv_admit.notify_all();
  }
  const bool srpt = S->cfg.schedule == NLGB_SCHEDULE_SRPT;
  const unsigned long long epoch_ns = S->cfg.epoch_ms > 0.0 ? (unsigned long long)(S->cfg.epoch_ms * 1e6) : 0ULL;
  runner.set_priority_plan(srpt);
  runner.set_epoch_ns(srpt ? epoch_ns : 0ULL);
  runner.set_reserve(kReserveCtas);
  if (S->trace) runner.set_timing(true);
  std::vector<SysState> states;
  std::vector<std::pair<Req*, int>> owner;   // system index -> (request, rhs)
  std::vector<std::unique_ptr<ViewGraph>> solos;   // graph executors of large systems
  auto finish_abort_all = [&]() {
    for (Req* r : S->active) {
      for (int k = 0; k < r->n_rhs; ++k)
        if (!r->sys_done[k]) {
          r->sys_done[k] = 1;
          r->res[k].status = NL_GB300_STATUS_ABORTED;
          r->res[k].iterations = r->sys_iter[k];   // as of the last epoch boundary
        }
      r->status = NL_GB300_STATUS_ABORTED;
      complete_request(S, r, su);
      std::lock_guard<std::mutex> lk(S->mu);
      S->sys_in_flight -= r->n_rhs;
    }
    S->active.clear();
  };
  while (S->fatal.empty()) {
    {
      std::unique_lock<std::mutex> lk(S->mu);
      while (!S->admitted.empty()) {
        S->active.push_back(S->admitted.front());
        S->admitted.pop_front();
      }
      if (S->active.empty()) {
        if (S->admitter_done) break;
        S->cv_work.wait_for(lk, std::chrono::milliseconds(50),
                            [&] { return !S->admitted.empty() || S->admitter_done || S->aborting; });
        if (!S->aborting) continue;
      }
    }
    if (S->aborting) {
      // active requests stop here (between epochs); the admission thread
      // fails the queued ones
      finish_abort_all();
      S->cv_admit.notify_all();
      std::unique_lock<std::mutex> lk(S->mu);
      if (S->admitter_done && S->admitted.empty()) break;
      S->cv_work.wait_for(lk, std::chrono::milliseconds(20));
      continue;
    }
    // The systems of this epoch.  SRPT: every active system, in order of
    // estimated remaining work (iterations left x bytes per iteration); a
    // system without an estimate yet comes first with a probe budget of
    // kProbeIters iterations; the launch is time-boxed to epoch_ms and the
    // plan gives teams in that order.  ALL: every system, epoch_iters
    // iterations, work-proportional teams.
    struct Cand { Req* r; int k; double key; };
    std::vector<Cand> cands;
    for (Req* r : S->active)
      for (int k = 0; k < r->n_rhs; ++k)
        if (!r->sys_done[k])
          cands.push_back({r, k, r->est_left[k] < 0.0 ? -1.0 : r->est_left[k] * r->iter_cost});
    if (srpt)
      std::stable_sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) {
        return a.key != b.key ? a.key < b.key : a.r->id < b.r->id;
      });
    std::vector<SysView> views;
    std::vector<long long> work;
    owner.clear();
    for (const Cand& c : cands) {
      SysView v = c.r->slots[c.k].view;
      v.budget = srpt ? (c.key < 0.0 ? kProbeIters : (epoch_ns ? 0 : S->cfg.epoch_iters)) : S->cfg.epoch_iters;
      views.push_back(v);
      work.push_back((long long)std::min(9.0e18, c.r->iter_cost * double(S->cfg.epoch_iters)));
      owner.push_back({c.r, c.k});
    }
    BatchLaunchStats bst;
    const double t_epoch0 = S->now();
    // When the epoch's systems are all large FP64 ones (at most
    // kMaxGraphSystems), each continues on its own graph executor, one after
    // the other in the epoch: faster per iteration than sharing the
    // persistent kernel once each fills the GPU alone (same iterates, see
    // ViewGraph).
    bool graph_epoch = !views.empty() && views.size() <= kMaxGraphSystems;
    for (size_t i = 0; graph_epoch && i < views.size(); ++i) {
      const Req* r = owner[i].first;
      const int k = owner[i].second;
      graph_epoch = !req_mixed(S, *r) && views[i].n_tiles >= kGraphMinTiles && r->sys_stage[k] == 1 &&
                    r->est_left[k] >= 0.0;
    }
    cudaError_t e = cudaSuccess;
    if (graph_epoch) {
      while (solos.size() < views.size()) solos.emplace_back(new ViewGraph());
      std::vector<float> gms(views.size(), 0.f);
      std::vector<long long> before(views.size());
      for (size_t i = 0; i < views.size() && e == cudaSuccess; ++i) {
        before[i] = owner[i].first->sys_iter[owner[i].second];
        // a chunk of about epoch_ms at ~2.8 TB/s, in whole passes of 4
        long long it = S->cfg.epoch_iters;
        if (srpt && epoch_ns) {
          const double per = owner[i].first->iter_cost / 2.8e12;
          it = std::max<long long>(16, std::min<long long>(4096, (long long)(double(epoch_ns) * 1e-9 / per)));
        }
        e = solos[i]->run(views[i], it, sc, &gms[i]);
      }
      if (e == cudaSuccess) {
        states.resize(views.size());
        for (size_t i = 0; i < views.size() && e == cudaSuccess; ++i)
          e = cudaMemcpyAsync(&states[i], views[i].st, sizeof(SysState), cudaMemcpyDeviceToHost, sc);
      }
      if (e == cudaSuccess) e = cudaStreamSynchronize(sc);
      double total_ms = 0.0, bytes = 0.0;
      for (size_t i = 0; i < views.size() && e == cudaSuccess; ++i) {
        e = solos[i]->finish(before[i], states[i].iter);
        total_ms += gms[i];
        const Req* r = owner[i].first;
        bytes += double(states[i].iter - before[i]) * (12.0 * double(r->A.nnz) + 108.0 * double(r->A.n));
      }
      bst.ms = total_ms;
      if (e == cudaSuccess) {
        std::lock_guard<std::mutex> lk(S->mu);
        S->st.graph_s += total_ms * 1e-3;
        S->st.graph_epochs += 1;
        S->st.graph_algo_bytes += bytes;
      }
    } else {
      e = runner.launch(views, work, srpt && epoch_ns ? 0 : S->cfg.epoch_iters);
      if (e == cudaSuccess) e = runner.finish(&bst);
      if (e == cudaSuccess) {
        states.resize(views.size());
        e = runner.gather_states(states.data(), (int)views.size());
      }
    }
    if (e != cudaSuccess) {
      std::lock_guard<std::mutex> lk(S->mu);
      S->fatal = last_error();
      S->cv_admit.notify_all();
      break;
    }
    double done_bytes = 0.0, done_algo = 0.0;
    for (size_t i = 0; i < views.size(); ++i) {
      const Req* r = owner[i].first;
      const long long di = states[i].iter - r->sys_iter[owner[i].second];
      done_bytes += double(di) * r->iter_cost;
      done_algo += double(di) * (r->slots[owner[i].second].mixed ? 8.0 * double(r->A.nnz) + 56.0 * double(r->A.n)
                                                                  : 12.0 * double(r->A.nnz) + 108.0 * double(r->A.n));
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->st.kernel_s += bst.ms * 1e-3;
      S->st.epochs += 1;
      S->st.epoch_algo_bytes += done_algo;
    }
    if (S->trace) {
      double tmin = 0.0, tmed = 0.0, tmax = 0.0, tq = 0.0;
      const std::vector<unsigned long long>& tt = runner.last_times();
      if (!graph_epoch && tt.size() >= 2 && tt[0] > 0) {
        std::vector<double> te;
        for (size_t t = 2; t < tt.size(); ++t)
          if (tt[t] > 0) te.push_back(1e-6 * double(tt[t] - tt[0]));
        std::sort(te.begin(), te.end());
        if (!te.empty()) { tmin = te.front(); tmed = te[te.size() / 2]; tmax = te.back(); }
        if (tt[1] > 0) tq = 1e-6 * double(tt[1] - tt[0]);
      }
      std::fprintf(S->trace, "E,%.6f,%.6f,%s,%zu,%d,%d,%d,%d,%.3f,%.3f,%.3f,%.3f,%.3f,%.3f,%.3f,%d,%.6f,%zu\n",
                   t_epoch0, S->now(), graph_epoch ? "graph" : "batch", views.size(), bst.n_teams, bst.team_ctas,
                   bst.queue_ctas, bst.grid, done_algo * 1e-9, done_bytes * 1e-9, bst.ms, tmin, tmed, tmax, tq,
                   0, 0.0, S->active.size());
    }
    for (size_t i = 0; i < views.size(); ++i) {
      Req* r = owner[i].first;
      const int k = owner[i].second;
      r->est_left[k] = estimate_left(r, k, states[i]);
      r->sys_stage[k] = states[i].stage;
      r->sys_iter[k] = states[i].iter;
      if (states[i].stage == 3) {
        r->sys_done[k] = 1;
        fill_result(r->res[k], states[i], bst.ms * 1e-3, r->A.n, r->A.nnz,
                    r->slots[k].mixed ? NL_GB300_PRECISION_MIXED
                                      : (r->slots[k].df ? NL_GB300_PRECISION_DOUBLE_FLOAT
                                                        : NL_GB300_PRECISION_DOUBLE));
      }
    }
    bool freed = false;
    for (size_t i = 0; i < S->active.size();) {
      Req* r = S->active[i];
      bool all = true;
      for (int d : r->sys_done) all = all && d;
      if (!all) { ++i; continue; }
      S->active.erase(S->active.begin() + (long)i);
      complete_request(S, r, su);
      {
        std::lock_guard<std::mutex> lk(S->mu);
        S->sys_in_flight -= r->n_rhs;
      }
      freed = true;
    }
    if (freed) S->cv_admit.notify_all();
  }
  if (!S->fatal.empty()) {
    for (Req* r : S->active) { r->error = S->fatal; release(S, r, su); finish_request(S, r, false); }
    S->active.clear();
    std::unique_lock<std::mutex> lk(S->mu);
    S->cv_admit.notify_all();
    // requests the admission thread hands over from now on fail too
    while (!S->admitter_done || !S->admitted.empty()) {
      while (!S->admitted.empty()) {
        Req* r = S->admitted.front();
        S->admitted.pop_front();
        lk.unlock();
        r->error = S->fatal;
        release(S, r, su);
        finish_request(S, r, false);
        lk.lock();
      }
      if (!S->admitter_done) S->cv_work.wait_for(lk, std::chrono::milliseconds(20));
    }
  }
  cudaStreamSynchronize(sc);
  cudaStreamDestroy(sc);
  cudaStreamDestroy(su);
}

// SRPT executor of the BATCHED server: `streams` CUDA streams, each running
// one system at a time as a chunk of CUDA-graph iterations (ViewGraph) of
// about epoch_ms.  Whenever a stream is free it takes the system with the
// least estimated remaining work that is not running already (a new system
// first, for a probe of kProbeIters iterations).  A system's chunks run one
// after the other (the next one is queued only after the previous one was
// seen to finish), so its iterates are those of the single-system solver.
// A lane's chunk has ended once its mirror's sequence number moved.
inline unsigned int mirror_seq(const ChunkMirror* m) {
  return __atomic_load_n(&m->seq, __ATOMIC_ACQUIRE);
}

// Completion thread of the SRPT stream executor: downloads the results of
// requests whose systems are all done, releases their memory
// (stream-ordered) and wakes the admission threads; the worker only hands
// them over, so that its chunk launches never wait on these copies.
void completer(nlgb_server_s* S) {
  cudaSetDevice(S->device);
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  cudaStream_t su = nullptr;
  cudaStreamCreateWithPriority(&su, cudaStreamNonBlocking, greatest);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    // destroy the chunk graphs of released requests while no chunk runs,
    // or the oldest ones once there are too many
    size_t n_bury = 0;
    if (S->lanes_busy.load() == 0) n_bury = S->graveyard.size();
    else if (S->graveyard.size() > kGraveyardCap) n_bury = S->graveyard.size() - kGraveyardCap / 2;
    if (n_bury > 0) {
      std::vector<std::unique_ptr<ViewGraph>> bury;
      bury.reserve(n_bury);
      for (size_t i = 0; i < n_bury; ++i) bury.push_back(std::move(S->graveyard[i]));
      S->graveyard.erase(S->graveyard.begin(), S->graveyard.begin() + (long)n_bury);
      lk.unlock();
      bury.clear();
      lk.lock();
      continue;
    }
    if (S->finished.empty()) {
      if (S->worker_done) break;
      S->cv_complete.wait_for(lk, std::chrono::milliseconds(50));
      continue;
    }
    Req* r = S->finished.front();
    S->finished.pop_front();
    lk.unlock();
    complete_request(S, r, su);
    lk.lock();
    S->sys_in_flight -= r->n_rhs;
    S->cv_admit.notify_all();
  }
  lk.unlock();
  cudaStreamSynchronize(su);
  cudaStreamDestroy(su);
}

void worker_streams(nlgb_server_s* S) {
  cudaSetDevice(S->device);
  const int ns = std::max(1, S->cfg.streams > 0 ? S->cfg.streams : 16);
  struct Lane {
    cudaStream_t s = nullptr;
    ChunkMirror* m = nullptr;   // the running system's mirror
    unsigned int seq0 = 0;      // its sequence number before the chunk
    Req* r = nullptr;
    int k = -1;
    long long iter_before = 0;
    double t_free = -1.0;       // server clock when the lane's last chunk was seen done (tracing)
    long long ctas = 0;         // CTAs per phase kernel of the running system
  };
  std::vector<Lane> lanes((size_t)ns);
  // CTA budget of the chunks in flight (config.chunk_cta_budget; 0: none)
  const long long cta_cap = S->cfg.chunk_cta_budget < 0 ? phase_resident_slots()
                                                        : (long long)S->cfg.chunk_cta_budget;
  long long running_ctas = 0;
  auto ctas_of = [](const Req* r) {
    return ((long long)r->A.n + r->A.tile_rows - 1) / std::max(1, r->A.tile_rows);
  };
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  cudaStream_t su = nullptr;   // aborts and failures: result downloads and releases
  cudaStreamCreateWithPriority(&su, cudaStreamNonBlocking, greatest);
  bool init_ok = true;
  for (Lane& l : lanes) init_ok = init_ok && cudaStreamCreateWithFlags(&l.s, cudaStreamNonBlocking) == cudaSuccess;
  if (!init_ok) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->fatal = std::string("server streams: ") + cudaGetErrorString(cudaGetLastError());
    S->cv_admit.notify_all();
  }
  const double target_ms = S->cfg.epoch_ms > 0.0 ? S->cfg.epoch_ms : 10.0;
  // host time of the worker's loop by part (tracing): retiring chunks,
  // completing requests, launching chunks (of which the graph launches),
  // waiting; and the time lanes sat finished before their next launch
  double w_retire = 0.0, w_complete = 0.0, w_launch = 0.0, w_run = 0.0, w_wait = 0.0, w_gap = 0.0;
  long long w_loops = 0, w_launches = 0;
  int n_busy = 0;
  double t_busy0 = 0.0;
  auto busy_change = [&](int delta) {
    const double t = S->now();
    if (n_busy > 0 && delta != 0) {
      std::lock_guard<std::mutex> lk(S->mu);
      S->st.kernel_s += t - t_busy0;
    }
    t_busy0 = t;
    n_busy += delta;
    S->lanes_busy.store(n_busy);
    if (n_busy == 0) S->cv_complete.notify_all();   // an idle moment for the graveyard
  };
  auto finish_abort_all = [&]() {
    for (Req* r : S->active) {
      for (int k = 0; k < r->n_rhs; ++k)
        if (!r->sys_done[k]) {
          r->sys_done[k] = 1;
          r->res[k].status = NL_GB300_STATUS_ABORTED;
          r->res[k].iterations = r->sys_iter[k];
        }
      r->status = NL_GB300_STATUS_ABORTED;
      complete_request(S, r, su);
      std::lock_guard<std::mutex> lk(S->mu);
      S->sys_in_flight -= r->n_rhs;
    }
    S->active.clear();
  };
  // one finished chunk: results, estimates, completion
  auto retire = [&](Lane& l) {
    Req* r = l.r;
    const int k = l.k;
    const SysState h = l.m->st;
    const float ms = float(double(l.m->t_ns) * 1e-6);
    r->graphs[k]->account(l.iter_before, h.iter);
    const long long di = h.iter - l.iter_before;
    const bool mixed_chunk = r->mixed_now[k] != 0;
    const double bytes_it = mixed_chunk ? 8.0 * double(r->A.nnz) + 56.0 * double(r->A.n)
                                        : 12.0 * double(r->A.nnz) + 108.0 * double(r->A.n);
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->st.epochs += 1;
      S->st.graph_epochs += 1;
      S->st.graph_s += ms * 1e-3;
      S->st.epoch_algo_bytes += double(di) * bytes_it;
      if (!mixed_chunk) S->st.graph_algo_bytes += double(di) * bytes_it;
    }
    if (S->trace)
      std::fprintf(S->trace, "C,%.6f,%lld,%d,%d,%lld,%lld,%.3f,%d,%d\n", S->now(), r->id, k, mixed_chunk ? 1 : 0,
                   l.iter_before, h.iter, ms, h.status, h.stage);
    if (di > 0) r->ms_per_iter[k] = double(ms) / double(di);
    r->est_left[k] = estimate_left(r, k, h);
    r->sys_stage[k] = h.stage;
    r->sys_iter[k] = h.iter;
    r->running[k] = 0;
    if (mixed_chunk && h.status == ST_STAGNATION && !h.fell_back && h.precision == 1) {
      // FP32 cannot track this system: it continues in FP64 from its x
      r->need_fallback[k] = 1;
      r->mixed_now[k] = 0;
      r->sys_stage[k] = 0;
    } else if (h.stage == 3) {
      r->sys_done[k] = 1;
      fill_result(r->res[k], h, ms * 1e-3, r->A.n, r->A.nnz,
                  r->slots[k].mixed ? NL_GB300_PRECISION_MIXED
                                    : (r->slots[k].df ? NL_GB300_PRECISION_DOUBLE_FLOAT
                                                      : NL_GB300_PRECISION_DOUBLE));
    }
    l.r = nullptr;
    l.k = -1;
    l.m = nullptr;
    running_ctas -= l.ctas;
    l.ctas = 0;
    busy_change(-1);
  };
  // requests whose systems are all done go to the completion threads
  auto hand_over_finished = [&]() {
    bool any = false;
    for (size_t i = 0; i < S->active.size();) {
      Req* r = S->active[i];
      bool all = true;
      for (int k = 0; k < r->n_rhs; ++k) all = all && r->sys_done[k] && !r->running[k];
      if (!all) { ++i; continue; }
      S->active.erase(S->active.begin() + (long)i);
      std::lock_guard<std::mutex> lk(S->mu);
      S->finished.push_back(r);
      any = true;
    }
    if (any) S->cv_complete.notify_all();
  };
  while (S->fatal.empty()) {
    bool have_admitted = false;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      while (!S->admitted.empty()) {
        S->active.push_back(S->admitted.front());
        S->admitted.pop_front();
        have_admitted = true;
      }
      if (S->active.empty() && n_busy == 0) {
        if (S->admitter_done) break;
        S->cv_work.wait_for(lk, std::chrono::milliseconds(50),
                            [&] { return !S->admitted.empty() || S->admitter_done || S->aborting; });
        if (!S->aborting) continue;
      }
    }
    // retire finished chunks
    bool progress = have_admitted;
    double tw = S->now();
    ++w_loops;
    for (Lane& l : lanes) {
      if (!l.r || mirror_seq(l.m) == l.seq0) continue;
      l.t_free = S->now();
      retire(l);
      progress = true;
    }
    {
      const double t = S->now();
      w_retire += t - tw;
      tw = t;
    }
    hand_over_finished();
    {
      const double t = S->now();
      w_complete += t - tw;
      tw = t;
    }
    if (S->aborting) {
      // running chunks see the abort flag within one loop pass; when they
      // are all back, the active requests end as aborted
      if (n_busy == 0) {
        finish_abort_all();
        S->cv_admit.notify_all();
        std::unique_lock<std::mutex> lk(S->mu);
        if (S->admitter_done && S->admitted.empty()) break;
        S->cv_work.wait_for(lk, std::chrono::milliseconds(20));
      } else {
        std::this_thread::sleep_for(std::chrono::microseconds(100));
      }
      continue;
    }
    // give every free lane the least-work system that is not running
    cudaError_t e = cudaSuccess;
    for (Lane& l : lanes) {
      if (l.r) continue;
      Req* best = nullptr;
      int bk = -1;
      double bkey = 0.0;
      for (Req* r : S->active)
        for (int k = 0; k < r->n_rhs; ++k) {
          if (r->sys_done[k] || r->running[k]) continue;
          // within the CTA budget (a system that does not fit waits; the
          // least-work one that fits runs meanwhile)
          if (cta_cap > 0 && running_ctas > 0 && running_ctas + ctas_of(r) > cta_cap) continue;
          const double key = r->est_left[k] < 0.0 ? -1.0 : r->est_left[k] * r->iter_cost;
          if (!best || key < bkey || (key == bkey && r->id < best->id)) { best = r; bk = k; bkey = key; }
        }
      if (!best) break;
      long long iters = kProbeIters;
      if (best->est_left[bk] >= 0.0) {
        const double mpi = best->ms_per_iter[bk] > 0.0 ? best->ms_per_iter[bk] : best->iter_cost / 2e8;
        iters = (long long)std::ceil(target_ms / std::max(1e-4, mpi));
        iters = std::max<long long>(kProbeIters, std::min<long long>(iters, 1LL << 22));
      }
      iters = (iters + kUnrollPlainIters - 1) / kUnrollPlainIters * kUnrollPlainIters;
      if (best->need_fallback[bk]) {
        e = chunk_fallback_fp64(best->slots[bk].view.st, l.s);
        best->need_fallback[bk] = 0;
      }
      ChunkMirror* m = &S->mirrors[best->mirror_idx[bk]];
      l.r = best;
      l.k = bk;
      l.m = m;
      l.iter_before = best->sys_iter[bk];
      l.seq0 = mirror_seq(m);
      best->running[bk] = 1;
      l.ctas = ctas_of(best);
      running_ctas += l.ctas;
      // the budget is read by the chunk's first kernel
      __atomic_store_n(&m->budget, iters, __ATOMIC_RELEASE);
      const double tr = S->now();
      if (l.t_free >= 0.0) w_gap += tr - l.t_free;
      // (a system switched to FP64 after a stagnation gets its FP64 graph
      // here; otherwise prepare keeps the graph)
      if (e == cudaSuccess)
        e = best->graphs[bk]->prepare(best->slots[bk].view, best->mixed_now[bk] != 0, m, l.s);
      if (e == cudaSuccess) e = best->graphs[bk]->launch(l.s);
      w_run += S->now() - tr;
      ++w_launches;
      busy_change(+1);
      progress = true;
      if (e != cudaSuccess) break;
    }
    if (e != cudaSuccess) {
      std::lock_guard<std::mutex> lk(S->mu);
      S->fatal = std::string("server chunk launch: ") + cudaGetErrorString(e);
      S->cv_admit.notify_all();
      break;
    }
    {
      const double t = S->now();
      w_launch += t - tw;
      tw = t;
    }
    if (!progress) {
      // chunks in flight: poll their mirrors again shortly (the admission
      // threads' notifications are seen at the top of the loop); idle: sleep
      // until a request is admitted or the server stops
      if (n_busy > 0) {
        std::this_thread::sleep_for(std::chrono::microseconds(20));
      } else {
        std::unique_lock<std::mutex> lk(S->mu);
        S->cv_work.wait_for(lk, std::chrono::milliseconds(20), [&] {
          return !S->admitted.empty() || S->admitter_done || S->aborting;
        });
      }
      w_wait += S->now() - tw;
    }
  }
  for (Lane& l : lanes) if (l.s) cudaStreamSynchronize(l.s);
  if (!S->fatal.empty()) {
    for (Req* r : S->active) { r->error = S->fatal; release(S, r, su); finish_request(S, r, false); }
    S->active.clear();
    std::unique_lock<std::mutex> lk(S->mu);
    S->cv_admit.notify_all();
    while (!S->admitter_done || !S->admitted.empty()) {
      while (!S->admitted.empty()) {
        Req* r = S->admitted.front();
        S->admitted.pop_front();
        lk.unlock();
        r->error = S->fatal;
        release(S, r, su);
        finish_request(S, r, false);
        lk.lock();
      }
      if (!S->admitter_done) S->cv_work.wait_for(lk, std::chrono::milliseconds(20));
    }
  }
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->worker_done = true;
    S->cv_complete.notify_all();
  }
  if (S->trace)
    std::fprintf(S->trace, "W,%.6f,%.6f,%.6f,%.6f,%.6f,%.6f,%.6f,%lld,%lld\n", S->now(), w_retire, w_complete,
                 w_launch, w_run, w_wait, w_gap, w_loops, w_launches);
  for (Lane& l : lanes)
    if (l.s) cudaStreamDestroy(l.s);
  cudaStreamDestroy(su);
}

void worker_serial(nlgb_server_s* S) {
  cudaSetDevice(S->device);
  cudaStream_t s = nullptr;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  while (true) {
    if (!intake(S, true)) break;
    if (S->aborting) { fail_all_waiting(S, "server aborted"); continue; }
    if (S->pending.empty()) continue;
    Req* r = S->pending.front();
    S->pending.erase(S->pending.begin());
    r->bytes = estimate_bytes(*r, req_precision(S, *r));
    add_used(S, (long long)r->bytes);
    // Reuse the admission upload/assembly, then solve each right-hand side
    // with the graph-captured single-system solver (which polls the abort
    // flag once per while-loop pass).
    bool ok = admit(S, r, s, false);
    const SolveParams prm = params_of(S, *r, req_precision(S, *r));
    if (ok) {
      PcgSolver pcg;
      ok = pcg.bind(&r->A, s) == cudaSuccess;
      pcg.set_abort_flag(S->abort_dev);
      for (int k = 0; ok && k < r->n_rhs; ++k) {
        SolveResult sr;
        const SysView& v = r->slots[k].view;
        ok = pcg.solve(v.b, v.x, prm, &sr) == cudaSuccess &&
             cudaMemcpyAsync(r->x_out + (size_t)k * r->n, v.x, sizeof(double) * r->n,
                             cudaMemcpyDeviceToHost, s) == cudaSuccess &&
             cudaStreamSynchronize(s) == cudaSuccess;
        nlgb_result& o = r->res[k];
        o.status = sr.status; o.iterations = sr.iterations; o.refinement_steps = sr.outer_steps;
        o.rel_residual = sr.rel_residual; o.true_rel_residual = sr.true_rel_residual;
        o.seconds = sr.seconds;
        o.algo_bytes = sr.algo_bytes;
        o.precision = sr.precision;
        if (sr.status != NL_GB300_STATUS_CONVERGED) r->status = sr.status;
        std::lock_guard<std::mutex> lk(S->mu);
        S->st.kernel_s += sr.seconds;
        if (r->status == NL_GB300_STATUS_ABORTED) break;
      }
      if (r->status == NL_GB300_STATUS_NONE) r->status = NL_GB300_STATUS_CONVERGED;
    }
    release(S, r, s);
    finish_request(S, r, ok);
  }
  cudaStreamDestroy(s);
}

long long enqueue(nlgb_server_s* S, std::unique_ptr<Req> r) {
  if (r->bytes > S->cfg.hbm_budget_bytes) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->st.rejected += 1;
    set_error("nlgb_server_submit: request footprint exceeds the HBM budget");
    return NLGB_E_NOMEM;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->stop || S->aborting) {
    set_error("nlgb_server_submit: server is stopping");
    return NLGB_E_STATE;
  }
  const long long id = S->next_id++;
  r->id = id;
  if (r->arrival < 0) r->arrival = S->now();
  if (S->first_arrival < 0 || r->arrival < S->first_arrival) S->first_arrival = r->arrival;
  S->st.submitted += 1;
  Req* raw = r.get();
  S->reqs[id] = std::move(r);
  S->incoming.push_back(raw);
  S->cv_work.notify_all();
  S->cv_admit.notify_all();
  return id;
}

}  // namespace

extern "C" {

void nlgb_server_default_config(nlgb_server_config* c) {
  if (!c) return;
  c->hbm_budget_bytes = (size_t)150e9;
  c->mode = NLGB_SERVER_BATCHED;
  c->precision = NL_GB300_PRECISION_MIXED;
  c->eps = 1e-10;
  c->max_iter = -1;
  c->inner_eps = 0.1;
  c->epoch_iters = 256;
  c->max_systems = 8192;
  c->schedule = NLGB_SCHEDULE_SRPT;
  c->epoch_ms = 10.0;
  c->streams = 16;
  c->eps_least_squares = 0.0;
  c->min_tile_rows = 0;
  c->chunk_cta_budget = 0;
}

nlgb_server nlgb_server_create(const nlgb_server_config* cfg) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("nlgb_server_create: no CUDA device available");
    return nullptr;
  }
  nlgb_server S = new nlgb_server_s();
  nlgb_server_default_config(&S->cfg);
  if (cfg) S->cfg = *cfg;
  if (S->cfg.epoch_iters <= 0) S->cfg.epoch_iters = 256;
  if (S->cfg.max_systems <= 0) S->cfg.max_systems = 8192;
  S->cfg.max_systems = std::min(S->cfg.max_systems, 65536);
  if (!(S->cfg.epoch_ms >= 0.0)) S->cfg.epoch_ms = 10.0;
  if (S->cfg.streams <= 0) S->cfg.streams = 16;
  S->cfg.streams = std::min(S->cfg.streams, 128);
  // tiles of a multiple of 128 rows, at most 2^20
  S->cfg.min_tile_rows = S->cfg.min_tile_rows <= 0 ? 0 : std::min(((S->cfg.min_tile_rows + 127) / 128) * 128, 1 << 20);
  if (S->cfg.schedule != NLGB_SCHEDULE_SRPT && S->cfg.schedule != NLGB_SCHEDULE_ALL) {
    set_error("nlgb_server_create: unknown schedule");
    delete S;
    return nullptr;
  }
  if (S->cfg.precision != NL_GB300_PRECISION_MIXED && S->cfg.precision != NL_GB300_PRECISION_DOUBLE &&
      S->cfg.precision != NL_GB300_PRECISION_AUTO && S->cfg.precision != NL_GB300_PRECISION_DOUBLE_FLOAT) {
    set_error("nlgb_server_create: unknown precision");
    delete S;
    return nullptr;
  }
  S->st.budget_bytes = S->cfg.hbm_budget_bytes;
  cudaGetDevice(&S->device);
  // Requests allocate and free their device memory stream-ordered from the
  // device's default pool; keeping freed memory in the pool makes the next
  // request's allocations cheap.
  cudaMemPool_t pool = nullptr;
  if (cudaDeviceGetDefaultMemPool(&pool, S->device) == cudaSuccess) {
    unsigned long long keep = ~0ULL;   // release threshold: never trim
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  cudaGetLastError();
  void* flag = nullptr;
  if (cudaHostAlloc(&flag, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer((void**)&S->abort_dev, flag, 0) != cudaSuccess) {
    set_error(std::string("nlgb_server_create: abort flag: ") + cudaGetErrorString(cudaGetLastError()));
    if (flag) cudaFreeHost(flag);
    delete S;
    return nullptr;
  }
  S->abort_host = static_cast<volatile int*>(flag);
  *S->abort_host = 0;
  const bool streams = S->cfg.mode != NLGB_SERVER_SERIAL && S->cfg.schedule == NLGB_SCHEDULE_SRPT;
  if (streams) {
    // one chunk mirror per system that may be in flight; the graphs embed
    // the device view of these pointers, the worker reads the host view
    // (the same address under unified addressing, checked here)
    void* mp = nullptr;
    void* md = nullptr;
    const size_t bytes = sizeof(ChunkMirror) * (size_t)S->cfg.max_systems;
    if (cudaHostAlloc(&mp, bytes, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer(&md, mp, 0) != cudaSuccess || md != mp) {
      set_error(std::string("nlgb_server_create: chunk mirrors: ") +
                (md && md != mp ? "mapped pointer differs from the host pointer"
                                : cudaGetErrorString(cudaGetLastError())));
      if (mp) cudaFreeHost(mp);
      cudaFreeHost(flag);
      delete S;
      return nullptr;
    }
    std::memset(mp, 0, bytes);
    S->mirrors = static_cast<ChunkMirror*>(mp);
    S->mirror_free.reserve((size_t)S->cfg.max_systems);
    for (int i = S->cfg.max_systems - 1; i >= 0; --i) S->mirror_free.push_back(i);
  }
  if (const char* tp = std::getenv("NLGB_SERVER_TRACE")) {
    S->trace = std::fopen(tp, "a");
    if (S->trace)
      std::fprintf(S->trace, "# E,t0,t1,kind,systems,teams,team_ctas,queue_ctas,grid,planned_GB,done_GB,ms,"
                             "team_ms_min,team_ms_med,team_ms_max,queue_ms,admits,admit_s,active_requests\n"
                             "# C,t,request,rhs,mixed,iter_before,iter_after,ms,status,stage\n"
                             "# A,t,request,mesh_kind,n,seconds,bytes,arrival,graph_seconds,build_seconds,prepare_seconds\n"
                             "# W,t,retire_s,complete_s,launch_s,graph_launch_s,wait_s,lane_idle_s,loops,launches\n"
                             "# D,t,request,n,download_s,release_s\n"
                             "# R,t,request,slots_s,graphs_s\n");
  }
  S->origin = Clock::now();
  S->th = std::thread(S->cfg.mode == NLGB_SERVER_SERIAL
                          ? worker_serial
                          : (S->cfg.schedule == NLGB_SCHEDULE_SRPT ? worker_streams : worker_batched),
                      S);
  if (S->cfg.mode != NLGB_SERVER_SERIAL) {
    // several admission threads: uploads, builds and graph instantiations
    // of different requests overlap
    S->admitters_live = kAdmitters;
    for (int i = 0; i < kAdmitters; ++i) S->adm_th.emplace_back(admitter, S);
  }
  if (streams)
    for (int i = 0; i < kCompleters; ++i) S->cmp_th.emplace_back(completer, S);
  return S;
}

void nlgb_server_reset_clock(nlgb_server S) {
  if (!S) return;
  std::lock_guard<std::mutex> lk(S->mu);
  S->origin = Clock::now();
  S->t_used = 0.0;
  S->st.byte_seconds = 0.0;
}

double nlgb_server_now(nlgb_server S) { return S ? S->now() : 0.0; }

long long nlgb_server_submit_crs(nlgb_server S, int n, const int* rp, const int* ci,
                                 const double* va, int n_rhs, const double* b, const double* x0,
                                 double* x_out, double arrival_s) {
  if (!S || n < 0 || !rp || !b || !x_out || n_rhs < 1) {
    set_error("nlgb_server_submit_crs: bad arguments");
    return NLGB_E_INVALID;
  }
  const long long nnz = rp[n];
  if (rp[0] != 0 || nnz < 0) { set_error("nlgb_server_submit_crs: bad row pointers"); return NLGB_E_INVALID; }
  for (int i = 0; i < n; ++i)
    if (rp[i + 1] < rp[i]) { set_error("nlgb_server_submit_crs: row pointers not monotone"); return NLGB_E_INVALID; }
  for (long long k = 0; k < nnz; ++k)
    if (ci[k] < 0 || ci[k] >= n) { set_error("nlgb_server_submit_crs: column out of range"); return NLGB_E_INVALID; }
  auto r = std::make_unique<Req>();
  r->kind = 0;
  r->n = n;
  r->n_rhs = n_rhs;
  r->rp.assign(rp, rp + n + 1);
  r->ci.assign(ci, ci + nnz);
  r->va.assign(va, va + nnz);
  r->b.assign(b, b + (size_t)n * n_rhs);
  if (x0) r->x0.assign(x0, x0 + (size_t)n * n_rhs);
  r->x_out = x_out;
  r->arrival = arrival_s;
  r->bytes = estimate_bytes(*r, req_precision(S, *r));
  return enqueue(S, std::move(r));
}

long long nlgb_server_submit_mesh(nlgb_server S, int mesh_kind, int n_verts, const double* xyz,
                                  int n_tris, const int* tris, const int* pins, const double* pin_uv,
                                  double lambda, int n_rhs, const double* b, const double* x0,
                                  double* x_out, double arrival_s) {
  const bool lscm = mesh_kind == NLGB_MESH_LSCM;
  if (!S || (mesh_kind != NLGB_MESH_LSCM && mesh_kind != NLGB_MESH_FAIRING) || n_verts < 3 ||
      n_tris < 0 || !xyz || (n_tris > 0 && !tris) || !x_out || n_rhs < 1 || (lscm && n_rhs != 1) ||
      (!lscm && (!b || !(lambda >= 0.0))) || n_verts > (1 << 30) - 1) {
    set_error("nlgb_server_submit_mesh: bad arguments");
    return NLGB_E_INVALID;
  }
  for (long long k = 0; k < 3LL * n_tris; ++k)
    if (tris[k] < 0 || tris[k] >= n_verts) {
      set_error("nlgb_server_submit_mesh: triangle index out of range");
      return NLGB_E_INVALID;
    }
  auto r = std::make_unique<Req>();
  r->kind = 2;
  r->mesh_kind = mesh_kind;
  r->least_squares = lscm ? 1 : 0;
  r->n_verts = n_verts;
  r->n_tris = n_tris;
  r->xyz.assign(xyz, xyz + 3 * (size_t)n_verts);
  r->tris.assign(tris, tris + 3 * (size_t)n_tris);
  if (lscm) {
    r->pins[0] = pins ? pins[0] : 0;
    r->pins[1] = pins ? pins[1] : n_verts - 1;
    if (pin_uv) std::memcpy(r->pin_uv, pin_uv, sizeof(r->pin_uv));
    if (r->pins[0] < 0 || r->pins[0] >= n_verts || r->pins[1] < 0 || r->pins[1] >= n_verts ||
        r->pins[0] == r->pins[1]) {
      set_error("nlgb_server_submit_mesh: the two pins must be distinct vertices");
      return NLGB_E_INVALID;
    }
  }
  r->lambda = lambda;
  r->n = lscm ? 2 * n_verts - 4 : n_verts;
  r->n_rhs = n_rhs;
  if (!lscm) r->b.assign(b, b + (size_t)n_rhs * r->n);
  if (x0) r->x0.assign(x0, x0 + (size_t)n_rhs * r->n);
  r->x_out = x_out;
  r->arrival = arrival_s;
  r->bytes = estimate_bytes(*r, req_precision(S, *r));
  return enqueue(S, std::move(r));
}

long long nlgb_server_submit_rows(nlgb_server S, int least_squares, long long n_rows,
                                  const long long* row_ptr, const int* col, const double* val,
                                  const double* rhs, const double* weight, int n_free, int n_vars,
                                  const double* xl, int n_rhs, const double* x0, double* x_out,
                                  double arrival_s) {
  if (!S || n_rows < 0 || !row_ptr || n_free < 0 || n_vars < n_free || !x_out || n_rhs < 1) {
    set_error("nlgb_server_submit_rows: bad arguments");
    return NLGB_E_INVALID;
  }
  const long long nc = row_ptr[n_rows];
  for (long long k = 0; k < nc; ++k) {
    const int c = col[k];
    if (c >= n_free || (c < 0 && (-(long long)c - 1) >= n_vars)) {
      set_error("nlgb_server_submit_rows: coefficient index out of range");
      return NLGB_E_INVALID;
    }
  }
  if (!least_squares && n_rows != n_free) {
    set_error("nlgb_server_submit_rows: a square system needs one row per free variable");
    return NLGB_E_INVALID;
  }
  auto r = std::make_unique<Req>();
  r->kind = 1;
  r->least_squares = least_squares ? 1 : 0;
  r->n = n_free;
  r->n_vars = n_vars;
  r->n_rhs = n_rhs;
  r->n_rows = n_rows;
  r->row_ptr.assign(row_ptr, row_ptr + n_rows + 1);
  r->col.assign(col, col + nc);
  r->val.assign(val, val + nc);
  if (rhs) { r->rhs.assign(rhs, rhs + (size_t)n_rows * n_rhs); r->has_rhs = true; }
  if (weight) { r->weight.assign(weight, weight + n_rows); r->has_weight = true; }
  if (xl) { r->xl.assign(xl, xl + (size_t)n_vars * n_rhs); r->has_xl = true; }
  if (x0) r->x0.assign(x0, x0 + (size_t)n_free * n_rhs);
  r->x_out = x_out;
  r->arrival = arrival_s;
  r->bytes = estimate_bytes(*r, req_precision(S, *r));
  return enqueue(S, std::move(r));
}

int nlgb_server_wait(nlgb_server S, long long ticket, nlgb_result* res, double* latency_s) {
  if (!S) return NLGB_E_INVALID;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) { set_error("nlgb_server_wait: unknown ticket"); return NLGB_E_INVALID; }
  Req* r = it->second.get();
  S->cv_done.wait(lk, [&] { return r->state == R_DONE || r->state == R_FAILED; });
  if (res)
    for (int k = 0; k < r->n_rhs; ++k) res[k] = k < (int)r->res.size() ? r->res[k] : nlgb_result{};
  if (latency_s) *latency_s = r->t_done - r->arrival;
  if (r->state == R_FAILED) {
    set_error(r->error.empty() ? "request failed" : r->error);
    return NLGB_E_DEVICE;
  }
  return NLGB_OK;
}

int nlgb_server_drain(nlgb_server S) {
  if (!S) return NLGB_E_INVALID;
  std::unique_lock<std::mutex> lk(S->mu);
  S->cv_done.wait(lk, [&] { return S->st.completed + S->st.failed >= S->st.submitted; });
  return S->st.failed ? NLGB_E_DEVICE : NLGB_OK;
}

int nlgb_server_get_stats(nlgb_server S, nlgb_server_stats* out) {
  if (!S || !out) return NLGB_E_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  nlgb_server_stats st = S->st;
  st.byte_seconds += double(S->used) * std::max(0.0, S->now() - S->t_used);
  st.p50_latency_s = percentile(S->latencies, 0.50);
  st.p99_latency_s = percentile(S->latencies, 0.99);
  double sum = 0.0, mx = 0.0;
  for (double l : S->latencies) { sum += l; mx = std::max(mx, l); }
  st.mean_latency_s = S->latencies.empty() ? 0.0 : sum / S->latencies.size();
  st.max_latency_s = mx;
  st.wall_s = S->first_arrival >= 0 ? std::max(0.0, S->last_done - S->first_arrival) : 0.0;
  st.solves_per_s = st.wall_s > 0 ? double(st.completed) / st.wall_s : 0.0;
  *out = st;
  return NLGB_OK;
}

void nlgb_server_abort(nlgb_server S) {
  if (!S) return;
  std::lock_guard<std::mutex> lk(S->mu);
  S->aborting = true;
  if (S->abort_host) *S->abort_host = 1;
  S->cv_work.notify_all();
  S->cv_admit.notify_all();
}

void nlgb_server_destroy(nlgb_server S) {
  if (!S) return;
  {
    // requests still queued or in flight are aborted (callers drain first)
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->aborting = true;
    S->cv_work.notify_all();
    S->cv_admit.notify_all();
  }
  if (S->th.joinable()) S->th.join();
  for (std::thread& t : S->adm_th)
    if (t.joinable()) t.join();
  for (std::thread& t : S->cmp_th)
    if (t.joinable()) t.join();
  S->graveyard.clear();
  if (S->mirrors) cudaFreeHost(S->mirrors);
  if (S->abort_host) cudaFreeHost(const_cast<int*>(S->abort_host));
  if (S->trace) std::fclose(S->trace);
  delete S;
}

}  // extern "C"
