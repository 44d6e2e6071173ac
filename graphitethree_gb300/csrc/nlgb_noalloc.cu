// nlgb_noalloc.cu -- nlgb_solve_noalloc: the FP64 Jacobi-PCG solve of
// nlgb_solve for callers that cannot allocate GPU memory.
//
// Some host applications reserve the whole device memory up front for their
// own pools and must keep their footprint fixed, and interactive loops cannot
// afford the implicit device synchronisation of cudaMalloc / cudaFree.  Such
// callers pass their own device buffers for the matrix (CRS), the right-hand
// side and the solution; every other array this solve needs (Jacobi
// diagonal, residual, search direction, A p, tile partials, scalar state)
// lives in one file-scope static device array of fixed size, which every GPU
// that loads the library keeps until the process exits.  Nothing here calls
// cudaMalloc, cudaFree or any allocating library routine.
//
// Limits and sharing: at most kNoAllocMaxRows rows (the array is 8.1 MiB);
// all calls share the one array and each call overwrites it, so calls that
// overlap on the GPU (several host threads, or several streams) race -- the
// caller must serialise them.  The first call on a device looks up the
// array's device address (cudaGetSymbolAddress) with that device current;
// that first call belongs before any stream capture.
#include "../../include/nl.h"
#include "../../include/nl_gb300.h"
#include "nlgb_core.cuh"
#include "nlgb_internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>

namespace nlgb {
namespace {

constexpr int kNoAllocMaxRows = 262144;
constexpr int kNoAllocMinTile = 128;
constexpr int kNoAllocMaxTiles = kNoAllocMaxRows / kNoAllocMinTile;
constexpr size_t kStateDoubles = (sizeof(SysState) + 7) / 8;
// dinv, r, p, q (rows) + tile partials + state + row-length histogram
constexpr size_t kScratchDoubles = 4 * (size_t)kNoAllocMaxRows + (size_t)kNoAllocMaxTiles * kParts +
                                   kStateDoubles + 32;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
double* g_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once
// per device, with that device current).
cudaError_t scratch_address(double** out) {
  int dev = 0;
  NLGB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("nlgb_solve_noalloc: device index out of range");
    return cudaErrorInvalidDevice;
  }
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    NLGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_addr[dev] = static_cast<double*>(p);
  }
  *out = g_addr[dev];
  return cudaSuccess;
}

// Last-CTA election over the tile partials (same protocol as the graph solver).
template <int K>
__device__ __forceinline__ bool na_publish(const SysView& s, int tile, const double (&v)[K], int slot,
                                           unsigned int* counter) {
  __shared__ int am_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) __stcg(s.part + (size_t)tile * kParts + slot + k, v[k]);
    __threadfence();
    const unsigned int prev = atomicAdd(counter, 1u);
    am_last = (prev == (unsigned int)s.n_tiles - 1u);
    if (am_last) *counter = 0u;
  }
  __syncthreads();
  if (am_last) __threadfence();
  return am_last != 0;
}

template <int K>
__device__ void na_reduce(const SysView& s, int slot, double (&o)[K]) {
  int comp[K];
#pragma unroll
  for (int k = 0; k < K; ++k) comp[k] = slot + k;
  canon_reduce<K>(s.part, s.n_tiles, comp, o);
}

__device__ __forceinline__ bool na_running(const SysView& s) { return __ldcg(&s.st->status) == ST_RUNNING; }

template <int T>
__global__ void __launch_bounds__(kCTA) na_init(SysView s) {
  double v[3];
  tile_residual<T>(s, blockIdx.x, v);
  if (na_publish<3>(s, blockIdx.x, v, kSlotInit, &s.st->cnt[0])) {
    double o[3];
    na_reduce<3>(s, kSlotInit, o);
    if (threadIdx.x == 0) scalar_after_init(s.st, o[0], o[1], o[2]);
  }
}

template <int T>
__global__ void __launch_bounds__(kCTA) na_spmv_pq(SysView s) {
  if (!na_running(s)) return;
  double v[1] = {tile_spmv_pq<T>(s, blockIdx.x)};
  if (na_publish<1>(s, blockIdx.x, v, kSlotPQ, &s.st->cnt[1])) {
    double o[1];
    na_reduce<1>(s, kSlotPQ, o);
    if (threadIdx.x == 0) scalar_after_pq(s.st, o[0]);
  }
}

__global__ void __launch_bounds__(kCTA) na_update_xr(SysView s) {
  if (!na_running(s)) return;
  double v[2];
  tile_update_xr(s, blockIdx.x, __ldcg(&s.st->alpha), v);
  if (na_publish<2>(s, blockIdx.x, v, kSlotXR, &s.st->cnt[2])) {
    double o[2];
    na_reduce<2>(s, kSlotXR, o);
    if (threadIdx.x == 0) scalar_after_xr(s.st, o[0], o[1]);
  }
}

__global__ void __launch_bounds__(kCTA) na_update_p(SysView s) {
  if (!na_running(s)) return;
  tile_update_p(s, blockIdx.x, __ldcg(&s.st->beta));
}

template <int T>
__global__ void __launch_bounds__(kCTA) na_final(SysView s) {
  double v[1] = {0.0};
  if (__ldcg(&s.st->zero_rhs)) tile_zero_x(s, blockIdx.x);
  else v[0] = tile_true_rr<T>(s, blockIdx.x);
  if (na_publish<1>(s, blockIdx.x, v, kSlotFinal, &s.st->cnt[3])) {
    double o[1];
    na_reduce<1>(s, kSlotFinal, o);
    if (threadIdx.x == 0) s.st->rr_true = o[0];
  }
}

// The true-residual check after na_final and the continuation it may ask
// for (the same steps as the other executors: the pending p update, then
// more iterations).
__global__ void na_check(SysState* st) {
  if (scalar_after_check(st)) st->stage = 4;
}

__global__ void __launch_bounds__(kCTA) na_resume_p(SysView s) {
  if (!na_running(s) || __ldcg(&s.st->stage) != 4) return;
  tile_update_p(s, blockIdx.x, __ldcg(&s.st->beta));
}

__global__ void na_resume_mark(SysState* st) {
  if (st->stage == 4) st->stage = 1;
}

// dinv[i] = 1 / a_ii (1 when the diagonal is missing or zero).
__global__ void na_jacobi(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                          const double* __restrict__ va, double* dinv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = 0.0;
  for (int k = rp[i]; k < rp[i + 1]; ++k)
    if (ci[k] == i) d += va[k];
  dinv[i] = (d != 0.0) ? 1.0 / d : 1.0;
}

// Row-length histogram (bins 0..31, 32 = longer) and longest row, into ints.
__global__ void na_hist(int n, const int* __restrict__ rp, int* hist34) {
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
  if (threadIdx.x < 33 && h[threadIdx.x]) atomicAdd(&hist34[threadIdx.x], h[threadIdx.x]);
  if (threadIdx.x == 0) atomicMax(&hist34[33], mx);
}

template <int T>
cudaError_t launch_iterations(const SysView& v, int grid, int iters, cudaStream_t s) {
  for (int i = 0; i < iters; ++i) {
    na_spmv_pq<T><<<grid, kCTA, 0, s>>>(v);
    na_update_xr<<<grid, kCTA, 0, s>>>(v);
    na_update_p<<<grid, kCTA, 0, s>>>(v);
  }
  count_launches(3LL * iters);
  return cudaGetLastError();
}

template <int T>
cudaError_t run_pcg(const SysView& v, long long max_iter, cudaStream_t s, SysState* h) {
  const int grid = v.n_tiles;
  na_init<T><<<grid, kCTA, 0, s>>>(v);
  count_launches(1);
  NLGB_CUDA_TRY(cudaGetLastError());
  // Host loop: 32 iterations per check of the status word.  The kernels do
  // nothing once the status leaves RUNNING, and the loop is capped by
  // max_iter independently of the device logic.  After the final residual,
  // a failed true-residual check continues the recurrence (at most
  // kMaxTrueChecks times).
  constexpr int kChunk = 32;
  const long long max_chunks = max_iter / kChunk + 2 + 2LL * (kMaxTrueChecks + 1);
  long long chunks = 0;
  for (int pass = 0; pass <= kMaxTrueChecks; ++pass) {
    for (; chunks < max_chunks; ++chunks) {
      int status = ST_RUNNING;
      NLGB_CUDA_TRY(cudaMemcpyAsync(&status, &v.st->status, sizeof(int), cudaMemcpyDeviceToHost, s));
      NLGB_CUDA_TRY(cudaStreamSynchronize(s));
      if (status != ST_RUNNING) break;
      NLGB_CUDA_TRY(launch_iterations<T>(v, grid, kChunk, s));
    }
    na_final<T><<<grid, kCTA, 0, s>>>(v);
    na_check<<<1, 1, 0, s>>>(v.st);
    count_launches(2);
    NLGB_CUDA_TRY(cudaGetLastError());
    NLGB_CUDA_TRY(cudaMemcpyAsync(h, v.st, sizeof(SysState), cudaMemcpyDeviceToHost, s));
    NLGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (h->status != ST_RUNNING) break;
    na_resume_p<<<grid, kCTA, 0, s>>>(v);
    na_resume_mark<<<1, 1, 0, s>>>(v.st);
    count_launches(2);
    NLGB_CUDA_TRY(cudaGetLastError());
  }
  return cudaSuccess;
}

}  // namespace
}  // namespace nlgb

using namespace nlgb;

extern "C" int nlgb_solve_noalloc(int n, const int* rp, const int* ci, const double* va,
                                  const double* b, double* x, const nlgb_params* prm,
                                  nlgb_result* res, void* stream) {
  if (n < 0 || n > kNoAllocMaxRows) {
    set_error("nlgb_solve_noalloc: n must be in [0, 262144] (the size of the static scratch array)");
    return NLGB_E_INVALID;
  }
  if (n > 0 && (!rp || !ci || !va || !b || !x)) {
    set_error("nlgb_solve_noalloc: null argument");
    return NLGB_E_INVALID;
  }
  if ((reinterpret_cast<uintptr_t>(x) & 15) != 0) {
    set_error("nlgb_solve_noalloc: x must be 16-byte aligned");
    return NLGB_E_INVALID;
  }
  nlgb_params p;
  nlgb_default_params(&p);
  if (prm) p = *prm;
  if (p.precision != NL_GB300_PRECISION_DOUBLE) {
    set_error("nlgb_solve_noalloc: only NL_GB300_PRECISION_DOUBLE is available without allocation");
    return NLGB_E_INVALID;
  }
  if (!(p.eps >= 0.0)) {
    set_error("nlgb_solve_noalloc: bad tolerance");
    return NLGB_E_INVALID;
  }
  if (n == 0) {
    // nothing to solve (and no row pointer to read)
    if (res) {
      std::memset(res, 0, sizeof(*res));
      res->status = NL_GB300_STATUS_CONVERGED;
      res->precision = NL_GB300_PRECISION_DOUBLE;
    }
    return NLGB_OK;
  }
  const auto t_start = std::chrono::steady_clock::now();
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* base = nullptr;
  if (scratch_address(&base) != cudaSuccess) return NLGB_E_DEVICE;
  auto device_error = [](const char* what, cudaError_t e) {
    set_error(std::string("nlgb_solve_noalloc: ") + what + ": " + cudaGetErrorString(e));
    return NLGB_E_DEVICE;
  };
  int dev = 0, sms = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (ce != cudaSuccess) return device_error("device query", ce);
  // Carve the static array: dinv | r | p | q | partials | state | histogram.
  double* dinv = base;
  double* r = dinv + kNoAllocMaxRows;
  double* pv = r + kNoAllocMaxRows;
  double* q = pv + kNoAllocMaxRows;
  double* part = q + kNoAllocMaxRows;
  SysState* st = reinterpret_cast<SysState*>(part + (size_t)kNoAllocMaxTiles * kParts);
  int* hist = reinterpret_cast<int*>(reinterpret_cast<double*>(st) + kStateDoubles);

  // Layout choice: the same autotuner as the allocating path.
  int h34[34] = {0};
  ce = cudaMemsetAsync(hist, 0, sizeof(h34), s);
  if (ce != cudaSuccess) return device_error("clearing the histogram", ce);
  // four 256-thread CTAs per SM at most (grid-stride loop)
  na_hist<<<std::max(1, std::min(4 * std::max(1, sms), (n + 255) / 256)), 256, 0, s>>>(n, rp, hist);
  count_launches(1);
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return device_error("histogram launch", ce);
  int nnz = 0;
  if ((ce = cudaMemcpyAsync(h34, hist, sizeof(h34), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (ce = cudaMemcpyAsync(&nnz, rp + n, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (ce = cudaStreamSynchronize(s)) != cudaSuccess)
    return device_error("reading the row-length histogram", ce);
  const TuneChoice tc = autotune(n, nnz, h34[33], h34);
  const int tile = std::max(kNoAllocMinTile, tc.tile_rows);
  SysView v;
  std::memset(&v, 0, sizeof(v));
  v.n = n;
  v.tile_rows = tile;
  v.n_tiles = std::max(1, (n + tile - 1) / tile);
  v.tpr = tc.tpr;
  v.rp = rp; v.ci = ci; v.va = va; v.dinv = dinv;
  v.b = b; v.x = x; v.r = r; v.p = pv; v.q = q;
  v.part = part;
  v.st = st;
  na_jacobi<<<(n + 255) / 256, 256, 0, s>>>(n, rp, ci, va, dinv);
  count_launches(1);
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return device_error("Jacobi launch", ce);
  // Fresh state (the array keeps the previous call's contents).
  SysState h;
  std::memset(&h, 0, sizeof(h));
  const long long max_iter = p.max_iter >= 0 ? p.max_iter : 5LL * n;
  h.thresh2 = p.eps * p.eps;
  h.max_iter = max_iter;
  h.status = ST_RUNNING;
  ce = cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s);
  if (ce != cudaSuccess) return device_error("state upload", ce);
  cudaError_t e;
  switch (v.tpr) {
    case 1: e = run_pcg<1>(v, max_iter, s, &h); break;
    case 2: e = run_pcg<2>(v, max_iter, s, &h); break;
    case 4: e = run_pcg<4>(v, max_iter, s, &h); break;
    case 8: e = run_pcg<8>(v, max_iter, s, &h); break;
    case 16: e = run_pcg<16>(v, max_iter, s, &h); break;
    default: e = run_pcg<32>(v, max_iter, s, &h); break;
  }
  if (e != cudaSuccess) return NLGB_E_DEVICE;   // message set by NLGB_CUDA_TRY
  if (res) {
    res->status = h.status == ST_RUNNING ? ST_MAX_ITER : h.status;
    res->iterations = h.iter;
    res->refinement_steps = 0;
    res->rel_residual = h.bnorm2 > 0 ? std::sqrt(h.rr / h.bnorm2) : 0.0;
    res->true_rel_residual = h.bnorm2 > 0 ? std::sqrt(h.rr_true / h.bnorm2) : 0.0;
    // host clock of the whole call (it returns when the solve is finished)
    res->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    res->algo_bytes = algo_bytes(n, nnz, h);
    res->precision = NL_GB300_PRECISION_DOUBLE;
  }
  return NLGB_OK;
}
