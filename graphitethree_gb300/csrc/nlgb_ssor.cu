// nlgb_ssor.cu -- the SSOR preconditioner on the GPU, and the CG solve that
// uses it.
//
// Replaces nlNewSSORPreconditioner(M, omega), which OGF::NL::Matrix creates
// for solve_iterative(..., SSOR) (src/lib/OGF/scene_graph/NL/matrix.cpp:
// 366-368, omega = 1.5) and hands to nlSolveSystemIterative (:390-393).
// For a symmetric A = L + D + L^T:
//   M = (D + w L) D^-1 (D + w L^T) / (w (2 - w)),
// applied as z = M^-1 r by a forward sweep
//   y_i = (w (2 - w) r_i - w sum_{j<i} a_ij y_j) / d_i
// and a backward sweep
//   z_i = y_i - (w / d_i) sum_{j>i} a_ij z_j.
// The sweeps are sequential by nature.  Here every row is computed exactly
// as the sequential sweep computes it (the same dependencies), but the rows
// are grouped into levels -- a row's level is one more than the highest
// level among the rows it reads -- and the rows of one level run in parallel
// (one warp per row), level after level.  Only the order of the additions
// inside a row's dot product differs from the sequential sweep.  The levels
// of a matrix are computed once, on the host, when the preconditioner is
// built; the launches of one application are captured in a CUDA graph.
#include "nlgb_core.cuh"
#include "nlgb_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace nlgb {

namespace {

__global__ void k_ssor_diag(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                            const double* __restrict__ va, double* diag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = 0.0;
  for (int k = rp[i]; k < rp[i + 1]; ++k)
    if (ci[k] == i) d += va[k];
  diag[i] = d != 0.0 ? d : 1.0;
}

// One warp per row of the level (the warp index is uniform in a warp, so a
// whole warp returns together).
__global__ void k_ssor_forward(int cnt, const int* __restrict__ rows, const int* __restrict__ rp,
                               const int* __restrict__ ci, const double* __restrict__ va,
                               const double* __restrict__ diag, double c, double omega,
                               const double* __restrict__ r, double* y) {
  const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= cnt) return;
  const int i = rows[w];
  double s = 0.0;
  for (int k = rp[i] + lane; k < rp[i + 1]; k += 32) {
    const int j = ci[k];
    if (j < i) s = fma(va[k], y[j], s);
  }
  s = warp_sum(s);
  if (lane == 0) y[i] = (c * r[i] - omega * s) / diag[i];
}

__global__ void k_ssor_backward(int cnt, const int* __restrict__ rows, const int* __restrict__ rp,
                                const int* __restrict__ ci, const double* __restrict__ va,
                                const double* __restrict__ diag, double omega,
                                const double* __restrict__ y, double* z) {
  const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= cnt) return;
  const int i = rows[w];
  double s = 0.0;
  for (int k = rp[i] + lane; k < rp[i + 1]; k += 32) {
    const int j = ci[k];
    if (j > i) s = fma(va[k], z[j], s);
  }
  s = warp_sum(s);
  if (lane == 0) z[i] = y[i] - omega * s / diag[i];
}

// p = z + beta p (the CG direction update)
__global__ void k_ssor_p(long long n, const double* __restrict__ z, double beta, double* p) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = z[i] + beta * p[i];
}

// r = b - r (r held A x)
__global__ void k_ssor_bmr(long long n, const double* __restrict__ b, double* r) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    r[i] = b[i] - r[i];
}

int blocks_of(long long n) { return (int)std::max(1LL, std::min<long long>((n + 255) / 256, 152LL * 16)); }

// Levels of the sweep over the rows in sweep order (increasing for the
// forward sweep, decreasing for the backward one), reading the entries
// whose column comes earlier in that order: rows grouped by level, in sweep
// order within a level.
void levels(int n, const std::vector<int>& rp, const std::vector<int>& ci, bool forward, std::vector<int>& ptr,
            std::vector<int>& rows) {
  std::vector<int> lvl((size_t)n, 0);
  int top = -1;
  for (int t = 0; t < n; ++t) {
    const int i = forward ? t : n - 1 - t;
    int l = 0;
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      const int j = ci[k];
      if (forward ? (j < i) : (j > i)) l = std::max(l, lvl[j] + 1);
    }
    lvl[i] = l;
    top = std::max(top, l);
  }
  ptr.assign((size_t)top + 2, 0);
  for (int i = 0; i < n; ++i) ptr[lvl[i] + 1] += 1;
  for (size_t l = 1; l < ptr.size(); ++l) ptr[l] += ptr[l - 1];
  rows.assign((size_t)n, 0);
  std::vector<int> cur(ptr.begin(), ptr.end() - 1);
  for (int t = 0; t < n; ++t) {
    const int i = forward ? t : n - 1 - t;
    rows[cur[lvl[i]]++] = i;
  }
}

}  // namespace

void SsorPrecond::release() {
  for (Cached& c : graphs) cudaGraphExecDestroy(c.exec);
  graphs.clear();
  cudaFree(rows_f); cudaFree(rows_b); cudaFree(diag); cudaFree(y);
  rows_f = rows_b = nullptr;
  diag = y = nullptr;
}

cudaError_t SsorPrecond::build(const DeviceCRS& Am, double w, cudaStream_t s) {
  release();
  A = &Am;
  n = Am.n;
  omega = w;
  std::vector<int> rp((size_t)n + 1), ci((size_t)std::max(1LL, Am.nnz));
  NLGB_CUDA_TRY(cudaMemcpyAsync(rp.data(), Am.rp, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
  if (Am.nnz > 0) NLGB_CUDA_TRY(cudaMemcpyAsync(ci.data(), Am.ci, sizeof(int) * Am.nnz, cudaMemcpyDeviceToHost, s));
  NLGB_CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<int> rf, rb;
  levels(n, rp, ci, true, ptr_f, rf);
  levels(n, rp, ci, false, ptr_b, rb);
  const size_t n1 = (size_t)std::max(1, n);
  NLGB_CUDA_TRY(cudaMalloc(&rows_f, sizeof(int) * n1));
  NLGB_CUDA_TRY(cudaMalloc(&rows_b, sizeof(int) * n1));
  NLGB_CUDA_TRY(cudaMalloc(&diag, sizeof(double) * n1));
  NLGB_CUDA_TRY(cudaMalloc(&y, sizeof(double) * n1));
  if (n > 0) {
    NLGB_CUDA_TRY(cudaMemcpyAsync(rows_f, rf.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    NLGB_CUDA_TRY(cudaMemcpyAsync(rows_b, rb.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    k_ssor_diag<<<(n + 255) / 256, 256, 0, s>>>(n, Am.rp, Am.ci, Am.va, diag);
    count_launches(1);
    NLGB_CUDA_TRY(cudaGetLastError());
  }
  return cudaStreamSynchronize(s);
}

cudaError_t SsorPrecond::launch_sweeps(const double* r, double* z, cudaStream_t s) {
  const double c = omega * (2.0 - omega);
  for (size_t l = 0; l + 1 < ptr_f.size(); ++l) {
    const int cnt = ptr_f[l + 1] - ptr_f[l];
    if (cnt <= 0) continue;
    k_ssor_forward<<<(cnt * 32 + 255) / 256, 256, 0, s>>>(cnt, rows_f + ptr_f[l], A->rp, A->ci, A->va, diag, c,
                                                         omega, r, y);
  }
  for (size_t l = 0; l + 1 < ptr_b.size(); ++l) {
    const int cnt = ptr_b[l + 1] - ptr_b[l];
    if (cnt <= 0) continue;
    k_ssor_backward<<<(cnt * 32 + 255) / 256, 256, 0, s>>>(cnt, rows_b + ptr_b[l], A->rp, A->ci, A->va, diag,
                                                          omega, y, z);
  }
  return cudaGetLastError();
}

cudaError_t SsorPrecond::apply(const double* r, double* z, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  // one CUDA graph per (r, z) pair: the sweeps of a solve replay it
  cudaGraphExec_t exec = nullptr;
  for (const Cached& c : graphs)
    if (c.r == r && c.z == z) exec = c.exec;
  if (!exec) {
    cudaStream_t cs = nullptr;
    NLGB_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      const cudaError_t e1 = launch_sweeps(r, z, cs);
      e = cudaStreamEndCapture(cs, &g);
      if (e == cudaSuccess) e = e1;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) {
      set_error(std::string("SSOR sweep graph: ") + cudaGetErrorString(e));
      return e;
    }
    graphs.push_back({r, z, exec});
  }
  count_launches((long long)(ptr_f.size() + ptr_b.size()) - 2);
  return cudaGraphLaunch(exec, s);
}

// CG with the SSOR preconditioner (host-driven: the dot products are read
// back every iteration), with the recursive-residual stop and the
// true-residual check of the other FP64 solvers (scalar_after_check).
cudaError_t pcg_ssor(const DeviceCRS& A, SsorPrecond& P, const double* b, double* x, double eps,
                     long long max_iter, cudaStream_t s, KrylovResult* res) {
  const long long n = A.n;
  res->status = ST_RUNNING;
  res->iterations = 0;
  if (n == 0) { res->status = ST_CONVERGED; return cudaSuccess; }
  double *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
  const size_t bytes = sizeof(double) * (size_t)n;
  NLGB_CUDA_TRY(cudaMalloc(&r, bytes));
  NLGB_CUDA_TRY(cudaMalloc(&z, bytes));
  NLGB_CUDA_TRY(cudaMalloc(&p, bytes));
  NLGB_CUDA_TRY(cudaMalloc(&q, bytes));
  cudaError_t e = cudaSuccess;
  auto dot = [&](const double* u, const double* v) {
    double o = 0.0;
    if (e == cudaSuccess) e = dev_dot(u, v, n, &o, s);
    return o;
  };
  SysState h;
  std::memset(&h, 0, sizeof(h));
  h.thresh2 = eps * eps;
  h.rthresh2 = h.thresh2;
  h.max_iter = max_iter;
  h.status = ST_RUNNING;
  h.bnorm2 = dot(b, b);
  // r = b - A x, z = M^-1 r, p = z
  if (e == cudaSuccess) e = spmv64(A, x, r, s);
  if (e == cudaSuccess) { k_ssor_bmr<<<blocks_of(n), 256, 0, s>>>(n, b, r); count_launches(1); e = cudaGetLastError(); }
  if (e == cudaSuccess) e = P.apply(r, z, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(p, z, bytes, cudaMemcpyDeviceToDevice, s);
  h.rho = dot(r, z);
  h.rr = dot(r, r);
  if (!(h.bnorm2 > 0.0)) {
    if (e == cudaSuccess) e = cudaMemsetAsync(x, 0, bytes, s);
    h.status = h.bnorm2 == 0.0 ? ST_CONVERGED : ST_BREAKDOWN;
  } else if (h.rr <= h.thresh2 * h.bnorm2) {
    h.status = ST_CONVERGED;
  }
  for (;;) {
    while (e == cudaSuccess && h.status == ST_RUNNING) {
      if (h.iter >= h.max_iter) { h.status = ST_MAX_ITER; break; }
      e = spmv64(A, p, q, s);
      const double pq = dot(p, q);
      if (e != cudaSuccess) break;
      if (!(pq > 0.0 && pq < 1e300)) { h.status = ST_BREAKDOWN; break; }
      const double alpha = h.rho / pq;
      if (e == cudaSuccess) e = dev_axpy(n, alpha, p, x, s);
      if (e == cudaSuccess) e = dev_axpy(n, -alpha, q, r, s);
      if (e == cudaSuccess) e = P.apply(r, z, s);
      const double rz = dot(r, z), rr = dot(r, r);
      if (e != cudaSuccess) break;
      h.iter += 1;
      h.rr = rr;
      const bool rz_ok = rz > 0.0 && rz < 1e300;
      h.cont_ok = rz_ok ? 1 : 0;
      if (rz_ok) { h.beta = rz / h.rho; h.rho = rz; }
      if (!(rr <= 1e300)) { h.status = ST_BREAKDOWN; break; }
      if (rr <= h.rthresh2 * h.bnorm2) { h.status = ST_CONVERGED; break; }
      if (!rz_ok) { h.status = ST_BREAKDOWN; break; }
      k_ssor_p<<<blocks_of(n), 256, 0, s>>>(n, z, h.beta, p);
      count_launches(1);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) break;
    // true residual ||b - A x||, and a continuation while it misses eps
    e = spmv64(A, x, q, s);
    if (e == cudaSuccess) { k_ssor_bmr<<<blocks_of(n), 256, 0, s>>>(n, b, q); count_launches(1); e = cudaGetLastError(); }
    h.rr_true = dot(q, q);
    if (e != cudaSuccess || !scalar_after_check(&h)) break;
    k_ssor_p<<<blocks_of(n), 256, 0, s>>>(n, z, h.beta, p);
    count_launches(1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(r); cudaFree(z); cudaFree(p); cudaFree(q);
  if (e != cudaSuccess) {
    set_error(std::string("SSOR-preconditioned CG: ") + cudaGetErrorString(e));
    return e;
  }
  res->status = h.status;
  res->iterations = h.iter;
  res->rel_residual = h.bnorm2 > 0.0 ? std::sqrt(h.rr / h.bnorm2) : 0.0;
  res->true_rel_residual = h.bnorm2 > 0.0 ? std::sqrt(h.rr_true / h.bnorm2) : 0.0;
  return cudaSuccess;
}

}  // namespace nlgb
