// nlgb_api.cpp -- explicit-handle C API (include/nl_gb300.h).
#include "../../include/nl.h"
#include "../../include/nl_gb300.h"
#include "nlgb_batch.h"
#include "nlgb_internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

using namespace nlgb;

struct nlgb_matrix_s {
  DeviceCRS A;
  PcgSolver pcg;
  bool bound = false;
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ~nlgb_matrix_s() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    crs_free(A);
  }
};

namespace {

int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}

bool ensure_ready() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error("no CUDA device available");
    return false;
  }
  return true;
}

// Copy a host-or-device array of `count` T into a fresh device allocation.
template <typename T>
cudaError_t to_device(const T* src, size_t count, T** dst, cudaStream_t s) {
  *dst = nullptr;
  NLGB_CUDA_TRY(cudaMalloc(dst, std::max<size_t>(1, count) * sizeof(T)));
  if (count) NLGB_CUDA_TRY(cudaMemcpyAsync(*dst, src, count * sizeof(T), cudaMemcpyDefault, s));
  return cudaSuccess;
}

struct Stage {
  double* d = nullptr;
  bool owned = false;
  ~Stage() { if (owned) cudaFree(d); }
  cudaError_t in(const double* p, size_t n, cudaStream_t s, bool copy) {
    if (is_device_pointer(p)) { d = const_cast<double*>(p); return cudaSuccess; }
    NLGB_CUDA_TRY(cudaMalloc(&d, std::max<size_t>(1, n) * sizeof(double)));
    owned = true;
    if (copy && n) NLGB_CUDA_TRY(cudaMemcpyAsync(d, p, n * sizeof(double), cudaMemcpyHostToDevice, s));
    return cudaSuccess;
  }
  cudaError_t out(double* p, size_t n, cudaStream_t s) {
    if (owned && n) NLGB_CUDA_TRY(cudaMemcpyAsync(p, d, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    return cudaSuccess;
  }
};

cudaError_t matrix_stream(nlgb_matrix M) {
  if (!M->stream) {
    NLGB_CUDA_TRY(cudaStreamCreateWithFlags(&M->stream, cudaStreamNonBlocking));
    NLGB_CUDA_TRY(cudaEventCreate(&M->e0));
    NLGB_CUDA_TRY(cudaEventCreate(&M->e1));
  }
  return cudaSuccess;
}

}  // namespace

extern "C" {

int nlgb_device_available(void) { return ensure_ready() ? 1 : 0; }
long long nlgb_kernel_launches(void) { return launch_count(); }
const char* nlgb_last_error(void) { return last_error(); }

void nlgb_default_params(nlgb_params* p) {
  if (!p) return;
  p->eps = 1e-10;
  p->max_iter = -1;
  p->precision = NL_GB300_PRECISION_DOUBLE;
  p->inner_eps = 0.1;
  p->max_outer = 100000;
}

nlgb_matrix nlgb_matrix_create(int n_rows, int n_cols, const int* rp, const int* ci,
                               const double* va) {
  if (n_rows < 0 || n_cols < 0 || !rp) { set_error("nlgb_matrix_create: bad arguments"); return nullptr; }
  if (!ensure_ready()) return nullptr;
  nlgb_matrix M = new nlgb_matrix_s();
  if (matrix_stream(M) != cudaSuccess) { delete M; return nullptr; }
  cudaStream_t s = M->stream;
  // Row pointers: validate on the host (monotone, in range) before upload.
  std::vector<int> hrp((size_t)n_rows + 1);
  if (cudaMemcpy(hrp.data(), rp, sizeof(int) * hrp.size(), cudaMemcpyDefault) != cudaSuccess) {
    set_error("nlgb_matrix_create: cannot read row pointers");
    delete M;
    return nullptr;
  }
  if (hrp[0] != 0) { set_error("nlgb_matrix_create: rp[0] != 0"); delete M; return nullptr; }
  for (int i = 0; i < n_rows; ++i)
    if (hrp[i + 1] < hrp[i]) { set_error("nlgb_matrix_create: row pointers not monotone"); delete M; return nullptr; }
  const long long nnz = hrp[n_rows];
  std::vector<int> hci((size_t)nnz);
  if (nnz && cudaMemcpy(hci.data(), ci, sizeof(int) * nnz, cudaMemcpyDefault) != cudaSuccess) {
    set_error("nlgb_matrix_create: cannot read column indices");
    delete M;
    return nullptr;
  }
  for (long long k = 0; k < nnz; ++k)
    if (hci[k] < 0 || hci[k] >= n_cols) { set_error("nlgb_matrix_create: column index out of range"); delete M; return nullptr; }
  int *drp = nullptr, *dci = nullptr;
  double* dva = nullptr;
  if (to_device(hrp.data(), hrp.size(), &drp, s) != cudaSuccess ||
      to_device(hci.data(), (size_t)nnz, &dci, s) != cudaSuccess ||
      to_device(va, (size_t)nnz, &dva, s) != cudaSuccess) {
    cudaFree(drp); cudaFree(dci); cudaFree(dva);
    delete M;
    return nullptr;
  }
  crs_adopt_device(M->A, n_rows, n_cols, nnz, drp, dci, dva, s);
  if (crs_prepare(M->A, false, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
    delete M;
    return nullptr;
  }
  return M;
}

void nlgb_matrix_destroy(nlgb_matrix A) {
  if (!A) return;
  if (A->stream) cudaStreamSynchronize(A->stream);
  cudaStream_t s = A->stream;
  delete A;
  if (s) cudaStreamDestroy(s);
}

int nlgb_matrix_info(nlgb_matrix A, int* n_rows, long long* nnz, int* tpr, int* tile_rows) {
  if (!A) return fail(NLGB_E_INVALID, "nlgb_matrix_info: null matrix");
  if (n_rows) *n_rows = A->A.n;
  if (nnz) *nnz = A->A.nnz;
  if (tpr) *tpr = A->A.tpr;
  if (tile_rows) *tile_rows = A->A.tile_rows;
  return NLGB_OK;
}

int nlgb_matrix_set_layout(nlgb_matrix A, int tpr, int tile_rows) {
  if (!A) return fail(NLGB_E_INVALID, "nlgb_matrix_set_layout: null matrix");
  if (tpr != 0 && tpr != 1 && tpr != 2 && tpr != 4 && tpr != 8 && tpr != 16 && tpr != 32)
    return fail(NLGB_E_INVALID, "threads_per_row must be 0 or a power of two <= 32");
  if (tile_rows != 0 && (tile_rows < 64 || tile_rows % 64 != 0 || tile_rows > (1 << 20)))
    return fail(NLGB_E_INVALID, "tile_rows must be a multiple of 64 in [64, 2^20]");
  if (tpr) A->A.tpr = tpr;
  if (tile_rows) A->A.tile_rows = tile_rows;
  A->bound = false;   // the solver's graphs embed the layout
  return NLGB_OK;
}

int nlgb_matrix_download(nlgb_matrix A, int* rp, int* ci, double* va) {
  if (!A) return fail(NLGB_E_INVALID, "nlgb_matrix_download: null matrix");
  if (rp && cudaMemcpy(rp, A->A.rp, sizeof(int) * (A->A.n + 1), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(NLGB_E_DEVICE, "download failed");
  if (ci && A->A.nnz && cudaMemcpy(ci, A->A.ci, sizeof(int) * A->A.nnz, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(NLGB_E_DEVICE, "download failed");
  if (va && A->A.nnz && cudaMemcpy(va, A->A.va, sizeof(double) * A->A.nnz, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(NLGB_E_DEVICE, "download failed");
  return NLGB_OK;
}

int nlgb_matrix_jacobi(nlgb_matrix A, double* dinv) {
  if (!A || !dinv) return fail(NLGB_E_INVALID, "nlgb_matrix_jacobi: bad arguments");
  if (cudaMemcpy(dinv, A->A.dinv, sizeof(double) * A->A.n, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(NLGB_E_DEVICE, "download failed");
  return NLGB_OK;
}

int nlgb_spmv(nlgb_matrix A, const double* x, double* y) {
  if (!A) return fail(NLGB_E_INVALID, "nlgb_spmv: null matrix");
  cudaStream_t s = A->stream;
  Stage sx, sy;
  if (sx.in(x, A->A.m, s, true) != cudaSuccess || sy.in(y, A->A.n, s, false) != cudaSuccess)
    return NLGB_E_DEVICE;
  if (spmv64(A->A, sx.d, sy.d, s) != cudaSuccess) return NLGB_E_DEVICE;
  if (sy.out(y, A->A.n, s) != cudaSuccess) return NLGB_E_DEVICE;
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail(NLGB_E_DEVICE, cudaGetErrorString(cudaGetLastError()));
  return NLGB_OK;
}

int nlgb_spmv32(nlgb_matrix A, const float* x, float* y) {
  if (!A) return fail(NLGB_E_INVALID, "nlgb_spmv32: null matrix");
  if (crs_prepare(A->A, true, A->stream) != cudaSuccess) return NLGB_E_DEVICE;
  if (spmv32(A->A, x, y, A->stream) != cudaSuccess) return NLGB_E_DEVICE;
  if (cudaStreamSynchronize(A->stream) != cudaSuccess) return fail(NLGB_E_DEVICE, cudaGetErrorString(cudaGetLastError()));
  return NLGB_OK;
}

int nlgb_spmv_timed(nlgb_matrix A, const double* x, double* y, int reps, double* ms) {
  if (!A || reps <= 0) return fail(NLGB_E_INVALID, "nlgb_spmv_timed: bad arguments");
  cudaStream_t s = A->stream;
  if (cudaEventRecord(A->e0, s) != cudaSuccess) return NLGB_E_DEVICE;
  for (int r = 0; r < reps; ++r)
    if (spmv64(A->A, x, y, s) != cudaSuccess) return NLGB_E_DEVICE;
  cudaEventRecord(A->e1, s);
  if (cudaEventSynchronize(A->e1) != cudaSuccess) return fail(NLGB_E_DEVICE, cudaGetErrorString(cudaGetLastError()));
  float t = 0.f;
  cudaEventElapsedTime(&t, A->e0, A->e1);
  if (ms) *ms = double(t) / reps;
  return NLGB_OK;
}

int nlgb_spmv32_timed(nlgb_matrix A, const float* x, float* y, int reps, double* ms) {
  if (!A || reps <= 0) return fail(NLGB_E_INVALID, "nlgb_spmv32_timed: bad arguments");
  cudaStream_t s = A->stream;
  if (crs_prepare(A->A, true, s) != cudaSuccess) return NLGB_E_DEVICE;
  if (cudaEventRecord(A->e0, s) != cudaSuccess) return NLGB_E_DEVICE;
  for (int r = 0; r < reps; ++r)
    if (spmv32(A->A, x, y, s) != cudaSuccess) return NLGB_E_DEVICE;
  cudaEventRecord(A->e1, s);
  if (cudaEventSynchronize(A->e1) != cudaSuccess) return fail(NLGB_E_DEVICE, cudaGetErrorString(cudaGetLastError()));
  float t = 0.f;
  cudaEventElapsedTime(&t, A->e0, A->e1);
  if (ms) *ms = double(t) / reps;
  return NLGB_OK;
}

int nlgb_solve(nlgb_matrix A, const double* b, double* x, const nlgb_params* prm, nlgb_result* res) {
  if (!A || !b || !x) return fail(NLGB_E_INVALID, "nlgb_solve: bad arguments");
  if (A->A.n != A->A.m) return fail(NLGB_E_INVALID, "nlgb_solve: matrix is not square");
  nlgb_params p;
  nlgb_default_params(&p);
  if (prm) p = *prm;
  if (p.precision != NL_GB300_PRECISION_DOUBLE && p.precision != NL_GB300_PRECISION_MIXED &&
      p.precision != NL_GB300_PRECISION_AUTO && p.precision != NL_GB300_PRECISION_DOUBLE_FLOAT)
    return fail(NLGB_E_INVALID, "nlgb_solve: unknown precision");
  // a matrix given directly is square: AUTO means mixed
  if (p.precision == NL_GB300_PRECISION_AUTO) p.precision = NL_GB300_PRECISION_MIXED;
  if (!(p.eps >= 0.0) || !(p.inner_eps > 0.0 && p.inner_eps < 1.0) || p.max_outer < 1)
    return fail(NLGB_E_INVALID, "nlgb_solve: bad tolerances");
  cudaStream_t s = A->stream;
  if (!A->bound) {
    if (A->pcg.bind(&A->A, s) != cudaSuccess) return NLGB_E_DEVICE;
    A->bound = true;
  }
  Stage sb, sx;
  const size_t n = (size_t)A->A.n;
  if (sb.in(b, n, s, true) != cudaSuccess || sx.in(x, n, s, true) != cudaSuccess) return NLGB_E_DEVICE;
  SolveParams sp;
  sp.eps = p.eps;
  sp.max_iter = p.max_iter;
  sp.precision = p.precision;
  sp.inner_eps = p.inner_eps;
  sp.max_outer = p.max_outer;
  SolveResult r;
  if (A->pcg.solve(sb.d, sx.d, sp, &r) != cudaSuccess) return NLGB_E_DEVICE;
  if (sx.out(x, n, s) != cudaSuccess) return NLGB_E_DEVICE;
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail(NLGB_E_DEVICE, cudaGetErrorString(cudaGetLastError()));
  if (res) {
    res->status = r.status;
    res->iterations = r.iterations;
    res->refinement_steps = r.outer_steps;
    res->rel_residual = r.rel_residual;
    res->true_rel_residual = r.true_rel_residual;
    res->seconds = r.seconds;
    res->algo_bytes = r.algo_bytes;
    res->precision = r.precision;
  }
  return NLGB_OK;
}

int nlgb_batch_solve(int n_sys, const nlgb_matrix* A, const double* const* b, double* const* x,
                     const nlgb_params* prm, nlgb_result* res, double* kernel_seconds) {
  if (n_sys < 0 || (n_sys > 0 && (!A || !b || !x))) return fail(NLGB_E_INVALID, "nlgb_batch_solve: bad arguments");
  for (int i = 0; i < n_sys; ++i) {
    if (!A[i] || !b[i] || !x[i]) return fail(NLGB_E_INVALID, "nlgb_batch_solve: null matrix or vector");
    if (A[i]->A.n != A[i]->A.m) return fail(NLGB_E_INVALID, "nlgb_batch_solve: matrix is not square");
  }
  nlgb_params p;
  nlgb_default_params(&p);
  if (prm) p = *prm;
  if (p.precision != NL_GB300_PRECISION_DOUBLE && p.precision != NL_GB300_PRECISION_MIXED &&
      p.precision != NL_GB300_PRECISION_AUTO && p.precision != NL_GB300_PRECISION_DOUBLE_FLOAT)
    return fail(NLGB_E_INVALID, "nlgb_batch_solve: unknown precision");
  // a matrix given directly is square: AUTO means mixed
  if (p.precision == NL_GB300_PRECISION_AUTO) p.precision = NL_GB300_PRECISION_MIXED;
  if (n_sys == 0) return NLGB_OK;
  if (!ensure_ready()) return NLGB_E_DEVICE;
  const bool mixed = p.precision == NL_GB300_PRECISION_MIXED;
  SolveParams sp;
  sp.eps = p.eps; sp.max_iter = p.max_iter; sp.precision = p.precision;
  sp.inner_eps = p.inner_eps; sp.max_outer = p.max_outer;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return NLGB_E_DEVICE;
  std::vector<SystemSlot> slots((size_t)n_sys);
  std::vector<SysView> views((size_t)n_sys);
  std::vector<long long> work((size_t)n_sys);
  int rc = NLGB_OK;
  {
    BatchRunner runner;
    if (runner.init(s) != cudaSuccess) rc = NLGB_E_DEVICE;
    for (int i = 0; i < n_sys && rc == NLGB_OK; ++i) {
      DeviceCRS& M = A[i]->A;
      bool dfl = false;
      if (crs_prepare(M, mixed, s) != cudaSuccess ||
          (p.precision == NL_GB300_PRECISION_DOUBLE_FLOAT && crs_prepare_df(M, &dfl, s) != cudaSuccess) ||
          slots[i].alloc(&M, mixed, s, dfl) != cudaSuccess || slots[i].start(b[i], x[i], sp, s) != cudaSuccess) {
        rc = NLGB_E_DEVICE;
        break;
      }
      views[i] = slots[i].view;
      // bytes per iteration x an iteration-count proxy: Jacobi-CG on a 2D
      // mesh operator needs O(sqrt(kappa)) = O(sqrt(n)) iterations
      work[i] = (long long)((double)(M.nnz + 8LL * M.n) * std::sqrt((double)std::max(1, M.n)));
    }
    BatchLaunchStats st;
    if (rc == NLGB_OK && runner.run(views, work, 0, &st) != cudaSuccess) rc = NLGB_E_DEVICE;
    if (rc == NLGB_OK && kernel_seconds) *kernel_seconds = st.ms * 1e-3;
    std::vector<SysState> hs((size_t)n_sys);
    for (int i = 0; i < n_sys && rc == NLGB_OK; ++i) {
      if ((slots[i].df && df_unpack(slots[i].view.x, A[i]->A.n, s) != cudaSuccess) ||
          cudaMemcpyAsync(x[i], slots[i].view.x, sizeof(double) * A[i]->A.n, cudaMemcpyDefault, s) != cudaSuccess ||
          cudaMemcpyAsync(&hs[i], slots[i].view.st, sizeof(SysState), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        rc = NLGB_E_DEVICE;
    }
    if (rc == NLGB_OK && cudaStreamSynchronize(s) != cudaSuccess) rc = NLGB_E_DEVICE;
    if (rc == NLGB_OK && res) {
      for (int i = 0; i < n_sys; ++i) {
        const SysState& h = hs[i];
        res[i].status = h.status;
        res[i].iterations = h.iter;
        res[i].refinement_steps = h.outer;
        res[i].rel_residual = h.bnorm2 > 0 ? std::sqrt(h.rr / h.bnorm2) : 0.0;
        res[i].true_rel_residual = h.bnorm2 > 0 ? std::sqrt(h.rr_true / h.bnorm2) : 0.0;
        res[i].seconds = st.ms * 1e-3;
        res[i].algo_bytes = algo_bytes(A[i]->A.n, A[i]->A.nnz, h);
        res[i].precision = mixed ? NL_GB300_PRECISION_MIXED
                                 : (slots[i].df ? NL_GB300_PRECISION_DOUBLE_FLOAT : NL_GB300_PRECISION_DOUBLE);
      }
    }
    for (auto& sl : slots) sl.release(s);
    cudaStreamSynchronize(s);
  }
  cudaStreamDestroy(s);
  if (rc != NLGB_OK && std::string(last_error()).empty()) set_error(cudaGetErrorString(cudaGetLastError()));
  return rc;
}

int nlgb_assemble(int least_squares, long long n_rows, const long long* row_ptr, const int* col,
                  const double* val, const double* rhs, const double* weight, int n_free,
                  int n_vars, const double* xl, int n_systems, nlgb_matrix* A_out,
                  double* rhs_out, double* seconds) {
  if (!A_out || !row_ptr || n_rows < 0 || n_free < 0 || n_systems < 1)
    return fail(NLGB_E_INVALID, "nlgb_assemble: bad arguments");
  *A_out = nullptr;
  const long long n_coefs = row_ptr[n_rows];
  for (long long k = 0; k < n_coefs; ++k) {
    const int c = col[k];
    if (c >= n_free || (c < 0 && (-(long long)c - 1) >= n_vars))
      return fail(NLGB_E_INVALID, "nlgb_assemble: coefficient index out of range");
  }
  if (!ensure_ready()) return NLGB_E_DEVICE;
  nlgb_matrix M = new nlgb_matrix_s();
  if (matrix_stream(M) != cudaSuccess) { delete M; return NLGB_E_DEVICE; }
  cudaStream_t s = M->stream;
  long long* drp = nullptr; int* dcol = nullptr;
  double *dval = nullptr, *drhs = nullptr, *dw = nullptr, *dxl = nullptr, *dout = nullptr;
  auto cleanup = [&]() { cudaFree(drp); cudaFree(dcol); cudaFree(dval); cudaFree(drhs); cudaFree(dw); cudaFree(dxl); cudaFree(dout); };
  const auto t0 = std::chrono::steady_clock::now();
  bool ok = to_device(row_ptr, (size_t)n_rows + 1, &drp, s) == cudaSuccess &&
            to_device(col, (size_t)n_coefs, &dcol, s) == cudaSuccess &&
            to_device(val, (size_t)n_coefs, &dval, s) == cudaSuccess &&
            to_device(rhs, rhs ? (size_t)n_systems * n_rows : 0, &drhs, s) == cudaSuccess &&
            to_device(weight, weight ? (size_t)n_rows : 0, &dw, s) == cudaSuccess &&
            to_device(xl, xl ? (size_t)n_systems * n_vars : 0, &dxl, s) == cudaSuccess &&
            cudaMalloc(&dout, sizeof(double) * std::max<size_t>(1, (size_t)n_systems * n_free)) == cudaSuccess;
  if (!ok) { cleanup(); delete M; return NLGB_E_DEVICE; }
  LSRowsDevice R;
  R.n_rows = n_rows; R.n_coefs = n_coefs; R.n_free = n_free; R.n_vars = n_vars;
  R.n_systems = n_systems; R.row_ptr = drp; R.col = dcol; R.val = dval;
  R.rhs = rhs ? drhs : nullptr; R.weight = weight ? dw : nullptr; R.xl = dxl;
  cudaError_t e = least_squares ? assemble_normal_equations(R, M->A, dout, s)
                                : assemble_square(R, M->A, dout, s);
  if (e != cudaSuccess) { cleanup(); delete M; return e == cudaErrorInvalidValue ? NLGB_E_INVALID : NLGB_E_DEVICE; }
  if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (rhs_out && n_free > 0 &&
      cudaMemcpyAsync(rhs_out, dout, sizeof(double) * (size_t)n_systems * n_free, cudaMemcpyDefault, s) != cudaSuccess) {
    cleanup(); delete M; return NLGB_E_DEVICE;
  }
  if (crs_prepare(M->A, false, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
    cleanup(); delete M; return NLGB_E_DEVICE;
  }
  cleanup();
  *A_out = M;
  return NLGB_OK;
}

int nlgb_solve_krylov(nlgb_matrix A, const double* b, double* x, int method, double eps,
                      long long max_iter, int restart, int jacobi, nlgb_result* res) {
  if (!A || !b || !x) return fail(NLGB_E_INVALID, "nlgb_solve_krylov: bad arguments");
  if (A->A.n != A->A.m) return fail(NLGB_E_INVALID, "nlgb_solve_krylov: matrix is not square");
  if (method != NLGB_KRYLOV_BICGSTAB && method != NLGB_KRYLOV_GMRES)
    return fail(NLGB_E_INVALID, "nlgb_solve_krylov: unknown method");
  if (!(eps >= 0.0) || restart < 1) return fail(NLGB_E_INVALID, "nlgb_solve_krylov: bad parameters");
  cudaStream_t s = A->stream;
  const size_t n = (size_t)A->A.n;
  Stage sb, sx;
  if (sb.in(b, n, s, true) != cudaSuccess || sx.in(x, n, s, true) != cudaSuccess) return NLGB_E_DEVICE;
  double* ones = nullptr;
  const double* dinv = A->A.dinv;
  if (!jacobi) {
    std::vector<double> h(std::max<size_t>(1, n), 1.0);
    if (cudaMalloc(&ones, sizeof(double) * h.size()) != cudaSuccess ||
        cudaMemcpy(ones, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaFree(ones);
      return fail(NLGB_E_DEVICE, "nlgb_solve_krylov: allocation failed");
    }
    dinv = ones;
  }
  cudaEventRecord(A->e0, s);
  KrylovResult kr;
  const cudaError_t e = krylov_solve(A->A, dinv, sb.d, sx.d,
                                     method == NLGB_KRYLOV_BICGSTAB ? KRYLOV_BICGSTAB : KRYLOV_GMRES, eps,
                                     max_iter >= 0 ? max_iter : 5LL * (long long)n, restart, s, &kr);
  cudaEventRecord(A->e1, s);
  cudaFree(ones);
  if (e != cudaSuccess) return fail(NLGB_E_DEVICE, cudaGetErrorString(e));
  if (sx.out(x, n, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) return NLGB_E_DEVICE;
  if (res) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, A->e0, A->e1);
    std::memset(res, 0, sizeof(*res));
    res->status = kr.status;
    res->iterations = kr.iterations;
    res->rel_residual = kr.rel_residual;
    res->true_rel_residual = kr.true_rel_residual;
    res->seconds = ms * 1e-3;
  }
  return NLGB_OK;
}

int nlgb_build_lscm(int n_verts, const double* xyz, int n_tris, const int* tris, const int* pins,
                    const double* pin_uv, nlgb_matrix* A_out, double* rhs_out, double* seconds) {
  if (!A_out) return fail(NLGB_E_INVALID, "nlgb_build_lscm: bad arguments");
  *A_out = nullptr;
  if (n_verts < 3 || n_tris < 0 || !xyz || (n_tris > 0 && !tris))
    return fail(NLGB_E_INVALID, "nlgb_build_lscm: bad arguments");
  if (n_verts > (1 << 30) - 1 || (long long)n_tris * 12 > (1LL << 40))
    return fail(NLGB_E_INVALID, "nlgb_build_lscm: mesh too large (2 n_verts variables must fit in int)");
  const int pv[2] = {pins ? pins[0] : 0, pins ? pins[1] : n_verts - 1};
  const double uv[4] = {pin_uv ? pin_uv[0] : 0.0, pin_uv ? pin_uv[1] : 0.0,
                        pin_uv ? pin_uv[2] : 1.0, pin_uv ? pin_uv[3] : 1.0};
  if (pv[0] < 0 || pv[0] >= n_verts || pv[1] < 0 || pv[1] >= n_verts || pv[0] == pv[1])
    return fail(NLGB_E_INVALID, "nlgb_build_lscm: the two pins must be distinct vertices");
  if (!ensure_ready()) return NLGB_E_DEVICE;
  nlgb_matrix M = new nlgb_matrix_s();
  if (matrix_stream(M) != cudaSuccess) { delete M; return NLGB_E_DEVICE; }
  cudaStream_t s = M->stream;
  const int n_free = 2 * n_verts - 4;
  double* drhs = nullptr;
  if (cudaMalloc(&drhs, sizeof(double) * (size_t)std::max(1, n_free)) != cudaSuccess) { delete M; return NLGB_E_DEVICE; }
  const auto t0 = std::chrono::steady_clock::now();
  bool bad = false;
  cudaError_t e = build_lscm_system(n_verts, xyz, n_tris, tris, pv, uv, M->A, drhs, s, &bad);
  if (e == cudaSuccess && !bad) e = crs_prepare(M->A, false, s);
  if (e == cudaSuccess && !bad) e = cudaStreamSynchronize(s);
  if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (e == cudaSuccess && !bad && rhs_out)
    e = cudaMemcpy(rhs_out, drhs, sizeof(double) * (size_t)n_free, cudaMemcpyDefault);
  cudaFree(drhs);
  if (bad) { delete M; return fail(NLGB_E_INVALID, "nlgb_build_lscm: triangle index out of range"); }
  if (e != cudaSuccess) { delete M; return fail(NLGB_E_DEVICE, cudaGetErrorString(e)); }
  *A_out = M;
  return NLGB_OK;
}

int nlgb_build_fairing(int n_verts, const double* xyz, int n_tris, const int* tris, double lambda,
                       nlgb_matrix* A_out, double* seconds) {
  if (!A_out) return fail(NLGB_E_INVALID, "nlgb_build_fairing: bad arguments");
  *A_out = nullptr;
  if (n_verts < 1 || n_tris < 0 || !xyz || (n_tris > 0 && !tris) || !(lambda >= 0.0))
    return fail(NLGB_E_INVALID, "nlgb_build_fairing: bad arguments");
  if (!ensure_ready()) return NLGB_E_DEVICE;
  nlgb_matrix M = new nlgb_matrix_s();
  if (matrix_stream(M) != cudaSuccess) { delete M; return NLGB_E_DEVICE; }
  cudaStream_t s = M->stream;
  const auto t0 = std::chrono::steady_clock::now();
  bool bad = false;
  cudaError_t e = build_fairing_system(n_verts, xyz, n_tris, tris, lambda, M->A, s, &bad);
  if (e == cudaSuccess && !bad) e = crs_prepare(M->A, false, s);
  if (e == cudaSuccess && !bad) e = cudaStreamSynchronize(s);
  if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (bad) { delete M; return fail(NLGB_E_INVALID, "nlgb_build_fairing: triangle index out of range"); }
  if (e != cudaSuccess) { delete M; return fail(NLGB_E_DEVICE, cudaGetErrorString(e)); }
  *A_out = M;
  return NLGB_OK;
}

}  // extern "C"
