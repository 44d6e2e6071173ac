// nlgb_internal.h -- host-side internals shared by the translation units of
// libnl_gb300 (not installed, not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

namespace nlgb {

struct SysState;
struct SysView;

// Thread-local error text reported by nlGetErrorString()/nlgb_last_error().
void set_error(const std::string& msg);
const char* last_error();

// Process-wide count of kernels launched by the library (host launches plus
// the kernel nodes executed by the solver graphs).
void count_launches(long long k);
long long launch_count();

#define NLGB_CUDA_TRY(expr)                                                     \
  do {                                                                          \
    cudaError_t e_ = (expr);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      ::nlgb::set_error(std::string(#expr) + ": " + cudaGetErrorString(e_));    \
      return e_;                                                                \
    }                                                                           \
  } while (0)

// A CRS matrix resident in GPU memory (int32 indices, FP64 values).
struct DeviceCRS {
  int n = 0;               // rows
  int m = 0;               // columns
  long long nnz = 0;
  int* rp = nullptr;
  int* ci = nullptr;
  double* va = nullptr;
  float* va32 = nullptr;   // lazily built for the mixed-precision solver
  double* dinv = nullptr;  // Jacobi inverse diagonal (lazily built)
  float* dinv32 = nullptr;
  float2* vadf = nullptr;    // double-float copies (hi, lo) of va and dinv,
  float2* dinvdf = nullptr;  //   lazily built for the double-float solver
  int df_state = 0;          // double-float range check: 0 not run, 1 usable, -1 out of range
  int tpr = 0;             // threads per row chosen by the autotuner
  int tile_rows = 0;
  int max_row = 0;         // longest row (nnz)
  bool owns = true;        // false: a view sharing another matrix's arrays
};

cudaError_t crs_upload(DeviceCRS& A, int n, int m, const int* rp, const int* ci,
                       const double* va, cudaStream_t s);
cudaError_t crs_adopt_device(DeviceCRS& A, int n, int m, long long nnz, int* rp, int* ci,
                             double* va, cudaStream_t s);
void crs_free(DeviceCRS& A);
// Stream-ordered release (no device-wide synchronisation): the arrays are
// freed when stream s reaches this point; work of other streams that used
// them must have completed.  The arrays of a DeviceCRS come from
// cudaMallocAsync (the device's default pool).
void crs_free_async(DeviceCRS& A, cudaStream_t s);
cudaError_t crs_prepare(DeviceCRS& A, bool need_fp32, cudaStream_t s);  // jacobi, fp32, tuning
// crs_prepare plus the double-float copies; *usable is false (and no copy is
// made) when a value or 1/diagonal lies outside [2^-100, 2^100] or is not
// finite: the double-float iteration would lose its precision there, and
// the caller runs FP64 instead.
cudaError_t crs_prepare_df(DeviceCRS& A, bool* usable, cudaStream_t s);
// In-place conversion of a device vector between FP64 and double-float
// (hi, lo) pairs, element by element (stream-ordered).
cudaError_t df_pack(double* x, long long n, cudaStream_t s);
cudaError_t df_unpack(double* x, long long n, cudaStream_t s);
long long device_bytes(const DeviceCRS& A);

// Autotuner: threads per row and tile rows from the nnz-per-row histogram.
struct TuneChoice { int tpr; int tile_rows; };
TuneChoice autotune(int n, long long nnz, int max_row, const int* hist33);
// 256-thread phase CTAs resident on the current device at once (SMs x 8).
long long phase_resident_slots();
cudaError_t row_histogram(const DeviceCRS& A, int* hist33_host, int* max_row, cudaStream_t s);

// SpMV y = A x with the autotuned layout (device pointers).
cudaError_t spmv64(const DeviceCRS& A, const double* x, double* y, cudaStream_t s);
cudaError_t spmv32(const DeviceCRS& A, const float* x, float* y, cudaStream_t s);

struct SolveParams {
  double eps = 1e-10;
  long long max_iter = -1;     // -1: 5 n
  int precision = 0;           // 0 FP64, 1 mixed, 3 double-float (NL_GB300_PRECISION_*)
  double inner_eps = 0.1;      // mixed: reliable update when the FP32 residual fell by this factor
  int max_outer = 100000;      // mixed: cap on reliable updates
  int tpr = 0;                 // 0: autotuned
};

struct SolveResult {
  int status = 0;
  long long iterations = 0;
  int outer_steps = 0;
  double rel_residual = 0;       // recursive (plain) / true FP64 (mixed) at stop
  double true_rel_residual = 0;  // ||b - A x|| / ||b|| recomputed in FP64
  double seconds = 0;
  double algo_bytes = 0;         // algorithmic HBM bytes of the solve
  int precision = 0;             // precision that ran (0 FP64, 1 mixed, 3 double-float)
};

// Plain FP64, double-float, or mixed FP32/FP64-refined Jacobi-PCG on one
// resident matrix.
// The whole iteration loop is a single CUDA-graph launch (while-conditional
// node); the host waits once per solve.
class PcgSolver {
 public:
  PcgSolver() = default;
  ~PcgSolver();
  PcgSolver(const PcgSolver&) = delete;
  PcgSolver& operator=(const PcgSolver&) = delete;

  cudaError_t bind(DeviceCRS* A, cudaStream_t stream);
  // b, x: device pointers of length n (x holds the initial guess on entry).
  cudaError_t solve(const double* b, double* x, const SolveParams& prm, SolveResult* res);
  void set_abort_flag(const volatile int* f) { abort_flag_ = f; }
  cudaStream_t stream() const { return stream_; }

 private:
  cudaError_t alloc(bool mixed);
  cudaError_t run_graph(bool mixed, bool df, const SolveParams& prm, long long max_iter,
                        long long done, int outer, float* ms);
  cudaError_t run_eager(bool mixed, bool df, SysState* h, bool cont = false);
  // continuation after a failed true-residual check (state: running, stage 4)
  cudaError_t run_cont(bool df, float* ms);
  cudaError_t add_plain_loop(cudaGraph_t g, cudaGraphNode_t dep, SysView* v, bool df,
                             cudaGraphNode_t* loop_out);
  cudaError_t build_plain_graph(bool df, bool cont = false);
  cudaError_t build_mixed_graph();
  void release();

  DeviceCRS* A_ = nullptr;
  cudaStream_t stream_ = nullptr;
  int tpr_ = 0;
  int n_ = 0, tile_rows_ = 0, n_tiles_ = 0;
  double *b_ = nullptr, *x_ = nullptr, *r_ = nullptr, *p_ = nullptr, *q_ = nullptr, *part_ = nullptr;
  float *r32_ = nullptr, *p32_ = nullptr, *q32_ = nullptr, *c32_ = nullptr;
  void* st_ = nullptr;          // SysState (device)
  void* st_host_ = nullptr;     // pinned staging
  const volatile int* abort_flag_ = nullptr;
  cudaGraphExec_t plain_exec_ = nullptr, mixed_exec_ = nullptr, df_exec_ = nullptr;
  cudaGraphExec_t cont_exec_ = nullptr, cont_df_exec_ = nullptr;
  // single-kernel cooperative iterations (small and mid-size systems)
  bool use_coop_ = false;
  int coop_grid_ = 0;
  unsigned long long* coop_bar_ = nullptr;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  bool mixed_alloc_ = false;
  long long graph_launches_ = 0;
};

// Least-squares normal equations assembled on the GPU (row-merge into CRS).
// Rows: coefficient ranges [row_ptr[r], row_ptr[r+1]) of (col, val) where
// col >= 0 is a free-variable index and col < 0 encodes locked variable
// (-col - 1); rhs[k * n_rows + r]; weight[r] (may be null: all 1).
// Locked values: xl[k * n_vars + var].  Output: CRS of A^T W A over the free
// variables and Aᵀ W (b - A_l x_l) for each of the k systems (device).
struct LSRowsDevice {
  long long n_rows = 0;
  long long n_coefs = 0;
  int n_free = 0;
  int n_vars = 0;
  int n_systems = 1;
  const long long* row_ptr = nullptr;
  const int* col = nullptr;
  const double* val = nullptr;
  const double* rhs = nullptr;
  const double* weight = nullptr;
  const double* xl = nullptr;
};
cudaError_t assemble_normal_equations(const LSRowsDevice& rows, DeviceCRS& out,
                                      double* rhs_out /* k * n_free, device */,
                                      cudaStream_t s);
// Square (non least-squares) system: rows are the equations of the free
// variables; locked columns move to the right-hand side.
cudaError_t assemble_square(const LSRowsDevice& rows, DeviceCRS& out, double* rhs_out,
                            cudaStream_t s);

// Mesh system builders (nlgb_build.cu).  Vertices xyz (n_verts x 3) and
// triangles (n_tris x 3) may be host or device arrays; *bad_input is set
// (and nothing built) when a triangle index is out of range.
// check_indices = false: the caller validated the triangle indices on the
// host (no device check, one host synchronisation less).
cudaError_t build_lscm_system(int n_verts, const double* xyz, int n_tris, const int* tris,
                              const int pins[2], const double pin_uv[4], DeviceCRS& out,
                              double* rhs_out /* 2 n_verts - 4, device */, cudaStream_t s,
                              bool* bad_input, bool check_indices = true);
cudaError_t build_fairing_system(int n_verts, const double* xyz, int n_tris, const int* tris,
                                 double lambda, DeviceCRS& out, cudaStream_t s, bool* bad_input,
                                 bool check_indices = true);

// Krylov solvers for general square systems (nlgb_krylov.cu): BiCGSTAB and
// restarted GMRES(restart), FP64, right preconditioning by dinv (Jacobi; all
// ones for none).  b, x: device vectors of A.n (x: initial guess, replaced).
enum { KRYLOV_BICGSTAB = 1, KRYLOV_GMRES = 2 };
struct KrylovResult {
  int status = 0;                 // ST_* (nlgb_core.cuh)
  long long iterations = 0;       // BiCGSTAB iterations / GMRES inner steps
  double rel_residual = 0.0;      // recursive (BiCGSTAB) / restart-time true (GMRES)
  double true_rel_residual = 0.0; // ||b - A x|| / ||b|| of the returned x
};
struct SsorPrecond;
// P (may be null): a general preconditioner (SSOR) applied instead of the
// diagonal one; dinv must then be all ones.
cudaError_t krylov_solve(const DeviceCRS& A, const double* dinv, const double* b, double* x,
                         int method, double eps, long long max_iter, int restart, cudaStream_t s,
                         KrylovResult* res, SsorPrecond* P = nullptr);

// SSOR preconditioner of a symmetric CRS matrix (nlgb_ssor.cu):
// M = (D + w L) D^-1 (D + w L^T) / (w (2 - w)); apply() computes z = M^-1 r
// by level-scheduled forward and backward sweeps (each row as the sequential
// sweep computes it, the rows of a level in parallel).  A must outlive it.
struct SsorPrecond {
  int n = 0;
  double omega = 1.5;
  const DeviceCRS* A = nullptr;
  int* rows_f = nullptr;         // rows grouped by forward-sweep level
  int* rows_b = nullptr;         // rows grouped by backward-sweep level
  std::vector<int> ptr_f, ptr_b; // level boundaries (host)
  double* diag = nullptr;        // a_ii (1 where missing or zero)
  double* y = nullptr;           // forward-sweep result
  struct Cached { const double* r; double* z; cudaGraphExec_t exec; };
  std::vector<Cached> graphs;    // captured sweeps per (r, z) pair of the solve
  SsorPrecond() = default;
  SsorPrecond(const SsorPrecond&) = delete;
  SsorPrecond& operator=(const SsorPrecond&) = delete;
  ~SsorPrecond() { release(); }
  cudaError_t build(const DeviceCRS& A, double omega, cudaStream_t s);
  cudaError_t apply(const double* r, double* z, cudaStream_t s);   // r, z device vectors
  void release();

 private:
  cudaError_t launch_sweeps(const double* r, double* z, cudaStream_t s);
};
struct KrylovResult;
// CG with the SSOR preconditioner (FP64; true-residual check as the other
// FP64 solvers).  b, x device vectors (x: initial guess, replaced).
cudaError_t pcg_ssor(const DeviceCRS& A, SsorPrecond& P, const double* b, double* x, double eps,
                     long long max_iter, cudaStream_t s, KrylovResult* res);

// Device BLAS-1 (FP64).
cudaError_t dev_dot(const double* x, const double* y, long long n, double* out_host, cudaStream_t s);
cudaError_t dev_axpy(long long n, double a, const double* x, double* y, cudaStream_t s);
cudaError_t dev_scal(long long n, double a, double* x, cudaStream_t s);
cudaError_t dev_mul(long long n, const double* x, double* y, cudaStream_t s);
// Strided BLAS-1 (increments as in BLAS, negative ones walk backwards).
cudaError_t dev_dot_s(const double* x, int incx, const double* y, int incy, long long n, double* out_host,
                      cudaStream_t s);
cudaError_t dev_axpy_s(long long n, double a, const double* x, int incx, double* y, int incy, cudaStream_t s);
cudaError_t dev_scal_s(long long n, double a, double* x, int incx, cudaStream_t s);
cudaError_t dev_copy_s(long long n, const double* x, int incx, double* y, int incy, cudaStream_t s);

// Process-wide default stream of the OpenNL API (created on first use).
cudaStream_t api_stream();
bool is_device_pointer(const void* p);

}  // namespace nlgb
