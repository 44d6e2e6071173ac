// nl_api.cpp -- the OpenNL C API of libnl_gb300 (declared in include/nl.h).
//
// Context API: the call sequence of plugins/OGF/WarpDrive/commands/
// voxel_grob_transport_commands.cpp:231-287 (nlNewContext, nlSolverParameteri,
// nlEnable, nlBegin/nlEnd(NL_SYSTEM/NL_MATRIX/NL_ROW), nlSetVariable,
// nlLockVariable, nlCoefficient, nlSolve, nlGetVariable, nlDeleteContext).
// Matrix API: src/lib/OGF/scene_graph/NL/matrix.cpp (nlSparseMatrixNew/Add,
// nlMatrixCompress, nlMultMatrixVector, nlNewJacobiPreconditioner,
// nlNewSSORPreconditioner, nlSolveSystemIterative, nlMatrixFactorize,
// nlInitExtension) and blas.cpp (nlHostBlas).
//
// The host side only records rows and variables; everything numeric (the
// normal-equation assembly, the SpMV, the PCG, BLAS-1) runs on the GPU.  There
// is no CPU fallback: without a CUDA device nlSolve reports an error and
// returns NL_FALSE.
#include "../../include/nl.h"
#include "nlgb_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

namespace nlgb {

static thread_local std::string g_error;
static thread_local NLenum g_error_code = NL_NO_ERROR;

void set_error(const std::string& msg) { g_error = msg; }
const char* last_error() { return g_error.c_str(); }

static std::atomic<long long> g_launches{0};
void count_launches(long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

static bool quiet() {
  static int q = -1;
  if (q < 0) {
    const char* e = std::getenv("NLGB_QUIET");
    q = (e && e[0] == '1') ? 1 : 0;
  }
  return q == 1;
}

static void nl_error(NLenum code, const std::string& msg) {
  g_error_code = code;
  g_error = msg;
  if (!quiet()) std::fprintf(stderr, "OpenNL(gb300) error: %s\n", msg.c_str());
}

static std::mutex g_stream_mu;
static cudaStream_t g_stream = nullptr;

cudaStream_t api_stream() {
  std::lock_guard<std::mutex> lk(g_stream_mu);
  if (!g_stream) cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking);
  return g_stream;
}

bool is_device_pointer(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static bool device_ready(std::string* why) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    if (why) *why = std::string("no CUDA device available (") + cudaGetErrorString(e) + ")";
    return false;
  }
  return true;
}

}  // namespace nlgb

using namespace nlgb;

// ===========================================================================
// Context
// ===========================================================================
namespace {

enum State {
  S_INITIAL, S_SYSTEM, S_MATRIX, S_ROW, S_MATRIX_CONSTRUCTED, S_SYSTEM_CONSTRUCTED, S_SOLVED
};

struct Context {
  // parameters
  long long nb_variables = 0;
  bool least_squares = false;
  NLenum solver = NL_SOLVER_DEFAULT;
  NLenum precond = NL_PRECOND_JACOBI;
  int inner_iterations = 5;     // GMRES restart length (NL_INNER_ITERATIONS)
  double threshold = 1e-10;
  long long max_iterations = -1;
  int nb_systems = 1;
  bool symmetric = false;
  int precision = NL_GB300_PRECISION_DOUBLE;
  double inner_threshold = 0.1;
  int max_refinement = 100000;
  int tpr_override = 0;
  bool verbose = false;
  bool normalize_rows = false;
  double omega = 1.5;

  State state = S_INITIAL;
  // variables (value[k * n + i])
  std::vector<double> values;
  std::vector<unsigned char> locked;
  std::vector<int> free_index;   // var -> free index, -1 if locked
  std::vector<int> free_vars;    // free index -> var
  // row stream (col >= 0: free index; col < 0: locked var -(col+1))
  std::vector<long long> row_ptr;
  std::vector<int> col;
  std::vector<double> val;
  std::vector<double> rhs;       // row-major: rhs[r * k + sys]
  std::vector<double> weight;
  bool any_weight = false;
  // current row
  std::vector<int> cur_var;
  std::vector<double> cur_val;
  std::unordered_map<int, int> cur_pos;   // used for long rows
  std::vector<double> cur_rhs;
  double cur_scale = 1.0;
  // IJ interface (square systems built by entries)
  std::vector<std::unordered_map<int, int>> ij_pos;
  std::vector<std::vector<std::pair<int, double>>> ij_rows;
  std::vector<double> ij_rhs;    // [free_row * k + sys]
  bool ij_used = false;
  // results
  long long used_iterations = 0;
  double error = 0.0;
  double true_error = 0.0;
  double elapsed = 0.0;
  double assembly_time = 0.0;
  int status = NL_GB300_STATUS_NONE;
  int refinement_steps = 0;
  double gflops = 0.0;
  // device
  bool assembled = false;
  DeviceCRS A;
  double* d_rhs = nullptr;   // k * n_free
  double* d_x = nullptr;     // n_free
  PcgSolver pcg;
  bool pcg_bound = false;

  ~Context() {
    cudaFree(d_rhs);
    cudaFree(d_x);
    crs_free(A);
  }
  int n_free() const { return (int)free_vars.size(); }
};

Context* g_current = nullptr;

Context* ctx_or_error(const char* fn) {
  if (!g_current) {
    nl_error(NL_INVALID_OPERATION, std::string(fn) + ": no current context");
    return nullptr;
  }
  return g_current;
}

bool check_state(Context* c, State s, const char* fn) {
  if (c->state != s) {
    nl_error(NL_INVALID_OPERATION, std::string(fn) + ": called in the wrong state");
    return false;
  }
  return true;
}

bool check_var(Context* c, NLuint i, const char* fn) {
  if ((long long)i >= c->nb_variables) {
    nl_error(NL_INVALID_VALUE, std::string(fn) + ": variable index out of range");
    return false;
  }
  return true;
}

void invalidate_device(Context* c) {
  c->assembled = false;
}

// Finish the current row: merge duplicates (first-occurrence order), apply
// scaling / normalisation, then append it to the row stream.
void end_row(Context* c) {
  const int k = c->nb_systems;
  const size_t len = c->cur_var.size();
  double w = c->cur_scale;
  if (c->normalize_rows) {
    double s2 = 0.0;
    for (size_t t = 0; t < len; ++t) s2 += c->cur_val[t] * c->cur_val[t];
    if (s2 > 0.0) w = w / s2;
  }
  for (size_t t = 0; t < len; ++t) {
    const int var = c->cur_var[t];
    const int fi = c->free_index[var];
    c->col.push_back(fi >= 0 ? fi : -(var + 1));
    c->val.push_back(c->cur_val[t]);
  }
  c->row_ptr.push_back((long long)c->col.size());
  for (int s = 0; s < k; ++s) c->rhs.push_back(c->cur_rhs[s]);
  c->weight.push_back(w);
  if (w != 1.0) c->any_weight = true;
  c->cur_var.clear();
  c->cur_val.clear();
  c->cur_pos.clear();
  std::fill(c->cur_rhs.begin(), c->cur_rhs.end(), 0.0);
  c->cur_scale = 1.0;
}

void add_coef(Context* c, int var, double a) {
  const size_t len = c->cur_var.size();
  if (len < 32) {
    for (size_t t = 0; t < len; ++t)
      if (c->cur_var[t] == var) { c->cur_val[t] += a; return; }
    if (len == 31) {   // switch to the hash index for long rows
      for (size_t t = 0; t < len; ++t) c->cur_pos[c->cur_var[t]] = (int)t;
      c->cur_pos[var] = (int)len;
    }
  } else {
    auto it = c->cur_pos.find(var);
    if (it != c->cur_pos.end()) { c->cur_val[it->second] += a; return; }
    c->cur_pos[var] = (int)len;
  }
  c->cur_var.push_back(var);
  c->cur_val.push_back(a);
}

// IJ entries become rows of the square system (one per free variable).
void ij_to_rows(Context* c) {
  const int nf = c->n_free();
  const int k = c->nb_systems;
  c->row_ptr.assign(1, 0);
  c->col.clear(); c->val.clear(); c->rhs.clear(); c->weight.clear();
  for (int r = 0; r < nf; ++r) {
    for (auto& e : c->ij_rows[r]) {
      const int var = e.first;
      const int fi = c->free_index[var];
      c->col.push_back(fi >= 0 ? fi : -(var + 1));
      c->val.push_back(e.second);
    }
    c->row_ptr.push_back((long long)c->col.size());
    for (int s = 0; s < k; ++s) c->rhs.push_back(c->ij_rhs[(size_t)r * k + s]);
    c->weight.push_back(1.0);
  }
}

// Upload the row stream and assemble the system on the GPU.
// NL_GB300_PRECISION_AUTO: FP64 for least-squares (normal-equation) systems,
// mixed for square ones.
int effective_precision(const Context* c) {
  if (c->precision != NL_GB300_PRECISION_AUTO) return c->precision;
  return c->least_squares ? NL_GB300_PRECISION_DOUBLE : NL_GB300_PRECISION_MIXED;
}

bool assemble(Context* c) {
  std::string why;
  if (!device_ready(&why)) { nl_error(NL_DEVICE_ERROR, "nlSolve: " + why); return false; }
  cudaStream_t s = api_stream();
  const auto t0 = std::chrono::steady_clock::now();
  const int k = c->nb_systems;
  const long long n_rows = (long long)c->row_ptr.size() - 1;
  const long long n_coefs = (long long)c->col.size();
  const int nf = c->n_free();
  // rhs stored row-major on the host; the device wants [sys][row].
  std::vector<double> rhs_t((size_t)k * std::max(1LL, n_rows));
  for (long long r = 0; r < n_rows; ++r)
    for (int sys = 0; sys < k; ++sys) rhs_t[(size_t)sys * n_rows + r] = c->rhs[(size_t)r * k + sys];
  long long* d_rp = nullptr; int* d_col = nullptr; double *d_val = nullptr, *d_rhs_rows = nullptr,
            *d_w = nullptr, *d_xl = nullptr;
  auto cleanup = [&]() {
    cudaFree(d_rp); cudaFree(d_col); cudaFree(d_val); cudaFree(d_rhs_rows); cudaFree(d_w); cudaFree(d_xl);
  };
  auto fail = [&](const char* what) {
    nl_error(NL_DEVICE_ERROR, std::string("nlSolve: ") + what + ": " + last_error());
    cleanup();
    return false;
  };
  if (cudaMalloc(&d_rp, sizeof(long long) * (n_rows + 1)) != cudaSuccess ||
      cudaMalloc(&d_col, sizeof(int) * std::max(1LL, n_coefs)) != cudaSuccess ||
      cudaMalloc(&d_val, sizeof(double) * std::max(1LL, n_coefs)) != cudaSuccess ||
      cudaMalloc(&d_rhs_rows, sizeof(double) * rhs_t.size()) != cudaSuccess ||
      cudaMalloc(&d_xl, sizeof(double) * std::max<size_t>(1, c->values.size())) != cudaSuccess ||
      (c->any_weight && cudaMalloc(&d_w, sizeof(double) * std::max(1LL, n_rows)) != cudaSuccess)) {
    set_error(cudaGetErrorString(cudaGetLastError()));
    return fail("device allocation");
  }
  cudaMemcpyAsync(d_rp, c->row_ptr.data(), sizeof(long long) * (n_rows + 1), cudaMemcpyHostToDevice, s);
  if (n_coefs) {
    cudaMemcpyAsync(d_col, c->col.data(), sizeof(int) * n_coefs, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_val, c->val.data(), sizeof(double) * n_coefs, cudaMemcpyHostToDevice, s);
  }
  cudaMemcpyAsync(d_rhs_rows, rhs_t.data(), sizeof(double) * rhs_t.size(), cudaMemcpyHostToDevice, s);
  if (!c->values.empty())
    cudaMemcpyAsync(d_xl, c->values.data(), sizeof(double) * c->values.size(), cudaMemcpyHostToDevice, s);
  if (d_w) cudaMemcpyAsync(d_w, c->weight.data(), sizeof(double) * n_rows, cudaMemcpyHostToDevice, s);
  LSRowsDevice R;
  R.n_rows = n_rows; R.n_coefs = n_coefs; R.n_free = nf; R.n_vars = (int)c->nb_variables;
  R.n_systems = k; R.row_ptr = d_rp; R.col = d_col; R.val = d_val; R.rhs = d_rhs_rows;
  R.weight = d_w; R.xl = d_xl;
  cudaFree(c->d_rhs); c->d_rhs = nullptr;
  cudaFree(c->d_x); c->d_x = nullptr;
  if (cudaMalloc(&c->d_rhs, sizeof(double) * (size_t)k * std::max(1, nf)) != cudaSuccess ||
      cudaMalloc(&c->d_x, sizeof(double) * (size_t)std::max(1, nf)) != cudaSuccess) {
    set_error(cudaGetErrorString(cudaGetLastError()));
    return fail("device allocation");
  }
  cudaError_t e = c->least_squares ? assemble_normal_equations(R, c->A, c->d_rhs, s)
                                   : assemble_square(R, c->A, c->d_rhs, s);
  if (e != cudaSuccess) return fail("assembly");
  if (c->tpr_override > 0) { c->A.tpr = c->tpr_override; }
  e = crs_prepare(c->A, effective_precision(c) == NL_GB300_PRECISION_MIXED, s);
  if (c->tpr_override > 0) c->A.tpr = c->tpr_override;
  if (e != cudaSuccess) return fail("matrix preparation");
  if (cudaStreamSynchronize(s) != cudaSuccess) { set_error(cudaGetErrorString(cudaGetLastError())); return fail("assembly"); }
  cleanup();
  c->pcg_bound = false;
  c->assembled = true;
  c->assembly_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return true;
}

}  // namespace

extern "C" {

NLContext nlNewContext(void) {
  Context* c = new Context();
  g_current = c;
  return c;
}

void nlDeleteContext(NLContext context) {
  Context* c = (Context*)context;
  if (!c) return;
  if (g_current == c) g_current = nullptr;
  delete c;
}

void nlMakeCurrent(NLContext context) { g_current = (Context*)context; }
NLContext nlGetCurrent(void) { return g_current; }

NLboolean nlInitExtension(const char* extension) {
  if (!extension) return NL_FALSE;
  const std::string e(extension);
  if (e == "GB300" || e == "CUDA") return device_ready(nullptr) ? NL_TRUE : NL_FALSE;
  return NL_FALSE;   // SUPERLU, CHOLMOD, ARPACK, MKL, ...: not provided
}

NLboolean nlExtensionIsInitialized(const char* extension) { return nlInitExtension(extension); }

void nlSolverParameterd(NLenum pname, NLdouble param) {
  Context* c = ctx_or_error("nlSolverParameterd");
  if (!c) return;
  switch (pname) {
    case NL_THRESHOLD:
      if (!(param >= 0.0)) { nl_error(NL_INVALID_VALUE, "NL_THRESHOLD must be >= 0"); return; }
      c->threshold = param; break;
    case NL_OMEGA: c->omega = param; break;
    case NL_GB300_INNER_THRESHOLD:
      if (!(param > 0.0 && param < 1.0)) { nl_error(NL_INVALID_VALUE, "inner threshold must be in (0,1)"); return; }
      c->inner_threshold = param; break;
    default: nlSolverParameteri(pname, (NLint)param); break;
  }
}

void nlSolverParameteri(NLenum pname, NLint param) {
  Context* c = ctx_or_error("nlSolverParameteri");
  if (!c) return;
  switch (pname) {
    case NL_SOLVER:
      if (param != (NLint)NL_CG && param != (NLint)NL_SOLVER_DEFAULT && param != (NLint)NL_BICGSTAB &&
          param != (NLint)NL_GMRES) { nl_error(NL_INVALID_ENUM, "unknown NL_SOLVER"); return; }
      c->solver = (NLenum)param; break;
    case NL_NB_VARIABLES:
      if (!check_state(c, S_INITIAL, "nlSolverParameteri(NL_NB_VARIABLES)")) return;
      if (param < 0) { nl_error(NL_INVALID_VALUE, "NL_NB_VARIABLES must be >= 0"); return; }
      c->nb_variables = param; break;
    case NL_NB_SYSTEMS:
      if (!check_state(c, S_INITIAL, "nlSolverParameteri(NL_NB_SYSTEMS)")) return;
      if (param < 1 || param > 64) { nl_error(NL_INVALID_VALUE, "NL_NB_SYSTEMS must be in 1..64"); return; }
      c->nb_systems = param; break;
    case NL_LEAST_SQUARES: c->least_squares = param != 0; break;
    case NL_MAX_ITERATIONS:
      if (param < 0) { nl_error(NL_INVALID_VALUE, "NL_MAX_ITERATIONS must be >= 0"); return; }
      c->max_iterations = param; break;
    case NL_SYMMETRIC: c->symmetric = param != 0; break;
    case NL_INNER_ITERATIONS:          // restart length of GMRES
      if (param < 1) { nl_error(NL_INVALID_VALUE, "NL_INNER_ITERATIONS must be >= 1"); return; }
      c->inner_iterations = param;
      break;
    case NL_PRECONDITIONER:
      if (param != (NLint)NL_PRECOND_JACOBI && param != (NLint)NL_PRECOND_NONE &&
          param != (NLint)NL_PRECOND_SSOR) { nl_error(NL_INVALID_ENUM, "unknown NL_PRECONDITIONER"); return; }
      c->precond = (NLenum)param; invalidate_device(c); break;
    case NL_GB300_PRECISION:
      if (param != NL_GB300_PRECISION_DOUBLE && param != NL_GB300_PRECISION_MIXED &&
          param != NL_GB300_PRECISION_AUTO && param != NL_GB300_PRECISION_DOUBLE_FLOAT) {
        nl_error(NL_INVALID_ENUM, "unknown NL_GB300_PRECISION"); return;
      }
      c->precision = param; invalidate_device(c); break;
    case NL_GB300_THREADS_PER_ROW:
      if (param != 0 && param != 1 && param != 2 && param != 4 && param != 8 && param != 16 && param != 32) {
        nl_error(NL_INVALID_VALUE, "NL_GB300_THREADS_PER_ROW must be 0 or a power of two <= 32"); return;
      }
      c->tpr_override = param; invalidate_device(c); break;
    case NL_GB300_MAX_REFINEMENT:
      if (param < 1) { nl_error(NL_INVALID_VALUE, "NL_GB300_MAX_REFINEMENT must be >= 1"); return; }
      c->max_refinement = param; break;
    case NL_THRESHOLD: nlSolverParameterd(pname, (double)param); break;
    default: nl_error(NL_INVALID_ENUM, "nlSolverParameteri: unknown parameter"); break;
  }
}

void nlGetIntegerv(NLenum pname, NLint* params) {
  Context* c = ctx_or_error("nlGetIntegerv");
  if (!c || !params) return;
  switch (pname) {
    case NL_SOLVER: *params = (NLint)c->solver; break;
    case NL_INNER_ITERATIONS: *params = (NLint)c->inner_iterations; break;
    case NL_NB_VARIABLES: *params = (NLint)c->nb_variables; break;
    case NL_NB_SYSTEMS: *params = c->nb_systems; break;
    case NL_LEAST_SQUARES: *params = c->least_squares; break;
    case NL_MAX_ITERATIONS: *params = (NLint)(c->max_iterations >= 0 ? c->max_iterations : 5LL * c->n_free()); break;
    case NL_SYMMETRIC: *params = c->symmetric; break;
    case NL_USED_ITERATIONS: *params = (NLint)c->used_iterations; break;
    case NL_PRECONDITIONER: *params = (NLint)c->precond; break;
    case NL_NNZ: *params = (NLint)c->A.nnz; break;
    case NL_GB300_PRECISION: *params = c->precision; break;
    case NL_GB300_REFINEMENT_STEPS: *params = c->refinement_steps; break;
    case NL_GB300_STATUS: *params = c->status; break;
    case NL_GB300_THREADS_PER_ROW: *params = c->A.tpr; break;
    case NL_GB300_MAX_REFINEMENT: *params = c->max_refinement; break;
    default: nl_error(NL_INVALID_ENUM, "nlGetIntegerv: unknown parameter"); break;
  }
}

void nlGetDoublev(NLenum pname, NLdouble* params) {
  Context* c = ctx_or_error("nlGetDoublev");
  if (!c || !params) return;
  switch (pname) {
    case NL_THRESHOLD: *params = c->threshold; break;
    case NL_ERROR: *params = c->error; break;
    case NL_ELAPSED_TIME: *params = c->elapsed; break;
    case NL_GFLOPS: *params = c->gflops; break;
    case NL_OMEGA: *params = c->omega; break;
    case NL_GB300_INNER_THRESHOLD: *params = c->inner_threshold; break;
    case NL_GB300_TRUE_RESIDUAL: *params = c->true_error; break;
    case NL_GB300_ASSEMBLY_TIME: *params = c->assembly_time; break;
    default: {
      NLint v = 0;
      nlGetIntegerv(pname, &v);
      *params = v;
    } break;
  }
}

void nlGetBooleanv(NLenum pname, NLboolean* params) {
  if (!params) return;
  NLint v = 0;
  if (pname == NL_VERBOSE || pname == NL_NORMALIZE_ROWS || pname == NL_NO_VARIABLES_INDIRECTION) {
    *params = nlIsEnabled(pname);
    return;
  }
  nlGetIntegerv(pname, &v);
  *params = v ? NL_TRUE : NL_FALSE;
}

void nlEnable(NLenum pname) {
  Context* c = ctx_or_error("nlEnable");
  if (!c) return;
  switch (pname) {
    case NL_VERBOSE: c->verbose = true; break;
    case NL_NORMALIZE_ROWS: c->normalize_rows = true; break;
    case NL_NO_VARIABLES_INDIRECTION:
      nl_error(NL_INVALID_ENUM, "NL_NO_VARIABLES_INDIRECTION is not supported"); break;
    default: nl_error(NL_INVALID_ENUM, "nlEnable: unknown flag"); break;
  }
}

void nlDisable(NLenum pname) {
  Context* c = ctx_or_error("nlDisable");
  if (!c) return;
  switch (pname) {
    case NL_VERBOSE: c->verbose = false; break;
    case NL_NORMALIZE_ROWS: c->normalize_rows = false; break;
    case NL_NO_VARIABLES_INDIRECTION: break;
    default: nl_error(NL_INVALID_ENUM, "nlDisable: unknown flag"); break;
  }
}

NLboolean nlIsEnabled(NLenum pname) {
  Context* c = ctx_or_error("nlIsEnabled");
  if (!c) return NL_FALSE;
  switch (pname) {
    case NL_VERBOSE: return c->verbose;
    case NL_NORMALIZE_ROWS: return c->normalize_rows;
    default: return NL_FALSE;
  }
}

NLenum nlGetError(void) {
  const NLenum e = g_error_code;
  g_error_code = NL_NO_ERROR;
  return e;
}

const char* nlGetErrorString(void) { return last_error(); }

void nlSetVariable(NLuint i, NLdouble value) { nlMultiSetVariable(i, 0, value); }

void nlMultiSetVariable(NLuint i, NLuint k, NLdouble value) {
  Context* c = ctx_or_error("nlSetVariable");
  if (!c) return;
  if (c->state == S_INITIAL) { nl_error(NL_INVALID_OPERATION, "nlSetVariable: call nlBegin(NL_SYSTEM) first"); return; }
  if (!check_var(c, i, "nlSetVariable")) return;
  if ((int)k >= c->nb_systems) { nl_error(NL_INVALID_VALUE, "nlMultiSetVariable: system index out of range"); return; }
  c->values[(size_t)k * c->nb_variables + i] = value;
}

NLdouble nlGetVariable(NLuint i) { return nlMultiGetVariable(i, 0); }

NLdouble nlMultiGetVariable(NLuint i, NLuint k) {
  Context* c = ctx_or_error("nlGetVariable");
  if (!c) return 0.0;
  if (c->state == S_INITIAL) { nl_error(NL_INVALID_OPERATION, "nlGetVariable: no system"); return 0.0; }
  if (!check_var(c, i, "nlGetVariable")) return 0.0;
  if ((int)k >= c->nb_systems) { nl_error(NL_INVALID_VALUE, "nlMultiGetVariable: system index out of range"); return 0.0; }
  return c->values[(size_t)k * c->nb_variables + i];
}

void nlLockVariable(NLuint i) {
  Context* c = ctx_or_error("nlLockVariable");
  if (!c) return;
  if (!check_state(c, S_SYSTEM, "nlLockVariable")) return;
  if (!check_var(c, i, "nlLockVariable")) return;
  c->locked[i] = 1;
}

void nlUnlockVariable(NLuint i) {
  Context* c = ctx_or_error("nlUnlockVariable");
  if (!c) return;
  if (!check_state(c, S_SYSTEM, "nlUnlockVariable")) return;
  if (!check_var(c, i, "nlUnlockVariable")) return;
  c->locked[i] = 0;
}

NLboolean nlVariableIsLocked(NLuint i) {
  Context* c = ctx_or_error("nlVariableIsLocked");
  if (!c || c->state == S_INITIAL || !check_var(c, i, "nlVariableIsLocked")) return NL_FALSE;
  return c->locked[i] ? NL_TRUE : NL_FALSE;
}

void nlBegin(NLenum prim) {
  Context* c = ctx_or_error("nlBegin");
  if (!c) return;
  switch (prim) {
    case NL_SYSTEM: {
      if (c->state != S_INITIAL && c->state != S_SOLVED && c->state != S_SYSTEM_CONSTRUCTED) {
        nl_error(NL_INVALID_OPERATION, "nlBegin(NL_SYSTEM): called in the wrong state"); return;
      }
      if (c->nb_variables <= 0) { nl_error(NL_INVALID_VALUE, "nlBegin(NL_SYSTEM): NL_NB_VARIABLES not set"); return; }
      if (c->state == S_INITIAL) {
        c->values.assign((size_t)c->nb_systems * c->nb_variables, 0.0);
        c->locked.assign((size_t)c->nb_variables, 0);
      }
      invalidate_device(c);
      c->state = S_SYSTEM;
    } break;
    case NL_MATRIX: {
      if (!check_state(c, S_SYSTEM, "nlBegin(NL_MATRIX)")) return;
      c->free_index.assign((size_t)c->nb_variables, -1);
      c->free_vars.clear();
      for (long long i = 0; i < c->nb_variables; ++i)
        if (!c->locked[i]) { c->free_index[i] = (int)c->free_vars.size(); c->free_vars.push_back((int)i); }
      c->row_ptr.assign(1, 0);
      c->col.clear(); c->val.clear(); c->rhs.clear(); c->weight.clear();
      c->any_weight = false;
      c->cur_rhs.assign((size_t)c->nb_systems, 0.0);
      c->cur_var.clear(); c->cur_val.clear(); c->cur_pos.clear(); c->cur_scale = 1.0;
      c->ij_used = false;
      c->ij_rows.clear(); c->ij_pos.clear(); c->ij_rhs.clear();
      invalidate_device(c);
      c->state = S_MATRIX;
    } break;
    case NL_ROW: {
      if (!check_state(c, S_MATRIX, "nlBegin(NL_ROW)")) return;
      if (c->ij_used) { nl_error(NL_INVALID_OPERATION, "nlBegin(NL_ROW): cannot mix rows with nlAddIJCoefficient"); return; }
      c->state = S_ROW;
    } break;
    default: nl_error(NL_INVALID_ENUM, "nlBegin: unknown primitive"); break;
  }
}

void nlEnd(NLenum prim) {
  Context* c = ctx_or_error("nlEnd");
  if (!c) return;
  switch (prim) {
    case NL_ROW:
      if (!check_state(c, S_ROW, "nlEnd(NL_ROW)")) return;
      end_row(c);
      c->state = S_MATRIX;
      break;
    case NL_MATRIX:
      if (!check_state(c, S_MATRIX, "nlEnd(NL_MATRIX)")) return;
      if (c->ij_used) ij_to_rows(c);
      if (!c->least_squares) {
        const long long n_rows = (long long)c->row_ptr.size() - 1;
        if (n_rows != c->n_free()) {
          nl_error(NL_INVALID_OPERATION,
                   "nlEnd(NL_MATRIX): a square system needs one row per free variable (got " +
                       std::to_string(n_rows) + " rows for " + std::to_string(c->n_free()) +
                       " free variables)");
          return;
        }
      }
      c->state = S_MATRIX_CONSTRUCTED;
      break;
    case NL_SYSTEM:
      if (!check_state(c, S_MATRIX_CONSTRUCTED, "nlEnd(NL_SYSTEM)")) return;
      c->state = S_SYSTEM_CONSTRUCTED;
      break;
    default: nl_error(NL_INVALID_ENUM, "nlEnd: unknown primitive"); break;
  }
}

void nlCoefficient(NLuint i, NLdouble value) {
  Context* c = ctx_or_error("nlCoefficient");
  if (!c) return;
  if (!check_state(c, S_ROW, "nlCoefficient")) return;
  if (!check_var(c, i, "nlCoefficient")) return;
  add_coef(c, (int)i, value);
}

void nlAddIJCoefficient(NLuint i, NLuint j, NLdouble value) {
  Context* c = ctx_or_error("nlAddIJCoefficient");
  if (!c) return;
  if (!check_state(c, S_MATRIX, "nlAddIJCoefficient")) return;
  if (!check_var(c, i, "nlAddIJCoefficient") || !check_var(c, j, "nlAddIJCoefficient")) return;
  if (c->least_squares) { nl_error(NL_INVALID_OPERATION, "nlAddIJCoefficient: not available in least-squares mode"); return; }
  if ((long long)c->col.size() > 0) { nl_error(NL_INVALID_OPERATION, "nlAddIJCoefficient: cannot mix with rows"); return; }
  const int fi = c->free_index[i];
  if (fi < 0) return;   // the equation of a locked variable is not part of the system
  if (!c->ij_used) {
    c->ij_used = true;
    c->ij_rows.assign((size_t)c->n_free(), {});
    c->ij_pos.assign((size_t)c->n_free(), {});
    c->ij_rhs.assign((size_t)c->n_free() * c->nb_systems, 0.0);
  }
  auto& pos = c->ij_pos[fi];
  auto it = pos.find((int)j);
  if (it != pos.end()) { c->ij_rows[fi][it->second].second += value; return; }
  pos[(int)j] = (int)c->ij_rows[fi].size();
  c->ij_rows[fi].push_back({(int)j, value});
}

void nlAddIRightHandSide(NLuint i, NLdouble value) { nlMultiAddIRightHandSide(i, 0, value); }

void nlMultiAddIRightHandSide(NLuint i, NLuint k, NLdouble value) {
  Context* c = ctx_or_error("nlAddIRightHandSide");
  if (!c) return;
  if (!check_state(c, S_MATRIX, "nlAddIRightHandSide")) return;
  if (!check_var(c, i, "nlAddIRightHandSide")) return;
  if ((int)k >= c->nb_systems) { nl_error(NL_INVALID_VALUE, "nlMultiAddIRightHandSide: system index out of range"); return; }
  if (c->least_squares) { nl_error(NL_INVALID_OPERATION, "nlAddIRightHandSide: not available in least-squares mode"); return; }
  const int fi = c->free_index[i];
  if (fi < 0) return;
  if (!c->ij_used) {
    c->ij_used = true;
    c->ij_rows.assign((size_t)c->n_free(), {});
    c->ij_pos.assign((size_t)c->n_free(), {});
    c->ij_rhs.assign((size_t)c->n_free() * c->nb_systems, 0.0);
  }
  c->ij_rhs[(size_t)fi * c->nb_systems + k] += value;
}

void nlRightHandSide(NLdouble value) { nlMultiRightHandSide(0, value); }

void nlMultiRightHandSide(NLuint k, NLdouble value) {
  Context* c = ctx_or_error("nlRightHandSide");
  if (!c) return;
  if (!check_state(c, S_ROW, "nlRightHandSide")) return;
  if ((int)k >= c->nb_systems) { nl_error(NL_INVALID_VALUE, "nlMultiRightHandSide: system index out of range"); return; }
  c->cur_rhs[k] = value;
}

void nlRowScaling(NLdouble value) {
  Context* c = ctx_or_error("nlRowScaling");
  if (!c) return;
  if (c->state != S_ROW && c->state != S_MATRIX) { nl_error(NL_INVALID_OPERATION, "nlRowScaling: called in the wrong state"); return; }
  c->cur_scale = value;
}

// NL_BICGSTAB / NL_GMRES: general (non-symmetric) square systems, FP64,
// Jacobi, SSOR or no right preconditioning (nlgb_krylov.cu); and NL_CG with
// the SSOR preconditioner (nlgb_ssor.cu).
static NLboolean solve_krylov(Context* c) {
  const int nf = c->n_free();
  const int k = c->nb_systems;
  cudaStream_t s = api_stream();
  double* ones = nullptr;
  const double* dinv = c->A.dinv;
  SsorPrecond ssor;
  const bool use_ssor = c->precond == NL_PRECOND_SSOR;
  if (use_ssor && ssor.build(c->A, c->omega, s) != cudaSuccess) {
    nl_error(NL_DEVICE_ERROR, std::string("nlSolve: SSOR preconditioner: ") + last_error());
    c->status = NL_GB300_STATUS_DEVICE_ERR;
    return NL_FALSE;
  }
  if (c->precond == NL_PRECOND_NONE || use_ssor) {
    std::vector<double> h((size_t)std::max(1, nf), 1.0);
    if (cudaMalloc(&ones, sizeof(double) * h.size()) != cudaSuccess ||
        cudaMemcpy(ones, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaFree(ones);
      nl_error(NL_DEVICE_ERROR, "nlSolve: device allocation failed");
      c->status = NL_GB300_STATUS_DEVICE_ERR;
      return NL_FALSE;
    }
    dinv = ones;
  }
  const int method = c->solver == NL_BICGSTAB ? KRYLOV_BICGSTAB
                   : c->solver == NL_GMRES  ? KRYLOV_GMRES
                                            : 0;   // CG (with SSOR)
  const long long max_iter = c->max_iterations >= 0 ? c->max_iterations : 5LL * nf;
  bool ok = true;
  long long iters = 0;
  double err = 0.0, terr = 0.0;
  int worst = NL_GB300_STATUS_CONVERGED;
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<double> xf((size_t)std::max(1, nf));
  for (int sys = 0; sys < k; ++sys) {
    for (int f = 0; f < nf; ++f) xf[f] = c->values[(size_t)sys * c->nb_variables + c->free_vars[f]];
    KrylovResult kr;
    cudaError_t e = cudaMemcpyAsync(c->d_x, xf.data(), sizeof(double) * nf, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && method == 0)
      e = pcg_ssor(c->A, ssor, c->d_rhs + (size_t)sys * nf, c->d_x, c->threshold, max_iter, s, &kr);
    else if (e == cudaSuccess)
      e = krylov_solve(c->A, dinv, c->d_rhs + (size_t)sys * nf, c->d_x, method, c->threshold, max_iter,
                       c->inner_iterations, s, &kr, use_ssor ? &ssor : nullptr);
    if (e == cudaSuccess) e = cudaMemcpyAsync(xf.data(), c->d_x, sizeof(double) * nf, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      cudaFree(ones);
      nl_error(NL_DEVICE_ERROR, std::string("nlSolve: ") + cudaGetErrorString(e));
      c->status = NL_GB300_STATUS_DEVICE_ERR;
      return NL_FALSE;
    }
    for (int f = 0; f < nf; ++f) c->values[(size_t)sys * c->nb_variables + c->free_vars[f]] = xf[f];
    iters += kr.iterations;
    err = std::max(err, kr.rel_residual);
    terr = std::max(terr, kr.true_rel_residual);
    if (kr.status != NL_GB300_STATUS_CONVERGED) {
      worst = kr.status;
      if (kr.status != NL_GB300_STATUS_TRUE_RESIDUAL_STALLED) ok = false;
    }
  }
  cudaFree(ones);
  c->used_iterations = iters;
  c->error = err;
  c->true_error = terr;
  c->elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  c->refinement_steps = 0;
  c->status = worst;
  c->gflops = 0.0;
  c->state = S_SOLVED;
  return ok ? NL_TRUE : NL_FALSE;
}

NLboolean nlSolve(void) {
  Context* c = ctx_or_error("nlSolve");
  if (!c) return NL_FALSE;
  if (c->state != S_SYSTEM_CONSTRUCTED && c->state != S_SOLVED) {
    nl_error(NL_INVALID_OPERATION, "nlSolve: the system is not constructed (nlEnd(NL_SYSTEM) missing)");
    return NL_FALSE;
  }
  c->status = NL_GB300_STATUS_NONE;
  if (!c->assembled && !assemble(c)) { c->status = NL_GB300_STATUS_DEVICE_ERR; return NL_FALSE; }
  const int nf = c->n_free();
  const int k = c->nb_systems;
  cudaStream_t s = api_stream();
  if (c->solver == NL_BICGSTAB || c->solver == NL_GMRES || c->precond == NL_PRECOND_SSOR)
    return solve_krylov(c);
  if (!c->pcg_bound) {
    if (c->precond == NL_PRECOND_NONE) {
      // Identity preconditioner: CG on the same matrix with D^-1 = 1.
      std::vector<double> ones((size_t)std::max(1, nf), 1.0);
      std::vector<float> ones32((size_t)std::max(1, nf), 1.0f);
      cudaMemcpy(c->A.dinv, ones.data(), sizeof(double) * ones.size(), cudaMemcpyHostToDevice);
      cudaMemcpy(c->A.dinv32, ones32.data(), sizeof(float) * ones32.size(), cudaMemcpyHostToDevice);
    }
    if (c->pcg.bind(&c->A, s) != cudaSuccess) {
      nl_error(NL_DEVICE_ERROR, std::string("nlSolve: ") + last_error());
      c->status = NL_GB300_STATUS_DEVICE_ERR;
      return NL_FALSE;
    }
    c->pcg_bound = true;
  }
  SolveParams prm;
  prm.eps = c->threshold;
  prm.max_iter = c->max_iterations >= 0 ? c->max_iterations : 5LL * nf;
  prm.precision = effective_precision(c);
  prm.inner_eps = c->inner_threshold;
  prm.max_outer = c->max_refinement;
  bool ok = true;
  long long iters = 0;
  double err = 0.0, terr = 0.0, secs = 0.0;
  int worst = NL_GB300_STATUS_CONVERGED, outer = 0;
  std::vector<double> xf((size_t)std::max(1, nf));
  for (int sys = 0; sys < k; ++sys) {
    for (int f = 0; f < nf; ++f) xf[f] = c->values[(size_t)sys * c->nb_variables + c->free_vars[f]];
    SolveResult res;
    cudaError_t e = cudaMemcpyAsync(c->d_x, xf.data(), sizeof(double) * nf, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = c->pcg.solve(c->d_rhs + (size_t)sys * nf, c->d_x, prm, &res);
    if (e == cudaSuccess) e = cudaMemcpyAsync(xf.data(), c->d_x, sizeof(double) * nf, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      nl_error(NL_DEVICE_ERROR, std::string("nlSolve: ") + last_error());
      c->status = NL_GB300_STATUS_DEVICE_ERR;
      return NL_FALSE;
    }
    for (int f = 0; f < nf; ++f) c->values[(size_t)sys * c->nb_variables + c->free_vars[f]] = xf[f];
    iters += res.iterations;
    err = std::max(err, res.rel_residual);
    terr = std::max(terr, res.true_rel_residual);
    secs += res.seconds;
    outer += res.outer_steps;
    // A stalled true residual still met OpenNL's own stopping rule (the
    // recursive residual): nlSolve succeeds, NL_GB300_STATUS says which.
    if (res.status != NL_GB300_STATUS_CONVERGED) {
      worst = res.status;
      if (res.status != NL_GB300_STATUS_TRUE_RESIDUAL_STALLED) ok = false;
    }
  }
  c->used_iterations = iters;
  c->error = err;
  c->true_error = terr;
  c->elapsed = secs;
  c->refinement_steps = outer;
  c->status = worst;
  const double flops = double(iters) * (2.0 * double(c->A.nnz) + 12.0 * nf);
  c->gflops = secs > 0 ? flops / secs * 1e-9 : 0.0;
  if (c->verbose && !quiet())
    std::fprintf(stderr, "OpenNL(gb300): n=%d nnz=%lld iterations=%lld rel.residual=%.3e (true %.3e) time=%.4fs status=%d\n",
                 nf, c->A.nnz, iters, err, terr, secs, worst);
  c->state = S_SOLVED;
  return ok ? NL_TRUE : NL_FALSE;
}

}  // extern "C"

// ---- bulk entry points of nl_gb300.h that act on the current context ----
#include "../../include/nl_gb300.h"

extern "C" {

int nlgb_add_rows(long long n_rows, const long long* row_ptr, const int* var, const double* val,
                  const double* rhs, const double* weight) {
  Context* c = ctx_or_error("nlgb_add_rows");
  if (!c) return NLGB_E_STATE;
  if (!check_state(c, S_MATRIX, "nlgb_add_rows")) return NLGB_E_STATE;
  if (c->ij_used) { nl_error(NL_INVALID_OPERATION, "nlgb_add_rows: cannot mix with nlAddIJCoefficient"); return NLGB_E_STATE; }
  if (n_rows < 0 || !row_ptr) { nl_error(NL_INVALID_VALUE, "nlgb_add_rows: bad arguments"); return NLGB_E_INVALID; }
  const long long total = row_ptr[n_rows];
  for (long long k = 0; k < total; ++k)
    if (var[k] < 0 || (long long)var[k] >= c->nb_variables) {
      nl_error(NL_INVALID_VALUE, "nlgb_add_rows: variable index out of range");
      return NLGB_E_INVALID;
    }
  const int ks = c->nb_systems;
  c->row_ptr.reserve(c->row_ptr.size() + n_rows);
  c->col.reserve(c->col.size() + total);
  c->val.reserve(c->val.size() + total);
  for (long long r = 0; r < n_rows; ++r) {
    for (long long k = row_ptr[r]; k < row_ptr[r + 1]; ++k) add_coef(c, var[k], val[k]);
    if (rhs)
      for (int s = 0; s < ks; ++s) c->cur_rhs[s] = rhs[r * ks + s];
    c->cur_scale = weight ? weight[r] : 1.0;
    end_row(c);
  }
  return NLGB_OK;
}

int nlgb_set_variables(const double* values, const unsigned char* locked) {
  Context* c = ctx_or_error("nlgb_set_variables");
  if (!c) return NLGB_E_STATE;
  if (c->state == S_INITIAL) { nl_error(NL_INVALID_OPERATION, "nlgb_set_variables: call nlBegin(NL_SYSTEM) first"); return NLGB_E_STATE; }
  if (locked && c->state != S_SYSTEM) { nl_error(NL_INVALID_OPERATION, "nlgb_set_variables: locking needs the NL_SYSTEM state"); return NLGB_E_STATE; }
  if (values) std::memcpy(c->values.data(), values, sizeof(double) * c->values.size());
  if (locked) std::memcpy(c->locked.data(), locked, c->locked.size());
  return NLGB_OK;
}

int nlgb_get_variables(double* values) {
  Context* c = ctx_or_error("nlgb_get_variables");
  if (!c) return NLGB_E_STATE;
  if (c->state == S_INITIAL) { nl_error(NL_INVALID_OPERATION, "nlgb_get_variables: no system"); return NLGB_E_STATE; }
  std::memcpy(values, c->values.data(), sizeof(double) * c->values.size());
  return NLGB_OK;
}

}  // extern "C"
