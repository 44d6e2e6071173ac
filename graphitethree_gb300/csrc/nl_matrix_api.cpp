// nl_matrix_api.cpp -- OpenNL's matrix-level API and BLAS table on the GPU.
//
// Mirrors what OGF::NL::Matrix / OGF::NL::Blas call (src/lib/OGF/scene_graph/
// NL/matrix.cpp:121-440, blas.cpp:66-144): dynamic sparse matrices filled by
// nlSparseMatrixAdd, compressed to CRS by nlMatrixCompress, multiplied by
// nlMultMatrixVector and solved by nlSolveSystemIterative(nlHostBlas(), M, P,
// b, x, NL_CG, eps, max_iter, inner_iter).  Every product and solve runs on
// the GPU; host vectors are staged through device buffers.  Preconditioners:
// Jacobi and SSOR (level-scheduled sweeps, nlgb_ssor.cu).  Direct solvers
// (nlMatrixFactorize) are not built and report NULL, which the reference
// wrapper already handles ("Could not factorize matrix", matrix.cpp:331).
#include "../../include/nl.h"
#include "nlgb_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <unordered_map>
#include <vector>

using namespace nlgb;

namespace {

enum Kind { K_DYNAMIC = 1, K_CRS = 2, K_JACOBI = 3, K_SSOR = 4 };

// Standard-layout objects: the public NLMatrixStruct header comes first so
// an NLMatrix handle points at it (matrix.cpp reads m, n and type directly).
struct LibMatrix {
  NLMatrixStruct pub;
  int kind;
  // dynamic: per-row (column -> slot) index and entries in insertion order
  std::vector<std::vector<std::pair<int, double>>>* rows;
  std::vector<std::unordered_map<int, int>>* index;
  // CRS (host copy) -- also the compressed form of a dynamic matrix
  std::vector<int>* rp;
  std::vector<int>* ci;
  std::vector<double>* va;
  // device copy (built on first use, dropped when the host side changes)
  DeviceCRS* dev;
  bool dev_valid;
  // Jacobi: inverse diagonal on the device
  double* dinv;
  double* ones;     // identity-preconditioner diagonal, built on demand
  float* ones32;
  // SSOR: the sweeps' data, built on the device copy of the matrix it was
  // created from (which must outlive it)
  SsorPrecond* ssor;
  DeviceCRS* ssor_base;
};

void destroy_matrix(NLMatrix M);
void mult_matrix(NLMatrix M, const double* x, double* y);

LibMatrix* new_matrix(NLuint m, NLuint n, int kind, NLenum type) {
  LibMatrix* L = new LibMatrix();
  std::memset(&L->pub, 0, sizeof(L->pub));
  L->pub.m = m;
  L->pub.n = n;
  L->pub.type = type;
  L->pub.destroy_func = destroy_matrix;
  L->pub.mult_func = mult_matrix;
  L->kind = kind;
  L->rows = nullptr; L->index = nullptr;
  L->rp = nullptr; L->ci = nullptr; L->va = nullptr;
  L->dev = nullptr; L->dev_valid = false;
  L->dinv = nullptr; L->ones = nullptr; L->ones32 = nullptr;
  L->ssor = nullptr; L->ssor_base = nullptr;
  return L;
}

void destroy_matrix(NLMatrix M) {
  LibMatrix* L = (LibMatrix*)M;
  if (!L) return;
  delete L->rows; delete L->index;
  delete L->rp; delete L->ci; delete L->va;
  if (L->dev) { crs_free(*L->dev); delete L->dev; }
  cudaFree(L->dinv); cudaFree(L->ones); cudaFree(L->ones32);
  delete L->ssor;
  delete L;
}

void report(const char* msg) {
  set_error(msg);
  const char* q = std::getenv("NLGB_QUIET");
  if (!(q && q[0] == '1')) std::fprintf(stderr, "OpenNL(gb300) error: %s\n", msg);
}

// Host CRS view of a dynamic or CRS matrix (dynamic rows are packed in
// insertion order).
void host_crs(LibMatrix* L, std::vector<int>& rp, std::vector<int>& ci, std::vector<double>& va) {
  if (L->kind == K_CRS) { rp = *L->rp; ci = *L->ci; va = *L->va; return; }
  rp.assign(L->pub.m + 1, 0);
  ci.clear(); va.clear();
  for (NLuint i = 0; i < L->pub.m; ++i) {
    for (auto& e : (*L->rows)[i]) { ci.push_back(e.first); va.push_back(e.second); }
    rp[i + 1] = (int)ci.size();
  }
}

// Make sure the matrix has a current device copy (Jacobi + tuning included).
bool ensure_device(LibMatrix* L, bool fp32) {
  if (L->kind != K_DYNAMIC && L->kind != K_CRS) { report("matrix has no CRS form"); return false; }
  cudaStream_t s = api_stream();
  if (!L->dev) L->dev = new DeviceCRS();
  if (!L->dev_valid) {
    std::vector<int> rp, ci;
    std::vector<double> va;
    host_crs(L, rp, ci, va);
    if (crs_upload(*L->dev, (int)L->pub.m, (int)L->pub.n, rp.data(), ci.data(), va.data(), s) != cudaSuccess)
      return false;
    L->dev_valid = true;
  }
  if (crs_prepare(*L->dev, fp32, s) != cudaSuccess) return false;
  return true;
}

// Stage a possibly-host vector on the device.
struct Staged {
  double* d = nullptr;
  bool owned = false;
  ~Staged() { if (owned) cudaFree(d); }
  bool in(const double* p, size_t n, cudaStream_t s) {
    if (is_device_pointer(p)) { d = const_cast<double*>(p); return true; }
    if (cudaMalloc(&d, std::max<size_t>(1, n) * sizeof(double)) != cudaSuccess) return false;
    owned = true;
    return n == 0 || cudaMemcpyAsync(d, p, n * sizeof(double), cudaMemcpyHostToDevice, s) == cudaSuccess;
  }
  bool out(double* p, size_t n, cudaStream_t s) {
    if (!owned || n == 0) return true;
    return cudaMemcpyAsync(p, d, n * sizeof(double), cudaMemcpyDeviceToHost, s) == cudaSuccess;
  }
};

void mult_matrix(NLMatrix M, const double* x, double* y) { nlMultMatrixVector(M, x, y); }

}  // namespace

extern "C" {

NLMatrix nlSparseMatrixNew(NLuint m, NLuint n, NLenum storage) {
  if (!(storage & NL_MATRIX_STORE_ROWS)) {
    report("nlSparseMatrixNew: only NL_MATRIX_STORE_ROWS storage is built");
    return nullptr;
  }
  LibMatrix* L = new_matrix(m, n, K_DYNAMIC, NL_MATRIX_SPARSE_DYNAMIC);
  L->rows = new std::vector<std::vector<std::pair<int, double>>>(m);
  L->index = new std::vector<std::unordered_map<int, int>>(m);
  return (NLMatrix)L;
}

void nlSparseMatrixAdd(NLMatrix M, NLuint i, NLuint j, NLdouble value) {
  LibMatrix* L = (LibMatrix*)M;
  if (!L || L->kind != K_DYNAMIC) { report("nlSparseMatrixAdd: not a dynamic sparse matrix"); return; }
  if (i >= L->pub.m || j >= L->pub.n) { report("nlSparseMatrixAdd: index out of bounds"); return; }
  auto& row = (*L->rows)[i];
  if (row.size() < 16) {
    for (auto& e : row) if (e.first == (int)j) { e.second += value; L->dev_valid = false; return; }
    row.push_back({(int)j, value});
    if (row.size() == 16) {
      auto& idx = (*L->index)[i];
      for (size_t t = 0; t < row.size(); ++t) idx[row[t].first] = (int)t;
    }
  } else {
    auto& idx = (*L->index)[i];
    auto it = idx.find((int)j);
    if (it != idx.end()) { row[it->second].second += value; L->dev_valid = false; return; }
    idx[(int)j] = (int)row.size();
    row.push_back({(int)j, value});
  }
  L->dev_valid = false;
}

void nlDeleteMatrix(NLMatrix M) {
  if (M && M->destroy_func) M->destroy_func(M);
}

NLuint nlMatrixNNZ(NLMatrix M) {
  LibMatrix* L = (LibMatrix*)M;
  if (!L) return 0;
  if (L->kind == K_CRS) return (NLuint)L->va->size();
  if (L->kind == K_DYNAMIC) {
    size_t n = 0;
    for (auto& r : *L->rows) n += r.size();
    return (NLuint)n;
  }
  return L->pub.n;
}

void nlMatrixCompress(NLMatrix* M) {
  if (!M || !*M) return;
  LibMatrix* L = (LibMatrix*)*M;
  if (L->kind != K_DYNAMIC) return;
  LibMatrix* C = new_matrix(L->pub.m, L->pub.n, K_CRS, NL_MATRIX_CRS);
  C->rp = new std::vector<int>();
  C->ci = new std::vector<int>();
  C->va = new std::vector<double>();
  host_crs(L, *C->rp, *C->ci, *C->va);
  nlDeleteMatrix(*M);
  *M = (NLMatrix)C;
}

void nlMultMatrixVector(NLMatrix M, const double* x, double* y) {
  LibMatrix* L = (LibMatrix*)M;
  if (!L) { report("nlMultMatrixVector: null matrix"); return; }
  cudaStream_t s = api_stream();
  if (L->kind == K_SSOR) {
    // the preconditioner as a matrix: y = M^-1 x
    Staged sx, sy;
    if (!sx.in(x, L->pub.n, s) || !sy.in(y, L->pub.n, s)) { report("nlMultMatrixVector: staging failed"); return; }
    if (L->ssor->apply(sx.d, sy.d, s) != cudaSuccess) report(last_error());
    sy.out(y, L->pub.n, s);
    cudaStreamSynchronize(s);
    return;
  }
  if (L->kind == K_JACOBI) {
    Staged sx, sy;
    if (!sx.in(x, L->pub.n, s) || !sy.in(y, L->pub.n, s)) { report("nlMultMatrixVector: staging failed"); return; }
    cudaMemcpyAsync(sy.d, sx.d, sizeof(double) * L->pub.n, cudaMemcpyDeviceToDevice, s);
    dev_mul(L->pub.n, L->dinv, sy.d, s);
    sy.out(y, L->pub.n, s);
    cudaStreamSynchronize(s);
    return;
  }
  if (!ensure_device(L, false)) { report("nlMultMatrixVector: device upload failed"); return; }
  Staged sx;
  if (!sx.in(x, L->pub.n, s)) { report("nlMultMatrixVector: staging failed"); return; }
  double* dy = y;
  const bool own_y = !is_device_pointer(y);
  if (own_y && cudaMalloc(&dy, sizeof(double) * std::max<NLuint>(1, L->pub.m)) != cudaSuccess) {
    report("nlMultMatrixVector: allocation failed");
    return;
  }
  if (spmv64(*L->dev, sx.d, dy, s) != cudaSuccess) report(last_error());
  else if (own_y && L->pub.m > 0) cudaMemcpyAsync(y, dy, sizeof(double) * L->pub.m, cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  if (own_y) cudaFree(dy);
}

NLMatrix nlNewJacobiPreconditioner(NLMatrix M) {
  LibMatrix* L = (LibMatrix*)M;
  if (!L || (L->kind != K_DYNAMIC && L->kind != K_CRS) || L->pub.m != L->pub.n) {
    report("nlNewJacobiPreconditioner: needs a square sparse matrix");
    return nullptr;
  }
  if (!ensure_device(L, false)) return nullptr;
  LibMatrix* P = new_matrix(L->pub.m, L->pub.n, K_JACOBI, NL_MATRIX_OTHER);
  if (cudaMalloc(&P->dinv, sizeof(double) * std::max<NLuint>(1, L->pub.n)) != cudaSuccess) {
    destroy_matrix((NLMatrix)P);
    return nullptr;
  }
  cudaMemcpyAsync(P->dinv, L->dev->dinv, sizeof(double) * L->pub.n, cudaMemcpyDeviceToDevice, api_stream());
  cudaStreamSynchronize(api_stream());
  return (NLMatrix)P;
}

NLMatrix nlNewSSORPreconditioner(NLMatrix M, double omega) {
  LibMatrix* L = (LibMatrix*)M;
  if (!L || (L->kind != K_DYNAMIC && L->kind != K_CRS) || L->pub.m != L->pub.n) {
    report("nlNewSSORPreconditioner: needs a square sparse matrix");
    return nullptr;
  }
  if (!(omega > 0.0 && omega < 2.0)) {
    report("nlNewSSORPreconditioner: omega must be in (0, 2)");
    return nullptr;
  }
  if (!ensure_device(L, false)) return nullptr;
  LibMatrix* P = new_matrix(L->pub.m, L->pub.n, K_SSOR, NL_MATRIX_OTHER);
  P->ssor = new SsorPrecond();
  P->ssor_base = L->dev;
  if (P->ssor->build(*L->dev, omega, api_stream()) != cudaSuccess) {
    report(last_error());
    destroy_matrix((NLMatrix)P);
    return nullptr;
  }
  return (NLMatrix)P;
}

NLMatrix nlMatrixFactorize(NLMatrix, NLenum) {
  report("nlMatrixFactorize: direct solvers (SuperLU/CHOLMOD) are not provided");
  return nullptr;
}

NLuint nlSolveSystemIterative(NLBlas_t, NLMatrix M, NLMatrix P, const double* b, double* x,
                              NLenum solver, double eps, NLuint max_iter, NLuint inner_iter) {
  LibMatrix* L = (LibMatrix*)M;
  if (!L || (L->kind != K_DYNAMIC && L->kind != K_CRS) || L->pub.m != L->pub.n) {
    report("nlSolveSystemIterative: needs a square sparse matrix");
    return 0;
  }
  if (solver != NL_CG && solver != NL_SOLVER_DEFAULT && solver != NL_BICGSTAB && solver != NL_GMRES) {
    report("nlSolveSystemIterative: unknown solver");
    return 0;
  }
  LibMatrix* PL = (LibMatrix*)P;
  if (PL && PL->kind != K_JACOBI && PL->kind != K_SSOR) {
    report("nlSolveSystemIterative: the preconditioner must be Jacobi, SSOR or NULL");
    return 0;
  }
  if (!ensure_device(L, false)) { report(last_error()); return 0; }
  if (PL && PL->kind == K_SSOR && (PL->ssor_base != L->dev || PL->pub.n != L->pub.n)) {
    report("nlSolveSystemIterative: the SSOR preconditioner was built for another matrix");
    return 0;
  }
  cudaStream_t s = api_stream();
  const NLuint n = L->pub.n;
  DeviceCRS view = *L->dev;   // shallow view with the requested preconditioner
  view.owns = false;
  SsorPrecond* ssor = (PL && PL->kind == K_SSOR) ? PL->ssor : nullptr;
  if (PL && !ssor) {
    view.dinv = PL->dinv;
  } else {
    if (!L->ones) {
      std::vector<double> one(std::max<NLuint>(1, n), 1.0);
      std::vector<float> one32(std::max<NLuint>(1, n), 1.0f);
      cudaMalloc(&L->ones, sizeof(double) * one.size());
      cudaMalloc(&L->ones32, sizeof(float) * one32.size());
      cudaMemcpy(L->ones, one.data(), sizeof(double) * one.size(), cudaMemcpyHostToDevice);
      cudaMemcpy(L->ones32, one32.data(), sizeof(float) * one32.size(), cudaMemcpyHostToDevice);
    }
    view.dinv = L->ones;
    view.dinv32 = L->ones32;
  }
  Staged sb, sx;
  if (!sb.in(b, n, s) || !sx.in(x, n, s)) { report("nlSolveSystemIterative: staging failed"); return 0; }
  if (solver == NL_BICGSTAB || solver == NL_GMRES) {
    // general square systems; inner_iter is GMRES's restart length
    KrylovResult kr;
    if (krylov_solve(*L->dev, view.dinv, sb.d, sx.d, solver == NL_BICGSTAB ? KRYLOV_BICGSTAB : KRYLOV_GMRES,
                     eps, max_iter, std::max<NLuint>(1, inner_iter), s, &kr, ssor) != cudaSuccess) {
      report(last_error());
      return 0;
    }
    sx.out(x, n, s);
    cudaStreamSynchronize(s);
    return (NLuint)kr.iterations;
  }
  if (ssor) {
    KrylovResult kr;
    if (pcg_ssor(*L->dev, *ssor, sb.d, sx.d, eps, max_iter, s, &kr) != cudaSuccess) {
      report(last_error());
      return 0;
    }
    sx.out(x, n, s);
    cudaStreamSynchronize(s);
    return (NLuint)kr.iterations;
  }
  PcgSolver pcg;
  SolveParams prm;
  prm.eps = eps;
  prm.max_iter = max_iter;
  SolveResult res;
  if (pcg.bind(&view, s) != cudaSuccess || pcg.solve(sb.d, sx.d, prm, &res) != cudaSuccess) {
    report(last_error());
    return 0;
  }
  sx.out(x, n, s);
  cudaStreamSynchronize(s);
  return (NLuint)res.iterations;
}

// ---- NLBlas table ----
// BLAS increments: element i of a strided n-vector sits at i * inc (inc > 0)
// or (n - 1 - i) * |inc| (inc < 0), so a vector spans 1 + (n - 1) |inc|
// doubles.  Host vectors are staged through device buffers of that span;
// the arithmetic always runs on the GPU.
static bool blas_inc_ok(int incx, int incy) {
  if (incx == 0 || incy == 0) { report("NLBlas: increments must be nonzero"); return false; }
  return true;
}

static size_t span(int n, int inc) { return n <= 0 ? 0 : 1 + (size_t)(n - 1) * (size_t)std::abs(inc); }

static void blas_copy(NLBlas_t, int n, const double* x, int incx, double* y, int incy) {
  if (!blas_inc_ok(incx, incy) || n <= 0) return;
  cudaStream_t s = api_stream();
  Staged sx, sy;
  // y is read too (a strided copy leaves the elements between strides alone)
  if (!sx.in(x, span(n, incx), s) || !sy.in(y, span(n, incy), s)) return;
  dev_copy_s(n, sx.d, incx, sy.d, incy, s);
  sy.out(y, span(n, incy), s);
  cudaStreamSynchronize(s);
}

static void blas_scal(NLBlas_t blas, int n, double a, double* x, int incx) {
  if (!blas_inc_ok(incx, 1) || n <= 0) return;
  cudaStream_t s = api_stream();
  Staged sx;
  if (!sx.in(x, span(n, incx), s)) return;
  dev_scal_s(n, a, sx.d, incx, s);
  sx.out(x, span(n, incx), s);
  cudaStreamSynchronize(s);
  if (blas) blas->flops += n;
}

static double blas_dot(NLBlas_t blas, int n, const double* x, int incx, const double* y, int incy) {
  if (!blas_inc_ok(incx, incy) || n <= 0) return 0.0;
  cudaStream_t s = api_stream();
  Staged sx, sy;
  if (!sx.in(x, span(n, incx), s) || !sy.in(y, span(n, incy), s)) return 0.0;
  double r = 0.0;
  dev_dot_s(sx.d, incx, sy.d, incy, n, &r, s);
  if (blas) blas->flops += 2.0 * n;
  return r;
}

static double blas_nrm2(NLBlas_t blas, int n, const double* x, int incx) {
  const double d = blas_dot(blas, n, x, incx, x, incx);
  return d > 0.0 ? std::sqrt(d) : 0.0;
}

static void blas_axpy(NLBlas_t blas, int n, double a, const double* x, int incx, double* y, int incy) {
  if (!blas_inc_ok(incx, incy) || n <= 0) return;
  cudaStream_t s = api_stream();
  Staged sx, sy;
  if (!sx.in(x, span(n, incx), s) || !sy.in(y, span(n, incy), s)) return;
  dev_axpy_s(n, a, sx.d, incx, sy.d, incy, s);
  sy.out(y, span(n, incy), s);
  cudaStreamSynchronize(s);
  if (blas) blas->flops += 2.0 * n;
}

static void blas_mul(NLBlas_t blas, int n, const double* x, double* y) {
  if (n <= 0) return;
  cudaStream_t s = api_stream();
  Staged sx, sy;
  if (!sx.in(x, n, s) || !sy.in(y, n, s)) return;
  dev_mul(n, sx.d, sy.d, s);
  sy.out(y, n, s);
  cudaStreamSynchronize(s);
  if (blas) blas->flops += n;
}

static NLBlas g_blas = {blas_copy, blas_scal, blas_dot, blas_nrm2, blas_axpy, blas_mul,
                        NL_TRUE, 0.0, {0, 0}, {0, 0}};

NLBlas_t nlHostBlas(void) { return &g_blas; }
NLBlas_t nlCUDABlas(void) { return &g_blas; }
void nlBlasResetStats(NLBlas_t blas) {
  if (!blas) return;
  blas->flops = 0.0;
  blas->used_ram[0] = blas->used_ram[1] = 0;
  blas->max_used_ram[0] = blas->max_used_ram[1] = 0;
}

}  // extern "C"
