// A C++ caller of libnl_gb300 written against geogram's OpenNL header paths,
// the way Graphite's sources include them (src/lib/OGF/scene_graph/NL/
// matrix.cpp:40-42, blas.cpp:40, plugins/OGF/WarpDrive/commands/
// voxel_grob_transport_commands.cpp:41): with libnl_gb300's include/ first
// on the include path, these resolve to the library's header.  It runs the
// call shapes those files use and writes the results for
// tests/test_caller_cpp.py (CPU: compile and link; GPU: run and compare with
// the oracle).
//
//   opennl_caller voxel  in.bin out.bin   -- least-squares voxel
//       interpolation through the context API (nlNewContext ... nlSolve ...
//       nlGetVariable), periodic 7-point rows, locked data voxels;
//   opennl_caller matrix in.bin out.bin   -- the OGF::NL::Matrix sequence:
//       nlSparseMatrixNew / nlSparseMatrixAdd on an (NLSparseMatrix*) cast /
//       nlMultMatrixVector / nlMatrixCompress / nlNewJacobiPreconditioner /
//       nlSolveSystemIterative(nlHostBlas(), ..., NL_CG, ...), and the
//       NLBlas table (Dcopy, Dscal, Ddot, Dnrm2, Daxpy).
#include <geogram/NL/nl.h>
#include <geogram/NL/nl_blas.h>
#include <geogram/NL/nl_iterative_solvers.h>
#include <geogram/NL/nl_matrix.h>
#include <geogram/NL/nl_preconditioners.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

template <typename T>
bool read_vec(FILE* f, std::vector<T>& v, size_t n) {
  v.resize(n);
  return n == 0 || std::fread(v.data(), sizeof(T), n, f) == n;
}

template <typename T>
void write_vec(FILE* f, const std::vector<T>& v) {
  if (!v.empty()) std::fwrite(v.data(), sizeof(T), v.size(), f);
}

// Voxel (u, v, w) of an nu x nv x nw periodic grid, u fastest.
int voxel(int u, int v, int w, int nu, int nv, int nw) {
  u = (u + nu) % nu;
  v = (v + nv) % nv;
  w = (w + nw) % nw;
  return (w * nv + v) * nu + u;
}

int run_voxel(FILE* in, FILE* out) {
  int32_t dims[3];
  if (std::fread(dims, sizeof(int32_t), 3, in) != 3) return 2;
  const int nu = dims[0], nv = dims[1], nw = dims[2];
  const int n = nu * nv * nw;
  std::vector<uint8_t> locked;
  std::vector<double> values;
  if (!read_vec(in, locked, (size_t)n) || !read_vec(in, values, (size_t)n)) return 2;

  nlNewContext();
  nlSolverParameteri(NL_LEAST_SQUARES, NL_TRUE);
  nlSolverParameteri(NL_NB_VARIABLES, NLint(n));
  nlBegin(NL_SYSTEM);
  for (int i = 0; i < n; ++i) {
    if (locked[i]) {
      nlSetVariable(NLuint(i), values[i]);
      nlLockVariable(NLuint(i));
    }
  }
  nlBegin(NL_MATRIX);
  // the discrete Laplacian of every voxel should vanish (least squares)
  for (int w = 0; w < nw; ++w)
    for (int v = 0; v < nv; ++v)
      for (int u = 0; u < nu; ++u) {
        nlBegin(NL_ROW);
        nlCoefficient(NLuint(voxel(u, v, w, nu, nv, nw)), -6.0);
        nlCoefficient(NLuint(voxel(u - 1, v, w, nu, nv, nw)), 1.0);
        nlCoefficient(NLuint(voxel(u + 1, v, w, nu, nv, nw)), 1.0);
        nlCoefficient(NLuint(voxel(u, v - 1, w, nu, nv, nw)), 1.0);
        nlCoefficient(NLuint(voxel(u, v + 1, w, nu, nv, nw)), 1.0);
        nlCoefficient(NLuint(voxel(u, v, w - 1, nu, nv, nw)), 1.0);
        nlCoefficient(NLuint(voxel(u, v, w + 1, nu, nv, nw)), 1.0);
        nlEnd(NL_ROW);
      }
  nlEnd(NL_MATRIX);
  nlEnd(NL_SYSTEM);
  const NLboolean ok = nlSolve();
  std::vector<double> x((size_t)n);
  for (int i = 0; i < n; ++i) x[i] = nlGetVariable(NLuint(i));
  NLint used = 0;
  nlGetIntegerv(NL_USED_ITERATIONS, &used);
  nlDeleteContext(nlGetCurrent());
  write_vec(out, x);
  const int32_t tail[2] = {int32_t(ok), int32_t(used)};
  std::fwrite(tail, sizeof(int32_t), 2, out);
  return 0;
}

int run_matrix(FILE* in, FILE* out) {
  int32_t hdr[2];
  if (std::fread(hdr, sizeof(int32_t), 2, in) != 2) return 2;
  const int n = hdr[0], nnz = hdr[1];
  std::vector<int32_t> I, J;
  std::vector<double> A, b;
  if (!read_vec(in, I, (size_t)nnz) || !read_vec(in, J, (size_t)nnz) || !read_vec(in, A, (size_t)nnz) ||
      !read_vec(in, b, (size_t)n))
    return 2;

  NLMatrix M = nlSparseMatrixNew(NLuint(n), NLuint(n), NL_MATRIX_STORE_ROWS);
  if (M == nullptr || M->m != NLuint(n) || M->n != NLuint(n) || M->type != NL_MATRIX_SPARSE_DYNAMIC) return 3;
  for (int k = 0; k < nnz; ++k) nlSparseMatrixAdd((NLSparseMatrix*)(M), NLuint(I[k]), NLuint(J[k]), A[k]);
  std::vector<double> y_dyn((size_t)n), y_crs((size_t)n), x((size_t)n, 0.0);
  nlMultMatrixVector(M, b.data(), y_dyn.data());
  nlMatrixCompress(&M);
  if (M->type != NL_MATRIX_CRS) return 4;
  nlMultMatrixVector(M, b.data(), y_crs.data());
  NLMatrix P = nlNewJacobiPreconditioner(M);
  const NLuint iters = nlSolveSystemIterative(nlHostBlas(), M, P, b.data(), x.data(), NL_CG, 1e-10,
                                              NLuint(5 * n), 5);
  if (P != nullptr) nlDeleteMatrix(P);
  nlDeleteMatrix(M);

  // NLBlas table, unit and non-unit increments
  NLBlas_t blas = nlHostBlas();
  std::vector<double> c((size_t)n), e(b), s2((size_t)(2 * n), -1.0);
  blas->Dcopy(blas, n, b.data(), 1, c.data(), 1);           // c = b
  blas->Dscal(blas, n, 2.0, c.data(), 1);                   // c = 2 b
  const double dot = blas->Ddot(blas, n, b.data(), 1, c.data(), 1);   // 2 |b|^2
  const double nrm = blas->Dnrm2(blas, n, b.data(), 1);               // |b|
  blas->Daxpy(blas, n, -0.25, c.data(), 1, e.data(), 1);    // e = b - 0.5 b
  blas->Dcopy(blas, n, b.data(), 1, s2.data(), 2);          // s2[2i] = b[i], odd slots stay -1
  blas->Dscal(blas, n, 3.0, s2.data(), 2);                  // s2[2i] = 3 b[i]
  const double dot_rev = blas->Ddot(blas, n, b.data(), 1, s2.data(), -2);   // sum b[i] * 3 b[n-1-i]

  write_vec(out, y_dyn);
  write_vec(out, y_crs);
  write_vec(out, x);
  write_vec(out, c);
  write_vec(out, e);
  write_vec(out, s2);
  const double scalars[4] = {dot, nrm, dot_rev, double(iters)};
  std::fwrite(scalars, sizeof(double), 4, out);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s voxel|matrix in.bin out.bin\n", argv[0]);
    return 1;
  }
  FILE* in = std::fopen(argv[2], "rb");
  FILE* out = std::fopen(argv[3], "wb");
  if (!in || !out) return 1;
  const int rc = std::strcmp(argv[1], "voxel") == 0 ? run_voxel(in, out)
               : std::strcmp(argv[1], "matrix") == 0 ? run_matrix(in, out) : 1;
  std::fclose(in);
  std::fclose(out);
  return rc;
}
