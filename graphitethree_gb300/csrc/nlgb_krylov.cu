// nlgb_krylov.cu -- Krylov solvers for general square systems: BiCGSTAB and
// restarted GMRES(m), FP64, with Jacobi (or no) right preconditioning.
//
// Reference context: OpenNL's NL_BICGSTAB and NL_GMRES solvers, selected
// through nlSolverParameteri(NL_SOLVER, ...) or nlSolveSystemIterative
// (src/lib/OGF/scene_graph/NL/matrix.cpp:390-393), used by the WarpDrive /
// optimal-transport Newton steps
// (plugins/OGF/WarpDrive/commands/mesh_grob_transport_commands.cpp:456-474),
// whose Jacobians are not symmetric.  Published algorithms restated here:
// BiCGSTAB, H. A. van der Vorst, SIAM J. Sci. Stat. Comput. 13 (1992);
// GMRES(m), Y. Saad & M. H. Schultz, SIAM J. Sci. Stat. Comput. 7 (1986),
// with Givens rotations and classical Gram-Schmidt applied twice (CGS2; as
// stable as modified Gram-Schmidt in practice, L. Giraud, J. Langou &
// M. Rozloznik 2005) so that an inner step needs two multi-dot passes
// instead of 2(j + 1) dependent dot/axpy passes.
//
// Layout: the matrix's own tiles (DeviceCRS::tile_rows, threads per row);
// every dot product is a set of per-tile partials reduced in a fixed order
// by one CTA (canon_reduce), and every scalar step runs on the device, so the
// host only enqueues kernels and polls the status once per chunk (BiCGSTAB)
// or per restart cycle (GMRES).  Kernels return at once when the system is no
// longer running, which makes overshooting a chunk harmless.
#include "nlgb_core.cuh"
#include "nlgb_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace nlgb {
namespace {

constexpr int kMaxRestart = 64;     // GMRES(m): m <= 64
constexpr int kChunk = 16;          // BiCGSTAB iterations between status polls

struct KrState {
  double rho, alpha, omega, beta;   // BiCGSTAB scalars
  double bnorm2, thresh2, rr, rr_true;
  double gnorm;                     // GMRES: |g_{j+1}| (residual estimate)
  long long iter, max_iter;
  int status;                       // ST_*
  int zero_rhs;
  int j;                            // GMRES: inner step of the cycle
  int cyc_done;                     // GMRES: this cycle is finished
  int m;                            // GMRES restart length
  int pad_;
  double H[(kMaxRestart + 1) * kMaxRestart];   // column-major, (m + 1) x m
  double cs[kMaxRestart], sn[kMaxRestart], g[kMaxRestart + 1], y[kMaxRestart];
  double hr[kMaxRestart + 1];       // GMRES: coefficients of the current Gram-Schmidt round
};

struct KrView {
  int n, tile_rows, n_tiles;
  const int* rp;
  const int* ci;
  const double* va;
  const double* dinv;
  double* part;      // n_tiles * kParts
  KrState* st;
  double* mpart;     // GMRES: n_tiles * (m + 1) multi-dot partials
  int mstride;
};

__device__ __forceinline__ bool running(const KrView& v) {
  return *((volatile int*)&v.st->status) == ST_RUNNING;
}
__device__ __forceinline__ int lo_of(const KrView& v) { return blockIdx.x * v.tile_rows; }
__device__ __forceinline__ int hi_of(const KrView& v) { return min(v.n, (int)(blockIdx.x + 1) * v.tile_rows); }

template <int K>
__device__ __forceinline__ void put_tile(const KrView& v, int slot, double (&a)[K]) {
  block_sum<K>(a);
  if (threadIdx.x == 0)
    for (int k = 0; k < K; ++k) v.part[(size_t)blockIdx.x * kParts + slot + k] = a[k];
}

template <int K>
__device__ __forceinline__ void sums(const KrView& v, int slot, double (&o)[K]) {
  int comp[K];
  for (int k = 0; k < K; ++k) comp[k] = slot + k;
  canon_reduce<K>(v.part, v.n_tiles, comp, o);
}

__device__ __forceinline__ bool finite_nz(double x) { return x == x && x != 0.0 && fabs(x) < 1e300; }

// y = A x on this CTA's tile, epi(row, (A x)_row) by the row's lane 0.
template <int T, typename Epi>
__device__ __forceinline__ void tile_spmv(const KrView& v, const double* x, Epi&& epi) {
  tile_rows_dot<T, double, double, double, false>(v.rp, v.ci, v.va, x, lo_of(v), hi_of(v), epi);
}

// ---------------------------------------------------------------------------
// BiCGSTAB (right preconditioning, M^-1 = D^-1):
//   r = b - A x, rh = r, rho = rh.r, p = v = 0, alpha = omega = 1
//   loop: p = r + beta (p - omega v); y = M^-1 p; v = A y; alpha = rho / rh.v
//         s = r - alpha v; z = M^-1 s; t = A z; omega = t.s / t.t
//         x += alpha y + omega z; r = s - omega t
//         stop on ||r|| <= eps ||b||; beta = (rh.r / rho)(alpha / omega)
// Vectors: r (holds s after the alpha step), rh, p, v, y, z, t.
// ---------------------------------------------------------------------------
struct BiVecs { const double* b; double *x, *r, *rh, *p, *v, *y, *z, *t; };

template <int T>
__global__ void __launch_bounds__(kCTA) k_bi_init(KrView v, BiVecs w) {
  double a[2] = {0.0, 0.0};
  tile_spmv<T>(v, w.x, [&](int i, double ax) {
    const double bi = w.b[i], ri = bi - ax;
    w.r[i] = ri; w.rh[i] = ri; w.p[i] = 0.0; w.v[i] = 0.0;
    a[0] = fma(bi, bi, a[0]);
    a[1] = fma(ri, ri, a[1]);
  });
  put_tile<2>(v, 0, a);
}

__global__ void k_bi_init_scalar(KrView v) {
  double o[2];
  sums<2>(v, 0, o);
  if (threadIdx.x != 0) return;
  KrState* st = v.st;
  st->bnorm2 = o[0];
  st->rr = o[1];
  st->rho = o[1];               // rh = r
  st->alpha = st->omega = 1.0;
  st->beta = o[1];              // (rho / 1) (1 / 1); p = r on the first step
  if (!(o[0] > 0.0)) { st->zero_rhs = o[0] == 0.0; st->status = o[0] == 0.0 ? ST_CONVERGED : ST_BREAKDOWN; return; }
  if (o[1] <= st->thresh2 * o[0]) { st->status = ST_CONVERGED; return; }
  if (st->max_iter <= 0) { st->status = ST_MAX_ITER; return; }
  st->status = ST_RUNNING;
}

__global__ void __launch_bounds__(kCTA) k_bi_p(KrView v, BiVecs w) {
  if (!running(v)) return;
  const double beta = v.st->beta, omega = v.st->omega;
  for (int i = lo_of(v) + threadIdx.x; i < hi_of(v); i += kCTA) {
    const double pi = w.r[i] + beta * (w.p[i] - omega * w.v[i]);
    w.p[i] = pi;
    w.y[i] = v.dinv[i] * pi;
  }
}

template <int T>
__global__ void __launch_bounds__(kCTA) k_bi_v(KrView v, BiVecs w) {
  if (!running(v)) return;
  double a[1] = {0.0};
  tile_spmv<T>(v, w.y, [&](int i, double q) { w.v[i] = q; a[0] = fma(w.rh[i], q, a[0]); });
  put_tile<1>(v, 0, a);
}

__global__ void k_bi_alpha(KrView v) {
  if (!running(v)) return;
  double o[1];
  sums<1>(v, 0, o);
  if (threadIdx.x != 0) return;
  if (!finite_nz(o[0])) { v.st->status = ST_BREAKDOWN; return; }
  v.st->alpha = v.st->rho / o[0];
}

__global__ void __launch_bounds__(kCTA) k_bi_s(KrView v, BiVecs w) {
  if (!running(v)) return;
  const double alpha = v.st->alpha;
  for (int i = lo_of(v) + threadIdx.x; i < hi_of(v); i += kCTA) {
    const double si = w.r[i] - alpha * w.v[i];
    w.r[i] = si;                      // r now holds s
    w.z[i] = v.dinv[i] * si;
  }
}

template <int T>
__global__ void __launch_bounds__(kCTA) k_bi_t(KrView v, BiVecs w) {
  if (!running(v)) return;
  double a[2] = {0.0, 0.0};
  tile_spmv<T>(v, w.z, [&](int i, double q) {
    w.t[i] = q;
    a[0] = fma(q, w.r[i], a[0]);      // t.s
    a[1] = fma(q, q, a[1]);           // t.t
  });
  put_tile<2>(v, 1, a);
}

__global__ void k_bi_omega(KrView v) {
  if (!running(v)) return;
  double o[2];
  sums<2>(v, 1, o);
  if (threadIdx.x != 0) return;
  v.st->omega = o[1] > 0.0 ? o[0] / o[1] : 0.0;
}

__global__ void __launch_bounds__(kCTA) k_bi_xr(KrView v, BiVecs w) {
  if (!running(v)) return;
  const double alpha = v.st->alpha, omega = v.st->omega;
  double a[2] = {0.0, 0.0};
  for (int i = lo_of(v) + threadIdx.x; i < hi_of(v); i += kCTA) {
    w.x[i] += alpha * w.y[i] + omega * w.z[i];
    const double ri = w.r[i] - omega * w.t[i];
    w.r[i] = ri;
    a[0] = fma(ri, ri, a[0]);
    a[1] = fma(w.rh[i], ri, a[1]);
  }
  put_tile<2>(v, 3, a);
}

__global__ void k_bi_end(KrView v) {
  if (!running(v)) return;
  double o[2];
  sums<2>(v, 3, o);
  if (threadIdx.x != 0) return;
  KrState* st = v.st;
  st->iter += 1;
  st->rr = o[0];
  if (!(o[0] <= 1e300)) { st->status = ST_BREAKDOWN; return; }
  if (o[0] <= st->thresh2 * st->bnorm2) { st->status = ST_CONVERGED; return; }
  if (st->iter >= st->max_iter) { st->status = ST_MAX_ITER; return; }
  if (!finite_nz(o[1]) || !finite_nz(st->omega)) { st->status = ST_BREAKDOWN; return; }
  st->beta = (o[1] / st->rho) * (st->alpha / st->omega);
  st->rho = o[1];
}

// True residual ||b - A x||^2 of the returned x (and x = 0 when b = 0).
template <int T>
__global__ void __launch_bounds__(kCTA) k_kr_true(KrView v, const double* b, double* x) {
  double a[1] = {0.0};
  if (v.st->zero_rhs) {
    for (int i = lo_of(v) + threadIdx.x; i < hi_of(v); i += kCTA) x[i] = 0.0;
  } else {
    tile_spmv<T>(v, x, [&](int i, double ax) { const double ri = b[i] - ax; a[0] = fma(ri, ri, a[0]); });
  }
  put_tile<1>(v, 6, a);
}

__global__ void k_kr_true_scalar(KrView v) {
  double o[1];
  sums<1>(v, 6, o);
  if (threadIdx.x == 0) v.st->rr_true = o[0];
}

// ---------------------------------------------------------------------------
// GMRES(m) (right preconditioning, M^-1 = D^-1), one cycle:
//   r = b - A x, beta = ||r||, V0 = r / beta, g = beta e1
//   for j < m: w = A M^-1 V_j; classical Gram-Schmidt against V_0..V_j,
//              twice (CGS2: h = V^T w, w -= V h; again; H_j = h + h2);
//              H_{j+1,j} = ||w||, V_{j+1} = w / H_{j+1,j}; Givens rotations
//              on column j, g; |g_{j+1}| is the residual norm
//   y = H^-1 g (upper triangular), x += M^-1 (V y)
// Convergence is decided on the true residual at the start of a cycle.
// ---------------------------------------------------------------------------
struct GmVecs { const double* b; double* x; double* V; double* u; size_t ld; };

template <int T>
__global__ void __launch_bounds__(kCTA) k_gm_residual(KrView v, GmVecs w) {
  if (*((volatile int*)&v.st->status) != ST_RUNNING) return;
  double a[2] = {0.0, 0.0};
  tile_spmv<T>(v, w.x, [&](int i, double ax) {
    const double bi = w.b[i], ri = bi - ax;
    w.V[i] = ri;
    a[0] = fma(bi, bi, a[0]);
    a[1] = fma(ri, ri, a[1]);
  });
  put_tile<2>(v, 0, a);
}

__global__ void k_gm_start(KrView v, int first) {
  if (*((volatile int*)&v.st->status) != ST_RUNNING) return;
  double o[2];
  sums<2>(v, 0, o);
  if (threadIdx.x != 0) return;
  KrState* st = v.st;
  if (first) {
    st->bnorm2 = o[0];
    if (!(o[0] > 0.0)) { st->zero_rhs = o[0] == 0.0; st->status = o[0] == 0.0 ? ST_CONVERGED : ST_BREAKDOWN; return; }
  }
  st->rr = o[1];
  if (!(o[1] <= 1e300)) { st->status = ST_BREAKDOWN; return; }
  if (o[1] <= st->thresh2 * st->bnorm2) { st->status = ST_CONVERGED; return; }
  if (st->iter >= st->max_iter) { st->status = ST_MAX_ITER; return; }
  const double beta = sqrt(o[1]);
  for (int k = 0; k <= st->m; ++k) st->g[k] = 0.0;
  st->g[0] = beta;
  st->gnorm = beta;
  st->j = 0;
  st->cyc_done = 0;
  st->beta = beta;
}

__global__ void k_gm_scale0(KrView v, GmVecs w) {
  if (*((volatile int*)&v.st->status) != ST_RUNNING || v.st->cyc_done) return;
  const double inv = 1.0 / v.st->beta;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < v.n; i += (long long)gridDim.x * blockDim.x)
    w.V[i] *= inv;
}

__device__ __forceinline__ bool gm_active(const KrView& v, int j) {
  return *((volatile int*)&v.st->status) == ST_RUNNING && !v.st->cyc_done && v.st->j == j;
}

// u = M^-1 V_j
__global__ void k_gm_precond(KrView v, GmVecs w, int j) {
  if (!gm_active(v, j)) return;
  const double* Vj = w.V + (size_t)j * w.ld;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < v.n; i += (long long)gridDim.x * blockDim.x)
    w.u[i] = v.dinv[i] * Vj[i];
}

// V_{j+1} = A u
template <int T>
__global__ void __launch_bounds__(kCTA) k_gm_spmv(KrView v, GmVecs w, int j) {
  if (!gm_active(v, j)) return;
  double* Wn = w.V + (size_t)(j + 1) * w.ld;
  tile_spmv<T>(v, w.u, [&](int i, double q) { Wn[i] = q; });
}

// Gram-Schmidt round, 1/3: per-tile partials of V_i . w for every i <= j
// (one sweep over the tile per i; w stays in L1 between them).  Measured on
// GB300: grouping eight coefficients per sweep was not faster.
__global__ void __launch_bounds__(kCTA) k_gm_multidot(KrView v, GmVecs w, int j) {
  if (!gm_active(v, j)) return;
  const double* Wn = w.V + (size_t)(j + 1) * w.ld;
  for (int i = 0; i <= j; ++i) {
    const double* Vi = w.V + (size_t)i * w.ld;
    double a[1] = {0.0};
    for (int r = lo_of(v) + threadIdx.x; r < hi_of(v); r += kCTA) a[0] = fma(Wn[r], Vi[r], a[0]);
    block_sum<1>(a);
    if (threadIdx.x == 0) v.mpart[(size_t)blockIdx.x * v.mstride + i] = a[0];
  }
}

// 2/3: CTA i reduces coefficient i over the tiles in the canonical order
// (thread t sums tiles t, t + 256, ..., then the fixed block tree).
__global__ void __launch_bounds__(kCTA) k_gm_hreduce(KrView v, int j, int round) {
  if (!gm_active(v, j)) return;
  const int i = blockIdx.x;
  double a[1] = {0.0};
  for (int t = threadIdx.x; t < v.n_tiles; t += kCTA) a[0] += v.mpart[(size_t)t * v.mstride + i];
  block_sum<1>(a);
  if (threadIdx.x == 0) {
    double* Hj = v.st->H + j * (kMaxRestart + 1);
    v.st->hr[i] = a[0];
    Hj[i] = round == 0 ? a[0] : Hj[i] + a[0];
  }
}

// 3/3: w -= sum_i hr_i V_i (i in order); after the second round also the
// partial of w.w for the norm.
__global__ void __launch_bounds__(kCTA) k_gm_update(KrView v, GmVecs w, int j, int with_norm) {
  if (!gm_active(v, j)) return;
  double* Wn = w.V + (size_t)(j + 1) * w.ld;
  const double* hr = v.st->hr;
  double a[1] = {0.0};
  for (int r = lo_of(v) + threadIdx.x; r < hi_of(v); r += kCTA) {
    double x = Wn[r];
    for (int i = 0; i <= j; ++i) x -= hr[i] * w.V[(size_t)i * w.ld + r];
    Wn[r] = x;
    a[0] = fma(x, x, a[0]);
  }
  if (with_norm) put_tile<1>(v, 0, a);
}

// H_{j+1,j} = ||w||, V_{j+1} /= it; Givens rotations; cycle control.
__global__ void k_gm_norm(KrView v, int j) {
  if (!gm_active(v, j)) return;
  double o[1];
  sums<1>(v, 0, o);
  if (threadIdx.x != 0) return;
  KrState* st = v.st;
  double* Hj = st->H + j * (kMaxRestart + 1);
  const double hn = sqrt(o[0]);
  Hj[j + 1] = hn;
  for (int k = 0; k < j; ++k) {              // previous rotations on column j
    const double a = Hj[k], b = Hj[k + 1];
    Hj[k] = st->cs[k] * a + st->sn[k] * b;
    Hj[k + 1] = -st->sn[k] * a + st->cs[k] * b;
  }
  const double a = Hj[j], b = Hj[j + 1];
  const double den = hypot(a, b);
  const double c = den > 0.0 ? a / den : 1.0, s = den > 0.0 ? b / den : 0.0;
  st->cs[j] = c; st->sn[j] = s;
  Hj[j] = den; Hj[j + 1] = 0.0;
  st->g[j + 1] = -s * st->g[j];
  st->g[j] = c * st->g[j];
  st->gnorm = fabs(st->g[j + 1]);
  st->iter += 1;
  st->j = j + 1;
  if (!(den > 0.0) || !(hn == hn)) { st->cyc_done = 1; if (!(den > 0.0)) st->status = ST_BREAKDOWN; return; }
  if (st->gnorm * st->gnorm <= st->thresh2 * st->bnorm2 || j + 1 >= st->m ||
      st->iter >= st->max_iter || !(hn > 0.0))
    st->cyc_done = 1;
  st->beta = hn;        // for the scaling of V_{j+1}
}

__global__ void k_gm_scale(KrView v, GmVecs w, int j) {
  // V_{j+1} /= H_{j+1,j} (skipped after a lucky breakdown, H_{j+1,j} = 0)
  if (*((volatile int*)&v.st->status) != ST_RUNNING || v.st->j != j + 1 || !(v.st->beta > 0.0)) return;
  double* Wn = w.V + (size_t)(j + 1) * w.ld;
  const double inv = 1.0 / v.st->beta;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < v.n; i += (long long)gridDim.x * blockDim.x)
    Wn[i] *= inv;
}

// End of a cycle: y = H^-1 g (back substitution over the k = j steps done)
__global__ void k_gm_solve_y(KrView v) {
  KrState* st = v.st;
  if (*((volatile int*)&st->status) != ST_RUNNING || threadIdx.x != 0) return;
  const int k = st->j;
  for (int i = k - 1; i >= 0; --i) {
    double s = st->g[i];
    for (int c = i + 1; c < k; ++c) s -= st->H[c * (kMaxRestart + 1) + i] * st->y[c];
    st->y[i] = s / st->H[i * (kMaxRestart + 1) + i];
  }
}

// x += M^-1 (V y)
__global__ void k_gm_update_x(KrView v, GmVecs w) {
  KrState* st = v.st;
  if (*((volatile int*)&st->status) != ST_RUNNING) return;
  const int k = st->j;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < v.n; i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < k; ++c) s += st->y[c] * w.V[(size_t)c * w.ld + i];
    w.x[i] += v.dinv[i] * s;
  }
}

// With a general (SSOR) preconditioner: t = V y (the correction before
// preconditioning), then x += M^-1 t.
__global__ void k_gm_vy(KrView v, GmVecs w, double* t) {
  KrState* st = v.st;
  if (*((volatile int*)&st->status) != ST_RUNNING) return;
  const int k = st->j;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < v.n; i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < k; ++c) s += st->y[c] * w.V[(size_t)c * w.ld + i];
    t[i] = s;
  }
}
__global__ void k_gm_add_x(KrView v, double* x, const double* z) {
  if (*((volatile int*)&v.st->status) != ST_RUNNING) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < v.n; i += (long long)gridDim.x * blockDim.x)
    x[i] += z[i];
}

int grid1(long long n) { return (int)std::max(1LL, std::min<long long>((n + 255) / 256, 152LL * 8)); }

}  // namespace

#define NLGB_KR_T(LAUNCH)                                         \
  switch (A.tpr) {                                                \
    case 1: { constexpr int T = 1; LAUNCH; } break;               \
    case 2: { constexpr int T = 2; LAUNCH; } break;               \
    case 4: { constexpr int T = 4; LAUNCH; } break;               \
    case 8: { constexpr int T = 8; LAUNCH; } break;               \
    case 16: { constexpr int T = 16; LAUNCH; } break;             \
    default: { constexpr int T = 32; LAUNCH; } break;             \
  }

cudaError_t krylov_solve(const DeviceCRS& A, const double* dinv, const double* b, double* x,
                         int method, double eps, long long max_iter, int restart, cudaStream_t s,
                         KrylovResult* res, SsorPrecond* P) {
  const int n = A.n;
  const int tile_rows = A.tile_rows > 0 ? A.tile_rows : 128;
  const int n_tiles = std::max(1, (n + tile_rows - 1) / tile_rows);
  const int m = std::max(1, std::min(restart, kMaxRestart));
  // work vectors (+ two for GMRES's correction around a general preconditioner)
  const int n_vec = method == KRYLOV_BICGSTAB ? 7 : (m + 2 + (P ? 2 : 0));
  const size_t ld = (size_t)((n + 31) / 32 * 32);
  double* work = nullptr;
  double* part = nullptr;
  KrState* st = nullptr;
  NLGB_CUDA_TRY(cudaMallocAsync(&work, sizeof(double) * ld * n_vec + 256, s));
  cudaError_t e = cudaMallocAsync(&part, sizeof(double) * (size_t)n_tiles * kParts, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&st, sizeof(KrState), s);
  double* mpart = nullptr;
  if (e == cudaSuccess && method == KRYLOV_GMRES)
    e = cudaMallocAsync(&mpart, sizeof(double) * (size_t)n_tiles * (m + 1), s);
  KrState h;
  std::memset(&h, 0, sizeof(h));
  h.thresh2 = eps * eps;
  h.max_iter = max_iter;
  h.status = ST_RUNNING;
  h.m = m;
  if (e == cudaSuccess) e = cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s);
  KrView v{n, tile_rows, n_tiles, A.rp, A.ci, A.va, dinv, part, st, mpart, m + 1};
  long long launches = 0;
  auto poll = [&](int* status) {
    cudaError_t pe = cudaMemcpyAsync(status, &st->status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (pe == cudaSuccess) pe = cudaStreamSynchronize(s);
    return pe;
  };
  if (e == cudaSuccess && method == KRYLOV_BICGSTAB) {
    BiVecs w{b, x, work, work + ld, work + 2 * ld, work + 3 * ld, work + 4 * ld, work + 5 * ld, work + 6 * ld};
    NLGB_KR_T((k_bi_init<T><<<n_tiles, kCTA, 0, s>>>(v, w)));
    k_bi_init_scalar<<<1, kCTA, 0, s>>>(v);
    launches += 2;
    int status = ST_RUNNING;
    while (e == cudaSuccess && status == ST_RUNNING) {
      for (int c = 0; c < kChunk; ++c) {
        // (with a general preconditioner dinv is all ones: y = p, z = s,
        // then y = M^-1 p, z = M^-1 s)
        k_bi_p<<<n_tiles, kCTA, 0, s>>>(v, w);
        if (P && e == cudaSuccess) e = P->apply(w.p, w.y, s);
        NLGB_KR_T((k_bi_v<T><<<n_tiles, kCTA, 0, s>>>(v, w)));
        k_bi_alpha<<<1, kCTA, 0, s>>>(v);
        k_bi_s<<<n_tiles, kCTA, 0, s>>>(v, w);
        if (P && e == cudaSuccess) e = P->apply(w.r, w.z, s);
        NLGB_KR_T((k_bi_t<T><<<n_tiles, kCTA, 0, s>>>(v, w)));
        k_bi_omega<<<1, kCTA, 0, s>>>(v);
        k_bi_xr<<<n_tiles, kCTA, 0, s>>>(v, w);
        k_bi_end<<<1, kCTA, 0, s>>>(v);
        launches += 8;
      }
      if (e == cudaSuccess) e = cudaGetLastError();
      if (e == cudaSuccess) e = poll(&status);
    }
  } else if (e == cudaSuccess) {
    GmVecs w{b, x, work, work + (size_t)(m + 1) * ld, ld};
    double* t = P ? work + (size_t)(m + 2) * ld : nullptr;
    double* tz = P ? work + (size_t)(m + 3) * ld : nullptr;
    int status = ST_RUNNING;
    bool first = true;
    while (e == cudaSuccess && status == ST_RUNNING) {
      NLGB_KR_T((k_gm_residual<T><<<n_tiles, kCTA, 0, s>>>(v, w)));
      k_gm_start<<<1, kCTA, 0, s>>>(v, first ? 1 : 0);
      k_gm_scale0<<<grid1(n), 256, 0, s>>>(v, w);
      launches += 3;
      first = false;
      for (int j = 0; j < m; ++j) {
        if (P) {
          if (e == cudaSuccess) e = P->apply(w.V + (size_t)j * ld, w.u, s);   // u = M^-1 V_j
        } else {
          k_gm_precond<<<grid1(n), 256, 0, s>>>(v, w, j);
        }
        NLGB_KR_T((k_gm_spmv<T><<<n_tiles, kCTA, 0, s>>>(v, w, j)));
        for (int round = 0; round < 2; ++round) {     // CGS2
          k_gm_multidot<<<n_tiles, kCTA, 0, s>>>(v, w, j);
          k_gm_hreduce<<<j + 1, kCTA, 0, s>>>(v, j, round);
          k_gm_update<<<n_tiles, kCTA, 0, s>>>(v, w, j, round);
        }
        k_gm_norm<<<1, kCTA, 0, s>>>(v, j);
        k_gm_scale<<<grid1(n), 256, 0, s>>>(v, w, j);
        launches += 10;
      }
      k_gm_solve_y<<<1, 32, 0, s>>>(v);
      if (P) {
        k_gm_vy<<<grid1(n), 256, 0, s>>>(v, w, t);
        if (e == cudaSuccess) e = P->apply(t, tz, s);
        k_gm_add_x<<<grid1(n), 256, 0, s>>>(v, w.x, tz);
        launches += 1;
      } else {
        k_gm_update_x<<<grid1(n), 256, 0, s>>>(v, w);
      }
      launches += 2;
      if (e == cudaSuccess) e = cudaGetLastError();
      if (e == cudaSuccess) e = poll(&status);
    }
  }
  if (e == cudaSuccess) {
    NLGB_KR_T((k_kr_true<T><<<n_tiles, kCTA, 0, s>>>(v, b, x)));
    k_kr_true_scalar<<<1, kCTA, 0, s>>>(v);
    launches += 2;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  count_launches(launches);
  cudaFreeAsync(work, s);
  if (part) cudaFreeAsync(part, s);
  if (st) cudaFreeAsync(st, s);
  if (mpart) cudaFreeAsync(mpart, s);
  if (e != cudaSuccess) return e;
  if (res) {
    res->status = h.status;
    res->iterations = h.iter;
    res->rel_residual = h.bnorm2 > 0 ? std::sqrt(h.rr / h.bnorm2) : 0.0;
    res->true_rel_residual = h.bnorm2 > 0 ? std::sqrt(h.rr_true / h.bnorm2) : 0.0;
  }
  return cudaSuccess;
}

}  // namespace nlgb
