// nlgb_build.cu -- the LSCM and cotangent-fairing systems of a triangle mesh,
// built on the GPU from the vertices and triangles.
//
// Reference context: Graphite's mesh_compute_LSCM and mesh_smooth commands
// (src/lib/OGF/mesh/commands/mesh_grob_surface_commands.cpp:759 and :703)
// hand the mesh to geogram's builders, which emit the system row by row
// through nlBegin(NL_ROW) / nlCoefficient / nlEnd(NL_ROW) on the host.  Here
// one thread per triangle writes the rows of its triangle straight into a
// device row stream, and the normal-equation assembly (nlgb_assembly.cu)
// turns the stream into the CRS system, so a mesh never round-trips through
// host-side rows.
//
// LSCM (Levy et al. 2002): per triangle, in an orthonormal frame of its
// plane, q0 = 0, q1 = (x1, 0), q2 = (x2, y2); with s = 1 / sqrt(x1 y2)
// (1 / sqrt(2 area)) the two rows are the real and imaginary parts of
// sum_j (E_j s) (u_j + i v_j) = 0, E_0 = q2 - q1, E_1 = q0 - q2,
// E_2 = q1 - q0.  Variables: u of vertex k is 2k, v is 2k + 1; the two pinned
// vertices are locked at their (u, v).
//
// Cotangent Laplacian + lambda I (Pinkall-Polthier 1993): as least-squares
// rows, every triangle corner o with opposite edge (i, j) contributes the row
// e_i - e_j with weight (cot of the angle at o) / 2, and every vertex the row
// e_k with weight lambda; the normal equations are then exactly L + lambda I.
//
// Arithmetic: the expressions of graphitethree_gb300/systems.py
// (lscm_coefficients, cotan_weights), operation by operation, with explicit
// round-to-nearest intrinsics so that nothing is contracted into FMAs.
#include "nlgb_internal.h"

#include <algorithm>
#include <cstring>

namespace nlgb {
namespace {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dadd_rn(a, -b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

// ((a0 * b0 + a1 * b1) + a2 * b2), each product and sum rounded
__device__ __forceinline__ double dot3(const double* a, const double* b) {
  return add(add(mul(a[0], b[0]), mul(a[1], b[1])), mul(a[2], b[2]));
}
__device__ __forceinline__ void cross3(const double* a, const double* b, double* c) {
  c[0] = sub(mul(a[1], b[2]), mul(a[2], b[1]));
  c[1] = sub(mul(a[2], b[0]), mul(a[0], b[2]));
  c[2] = sub(mul(a[0], b[1]), mul(a[1], b[0]));
}
__device__ __forceinline__ double norm3(const double* a) { return __dsqrt_rn(dot3(a, a)); }

// Free index of variable v, or -(v + 1) if v is one of the 4 locked ones
// (sorted ascending in lk).
__device__ __forceinline__ int encode_var(int v, const int4 lk) {
  if (v == lk.x || v == lk.y || v == lk.z || v == lk.w) return -(v + 1);
  return v - (int)(v > lk.x) - (int)(v > lk.y) - (int)(v > lk.z) - (int)(v > lk.w);
}

__global__ void k_check_tris(long long n_idx, const int* __restrict__ tris, int n_verts, int* bad) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n_idx;
       k += (long long)gridDim.x * blockDim.x) {
    const int v = tris[k];
    if (v < 0 || v >= n_verts) atomicExch(bad, 1);
  }
}

// Two rows of 6 coefficients per triangle: row 2t (real part), 2t + 1
// (imaginary part), coefficients in the order u0 v0 u1 v1 u2 v2.
__global__ void k_lscm_rows(int n_tris, const double* __restrict__ xyz, const int* __restrict__ tris,
                            int4 locked, int* __restrict__ col, double* __restrict__ val) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tris) return;
  const int f[3] = {tris[3LL * t], tris[3LL * t + 1], tris[3LL * t + 2]};
  double p[3][3];
  for (int j = 0; j < 3; ++j)
    for (int c = 0; c < 3; ++c) p[j][c] = xyz[3 * (long long)f[j] + c];
  double e1[3], e2[3];
  for (int c = 0; c < 3; ++c) { e1[c] = sub(p[1][c], p[0][c]); e2[c] = sub(p[2][c], p[0][c]); }
  const double l1 = norm3(e1);
  const double dl = l1 > 0.0 ? l1 : 1.0;
  double X[3], N[3], nh[3], Y[3];
  for (int c = 0; c < 3; ++c) X[c] = dvd(e1[c], dl);
  cross3(e1, e2, N);
  const double nN = norm3(N);
  const double dn = nN > 0.0 ? nN : 1.0;
  for (int c = 0; c < 3; ++c) nh[c] = dvd(N[c], dn);
  cross3(nh, X, Y);
  const double x1 = l1, x2 = dot3(e2, X), y2 = dot3(e2, Y);
  const double d = mul(x1, y2);
  const double s = d > 0.0 ? dvd(1.0, __dsqrt_rn(d)) : 0.0;
  const double a[3] = {mul(sub(x2, x1), s), mul(-x2, s), mul(x1, s)};
  const double b[3] = {mul(y2, s), mul(-y2, s), 0.0};
  const long long o = 12LL * t;
  for (int j = 0; j < 3; ++j) {
    const int cu = encode_var(2 * f[j], locked), cv = encode_var(2 * f[j] + 1, locked);
    col[o + 2 * j] = cu;      val[o + 2 * j] = a[j];        // real: a u - b v
    col[o + 2 * j + 1] = cv;  val[o + 2 * j + 1] = -b[j];
    col[o + 6 + 2 * j] = cu;  val[o + 6 + 2 * j] = b[j];    // imaginary: b u + a v
    col[o + 6 + 2 * j + 1] = cv; val[o + 6 + 2 * j + 1] = a[j];
  }
}

// Row 3t + k: e_i - e_j, weight cot(angle at corner k) / 2, (i, j) the edge
// opposite corner k = (tri[k+1], tri[k+2]).
__global__ void k_cotan_rows(int n_tris, const double* __restrict__ xyz, const int* __restrict__ tris,
                             int* __restrict__ col, double* __restrict__ val, double* __restrict__ w) {
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= 3LL * n_tris) return;
  const int t = (int)(r / 3), k = (int)(r % 3);
  const int o = tris[3LL * t + k], i = tris[3LL * t + (k + 1) % 3], j = tris[3LL * t + (k + 2) % 3];
  double u[3], v[3], c[3];
  for (int q = 0; q < 3; ++q) {
    u[q] = sub(xyz[3 * (long long)i + q], xyz[3 * (long long)o + q]);
    v[q] = sub(xyz[3 * (long long)j + q], xyz[3 * (long long)o + q]);
  }
  cross3(u, v, c);
  const double cr = norm3(c);
  const double cot = cr > 0.0 ? dvd(dot3(u, v), cr) : 0.0;
  col[2 * r] = i;      val[2 * r] = 1.0;
  col[2 * r + 1] = j;  val[2 * r + 1] = -1.0;
  w[r] = mul(0.5, cot);
}

// Rows 3T + k (k < n_verts): e_k with weight lambda.
__global__ void k_diag_rows(int n_verts, long long first_row, long long first_coef, double lambda,
                            int* __restrict__ col, double* __restrict__ val, double* __restrict__ w) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_verts) return;
  col[first_coef + k] = k;
  val[first_coef + k] = 1.0;
  w[first_row + k] = lambda;
}

// Row pointers: `stride` coefficients for rows below `split`, then one each.
__global__ void k_row_ptr(long long n_rows, long long split, int stride, long long* __restrict__ rp) {
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r > n_rows) return;
  rp[r] = r <= split ? r * stride : split * stride + (r - split);
}

__global__ void k_set_locked(double* xl, int4 vars, double4 values) {
  xl[vars.x] = values.x; xl[vars.y] = values.y; xl[vars.z] = values.z; xl[vars.w] = values.w;
}

int grid_of(long long n, int block) { return (int)std::max(1LL, std::min<long long>((n + block - 1) / block, 1LL << 30)); }

// Stream-ordered scratch (cudaMallocAsync / cudaFreeAsync): no device-wide
// synchronisation, so a build can run while a solver kernel occupies the
// GPU (the solve server admits requests during an epoch).
struct DevBuf {
  void* p = nullptr;
  cudaStream_t st = nullptr;
  ~DevBuf() { if (p) cudaFreeAsync(p, st); }
  template <typename T>
  cudaError_t alloc(size_t count, cudaStream_t s) {
    st = s;
    return cudaMallocAsync(&p, std::max<size_t>(1, count) * sizeof(T), s);
  }
  template <typename T>
  T* as() const { return static_cast<T*>(p); }
};

// Device copies of the mesh (the caller's arrays may be host or device) and
// the triangle-index check.
cudaError_t mesh_to_device(int n_verts, const double* xyz, int n_tris, const int* tris, DevBuf& dx,
                           DevBuf& dt, cudaStream_t s, bool* bad_index, bool check) {
  NLGB_CUDA_TRY(dx.alloc<double>(3 * (size_t)n_verts, s));
  NLGB_CUDA_TRY(dt.alloc<int>(3 * (size_t)n_tris, s));
  if (n_verts > 0)
    NLGB_CUDA_TRY(cudaMemcpyAsync(dx.p, xyz, sizeof(double) * 3 * (size_t)n_verts, cudaMemcpyDefault, s));
  if (n_tris > 0)
    NLGB_CUDA_TRY(cudaMemcpyAsync(dt.p, tris, sizeof(int) * 3 * (size_t)n_tris, cudaMemcpyDefault, s));
  *bad_index = false;
  if (!check) return cudaSuccess;
  DevBuf flag;
  NLGB_CUDA_TRY(flag.alloc<int>(1, s));
  NLGB_CUDA_TRY(cudaMemsetAsync(flag.p, 0, sizeof(int), s));
  if (n_tris > 0) {
    k_check_tris<<<grid_of(3LL * n_tris, 256), 256, 0, s>>>(3LL * n_tris, dt.as<int>(), n_verts, flag.as<int>());
    count_launches(1);
    NLGB_CUDA_TRY(cudaGetLastError());
  }
  int h = 0;
  NLGB_CUDA_TRY(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  NLGB_CUDA_TRY(cudaStreamSynchronize(s));
  *bad_index = h != 0;
  return cudaSuccess;
}

}  // namespace

cudaError_t build_lscm_system(int n_verts, const double* xyz, int n_tris, const int* tris,
                              const int pins[2], const double pin_uv[4], DeviceCRS& out,
                              double* rhs_out, cudaStream_t s, bool* bad_input, bool check_indices) {
  *bad_input = false;
  DevBuf dx, dt;
  NLGB_CUDA_TRY(mesh_to_device(n_verts, xyz, n_tris, tris, dx, dt, s, bad_input, check_indices));
  if (*bad_input) return cudaSuccess;
  const int p0 = std::min(pins[0], pins[1]), p1 = std::max(pins[0], pins[1]);
  const double* uv0 = pins[0] <= pins[1] ? pin_uv : pin_uv + 2;
  const double* uv1 = pins[0] <= pins[1] ? pin_uv + 2 : pin_uv;
  const int4 locked = make_int4(2 * p0, 2 * p0 + 1, 2 * p1, 2 * p1 + 1);
  const int n_vars = 2 * n_verts, n_free = n_vars - 4;
  const long long n_rows = 2LL * n_tris, n_coefs = 6 * n_rows;
  DevBuf rp, col, val, xl;
  NLGB_CUDA_TRY(rp.alloc<long long>((size_t)n_rows + 1, s));
  NLGB_CUDA_TRY(col.alloc<int>((size_t)n_coefs, s));
  NLGB_CUDA_TRY(val.alloc<double>((size_t)n_coefs, s));
  NLGB_CUDA_TRY(xl.alloc<double>((size_t)n_vars, s));
  NLGB_CUDA_TRY(cudaMemsetAsync(xl.p, 0, sizeof(double) * (size_t)n_vars, s));
  k_set_locked<<<1, 1, 0, s>>>(xl.as<double>(), locked, make_double4(uv0[0], uv0[1], uv1[0], uv1[1]));
  k_row_ptr<<<grid_of(n_rows + 1, 256), 256, 0, s>>>(n_rows, n_rows, 6, rp.as<long long>());
  count_launches(2);
  if (n_tris > 0) {
    k_lscm_rows<<<grid_of(n_tris, 128), 128, 0, s>>>(n_tris, dx.as<double>(), dt.as<int>(), locked,
                                                      col.as<int>(), val.as<double>());
    count_launches(1);
  }
  NLGB_CUDA_TRY(cudaGetLastError());
  LSRowsDevice R;
  R.n_rows = n_rows; R.n_coefs = n_coefs; R.n_free = n_free; R.n_vars = n_vars; R.n_systems = 1;
  R.row_ptr = rp.as<long long>(); R.col = col.as<int>(); R.val = val.as<double>();
  R.rhs = nullptr; R.weight = nullptr; R.xl = xl.as<double>();
  NLGB_CUDA_TRY(assemble_normal_equations(R, out, rhs_out, s));
  return cudaStreamSynchronize(s);
}

cudaError_t build_fairing_system(int n_verts, const double* xyz, int n_tris, const int* tris,
                                 double lambda, DeviceCRS& out, cudaStream_t s, bool* bad_input,
                                 bool check_indices) {
  *bad_input = false;
  DevBuf dx, dt;
  NLGB_CUDA_TRY(mesh_to_device(n_verts, xyz, n_tris, tris, dx, dt, s, bad_input, check_indices));
  if (*bad_input) return cudaSuccess;
  const long long n_edge_rows = 3LL * n_tris, n_rows = n_edge_rows + n_verts;
  const long long n_coefs = 2 * n_edge_rows + n_verts;
  DevBuf rp, col, val, w, xl, rhs;
  NLGB_CUDA_TRY(rp.alloc<long long>((size_t)n_rows + 1, s));
  NLGB_CUDA_TRY(col.alloc<int>((size_t)n_coefs, s));
  NLGB_CUDA_TRY(val.alloc<double>((size_t)n_coefs, s));
  NLGB_CUDA_TRY(w.alloc<double>((size_t)n_rows, s));
  NLGB_CUDA_TRY(xl.alloc<double>(1, s));
  NLGB_CUDA_TRY(rhs.alloc<double>((size_t)n_verts, s));
  NLGB_CUDA_TRY(cudaMemsetAsync(xl.p, 0, sizeof(double), s));
  k_row_ptr<<<grid_of(n_rows + 1, 256), 256, 0, s>>>(n_rows, n_edge_rows, 2, rp.as<long long>());
  count_launches(1);
  if (n_tris > 0) {
    k_cotan_rows<<<grid_of(n_edge_rows, 256), 256, 0, s>>>(n_tris, dx.as<double>(), dt.as<int>(),
                                                          col.as<int>(), val.as<double>(), w.as<double>());
    count_launches(1);
  }
  if (n_verts > 0) {
    k_diag_rows<<<grid_of(n_verts, 256), 256, 0, s>>>(n_verts, n_edge_rows, 2 * n_edge_rows, lambda,
                                                     col.as<int>(), val.as<double>(), w.as<double>());
    count_launches(1);
  }
  NLGB_CUDA_TRY(cudaGetLastError());
  LSRowsDevice R;
  R.n_rows = n_rows; R.n_coefs = n_coefs; R.n_free = n_verts; R.n_vars = n_verts; R.n_systems = 1;
  R.row_ptr = rp.as<long long>(); R.col = col.as<int>(); R.val = val.as<double>();
  R.rhs = nullptr; R.weight = w.as<double>(); R.xl = xl.as<double>();
  NLGB_CUDA_TRY(assemble_normal_equations(R, out, rhs.as<double>(), s));
  return cudaStreamSynchronize(s);
}

}  // namespace nlgb
