// nlgb_blas.cu -- FP64 BLAS-1 on the GPU behind OpenNL's NLBlas table
// (Dcopy/Dscal/Ddot/Dnrm2/Daxpy used by src/lib/OGF/scene_graph/NL/blas.cpp:
// 86,96,115,125,144).  Reductions are two-level with a fixed order.
#include "nlgb_internal.h"

#include <algorithm>

namespace nlgb {

namespace {
constexpr int kT = 256;
constexpr int kMaxBlocks = 1216;   // 152 SMs x 8

__global__ void k_dot_part(const double* __restrict__ x, const double* __restrict__ y, long long n,
                           double* part) {
  __shared__ double sh[kT / 32];
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)kT + threadIdx.x; i < n; i += (long long)gridDim.x * kT)
    s = fma(x[i], y[i], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kT / 32; ++w) t += sh[w];
    part[blockIdx.x] = t;
  }
}

__global__ void k_sum_parts(const double* part, int n, double* out) {
  __shared__ double sh[kT / 32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += kT) s += part[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kT / 32; ++w) t += sh[w];
    *out = t;
  }
}

__global__ void k_axpy(long long n, double a, const double* __restrict__ x, double* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)kT + threadIdx.x; i < n; i += (long long)gridDim.x * kT)
    y[i] = fma(a, x[i], y[i]);
}
__global__ void k_scal(long long n, double a, double* __restrict__ x) {
  for (long long i = blockIdx.x * (long long)kT + threadIdx.x; i < n; i += (long long)gridDim.x * kT)
    x[i] *= a;
}
__global__ void k_mul(long long n, const double* __restrict__ x, double* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)kT + threadIdx.x; i < n; i += (long long)gridDim.x * kT)
    y[i] *= x[i];
}
int blocks(long long n) { return (int)std::max(1LL, std::min<long long>((n + kT - 1) / kT, kMaxBlocks)); }

// BLAS addressing of element i of an n-vector with stride inc: i * inc for
// inc > 0, (n - 1 - i) * |inc| for inc < 0 (the vector is walked backwards
// from its last element).
__device__ __forceinline__ long long at(long long i, long long n, int inc) {
  return inc >= 0 ? i * inc : (n - 1 - i) * (long long)(-inc);
}

__global__ void k_dot_part_s(const double* __restrict__ x, int incx, const double* __restrict__ y, int incy,
                             long long n, double* part) {
  __shared__ double sh[kT / 32];
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)kT + threadIdx.x; i < n; i += (long long)gridDim.x * kT)
    s = fma(x[at(i, n, incx)], y[at(i, n, incy)], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kT / 32; ++w) t += sh[w];
    part[blockIdx.x] = t;
  }
}
__global__ void k_axpy_s(long long n, double a, const double* __restrict__ x, int incx, double* __restrict__ y,
                         int incy) {
  for (long long i = blockIdx.x * (long long)kT + threadIdx.x; i < n; i += (long long)gridDim.x * kT) {
    const long long j = at(i, n, incy);
    y[j] = fma(a, x[at(i, n, incx)], y[j]);
  }
}
__global__ void k_scal_s(long long n, double a, double* __restrict__ x, int incx) {
  for (long long i = blockIdx.x * (long long)kT + threadIdx.x; i < n; i += (long long)gridDim.x * kT)
    x[at(i, n, incx)] *= a;
}
__global__ void k_copy_s(long long n, const double* __restrict__ x, int incx, double* __restrict__ y, int incy) {
  for (long long i = blockIdx.x * (long long)kT + threadIdx.x; i < n; i += (long long)gridDim.x * kT)
    y[at(i, n, incy)] = x[at(i, n, incx)];
}
}  // namespace

// Strided forms (BLAS increments; x, y device pointers to the first element
// in memory of each strided vector).
cudaError_t dev_dot_s(const double* x, int incx, const double* y, int incy, long long n, double* out_host,
                      cudaStream_t s) {
  const int nb = blocks(n);
  double* part = nullptr;
  NLGB_CUDA_TRY(cudaMallocAsync(&part, sizeof(double) * (nb + 1), s));
  k_dot_part_s<<<nb, kT, 0, s>>>(x, incx, y, incy, n, part);
  count_launches(1);
  k_sum_parts<<<1, kT, 0, s>>>(part, nb, part + nb);
  count_launches(1);
  NLGB_CUDA_TRY(cudaGetLastError());
  NLGB_CUDA_TRY(cudaMemcpyAsync(out_host, part + nb, sizeof(double), cudaMemcpyDeviceToHost, s));
  NLGB_CUDA_TRY(cudaFreeAsync(part, s));
  NLGB_CUDA_TRY(cudaStreamSynchronize(s));
  return cudaSuccess;
}
cudaError_t dev_axpy_s(long long n, double a, const double* x, int incx, double* y, int incy, cudaStream_t s) {
  if (n > 0) {
    k_axpy_s<<<blocks(n), kT, 0, s>>>(n, a, x, incx, y, incy);
    count_launches(1);
  }
  return cudaGetLastError();
}
cudaError_t dev_scal_s(long long n, double a, double* x, int incx, cudaStream_t s) {
  if (n > 0) {
    k_scal_s<<<blocks(n), kT, 0, s>>>(n, a, x, incx);
    count_launches(1);
  }
  return cudaGetLastError();
}
cudaError_t dev_copy_s(long long n, const double* x, int incx, double* y, int incy, cudaStream_t s) {
  if (n > 0) {
    k_copy_s<<<blocks(n), kT, 0, s>>>(n, x, incx, y, incy);
    count_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t dev_dot(const double* x, const double* y, long long n, double* out_host, cudaStream_t s) {
  const int nb = blocks(n);
  double* part = nullptr;
  NLGB_CUDA_TRY(cudaMallocAsync(&part, sizeof(double) * (nb + 1), s));
  k_dot_part<<<nb, kT, 0, s>>>(x, y, n, part);
  count_launches(1);
  k_sum_parts<<<1, kT, 0, s>>>(part, nb, part + nb);
  count_launches(1);
  NLGB_CUDA_TRY(cudaGetLastError());
  NLGB_CUDA_TRY(cudaMemcpyAsync(out_host, part + nb, sizeof(double), cudaMemcpyDeviceToHost, s));
  NLGB_CUDA_TRY(cudaFreeAsync(part, s));
  NLGB_CUDA_TRY(cudaStreamSynchronize(s));
  return cudaSuccess;
}

cudaError_t dev_axpy(long long n, double a, const double* x, double* y, cudaStream_t s) {
  if (n > 0) {
    k_axpy<<<blocks(n), kT, 0, s>>>(n, a, x, y);
    count_launches(1);
  }
  return cudaGetLastError();
}
cudaError_t dev_scal(long long n, double a, double* x, cudaStream_t s) {
  if (n > 0) {
    k_scal<<<blocks(n), kT, 0, s>>>(n, a, x);
    count_launches(1);
  }
  return cudaGetLastError();
}
cudaError_t dev_mul(long long n, const double* x, double* y, cudaStream_t s) {
  if (n > 0) {
    k_mul<<<blocks(n), kT, 0, s>>>(n, x, y);
    count_launches(1);
  }
  return cudaGetLastError();
}

}  // namespace nlgb
