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
}  // namespace

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
