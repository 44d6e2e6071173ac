// nlgb_assembly.cu -- OpenNL system assembly on the GPU.
//
// Least-squares mode (nlSolverParameteri(NL_LEAST_SQUARES, NL_TRUE), used at
// plugins/OGF/WarpDrive/commands/voxel_grob_transport_commands.cpp:232 and by
// geogram's LSCM builder behind mesh_grob_surface_commands.cpp:759): every
// row r (coefficients a_r, right-hand side b_r, weight w_r) contributes
// w_r a_r,f a_r,f^T to the normal matrix over the free variables and
// w_r a_r,f (b_r - a_r,l . x_l) to its right-hand side.
//
// GPU row-merge: (1) per LS row, s_r = b_r - sum_locked a x (coefficient
// order); (2) transpose the free coefficients into per-variable column lists;
// (3) for each output row i, merge the rows that contain i: candidates
// (j, r) -> (w a_ri) a_rj are sorted by (j, r) in shared memory and each run
// of equal j is summed sequentially in ascending r.  The sum order is exactly
// that of a sequential row-by-row CPU build, and products and sums use
// explicitly rounded intrinsics (no FMA contraction), so the assembled
// matrix and right-hand side are bit-identical to the CPU oracle's.
#include "nlgb_internal.h"

#include <algorithm>
#include <cstdint>
#include <cstdio>

namespace nlgb {

namespace {

constexpr int kWarpCap = 256;    // candidates per output row, warp path
constexpr int kBlockCap = 4096;  // candidates per output row, CTA path
constexpr int kAsmCTA = 256;

// ---- (1) per-row reduced right-hand side and free-coefficient count ----
__global__ void k_rows_prepare(LSRowsDevice R, double* __restrict__ s, int* __restrict__ nfree) {
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= R.n_rows) return;
  const long long k0 = R.row_ptr[r], k1 = R.row_ptr[r + 1];
  int nf = 0;
  for (long long k = k0; k < k1; ++k) nf += (R.col[k] >= 0);
  nfree[r] = nf;
  for (int sys = 0; sys < R.n_systems; ++sys) {
    double acc = R.rhs ? R.rhs[(size_t)sys * R.n_rows + r] : 0.0;
    for (long long k = k0; k < k1; ++k) {
      const int c = R.col[k];
      if (c < 0) {
        const int var = -c - 1;
        acc = __dsub_rn(acc, __dmul_rn(R.val[k], R.xl[(size_t)sys * R.n_vars + var]));
      }
    }
    s[(size_t)sys * R.n_rows + r] = acc;
  }
}

// ---- (2) column counts, then scatter into column lists ----
__global__ void k_col_count(LSRowsDevice R, int* __restrict__ colcnt) {
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= R.n_rows) return;
  for (long long k = R.row_ptr[r]; k < R.row_ptr[r + 1]; ++k) {
    const int c = R.col[k];
    if (c >= 0) atomicAdd(colcnt + c, 1);
  }
}

__global__ void k_col_scatter(LSRowsDevice R, const long long* __restrict__ colptr,
                              int* __restrict__ cursor, int* __restrict__ colrow,
                              double* __restrict__ colwa) {
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= R.n_rows) return;
  const double w = R.weight ? R.weight[r] : 1.0;
  for (long long k = R.row_ptr[r]; k < R.row_ptr[r + 1]; ++k) {
    const int c = R.col[k];
    if (c >= 0) {
      const long long pos = colptr[c] + atomicAdd(cursor + c, 1);
      colrow[pos] = (int)r;
      colwa[pos] = __dmul_rn(w, R.val[k]);
    }
  }
}

// ---- (3a) candidate count per output row ----
__global__ void k_cand_count(int n_free, const long long* __restrict__ colptr,
                             const int* __restrict__ colrow, const int* __restrict__ nfree,
                             int* __restrict__ cand) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_free) return;
  long long c = 0;
  for (long long e = colptr[i]; e < colptr[i + 1]; ++e) c += nfree[colrow[e]];
  cand[i] = (int)(c < (1LL << 30) ? c : (1LL << 30));
}

// ---- (3b) merge: shared-memory sort of (j, r) candidates ----
struct MergeArgs {
  LSRowsDevice R;
  int n_free;
  const long long* colptr;
  const int* colrow;
  const double* colwa;
  const int* nfree;
  const double* s;       // n_systems * n_rows
  const int* cand;
  const int* rows;       // output rows handled by this launch (null: all)
  int n_rows_list;
  int* row_nnz;          // symbolic output
  const int* rp;         // numeric: CRS row pointers
  int* ci;
  double* va;
  double* rhs;           // n_systems * n_free
  int numeric;
  int* err;              // set to 1 when a row exceeds the CTA cap
};

// Exclusive scan of v over a group of G threads (G == 32: one warp,
// G == kAsmCTA: the whole CTA, which then must call it uniformly).
template <int G>
__device__ __forceinline__ int group_excl_scan(int v, int g, int* total) {
  if constexpr (G == 32) {
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, inc, o);
      if (g >= o) inc += t;
    }
    *total = __shfl_sync(0xffffffffu, inc, 31);
    return inc - v;
  } else {
    __shared__ int sh[G];
    __syncthreads();
    sh[g] = v;
    __syncthreads();
    for (int o = 1; o < G; o <<= 1) {
      const int t = g >= o ? sh[g - o] : 0;
      __syncthreads();
      sh[g] += t;
      __syncthreads();
    }
    *total = sh[G - 1];
    return sh[g] - v;
  }
}

// Fill the candidates of output row i into shared memory (group of G
// threads, lane g).  The fill order is irrelevant: keys (j, r) are unique
// and sorted afterwards.  For G == 32 the loop is warp-uniform; for
// G == kAsmCTA it is CTA-uniform.
template <int G>
__device__ int fill_candidates(const MergeArgs& A, int i, bool active, unsigned long long* key,
                               double* val, double* aux, int g, int cap) {
  const long long e0 = active ? A.colptr[i] : 0, e1 = active ? A.colptr[i + 1] : 0;
  int running = 0;
  for (long long eb = e0; eb < e1; eb += G) {
    const long long e = eb + g;
    int r = 0, cnt = 0;
    double wa = 0.0;
    if (e < e1) { r = A.colrow[e]; wa = A.colwa[e]; cnt = A.nfree[r]; }
    int tot = 0;
    const int off = group_excl_scan<G>(cnt, g, &tot);
    int slot = running + off;
    if (e < e1) {
      const long long k0 = A.R.row_ptr[r], k1 = A.R.row_ptr[r + 1];
      for (long long k = k0; k < k1; ++k) {
        const int j = A.R.col[k];
        if (j < 0) continue;
        if (slot < cap) {
          key[slot] = ((unsigned long long)(unsigned)j << 32) | (unsigned)r;
          val[slot] = __dmul_rn(wa, A.R.val[k]);
          aux[slot] = wa;
        }
        ++slot;
      }
    }
    running += tot;
  }
  return running;
}

template <int G>
__device__ void bitonic(unsigned long long* key, double* val, double* aux, int P, int g) {
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = g; t < P; t += G) {
        const int ixj = t ^ j;
        if (ixj > t) {
          const bool up = (t & k) == 0;
          const unsigned long long a = key[t], b = key[ixj];
          if ((a > b) == up) {
            key[t] = b; key[ixj] = a;
            const double v = val[t]; val[t] = val[ixj]; val[ixj] = v;
            const double x = aux[t]; aux[t] = aux[ixj]; aux[ixj] = x;
          }
        }
      }
      __syncthreads();
    }
  }
}

// One output row per CTA-sized group (G = kAsmCTA threads) -- used for both
// paths; the warp path packs 8 rows per CTA with G = 32.
template <int G, int CAP>
__global__ void __launch_bounds__(kAsmCTA) k_merge(MergeArgs A) {
  extern __shared__ unsigned char smem_raw[];
  constexpr int kGroups = kAsmCTA / G;
  const int grp = threadIdx.x / G, g = threadIdx.x % G;
  unsigned long long* key = reinterpret_cast<unsigned long long*>(smem_raw) + (size_t)grp * CAP;
  double* val = reinterpret_cast<double*>(smem_raw + sizeof(unsigned long long) * CAP * kGroups) +
                (size_t)grp * CAP;
  double* aux = reinterpret_cast<double*>(smem_raw + (sizeof(unsigned long long) + sizeof(double)) *
                                                         CAP * kGroups) +
                (size_t)grp * CAP;
  __shared__ int heads_cnt[kGroups];
  const long long idx = (long long)blockIdx.x * kGroups + grp;
  const long long total = A.rows ? A.n_rows_list : A.n_free;
  const bool active = idx < total;
  const int i = active ? (A.rows ? A.rows[idx] : (int)idx) : 0;
  const bool mine = active && (A.rows != nullptr || A.cand[i] <= CAP);
  // All threads take part in fills/sorts (they contain __syncthreads); an
  // inactive group fills nothing.
  int cnt = fill_candidates<G>(A, i, mine, key, val, aux, g, CAP);
  if (mine && cnt > CAP && g == 0) atomicExch(A.err, 1);
  if (cnt > CAP) cnt = 0;
  int P = 1;
  while (P < cnt) P <<= 1;
  for (int t = cnt + g; t < P; t += G) key[t] = ~0ULL;
  __syncthreads();
  // Largest P over groups so every thread runs the same barrier sequence.
  __shared__ int pmax;
  if (threadIdx.x == 0) pmax = 1;
  __syncthreads();
  atomicMax(&pmax, P);
  __syncthreads();
  const int Pall = pmax;
  for (int t = P + g; t < Pall; t += G) key[t] = ~0ULL;
  __syncthreads();
  bitonic<G>(key, val, aux, Pall, g);
  // Run heads.
  if (g == 0) heads_cnt[grp] = 0;
  __syncthreads();
  int local_heads = 0;
  for (int t = g; t < cnt; t += G) {
    const bool head = (t == 0) || ((key[t] >> 32) != (key[t - 1] >> 32));
    local_heads += head;
  }
  if (local_heads) atomicAdd(&heads_cnt[grp], local_heads);
  __syncthreads();
  if (!mine) return;
  if (!A.numeric) {
    if (g == 0) A.row_nnz[i] = heads_cnt[grp];
    return;
  }
  // Numeric: output slot of a head = number of heads before it (sequential
  // by lane g == 0 is simplest and rows are short).
  if (g == 0) {
    int out = A.rp[i];
    for (int t = 0; t < cnt;) {
      const unsigned j = (unsigned)(key[t] >> 32);
      double v = 0.0;
      int t2 = t;
      while (t2 < cnt && (unsigned)(key[t2] >> 32) == j) { v = __dadd_rn(v, val[t2]); ++t2; }
      A.ci[out] = (int)j;
      A.va[out] = v;
      ++out;
      if ((int)j == i) {
        for (int sys = 0; sys < A.R.n_systems; ++sys) {
          double acc = 0.0;
          for (int u = t; u < t2; ++u) {
            const unsigned r = (unsigned)(key[u] & 0xffffffffULL);
            acc = __dadd_rn(acc, __dmul_rn(aux[u], A.s[(size_t)sys * A.R.n_rows + r]));
          }
          A.rhs[(size_t)sys * A.n_free + i] = acc;
        }
      }
      t = t2;
    }
  }
}

// Rows whose candidates exceed the warp cap (compacted list).
__global__ void k_collect_big(int n_free, const int* cand, int cap, int* list, int* count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_free && cand[i] > cap) list[atomicAdd(count, 1)] = i;
}

// Rows with no candidates still need an RHS of 0 (and no entries).
__global__ void k_zero(double* p, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    p[i] = 0.0;
}

// ---- exclusive scan (int -> long long), three-phase ----
constexpr int kScanItems = 8;
constexpr int kScanTile = kAsmCTA * kScanItems;

template <typename In>
__global__ void k_scan_tiles(const In* __restrict__ in, long long n, long long* __restrict__ out,
                             long long* __restrict__ tile_sums) {
  __shared__ long long sh[kAsmCTA];
  const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  long long v[kScanItems];
  long long s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const long long i = base + k;
    v[k] = i < n ? (long long)in[i] : 0;
    s += v[k];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < kAsmCTA; o <<= 1) {
    const long long t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  long long run = sh[threadIdx.x] - s;   // exclusive prefix of this thread
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const long long i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
  if (threadIdx.x == kAsmCTA - 1) tile_sums[blockIdx.x] = sh[threadIdx.x];
}

__global__ void k_scan_add(long long* out, long long n, const long long* __restrict__ tile_off) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] += tile_off[i / kScanTile];
}

template <typename In>
cudaError_t exclusive_scan(const In* in, long long n, long long* out, long long* total,
                           cudaStream_t s) {
  // out[0..n) = exclusive prefix sums; *total (host) = sum.
  const long long tiles = std::max(1LL, (n + kScanTile - 1) / kScanTile);
  long long* sums = nullptr;
  long long* offs = nullptr;
  NLGB_CUDA_TRY(cudaMallocAsync(&sums, (size_t)tiles * sizeof(long long), s));
  NLGB_CUDA_TRY(cudaMallocAsync(&offs, (size_t)(tiles + 1) * sizeof(long long), s));
  if (n > 0) {
    k_scan_tiles<In><<<(unsigned)tiles, kAsmCTA, 0, s>>>(in, n, out, sums);
    count_launches(1);
  }
  NLGB_CUDA_TRY(cudaGetLastError());
  long long tot = 0;
  if (tiles > 1) {
    long long t2 = 0;
    NLGB_CUDA_TRY(exclusive_scan<long long>(sums, tiles, offs, &t2, s));
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, n, offs);
    count_launches(1);
    NLGB_CUDA_TRY(cudaGetLastError());
    tot = t2;
  } else {
    if (n > 0) NLGB_CUDA_TRY(cudaMemcpyAsync(&tot, sums, sizeof(long long), cudaMemcpyDeviceToHost, s));
    NLGB_CUDA_TRY(cudaStreamSynchronize(s));
  }
  NLGB_CUDA_TRY(cudaFreeAsync(sums, s));
  NLGB_CUDA_TRY(cudaFreeAsync(offs, s));
  *total = tot;
  return cudaSuccess;
}

__global__ void k_to_int(const long long* in, int* out, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (int)in[i];
}

inline unsigned blocks_for(long long n, int t = 256) { return (unsigned)std::max(1LL, (n + t - 1) / t); }

template <typename T>
struct DevBuf {
  T* p = nullptr;
  cudaStream_t s = nullptr;
  cudaError_t alloc(size_t n, cudaStream_t st) {
    s = st;
    return cudaMallocAsync(&p, std::max<size_t>(1, n) * sizeof(T), st);
  }
  ~DevBuf() { if (p) cudaFreeAsync(p, s); }
};

}  // namespace

cudaError_t assemble_normal_equations(const LSRowsDevice& R, DeviceCRS& out, double* rhs_out,
                                      cudaStream_t s) {
  const int nf = R.n_free;
  if (R.n_rows >= (1LL << 31) - 1) {
    set_error("least-squares assembly: more than 2^31-1 rows");
    return cudaErrorInvalidValue;
  }
  DevBuf<double> sbuf; DevBuf<int> nfree, colcnt, cursor, colrow, cand, row_nnz, big, big_n, err;
  DevBuf<long long> colptr, rp64;
  DevBuf<double> colwa;
  NLGB_CUDA_TRY(sbuf.alloc((size_t)R.n_systems * R.n_rows, s));
  NLGB_CUDA_TRY(nfree.alloc(R.n_rows, s));
  NLGB_CUDA_TRY(colcnt.alloc(nf + 1, s));
  NLGB_CUDA_TRY(cursor.alloc(nf + 1, s));
  NLGB_CUDA_TRY(colptr.alloc(nf + 1, s));
  NLGB_CUDA_TRY(cudaMemsetAsync(colcnt.p, 0, sizeof(int) * (nf + 1), s));
  NLGB_CUDA_TRY(cudaMemsetAsync(cursor.p, 0, sizeof(int) * (nf + 1), s));
  if (R.n_rows > 0) {
    k_rows_prepare<<<blocks_for(R.n_rows), 256, 0, s>>>(R, sbuf.p, nfree.p);
    count_launches(1);
    k_col_count<<<blocks_for(R.n_rows), 256, 0, s>>>(R, colcnt.p);
    count_launches(1);
  }
  NLGB_CUDA_TRY(cudaGetLastError());
  long long n_free_coefs = 0;
  NLGB_CUDA_TRY(exclusive_scan<int>(colcnt.p, nf + 1, colptr.p, &n_free_coefs, s));
  NLGB_CUDA_TRY(colrow.alloc(n_free_coefs, s));
  NLGB_CUDA_TRY(colwa.alloc(n_free_coefs, s));
  if (R.n_rows > 0) {
    k_col_scatter<<<blocks_for(R.n_rows), 256, 0, s>>>(R, colptr.p, cursor.p, colrow.p, colwa.p);
    count_launches(1);
  }
  NLGB_CUDA_TRY(cand.alloc(nf + 1, s));
  NLGB_CUDA_TRY(row_nnz.alloc(nf + 1, s));
  NLGB_CUDA_TRY(big.alloc(nf + 1, s));
  NLGB_CUDA_TRY(big_n.alloc(1, s));
  NLGB_CUDA_TRY(err.alloc(1, s));
  NLGB_CUDA_TRY(cudaMemsetAsync(big_n.p, 0, sizeof(int), s));
  NLGB_CUDA_TRY(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  NLGB_CUDA_TRY(cudaMemsetAsync(row_nnz.p, 0, sizeof(int) * (nf + 1), s));
  if (nf > 0) {
    k_cand_count<<<blocks_for(nf), 256, 0, s>>>(nf, colptr.p, colrow.p, nfree.p, cand.p);
    count_launches(1);
    k_collect_big<<<blocks_for(nf), 256, 0, s>>>(nf, cand.p, kWarpCap, big.p, big_n.p);
    count_launches(1);
  }
  NLGB_CUDA_TRY(cudaGetLastError());
  int n_big = 0;
  NLGB_CUDA_TRY(cudaMemcpyAsync(&n_big, big_n.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  NLGB_CUDA_TRY(cudaStreamSynchronize(s));

  MergeArgs M;
  M.R = R; M.n_free = nf; M.colptr = colptr.p; M.colrow = colrow.p; M.colwa = colwa.p;
  M.nfree = nfree.p; M.s = sbuf.p; M.cand = cand.p; M.row_nnz = row_nnz.p; M.err = err.p;
  M.rp = nullptr; M.ci = nullptr; M.va = nullptr; M.rhs = rhs_out; M.numeric = 0;
  constexpr int kWarpGroups = kAsmCTA / 32;
  const size_t smem_warp = (size_t)kWarpCap * kWarpGroups * 24;
  const size_t smem_block = (size_t)kBlockCap * 24;
  NLGB_CUDA_TRY(cudaFuncSetAttribute(k_merge<32, kWarpCap>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_warp));
  NLGB_CUDA_TRY(cudaFuncSetAttribute(k_merge<kAsmCTA, kBlockCap>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_block));
  auto run_merge = [&](int numeric) -> cudaError_t {
    M.numeric = numeric;
    M.rows = nullptr; M.n_rows_list = 0;
    if (nf > 0) {
      k_merge<32, kWarpCap><<<blocks_for(nf, kWarpGroups), kAsmCTA, smem_warp, s>>>(M);
      count_launches(1);
    }
    NLGB_CUDA_TRY(cudaGetLastError());
    if (n_big > 0) {
      M.rows = big.p; M.n_rows_list = n_big;
      k_merge<kAsmCTA, kBlockCap><<<(unsigned)n_big, kAsmCTA, smem_block, s>>>(M);
      count_launches(1);
      NLGB_CUDA_TRY(cudaGetLastError());
    }
    return cudaSuccess;
  };
  NLGB_CUDA_TRY(run_merge(0));
  int herr = 0;
  NLGB_CUDA_TRY(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  NLGB_CUDA_TRY(rp64.alloc(nf + 1, s));
  long long nnz = 0;
  NLGB_CUDA_TRY(exclusive_scan<int>(row_nnz.p, nf + 1, rp64.p, &nnz, s));
  if (herr) {
    set_error("least-squares assembly: a variable's normal-equation row merges more than 4096 "
              "coefficients (rows too dense for the GPU row-merge)");
    return cudaErrorInvalidValue;
  }
  if (nnz >= (1LL << 31) - 1) {
    set_error("least-squares assembly: normal matrix has more than 2^31-1 nonzeros");
    return cudaErrorInvalidValue;
  }
  crs_free(out);
  out.n = nf; out.m = nf; out.nnz = nnz;
  NLGB_CUDA_TRY(cudaMallocAsync(&out.rp, sizeof(int) * (nf + 1), s));
  NLGB_CUDA_TRY(cudaMallocAsync(&out.ci, sizeof(int) * std::max(1LL, nnz), s));
  NLGB_CUDA_TRY(cudaMallocAsync(&out.va, sizeof(double) * std::max(1LL, nnz), s));
  k_to_int<<<blocks_for(nf + 1), 256, 0, s>>>(rp64.p, out.rp, nf + 1);
  count_launches(1);
  NLGB_CUDA_TRY(cudaGetLastError());
  // RHS of variables without any row stays 0.
  k_zero<<<blocks_for((long long)R.n_systems * nf), 256, 0, s>>>(rhs_out, (long long)R.n_systems * nf);
  count_launches(1);
  M.rp = out.rp; M.ci = out.ci; M.va = out.va;
  NLGB_CUDA_TRY(run_merge(1));
  NLGB_CUDA_TRY(cudaStreamSynchronize(s));
  return cudaSuccess;
}

namespace {
__global__ void k_square_count(LSRowsDevice R, int* cnt) {
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= R.n_rows) return;
  int c = 0;
  for (long long k = R.row_ptr[r]; k < R.row_ptr[r + 1]; ++k) c += R.col[k] >= 0;
  cnt[r] = c;
}
__global__ void k_square_fill(LSRowsDevice R, const long long* rp64, int* ci, double* va,
                              const double* s, double* rhs) {
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= R.n_rows) return;
  long long o = rp64[r];
  for (long long k = R.row_ptr[r]; k < R.row_ptr[r + 1]; ++k) {
    const int c = R.col[k];
    if (c >= 0) { ci[o] = c; va[o] = R.val[k]; ++o; }
  }
  for (int sys = 0; sys < R.n_systems; ++sys)
    rhs[(size_t)sys * R.n_rows + r] = s[(size_t)sys * R.n_rows + r];
}
}  // namespace

cudaError_t assemble_square(const LSRowsDevice& R, DeviceCRS& out, double* rhs_out, cudaStream_t s) {
  const long long n = R.n_rows;
  if (n != R.n_free) {
    set_error("square system: the number of rows must equal the number of free variables");
    return cudaErrorInvalidValue;
  }
  DevBuf<double> sbuf; DevBuf<int> nfree, cnt; DevBuf<long long> rp64;
  NLGB_CUDA_TRY(sbuf.alloc((size_t)R.n_systems * n, s));
  NLGB_CUDA_TRY(nfree.alloc(n, s));
  NLGB_CUDA_TRY(cnt.alloc(n + 1, s));
  NLGB_CUDA_TRY(rp64.alloc(n + 1, s));
  NLGB_CUDA_TRY(cudaMemsetAsync(cnt.p, 0, sizeof(int) * (n + 1), s));
  if (n > 0) {
    k_rows_prepare<<<blocks_for(n), 256, 0, s>>>(R, sbuf.p, nfree.p);
    count_launches(1);
    k_square_count<<<blocks_for(n), 256, 0, s>>>(R, cnt.p);
    count_launches(1);
  }
  NLGB_CUDA_TRY(cudaGetLastError());
  long long nnz = 0;
  NLGB_CUDA_TRY(exclusive_scan<int>(cnt.p, n + 1, rp64.p, &nnz, s));
  if (nnz >= (1LL << 31) - 1) {
    set_error("square system: more than 2^31-1 nonzeros");
    return cudaErrorInvalidValue;
  }
  crs_free(out);
  out.n = (int)n; out.m = (int)n; out.nnz = nnz;
  NLGB_CUDA_TRY(cudaMallocAsync(&out.rp, sizeof(int) * (n + 1), s));
  NLGB_CUDA_TRY(cudaMallocAsync(&out.ci, sizeof(int) * std::max(1LL, nnz), s));
  NLGB_CUDA_TRY(cudaMallocAsync(&out.va, sizeof(double) * std::max(1LL, nnz), s));
  k_to_int<<<blocks_for(n + 1), 256, 0, s>>>(rp64.p, out.rp, n + 1);
  count_launches(1);
  if (n > 0) {
    k_square_fill<<<blocks_for(n), 256, 0, s>>>(R, rp64.p, out.ci, out.va, sbuf.p, rhs_out);
    count_launches(1);
  }
  NLGB_CUDA_TRY(cudaGetLastError());
  NLGB_CUDA_TRY(cudaStreamSynchronize(s));
  return cudaSuccess;
}

}  // namespace nlgb
