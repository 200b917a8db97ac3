// adjoint.cu -- transposed CRS and the sparse outer-product gradient.
//
// Transpose (set-up, once per matrix), all on the device:
//   1. count the entries of every column (atomics on int counters);
//   2. exclusive scan -> row pointers of K^T;
//   3. one thread per row of K scatters the ORIGINAL positions p of its
//      entries into the rows of K^T (arrival order inside a row is random);
//   4. every position q of K^T ranks its key p inside its row (the row found
//      by binary search on the row pointers): the keys of a row become sorted,
//      i.e. ascending row index of K -- deterministic, and the order of a
//      serial counting sort;
//   5. gather column indices (the row of p) and values.
// Step 4 costs O(L) per entry for a row of length L; the rows of K^T are the
// columns of K (7 for the stencil matrices, ~Poisson(12) for the PageRank
// matrix), so it stays a small fraction of the transpose.
//
// Gradient: one block per 256 consecutive rows; the block stages its row
// pointers and lambda in shared memory, expands the local row id of each of
// its nonzeros into shared memory (binary search instead when a block holds
// more than 4096 nonzeros), and its threads sweep the nonzeros in order
// (coalesced col_ind / grad traffic).
#include <stdexcept>
#include <vector>

#include "adjoint.h"

namespace idrs {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanPer = 4;
constexpr long kScanChunk = (long)kScanThreads * kScanPer;  // elements per scan block

__global__ void k_col_count(long nnz, const int* __restrict__ ci, int* __restrict__ cnt) {
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * (long)blockDim.x)
    atomicAdd(&cnt[ci[p]], 1);
}

// Exclusive scan of one chunk of kScanChunk ints per block; block totals to bsum.
__global__ void __launch_bounds__(kScanThreads) k_scan_chunk(long n, const int* __restrict__ in,
                                                             int* __restrict__ out,
                                                             int* __restrict__ bsum) {
  __shared__ int warp_tot[kScanThreads / 32];
  const long base = blockIdx.x * kScanChunk + (long)threadIdx.x * kScanPer;
  int v[kScanPer];
  int local = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    local += v[k];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = local;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  int woff = 0, total = 0;
  for (int w = 0; w < kScanThreads / 32; ++w) {
    if (w < wid) woff += warp_tot[w];
    total += warp_tot[w];
  }
  int run = woff + incl - local;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0 && bsum) bsum[blockIdx.x] = total;
}

__global__ void k_scan_add(long n, int* __restrict__ out, const int* __restrict__ boff) {
  const long i = blockIdx.x * kScanChunk + threadIdx.x;
  const int add = boff[blockIdx.x];
  for (long k = i; k < n && k < (blockIdx.x + 1) * kScanChunk; k += blockDim.x) out[k] += add;
}

// out[i] = sum_{k < i} in[k], i < n (device, ints; the sums must fit int32)
void exclusive_scan(long n, const int* in, int* out, cudaStream_t st) {
  const long blocks = (n + kScanChunk - 1) / kScanChunk;
  if (blocks <= 1) {
    k_scan_chunk<<<1, kScanThreads, 0, st>>>(n, in, out, nullptr);
    IDRS_LAUNCH_CHECK();
    return;
  }
  int *bsum = nullptr, *boff = nullptr;
  IDRS_CUDA(cudaMallocAsync((void**)&bsum, sizeof(int) * blocks, st));
  IDRS_CUDA(cudaMallocAsync((void**)&boff, sizeof(int) * blocks, st));
  k_scan_chunk<<<(unsigned)blocks, kScanThreads, 0, st>>>(n, in, out, bsum);
  IDRS_LAUNCH_CHECK();
  exclusive_scan(blocks, bsum, boff, st);
  k_scan_add<<<(unsigned)blocks, kScanThreads, 0, st>>>(n, out, boff);
  IDRS_LAUNCH_CHECK();
  IDRS_CUDA(cudaFreeAsync(bsum, st));
  IDRS_CUDA(cudaFreeAsync(boff, st));
}

__global__ void k_fill_rows(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                            const int* __restrict__ rpT, int* __restrict__ cursor,
                            int* __restrict__ keyT, int* __restrict__ rowidx) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int p = rp[i]; p < rp[i + 1]; ++p) {
      const int j = ci[p];
      keyT[rpT[j] + atomicAdd(&cursor[j], 1)] = p;
      rowidx[p] = i;
    }
}

// row of position q: largest r with rpT[r] <= q (rows may be empty)
__device__ inline int row_of(const int* __restrict__ rpT, int m, int q) {
  int lo = 0, hi = m;  // rpT[lo] <= q < rpT[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (rpT[mid] <= q) lo = mid; else hi = mid;
  }
  return lo;
}

__global__ void k_rank_sort(long nnz, int m, const int* __restrict__ rpT, const int* __restrict__ keyT,
                            int* __restrict__ keyS) {
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < nnz; q += gridDim.x * (long)blockDim.x) {
    const int r = row_of(rpT, m, (int)q);
    const int a = rpT[r], b = rpT[r + 1];
    const int key = keyT[q];
    int rank = 0;
    for (int t = a; t < b; ++t) rank += (keyT[t] < key);
    keyS[a + rank] = key;
  }
}

template <class V>
__global__ void k_gather_T(long nnz, const int* __restrict__ keyS, const int* __restrict__ rowidx,
                           const V* __restrict__ val, int* __restrict__ ciT, V* __restrict__ valT) {
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < nnz; q += gridDim.x * (long)blockDim.x) {
    const int p = keyS[q];
    ciT[q] = rowidx[p];
    if (valT) valT[q] = val[p];
  }
}

constexpr int kGradRows = 256;
constexpr int kGradMaxNnz = 4096;  // nonzeros of a block whose local row ids fit in shared memory

__global__ void __launch_bounds__(kGradRows) k_outer_grad(int n, const int* __restrict__ rp,
                                                          const int* __restrict__ ci,
                                                          const double* __restrict__ lambda,
                                                          const double* __restrict__ x,
                                                          double* __restrict__ grad) {
  __shared__ int srp[kGradRows + 1];
  __shared__ double slam[kGradRows];
  __shared__ unsigned char srow[kGradMaxNnz];  // local row (< 256) of each nonzero
  const int r0 = blockIdx.x * kGradRows;
  const int rows = min(kGradRows, n - r0);
  for (int t = threadIdx.x; t <= rows; t += blockDim.x) srp[t] = rp[r0 + t];
  for (int t = threadIdx.x; t < rows; t += blockDim.x) slam[t] = lambda[r0 + t];
  __syncthreads();
  const int p0 = srp[0], p1 = srp[rows];
  if (p1 - p0 <= kGradMaxNnz) {  // uniform over the block
    for (int t = threadIdx.x; t < rows; t += blockDim.x)
      for (int q = srp[t]; q < srp[t + 1]; ++q) srow[q - p0] = (unsigned char)t;
    __syncthreads();
#pragma unroll 4
    for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) grad[p] = -slam[srow[p - p0]] * x[ci[p]];
    return;
  }
  for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    int lo = 0, hi = rows;  // srp[lo] <= p < srp[hi]
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (srp[mid] <= p) lo = mid; else hi = mid;
    }
    grad[p] = -slam[lo] * x[ci[p]];
  }
}

}  // namespace

void crs_transpose(const UserMatrix& K, UserMatrix& Tm, cudaStream_t st) {
  if (K.format != FMT_CRS) throw std::runtime_error("crs_transpose: CRS matrix required");
  if (K.nnz > 2147483647L) throw std::runtime_error("crs_transpose: nnz exceeds int32");
  const int n = K.nrows, m = K.ncols;
  const long nnz = K.nnz;
  UserMatrix* T = &Tm;
  T->format = FMT_CRS;
  T->nrows = m;
  T->ncols = n;
  T->nnz = nnz;
  T->vals = K.vals;
  T->group = K.group;
  const size_t vs = (K.vals == 2) ? 16 : 8;
  int *cnt = nullptr, *cursor = nullptr, *keyT = nullptr, *keyS = nullptr, *rowidx = nullptr;
  try {
    IDRS_CUDA(cudaMalloc((void**)&T->row_ptr, sizeof(int) * (m + 1)));
    IDRS_CUDA(cudaMalloc((void**)&T->col_ind, sizeof(int) * std::max<long>(nnz, 1)));
    if (K.vals != 0) IDRS_CUDA(cudaMalloc(&T->val, vs * std::max<long>(nnz, 1)));
    IDRS_CUDA(cudaMallocAsync((void**)&cnt, sizeof(int) * (m + 1), st));
    IDRS_CUDA(cudaMallocAsync((void**)&cursor, sizeof(int) * std::max(m, 1), st));
    IDRS_CUDA(cudaMallocAsync((void**)&keyT, sizeof(int) * std::max<long>(nnz, 1), st));
    IDRS_CUDA(cudaMallocAsync((void**)&keyS, sizeof(int) * std::max<long>(nnz, 1), st));
    IDRS_CUDA(cudaMallocAsync((void**)&rowidx, sizeof(int) * std::max<long>(nnz, 1), st));
    IDRS_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (m + 1), st));
    IDRS_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int) * std::max(m, 1), st));
    const int g = stream_grid(std::max<long>(nnz, 1));
    if (nnz > 0) {
      k_col_count<<<g, kThreads, 0, st>>>(nnz, K.col_ind, cnt);
      IDRS_LAUNCH_CHECK();
    }
    exclusive_scan(m + 1, cnt, T->row_ptr, st);
    if (nnz > 0) {
      k_fill_rows<<<stream_grid(std::max(n, 1)), kThreads, 0, st>>>(n, K.row_ptr, K.col_ind, T->row_ptr,
                                                                    cursor, keyT, rowidx);
      IDRS_LAUNCH_CHECK();
      k_rank_sort<<<g, kThreads, 0, st>>>(nnz, m, T->row_ptr, keyT, keyS);
      IDRS_LAUNCH_CHECK();
      if (K.vals == 2)
        k_gather_T<c128><<<g, kThreads, 0, st>>>(nnz, keyS, rowidx, (const c128*)K.val, T->col_ind, (c128*)T->val);
      else if (K.vals == 1)
        k_gather_T<double><<<g, kThreads, 0, st>>>(nnz, keyS, rowidx, (const double*)K.val, T->col_ind, (double*)T->val);
      else
        k_gather_T<double><<<g, kThreads, 0, st>>>(nnz, keyS, rowidx, nullptr, T->col_ind, nullptr);
      IDRS_LAUNCH_CHECK();
    }
    for (int* p : {cnt, cursor, keyT, keyS, rowidx}) IDRS_CUDA(cudaFreeAsync(p, st));
    IDRS_CUDA(cudaStreamSynchronize(st));
    std::vector<int> rp_host(m + 1);
    IDRS_CUDA(cudaMemcpy(rp_host.data(), T->row_ptr, sizeof(int) * (m + 1), cudaMemcpyDeviceToHost));
    build_row_plan(*T, rp_host.data());
  } catch (...) {
    for (int* p : {cnt, cursor, keyT, keyS, rowidx})
      if (p) cudaFreeAsync(p, st);
    cudaFree(T->row_ptr); cudaFree(T->col_ind); cudaFree(T->val);
    cudaFree(T->med_rows); cudaFree(T->long_rows); cudaFree(T->seg_ptr); cudaFree(T->partial);
    T->row_ptr = T->col_ind = T->med_rows = T->long_rows = T->seg_ptr = nullptr;
    T->val = T->partial = nullptr;
    T->n_med = T->n_long = T->n_seg = T->bin_short = 0;
    throw;
  }
}

void sparse_outer_grad(const UserMatrix& K, const double* lambda, const double* x, double* grad,
                       cudaStream_t st) {
  if (K.format != FMT_CRS) throw std::runtime_error("sparse_outer_grad: CRS matrix required");
  if (K.vals == 2) throw std::runtime_error("sparse_outer_grad: real values required");
  if (K.nrows == 0 || K.nnz == 0) return;
  const int blocks = (K.nrows + kGradRows - 1) / kGradRows;
  k_outer_grad<<<blocks, kGradRows, 0, st>>>(K.nrows, K.row_ptr, K.col_ind, lambda, x, grad);
  IDRS_LAUNCH_CHECK();
}

}  // namespace idrs
