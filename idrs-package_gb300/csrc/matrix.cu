// matrix.cu -- SpMV kernels (stencil, CRS, CDS, dense), the scaled operator
// build and the Horner chain of the polynomial preconditioner.
#include <algorithm>
#include <cstdlib>
#include <climits>
#include <atomic>
#include <mutex>

#include "matrix.cuh"
#include "stencil.cuh"
#include "tma.cuh"

namespace idrs {

// ---------------------------------------------------------------------------
// runtime basics
// ---------------------------------------------------------------------------
static thread_local std::string g_error;
static std::atomic<long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void uncount_launches(long k) { g_launches.fetch_sub(k, std::memory_order_relaxed); }
long launch_count() { return g_launches.load(std::memory_order_relaxed); }
bool pdl_enabled() {
  static const bool on = [] {
    const char* e = getenv("IDRS_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}
void set_error(const std::string& msg) { g_error = msg; }
const char* last_error() { return g_error.c_str(); }

int num_sms() {
  static int sms = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
      sms = 152;
  });
  return sms;
}

RedBuf alloc_redbuf(cudaStream_t st) {
  RedBuf rb{nullptr, nullptr};
  IDRS_CUDA(cudaMallocAsync((void**)&rb.ticket, sizeof(unsigned int) * 32, st));
  IDRS_CUDA(cudaMemsetAsync(rb.ticket, 0, sizeof(unsigned int) * 32, st));
  IDRS_CUDA(cudaMallocAsync(&rb.partials, (size_t)kMaxRedBlocks * kMaxND * sizeof(c128), st));
  return rb;
}
void free_redbuf(RedBuf rb, cudaStream_t st) {
  if (rb.ticket) cudaFreeAsync(rb.ticket, st);
  if (rb.partials) cudaFreeAsync(rb.partials, st);
}

// ---------------------------------------------------------------------------
// small generic helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double shfl_x(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ float shfl_x(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ c128 shfl_x(c128 v, int m) { return c128(shfl_x(v.x, m), shfl_x(v.y, m)); }
__device__ __forceinline__ c64 shfl_x(c64 v, int m) { return c64(shfl_x(v.x, m), shfl_x(v.y, m)); }
__device__ __forceinline__ double shfl_up_t(double v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
__device__ __forceinline__ float shfl_up_t(float v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
__device__ __forceinline__ c128 shfl_up_t(c128 v, int d) { return c128(shfl_up_t(v.x, d), shfl_up_t(v.y, d)); }
__device__ __forceinline__ c64 shfl_up_t(c64 v, int d) { return c64(shfl_up_t(v.x, d), shfl_up_t(v.y, d)); }
__device__ __forceinline__ double shfl_idx_t(double v, int l) { return __shfl_sync(0xffffffffu, v, l); }
__device__ __forceinline__ float shfl_idx_t(float v, int l) { return __shfl_sync(0xffffffffu, v, l); }
__device__ __forceinline__ c128 shfl_idx_t(c128 v, int l) { return c128(shfl_idx_t(v.x, l), shfl_idx_t(v.y, l)); }
__device__ __forceinline__ c64 shfl_idx_t(c64 v, int l) { return c64(shfl_idx_t(v.x, l), shfl_idx_t(v.y, l)); }

template <class V, class T> __device__ __forceinline__ T mulvt(V a, T b) { return a * b; }

// Matrix values and column indices are read once per product.  Where a
// warp consumes every line it loads in one instruction (the long-row
// segments), evict-first loads (ld.global.cs) keep them from displacing the
// gathered vector x from L2; the row kernels re-read a line across their
// loop steps and load normally (evict-first measured slower there).
__device__ __forceinline__ double ld_stream(const double* p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float* p) { return __ldcs(p); }
__device__ __forceinline__ int ld_stream(const int* p) { return __ldcs(p); }
__device__ __forceinline__ c128 ld_stream(const c128* p) {
  const double2 v = __ldcs(reinterpret_cast<const double2*>(p));
  return c128(v.x, v.y);
}
__device__ __forceinline__ c64 ld_stream(const c64* p) {
  const float2 v = __ldcs(reinterpret_cast<const float2*>(p));
  return c64(v.x, v.y);
}
// L2-only evict-first loads: an L2 cache-policy hint on a read-only load,
// L1 allocation unchanged (the row kernels re-read their lines from L1)
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ double ld_l2ef(const double* a, uint64_t pol) {
  double v;
  asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ float ld_l2ef(const float* a, uint64_t pol) {
  float v;
  asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ int ld_l2ef(const int* a, uint64_t pol) {
  int v;
  asm("ld.global.nc.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ c128 ld_l2ef(const c128* a, uint64_t pol) {
  double x, y;
  asm("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(x), "=d"(y) : "l"(a), "l"(pol));
  return c128(x, y);
}
__device__ __forceinline__ c64 ld_l2ef(const c64* a, uint64_t pol) {
  float x, y;
  asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(x), "=f"(y) : "l"(a), "l"(pol));
  return c64(x, y);
}

// val[k] * x[ci[k]], the streamed operands evict-first when STREAM
template <bool STREAM = false, class V, class T>
__device__ __forceinline__ T crs_term(const V* __restrict__ val, const int* __restrict__ ci, const T* __restrict__ x,
                                      long k) {
  if constexpr (STREAM) return mulvt(ld_stream(val + k), x[ld_stream(ci + k)]);
  else return mulvt(val[k], x[ci[k]]);
}
// the same with the L2-only evict-first policy pol
template <class V, class T>
__device__ __forceinline__ T crs_term_l2(const V* __restrict__ val, const int* __restrict__ ci,
                                         const T* __restrict__ x, long k, uint64_t pol) {
  return mulvt(ld_l2ef(val + k, pol), x[ld_l2ef(ci + k, pol)]);
}

MatView UserMatrix::view64() const {
  MatView v;
  v.format = format;
  v.nrows = nrows;
  v.ncols = ncols;
  v.nnz = nnz;
  v.rp = row_ptr;
  v.ci = col_ind;
  v.hb = half_band;
  v.nx = nx; v.ny = ny; v.nz = nz;
  for (int i = 0; i < 7; ++i) v.st[i] = st[i];
  v.vcplx = (vals == 2);
  v.group = group;
  v.bin_short = bin_short;
  v.n_med = n_med;
  v.n_long = n_long;
  v.n_seg = n_seg;
  v.med_rows = med_rows;
  v.long_rows = long_rows;
  v.seg_ptr = seg_ptr;
  v.partial = partial;
  v.ri = row_ind;
  v.n_empty = n_empty;
  v.empty_rows = empty_rows;
  v.carry = carry;
  if (format == FMT_CRS || format == FMT_COO) v.val = val;
  else if (format == FMT_CDS) v.val = band;
  else if (format == FMT_DENSE) v.val = mat;
  return v;
}

long UserMatrix::bytes() const {
  size_t vs = (vals == 2) ? 16 : 8;
  switch (format) {
    case FMT_CRS: case FMT_COO: return (long)(4 * (nrows + 1) + nnz * (4 + vs));
    case FMT_CDS: return (long)nrows * (2 * half_band + 1) * vs;
    case FMT_DENSE: return (long)nrows * ncols * vs;
    default: return 0;
  }
}

void user_matrix_release(UserMatrix* K) {
  if (!K) return;
  if (--K->refcount > 0) return;
  cudaFree(K->row_ptr); cudaFree(K->col_ind); cudaFree(K->val); cudaFree(K->band);
  cudaFree(K->mat); cudaFree(K->diag);
  cudaFree(K->med_rows); cudaFree(K->long_rows); cudaFree(K->seg_ptr); cudaFree(K->partial);
  cudaFree(K->row_ind); cudaFree(K->empty_rows); cudaFree(K->carry);
  delete K;
}

// empty rows and the carries of the nonzero-balanced segmented reduction
static void build_seg_reduce(UserMatrix& M, const int* rp) {
  std::vector<int> empty;
  for (int i = 0; i < M.nrows; ++i)
    if (rp[i + 1] == rp[i]) empty.push_back(i);
  M.n_empty = (int)empty.size();
  if (!empty.empty()) {
    IDRS_CUDA(cudaMalloc((void**)&M.empty_rows, sizeof(int) * empty.size()));
    IDRS_CUDA(cudaMemcpy(M.empty_rows, empty.data(), sizeof(int) * empty.size(), cudaMemcpyHostToDevice));
  }
  const long warps = (M.nnz + kCooWarpNnz - 1) / kCooWarpNnz;
  IDRS_CUDA(cudaMalloc(&M.carry, 2 * 16 * (size_t)std::max<long>(warps, 1)));
}

static int* upload_ints(const std::vector<int>& h) {
  int* d = nullptr;
  IDRS_CUDA(cudaMalloc((void**)&d, sizeof(int) * std::max<size_t>(h.size(), 1)));
  if (!h.empty()) IDRS_CUDA(cudaMemcpy(d, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice));
  return d;
}

void build_row_plan(UserMatrix& M, const int* rp) {
  // rows far longer than the lanes given to a row would serialise a warp
  const long th = 32L * std::max(M.group, 1);
  bool skewed = false;
  for (int i = 0; i < M.nrows && !skewed; ++i) skewed = (long)rp[i + 1] - rp[i] > th;
  if (!skewed) return;
  // one lane per row: short / middle / long bins; G lanes per row: rows up to 32 G / long
  const long short_max = (M.group == 1) ? kBinShort : th;
  const long med_max = (M.group == 1) ? kBinLong : th;
  std::vector<std::pair<int, int>> med;  // (length, row)
  std::vector<int> longr, segp(1, 0);
  for (int i = 0; i < M.nrows; ++i) {
    const long len = (long)rp[i + 1] - rp[i];
    if (len <= short_max) continue;
    if (len <= med_max) {
      med.emplace_back((int)len, i);
    } else {
      longr.push_back(i);
      segp.push_back(segp.back() + (int)((len + kSegNnz - 1) / kSegNnz));
    }
  }
  // longest first, rows ascending within a length: the rows of one warp have
  // nearly equal lengths
  std::stable_sort(med.begin(), med.end(), [](const std::pair<int, int>& a, const std::pair<int, int>& b) {
    return a.first > b.first;
  });
  std::vector<int> medr(med.size());
  for (size_t q = 0; q < med.size(); ++q) medr[q] = med[q].second;
  M.bin_short = (int)short_max;
  M.n_med = (int)medr.size();
  M.n_long = (int)longr.size();
  M.n_seg = segp.back();
  if (M.n_med) M.med_rows = upload_ints(medr);
  if (M.n_long) {
    M.long_rows = upload_ints(longr);
    M.seg_ptr = upload_ints(segp);
    IDRS_CUDA(cudaMalloc(&M.partial, 16 * (size_t)M.n_seg));
  }
}

void build_coo_rows(UserMatrix& M, const int* rp) {
  std::vector<int> ri(std::max<long>(M.nnz, 1));
  for (int i = 0; i < M.nrows; ++i)
    for (int k = rp[i]; k < rp[i + 1]; ++k) ri[k] = i;
  IDRS_CUDA(cudaMalloc((void**)&M.row_ind, sizeof(int) * ri.size()));
  IDRS_CUDA(cudaMemcpy(M.row_ind, ri.data(), sizeof(int) * ri.size(), cudaMemcpyHostToDevice));
  build_seg_reduce(M, rp);
}

// ---------------------------------------------------------------------------
// SpMV kernels.  All compute y = a * (M x) + cv * v and return at once when
// *skip is non-zero (solver already stopped on the device).
// ---------------------------------------------------------------------------

// Matrix-free 7-point stencil (E/STENCIL/user_module.f90:155-160): 2-D thread
// tiles in x-y march along z keeping x(z-1), x(z), x(z+1) in registers; the
// x/y neighbours come from L1/L2.  Dirichlet zero outside the grid.  GB300's
// FP64 pipe is narrow, so the fp64 form spends as few FP64 instructions as
// possible: the epilogue scale is folded into the coefficients on the host
// (SCALE == false) and the sum is one multiply plus an FMA chain.
template <class T, class R, bool SCALE>
__global__ void __launch_bounds__(256) k_stencil7(int nx, int ny, int nz, int zc, R c0, R cw, R ce,
                                                  R cs, R cn, R cf, R cb, const T* __restrict__ x,
                                                  T* __restrict__ y, T a, T cv,
                                                  const T* __restrict__ v, T cu,
                                                  const T* __restrict__ u,
                                                  const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const int z0 = blockIdx.z * zc;
  const int z1 = min(nz, z0 + zc);
  const long plane = (long)nx * ny;
  long p = i + (long)nx * (j + (long)ny * z0);
  T xm = z0 > 0 ? x[p - plane] : T(0);
  T xc = x[p];
  for (int z = z0; z < z1; ++z, p += plane) {
    T xp = (z + 1 < nz) ? x[p + plane] : T(0);
    T xw = i > 0 ? x[p - 1] : T(0);
    T xe = i < nx - 1 ? x[p + 1] : T(0);
    T xs = j > 0 ? x[p - nx] : T(0);
    T xn = j < ny - 1 ? x[p + nx] : T(0);
    T s = c0 * xc + cw * xw + ce * xe + cs * xs + cn * xn + cf * xm + cb * xp;
    T out = SCALE ? a * s : s;
    if (u) out = out + cu * u[p];
    if (v) out = out + cv * v[p];
    y[p] = out;
    xm = xc;
    xc = xp;
  }
}

// fp32 stencil, four x-points per thread (float4): a warp covers 128
// consecutive x-points of one row, the x-neighbours come from the adjacent
// lanes by shuffles (the two row ends of a warp from L1), the y-neighbours
// are float4 loads of the rows of the neighbouring warps (L1 hits), and the
// z-neighbours stay in registers while the block marches along z.  One
// 16-byte load per operand and point quadruple instead of seven scalar loads
// per point.  Needs nx % 4 == 0 and 16-byte aligned vectors (checked by the
// launcher).  SCALE == false form: a and the centre term are folded into the
// coefficients.
// St7, st7_point, st7_apply, axpy4, ld4 and kF4Rows: stencil.cuh

__global__ void __launch_bounds__(32 * kF4Rows, 4) k_stencil7_f4(
    int nx, int ny, int nz, int zc, float c0, float cw, float ce, float cs, float cn, float cf,
    float cb, const float* __restrict__ x, float* __restrict__ y, float cv,
    const float* __restrict__ v, float cu, const float* __restrict__ u,
    const int* __restrict__ skip) {
  pdl_wait();
  pdl_trigger();
  if (skip && *skip) return;
  const int lane = threadIdx.x;
  const int i0 = (blockIdx.x * 32 + lane) * 4;
  const int j = blockIdx.y * kF4Rows + threadIdx.y;
  const int z0 = blockIdx.z * zc;
  const int z1 = min(nz, z0 + zc);
  const bool in = (i0 < nx) && (j < ny);
  const long plane = (long)nx * ny;
  long p = (long)j * nx + i0 + plane * z0;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  // software pipeline: the HBM streams (plane z+2 of x, plane z+1 of u and v)
  // are requested one iteration ahead of their use
  float4 xm = (in && z0 > 0) ? ld4(x + p - plane) : zero;
  float4 xc = in ? ld4(x + p) : zero;
  float4 xp = (in && z0 + 1 < nz) ? ld4(x + p + plane) : zero;
  float4 uc = (in && u) ? ld4(u + p) : zero;
  float4 vc = (in && v) ? ld4(v + p) : zero;
  for (int z = z0; z < z1; ++z, p += plane) {
    const bool more = z + 1 < z1;
    const float4 xpp = (in && z + 2 < nz) ? ld4(x + p + 2 * plane) : zero;
    const float4 un = (in && u && more) ? ld4(u + p + plane) : zero;
    const float4 vn = (in && v && more) ? ld4(v + p + plane) : zero;
    const float4 xs = (in && j > 0) ? ld4(x + p - nx) : zero;
    const float4 xn = (in && j + 1 < ny) ? ld4(x + p + nx) : zero;
    float left = __shfl_up_sync(0xffffffffu, xc.w, 1);
    float right = __shfl_down_sync(0xffffffffu, xc.x, 1);
    if (lane == 0) left = (in && i0 > 0) ? __ldg(x + p - 1) : 0.f;
    if (lane == 31) right = (in && i0 + 4 < nx) ? __ldg(x + p + 4) : 0.f;
    if (in) {
      float4 r = st7_apply(St7{c0, cw, ce, cs, cn, cf, cb}, xm, xc, xp, xs, xn, left, right);
      if (u) axpy4(r, cu, uc);
      if (v) axpy4(r, cv, vc);
      *reinterpret_cast<float4*>(y + p) = r;
    }
    xm = xc;
    xc = xp;
    xp = xpp;
    uc = un;
    vc = vn;
  }
}

static inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// Two consecutive fp32 stencil steps in one pass (temporal blocking of the
// polynomial chain):
//   yA = S_a xin + cua u + cva v          (S_a: stencil with its scale folded in)
//   yB = S_b yA  + cub xin + cvb vb
// A block owns kX2Rows output rows of the full x extent (nx <= 256, four
// x-points per thread) over zc planes.  Marching in z, it computes yA one
// plane ahead for its rows plus one halo row on each side (recomputed, not
// read back), keeps the last three yA planes in shared memory, and forms yB
// from them, so yA never travels through HBM on its way into step B (it is
// written out only when a later step reads it).  Per pair of steps it moves
// xin, u, v, vb and the outputs once instead of twice: 5 vectors instead of 8
// in the middle of a Chebyshev recurrence.
constexpr int kX2Rows = 8;
constexpr int kX2Halo = kX2Rows + 2;
constexpr int kX2MaxNx = 256;


__global__ void __launch_bounds__(64 * kX2Halo, 2) k_stencil7_f4x2(
    int nx, int ny, int nz, int zc, St7 ca, float cua, float cva, St7 cb, float cub, float cvb,
    const float* __restrict__ xin, const float* __restrict__ u, const float* __restrict__ v,
    const float* __restrict__ vb, float* __restrict__ ya, float* __restrict__ yb,
    const int* __restrict__ skip) {
  if (skip && *skip) return;
  // ring of four yA planes: step A writes plane z+2 while step B reads z-1..z+1,
  // so one barrier per plane suffices
  __shared__ __align__(16) float sA[4][kX2Halo][kX2MaxNx];
  const int tx = threadIdx.x;
  const int lane = tx & 31;
  const int ty = threadIdx.y;
  const int i0 = tx * 4;
  const int j = blockIdx.x * kX2Rows - 1 + ty;  // row of this thread (one halo row each side)
  const int z0 = blockIdx.y * zc;
  const int z1 = min(nz, z0 + zc);
  const bool xok = i0 < nx;
  const bool act = xok && j >= 0 && j < ny;
  const bool interior = act && ty >= 1 && ty <= kX2Rows;
  const long plane = (long)nx * ny;
  const long roff = act ? (long)j * nx + i0 : 0;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  auto ld = [&](const float* a, int z) -> float4 {
    return (a && act && z >= 0 && z < nz) ? ld4(a + z * plane + roff) : zero;
  };
  // step A at plane zp from xm, xc, xp = xin(zp-1 .. zp+1) and uc, vc = u(zp), v(zp)
  auto stepA = [&](int zp, float4 xm, float4 xc, float4 xp, float4 uc, float4 vc) {
    float4 r = zero;
    if (zp >= 0 && zp < nz) {  // uniform over the block
      const long o = zp * plane + roff;
      const float4 xs = (act && j > 0) ? ld4(xin + o - nx) : zero;
      const float4 xn = (act && j + 1 < ny) ? ld4(xin + o + nx) : zero;
      float left = __shfl_up_sync(0xffffffffu, xc.w, 1);
      float right = __shfl_down_sync(0xffffffffu, xc.x, 1);
      if (lane == 0) left = (act && i0 > 0) ? __ldg(xin + o - 1) : 0.f;
      if (lane == 31) right = (act && i0 + 4 < nx) ? __ldg(xin + o + 4) : 0.f;
      if (act) {
        r = st7_apply(ca, xm, xc, xp, xs, xn, left, right);
        axpy4(r, cua, uc);
        axpy4(r, cva, vc);
        if (ya && interior && zp >= z0 && zp < z1) *reinterpret_cast<float4*>(ya + o) = r;
      }
    }
    if (xok) *reinterpret_cast<float4*>(&sA[(zp + 4) & 3][ty][i0]) = r;
  };
  float4 m = ld(xin, z0 - 2), c = ld(xin, z0 - 1), p = ld(xin, z0);
  stepA(z0 - 1, m, c, p, ld(u, z0 - 1), ld(v, z0 - 1));
  m = c; c = p; p = ld(xin, z0 + 1);
  stepA(z0, m, c, p, ld(u, z0), ld(v, z0));
  for (int z = z0; z < z1; ++z) {
    const float4 xz = c;  // xin(z)
    m = c; c = p; p = ld(xin, z + 2);
    stepA(z + 1, m, c, p, ld(u, z + 1), ld(v, z + 1));
    __syncthreads();
    // step B; every lane runs the shuffles (lanes past the grid hold zeros)
    const int s0 = (z + 3) & 3, s1 = z & 3, s2 = (z + 1) & 3;  // planes z-1, z, z+1
    float4 bm = zero, bc = zero, bp = zero, bs = zero, bn = zero;
    if (interior) {
      bm = *reinterpret_cast<const float4*>(&sA[s0][ty][i0]);
      bc = *reinterpret_cast<const float4*>(&sA[s1][ty][i0]);
      bp = *reinterpret_cast<const float4*>(&sA[s2][ty][i0]);
      bs = *reinterpret_cast<const float4*>(&sA[s1][ty - 1][i0]);
      bn = *reinterpret_cast<const float4*>(&sA[s1][ty + 1][i0]);
    }
    float bl = __shfl_up_sync(0xffffffffu, bc.w, 1);
    float br = __shfl_down_sync(0xffffffffu, bc.x, 1);
    if (interior) {
      if (lane == 0) bl = (i0 > 0) ? sA[s1][ty][i0 - 1] : 0.f;
      if (lane == 31) br = (i0 + 4 < nx) ? sA[s1][ty][i0 + 4] : 0.f;
      float4 r = st7_apply(cb, bm, bc, bp, bs, bn, bl, br);
      axpy4(r, cub, xz);
      axpy4(r, cvb, ld(vb, z));
      *reinterpret_cast<float4*>(yb + z * plane + roff) = r;
    }
  }
}



// The same two steps with eight x-points per thread: one warp spans a row of
// nx <= 256 points (nx % 8 == 0), so the x-neighbours are shuffles with zero
// fill at both ends (no edge loads), and every per-thread overhead (address
// arithmetic, bounds predicates, shuffles, the barrier) is spread over twice
// as many points.  The kernel is instruction-issue bound (ncu: 72 % issue
// active against 29 % DRAM throughput with four points per thread), so points
// per instruction is what sets its speed.  yA planes live in shared memory
// as two half-planes (points 0-3 and 4-7 of every lane) so that each 16-byte
// shared access of a warp is conflict-free.  Streams advance by one plane
// pointer increment per iteration.
constexpr int kX8Rows = 8;
constexpr int kX8Halo = kX8Rows + 2;

struct F8 {
  float4 a, b;
};
__device__ __forceinline__ F8 ld8(const float* p) { return F8{ld4(p), ld4(p + 4)}; }
__device__ __forceinline__ F8 zero8() { return F8{make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)}; }
__device__ __forceinline__ void axpy8(F8& r, float a, const F8& x) { axpy4(r.a, a, x.a); axpy4(r.b, a, x.b); }
// 7-point stencil on eight consecutive points: left / right are the x-neighbours
// of the first / last point
__device__ __forceinline__ F8 st7_apply8(const St7& c, const F8& xm, const F8& xc, const F8& xp, const F8& xs,
                                         const F8& xn, float left, float right) {
  F8 r;
  r.a = st7_apply(c, xm.a, xc.a, xp.a, xs.a, xn.a, left, xc.b.x);
  r.b = st7_apply(c, xm.b, xc.b, xp.b, xs.b, xn.b, xc.a.w, right);
  return r;
}

__global__ void __launch_bounds__(32 * kX8Halo, 2) k_stencil7_f8x2(
    int nx, int ny, int nz, int zc, St7 ca, float cua, float cva, St7 cb, float cub, float cvb,
    const float* __restrict__ xin, const float* __restrict__ u, const float* __restrict__ v,
    const float* __restrict__ vb, float* __restrict__ ya, float* __restrict__ yb,
    const int* __restrict__ skip) {
  if (skip && *skip) return;
  // [plane ring 4][row][half][lane * 4]
  __shared__ __align__(16) float sA[4][kX8Halo][2][128];
  const int lane = threadIdx.x, ty = threadIdx.y;
  const int i0 = lane * 8;
  const int j = blockIdx.x * kX8Rows - 1 + ty;
  const int z0 = blockIdx.y * zc;
  const int z1 = min(nz, z0 + zc);
  const bool act = i0 < nx && j >= 0 && j < ny;
  const bool interior = act && ty >= 1 && ty <= kX8Rows;
  const bool has_s = act && j > 0, has_n = act && j + 1 < ny;
  const long plane = (long)nx * ny;
  const long roff = act ? (long)j * nx + i0 : 0;
  auto at = [&](const float* a, int z) { return a + (long)z * plane + roff; };
  auto atw = [&](float* a, int z) { return a + (long)z * plane + roff; };
  auto ld = [&](const float* a, int z) -> F8 { return (a && act && z >= 0 && z < nz) ? ld8(at(a, z)) : zero8(); };
  auto put = [&](int zp, const F8& r) {
    float* q = &sA[(zp + 4) & 3][ty][0][lane * 4];
    *reinterpret_cast<float4*>(q) = r.a;
    *reinterpret_cast<float4*>(q + 128) = r.b;
  };
  // step A at plane zp from xm, xc, xp = xin(zp-1 .. zp+1)
  auto stepA = [&](int zp, const F8& xm, const F8& xc, const F8& xp) {
    F8 r = zero8();
    if (zp >= 0 && zp < nz) {  // uniform over the block
      const float* o = at(xin, zp);
      const F8 xs = has_s ? ld8(o - nx) : zero8();
      const F8 xn = has_n ? ld8(o + nx) : zero8();
      float left = __shfl_up_sync(0xffffffffu, xc.b.w, 1);
      float right = __shfl_down_sync(0xffffffffu, xc.a.x, 1);
      if (lane == 0) left = 0.f;
      if (lane == 31) right = 0.f;
      if (act) {
        r = st7_apply8(ca, xm, xc, xp, xs, xn, left, right);
        if (u) axpy8(r, cua, ld8(at(u, zp)));
        if (v) axpy8(r, cva, ld8(at(v, zp)));
        if (ya && interior && zp >= z0 && zp < z1) {
          float* w = atw(ya, zp);
          *reinterpret_cast<float4*>(w) = r.a;
          *reinterpret_cast<float4*>(w + 4) = r.b;
        }
      }
    }
    put(zp, r);
  };
  F8 m = ld(xin, z0 - 2), c = ld(xin, z0 - 1), p = ld(xin, z0);
  stepA(z0 - 1, m, c, p);
  m = c; c = p; p = ld(xin, z0 + 1);
  stepA(z0, m, c, p);
  for (int z = z0; z < z1; ++z) {
    // step B's vb row is requested before step A and the barrier, so its
    // latency overlaps them instead of stalling every warp after the barrier
    const F8 vbz = (vb && interior) ? ld8(at(vb, z)) : zero8();
    m = c; c = p; p = ld(xin, z + 2);  // m = xin(z)
    stepA(z + 1, m, c, p);
    __syncthreads();
    // step B at plane z; every lane runs the shuffles (lanes past the grid hold zeros)
    const int s0 = (z + 3) & 3, s1 = z & 3, s2 = (z + 1) & 3;  // planes z-1, z, z+1
    auto get = [&](int s, int row) {
      const float* q = &sA[s][row][0][lane * 4];
      return F8{*reinterpret_cast<const float4*>(q), *reinterpret_cast<const float4*>(q + 128)};
    };
    const F8 bc = interior ? get(s1, ty) : zero8();
    float bl = __shfl_up_sync(0xffffffffu, bc.b.w, 1);
    float br = __shfl_down_sync(0xffffffffu, bc.a.x, 1);
    if (lane == 0) bl = 0.f;
    if (lane == 31) br = 0.f;
    if (interior) {
      F8 r = st7_apply8(cb, get(s0, ty), bc, get(s2, ty), get(s1, ty - 1), get(s1, ty + 1), bl, br);
      axpy8(r, cub, m);
      if (vb) axpy8(r, cvb, vbz);
      float* w = atw(yb, z);
      *reinterpret_cast<float4*>(w) = r.a;
      *reinterpret_cast<float4*>(w + 4) = r.b;
    }
  }
}

// The same pair with its HBM streams staged in shared memory one plane
// ahead by bulk asynchronous copies (cp.async.bulk, mbarrier completion), so
// no warp waits for HBM inside an iteration: while a block computes plane
// zp, the copies of xin(zp+2) and u, v(zp+1) are in flight.  The block's rows
// j0-1 .. j0+8 of a plane are one contiguous run of each vector, so a plane
// is three copies issued by one thread.  The halo rows' outer y-neighbours
// (rows j0-2 and j0+9, read by two warps only) are loaded into registers a
// plane ahead instead.  Three xin stages, two u / v stages and a ring of
// four yA planes (one barrier per plane) keep the block at 110 KB of shared
// memory, two blocks per SM.  Stage slots and mbarrier phases advance by
// counters (every copied plane is waited for once, in order).  Each thread
// owns two half-rows of four points (i0 = 4 lane and nx/2 + i0), so every
// 16-byte shared-memory access of a warp is conflict-free; each point is
// computed by the same FMAs as in k_stencil7_f8x2 (bitwise equal results).
// A copy that has not landed after kTmaWaitCycles sets a shared flag: the
// block then stops waiting, writes NaN into its output rows and records the
// fault.
constexpr int kT8XStages = 3;
constexpr int kT8UStages = 2;
constexpr int kT8ARing = 4;

static size_t t8_smem(int nx) {
  return 128 + sizeof(float) * (size_t)nx * kX8Halo * (kT8XStages + 2 * kT8UStages + kT8ARing);
}

// two half-rows of four points: [i0, i0+4) and [hx+i0, hx+i0+4)
__device__ __forceinline__ F8 ld8h(const float* row, int i0, int hx) {
  return F8{*reinterpret_cast<const float4*>(row + i0), *reinterpret_cast<const float4*>(row + hx + i0)};
}
__device__ __forceinline__ F8 ld8hg(const float* row, int i0, int hx) { return F8{ld4(row + i0), ld4(row + hx + i0)}; }
__device__ __forceinline__ void st8h(float* row, int i0, int hx, const F8& r) {
  *reinterpret_cast<float4*>(row + i0) = r.a;
  *reinterpret_cast<float4*>(row + hx + i0) = r.b;
}
// the x-neighbours of both half-rows (lane L holds the last points of each
// half; the domain ends are zero); every lane runs the shuffles
struct XNb {
  float la, ra, lb, rb;
};
__device__ __forceinline__ XNb x_neighbours(const F8& c, int lane, int L) {
  const float ua = __shfl_up_sync(0xffffffffu, c.a.w, 1), da = __shfl_down_sync(0xffffffffu, c.a.x, 1);
  const float ub = __shfl_up_sync(0xffffffffu, c.b.w, 1), db = __shfl_down_sync(0xffffffffu, c.b.x, 1);
  const float b0 = __shfl_sync(0xffffffffu, c.b.x, 0), aL = __shfl_sync(0xffffffffu, c.a.w, L);
  return XNb{lane == 0 ? 0.f : ua, lane == L ? b0 : da, lane == 0 ? aL : ub, lane == L ? 0.f : db};
}
__device__ __forceinline__ F8 st7_apply8h(const St7& c, const F8& xm, const F8& xc, const F8& xp, const F8& xs,
                                          const F8& xn, const XNb& nb) {
  return F8{st7_apply(c, xm.a, xc.a, xp.a, xs.a, xn.a, nb.la, nb.ra),
            st7_apply(c, xm.b, xc.b, xp.b, xs.b, xn.b, nb.lb, nb.rb)};
}
__device__ __forceinline__ int next_slot(int s, int n) { return s + 1 == n ? 0 : s + 1; }

// NXC: the row length as a compile-time constant (0: nx at run time), so the
// row, half-row and slot offsets of the common 256-point rows are immediates.
// VBM: where step B's vb term comes from.  In a polynomial chain vb is the
// chain's input, which is also step A's v (VBM 1) or, in the first pair,
// step A's xin (VBM 2); the thread then already holds vb(zp-1) from the
// previous plane (step A's v, kept one plane in registers, or xm), and no
// global load sits in step B.  VBM 0 loads vb from global memory.
template <int NXC, int VBM>
__global__ void __launch_bounds__(32 * kX8Halo, 2) k_stencil7_f8x2t(
    int nx_rt, int ny, int nz, int zc, St7 ca, float cua, float cva, St7 cb, float cub, float cvb,
    const float* __restrict__ xin, const float* __restrict__ u, const float* __restrict__ v,
    const float* __restrict__ vb, float* __restrict__ ya, float* __restrict__ yb,
    const int* __restrict__ skip, int* fault) {
  pdl_wait();
  pdl_trigger();
  if (skip && *skip) return;
  const int nx = NXC ? NXC : nx_rt;
  extern __shared__ __align__(128) unsigned char sm[];
  uint64_t* mbX = reinterpret_cast<uint64_t*>(sm);
  uint64_t* mbU = mbX + kT8XStages;
  volatile int* sflag = reinterpret_cast<volatile int*>(sm + 64);
  const int rstride = kX8Halo * nx;  // one stage / ring slot (floats)
  float* Xs = reinterpret_cast<float*>(sm + 128);
  float* Us = Xs + kT8XStages * rstride;
  float* Vs = Us + kT8UStages * rstride;
  float* sA = Vs + kT8UStages * rstride;
  const int lane = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + lane;
  const int hx = nx >> 1, L = (nx >> 3) - 1, i0 = lane * 4;
  const int j0 = blockIdx.x * kX8Rows, j = j0 - 1 + ty;
  const int z0 = blockIdx.y * zc, z1 = min(nz, z0 + zc), zb = z0 - 1;
  const bool lact = lane <= L;
  const bool act = lact && j >= 0 && j < ny;
  const bool interior = act && ty >= 1 && ty <= kX8Rows;
  const bool has_s = act && j > 0, has_n = act && j + 1 < ny;
  const long plane = (long)nx * ny;
  const int r0 = max(j0 - 1, 0), r1 = min(j0 + kX8Rows, ny - 1);
  const unsigned rbytes = (unsigned)((r1 - r0 + 1) * nx * 4);
  const int roff = (r0 - (j0 - 1)) * nx;
  const bool have_uv = (u != nullptr) || (v != nullptr);
  // planes of the stage sequences: xin zb .. z1+1, u / v zb .. z1, inside the
  // grid, copied and waited for in order from qa
  const int qa = max(zb, 0);
  const int xlast = min(nz - 1, z1 + 1), ulast = have_uv ? min(nz - 1, z1) : qa - 1;
  // this thread's element in every stage and ring slot (row ty, first half)
  const int toff = ty * nx + i0;
  float* const X0 = Xs + toff;
  float* const X1 = X0 + rstride;
  float* const X2 = X1 + rstride;
  const float* const U0 = Us + toff;
  const float* const U1 = U0 + rstride;
  const float* const V0 = Vs + toff;
  const float* const V1 = V0 + rstride;
  float* const A0 = sA + toff;
  auto xslot = [&](int s) { return s == 0 ? X0 : (s == 1 ? X1 : X2); };
  auto aslot = [&](int q) { return A0 + ((q - zb) & (kT8ARing - 1)) * rstride; };
  // global streams of this thread, advanced one plane per iteration
  const long goff = (long)j * nx + i0;
  const float* gvb = (VBM == 0 && vb) ? vb + (long)(zb - 1) * plane + goff : nullptr;  // vb(zp-1)
  F8 vprev = zero8();  // VBM 1: v(zp-1) of this thread's row, from step A of the previous plane
  float* gya = ya ? ya + (long)zb * plane + goff : nullptr;              // ya(zp)
  float* gyb = yb + (long)(zb - 1) * plane + goff;                        // yb(zp-1)
  // the halo warps' outer neighbour row (ty 0: j-1, ty 9: j+1)
  const int hrow = ty == 0 ? j - 1 : j + 1;
  const bool hact = lact && j >= 0 && j < ny && (ty == 0 || ty == kX8Halo - 1) && hrow >= 0 && hrow < ny;
  const float* ghalo = hact ? xin + (long)zb * plane + (long)hrow * nx + i0 : xin;  // plane zp
  int ix = 0, iu = 0;  // thread 0: next stage to fill
  auto issueX = [&](int q) {
    if (q < qa || q > xlast) return;
    mbar_expect_tx(&mbX[ix], rbytes);
    bulk_g2s(Xs + ix * rstride + roff, xin + q * plane + (long)r0 * nx, rbytes, &mbX[ix]);
    ix = next_slot(ix, kT8XStages);
  };
  auto issueU = [&](int q) {
    if (q < qa || q > ulast) return;
    mbar_expect_tx(&mbU[iu], (u ? rbytes : 0u) + (v ? rbytes : 0u));
    if (u) bulk_g2s(Us + iu * rstride + roff, u + q * plane + (long)r0 * nx, rbytes, &mbU[iu]);
    if (v) bulk_g2s(Vs + iu * rstride + roff, v + q * plane + (long)r0 * nx, rbytes, &mbU[iu]);
    iu = next_slot(iu, kT8UStages);
  };
  int wx = 0, wu = 0;          // next stage to wait for
  unsigned phx = 0, phu = 0;   // expected phase parity of each stage (bit s)
  auto wait_on = [&](uint64_t* bar, unsigned par) {
    if (mbar_try_wait(bar, par)) return;
    if (!*sflag && !mbar_wait_sleep(bar, par)) *sflag = 1;
  };
  auto waitX = [&](int q) {
    if (q < qa || q > xlast) return;
    wait_on(&mbX[wx], (phx >> wx) & 1u);
    phx ^= 1u << wx;
    wx = next_slot(wx, kT8XStages);
  };
  auto waitU = [&](int q) {
    if (q < qa || q > ulast) return;
    wait_on(&mbU[wu], (phu >> wu) & 1u);
    phu ^= 1u << wu;
    wu = next_slot(wu, kT8UStages);
  };
  if (tid == 0) {
    for (int s = 0; s < kT8XStages; ++s) mbar_init(&mbX[s], 1);
    for (int s = 0; s < kT8UStages; ++s) mbar_init(&mbU[s], 1);
    *sflag = 0;
    mbar_init_fence();
    issueX(zb);
    issueX(zb + 1);
    issueU(zb);
  }
  __syncthreads();
  const F8 z8 = zero8();
  // stage slots of xin(zp), xin(zp+1) and u / v(zp) for the reads
  int rx1 = zb + 1 - qa;                    // 0 or 1
  int rx0 = rx1 == 0 ? kT8XStages - 1 : 0;  // plane zb (unused when zb < 0)
  int ru = 0;
  F8 xm = (act && zb - 1 >= 0) ? ld8hg(xin + (long)(zb - 1) * plane + goff - i0, i0, hx) : z8;
  F8 hcur = (hact && zb >= 0) ? ld8hg(ghalo, 0, hx) : z8;
  if (zb == qa) waitX(zb);
  F8 xc = (act && zb >= 0) ? ld8h(xslot(rx0), 0, hx) : z8;  // xin(zp), carried in registers
  for (int zp = zb; zp <= z1; ++zp) {
    if (tid == 0) {
      proxy_async_fence();  // the reads of the refilled stages were before the last barrier
      issueX(zp + 2);
      issueU(zp + 1);
    }
    const bool doB = zp - 1 >= z0;
    const F8 vbz = (VBM == 0 && gvb && interior && doB) ? ld8hg(gvb, 0, hx) : z8;
    F8 vcur = z8;
    ghalo += plane;
    const F8 hnext = (hact && zp + 1 < nz) ? ld8hg(ghalo, 0, hx) : z8;
    waitX(zp + 1);
    waitU(zp);
    // xin(zp+1): this step's upper z-neighbour and the next plane's centre
    // (loaded also when step A is outside the grid, zp = -1)
    const F8 xp = (act && zp + 1 >= qa && zp + 1 <= xlast) ? ld8h(xslot(rx1), 0, hx) : z8;
    // step A at plane zp
    F8 r = z8;
    if (zp >= 0 && zp < nz) {  // uniform over the block
      const float* Xc = xslot(rx0);
      F8 xs = z8, xn = z8;
      if (ty == 0) xs = hcur;
      else if (has_s) xs = ld8h(Xc - nx, 0, hx);
      if (ty == kX8Halo - 1) xn = hcur;
      else if (has_n) xn = ld8h(Xc + nx, 0, hx);
      const XNb nb = x_neighbours(xc, lane, L);
      if (act) {
        r = st7_apply8h(ca, xm, xc, xp, xs, xn, nb);
        if (u) axpy8(r, cua, ld8h(ru ? U1 : U0, 0, hx));
        if (v) {
          vcur = ld8h(ru ? V1 : V0, 0, hx);
          axpy8(r, cva, vcur);
        }
        if (gya && interior && zp >= z0 && zp < z1) st8h(gya, 0, hx, r);
      }
    }
    if (lact) st8h(aslot(zp), 0, hx, r);
    __syncthreads();
    // step B at plane zp-1 from yA(zp-2 .. zp) and xin(zp-1) (= xm); step A
    // of the next plane writes the ring slot of zp-3, which nothing reads now
    if (doB) {
      const float* Aq = aslot(zp - 1);
      const F8 bc = interior ? ld8h(Aq, 0, hx) : z8;
      const XNb nb = x_neighbours(bc, lane, L);
      if (interior) {
        F8 rb = st7_apply8h(cb, ld8h(aslot(zp - 2), 0, hx), bc, ld8h(aslot(zp), 0, hx), ld8h(Aq - nx, 0, hx),
                            ld8h(Aq + nx, 0, hx), nb);
        axpy8(rb, cub, xm);
        if (VBM == 1) axpy8(rb, cvb, vprev);
        else if (VBM == 2) axpy8(rb, cvb, xm);
        else if (vb) axpy8(rb, cvb, vbz);
        st8h(gyb, 0, hx, rb);
      }
    }
    xm = xc;
    xc = xp;
    hcur = hnext;
    if (VBM == 1) vprev = vcur;
    rx0 = rx1;
    rx1 = next_slot(rx1, kT8XStages);
    if (zp >= qa && zp <= ulast) ru ^= 1;
    if (gvb) gvb += plane;
    if (gya) gya += plane;
    gyb += plane;
  }
  __syncthreads();  // every wait is behind: the flag is final and the same for all threads
  if (*sflag) {
    // a copy never landed: let the last copy of every stage finish (bounded),
    // then poison this block's outputs and report
    if (tid == 0) {
      for (int q = xlast, c = 0; q >= qa && c < kT8XStages; --q, ++c)
        mbar_wait(&mbX[(q - qa) % kT8XStages], ((q - qa) / kT8XStages) & 1);
      for (int q = ulast, c = 0; q >= qa && c < kT8UStages; --q, ++c)
        mbar_wait(&mbU[(q - qa) % kT8UStages], ((q - qa) / kT8UStages) & 1);
      *(volatile int*)fault = 1;
    }
    const float qn = nanf("");
    const F8 nan8 = F8{make_float4(qn, qn, qn, qn), make_float4(qn, qn, qn, qn)};
    if (interior)
      for (int z = z0; z < z1; ++z) {
        st8h(yb + (long)z * plane + goff, 0, hx, nan8);
        if (ya) st8h(ya + (long)z * plane + goff, 0, hx, nan8);
      }
  }
}

// CRS, G lanes per row (G | 32).  Warp-uniform loop so the shuffles are
// always executed by the full warp.
template <int G, class T, class V>
__global__ void __launch_bounds__(256) k_crs(int nrows, const int* __restrict__ rp,
                                             const int* __restrict__ ci, const V* __restrict__ val,
                                             const T* __restrict__ x, T* __restrict__ y, T a, T cv,
                                             const T* __restrict__ v, T cx, T cu,
                                             const T* __restrict__ u,
                                             const int* __restrict__ skip, int max_len) {
  if (skip && *skip) return;
  constexpr int RPW = 32 / G;
  const int lane = threadIdx.x & 31;
  const int sub = lane / G;
  const int gl = lane & (G - 1);
  const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  const long nwarps = (gridDim.x * (long)blockDim.x) >> 5;
  const uint64_t pol = l2_evict_first_policy();
  for (long base = warp * RPW; base < nrows; base += nwarps * RPW) {
    const long row = base + sub;
    T sum = T(0);
    bool mine = row < nrows;
    if (mine) {
      const int beg = rp[row], end = rp[row + 1];
      mine = (end - beg) <= max_len;  // longer rows: the bin kernels
      if (mine)
        for (int k = beg + gl; k < end; k += G) sum = sum + crs_term_l2(val, ci, x, k, pol);
    }
#pragma unroll
    for (int m = G / 2; m >= 1; m >>= 1) sum = sum + shfl_x(sum, m);
    if (mine && gl == 0) {
      T out = a * sum;
      if (cx != T(0)) out = out + cx * x[row];
      if (u) out = out + cu * u[row];
      if (v) out = out + cv * v[row];
      y[row] = out;
    }
  }
}

// CRS, one thread per row: no cross-lane reduction, so a row of k nonzeros
// costs k FMAs (the FP64 pipe of GB300 is the limit of short-row fp64 SpMV).
template <class T, class V>
__global__ void __launch_bounds__(256) k_crs_row(int nrows, const int* __restrict__ rp,
                                                 const int* __restrict__ ci, const V* __restrict__ val,
                                                 const T* __restrict__ x, T* __restrict__ y, T a, T cv,
                                                 const T* __restrict__ v, T cx, T cu,
                                                 const T* __restrict__ u,
                                                 const int* __restrict__ skip, int max_len) {
  if (skip && *skip) return;
  const uint64_t pol = l2_evict_first_policy();
  for (long row = blockIdx.x * (long)blockDim.x + threadIdx.x; row < nrows;
       row += gridDim.x * (long)blockDim.x) {
    const int beg = rp[row], end = rp[row + 1];
    if (end - beg > max_len) continue;  // written by the bin kernels
    T sum = T(0);
#pragma unroll 4
    for (int k = beg; k < end; ++k) sum = sum + crs_term_l2(val, ci, x, k, pol);
    T out = a * sum;
    if (cx != T(0)) out = out + cx * x[row];
    if (u) out = out + cu * u[row];
    if (v) out = out + cv * v[row];
    y[row] = out;
  }
}

template <class T>
__device__ __forceinline__ T epilogue(T sum, long row, T a, T cv, const T* __restrict__ v, T cx, T cu,
                                      const T* __restrict__ u, const T* __restrict__ x) {
  T out = a * sum;
  if (cx != T(0)) out = out + cx * x[row];
  if (u) out = out + cu * u[row];
  if (v) out = out + cv * v[row];
  return out;
}

// CRS middle bin: G lanes per listed row (rows sorted by length, so the rows
// of a warp need about the same number of steps).
template <int G, class T, class V>
__global__ void __launch_bounds__(256) k_crs_list(int nlist, const int* __restrict__ rows,
                                                  const int* __restrict__ rp, const int* __restrict__ ci,
                                                  const V* __restrict__ val, const T* __restrict__ x,
                                                  T* __restrict__ y, T a, T cv, const T* __restrict__ v, T cx,
                                                  T cu, const T* __restrict__ u, const int* __restrict__ skip) {
  if (skip && *skip) return;
  constexpr int RPW = 32 / G;
  const int lane = threadIdx.x & 31;
  const int sub = lane / G;
  const int gl = lane & (G - 1);
  const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  const long nwarps = (gridDim.x * (long)blockDim.x) >> 5;
  const uint64_t pol = l2_evict_first_policy();
  for (long base = warp * RPW; base < nlist; base += nwarps * RPW) {
    const long idx = base + sub;
    T sum = T(0);
    int row = 0;
    if (idx < nlist) {
      row = rows[idx];
      const int beg = rp[row], end = rp[row + 1];
#pragma unroll 4
      for (int k = beg + gl; k < end; k += G) sum = sum + crs_term_l2(val, ci, x, k, pol);
    }
#pragma unroll
    for (int m = G / 2; m >= 1; m >>= 1) sum = sum + shfl_x(sum, m);
    if (idx < nlist && gl == 0) y[row] = epilogue(sum, row, a, cv, v, cx, cu, u, x);
  }
}

// CRS long bin: one warp per kSegNnz-nonzero segment of a long row.
template <class T, class V>
__global__ void __launch_bounds__(256) k_crs_seg(int n_seg, int n_long, const int* __restrict__ long_rows,
                                                 const int* __restrict__ seg_ptr,
                                                 const int* __restrict__ rp, const int* __restrict__ ci,
                                                 const V* __restrict__ val, const T* __restrict__ x,
                                                 T* __restrict__ partial, const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int lane = threadIdx.x & 31;
  const long g = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  if (g >= n_seg) return;  // whole warp
  int lo = 0, hi = n_long;  // seg_ptr[lo] <= g < seg_ptr[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (seg_ptr[mid] <= g) lo = mid; else hi = mid;
  }
  const int row = long_rows[lo];
  const long beg = rp[row] + (g - seg_ptr[lo]) * (long)kSegNnz;
  const long end = min((long)rp[row + 1], beg + kSegNnz);
  T sum = T(0);
#pragma unroll 8
  for (int j = 0; j < kSegNnz / 32; ++j) {
    const long k = beg + lane + 32L * j;
    if (k < end) sum = sum + crs_term<true>(val, ci, x, k);
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) sum = sum + shfl_x(sum, m);
  if (lane == 0) partial[g] = sum;
}

// CRS long bin: one warp per long row adds its segments in a fixed order.
template <class T>
__global__ void __launch_bounds__(256) k_crs_fin(int n_long, const int* __restrict__ long_rows,
                                                 const int* __restrict__ seg_ptr,
                                                 const T* __restrict__ partial, const T* __restrict__ x,
                                                 T* __restrict__ y, T a, T cv, const T* __restrict__ v, T cx,
                                                 T cu, const T* __restrict__ u, const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int lane = threadIdx.x & 31;
  const long w = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  if (w >= n_long) return;
  T sum = T(0);
  for (int g = seg_ptr[w] + lane; g < seg_ptr[w + 1]; g += 32) sum = sum + partial[g];
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) sum = sum + shfl_x(sum, m);
  if (lane == 0) {
    const int row = long_rows[w];
    y[row] = epilogue(sum, row, a, cv, v, cx, cu, u, x);
  }
}

// Row index of an entry for the segmented reduction (stored with the COO
// entries).  rows_of() gives the rows of a lane's entries k0 .. k0+cnt-1.
struct RowsStored {
  const int* __restrict__ ri;
  const int* __restrict__ rp;
  __device__ int find(long k) const { return ri[k]; }
  __device__ bool first_open(long beg, int row_first) const { return beg > 0 && ri[beg - 1] == row_first; }
  __device__ bool last_open(long end, long nnz, int row_last) const { return end < nnz && ri[end] == row_last; }
  template <int IT>
  __device__ void rows_of(long k0, int cnt, int, int, int (&rows)[IT]) const {
    if (cnt == IT && IT % 4 == 0) {
#pragma unroll
      for (int q = 0; q < IT / 4; ++q) {
        const int4 r4 = __ldg(reinterpret_cast<const int4*>(ri + k0) + q);
        rows[4 * q] = r4.x; rows[4 * q + 1] = r4.y; rows[4 * q + 2] = r4.z; rows[4 * q + 3] = r4.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < IT; ++j) rows[j] = (j < cnt) ? ri[k0 + j] : -1;
    }
  }
};
// ci and values of a lane's IT consecutive entries (16-byte loads when whole)
template <int IT>
__device__ __forceinline__ void load_cols(const int* __restrict__ ci, long k0, int cnt, int (&c)[IT]) {
  if (cnt == IT && IT % 4 == 0) {
#pragma unroll
    for (int q = 0; q < IT / 4; ++q) {
      const int4 c4 = __ldg(reinterpret_cast<const int4*>(ci + k0) + q);
      c[4 * q] = c4.x; c[4 * q + 1] = c4.y; c[4 * q + 2] = c4.z; c[4 * q + 3] = c4.w;
    }
  } else {
#pragma unroll
    for (int j = 0; j < IT; ++j) c[j] = (j < cnt) ? ci[k0 + j] : 0;
  }
}
template <int IT, class V>
__device__ __forceinline__ void load_vals(const V* __restrict__ val, long k0, int cnt, V (&vv)[IT]) {
  if constexpr (std::is_same<V, double>::value) {
    if (cnt == IT && IT % 2 == 0) {
#pragma unroll
      for (int q = 0; q < IT / 2; ++q) {
        const double2 d2 = __ldg(reinterpret_cast<const double2*>(val + k0) + q);
        vv[2 * q] = d2.x; vv[2 * q + 1] = d2.y;
      }
      return;
    }
  } else if constexpr (std::is_same<V, float>::value) {
    if (cnt == IT && IT % 4 == 0) {
#pragma unroll
      for (int q = 0; q < IT / 4; ++q) {
        const float4 f4 = __ldg(reinterpret_cast<const float4*>(val + k0) + q);
        vv[4 * q] = f4.x; vv[4 * q + 1] = f4.y; vv[4 * q + 2] = f4.z; vv[4 * q + 3] = f4.w;
      }
      return;
    }
  }
#pragma unroll
  for (int j = 0; j < IT; ++j) vv[j] = (j < cnt) ? val[k0 + j] : V(0);
}

// Segmented-reduction SpMV for COO (user_module.f90:525-585 computes the same
// sums by a serial scatter-add).  The
// entries are row-sorted (COO: the caller's order inside a row); every warp
// takes a fixed share of kCooWarpNnz entries, whatever the row lengths, and
// each lane IT consecutive ones: the lane sums its runs of equal rows
// sequentially (one FMA per entry; GB300's FP64 pipe is narrow), rows that
// start and end inside the lane are written at once, and one shuffle
// segmented scan over the lanes' last runs joins rows that cross lanes.
// A share's first row, when it began in an earlier share, leaves its partial
// sum in carry[2w]; its last row, when it continues into a later share,
// leaves it in carry[2w+1] and this share owns it: k_seg_fix adds the later
// shares' partials in order.
template <class T, class V, class Rows>
__global__ void __launch_bounds__(256) k_seg_reduce(long nnz, long nwarps, Rows R,
                                                    const int* __restrict__ ci, const V* __restrict__ val,
                                                    const T* __restrict__ x, T* __restrict__ y, T a, T cv,
                                                    const T* __restrict__ v, T cx, T cu,
                                                    const T* __restrict__ u, T* __restrict__ carry,
                                                    const int* __restrict__ skip) {
  if (skip && *skip) return;
  constexpr int IT = kCooWarpNnz / 32;
  const int lane = threadIdx.x & 31;
  const long w = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  if (w >= nwarps) return;  // whole warp
  const long beg = w * (long)kCooWarpNnz;
  const long end = min(nnz, beg + kCooWarpNnz);
  const int row_first = R.find(beg);
  const int row_last = R.find(end - 1);
  const bool first_open = R.first_open(beg, row_first);
  const bool last_open = R.last_open(end, nnz, row_last);
  const long k0 = beg + (long)lane * IT;
  const int cnt = (int)max(0L, min((long)IT, end - k0));
  int rows[IT], cols[IT];
  V vals[IT];
  R.rows_of(k0, cnt, row_first, row_last, rows);
  load_cols(ci, k0, cnt, cols);
  load_vals(val, k0, cnt, vals);
  T prod[IT];
#pragma unroll
  for (int j = 0; j < IT; ++j) prod[j] = (j < cnt) ? mulvt(vals[j], x[cols[j]]) : T(0);
  // runs of equal rows inside the lane
  const int head_row = (cnt > 0) ? rows[0] : -2 - lane;  // distinct sentinel for an empty lane
  int cur = head_row;
  T acc = T(0), head = T(0);
  bool multi = false;
#pragma unroll
  for (int j = 0; j < IT; ++j) {
    if (j < cnt) {
      if (rows[j] != cur) {
        if (!multi) {
          head = acc;  // the lane's first run may continue an earlier lane's row
          multi = true;
        } else {
          y[cur] = epilogue(acc, cur, a, cv, v, cx, cu, u, x);  // starts and ends in this lane
        }
        cur = rows[j];
        acc = prod[j];
      } else {
        acc = acc + prod[j];
      }
    }
  }
  const int tail_row = cur;
  // segmented inclusive scan of the lanes' last runs, keyed by their row
  T sc = acc;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T su = shfl_up_t(sc, d);
    const int ku = __shfl_up_sync(0xffffffffu, tail_row, d);
    if (lane >= d && ku == tail_row) sc = sc + su;
  }
  const T prev = shfl_up_t(sc, 1);
  const int prev_row = __shfl_up_sync(0xffffffffu, tail_row, 1);
  const int next_head = __shfl_down_sync(0xffffffffu, head_row, 1);
  if (multi) {  // the head run ends inside this lane
    const T tot = (lane > 0 && prev_row == head_row) ? head + prev : head;
    if (head_row == row_first && first_open) carry[2 * w] = tot;
    else y[head_row] = epilogue(tot, head_row, a, cv, v, cx, cu, u, x);
  }
  const bool last_lane = (cnt > 0) && (k0 + cnt == end);
  if (cnt > 0 && (last_lane || next_head != tail_row)) {  // the tail run ends here
    if (tail_row == row_first && first_open) carry[2 * w] = sc;
    else if (last_lane && last_open) carry[2 * w + 1] = sc;
    else y[tail_row] = epilogue(sc, tail_row, a, cv, v, cx, cu, u, x);
  }
}

// Rows spanning shares: the share where a row starts (and runs on) adds the
// first-row partials of the following shares in order.
template <class T, class Rows>
__global__ void __launch_bounds__(256) k_seg_fix(long nnz, long nwarps, Rows R,
                                                 const int* __restrict__ rp, const T* __restrict__ carry,
                                                 const T* __restrict__ x, T* __restrict__ y, T a, T cv,
                                                 const T* __restrict__ v, T cx, T cu,
                                                 const T* __restrict__ u, const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int lane = threadIdx.x & 31;
  const long w = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  if (w >= nwarps) return;
  const long beg = w * (long)kCooWarpNnz;
  const long end = min(nnz, beg + kCooWarpNnz);
  const int row = R.find(end - 1);
  if (!R.last_open(end, nnz, row)) return;
  const int row_first = R.find(beg);
  if (row_first == row && R.first_open(beg, row_first)) return;  // middle share: not the owner
  const long wlast = ((long)rp[row + 1] - 1) / kCooWarpNnz;  // share holding the row's last entry
  T sum = T(0);
  for (long q = w + 1 + lane; q <= wlast; q += 32) sum = sum + carry[2 * q];
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) sum = sum + shfl_x(sum, m);
  if (lane == 0) y[row] = epilogue(carry[2 * w + 1] + sum, row, a, cv, v, cx, cu, u, x);
}

template <class T>
__global__ void k_empty_rows(int n_empty, const int* __restrict__ rows, const T* __restrict__ x,
                             T* __restrict__ y, T a, T cv, const T* __restrict__ v, T cx, T cu,
                             const T* __restrict__ u, const int* __restrict__ skip) {
  if (skip && *skip) return;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n_empty; q += gridDim.x * blockDim.x) {
    const int row = rows[q];
    y[row] = epilogue(T(0), row, a, cv, v, cx, cu, u, x);
  }
}

// CDS: w(i) = sum_d band(i,d) * x(i+d)  (user_module.f90:728-733)
template <class T, class V>
__global__ void __launch_bounds__(256) k_cds(int n, int hb, const V* __restrict__ band,
                                             const T* __restrict__ x, T* __restrict__ y, T a, T cv,
                                             const T* __restrict__ v, T cx, T cu,
                                             const T* __restrict__ u, const int* __restrict__ skip) {
  if (skip && *skip) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x) {
    T s = T(0);
    for (int d = -hb; d <= hb; ++d) {
      long j = i + d;
      if (j >= 0 && j < n) s = s + mulvt(band[i + (long)n * (d + hb)], x[j]);
    }
    T out = a * s;
    if (cx != T(0)) out = out + cx * x[i];
    if (u) out = out + cu * u[i];
    if (v) out = out + cv * v[i];
    y[i] = out;
  }
}

// Dense column-major (user_module.f90:587-606), one thread per row.
template <class T, class V>
__global__ void __launch_bounds__(256) k_dense(int nrows, int ncols, const V* __restrict__ mat,
                                               const T* __restrict__ x, T* __restrict__ y, T a,
                                               T cv, const T* __restrict__ v, T cx, T cu,
                                               const T* __restrict__ u,
                                               const int* __restrict__ skip) {
  if (skip && *skip) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nrows; i += gridDim.x * (long)blockDim.x) {
    T s = T(0);
    for (long j = 0; j < ncols; ++j) s = s + mulvt(mat[i + (long)nrows * j], x[j]);
    T out = a * s;
    if (cx != T(0)) out = out + cx * x[i];
    if (u) out = out + cu * u[i];
    if (v) out = out + cv * v[i];
    y[i] = out;
  }
}

template <class T, class V, class Rows>
static void launch_seg_reduce(const MatView& M, Rows R, const V* val, const T* x, T* y, T a, T cv,
                              const T* v, T cx, T cu, const T* u, const int* skip, cudaStream_t st) {
  const long warps = (M.nnz + kCooWarpNnz - 1) / kCooWarpNnz;
  if (warps > 0) {
    const long blocks = (warps * 32 + kThreads - 1) / kThreads;
    k_seg_reduce<T, V, Rows><<<(unsigned)blocks, kThreads, 0, st>>>(M.nnz, warps, R, M.ci, val, x, y, a, cv, v, cx,
                                                                     cu, u, (T*)M.carry, skip);
    IDRS_LAUNCH_CHECK();
    k_seg_fix<T, Rows><<<(unsigned)blocks, kThreads, 0, st>>>(M.nnz, warps, R, M.rp, (const T*)M.carry, x, y, a,
                                                              cv, v, cx, cu, u, skip);
    IDRS_LAUNCH_CHECK();
  }
  if (M.n_empty > 0) {
    k_empty_rows<T><<<stream_grid(M.n_empty), kThreads, 0, st>>>(M.n_empty, M.empty_rows, x, y, a, cv, v, cx, cu,
                                                                 u, skip);
    IDRS_LAUNCH_CHECK();
  }
}

// A side stream of the calling thread on the current device, with the two
// events that fork it from and join it to a caller's stream (a pattern a
// stream capture records too).  IDRS_CRS_OVERLAP=0 in the environment keeps
// every bin on the caller's stream (read once per process; for comparisons).
struct SideStream {
  int dev = -1;
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
static bool side_stream(SideStream*& out) {
  static const bool on = [] {
    const char* e = getenv("IDRS_CRS_OVERLAP");
    return !(e && e[0] == '0');
  }();
  if (!on) return false;
  static thread_local SideStream ss;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (ss.dev != dev) {
    if (ss.s) {
      cudaStreamDestroy(ss.s);
      cudaEventDestroy(ss.fork);
      cudaEventDestroy(ss.join);
      ss = SideStream{};
    }
    if (cudaStreamCreateWithFlags(&ss.s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ss.fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ss.join, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      ss = SideStream{};
      return false;
    }
    ss.dev = dev;
  }
  out = &ss;
  return true;
}

template <class T, class V>
static void launch_crs(const MatView& M, const V* val, const T* x, T* y, T a, T cv, const T* v,
                       T cx, T cu, const T* u, const int* skip, cudaStream_t st) {
  if (M.format == FMT_COO && M.ri) {
    launch_seg_reduce<T, V>(M, RowsStored{M.ri, M.rp}, val, x, y, a, cv, v, cx, cu, u, skip, st);
    return;
  }
  long rows_per_block = kThreads / M.group;
  long need = (M.nrows + rows_per_block - 1) / rows_per_block;
  int grid = (int)std::max(1L, std::min(need, (long)num_sms() * 8));
  const int max_len = (M.bin_short > 0) ? M.bin_short : INT_MAX;
  // the long bin writes rows of its own: it runs beside the short and middle
  // bins on a side stream forked here and joined at the end
  auto launch_long = [&](cudaStream_t ls) {
    const long sb = ((long)M.n_seg * 32 + kThreads - 1) / kThreads;
    k_crs_seg<T, V><<<(unsigned)sb, kThreads, 0, ls>>>(M.n_seg, M.n_long, M.long_rows, M.seg_ptr, M.rp, M.ci, val,
                                                       x, (T*)M.partial, skip);
    IDRS_LAUNCH_CHECK();
    const long fb = ((long)M.n_long * 32 + kThreads - 1) / kThreads;
    k_crs_fin<T><<<(unsigned)fb, kThreads, 0, ls>>>(M.n_long, M.long_rows, M.seg_ptr, (const T*)M.partial, x, y,
                                                    a, cv, v, cx, cu, u, skip);
  };
  SideStream* side = nullptr;
  const bool forked = M.n_long > 0 && side_stream(side);
  if (forked) {
    IDRS_CUDA(cudaEventRecord(side->fork, st));
    IDRS_CUDA(cudaStreamWaitEvent(side->s, side->fork, 0));
    launch_long(side->s);
    IDRS_LAUNCH_CHECK();
  }
  if (M.group == 1) {
    k_crs_row<T, V><<<stream_grid(M.nrows), kThreads, 0, st>>>(M.nrows, M.rp, M.ci, val, x, y, a, cv, v, cx, cu,
                                                               u, skip, max_len);
  } else {
    switch (M.group) {
      case 2: k_crs<2><<<grid, kThreads, 0, st>>>(M.nrows, M.rp, M.ci, val, x, y, a, cv, v, cx, cu, u, skip, max_len); break;
      case 4: k_crs<4><<<grid, kThreads, 0, st>>>(M.nrows, M.rp, M.ci, val, x, y, a, cv, v, cx, cu, u, skip, max_len); break;
      case 8: k_crs<8><<<grid, kThreads, 0, st>>>(M.nrows, M.rp, M.ci, val, x, y, a, cv, v, cx, cu, u, skip, max_len); break;
      case 16: k_crs<16><<<grid, kThreads, 0, st>>>(M.nrows, M.rp, M.ci, val, x, y, a, cv, v, cx, cu, u, skip, max_len); break;
      default: k_crs<32><<<grid, kThreads, 0, st>>>(M.nrows, M.rp, M.ci, val, x, y, a, cv, v, cx, cu, u, skip, max_len); break;
    }
  }
  if (M.n_med > 0) {
    IDRS_LAUNCH_CHECK();
    const long mb = std::min(((long)M.n_med * kBinLanes + kThreads - 1) / kThreads, (long)num_sms() * 16);
    k_crs_list<kBinLanes, T, V><<<(unsigned)std::max(mb, 1L), kThreads, 0, st>>>(
        M.n_med, M.med_rows, M.rp, M.ci, val, x, y, a, cv, v, cx, cu, u, skip);
  }
  if (forked) {  // the caller counts and checks the last launch on st
    IDRS_CUDA(cudaEventRecord(side->join, side->s));
    IDRS_CUDA(cudaStreamWaitEvent(st, side->join, 0));
  } else if (M.n_long > 0) {
    IDRS_LAUNCH_CHECK();
    launch_long(st);
  }
}

template <class T, class V>
static void launch_valued(const MatView& M, const V* val, const T* x, T* y, T a, T cv, const T* v,
                          T cx, T cu, const T* u, const int* skip, cudaStream_t st) {
  switch (M.format) {
    case FMT_CRS:
    case FMT_COO:
      launch_crs<T, V>(M, val, x, y, a, cv, v, cx, cu, u, skip, st);
      break;
    case FMT_CDS:
      k_cds<T, V><<<stream_grid(M.nrows), kThreads, 0, st>>>(M.nrows, M.hb, val, x, y, a, cv, v, cx, cu, u, skip);
      break;
    case FMT_DENSE:
      k_dense<T, V><<<stream_grid(M.nrows), kThreads, 0, st>>>(M.nrows, M.ncols, val, x, y, a, cv, v, cx, cu, u, skip);
      break;
    default:
      throw std::runtime_error("spmv: unsupported format");
  }
}

template <class T>
static void launch_stencil(const MatView& M, const T* x, T* y, T a, T cv, const T* v, T cx, T cu,
                           const T* u, const int* skip, cudaStream_t st) {
  using R = typename traits<T>::real;
  dim3 blk(32, 8, 1);
  int gx = (M.nx + 31) / 32, gy = (M.ny + 7) / 8;
  long xy = (long)gx * gy;
  long target = (long)num_sms() * 8;
  int zc = (int)std::max(1L, std::min((long)M.nz, (M.nz * xy + target - 1) / target));
  if (zc < 4 && M.nz >= 4) zc = 4;  // keep some register reuse along z
  int gz = (M.nz + zc - 1) / zc;
  dim3 grid(gx, gy, gz);
  const bool real_a = (imag_(a) == 0) && (imag_(cx) == 0);
  if constexpr (std::is_same<T, float>::value) {
    if (M.nx % 4 == 0 && aligned16(x) && aligned16(y) && aligned16(u) && aligned16(v)) {
      dim3 blk4(32, kF4Rows, 1);
      int gx4 = (M.nx + 127) / 128, gy4 = (M.ny + kF4Rows - 1) / kF4Rows;
      long xy4 = (long)gx4 * gy4;
      int zc4 = (int)std::max(1L, std::min((long)M.nz, (M.nz * xy4 + target - 1) / target));
      if (zc4 < 4 && M.nz >= 4) zc4 = 4;
      dim3 grid4(gx4, gy4, (M.nz + zc4 - 1) / zc4);
      const double ar = (double)a;
      launch_pdl(k_stencil7_f4, grid4, blk4, 0, st, M.nx, M.ny, M.nz, zc4, float(ar * M.st[0] + (double)cx),
                 float(ar * M.st[1]), float(ar * M.st[2]), float(ar * M.st[3]), float(ar * M.st[4]),
                 float(ar * M.st[5]), float(ar * M.st[6]), x, y, cv, v, cu, u, skip);
      return;
    }
  }
  if (real_a) {  // fold the real scale (and the centre term cx*x) into the coefficients
    double ar = (double)real_(a);
    double c0 = ar * M.st[0] + (double)real_(cx);
    k_stencil7<T, R, false><<<grid, blk, 0, st>>>(
        M.nx, M.ny, M.nz, zc, R(c0), R(ar * M.st[1]), R(ar * M.st[2]), R(ar * M.st[3]),
        R(ar * M.st[4]), R(ar * M.st[5]), R(ar * M.st[6]), x, y, a, cv, v, cu, u, skip);
  } else {
    if (cx != T(0)) throw std::runtime_error("stencil: complex centre term unsupported");
    k_stencil7<T, R, true><<<grid, blk, 0, st>>>(
        M.nx, M.ny, M.nz, zc, R(M.st[0]), R(M.st[1]), R(M.st[2]), R(M.st[3]), R(M.st[4]),
        R(M.st[5]), R(M.st[6]), x, y, a, cv, v, cu, u, skip);
  }
}

template <class T>
void spmv_ex(const MatView& M, const T* x, T* y, const Epi<T>& e, const int* skip, cudaStream_t st) {
  using R = typename traits<T>::real;
  using C = cplx<R>;
  if (M.format == FMT_STENCIL7) {
    launch_stencil<T>(M, x, y, e.a, e.cv, e.v, e.cx, e.cu, e.u, skip, st);
  } else if (M.vcplx) {
    if constexpr (traits<T>::is_cplx) launch_valued<T, C>(M, (const C*)M.val, x, y, e.a, e.cv, e.v, e.cx, e.cu, e.u, skip, st);
    else throw std::runtime_error("spmv: complex matrix applied to a real vector");
  } else {
    launch_valued<T, R>(M, (const R*)M.val, x, y, e.a, e.cv, e.v, e.cx, e.cu, e.u, skip, st);
  }
  IDRS_LAUNCH_CHECK();
}

template <class T>
void spmv(const MatView& M, const T* x, T* y, T a, T cv, const T* v, const int* skip,
          cudaStream_t st) {
  Epi<T> e;
  e.a = a;
  e.cv = cv;
  e.v = v;
  spmv_ex<T>(M, x, y, e, skip, st);
}

// ---------------------------------------------------------------------------
// Horner chain (rpolpre + real_mv, matrix_module.f90:152-167, 266-284)
// ---------------------------------------------------------------------------
template <class T> static inline T narrow_c(c128 v) { return narrow<T>(v); }

template <class T>
void ks_mv(const MatView& Ks, const T* x, T* y, T a, T cv, const T* v, const int* skip,
           cudaStream_t st) {
  if constexpr (sizeof(typename traits<T>::real) == 8) {
    if (Ks.lu && Ks.si_C) {
      block_si_precon<T>(Ks, Ks.nrows / 2, x, (T*)Ks.lu_tmp, skip, st);
      x = (const T*)Ks.lu_tmp;
    } else if (Ks.lu) {
      lu_solve<T>(*Ks.lu, x, (T*)Ks.lu_tmp, skip, st);
      x = (const T*)Ks.lu_tmp;
    }
  }
  spmv<T>(Ks, x, y, a, cv, v, skip, st);
}

// The last product of a chain: w = fa * Pmul(Ks u) + fcv * fv (Pmul only with
// a deflated fp64 operator).
template <class T>
static void chain_last(const MatView& Ks, const T* u, T* w, T fa, T fcv, const T* fv, const int* skip,
                       cudaStream_t st) {
  if constexpr (sizeof(typename traits<T>::real) == 8) {
    if (Ks.defl && Ks.defl->k > 0) {
      T* tmp = (T*)Ks.defl->tmp;
      ks_mv<T>(Ks, u, tmp, T(1), T(0), nullptr, skip, st);
      deflation_pmul<T>(*Ks.defl, tmp, w, fa, fcv, fv, skip, st);
      return;
    }
  }
  ks_mv<T>(Ks, u, w, fa, fcv, fv, skip, st);
}

template <class T>
void op_chain(const MatView& Ks, const std::vector<c128>& alpha, int degree, const T* v, T* w,
              T* t1, T* t2, const int* skip, cudaStream_t st, T fa, T fcv, const T* fv) {
  if (degree == 0) {
    chain_last<T>(Ks, v, w, fa, fcv, fv, skip, st);
    return;
  }
  // u_{d-1} = Ks (alpha_d v) + alpha_{d-1} v
  ks_mv<T>(Ks, v, t1, narrow_c<T>(alpha[degree]), narrow_c<T>(alpha[degree - 1]), v, skip, st);
  T* cur = t1;
  T* nxt = t2;
  for (int k = degree - 2; k >= 0; --k) {
    ks_mv<T>(Ks, cur, nxt, T(1), narrow_c<T>(alpha[k]), v, skip, st);
    std::swap(cur, nxt);
  }
  chain_last<T>(Ks, cur, w, fa, fcv, fv, skip, st);
}

// One step of a polynomial chain: out = Epi(Ks in).
template <class T>
struct ChainStep {
  const T* in;
  T* out;
  Epi<T> e;
};

static int f4x2_resident() {
  static const int b = [] {
    int r = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_stencil7_f4x2, 64 * kX2Halo, 0) != cudaSuccess) r = 0;
    return r > 0 ? r : 1;
  }();
  return b;
}

// The staged pair (k_stencil7_f8x2t) for this nx on the current device:
// resident blocks per SM, or 0 when it cannot run (shared memory) or
// IDRS_STAGED_PAIR=0 asks for the unstaged kernel.
static int f8x2t_resident(int nx) {
  static const bool enabled = [] {
    const char* e = getenv("IDRS_STAGED_PAIR");
    return !(e && e[0] == '0');
  }();
  if (!enabled) return 0;
  static std::mutex mu;
  static std::atomic<uint64_t> attr_set{0};
  static int cache_dev = -1, cache_nx = -1, cache_r = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  std::lock_guard<std::mutex> lock(mu);
  if (dev == cache_dev && nx == cache_nx) return cache_r;
  const uint64_t bit = dev < 64 ? uint64_t(1) << dev : 0;
  if (!bit || !(attr_set.load() & bit)) {
    bool ok = true;
    for (auto kern : {k_stencil7_f8x2t<0, 0>, k_stencil7_f8x2t<0, 1>, k_stencil7_f8x2t<0, 2>,
                      k_stencil7_f8x2t<kX2MaxNx, 0>, k_stencil7_f8x2t<kX2MaxNx, 1>, k_stencil7_f8x2t<kX2MaxNx, 2>})
      ok = ok && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)t8_smem(kX2MaxNx)) ==
                     cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      return 0;
    }
    attr_set.fetch_or(bit);
  }
  int r = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &r, nx == kX2MaxNx ? k_stencil7_f8x2t<kX2MaxNx, 1> : k_stencil7_f8x2t<0, 1>, 32 * kX8Halo, t8_smem(nx)) !=
      cudaSuccess) {
    cudaGetLastError();
    r = 0;
  }
  cache_dev = dev;
  cache_nx = nx;
  cache_r = r;
  return r;
}

static int f8x2_resident() {
  static const int b = [] {
    int r = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_stencil7_f8x2, 32 * kX8Halo, 0) != cudaSuccess) r = 0;
    return r > 0 ? r : 1;
  }();
  return b;
}

// Can two fp32 steps share one k_stencil7_f4x2 pass?
static bool f4x2_ok(const MatView& M, const ChainStep<float>& A, const ChainStep<float>& B) {
  if (M.format != FMT_STENCIL7 || M.nx % 4 != 0 || M.nx > kX2MaxNx) return false;
  if (B.in != A.out || (B.e.u && B.e.u != A.in)) return false;
  // B writes while A still reads: its output must not be one of A's inputs
  if (B.out == A.in || (A.e.u && B.out == A.e.u) || (A.e.v && B.out == A.e.v) ||
      (B.e.v && (B.out == B.e.v || A.out == B.e.v)))
    return false;
  for (const void* q : {(const void*)A.in, (const void*)A.out, (const void*)A.e.u, (const void*)A.e.v,
                        (const void*)B.out, (const void*)B.e.v})
    if (!aligned16(q)) return false;
  return true;
}

static St7 st7_of(const MatView& M, float a, float cx) {
  const double ar = (double)a;
  return St7{float(ar * M.st[0] + (double)cx), float(ar * M.st[1]), float(ar * M.st[2]), float(ar * M.st[3]),
             float(ar * M.st[4]), float(ar * M.st[5]), float(ar * M.st[6])};
}

template <class T>
static void run_chain(const MatView& Ks, const std::vector<ChainStep<T>>& steps, const int* skip, cudaStream_t st) {
  size_t k = 0;
  while (k < steps.size()) {
    if constexpr (std::is_same<T, float>::value) {
      if (k + 1 < steps.size() && f4x2_ok(Ks, steps[k], steps[k + 1])) {
        const ChainStep<float>& A = steps[k];
        const ChainStep<float>& B = steps[k + 1];
        // A's output goes to HBM only if a later step reads it before it is overwritten
        bool need = false;
        for (size_t q = k + 2; q < steps.size(); ++q) {
          if (steps[q].in == A.out || steps[q].e.u == A.out) { need = true; break; }
          if (steps[q].out == A.out) break;
        }
        const int gy = (Ks.ny + kX2Rows - 1) / kX2Rows;
        const int staged = Ks.nx % 8 == 0 ? f8x2t_resident(Ks.nx) : 0;
        if (staged > 0) {
          const long target = 2L * num_sms() * staged;
          const long chunks = std::max(1L, std::min((long)Ks.nz, (target + gy - 1) / gy));
          const int zc = (int)std::max(4L, ((long)Ks.nz + chunks - 1) / chunks);
          dim3 blk(32, kX8Halo, 1);
          dim3 grid((Ks.ny + kX8Rows - 1) / kX8Rows, (Ks.nz + zc - 1) / zc, 1);
          // step B's vb: step A's v, step A's xin, or a vector of its own
          const int vbm = (B.e.v && B.e.v == A.e.v) ? 1 : (B.e.v && B.e.v == A.in) ? 2 : 0;
          const bool c256 = Ks.nx == kX2MaxNx;
          auto kern = vbm == 1 ? (c256 ? k_stencil7_f8x2t<kX2MaxNx, 1> : k_stencil7_f8x2t<0, 1>)
                    : vbm == 2 ? (c256 ? k_stencil7_f8x2t<kX2MaxNx, 2> : k_stencil7_f8x2t<0, 2>)
                               : (c256 ? k_stencil7_f8x2t<kX2MaxNx, 0> : k_stencil7_f8x2t<0, 0>);
          launch_pdl(kern, grid, blk, t8_smem(Ks.nx), st, Ks.nx, Ks.ny, Ks.nz, zc, st7_of(Ks, A.e.a, A.e.cx),
                     A.e.u ? A.e.cu : 0.f, A.e.v ? A.e.cv : 0.f, st7_of(Ks, B.e.a, B.e.cx),
                     B.e.u ? B.e.cu : 0.f, B.e.v ? B.e.cv : 0.f, A.in, A.e.u, A.e.v,
                     vbm == 0 ? B.e.v : nullptr, need ? A.out : nullptr, B.out, skip, device_fault_word());
          IDRS_LAUNCH_CHECK();
          k += 2;
          continue;
        }
        if (Ks.nx % 8 == 0) {
          const long target = 2L * num_sms() * f8x2_resident();
          const long chunks = std::max(1L, std::min((long)Ks.nz, (target + gy - 1) / gy));
          const int zc = (int)std::max(4L, ((long)Ks.nz + chunks - 1) / chunks);
          dim3 blk(32, kX8Halo, 1);
          dim3 grid((Ks.ny + kX8Rows - 1) / kX8Rows, (Ks.nz + zc - 1) / zc, 1);
          k_stencil7_f8x2<<<grid, blk, 0, st>>>(
              Ks.nx, Ks.ny, Ks.nz, zc, st7_of(Ks, A.e.a, A.e.cx), A.e.u ? A.e.cu : 0.f,
              A.e.v ? A.e.cv : 0.f, st7_of(Ks, B.e.a, B.e.cx), B.e.u ? B.e.cu : 0.f, B.e.v ? B.e.cv : 0.f,
              A.in, A.e.u, A.e.v, B.e.v, need ? A.out : nullptr, B.out, skip);
          IDRS_LAUNCH_CHECK();
          k += 2;
          continue;
        }
        // two full waves of resident blocks (each SM holds f4x2_resident() blocks)
        const long target = 2L * num_sms() * f4x2_resident();
        const long chunks = std::max(1L, std::min((long)Ks.nz, (target + gy - 1) / gy));
        int zc = (int)std::max(4L, ((long)Ks.nz + chunks - 1) / chunks);
        dim3 blk(32 * ((Ks.nx + 127) / 128), kX2Halo, 1);
        dim3 grid(gy, (Ks.nz + zc - 1) / zc, 1);
        k_stencil7_f4x2<<<grid, blk, 0, st>>>(
            Ks.nx, Ks.ny, Ks.nz, zc, st7_of(Ks, A.e.a, A.e.cx), A.e.u ? A.e.cu : 0.f, A.e.v ? A.e.cv : 0.f,
            st7_of(Ks, B.e.a, B.e.cx), B.e.u ? B.e.cu : 0.f, B.e.v ? B.e.cv : 0.f, A.in, A.e.u, A.e.v, B.e.v,
            need ? A.out : nullptr, B.out, skip);
        IDRS_LAUNCH_CHECK();
        k += 2;
        continue;
      }
    }
    spmv_ex<T>(Ks, steps[k].in, steps[k].out, steps[k].e, skip, st);
    ++k;
  }
}

// A p(A) v with p evaluated through the three-term recurrence of its
// tridiagonal Jacobi matrix (Chebyshev / Neumann, matrix_module.f90:851-941)
// instead of monomial Horner.  With r_i(t) = 1 - t p_i(t) and column i of J
// holding (a_i, b_i, c_i) = (J(i-1,i), J(i,i), J(i+1,i)), a_i + b_i + c_i = 0:
//   y_0 = 0,  y_1 = -v / c_1,
//   y_i = (A y_{i-1} - b_i y_{i-1} - a_i y_{i-2} - v) / c_i ,  i = 2..d+1
// and p(A) v = y_{d+1}.  The iterates stay of the size of A^-1 v, so the fp32
// form keeps its accuracy where the monomial coefficients (|alpha| ~ 10^3-10^4
// with alternating signs for a degree-8 Chebyshev polynomial) cancel.
// fp32 stencil chains run two steps per pass (k_stencil7_f4x2).
// The steps y_2 .. y_{d+1} of the recurrence (degree d >= 1), y_i written
// to buf[(i - 2) % nbuf]; `last` (if given) receives y_{d+1} instead.
template <class T>
static std::vector<ChainStep<T>> recur_steps(const JacobiCols& J, int degree, const T* v, T* const* buf,
                                             int nbuf, T* last) {
  auto C = [](c128 z) { return narrow<T>(z); };
  std::vector<ChainStep<T>> steps;
  const T* ym2 = nullptr;  // y_{i-2}
  const T* ym1 = nullptr;  // y_{i-1}
  {
    // y_1 = -v/c_1 ; y_2 = (A y_1 - b_2 y_1 - v)/c_2 read from v alone
    c128 c1 = J.c[0], b2 = J.b[1], c2 = J.c[1];
    c128 s1 = c128(-1.0) / c1;  // y_1 = s1 v, kept implicit
    ChainStep<T> s0{v, buf[0], Epi<T>()};
    s0.e.a = C(s1 / c2);                                   // (A y_1)/c2
    s0.e.cx = C((c128(0.0) - b2 * s1 - c128(1.0)) / c2);  // (-b2 y_1 - v)/c2, y_1 and v share v
    steps.push_back(s0);
    ym1 = buf[0];
  }
  int nb = 1;
  for (int i = 3; i <= degree + 1; ++i) {
    c128 ai = J.a[i - 1], bi = J.b[i - 1], ci = J.c[i - 1];
    ChainStep<T> sk{ym1, buf[nb % nbuf], Epi<T>()};
    sk.e.a = C(c128(1.0) / ci);
    sk.e.cx = C(c128(0.0) - bi / ci);
    sk.e.cv = C(c128(-1.0) / ci);
    sk.e.v = v;
    if (i == 3) {  // y_{i-2} = y_1 = s1 v: fold into the v term
      c128 s1 = c128(-1.0) / J.c[0];
      sk.e.cv = C((c128(-1.0) - ai * s1) / ci);
    } else if (ai != c128(0.0)) {  // Neumann: a_i = 0, no y_{i-2} read
      sk.e.cu = C(c128(0.0) - ai / ci);
      sk.e.u = ym2;
    }
    steps.push_back(sk);
    ym2 = ym1;
    ym1 = sk.out;
    ++nb;
  }
  if (last) steps.back().out = last;
  return steps;
}

template <class T>
void op_chain_recur(const MatView& Ks, const JacobiCols& J, int degree, const T* v, T* w, T* t1,
                    T* t2, T* t3, T* t4, const int* skip, cudaStream_t st, T fa, T fcv, const T* fv) {
  if (degree == 0) {
    spmv<T>(Ks, v, w, fa, fcv, fv, skip, st);
    return;
  }
  T* buf[4] = {t1, t2, t3, t4};
  std::vector<ChainStep<T>> steps = recur_steps<T>(J, degree, v, buf, t4 ? 4 : 3, nullptr);
  ChainStep<T> fin{steps.back().out, w, Epi<T>()};
  fin.e.a = fa;
  fin.e.cv = fcv;
  fin.e.v = fv;
  steps.push_back(fin);
  run_chain<T>(Ks, steps, skip, st);
}

template <class T>
const T* op_chain_recur_head(const MatView& Ks, const JacobiCols& J, int degree, const T* v, T* t1, T* t2, T* t3,
                             T* t4, const int* skip, cudaStream_t st) {
  if (degree == 0) return v;
  T* buf[4] = {t1, t2, t3, t4};
  const std::vector<ChainStep<T>> steps = recur_steps<T>(J, degree, v, buf, t4 ? 4 : 3, nullptr);
  run_chain<T>(Ks, steps, skip, st);
  return steps.back().out;
}

template <class T>
void op_apply(Operator& A, int prec, const T* v, T* w, T* t1, T* t2, T* t3, T* t4, const int* skip,
              cudaStream_t st, T fa, T fcv, const T* fv) {
  const MatView& Ks = A.view(prec);
  if (use_recurrence(A, prec) && t3)
    op_chain_recur<T>(Ks, A.jac, A.degree, v, w, t1, t2, t3, t4, skip, st, fa, fcv, fv);
  else
    op_chain<T>(Ks, A.alpha_p, A.degree, v, w, t1, t2, skip, st, fa, fcv, fv);
}

// ---------------------------------------------------------------------------
// elementwise kernels
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_copy(long n, const T* __restrict__ a, T* __restrict__ b, const int* skip) {
  if (skip && *skip) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x) b[i] = a[i];
}
template <class T, class D>
__global__ void k_scale_vec(long n, const D* __restrict__ d, const T* __restrict__ a, T* __restrict__ b,
                            const int* skip) {
  if (skip && *skip) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x)
    b[i] = mulvt(d[i], a[i]);
}
template <class T>
__global__ void k_scale_uniform(long n, T d, const T* __restrict__ a, T* __restrict__ b, const int* skip) {
  if (skip && *skip) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x)
    b[i] = d * a[i];
}
template <class Tin, class Tout>
__global__ void k_convert(long n, const Tin* __restrict__ a, Tout* __restrict__ b, const int* skip) {
  if (skip && *skip) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x)
    b[i] = Tout(a[i]);
}

template <class T>
void vec_copy(long n, const T* a, T* b, const int* skip, cudaStream_t st) {
  if (a == b) return;
  k_copy<T><<<stream_grid(n), kThreads, 0, st>>>(n, a, b, skip);
  IDRS_LAUNCH_CHECK();
}
template <class Tin, class Tout>
void vec_convert(long n, const Tin* a, Tout* b, const int* skip, cudaStream_t st) {
  k_convert<Tin, Tout><<<stream_grid(n), kThreads, 0, st>>>(n, a, b, skip);
  IDRS_LAUNCH_CHECK();
}

template <class T> struct real_of_prec;
template <> struct real_of_prec<double> { using R = double; using C = c128; };
template <> struct real_of_prec<c128> { using R = double; using C = c128; };
template <> struct real_of_prec<float> { using R = float; using C = c64; };
template <> struct real_of_prec<c64> { using R = float; using C = c64; };

template <class T>
void vec_scale_vec(long n, const void* d, bool dcplx, const T* a, T* b, const int* skip,
                   cudaStream_t st) {
  using R = typename real_of_prec<T>::R;
  using C = typename real_of_prec<T>::C;
  if constexpr (traits<T>::is_cplx) {
    if (dcplx) k_scale_vec<T, C><<<stream_grid(n), kThreads, 0, st>>>(n, (const C*)d, a, b, skip);
    else k_scale_vec<T, R><<<stream_grid(n), kThreads, 0, st>>>(n, (const R*)d, a, b, skip);
  } else {
    if (dcplx) throw std::runtime_error("complex diagonal scaling of a real vector");
    k_scale_vec<T, R><<<stream_grid(n), kThreads, 0, st>>>(n, (const R*)d, a, b, skip);
  }
  IDRS_LAUNCH_CHECK();
}

template <class T>
void op_precon(Operator& A, int prec, const T* v, T* w, const int* skip, cudaStream_t st) {
  long n = A.n();
  if (A.P && (A.P->which_precon == 2 || A.P->which_precon == 3)) {
    if constexpr (sizeof(typename traits<T>::real) == 8) {
      if (A.si_C) block_si_precon<T>(A.view(64), n / 2, v, w, skip, st);
      else lu_solve<T>(*A.P, v, w, skip, st);
      return;
    } else {
      throw std::runtime_error("shift-and-invert is not available in fp32 (inner_precision 32)");
    }
  }
  if (A.dkind == 0) {
    vec_copy<T>(n, v, w, skip, st);
  } else if (A.dkind == 1) {
    k_scale_uniform<T><<<stream_grid(n), kThreads, 0, st>>>(n, narrow<T>(A.dinv_u), v, w, skip);
    IDRS_LAUNCH_CHECK();
  } else {
    if (prec == 32 && !A.dinv32) A.view(32);
    vec_scale_vec<T>(n, prec == 32 ? A.dinv32 : A.dinv64, A.dinv_cplx, v, w, skip, st);
  }
}

template <class T>
void op_scaleback(Operator& A, int prec, const std::vector<c128>& alpha, int degree, const T* y,
                  T* x, T* t1, T* t2, const int* skip, cudaStream_t st, const T* b, c128 sigma_s,
                  c128 factor) {
  const MatView& Ks = A.view(prec);
  long n = A.n();
  if constexpr (sizeof(typename traits<T>::real) == 8) {
    const bool defl = A.defl && A.defl->k > 0;
    const bool lu = A.P && (A.P->which_precon == 2 || A.P->which_precon == 3);
    if (defl || lu || factor.x != 1.0 || factor.y != 0.0) {
      if (defl && !b) throw std::runtime_error("scaleback: a deflated operator needs the right-hand side b");
      // p = polpre(y) with real_mv; add_deflation; the shift-and-invert factor; x = p / A
      const T* cur = y;
      T* bufs[2] = {t1, t2};
      int nb = 0;
      for (int k = degree - 1; k >= 0; --k) {
        T a = (k == degree - 1) ? narrow<T>(alpha[degree]) : T(1);
        T* dst = bufs[nb];
        nb ^= 1;
        ks_mv<T>(Ks, cur, dst, a, narrow<T>(alpha[k]), y, skip, st);
        cur = dst;
      }
      if (defl) {
        T* q = bufs[nb];
        nb ^= 1;
        deflation_add<T>(A, sigma_s, b, cur, q, skip, st);
        cur = q;
      }
      if (factor.x != 1.0 || factor.y != 0.0) {
        T* q = bufs[nb];
        k_scale_uniform<T><<<stream_grid(n), kThreads, 0, st>>>(n, narrow<T>(factor), cur, q, skip);
        IDRS_LAUNCH_CHECK();
        cur = q;
      }
      op_precon<T>(A, prec, cur, x, skip, st);
      return;
    }
  }
  if (degree == 0) {
    op_precon<T>(A, prec, y, x, skip, st);
    return;
  }
  T du = (A.dkind == 1) ? narrow<T>(A.dinv_u) : T(1);
  if (use_recurrence(A, prec) && alpha.data() == A.alpha_p.data() && degree == A.degree) {
    // p(Ks) y = y_{d+1} of the three-term recurrence; the rotation puts
    // y_{d+1} into x (x never holds y_d or y_{d-1} when it is written)
    T* buf[3];
    buf[(degree - 1) % 3] = x;
    buf[degree % 3] = t1;
    buf[(degree + 1) % 3] = t2;
    std::vector<ChainStep<T>> steps = recur_steps<T>(A.jac, degree, y, buf, 3, nullptr);
    if (A.dkind == 1) {
      Epi<T>& e = steps.back().e;
      e.a = e.a * du; e.cx = e.cx * du; e.cu = e.cu * du; e.cv = e.cv * du;
    }
    run_chain<T>(Ks, steps, skip, st);
    if (A.dkind == 2) {
      if (prec == 32 && !A.dinv32) A.view(32);
      vec_scale_vec<T>(n, prec == 32 ? A.dinv32 : A.dinv64, A.dinv_cplx, x, x, skip, st);
    }
    return;
  }
  const T* cur = y;
  T* bufs[2] = {t1, t2};
  int nb = 0;
  for (int k = degree - 1; k >= 0; --k) {
    T a = (k == degree - 1) ? narrow<T>(alpha[degree]) : T(1);
    T cv = narrow<T>(alpha[k]);
    T* dst;
    if (k == 0 && A.dkind != 2) {
      dst = x;
      if (A.dkind == 1) { a = a * du; cv = cv * du; }
    } else {
      dst = bufs[nb];
      nb ^= 1;
    }
    spmv<T>(Ks, cur, dst, a, cv, y, skip, st);
    cur = dst;
  }
  if (A.dkind == 2) {
    if (prec == 32 && !A.dinv32) A.view(32);
    vec_scale_vec<T>(n, prec == 32 ? A.dinv32 : A.dinv64, A.dinv_cplx, cur, x, skip, st);
  }
}

// ---------------------------------------------------------------------------
// operator build: Ks = (K - seed I) D^-1 folded into a scaled copy
// ---------------------------------------------------------------------------
template <class V, class D>
__global__ void k_scale_crs(int nrows, const int* rp, const int* ci, const V* val, const D* dinv,
                            V seed, V* out, int* missing_diag) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nrows; i += gridDim.x * (long)blockDim.x) {
    bool found = false;
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      int j = ci[k];
      V a = val ? val[k] : V(1);
      if (j == i && !found) { a = a - seed; found = true; }
      out[k] = dinv ? mulvt(dinv[j], a) : a;
    }
    if (!found && seed != V(0)) atomicAdd(missing_diag, 1);
  }
}
template <class V, class D>
__global__ void k_scale_cds(int n, int hb, const V* band, const D* dinv, V seed, V* out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x)
    for (int d = -hb; d <= hb; ++d) {
      long j = i + d;
      long k = i + (long)n * (d + hb);
      V a = band ? band[k] : V(1);
      if (d == 0) a = a - seed;
      out[k] = (dinv && j >= 0 && j < n) ? mulvt(dinv[j], a) : a;
    }
}
template <class V, class D>
__global__ void k_scale_dense(int nrows, int ncols, const V* mat, const D* dinv, V seed, V* out) {
  long tot = (long)nrows * ncols;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < tot; k += gridDim.x * (long)blockDim.x) {
    long i = k % nrows, j = k / nrows;
    V a = mat[k];
    if (i == j) a = a - seed;
    out[k] = dinv ? mulvt(dinv[j], a) : a;
  }
}
template <class D>
__global__ void k_invert(long n, const D* d, D* out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x)
    out[i] = D(1) / d[i];
}
__global__ void k_c2r(long n, const c128* a, double* b) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x) b[i] = a[i].x;
}
__global__ void k_r2c(long n, const double* a, c128* b) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x) b[i] = c128(a[i], 0.0);
}

template <class V, class D>
static void scale_values(const UserMatrix& K, const void* kval, const D* dinv, V seed, V* out,
                         cudaStream_t st, int* d_missing) {
  switch (K.format) {
    case FMT_CRS:
    case FMT_COO:
      k_scale_crs<V, D><<<stream_grid(K.nrows), kThreads, 0, st>>>(K.nrows, K.row_ptr, K.col_ind,
                                                                   (const V*)kval, dinv, seed, out, d_missing);
      break;
    case FMT_CDS:
      k_scale_cds<V, D><<<stream_grid(K.nrows), kThreads, 0, st>>>(K.nrows, K.half_band, (const V*)kval,
                                                                   dinv, seed, out);
      break;
    case FMT_DENSE:
      k_scale_dense<V, D><<<stream_grid((long)K.nrows * K.ncols), kThreads, 0, st>>>(
          K.nrows, K.ncols, (const V*)kval, dinv, seed, out);
      break;
  }
  IDRS_LAUNCH_CHECK();
}

static long value_count(const UserMatrix& K) {
  switch (K.format) {
    case FMT_CRS: case FMT_COO: return K.nnz;
    case FMT_CDS: return (long)K.nrows * (2 * K.half_band + 1);
    case FMT_DENSE: return (long)K.nrows * K.ncols;
    default: return 0;
  }
}
static const void* value_ptr(const UserMatrix& K) {
  switch (K.format) {
    case FMT_CRS: case FMT_COO: return K.val;
    case FMT_CDS: return K.band;
    case FMT_DENSE: return K.mat;
    default: return nullptr;
  }
}

int build_operator(Operator* A) {
  UserMatrix& K = *A->K;
  cudaStream_t st = A->stream;
  long n = K.nrows;
  if (A->ks_val64) { cudaFreeAsync(A->ks_val64, st); A->ks_val64 = nullptr; }
  if (A->ks_val32) { cudaFreeAsync(A->ks_val32, st); A->ks_val32 = nullptr; }
  if (A->dinv64) { cudaFreeAsync(A->dinv64, st); A->dinv64 = nullptr; }
  if (A->dinv32) { cudaFreeAsync(A->dinv32, st); A->dinv32 = nullptr; }
  A->k64 = K.view64();
  if (K.carry && !A->lb_carry) {
    const long warps = (K.nnz + kCooWarpNnz - 1) / kCooWarpNnz;
    IDRS_CUDA(cudaMallocAsync(&A->lb_carry, 2 * 16 * (size_t)std::max<long>(warps, 1), st));
  }
  if (K.n_seg > 0 && !A->lb_partial) IDRS_CUDA(cudaMallocAsync(&A->lb_partial, 16 * (size_t)K.n_seg, st));
  A->k64.partial = A->lb_partial;
  A->k64.carry = A->lb_carry;
  A->ks64 = A->k64;
  A->ks32 = MatView();
  if (A->P && (A->P->which_precon == 2 || A->P->which_precon == 3)) {
    if (A->P->nrows != (int)n) { set_error("shift-and-invert preconditioner size mismatch"); return 1; }
    if (A->P->vals == 2 && !A->cplx) { set_error("complex LU preconditioner on a real problem"); return 1; }
    if (!A->lu_tmp) IDRS_CUDA(cudaMallocAsync(&A->lu_tmp, (A->cplx ? 16 : 8) * std::max<long>(n, 1), st));
  }
  A->dkind = 0;
  A->dinv_u = c128(1.0, 0.0);
  A->dinv_cplx = false;
  // diagonal scaling
  if (A->P && A->P->which_precon == 1) {
    UserMatrix& P = *A->P;
    if (P.diag_uniform) {
      A->dkind = 1;
      A->dinv_u = c128(1.0, 0.0) / P.diag_u;
      if (!A->cplx && A->dinv_u.y != 0.0) { set_error("complex diagonal on a real problem"); return 1; }
    } else {
      A->dkind = 2;
      A->dinv_cplx = P.diag_cplx;
      if (!A->cplx && P.diag_cplx) { set_error("complex diagonal on a real problem"); return 1; }
      size_t es = P.diag_cplx ? 16 : 8;
      IDRS_CUDA(cudaMallocAsync(&A->dinv64, es * n, st));
      if (P.diag_cplx) k_invert<c128><<<stream_grid(n), kThreads, 0, st>>>(n, (const c128*)P.diag, (c128*)A->dinv64);
      else k_invert<double><<<stream_grid(n), kThreads, 0, st>>>(n, (const double*)P.diag, (double*)A->dinv64);
      IDRS_LAUNCH_CHECK();
    }
  }
  if (!A->cplx && A->seed.y != 0.0) { set_error("complex seed on a real problem"); return 1; }
  // a seed already folded into an assembled system matrix is not applied again
  const c128 es = A->seed_folded ? c128(0.0, 0.0) : A->seed;
  bool seeded = (es.x != 0.0 || es.y != 0.0);
  if (K.format == FMT_STENCIL7) {
    if (A->dkind == 2) { set_error("stencil operator: only a constant diagonal scaling is supported"); return 5; }
    if (es.y != 0.0 || A->dinv_u.y != 0.0) { set_error("stencil operator: complex seed/scaling unsupported"); return 5; }
    double du = A->dinv_u.x;
    A->ks64.st[0] = (K.st[0] - es.x) * du;
    for (int i = 1; i < 7; ++i) A->ks64.st[i] = K.st[i] * du;
    return 0;
  }
  if (A->dkind == 0 && !seeded) return 0;  // Ks == K
  // scaled copy of the values
  long cnt = value_count(K);
  bool dvec_cplx = (A->dkind == 2 && A->dinv_cplx) || (A->dkind == 1 && A->dinv_u.y != 0.0);
  bool out_cplx = (K.vals == 2) || dvec_cplx || es.y != 0.0;
  // uniform scaling is applied through a temporary constant vector for simplicity
  void* dtmp = nullptr;
  const void* dptr = A->dinv64;
  bool dcplx = A->dinv_cplx;
  if (A->dkind == 1) {
    size_t es = dvec_cplx ? 16 : 8;
    IDRS_CUDA(cudaMallocAsync(&dtmp, es * std::max<long>(n, 1), st));
    if (dvec_cplx) {
      std::vector<c128> h(n, A->dinv_u);
      IDRS_CUDA(cudaMemcpyAsync(dtmp, h.data(), es * n, cudaMemcpyHostToDevice, st));
      IDRS_CUDA(cudaStreamSynchronize(st));
    } else {
      std::vector<double> h(n, A->dinv_u.x);
      IDRS_CUDA(cudaMemcpyAsync(dtmp, h.data(), es * n, cudaMemcpyHostToDevice, st));
      IDRS_CUDA(cudaStreamSynchronize(st));
    }
    dptr = dtmp;
    dcplx = dvec_cplx;
  }
  int* d_missing = nullptr;
  IDRS_CUDA(cudaMallocAsync((void**)&d_missing, sizeof(int), st));
  IDRS_CUDA(cudaMemsetAsync(d_missing, 0, sizeof(int), st));
  const void* kval = value_ptr(K);
  void* kval_tmp = nullptr;
  if (out_cplx) {
    IDRS_CUDA(cudaMallocAsync(&A->ks_val64, 16 * std::max<long>(cnt, 1), st));
    const c128* kv = (const c128*)kval;
    if (K.vals == 1 && kval) {  // promote real values
      IDRS_CUDA(cudaMallocAsync(&kval_tmp, 16 * std::max<long>(cnt, 1), st));
      k_r2c<<<stream_grid(cnt), kThreads, 0, st>>>(cnt, (const double*)kval, (c128*)kval_tmp);
      IDRS_LAUNCH_CHECK();
      kv = (const c128*)kval_tmp;
    }
    if (dptr && !dcplx) scale_values<c128, double>(K, kv, (const double*)dptr, es, (c128*)A->ks_val64, st, d_missing);
    else scale_values<c128, c128>(K, kv, (const c128*)dptr, es, (c128*)A->ks_val64, st, d_missing);
  } else {
    IDRS_CUDA(cudaMallocAsync(&A->ks_val64, 8 * std::max<long>(cnt, 1), st));
    scale_values<double, double>(K, kval, (const double*)dptr, es.x, (double*)A->ks_val64, st, d_missing);
  }
  int missing = 0;
  IDRS_CUDA(cudaMemcpyAsync(&missing, d_missing, sizeof(int), cudaMemcpyDeviceToHost, st));
  IDRS_CUDA(cudaStreamSynchronize(st));
  cudaFreeAsync(d_missing, st);
  if (dtmp) cudaFreeAsync(dtmp, st);
  if (kval_tmp) cudaFreeAsync(kval_tmp, st);
  if (missing) {
    set_error("seed shift needs every diagonal entry present in the sparsity pattern");
    return 5;
  }
  A->ks64.val = A->ks_val64;
  A->ks64.vcplx = out_cplx;
  return 0;
}

template <class Tin, class Tout>
__global__ void k_narrow(long n, const Tin* a, Tout* b) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x)
    b[i] = narrow<Tout>(widen(a[i]));
}

const MatView& Operator::view(int prec) {
  const bool lu = P && (P->which_precon == 2 || P->which_precon == 3);
  if (prec != 32) {
    ks64.defl = defl;
    ks64.lu = lu ? P : nullptr;
    ks64.lu_tmp = lu_tmp;
    ks64.si_C = si_C;
    ks64.si_M = si_M;
    ks64.si_shift = shift;
    ks64.si_tmp = si_tmp;
    return ks64;
  }
  if (defl && defl->k > 0)
    throw std::runtime_error("deflation is not available in the fp32 operator (inner_precision 32)");
  if (lu) throw std::runtime_error("shift-and-invert is not available in the fp32 operator (inner_precision 32)");
  if (ks32.format != FMT_NONE) return ks32;
  ks32 = ks64;
  cudaStream_t st = stream;
  if (ks64.format != FMT_STENCIL7) {
    long cnt = value_count(*K);
    if (ks64.vcplx) {
      IDRS_CUDA(cudaMallocAsync(&ks_val32, 8 * std::max<long>(cnt, 1), st));
      k_narrow<c128, c64><<<stream_grid(cnt), kThreads, 0, st>>>(cnt, (const c128*)ks64.val, (c64*)ks_val32);
    } else {
      IDRS_CUDA(cudaMallocAsync(&ks_val32, 4 * std::max<long>(cnt, 1), st));
      k_narrow<double, float><<<stream_grid(cnt), kThreads, 0, st>>>(cnt, (const double*)ks64.val, (float*)ks_val32);
    }
    IDRS_LAUNCH_CHECK();
    ks32.val = ks_val32;
  }
  if (dkind == 2 && !dinv32) {
    long nn = n();
    if (dinv_cplx) {
      IDRS_CUDA(cudaMallocAsync(&dinv32, 8 * nn, st));
      k_narrow<c128, c64><<<stream_grid(nn), kThreads, 0, st>>>(nn, (const c128*)dinv64, (c64*)dinv32);
    } else {
      IDRS_CUDA(cudaMallocAsync(&dinv32, 4 * nn, st));
      k_narrow<double, float><<<stream_grid(nn), kThreads, 0, st>>>(nn, (const double*)dinv64, (float*)dinv32);
    }
    IDRS_LAUNCH_CHECK();
  }
  return ks32;
}

void operator_free(Operator* A) {
  cudaStream_t st = A->stream;
  if (A->ks_val64) cudaFreeAsync(A->ks_val64, st);
  if (A->ks_val32) cudaFreeAsync(A->ks_val32, st);
  if (A->dinv64) cudaFreeAsync(A->dinv64, st);
  if (A->dinv32) cudaFreeAsync(A->dinv32, st);
  if (A->lb_partial) cudaFreeAsync(A->lb_partial, st);
  if (A->lb_carry) cudaFreeAsync(A->lb_carry, st);
  for (auto& p : A->shadows) cudaFreeAsync(p.second, st);
  A->shadows.clear();
  if (A->defl) { deflation_free(A->defl); A->defl = nullptr; }
  if (A->lu_tmp) { cudaFreeAsync(A->lu_tmp, st); A->lu_tmp = nullptr; }
  if (A->si_tmp) { cudaFreeAsync(A->si_tmp, st); A->si_tmp = nullptr; }
  if (A->si_C) { user_matrix_release(A->si_C); A->si_C = nullptr; }
  if (A->si_M) { user_matrix_release(A->si_M); A->si_M = nullptr; }
  free_redbuf(A->red, st);
  cudaStreamSynchronize(st);
  if (A->own_stream) cudaStreamDestroy(st);
  user_matrix_release(A->K);
  user_matrix_release(A->P);
}

// ---------------------------------------------------------------------------
// explicit instantiations
// ---------------------------------------------------------------------------
#define IDRS_INST(T)                                                                              \
  template void spmv<T>(const MatView&, const T*, T*, T, T, const T*, const int*, cudaStream_t);    \
  template void spmv_ex<T>(const MatView&, const T*, T*, const Epi<T>&, const int*, cudaStream_t); \
  template void op_chain_recur<T>(const MatView&, const JacobiCols&, int, const T*, T*, T*, T*, T*, T*, \
                                  const int*, cudaStream_t, T, T, const T*);                       \
  template const T* op_chain_recur_head<T>(const MatView&, const JacobiCols&, int, const T*, T*, T*, T*, T*, \
                                           const int*, cudaStream_t);                                     \
  template void op_apply<T>(Operator&, int, const T*, T*, T*, T*, T*, T*, const int*, cudaStream_t, T, T, \
                            const T*);                                                             \
  template void op_chain<T>(const MatView&, const std::vector<c128>&, int, const T*, T*, T*, T*,   \
                            const int*, cudaStream_t, T, T, const T*);                            \
  template void op_scaleback<T>(Operator&, int, const std::vector<c128>&, int, const T*, T*, T*,  \
                                T*, const int*, cudaStream_t, const T*, c128, c128);               \
  template void ks_mv<T>(const MatView&, const T*, T*, T, T, const T*, const int*, cudaStream_t); \
  template void op_precon<T>(Operator&, int, const T*, T*, const int*, cudaStream_t);             \
  template void vec_copy<T>(long, const T*, T*, const int*, cudaStream_t);                        \
  template void vec_scale_vec<T>(long, const void*, bool, const T*, T*, const int*, cudaStream_t);
IDRS_INST(double)
IDRS_INST(float)
IDRS_INST(c128)
IDRS_INST(c64)
#undef IDRS_INST
template void vec_convert<double, float>(long, const double*, float*, const int*, cudaStream_t);
template void vec_convert<float, double>(long, const float*, double*, const int*, cudaStream_t);
template void vec_convert<c128, c64>(long, const c128*, c64*, const int*, cudaStream_t);
template void vec_convert<c64, c128>(long, const c64*, c128*, const int*, cudaStream_t);

}  // namespace idrs
