// noalloc.cu -- INPROD(u, v) with no device allocation at all.
//
// Some callers cannot call cudaMalloc: applications whose device memory is
// owned by another allocator (a framework that reserves the GPU up front, so
// a foreign allocation may fail or fragment its pool), and latency-critical
// loops whose policy forbids allocating after start-up.  For them this file
// provides idrs_rinprod_noalloc: the caller passes device inputs and a device
// output, and the reduction's scratch (one completion ticket and one partial
// sum per block) lives in a file-scope __device__ array that every GPU which
// loads this library holds until the process exits.
//
// Limits and rules
//  * Scratch: 256 B for the ticket + kNoAllocMaxBlocks doubles (128 KiB).
//    One block reduces kNoAllocChunk = 4096 elements, so n is limited to
//    kNoAllocMaxBlocks * kNoAllocChunk = 67,108,864; longer vectors are
//    rejected with IDRS_ERR_ARG before anything is launched.
//  * Set-up: the first call on each device looks up the array's device
//    address (cudaGetSymbolAddress) with that device current and caches it;
//    make that first call before any stream capture begins.
//  * Every call shares the one array: the ticket is cleared (cudaMemsetAsync
//    on the symbol address, no allocation) at the start of each call, and
//    calls that overlap on the GPU -- on different streams, or from different
//    threads without ordering -- race on the scratch.  Order them.
//  * u, v and uv must be device memory of the current device (or managed
//    memory); any other pointer is refused with IDRS_ERR_ARG before a launch.
//  * The call is asynchronous on `stream`; *uv is valid once it completes.
#include <mutex>

#include "../../include/idrs_gb300.h"
#include "common.cuh"

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocPerThread = 16;
constexpr long kNoAllocChunk = (long)kNoAllocThreads * kNoAllocPerThread;  // 4096
constexpr int kNoAllocMaxBlocks = 16384;
constexpr long kNoAllocMaxN = kNoAllocChunk * kNoAllocMaxBlocks;           // 2^26

// [0, 256): completion ticket (unsigned int at offset 0); [256, ...): partials
static __device__ __align__(256) unsigned char g_noalloc_scratch[256 + kNoAllocMaxBlocks * sizeof(double)];

__global__ void __launch_bounds__(kNoAllocThreads)
k_inprod_noalloc(long n, const double* __restrict__ u, const double* __restrict__ v,
                 double* __restrict__ uv, unsigned char* scratch) {
  unsigned int* ticket = reinterpret_cast<unsigned int*>(scratch);
  double* part = reinterpret_cast<double*>(scratch + 256);
  __shared__ double sh[kNoAllocThreads / 32];
  __shared__ bool is_last;
  const long base = (long)blockIdx.x * kNoAllocChunk;
  double acc = 0.0;
#pragma unroll
  for (int k = 0; k < kNoAllocPerThread; ++k) {
    long i = base + (long)k * kNoAllocThreads + threadIdx.x;
    if (i < n) acc += u[i] * v[i];
  }
  for (int m = 16; m >= 1; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kNoAllocThreads / 32; ++w) t += sh[w];
    part[blockIdx.x] = t;
    __threadfence();
    unsigned int prev = atomicAdd(ticket, 1u);
    is_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  // last block: fixed-order sum of the partials
  double t = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += kNoAllocThreads) t += __ldcg(part + b);
  for (int m = 16; m >= 1; m >>= 1) t += __shfl_xor_sync(0xffffffffu, t, m);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kNoAllocThreads / 32; ++w) s += sh[w];
    *uv = s;
    *ticket = 0u;
  }
}

std::mutex g_noalloc_mutex;
void* g_noalloc_addr[256] = {nullptr};  // per device: device address of the scratch array

}  // namespace

extern "C" int idrs_rinprod_noalloc(long n, const double* u, const double* v, double* uv,
                                    void* stream) {
  if (n < 0 || (n > 0 && (!u || !v)) || !uv) {
    idrs::set_error("rinprod_noalloc: u, v and uv must be device pointers and n >= 0");
    return IDRS_ERR_ARG;
  }
  if (n > kNoAllocMaxN) {
    idrs::set_error("rinprod_noalloc: n exceeds the no-allocation limit of 67108864 elements "
                    "(128 KiB of static scratch); use idrs_rinprod");
    return IDRS_ERR_ARG;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 256) {
    idrs::set_error(std::string("rinprod_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return IDRS_ERR_CUDA;
  }
  // u, v and uv must be memory this device can address: device memory of
  // this device, or managed memory.  A host pointer is refused here, before
  // anything is launched.
  for (const void* p : {(const void*)u, (const void*)v, (const void*)uv}) {
    if (!p) continue;
    cudaPointerAttributes at{};
    e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
      cudaGetLastError();
      idrs::set_error(std::string("rinprod_noalloc: cudaPointerGetAttributes: ") + cudaGetErrorString(e));
      return IDRS_ERR_ARG;
    }
    const bool ok = at.type == cudaMemoryTypeManaged || (at.type == cudaMemoryTypeDevice && at.device == dev);
    if (!ok) {
      idrs::set_error("rinprod_noalloc: u, v and uv must be device (or managed) pointers of the current device");
      return IDRS_ERR_ARG;
    }
  }
  void* scratch = nullptr;
  {
    // set-up once per device, with that device current
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        idrs::set_error(std::string("rinprod_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return IDRS_ERR_CUDA;
      }
      g_noalloc_addr[dev] = ptr;
    }
    scratch = g_noalloc_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  // the ticket must start at zero
  e = cudaMemsetAsync(scratch, 0, sizeof(unsigned int), st);
  if (e != cudaSuccess) {
    idrs::set_error(std::string("rinprod_noalloc: cudaMemsetAsync: ") + cudaGetErrorString(e));
    return IDRS_ERR_CUDA;
  }
  long blocks = (n + kNoAllocChunk - 1) / kNoAllocChunk;
  if (blocks < 1) blocks = 1;
  k_inprod_noalloc<<<(unsigned)blocks, kNoAllocThreads, 0, st>>>(n, u, v, uv, (unsigned char*)scratch);
  e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    idrs::set_error(std::string("rinprod_noalloc: launch: ") + cudaGetErrorString(e));
    return IDRS_ERR_CUDA;
  }
  idrs::count_launch();
  return IDRS_OK;
}
