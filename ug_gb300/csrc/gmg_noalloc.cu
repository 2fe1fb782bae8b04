// gmg_nrm2x_static: per-component 2-norms of a device array, with the
// kernel's scratch memory in a file-scope device array instead of memory the
// library allocates.
//
// Who needs this: callers that cannot let a library call cudaMalloc -- for
// example a host framework whose own memory manager owns all device memory
// (UG manages every byte of its data on its own heap) and only hands device
// buffers to the solver, or a process that runs under a fixed device-memory
// budget it has already spent.  Such a caller passes its input and output
// buffers; the partial sums the reduction needs live in `g_nrm_scratch`.
//
// Limits and rules:
//   * at most GMG_MAX_S (8) components per row; larger s is rejected;
//   * the scratch (NRM_BLOCKS x GMG_MAX_S partial sums + a ticket counter,
//     about 20 KB) exists once per device that loads the library and stays
//     allocated until the process exits;
//   * the first call on a device looks up the scratch's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture;
//   * that address is kept per device ordinal for the life of the process and
//     is not looked up again: after cudaDeviceReset (or any other teardown of
//     the device's primary context) it is stale, so do not call this entry
//     point again in that process;
//   * every call shares the one scratch array: calls whose kernels overlap on
//     the GPU (different streams, no ordering between them) race and give
//     wrong norms; order them on one stream or synchronise between them;
//   * the ticket counter is cleared on the caller's stream before each launch,
//     the partial sums are overwritten, so nothing from an earlier call leaks in;
//   * no cudaMalloc, cudaFree or allocating library routine is called.
#include <cuda_runtime.h>

#include <climits>
#include <mutex>

#include "gmg_internal.h"

namespace {

constexpr int NRM_BLOCKS = 304;  // 2 per SM on a 152-SM GB300
constexpr int NRM_THREADS = 256;
constexpr int SCRATCH_DOUBLES = NRM_BLOCKS * GMG_MAX_S + 8;  // partial sums + ticket

__device__ __align__(256) double g_nrm_scratch[SCRATCH_DOUBLES];

// Stage 1 per block into scratch; the block drawing the last ticket adds the
// partials in block order, writes sqrt() of each component and resets the
// ticket.  Same arithmetic and order as the library's nrm_kernel.
template <int S>
__global__ void __launch_bounds__(NRM_THREADS) nrm_static_kernel(long long n, const double *__restrict__ x,
                                                               double *__restrict__ out, double *scratch) {
  double acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
#pragma unroll
    for (int r = 0; r < S; ++r) {
      const double v = x[i * S + r];
      acc[r] = fma(v, v, acc[r]);
    }
  __shared__ double sh[NRM_THREADS / 32][S];
  __shared__ double red[NRM_THREADS];
  __shared__ bool last;
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][r] = v;
  }
  __syncthreads();
  if (threadIdx.x < S) {
    double v = 0.0;
    for (int w = 0; w < NRM_THREADS / 32; ++w) v += sh[w][threadIdx.x];
    scratch[blockIdx.x * S + threadIdx.x] = v;
  }
  unsigned *ticket = reinterpret_cast<unsigned *>(scratch + NRM_BLOCKS * GMG_MAX_S);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int r = 0; r < S; ++r) {
    double v = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) v += __ldcg(scratch + b * S + r);
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[r] = sqrt(red[0]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

std::mutex g_mu;
double *g_scratch_addr[256] = {};  // per device ordinal

}  // namespace

extern "C" int gmg_nrm2x_static(const double *x_dev, long long n, int s, double *norms_dev, void *stream) {
  using gmg::set_error;
  if (s < 1 || s > GMG_MAX_S) {
    set_error("gmg_nrm2x_static: %d components per row; the static scratch holds at most %d", s, GMG_MAX_S);
    return 1;
  }
  if (n < 0 || (n > 0 && !x_dev) || !norms_dev) {
    set_error("gmg_nrm2x_static: bad arguments (n=%lld)", n);
    return 1;
  }
  if (n > LLONG_MAX / GMG_MAX_S) {
    set_error("gmg_nrm2x_static: n=%lld rows is too large", n);
    return 1;
  }
  int dev = 0;
  GMG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) {
    set_error("gmg_nrm2x_static: device ordinal %d out of range", dev);
    return 1;
  }
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
      // host code must not use g_nrm_scratch's name as a device address
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_nrm_scratch);
      if (e != cudaSuccess || !p) {
        set_error("gmg_nrm2x_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        return 1;
      }
      g_scratch_addr[dev] = static_cast<double *>(p);
    }
    scratch = g_scratch_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  GMG_CUDA(cudaMemsetAsync(scratch + NRM_BLOCKS * GMG_MAX_S, 0, sizeof(unsigned), st));
  switch (s) {
#define CASE(SS) \
  case SS: nrm_static_kernel<SS><<<NRM_BLOCKS, NRM_THREADS, 0, st>>>(n, x_dev, norms_dev, scratch); break;
    CASE(1) CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8)
#undef CASE
  }
  GMG_CUDA(cudaGetLastError());
  return 0;
}
