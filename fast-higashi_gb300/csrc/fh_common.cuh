// Shared definitions of the fh_gb300 CUDA library (sm_103a).
#pragma once
#include <cstdint>
#include <mutex>
#include <unordered_map>
#include <cuda_runtime.h>

#include "fhgb300.h"

#define FH_CHECK_LAUNCH()                                   \
  do {                                                      \
    cudaError_t e_ = cudaGetLastError();                    \
    if (e_ != cudaSuccess) return FH_ERR_LAUNCH;            \
  } while (0)

namespace fh {

constexpr int kMaxBinRows = 128;   // b: rows of a bin batch handled by the fused RWR kernels
constexpr int kMaxWidth = 320;     // n: columns of a compact tile (b + 2 * flank)
constexpr int kMaxRank = 128;      // R (meta rank) and r (per-chromosome rank)

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Row stride (floats) of a shared-memory tile so that rows start on distinct banks when
// a warp reads one element from each of 16 consecutive rows.
__host__ __device__ inline int lds_stride_odd(int n) { return ((n + 31) / 32) * 32 + 1; }

template <typename T>
__device__ inline T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic block-wide sum (fixed reduction tree); every thread gets the result.
template <typename T>
__device__ inline T block_sum(T v, T* scratch /* >= 32 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  T s = 0;
  for (int w = 0; w < nwarps; ++w) s += scratch[w];
  return s;
}

// out[i] = sum over k of partial[k][i] in a fixed order (deterministic split-K reduction),
// added in fp64 and rounded once; with accumulate the sum starts from out[i] (a pass over X
// held in several row ranges adds each range's sum into one result).
template <typename T>
__global__ void reduce_splits_kernel(const T* __restrict__ partial, int splits, int64_t n,
                                     T* __restrict__ out, bool accumulate) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = accumulate ? (double)out[i] : 0.0;
    for (int k = 0; k < splits; ++k) s += (double)partial[(int64_t)k * n + i];
    out[i] = (T)s;
  }
}

// 16-byte global -> shared copy (cp.async, L2 only); valid = false fills zeros.
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gsrc), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ inline void set_status(int* status, int code) {
  if (status) atomicCAS(status, 0, code);
}

// Raises a kernel's dynamic shared-memory limit once per (device, kernel, size) so that
// later calls, including calls made while a stream is being captured into a graph, issue
// no attribute changes.
inline cudaError_t ensure_smem(const void* kernel, size_t bytes) {
  static std::mutex mu;
  static std::unordered_map<uint64_t, size_t> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t key = ((uint64_t)(uintptr_t)kernel) ^ ((uint64_t)dev << 56);
  std::lock_guard<std::mutex> g(mu);
  auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) done[key] = bytes;
  return e;
}

}  // namespace fh
