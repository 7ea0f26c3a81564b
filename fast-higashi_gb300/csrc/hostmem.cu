// Host memory for X held partly outside HBM.
//
// When X does not fit the HBM budget (50,000 cells at R = 128, band 40: 179 GB in two bf16
// planes), the last chromosomes' band rows live in page-locked host memory and pass through
// two staging slots in HBM once per pass over X.  The copies are plain cudaMemcpyAsync calls
// on a copy stream (one per window, contiguous on both sides), so a CUDA graph captures them as
// memcpy nodes between the kernels that use the slots.  The contact build copies a
// chromosome's host COO in chunks the same way.
#include "fh_common.cuh"

extern "C" int fh_host_alloc(int64_t bytes, void** out) {
  if (!out || bytes <= 0) return FH_ERR_ARG;
  *out = nullptr;
  void* p = nullptr;
  if (cudaHostAlloc(&p, (size_t)bytes, cudaHostAllocPortable | cudaHostAllocMapped) !=
      cudaSuccess) {
    cudaGetLastError();
    return FH_ERR_LAUNCH;
  }
  *out = p;
  return FH_OK;
}

extern "C" int fh_host_free(void* p) {
  if (!p) return FH_ERR_ARG;
  if (cudaFreeHost(p) != cudaSuccess) {
    cudaGetLastError();
    return FH_ERR_LAUNCH;
  }
  return FH_OK;
}

extern "C" int fh_memcpy_async(void* dst, const void* src, int64_t bytes, void* stream) {
  if (!dst || !src || bytes < 0) return FH_ERR_ARG;
  if (bytes == 0) return FH_OK;
  if (cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDefault, (cudaStream_t)stream) !=
      cudaSuccess) {
    cudaGetLastError();
    return FH_ERR_LAUNCH;
  }
  return FH_OK;
}
