// Self-test of the bounded device-side waits of the tensor-core kernels.
//
// Every mbarrier wait in tc_common.cuh gives up after a time limit, sets FH_ERR_TIMEOUT in the
// caller's status word and lets the kernel release its tensor memory and return, so a lost
// producer costs an error code instead of a hung stream.  fh_selftest_wait exercises that
// path on purpose: one warp allocates tensor memory, waits on an mbarrier that nothing ever
// arrives on, with the caller's short limit, records the timeout, frees the tensor memory and
// exits.  The context stays usable, and the next kernel that allocates tensor memory on the
// same SM must still succeed.  No reference counterpart (the reference has no device code).
#include "tc_common.cuh"

namespace fh {

__global__ void __launch_bounds__(32) selftest_wait_kernel(int* status, uint64_t limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  const uint32_t b = smem_u32(&bar);
  if (threadIdx.x == 0) {
    mbar_init(b, 1);
    mbar_fence_init();
  }
  tmem_alloc(smem_u32(&tbase), 32);
  tmem_relinquish();
  tc_fence_before();
  __syncwarp();
  tc_fence_after();
  const uint32_t tmem = tbase;
  // nothing arrives on bar: the wait runs out after limit_ns
  const bool got = __all_sync(0xffffffffu, mbar_wait_ns(b, 0, nullptr, limit_ns));
  if (!got && threadIdx.x == 0) set_status(status, FH_ERR_TIMEOUT);
  tc_fence_before();
  __syncwarp();
  tc_fence_after();
  tmem_dealloc(tmem, 32);
}

}  // namespace fh

using namespace fh;

extern "C" int fh_selftest_wait(int* status, int64_t limit_ns, void* stream) {
  if (!status || limit_ns <= 0 || limit_ns > 1000000000LL) return FH_ERR_ARG;
  selftest_wait_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(status, (uint64_t)limit_ns);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
