// Self-test of the failure path of the bounded device waits.
//
// Every wait in the kernels (TMA completion, row arrivals, grid barriers) gives
// up after a time limit, records DEV_TIMEOUT in the engine's error word and
// lets its kernel run to the end, so the host reports SDNN_ERR_TIMEOUT and the
// context stays usable.  This kernel waits, with that same helper, on an
// mbarrier phase that nothing ever completes -- the wait must run out.
#include "layer_kernel.cuh"

namespace sdnn {

namespace {

__global__ void wait_selftest_kernel(int32_t* err, uint64_t limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);  // one arrival expected; none is ever made
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait_bounded(&bar, 0, err, limit_ns);
}

}  // namespace

cudaError_t launch_wait_selftest(int32_t* err, uint64_t limit_ns, cudaStream_t s) {
  wait_selftest_kernel<<<1, 32, 0, s>>>(err, limit_ns);
  return cudaGetLastError();
}

}  // namespace sdnn
