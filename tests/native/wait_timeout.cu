// wait_timeout.cu -- test kernel for the library's bounded device-side waits
// (built by tests/test_gpu_timeout.py; not part of the library).
//
// Every thread of one block waits, through the library's own
// mbar_wait_bounded, on an mbarrier that no thread arrives at and no copy
// targets, with a short clock limit: the wait must give up, the block must
// record WAH_ETIMEOUT through set_status (first error wins) and return.
// Nothing is in flight when it does, so the context stays usable.
#include "wah_common.cuh"

namespace {

__global__ void k_wait_on_nobody(uint32_t* status, uint32_t* completed, long long limit) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    wah::mbar_init(&bar, 1);
    wah::fence_mbar_init();
  }
  __syncthreads();
  if (!wah::mbar_wait_bounded(&bar, 0, limit)) wah::set_status(status, WAH_ETIMEOUT);
  else atomicAdd(completed, 1u);
}

}  // namespace

extern "C" int test_wait_on_nobody(uint32_t* d_status, uint32_t* d_completed,
                                   long long limit_cycles, int threads, void* stream) {
  if (threads <= 0 || threads > 1024 || limit_cycles <= 0 || limit_cycles > 100000000ll)
    return WAH_EINVAL;
  k_wait_on_nobody<<<1, threads, 0, static_cast<cudaStream_t>(stream)>>>(d_status, d_completed,
                                                                         limit_cycles);
  return cudaGetLastError() == cudaSuccess ? WAH_OK : WAH_ECUDA;
}
