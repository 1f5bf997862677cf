// Check of the library's bounded device-side wait: the mbarrier wait of the
// bulk-copy / tensor-core pipelines (tma.cuh: mbar_wait_bounded, used by the
// element-Hessian matvec, the tcgen05 element-Hessian formation and the
// tcgen05 convolutions), either released normally or on a barrier nothing
// arrives at, with a short poll bound.  It reports what the production path
// reports: VDVC_OK, or VDVC_ERR_TIMEOUT with the block returned and the
// CUDA context usable.  Nothing here faults, traps or hangs a GPU.
#include "ops.cuh"
#include "tma.cuh"

namespace vdvc {
namespace {

__device__ int g_err;
__device__ int g_released;  // blocks that passed the wait

__global__ void k_selftest_mbarrier(int release, long long max_polls) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (release && threadIdx.x == 0) mbar_arrive(&bar);
  const bool ok = mbar_wait_bounded(&bar, 0, max_polls);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (ok)
      atomicAdd(&g_released, 1);
    else
      atomicExch(&g_err, 1);
  }
}

}  // namespace
}  // namespace vdvc

using namespace vdvc;

extern "C" {

int vdvc_selftest_bounded_wait(int which, long long max_polls, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(which == 0 || which == 1, "which must be 0 or 1");
  VDVC_CHECK_ARG(max_polls >= 1 && max_polls <= (1LL << 24), "max_polls must be in [1, 2^24]");
  cudaStream_t s = (cudaStream_t)stream;
  void *err = nullptr, *rel = nullptr;
  VDVC_CUDA(cudaGetSymbolAddress(&err, g_err));
  VDVC_CUDA(cudaGetSymbolAddress(&rel, g_released));
  VDVC_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  VDVC_CUDA(cudaMemsetAsync(rel, 0, sizeof(int), s));
  // which 0: a one-arrival mbarrier nobody arrives at; 1: thread 0 arrives
  k_selftest_mbarrier<<<1, 64, 0, s>>>(which, max_polls);
  VDVC_LAUNCHED();
  int h_err = 0, h_rel = 0;
  VDVC_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaMemcpyAsync(&h_rel, rel, sizeof(int), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaStreamSynchronize(s));
  if (h_err) return set_error(VDVC_ERR_TIMEOUT, "self-test: the bounded mbarrier wait ran out after %lld polls",
                              max_polls);
  if (h_rel != 1) return set_error(VDVC_ERR_CUDA, "self-test: the released wait did not pass");
  return VDVC_OK;
}

}  // extern "C"
