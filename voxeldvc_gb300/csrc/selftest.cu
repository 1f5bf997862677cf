// Checks of the library's bounded device-side waits.  Each runs a wait the
// production kernels use -- the grid barrier of the fused PCG iteration
// (common.cuh) or the mbarrier wait of the bulk-copy staging (tma.cuh) --
// either released normally or in a situation where nothing releases it,
// with a short poll bound, and reports what the production path reports:
// VDVC_OK, or VDVC_ERR_TIMEOUT with every block returned and the CUDA
// context usable.  Nothing here faults, traps or hangs a GPU.
#include "ops.cuh"
#include "tma.cuh"

namespace vdvc {
namespace {

__device__ unsigned int g_bar[4];  // count, generation, (unused), (unused)
__device__ int g_err;
__device__ int g_released;  // blocks that passed the wait

__global__ void k_selftest_grid_barrier(unsigned int extra, long long max_polls) {
  if (grid_barrier(g_bar, &g_err, gridDim.x + extra, max_polls) && threadIdx.x == 0) atomicAdd(&g_released, 1);
}

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

template <typename V>
int symbol_ptr(const V& sym, void** p) {
  VDVC_CUDA(cudaGetSymbolAddress(p, sym));
  return VDVC_OK;
}

}  // namespace
}  // namespace vdvc

using namespace vdvc;

extern "C" {

int vdvc_selftest_bounded_wait(int which, long long max_polls, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(which >= 0 && which <= 3, "which must be 0..3");
  VDVC_CHECK_ARG(max_polls >= 1 && max_polls <= kBarrierSpinLimit, "max_polls must be in [1, %lld]",
                 (long long)kBarrierSpinLimit);
  cudaStream_t s = (cudaStream_t)stream;
  void *bar = nullptr, *err = nullptr, *rel = nullptr;
  int st;
  if ((st = symbol_ptr(g_bar, &bar)) || (st = symbol_ptr(g_err, &err)) || (st = symbol_ptr(g_released, &rel)))
    return st;
  VDVC_CUDA(cudaMemsetAsync(bar, 0, sizeof(g_bar), s));
  VDVC_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  VDVC_CUDA(cudaMemsetAsync(rel, 0, sizeof(int), s));
  int blocks = 1;
  if (which == 0 || which == 2) {
    // a grid barrier of 2 blocks per SM, all resident (cooperative launch)
    int dev = 0, nsm = 0, per_sm = 0;
    VDVC_CUDA(cudaGetDevice(&dev));
    VDVC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    VDVC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_selftest_grid_barrier, 128, 0));
    blocks = nsm * (per_sm < 2 ? per_sm : 2);
    if (blocks < 1) return set_error(VDVC_ERR_UNSUPPORTED, "barrier kernel does not fit on an SM");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(128);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    // which 0: one arrival more than the grid has -- nothing releases it
    VDVC_CUDA(cudaLaunchKernelEx(&cfg, k_selftest_grid_barrier, (unsigned int)(which == 0 ? 1 : 0), max_polls));
    count_launch();
  } else {
    // which 1: a one-arrival mbarrier nobody arrives at; 3: thread 0 arrives
    k_selftest_mbarrier<<<1, 64, 0, s>>>(which == 3 ? 1 : 0, max_polls);
    VDVC_LAUNCHED();
  }
  int h_err = 0, h_rel = 0;
  VDVC_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaMemcpyAsync(&h_rel, rel, sizeof(int), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaStreamSynchronize(s));
  if (h_err) {
    if (h_rel != 0 && (which == 1 || which == 3))
      return set_error(VDVC_ERR_CUDA, "self-test: inconsistent mbarrier outcome");
    return set_error(VDVC_ERR_TIMEOUT, "self-test %d: the bounded wait ran out after %lld polls (%d of %d blocks released)",
                     which, max_polls, h_rel, blocks);
  }
  if (h_rel != blocks) return set_error(VDVC_ERR_CUDA, "self-test %d: %d of %d blocks released", which, h_rel, blocks);
  return VDVC_OK;
}

}  // extern "C"
