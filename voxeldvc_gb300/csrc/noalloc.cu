// vdvc_matvec_H_noalloc: the float32 Hessian matvec for callers that cannot
// allocate device memory.
//
// Some host applications cannot call cudaMalloc at the point where they
// apply the operator: a plugin whose host application owns all device memory
// through its own pool, or a latency-critical loop where an allocation (and
// the device synchronisation cudaMalloc may imply) is not allowed.  This
// entry point takes only the inputs and the output; its scratch -- the
// [24][Ne] element-vector buffer of the element pass -- is the file-scope
// device array below, which every GPU that loads this library holds until
// the process exits.
//
// Host code cannot use the array's name as a device address (on the host it
// names a host-side stand-in), so the first call on each device looks the
// address up with cudaGetSymbolAddress, with that device current, and keeps
// it.  That first call therefore does set-up work and should come before any
// stream capture.  All calls share the one array: the element pass writes
// every entry it later reads (no clearing is needed), and calls whose
// kernels overlap on the GPU -- on different streams, or from different host
// threads -- race on it.
#include <mutex>

#include "ops.cuh"

namespace vdvc {
namespace {

// 32 MiB: element vectors of up to 349,525 elements (e.g. 64^3 = 262,144).
constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {nullptr};

int scratch_address(void** out) {
  int dev = 0;
  VDVC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(VDVC_ERR_UNSUPPORTED, "device index %d", dev);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return set_error(VDVC_ERR_CUDA, "cudaGetSymbolAddress of the no-alloc scratch on device %d: %s", dev,
                       cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return VDVC_OK;
}

}  // namespace
}  // namespace vdvc

using namespace vdvc;

extern "C" {

size_t vdvc_matvec_H_noalloc_max_elements(void) { return kNoAllocScratchBytes / (24 * sizeof(float)); }

int vdvc_matvec_H_noalloc(const float* v, const float* grad, const uint8_t* mask, int h, int Nx, int Ny, int Nz,
                          float* out, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(h, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(v && grad && mask && out, "null pointer");
  const size_t need = (size_t)24 * (size_t)m.Ne * sizeof(float);
  if (need > kNoAllocScratchBytes)
    return set_error(VDVC_ERR_ARG,
                     "vdvc_matvec_H_noalloc: a mesh of %lld elements needs %zu bytes of scratch, more than its fixed "
                     "%zu bytes (at most %zu elements); use vdvc_matvec_H with a caller-provided workspace",
                     m.Ne, need, kNoAllocScratchBytes, vdvc_matvec_H_noalloc_max_elements());
  void* scratch = nullptr;
  if ((st = scratch_address(&scratch))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  StripArgs<float> a{};
  a.m = m;
  a.v = v;
  a.grad = grad;
  a.mask = mask;
  a.evA = (float*)scratch;
  if ((st = launch_strip<float, kModeHv>(a, nullptr, s))) return st;
  return launch_gather<float>(m, (const float*)scratch, out, s);
}

}  // extern "C"
