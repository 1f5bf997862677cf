// Library-level entry points: ABI version, status strings, per-thread error
// detail, launch counter and mesh validation.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <climits>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "common.cuh"

namespace vdvc {

static thread_local char g_last_error[512] = "";
static std::atomic<long long> g_launches{0};

int set_error(int status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return status;
}

void count_launch(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Pools of the per-solver CUDA objects.  Creating a stream, two events and
// a pinned read-back block for every solver of every pyramid level costs
// more than the coarse levels' solves of small problems; returned objects
// are idle (their owner synchronised) and are handed out again.
static std::mutex g_pool_mu;
static std::map<int, std::vector<cudaStream_t>> g_streams;  // device -> idle non-blocking streams
static std::map<int, std::vector<cudaEvent_t>> g_events;    // device -> idle timing-free events
static std::vector<void*> g_pinned;                          // idle kPinnedSlot-byte pinned blocks

int pool_stream(cudaStream_t* out) {
  int dev = 0;
  VDVC_CUDA(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    auto& v = g_streams[dev];
    if (!v.empty()) {
      *out = v.back();
      v.pop_back();
      return VDVC_OK;
    }
  }
  VDVC_CUDA(cudaStreamCreateWithFlags(out, cudaStreamNonBlocking));
  return VDVC_OK;
}

void pool_stream_return(cudaStream_t s) {
  if (!s) return;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    cudaStreamDestroy(s);
    return;
  }
  std::lock_guard<std::mutex> lk(g_pool_mu);
  g_streams[dev].push_back(s);
}

int pool_event(cudaEvent_t* out) {
  int dev = 0;
  VDVC_CUDA(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    auto& v = g_events[dev];
    if (!v.empty()) {
      *out = v.back();
      v.pop_back();
      return VDVC_OK;
    }
  }
  VDVC_CUDA(cudaEventCreateWithFlags(out, cudaEventDisableTiming));
  return VDVC_OK;
}

void pool_event_return(cudaEvent_t e) {
  if (!e) return;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    cudaEventDestroy(e);
    return;
  }
  std::lock_guard<std::mutex> lk(g_pool_mu);
  g_events[dev].push_back(e);
}

int pool_pinned(void** out) {
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pinned.empty()) {
      *out = g_pinned.back();
      g_pinned.pop_back();
      return VDVC_OK;
    }
  }
  VDVC_CUDA(cudaMallocHost(out, kPinnedSlot));
  return VDVC_OK;
}

void pool_pinned_return(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  g_pinned.push_back(p);
}

int ensure_dyn_smem(const void* func, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> done;  // (function, device) -> bytes set
  int dev = 0;
  VDVC_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  auto it = done.find({func, dev});
  if (it != done.end() && it->second >= bytes) return VDVC_OK;
  VDVC_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  done[{func, dev}] = bytes;
  return VDVC_OK;
}

int make_mesh(int h, int Nx, int Ny, int Nz, Mesh* m) {
  VDVC_CHECK_ARG(h >= 1 && h <= 1024, "h=%d must be in [1, 1024]", h);
  VDVC_CHECK_ARG(Nx >= 1 && Ny >= 1 && Nz >= 1, "element counts must be >= 1 (got %d,%d,%d)", Nx, Ny, Nz);
  m->Nx = Nx; m->Ny = Ny; m->Nz = Nz; m->h = h;
  const long long nvx = (long long)Nx * h + 1, nvy = (long long)Ny * h + 1, nvz = (long long)Nz * h + 1;
  const long long nvox = nvx * nvy * nvz;
  const long long nnodes = (long long)(Nx + 1) * (Ny + 1) * (Nz + 1);
  // Same int32 guard as the reference (engine/correlate_gpu.py:933-936).
  if (nvox > INT_MAX || 3 * nnodes > INT_MAX)
    return set_error(VDVC_ERR_INDEX_RANGE,
                     "Nvox=%lld / Ndof=%lld exceed int32 range; matrix-free index arrays assume int32 indices",
                     nvox, 3 * nnodes);
  m->Nvx = (int)nvx; m->Nvy = (int)nvy; m->Nvz = (int)nvz;
  m->Nnx = Nx + 1; m->Nny = Ny + 1; m->Nnz = Nz + 1;
  m->Nvox = nvox;
  m->Nnodes = nnodes;
  m->Ndof = 3 * nnodes;
  m->Ne = (long long)Nx * Ny * Nz;
  m->NvxNvy = nvx * nvy;
  m->NnxNny = (long long)(Nx + 1) * (Ny + 1);
  m->inv_h = 1.0f / (float)h;
  return VDVC_OK;
}

}  // namespace vdvc

extern "C" {

int vdvc_abi_version(void) { return 1; }

const char* vdvc_status_string(int status) {
  switch (status) {
    case VDVC_OK: return "ok";
    case VDVC_ERR_ARG: return "invalid argument";
    case VDVC_ERR_INDEX_RANGE: return "index range exceeds int32";
    case VDVC_ERR_CUDA: return "CUDA error";
    case VDVC_ERR_WORKSPACE: return "workspace too small";
    case VDVC_ERR_NONFINITE: return "non-finite value";
    case VDVC_ERR_ZERO_DIVISION: return "division by zero";
    case VDVC_ERR_CUFFT: return "cuFFT error";
    case VDVC_ERR_UNSUPPORTED: return "unsupported";
    case VDVC_ERR_TIMEOUT: return "device-side wait timed out";
  }
  return "unknown status";
}

const char* vdvc_last_error(void) { return vdvc::g_last_error; }

long long vdvc_launch_count(void) { return vdvc::g_launches.load(); }

int vdvc_device_reads_pageable(int device) {
  // pageable access through the host's own page tables (address translation
  // services): the device reads host pages in place, without migrating them
  int pageable = 0, host_tables = 0;
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess ||
      cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (pageable && host_tables) ? 1 : 0;
}

}  // extern "C"
