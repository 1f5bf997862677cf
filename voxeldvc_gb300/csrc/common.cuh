// Shared helpers of the vdvc CUDA library: status plumbing, mesh geometry,
// the Hex8 corner numbering and deterministic block reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "vdvc.h"

namespace vdvc {

// ---- status plumbing ------------------------------------------------------

int set_error(int status, const char* fmt, ...);
void count_launch(long long n = 1);

// Raises `func`'s dynamic shared-memory limit to `bytes` on the current
// device, once per (function, device): the attribute is per device, and a
// process may drive several GPUs from several threads.  VDVC_OK or
// VDVC_ERR_CUDA.
int ensure_dyn_smem(const void* func, int bytes);

// Pools of per-solver CUDA objects (lib.cu): idle non-blocking streams and
// timing-free events of the current device, pinned host blocks of
// kPinnedSlot bytes.  Returned streams are synchronised first.
constexpr size_t kPinnedSlot = 4096;
int pool_stream(cudaStream_t* out);
void pool_stream_return(cudaStream_t s);
int pool_event(cudaEvent_t* out);
void pool_event_return(cudaEvent_t e);
int pool_pinned(void** out);
void pool_pinned_return(void* p);

#define VDVC_CHECK_ARG(cond, ...)                                   \
  do {                                                              \
    if (!(cond)) return ::vdvc::set_error(VDVC_ERR_ARG, __VA_ARGS__); \
  } while (0)

#define VDVC_CUDA(expr)                                                      \
  do {                                                                       \
    cudaError_t e_ = (expr);                                                 \
    if (e_ != cudaSuccess)                                                   \
      return ::vdvc::set_error(VDVC_ERR_CUDA, "%s: %s (%s:%d)", #expr,       \
                               cudaGetErrorString(e_), __FILE__, __LINE__);  \
  } while (0)

// After a kernel launch: count it and surface launch-configuration errors.
#define VDVC_LAUNCHED()                                                      \
  do {                                                                       \
    ::vdvc::count_launch();                                                  \
    cudaError_t e_ = cudaGetLastError();                                     \
    if (e_ != cudaSuccess)                                                   \
      return ::vdvc::set_error(VDVC_ERR_CUDA, "launch: %s (%s:%d)",         \
                               cudaGetErrorString(e_), __FILE__, __LINE__);  \
  } while (0)

// ---- mesh geometry --------------------------------------------------------

// Structured Hex8 mesh of Nx*Ny*Nz elements of edge h voxels covering a
// (Nx*h+1, Ny*h+1, Nz*h+1) voxel grid.  Voxel, node and element indices are
// x fastest (engine/kernels_dvc.py:9-21).
struct Mesh {
  int Nx, Ny, Nz, h;
  int Nvx, Nvy, Nvz;
  int Nnx, Nny, Nnz;
  long long Nvox, Nnodes, Ndof, Ne;
  long long NvxNvy, NnxNny;
  float inv_h;
};

int make_mesh(int h, int Nx, int Ny, int Nz, Mesh* m);

// Element (i, j, k) of element index e (x fastest) in 32-bit arithmetic:
// make_mesh keeps 3 Nnodes (> Ne) within int32, and a 64-bit division costs
// tens of instructions per thread.
__device__ __forceinline__ void elem_ijk(const Mesh& m, long long e, int& i, int& j, int& k) {
  const unsigned int eu = (unsigned int)e, nx = (unsigned int)m.Nx, ny = (unsigned int)m.Ny;
  const unsigned int r = eu / nx;
  i = (int)(eu - r * nx);
  j = (int)(r % ny);
  k = (int)(r / ny);
}

// Local corner a (0..7) of a Hex8 element -> offsets, in the reference's
// order (000,100,110,010,001,101,111,011) (engine/geometry_dvc.py:14-17).
__host__ __device__ inline int corner_dx(int a) { return ((a + 1) >> 1) & 1; }
__host__ __device__ inline int corner_dy(int a) { return (a >> 1) & 1; }
__host__ __device__ inline int corner_dz(int a) { return (a >> 2) & 1; }
// Inverse map (dx,dy,dz) -> a.
__host__ __device__ inline int corner_of(int dx, int dy, int dz) {
  return dz * 4 + (dy ? (dx ? 2 : 3) : (dx ? 1 : 0));
}

// Multiplicity of a voxel coordinate along one axis in the
// (element, stencil point) array: 2 on interior element-boundary planes,
// 1 elsewhere (engine/correlate_gpu.py:97-110, 113-157).
__device__ __forceinline__ int axis_multiplicity(int v, int h, int N) {
  return (v > 0 && v < N * h && (v % h) == 0) ? 2 : 1;
}

// ---- numeric type traits --------------------------------------------------

template <typename T> struct TypeCode;
template <> struct TypeCode<float> { static const int value = VDVC_F32; };
template <> struct TypeCode<double> { static const int value = VDVC_F64; };

inline size_t dtype_size(int dtype) {
  switch (dtype) {
    case VDVC_F32: return 4;
    case VDVC_F64: return 8;
    case VDVC_U8: return 1;
    case VDVC_U16: return 2;
    case VDVC_I16: return 2;
    case VDVC_I32: return 4;
  }
  return 0;
}

// Type-exact floor / min / max: the float forms never promote to double
// (GB300's FP64 pipe is a small fraction of its FP32 rate).
__device__ __forceinline__ float tfloor(float x) { return floorf(x); }
__device__ __forceinline__ double tfloor(double x) { return floor(x); }
__device__ __forceinline__ float tmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double tmin(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float tmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double tmax(double a, double b) { return fmax(a, b); }

// ---- reductions -----------------------------------------------------------

// Sum of `v` over the block; result valid in thread 0.  `smem` holds
// blockDim.x/32 doubles.  blockDim.x must be a multiple of 32.
__device__ __forceinline__ double block_sum(double v, double* smem) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int w = 0; w < nw; ++w) s += smem[w];
  }
  return s;
}

// Sum of float partials over the block, result (float64) valid in thread 0:
// the warp stage shuffles in FP32 and only the per-warp sums are added in
// FP64 -- a float64 shuffle tree per warp would keep GB300's narrow FP64
// pipe busy for microseconds per launch.  Same contract as block_sum.
__device__ __forceinline__ double block_sum_f(float v, double* smem) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smem[warp] = (double)v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int w = 0; w < nw; ++w) s += smem[w];
  }
  return s;
}
__device__ __forceinline__ double block_sum_f(double v, double* smem) { return block_sum(v, smem); }

__device__ __forceinline__ double block_min(double v, double* smem) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  double s = v;
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    s = smem[0];
    for (int w = 1; w < nw; ++w) s = fmin(s, smem[w]);
  }
  return s;
}

// Deterministic grid reduction.  Every block publishes NV block-level values
// to partials[bid*NV + i]; the last block to take a ticket sums all partials
// with a fixed thread->range assignment followed by a fixed-order block
// reduction, so the result does not depend on block arrival order.  The
// ticket is reset for the next launch.
struct GridReduce {
  double* partials;     // nblocks * NV doubles
  unsigned int* ticket; // one counter, zero between launches
};

__device__ __forceinline__ unsigned int flat_block_id() {
  return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
}
__device__ __forceinline__ unsigned int flat_grid_size() { return gridDim.x * gridDim.y * gridDim.z; }

// All threads of the block must call this.  `mine` is read from thread 0
// only (a block-reduced value).  Returns true in every thread of the last
// block; `out` is then valid in thread 0.  `red_smem` holds blockDim.x/32
// doubles.
template <int NV>
__device__ bool grid_reduce_sum(const GridReduce& gr, const double (&mine)[NV], double (&out)[NV],
                                double* red_smem) {
  __shared__ bool s_last;
  const unsigned int nb = flat_grid_size();
  if (threadIdx.x == 0) {
    const unsigned int bid = flat_block_id();
    for (int i = 0; i < NV; ++i) gr.partials[(size_t)bid * NV + i] = mine[i];
    __threadfence();
    const unsigned int t = atomicAdd(gr.ticket, 1u);
    s_last = (t == nb - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  // Thread t sums the partials of blocks t, t + blockDim.x, ... (coalesced
  // loads, a fixed assignment, so the result does not depend on block
  // arrival order).
  double acc[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) acc[i] = 0.0;
#pragma unroll 4
  for (unsigned int b = threadIdx.x; b < nb; b += blockDim.x)
#pragma unroll
    for (int i = 0; i < NV; ++i) acc[i] += __ldcg(gr.partials + (size_t)b * NV + i);
  for (int i = 0; i < NV; ++i) out[i] = block_sum(acc[i], red_smem);
  if (threadIdx.x == 0) *gr.ticket = 0u;
  return true;
}

// Scratch carving helper: successive 256-byte aligned sub-buffers of ws.
struct Carve {
  char* base;
  size_t off, cap;
  __host__ Carve(void* p, size_t bytes) : base((char*)p), off(0), cap(bytes) {}
  template <typename U>
  __host__ U* take(size_t n) {
    off = (off + 255) & ~(size_t)255;
    U* r = (U*)(base ? base + off : nullptr);
    off += n * sizeof(U);
    return r;
  }
  __host__ bool fits() const { return off <= cap; }
};

// A 24x24 element operator (row-major float64) passed by value as a kernel
// parameter.
struct Kmat {
  double k[576];
};

constexpr int kReduceBlocks = 1024;  // upper bound of blocks in reduction grids
constexpr int kReduceThreads = 256;

}  // namespace vdvc
