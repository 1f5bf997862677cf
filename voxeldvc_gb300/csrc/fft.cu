// Rigid voxel shift by FFT phase correlation (fft_rigid_shift,
// engine/correlate_gpu.py:381-414), plus a float64 dot/sum reduction.
//
// The volumes are vox layout (x fastest), i.e. C-order arrays of shape
// (nz, ny, nx); the transforms are cuFFT transforms of that shape (library
// calls), the cross-power normalisation and the arg-max are kernels here.
// Precision follows the volumes' dtype, as the reference's fftn does (its
// float64 cast is commented out, so its CuPy path transforms float32 volumes
// in complex64): float32 volumes take R2C/C2R, float64 ones D2Z/Z2D -- the
// single-precision transforms also keep the 129^3 coarse level's FFTs
// (radix 3 x 43) off GB300's narrow FP64 pipe.
// numpy's argmax returns the first maximum in C order of pix[x,y,z]
// (x slowest); the arg-max kernel breaks ties the same way.
#include <cstdint>
#include <mutex>
#include <new>
#include <type_traits>
#include <vector>
#include <cufft.h>

#include "ops.cuh"

namespace vdvc {

template <typename T, typename U>
__global__ void k_crop_to(const T* __restrict__ in, int nx, int ny, int sx, int sy, int sz, U* __restrict__ out) {
  const long long n = (long long)sx * sy * sz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(t % sx);
    const long long r = t / sx;
    const int y = (int)(r % sy), z = (int)(r / sy);
    out[t] = (U)in[(long long)x + (long long)y * nx + (long long)z * nx * ny];
  }
}

// R = F conj(G) / (|F conj(G)| + 1e-12), written over F, in the transforms'
// precision.
__device__ __forceinline__ double cabs_of(double re, double im) { return hypot(re, im); }
__device__ __forceinline__ float cabs_of(float re, float im) { return hypotf(re, im); }

template <typename C, typename R>
__global__ void k_cross_power(C* __restrict__ F, const C* __restrict__ G, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const C a = F[i], b = G[i];
    const R re = a.x * b.x + a.y * b.y;  // a * conj(b)
    const R im = a.y * b.x - a.x * b.y;
    const R den = cabs_of(re, im) + (R)1e-12;
    F[i].x = re / den;
    F[i].y = im / den;
  }
}

struct ArgMax {
  double v;
  long long cidx;  // C-order index of pix[x,y,z]
};

__device__ __forceinline__ ArgMax better(ArgMax a, ArgMax b) {
  if (b.v > a.v || (b.v == a.v && b.cidx < a.cidx)) return b;
  return a;
}

template <typename T>
__global__ void __launch_bounds__(256) k_argmax(const T* __restrict__ r, int sx, int sy, int sz,
                                                ArgMax* __restrict__ partial, unsigned int* ticket,
                                                ArgMax* __restrict__ result) {
  __shared__ ArgMax s[256];
  __shared__ bool s_last;
  const long long n = (long long)sx * sy * sz;
  ArgMax best{-1.0e300, (long long)1 << 62};
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(t % sx);
    const long long q = t / sx;
    const int y = (int)(q % sy), z = (int)(q / sy);
    const ArgMax c{(double)r[t], ((long long)x * sy + y) * sz + z};
    best = better(best, c);
  }
  s[threadIdx.x] = best;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] = better(s[threadIdx.x], s[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = s[0];
    __threadfence();
    s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    ArgMax b, b2;
    b.v = ((volatile double*)&partial[0].v)[0];
    b.cidx = ((volatile long long*)&partial[0].cidx)[0];
    for (unsigned int i = 1; i < gridDim.x; ++i) {
      b2.v = ((volatile double*)&partial[i].v)[0];
      b2.cidx = ((volatile long long*)&partial[i].cidx)[0];
      b = better(b, b2);
    }
    *result = b;
    *ticket = 0u;
  }
}

// float: four products (or values) summed in FP32 per float4, then one FP64
// add -- FP64 arithmetic per element would run on GB300's narrow FP64 pipe.
template <typename T>
__global__ void __launch_bounds__(256) k_dot(const T* __restrict__ a, const T* __restrict__ b, long long n,
                                             GridReduce red, double* __restrict__ out, bool vec4) {
  __shared__ double s_red[8];
  double acc = 0.0;
  const long long gtid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i0 = 0;
  if constexpr (std::is_same<T, float>::value) {
    if (vec4) {
      const long long n4 = n >> 2;
      for (long long q = gtid; q < n4; q += stride) {
        const float4 x = __ldg((const float4*)a + q);
        float s4;
        if (b) {
          const float4 y = __ldg((const float4*)b + q);
          s4 = x.x * y.x + x.y * y.y + x.z * y.z + x.w * y.w;
        } else {
          s4 = (x.x + x.y) + (x.z + x.w);
        }
        acc += (double)s4;
      }
      i0 = n4 << 2;
    }
  }
  for (long long i = i0 + gtid; i < n; i += stride)
    acc += b ? (double)a[i] * (double)b[i] : (double)a[i];
  double mine[1] = {block_sum(acc, s_red)}, o[1];
  if (grid_reduce_sum<1>(red, mine, o, s_red) && threadIdx.x == 0) *out = o[0];
}

// cuFFT plans and work buffers of the phase correlation, cached per
// (device, shape): creating a plan pair costs milliseconds (a workspace
// allocation and the plan build), against well under a millisecond for the
// transforms of a pyramid's coarsest level.  A plan is taken out of the
// cache for the duration of a call (never shared by two calls at once) and
// put back after the call's stream has finished with it.
struct FftPlan {
  int dev, sx, sy, sz;
  bool single;  // R2C / C2R on float and cufftComplex buffers (else D2Z / Z2D on double)
  cufftHandle pf, pi;
  void *fr, *gr;  // real volumes
  void *Fc, *Gc;  // half spectra
  ArgMax *partial, *result;
  unsigned int* ticket;
  cudaEvent_t done;  // recorded after a call's last use; the next user's stream waits on it
  size_t bytes;
  unsigned long long stamp;
};

static std::mutex g_fft_mu;
static std::vector<FftPlan*> g_fft_cache;
static unsigned long long g_fft_clock = 0;
constexpr size_t kFftCacheBytes = (size_t)4 << 30;
constexpr size_t kFftCacheEntries = 32;

static void fft_destroy(FftPlan* P) {
  if (!P) return;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != P->dev) cudaSetDevice(P->dev);
  if (P->done) {
    cudaEventSynchronize(P->done);  // no call still uses the buffers
    cudaEventDestroy(P->done);
  }
  if (P->pf) cufftDestroy(P->pf);
  if (P->pi) cufftDestroy(P->pi);
  cudaFree(P->fr);
  cudaFree(P->gr);
  cudaFree(P->Fc);
  cudaFree(P->Gc);
  cudaFree(P->partial);
  cudaFree(P->result);
  cudaFree(P->ticket);
  if (cur != P->dev) cudaSetDevice(cur);
  delete P;
}

static int fft_acquire(int sx, int sy, int sz, bool single, cudaStream_t s, FftPlan** out) {
  int dev = 0;
  VDVC_CUDA(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lk(g_fft_mu);
    for (size_t i = 0; i < g_fft_cache.size(); ++i) {
      FftPlan* P = g_fft_cache[i];
      if (P->dev == dev && P->sx == sx && P->sy == sy && P->sz == sz && P->single == single) {
        g_fft_cache.erase(g_fft_cache.begin() + i);
        *out = P;
        // the previous call may still be running on its stream
        VDVC_CUDA(cudaStreamWaitEvent(s, P->done, 0));
        return VDVC_OK;
      }
    }
  }
  const long long n = (long long)sx * sy * sz;
  const long long nc = (long long)sz * sy * (sx / 2 + 1);
  FftPlan* P = new (std::nothrow) FftPlan{};
  if (!P) return set_error(VDVC_ERR_ARG, "host allocation failed");
  P->dev = dev;
  P->sx = sx;
  P->sy = sy;
  P->sz = sz;
  P->single = single;
  const size_t rb = single ? sizeof(float) : sizeof(double);
  const size_t cb = single ? sizeof(cufftComplex) : sizeof(cufftDoubleComplex);
  P->bytes = (size_t)(2 * n) * rb + (size_t)(2 * nc) * cb;
  if (cudaMalloc(&P->fr, n * rb) != cudaSuccess || cudaMalloc(&P->gr, n * rb) != cudaSuccess ||
      cudaMalloc(&P->Fc, nc * cb) != cudaSuccess || cudaMalloc(&P->Gc, nc * cb) != cudaSuccess ||
      cudaMalloc((void**)&P->partial, kReduceBlocks * sizeof(ArgMax)) != cudaSuccess ||
      cudaMalloc((void**)&P->result, sizeof(ArgMax)) != cudaSuccess ||
      cudaMalloc((void**)&P->ticket, sizeof(unsigned int)) != cudaSuccess ||
      cudaEventCreateWithFlags(&P->done, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    fft_destroy(P);
    return set_error(VDVC_ERR_CUDA, "fft_rigid_shift: device allocation failed");
  }
  if (cufftPlan3d(&P->pf, sz, sy, sx, single ? CUFFT_R2C : CUFFT_D2Z) != CUFFT_SUCCESS) {
    P->pf = 0;
    fft_destroy(P);
    return set_error(VDVC_ERR_CUFFT, "fft_rigid_shift: plan creation failed");
  }
  if (cufftPlan3d(&P->pi, sz, sy, sx, single ? CUFFT_C2R : CUFFT_Z2D) != CUFFT_SUCCESS) {
    P->pi = 0;
    fft_destroy(P);
    return set_error(VDVC_ERR_CUFFT, "fft_rigid_shift: plan creation failed");
  }
  *out = P;
  return VDVC_OK;
}

static void fft_release(FftPlan* P, bool reuse, cudaStream_t s) {
  if (!reuse || cudaEventRecord(P->done, s) != cudaSuccess) {
    fft_destroy(P);
    return;
  }
  std::vector<FftPlan*> evicted;
  {
    std::lock_guard<std::mutex> lk(g_fft_mu);
    P->stamp = ++g_fft_clock;
    g_fft_cache.push_back(P);
    size_t total = 0;
    for (FftPlan* q : g_fft_cache) total += q->bytes;
    while (g_fft_cache.size() > 1 && (total > kFftCacheBytes || g_fft_cache.size() > kFftCacheEntries)) {
      size_t oldest = 0;
      for (size_t i = 1; i < g_fft_cache.size(); ++i)
        if (g_fft_cache[i]->stamp < g_fft_cache[oldest]->stamp) oldest = i;
      total -= g_fft_cache[oldest]->bytes;
      evicted.push_back(g_fft_cache[oldest]);
      g_fft_cache.erase(g_fft_cache.begin() + oldest);
    }
  }
  for (FftPlan* q : evicted) fft_destroy(q);
}

}  // namespace vdvc

using namespace vdvc;

#define VDVC_CUFFT(expr)                                                                 \
  do {                                                                                   \
    cufftResult r_ = (expr);                                                             \
    if (r_ != CUFFT_SUCCESS) {                                                           \
      st = set_error(VDVC_ERR_CUFFT, "%s failed with cufftResult %d", #expr, (int)r_);  \
      goto cleanup;                                                                      \
    }                                                                                    \
  } while (0)

extern "C" {

int vdvc_dot(const void* a, const void* b, int dtype, long long n, double* out_host, void* ws, size_t ws_bytes,
             vdvc_stream_t stream) {
  VDVC_CHECK_ARG(out_host, "bad arguments");
  Carve cv(ws, ws_bytes);
  cv.take<double>(kReduceBlocks);
  cv.take<unsigned int>(1);
  double* res = cv.take<double>(1);
  if (!ws || !cv.fits()) return set_error(VDVC_ERR_WORKSPACE, "dot needs %zu bytes", cv.off);
  int st = vdvc_dot_device(a, b, dtype, n, res, ws, ws_bytes, stream);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemcpyAsync(out_host, res, sizeof(double), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaStreamSynchronize(s));
  return VDVC_OK;
}

int vdvc_dot_device(const void* a, const void* b, int dtype, long long n, double* out_dev, void* ws, size_t ws_bytes,
                    vdvc_stream_t stream) {
  VDVC_CHECK_ARG(a && out_dev && n >= 1, "bad arguments");
  Carve cv(ws, ws_bytes);
  double* partials = cv.take<double>(kReduceBlocks);
  unsigned int* ticket = cv.take<unsigned int>(1);
  double* res = out_dev;
  if (!ws || !cv.fits()) return set_error(VDVC_ERR_WORKSPACE, "dot needs %zu bytes", cv.off);
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s));
  GridReduce red{partials, ticket};
  const bool vec4 = (((uintptr_t)a | (uintptr_t)b) & 15u) == 0;
  const int nb = grid_blocks(dtype == VDVC_F32 && vec4 ? (n + 3) / 4 : n, 256, kReduceBlocks);
  if (dtype == VDVC_F32)
    k_dot<float><<<nb, 256, 0, s>>>((const float*)a, (const float*)b, n, red, res, vec4);
  else if (dtype == VDVC_F64)
    k_dot<double><<<nb, 256, 0, s>>>((const double*)a, (const double*)b, n, red, res, false);
  else
    return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

// The shift from the arg-max's C-order index of pix[x,y,z]: (x,y,z)
// wrapped to (-n/2, n/2] per axis, d = -peak.
__host__ __device__ inline void shift_from_cidx(long long c, int sx, int sy, int sz, double* d) {
  const int pz = (int)(c % sz);
  c /= sz;
  const int py = (int)(c % sy);
  const int px = (int)(c / sy);
  const int p[3] = {px, py, pz}, ns[3] = {sx, sy, sz};
  for (int a = 0; a < 3; ++a) {
    int q = p[a];
    if (q > ns[a] / 2) q -= ns[a];
    d[a] = -(double)q;
  }
}

__global__ void k_shift_out(const ArgMax* __restrict__ r, int sx, int sy, int sz, double* __restrict__ d) {
  if (threadIdx.x == 0 && blockIdx.x == 0) shift_from_cidx(r->cidx, sx, sy, sz, d);
}

// Enqueues the phase correlation; the shift goes to d_dev (device, no host
// synchronisation) or, when d_dev is null, to d_host after a synchronisation.
static int fft_shift(const void* f_vox, int fnx, int fny, int fnz, const void* g_vox, int gnx, int gny, int gnz,
                     int dtype, double* d_host, double* d_dev, cudaStream_t s) {
  const int sx = fnx < gnx ? fnx : gnx, sy = fny < gny ? fny : gny, sz = fnz < gnz ? fnz : gnz;
  const long long n = (long long)sx * sy * sz;
  const long long nc = (long long)sz * sy * (sx / 2 + 1);
  const bool single = dtype == VDVC_F32;
  FftPlan* P = nullptr;
  int st = fft_acquire(sx, sy, sz, single, s, &P);
  if (st) return st;
  const int nb = grid_blocks(n, 256, kReduceBlocks);
  ArgMax host;
  bool ok = cudaMemsetAsync(P->ticket, 0, sizeof(unsigned int), s) == cudaSuccess;
  if (ok) {
    if (single) {
      k_crop_to<float, float><<<nb, 256, 0, s>>>((const float*)f_vox, fnx, fny, sx, sy, sz, (float*)P->fr);
      k_crop_to<float, float><<<nb, 256, 0, s>>>((const float*)g_vox, gnx, gny, sx, sy, sz, (float*)P->gr);
    } else {
      k_crop_to<double, double><<<nb, 256, 0, s>>>((const double*)f_vox, fnx, fny, sx, sy, sz, (double*)P->fr);
      k_crop_to<double, double><<<nb, 256, 0, s>>>((const double*)g_vox, gnx, gny, sx, sy, sz, (double*)P->gr);
    }
    count_launch(2);
    ok = cufftSetStream(P->pf, s) == CUFFT_SUCCESS && cufftSetStream(P->pi, s) == CUFFT_SUCCESS;
    if (ok && single)
      ok = cufftExecR2C(P->pf, (cufftReal*)P->fr, (cufftComplex*)P->Fc) == CUFFT_SUCCESS &&
           cufftExecR2C(P->pf, (cufftReal*)P->gr, (cufftComplex*)P->Gc) == CUFFT_SUCCESS;
    else if (ok)
      ok = cufftExecD2Z(P->pf, (cufftDoubleReal*)P->fr, (cufftDoubleComplex*)P->Fc) == CUFFT_SUCCESS &&
           cufftExecD2Z(P->pf, (cufftDoubleReal*)P->gr, (cufftDoubleComplex*)P->Gc) == CUFFT_SUCCESS;
    if (!ok) st = set_error(VDVC_ERR_CUFFT, "fft_rigid_shift: forward transforms failed");
  } else {
    st = set_error(VDVC_ERR_CUDA, "memset");
  }
  if (ok) {
    const int nbc = grid_blocks(nc, 256, 152 * 16);
    if (single) {
      k_cross_power<cufftComplex, float><<<nbc, 256, 0, s>>>((cufftComplex*)P->Fc, (const cufftComplex*)P->Gc, nc);
      count_launch();
      ok = cufftExecC2R(P->pi, (cufftComplex*)P->Fc, (cufftReal*)P->fr) == CUFFT_SUCCESS;
    } else {
      k_cross_power<cufftDoubleComplex, double><<<nbc, 256, 0, s>>>((cufftDoubleComplex*)P->Fc,
                                                                     (const cufftDoubleComplex*)P->Gc, nc);
      count_launch();
      ok = cufftExecZ2D(P->pi, (cufftDoubleComplex*)P->Fc, (cufftDoubleReal*)P->fr) == CUFFT_SUCCESS;
    }
    if (!ok) st = set_error(VDVC_ERR_CUFFT, "fft_rigid_shift: inverse transform failed");
  }
  if (ok) {
    if (single)
      k_argmax<float><<<nb, 256, 0, s>>>((const float*)P->fr, sx, sy, sz, P->partial, P->ticket, P->result);
    else
      k_argmax<double><<<nb, 256, 0, s>>>((const double*)P->fr, sx, sy, sz, P->partial, P->ticket, P->result);
    count_launch();
    if (d_dev) {
      k_shift_out<<<1, 32, 0, s>>>(P->result, sx, sy, sz, d_dev);
      count_launch();
      ok = cudaGetLastError() == cudaSuccess;
    } else {
      ok = cudaMemcpyAsync(&host, P->result, sizeof(ArgMax), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
           cudaStreamSynchronize(s) == cudaSuccess;
    }
    if (!ok) st = set_error(VDVC_ERR_CUDA, "fft_rigid_shift: %s", cudaGetErrorString(cudaGetLastError()));
  }
  if (ok && !d_dev) shift_from_cidx(host.cidx, sx, sy, sz, d_host);
  // the plan goes back with an event after its last use on this stream (the
  // next user's stream waits on it); after a failure it is dropped
  fft_release(P, ok, s);
  return st;
}

int vdvc_fft_rigid_shift(const void* f_vox, int fnx, int fny, int fnz, const void* g_vox, int gnx, int gny, int gnz,
                         int dtype, double* d_out3, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f_vox && g_vox && d_out3, "null pointer");
  VDVC_CHECK_ARG(fnx >= 1 && fny >= 1 && fnz >= 1 && gnx >= 1 && gny >= 1 && gnz >= 1, "bad shapes");
  VDVC_CHECK_ARG(dtype == VDVC_F32 || dtype == VDVC_F64, "dtype %d", dtype);
  return fft_shift(f_vox, fnx, fny, fnz, g_vox, gnx, gny, gnz, dtype, d_out3, nullptr, (cudaStream_t)stream);
}

int vdvc_fft_rigid_shift_device(const void* f_vox, int fnx, int fny, int fnz, const void* g_vox, int gnx, int gny,
                                int gnz, int dtype, double* d_dev3, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f_vox && g_vox && d_dev3, "null pointer");
  VDVC_CHECK_ARG(fnx >= 1 && fny >= 1 && fnz >= 1 && gnx >= 1 && gny >= 1 && gnz >= 1, "bad shapes");
  VDVC_CHECK_ARG(dtype == VDVC_F32 || dtype == VDVC_F64, "dtype %d", dtype);
  return fft_shift(f_vox, fnx, fny, fnz, g_vox, gnx, gny, gnz, dtype, nullptr, d_dev3, (cudaStream_t)stream);
}

}  // extern "C"
