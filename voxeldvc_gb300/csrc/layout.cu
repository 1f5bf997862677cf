// Image layout and reference-image preparation kernels:
//   pix -> vox transpose with cast, strided decimation, the xp.gradient
//   stencil with the mask0 / 6-neighbour erosion fused in (and, for a GN
//   level, the reference statistics over mask0), and the erosion on its own.
#include "ops.cuh"

namespace vdvc {
namespace {

// C-order (nx,ny,nz) -> x-fastest: 32x32 (z,x) tiles of kP2vPlanes
// consecutive y planes per block (blockIdx.z), staged through shared memory
// so both sides are coalesced; a thread has 4 * kP2vPlanes loads in flight.
// With a step s > 1 the output is the every-s-th-voxel grid
// (nx, ny, nz here being its extents): the transpose of the strided
// decimation, reading only those voxels (a warp's 32 z-values span 32 s
// consecutive source elements).
constexpr int kP2vPlanes = 4;

// Tiles are numbered z-tile fastest; a block walks tiles blockIdx.x,
// blockIdx.x + gridDim.x, ... (one tile per block, or a bounded grid for a
// transpose that runs in the background of other work).
template <typename Tin, typename Tout>
__global__ void __launch_bounds__(256) k_pix_to_vox(const Tin* __restrict__ in, Tout* __restrict__ out,
                                                    int nx, int ny, int nz, int s, int sny, int snz) {
  __shared__ Tout tile[kP2vPlanes][32][33];
  const long long nzt = (nz + 31) / 32, nxt = (nx + 31) / 32, nyt = (ny + kP2vPlanes - 1) / kP2vPlanes;
  for (long long tl = blockIdx.x; tl < nzt * nxt * nyt; tl += gridDim.x) {
    const int z0 = (int)(tl % nzt) * 32, x0 = (int)((tl / nzt) % nxt) * 32;
    const int y0 = (int)(tl / (nzt * nxt)) * kP2vPlanes;
    __syncthreads();  // the previous tile's reads of `tile` are done
#pragma unroll
    for (int p = 0; p < kP2vPlanes; ++p) {
      const int y = y0 + p;
#pragma unroll
      for (int r = threadIdx.y; r < 32; r += 8) {
        const int x = x0 + r, z = z0 + threadIdx.x;
        if (y < ny && x < nx && z < nz)
          tile[p][r][threadIdx.x] = (Tout)in[((size_t)x * s * sny + (size_t)y * s) * snz + (size_t)z * s];
      }
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < kP2vPlanes; ++p) {
      const int y = y0 + p;
#pragma unroll
      for (int r = threadIdx.y; r < 32; r += 8) {
        const int z = z0 + r, x = x0 + threadIdx.x;
        if (y < ny && x < nx && z < nz)
          out[(size_t)x + (size_t)y * nx + (size_t)z * nx * ny] = tile[p][threadIdx.x][r];
      }
    }
  }
}

template <typename E>
__global__ void k_decimate(const E* __restrict__ in, E* __restrict__ out, int nx, int ny, int ox, int oy,
                           int oz, int s) {
  const long long n = (long long)ox * oy * oz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(t % ox);
    const long long r = t / ox;
    const int y = (int)(r % oy), z = (int)(r / oy);
    out[t] = in[(size_t)x * s + (size_t)y * s * nx + (size_t)z * s * nx * ny];
  }
}

// One component of xp.gradient with edge_order=1 (numpy's default): central
// difference / 2 inside, first-order one-sided difference at both ends.
template <typename T>
__device__ __forceinline__ T gradient_1d(T fm, T f0, T fp, int i, int n) {
  if (i == 0) return fp - f0;
  if (i == n - 1) return f0 - fm;
  return (fp - fm) * T(0.5);
}

template <typename T>
__global__ void __launch_bounds__(256) k_image_grad(const T* __restrict__ f, int nx, int ny, int nz, T glt,
                                                    T* __restrict__ grad, uint8_t* __restrict__ mask0,
                                                    bool with_mask) {
  const long long nxy = (long long)nx * ny, n = nxy * nz;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(v % nx);
    const long long r = v / nx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    const long long xm = v - (x > 0), xp = v + (x < nx - 1);
    const long long ym = v - (y > 0) * nx, yp = v + (y < ny - 1) * (long long)nx;
    const long long zm = v - (z > 0) * nxy, zp = v + (z < nz - 1) * nxy;
    const T c = f[v];
    const T fxm = f[xm], fxp = f[xp], fym = f[ym], fyp = f[yp], fzm = f[zm], fzp = f[zp];
    T gx = gradient_1d(fxm, c, fxp, x, nx);
    T gy = gradient_1d(fym, c, fyp, y, ny);
    T gz = gradient_1d(fzm, c, fzp, z, nz);
    if (with_mask) {
      const bool m = c > glt;
      // minimum_filter with the 6-neighbour footprint, mode 'nearest': a
      // clamped neighbour is the voxel itself.
      const bool keep = m && (fxm > glt) && (fxp > glt) && (fym > glt) && (fyp > glt) && (fzm > glt) &&
                        (fzp > glt);
      mask0[v] = m ? 1 : 0;
      if (!keep) gx = gy = gz = T(0);
    }
    grad[3 * v + 0] = gx;
    grad[3 * v + 1] = gy;
    grad[3 * v + 2] = gz;
  }
}

// Blocks of the fused pass: enough 256-thread blocks for ~7 voxel loads in
// flight per thread to cover HBM latency (1024 left it latency-bound), one
// float64 partial triple each.
constexpr int kImageGradStatsBlocks = 8192;

// k_image_grad<float> with mask0 plus the multiplicity-weighted sums of f
// over mask0 (vdvc_masked_stats' count, sum, sum of squares) in the same
// read of f: 32-bit voxel indices, float partials folded into float64
// every 64 voxels of a thread (GB300's FP64 pipe is narrow), one block
// partial each, grid-reduced.
__global__ void __launch_bounds__(256) k_image_grad_stats(const float* __restrict__ f, int nx, int ny, int nz,
                                                          float glt, float* __restrict__ grad,
                                                          uint8_t* __restrict__ mask0, int h, int Ex, int Ey,
                                                          int Ez, GridReduce red, double* __restrict__ out3) {
  __shared__ double s_red[8];
  const unsigned int unx = (unsigned int)nx, uny = (unsigned int)ny;
  const unsigned int nxy = unx * uny, n = nxy * (unsigned int)nz;
  double acc[3] = {0.0, 0.0, 0.0};
  float fc = 0.f, f1 = 0.f, f2 = 0.f;
  int cnt = 0;
  for (unsigned int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const unsigned int r = v / unx;
    const int x = (int)(v - r * unx), y = (int)(r % uny), z = (int)(r / uny);
    const unsigned int xm = v - (x > 0), xp = v + (x < nx - 1);
    const unsigned int ym = v - (y > 0) * unx, yp = v + (y < ny - 1) * unx;
    const unsigned int zm = v - (z > 0) * nxy, zp = v + (z < nz - 1) * nxy;
    const float c = f[v];
    const float fxm = f[xm], fxp = f[xp], fym = f[ym], fyp = f[yp], fzm = f[zm], fzp = f[zp];
    float gx = gradient_1d(fxm, c, fxp, x, nx);
    float gy = gradient_1d(fym, c, fyp, y, ny);
    float gz = gradient_1d(fzm, c, fzp, z, nz);
    const bool m = c > glt;
    const bool keep = m && (fxm > glt) && (fxp > glt) && (fym > glt) && (fyp > glt) && (fzm > glt) && (fzp > glt);
    mask0[v] = m ? 1 : 0;
    if (!keep) gx = gy = gz = 0.f;
    grad[3 * (size_t)v + 0] = gx;
    grad[3 * (size_t)v + 1] = gy;
    grad[3 * (size_t)v + 2] = gz;
    if (m) {
      const float mult =
          (float)(axis_multiplicity(x, h, Ex) * axis_multiplicity(y, h, Ey) * axis_multiplicity(z, h, Ez));
      fc += mult;
      f1 += mult * c;
      f2 += mult * c * c;
    }
    if (++cnt == 64) {
      acc[0] += fc;
      acc[1] += f1;
      acc[2] += f2;
      fc = f1 = f2 = 0.f;
      cnt = 0;
    }
  }
  acc[0] += fc;
  acc[1] += f1;
  acc[2] += f2;
  double b3[3], o3[3];
  for (int q = 0; q < 3; ++q) b3[q] = block_sum(acc[q], s_red);
  if (grid_reduce_sum<3>(red, b3, o3, s_red) && threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) out3[q] = o3[q];
}

__global__ void k_erode(const uint8_t* __restrict__ m, int nx, int ny, int nz, uint8_t* __restrict__ out) {
  const long long nxy = (long long)nx * ny, n = nxy * nz;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(v % nx);
    const long long r = v / nx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    bool keep = m[v] && m[v - (x > 0)] && m[v + (x < nx - 1)] && m[v - (y > 0) * nx] &&
                m[v + (y < ny - 1) * (long long)nx] && m[v - (z > 0) * nxy] && m[v + (z < nz - 1) * nxy];
    out[v] = keep ? 1 : 0;
  }
}

inline int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 152LL * 64) b = 152LL * 64;
  if (b < 1) b = 1;
  return (int)b;
}

// (nx, ny, nz): the source; the output grid is ceil(n / step) per axis;
// max_blocks > 0 bounds the grid (the blocks then walk the tiles)
template <typename Tin, typename Tout>
int launch_p2v(const void* pix, int nx, int ny, int nz, int step, long long max_blocks, void* vox, cudaStream_t s) {
  const int ox = (nx + step - 1) / step, oy = (ny + step - 1) / step, oz = (nz + step - 1) / step;
  long long tiles = (long long)((oz + 31) / 32) * ((ox + 31) / 32) * ((oy + kP2vPlanes - 1) / kP2vPlanes);
  if (max_blocks > 0 && tiles > max_blocks) tiles = max_blocks;
  if (tiles >= 0x7fffffffLL) return set_error(VDVC_ERR_ARG, "image too large");
  k_pix_to_vox<Tin, Tout><<<(unsigned)tiles, dim3(32, 8), 0, s>>>((const Tin*)pix, (Tout*)vox, ox, oy, oz, step, ny,
                                                                  nz);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

template <typename Tout>
int p2v_dispatch(const void* pix, int pix_dtype, int nx, int ny, int nz, int step, long long mb, void* vox,
                 cudaStream_t s) {
  switch (pix_dtype) {
    case VDVC_F32: return launch_p2v<float, Tout>(pix, nx, ny, nz, step, mb, vox, s);
    case VDVC_F64: return launch_p2v<double, Tout>(pix, nx, ny, nz, step, mb, vox, s);
    case VDVC_U8: return launch_p2v<uint8_t, Tout>(pix, nx, ny, nz, step, mb, vox, s);
    case VDVC_U16: return launch_p2v<uint16_t, Tout>(pix, nx, ny, nz, step, mb, vox, s);
    case VDVC_I16: return launch_p2v<int16_t, Tout>(pix, nx, ny, nz, step, mb, vox, s);
    case VDVC_I32: return launch_p2v<int32_t, Tout>(pix, nx, ny, nz, step, mb, vox, s);
  }
  return set_error(VDVC_ERR_ARG, "pix_dtype %d not supported", pix_dtype);
}

}  // namespace
}  // namespace vdvc

using namespace vdvc;

extern "C" {

int vdvc_pix_to_vox(const void* pix, int pix_dtype, int nx, int ny, int nz, void* vox, int dtype,
                    vdvc_stream_t stream) {
  VDVC_CHECK_ARG(pix && vox, "null pointer");
  VDVC_CHECK_ARG(nx >= 1 && ny >= 1 && nz >= 1 && ny <= 65535, "bad image shape (%d,%d,%d)", nx, ny, nz);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == VDVC_F32) return p2v_dispatch<float>(pix, pix_dtype, nx, ny, nz, 1, 0, vox, s);
  if (dtype == VDVC_F64) return p2v_dispatch<double>(pix, pix_dtype, nx, ny, nz, 1, 0, vox, s);
  return set_error(VDVC_ERR_ARG, "dtype %d must be VDVC_F32 or VDVC_F64", dtype);
}

int vdvc_pix_to_vox_strided(const void* pix, int pix_dtype, int nx, int ny, int nz, int step, int max_blocks,
                            void* vox, int dtype, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(pix && vox, "null pointer");
  VDVC_CHECK_ARG(step >= 1 && step <= 64, "step %d must be in [1, 64]", step);
  VDVC_CHECK_ARG(max_blocks >= 0, "max_blocks must be >= 0");
  VDVC_CHECK_ARG(nx >= 1 && ny >= 1 && nz >= 1, "bad image shape (%d,%d,%d)", nx, ny, nz);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == VDVC_F32) return p2v_dispatch<float>(pix, pix_dtype, nx, ny, nz, step, max_blocks, vox, s);
  if (dtype == VDVC_F64) return p2v_dispatch<double>(pix, pix_dtype, nx, ny, nz, step, max_blocks, vox, s);
  return set_error(VDVC_ERR_ARG, "dtype %d must be VDVC_F32 or VDVC_F64", dtype);
}

int vdvc_decimate(const void* in, int dtype, int nx, int ny, int nz, int s, void* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(in && out, "null pointer");
  VDVC_CHECK_ARG(nx >= 1 && ny >= 1 && nz >= 1 && s >= 1, "bad shape/stride");
  const int ox = (nx + s - 1) / s, oy = (ny + s - 1) / s, oz = (nz + s - 1) / s;
  const long long n = (long long)ox * oy * oz;
  const int threads = 256, blocks = grid_for(n, threads);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t es = dtype_size(dtype);
  if (es == 4)
    k_decimate<uint32_t><<<blocks, threads, 0, st>>>((const uint32_t*)in, (uint32_t*)out, nx, ny, ox, oy, oz, s);
  else if (es == 8)
    k_decimate<uint64_t><<<blocks, threads, 0, st>>>((const uint64_t*)in, (uint64_t*)out, nx, ny, ox, oy, oz, s);
  else if (es == 2)
    k_decimate<uint16_t><<<blocks, threads, 0, st>>>((const uint16_t*)in, (uint16_t*)out, nx, ny, ox, oy, oz, s);
  else if (es == 1)
    k_decimate<uint8_t><<<blocks, threads, 0, st>>>((const uint8_t*)in, (uint8_t*)out, nx, ny, ox, oy, oz, s);
  else
    return set_error(VDVC_ERR_ARG, "dtype %d not supported", dtype);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_image_grad(const void* f_vox, int dtype, int Nvx, int Nvy, int Nvz, double glt, void* grad,
                    uint8_t* mask0, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f_vox && grad, "null pointer");
  // numpy's gradient needs at least 2 samples per axis (edge_order + 1).
  VDVC_CHECK_ARG(Nvx >= 2 && Nvy >= 2 && Nvz >= 2, "gradient needs >= 2 voxels per axis");
  const long long n = (long long)Nvx * Nvy * Nvz;
  const int threads = 256, blocks = grid_for(n, threads);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == VDVC_F32)
    k_image_grad<float><<<blocks, threads, 0, s>>>((const float*)f_vox, Nvx, Nvy, Nvz, (float)glt, (float*)grad,
                                                   mask0, mask0 != nullptr);
  else if (dtype == VDVC_F64)
    k_image_grad<double><<<blocks, threads, 0, s>>>((const double*)f_vox, Nvx, Nvy, Nvz, glt, (double*)grad,
                                                    mask0, mask0 != nullptr);
  else
    return set_error(VDVC_ERR_ARG, "dtype %d must be VDVC_F32 or VDVC_F64", dtype);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_image_grad_stats(const float* f_vox, int Nvx, int Nvy, int Nvz, double glt, float* grad, uint8_t* mask0,
                          int h, int Nx, int Ny, int Nz, double* out3, void* ws, size_t ws_bytes,
                          vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f_vox && grad && mask0 && out3, "null pointer");
  VDVC_CHECK_ARG(Nvx >= 2 && Nvy >= 2 && Nvz >= 2, "gradient needs >= 2 voxels per axis");
  Mesh m;
  if (int st = make_mesh(h, Nx, Ny, Nz, &m)) return st;
  VDVC_CHECK_ARG(m.Nvx == Nvx && m.Nvy == Nvy && m.Nvz == Nvz, "image (%d,%d,%d) is not the mesh's voxel grid",
                 Nvx, Nvy, Nvz);
  Carve cv(ws, ws_bytes);
  GridReduce red;
  red.partials = cv.take<double>(3 * kImageGradStatsBlocks);
  red.ticket = cv.take<unsigned int>(1);
  VDVC_CHECK_ARG(ws && cv.fits(), "image_grad_stats needs %zu bytes of workspace", cv.off);
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(red.ticket, 0, sizeof(unsigned int), s));
  const long long n = (long long)Nvx * Nvy * Nvz;
  k_image_grad_stats<<<grid_blocks(n, 256, kImageGradStatsBlocks), 256, 0, s>>>(f_vox, Nvx, Nvy, Nvz, (float)glt,
                                                                               grad, mask0, h, Nx, Ny, Nz, red, out3);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_erode_mask(const uint8_t* mask, int Nvx, int Nvy, int Nvz, uint8_t* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(mask && out && mask != out, "null or aliased pointer");
  VDVC_CHECK_ARG(Nvx >= 1 && Nvy >= 1 && Nvz >= 1, "bad shape");
  const long long n = (long long)Nvx * Nvy * Nvz;
  const int threads = 256, blocks = grid_for(n, threads);
  k_erode<<<blocks, threads, 0, (cudaStream_t)stream>>>(mask, Nvx, Nvy, Nvz, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

}  // extern "C"
