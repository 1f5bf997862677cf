// Post-solve voxel stages of `voxeldvc run`'s outputs
// (engine/write_output.py): pushing a voxel field forward by the recovered
// displacement, and the ZNCC correlation-quality figure.
//
// Both are float64 passes over the voxel grid, run once per solve: the
// push's sample coordinates x - u(x) decide nearest-neighbour picks of label
// fields at half-integers, so they are formed in float64 as the reference's
// float64 displacement and index ramps are; the ZNCC sums follow the
// reference's two passes (means, then centred sums).
#include <limits>

#include "ops.cuh"

namespace vdvc {

// scipy.ndimage.map_coordinates semantics (the reference samples with it):
// order 0 picks floor(c + 1/2) per axis, order 1 is trilinear; mode
// 'nearest' clamps to [0, n-1], mode 'constant' returns cval when any axis
// coordinate lies outside [0, n-1].
template <typename T>
__global__ void k_push(const T* __restrict__ field, const double* __restrict__ u, int nx, int ny, int nz, int order,
                       int constant_mode, double cval, T* __restrict__ out) {
  const long long n = (long long)nx * ny * nz;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(v % nx);
    const long long r = v / nx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    double c[3] = {(double)x - u[v], (double)y - u[n + v], (double)z - u[2 * n + v]};
    const int dims[3] = {nx, ny, nz};
    bool inside = true;
    for (int k = 0; k < 3; ++k) inside = inside && c[k] >= 0.0 && c[k] <= (double)(dims[k] - 1);
    if (constant_mode && !inside) {
      out[v] = (T)cval;
      continue;
    }
    for (int k = 0; k < 3; ++k) c[k] = fmin(fmax(c[k], 0.0), (double)(dims[k] - 1));
    if (order == 0) {
      int id[3];
      for (int k = 0; k < 3; ++k) id[k] = min((int)floor(c[k] + 0.5), dims[k] - 1);
      out[v] = field[((long long)id[2] * ny + id[1]) * nx + id[0]];
      continue;
    }
    int i0[3], i1[3];
    double t[3];
    for (int k = 0; k < 3; ++k) {
      const double fl = floor(c[k]);
      i0[k] = (int)fl;
      i1[k] = min(i0[k] + 1, dims[k] - 1);
      t[k] = c[k] - fl;
    }
    auto at = [&](int xx, int yy, int zz) { return (double)field[((long long)zz * ny + yy) * nx + xx]; };
    const double a00 = at(i0[0], i0[1], i0[2]) * (1 - t[0]) + at(i1[0], i0[1], i0[2]) * t[0];
    const double a10 = at(i0[0], i1[1], i0[2]) * (1 - t[0]) + at(i1[0], i1[1], i0[2]) * t[0];
    const double a01 = at(i0[0], i0[1], i1[2]) * (1 - t[0]) + at(i1[0], i0[1], i1[2]) * t[0];
    const double a11 = at(i0[0], i1[1], i1[2]) * (1 - t[0]) + at(i1[0], i1[1], i1[2]) * t[0];
    const double b0 = a00 * (1 - t[1]) + a10 * t[1], b1 = a01 * (1 - t[1]) + a11 * t[1];
    out[v] = (T)(b0 * (1 - t[2]) + b1 * t[2]);
  }
}

// pass 1: count, sum f, sum g over the mask; pass 2: centred products
template <typename T, int PASS>
__global__ void __launch_bounds__(256) k_zncc(const T* __restrict__ f, const T* __restrict__ g,
                                              const uint8_t* __restrict__ mask, long long n, const double* means,
                                              GridReduce red, double* out3) {
  __shared__ double s_red[8];
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  const double mf = PASS == 2 ? means[1] / means[0] : 0.0, mg = PASS == 2 ? means[2] / means[0] : 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (!mask[i]) continue;
    const double fv = (double)f[i], gv = (double)g[i];
    if (PASS == 1) {
      a0 += 1.0;
      a1 += fv;
      a2 += gv;
    } else {
      const double df = fv - mf, dg = gv - mg;
      a0 += df * dg;
      a1 += df * df;
      a2 += dg * dg;
    }
  }
  double b3[3] = {block_sum(a0, s_red), block_sum(a1, s_red), block_sum(a2, s_red)}, o3[3];
  if (grid_reduce_sum<3>(red, b3, o3, s_red) && threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) out3[q] = o3[q];
}

// float64 -> integer field with scipy.ndimage's output rounding (half away
// from zero) and saturation to the type's range; float32 by round-to-nearest
template <typename T>
__global__ void k_cast_round(const double* __restrict__ in, long long n, double lo, double hi, T* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double r = round(in[i]);
    out[i] = (T)fmin(fmax(r, lo), hi);
  }
}

__global__ void k_cast_f32(const double* __restrict__ in, long long n, float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

}  // namespace vdvc

using namespace vdvc;

extern "C" {

int vdvc_push_field(const void* field, int dtype, const double* u_cf, int nx, int ny, int nz, int order, int mode,
                    double cval, void* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(field && u_cf && out && nx >= 1 && ny >= 1 && nz >= 1, "bad arguments");
  VDVC_CHECK_ARG(order == 0 || order == 1, "order must be 0 or 1");
  VDVC_CHECK_ARG(mode == VDVC_MODE_NEAREST || mode == VDVC_MODE_CONSTANT, "mode must be nearest or constant");
  const long long n = (long long)nx * ny * nz;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = grid_blocks(n, 256, 152 * 32);
  if (dtype == VDVC_F32)
    k_push<float><<<nb, 256, 0, s>>>((const float*)field, u_cf, nx, ny, nz, order, mode == VDVC_MODE_CONSTANT, cval,
                                     (float*)out);
  else if (dtype == VDVC_F64)
    k_push<double><<<nb, 256, 0, s>>>((const double*)field, u_cf, nx, ny, nz, order, mode == VDVC_MODE_CONSTANT,
                                      cval, (double*)out);
  else if (dtype == VDVC_U8)
    k_push<uint8_t><<<nb, 256, 0, s>>>((const uint8_t*)field, u_cf, nx, ny, nz, order, mode == VDVC_MODE_CONSTANT,
                                       cval, (uint8_t*)out);
  else
    return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cast_round(const double* in, long long n, int dtype, void* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(in && out && n >= 0, "bad arguments");
  if (n == 0) return VDVC_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = grid_blocks(n, 256, 152 * 32);
  switch (dtype) {
    case VDVC_F32: k_cast_f32<<<nb, 256, 0, s>>>(in, n, (float*)out); break;
    case VDVC_U8: k_cast_round<uint8_t><<<nb, 256, 0, s>>>(in, n, 0.0, 255.0, (uint8_t*)out); break;
    case VDVC_U16: k_cast_round<uint16_t><<<nb, 256, 0, s>>>(in, n, 0.0, 65535.0, (uint16_t*)out); break;
    case VDVC_I16: k_cast_round<int16_t><<<nb, 256, 0, s>>>(in, n, -32768.0, 32767.0, (int16_t*)out); break;
    case VDVC_I32:
      k_cast_round<int32_t><<<nb, 256, 0, s>>>(in, n, -2147483648.0, 2147483647.0, (int32_t*)out);
      break;
    default: return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
  }
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_zncc(const void* f, const void* g, int dtype, const uint8_t* mask, long long n, double* out_host, void* ws,
              size_t ws_bytes, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f && g && mask && out_host && n >= 1, "bad arguments");
  Carve cv(ws, ws_bytes);
  double* partials = cv.take<double>((size_t)kReduceBlocks * 3);
  unsigned int* ticket = cv.take<unsigned int>(1);
  double* sums = cv.take<double>(6);
  if (!ws || !cv.fits()) return set_error(VDVC_ERR_WORKSPACE, "zncc needs %zu bytes", cv.off);
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s));
  GridReduce red{partials, ticket};
  const int nb = grid_blocks(n, 256, kReduceBlocks);
  if (dtype == VDVC_F32) {
    k_zncc<float, 1><<<nb, 256, 0, s>>>((const float*)f, (const float*)g, mask, n, nullptr, red, sums);
    k_zncc<float, 2><<<nb, 256, 0, s>>>((const float*)f, (const float*)g, mask, n, sums, red, sums + 3);
  } else if (dtype == VDVC_F64) {
    k_zncc<double, 1><<<nb, 256, 0, s>>>((const double*)f, (const double*)g, mask, n, nullptr, red, sums);
    k_zncc<double, 2><<<nb, 256, 0, s>>>((const double*)f, (const double*)g, mask, n, sums, red, sums + 3);
  } else {
    return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
  }
  count_launch(2);
  double h[6];
  VDVC_CUDA(cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaStreamSynchronize(s));
  if (h[0] < 1.0) {
    *out_host = std::numeric_limits<double>::quiet_NaN();  // empty mask: the reference's mean of nothing
    return VDVC_OK;
  }
  const double denom = sqrt(h[4] * h[5]);
  *out_host = denom > 0.0 ? h[3] / denom : std::numeric_limits<double>::quiet_NaN();
  return VDVC_OK;
}

}  // extern "C"
