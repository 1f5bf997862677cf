// Pre-processing kernels of `voxeldvc preprocess` (preprocess.py): the
// affine warp of the deformed volume onto the reference grid, integer
// binning, and the axis projections of the valid-overlap mask that the crop
// search reads.  Volumes are numpy's pix[x, y, z] arrays in C order (z
// fastest), as the reference holds them.
#include "ops.cuh"

namespace vdvc {

struct Affine3 {
  float A[9], c[3], t[3];
};

// warp_onto_ref_grid (preprocess.py:233-285): out[i,j,k] = g sampled at
// A (x - c) + c + t, x = (i, j, k), coordinates formed in float32 as the
// reference forms them; order-1 interpolation, 0 outside [0, n-1]
// (map_coordinates mode 'constant').
__global__ void k_warp_affine(const float* __restrict__ g, int gx, int gy, int gz, Affine3 af, int nx, int ny, int nz,
                              float* __restrict__ out) {
  const long long n = (long long)nx * ny * nz;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(v % nz);
    const long long r = v / nz;
    const int j = (int)(r % ny), i = (int)(r / ny);
    const float d[3] = {(float)i - af.c[0], (float)j - af.c[1], (float)k - af.c[2]};
    float p[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float m = __fadd_rn(__fadd_rn(__fmul_rn(af.A[3 * a], d[0]), __fmul_rn(af.A[3 * a + 1], d[1])),
                                __fmul_rn(af.A[3 * a + 2], d[2]));
      p[a] = __fadd_rn(__fadd_rn(m, af.c[a]), af.t[a]);
    }
    const int dims[3] = {gx, gy, gz};
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) inside = inside && p[a] >= 0.f && p[a] <= (float)(dims[a] - 1);
    if (!inside) {
      out[v] = 0.f;
      continue;
    }
    int i0[3], i1[3];
    double t[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double c = (double)p[a];
      const double fl = floor(c);
      i0[a] = (int)fl;
      i1[a] = min(i0[a] + 1, dims[a] - 1);
      t[a] = c - fl;
    }
    // g is C-order: index ((x * gy) + y) * gz + z
    auto at = [&](int xx, int yy, int zz) { return (double)g[((long long)xx * gy + yy) * gz + zz]; };
    const double a00 = at(i0[0], i0[1], i0[2]) * (1 - t[2]) + at(i0[0], i0[1], i1[2]) * t[2];
    const double a01 = at(i0[0], i1[1], i0[2]) * (1 - t[2]) + at(i0[0], i1[1], i1[2]) * t[2];
    const double a10 = at(i1[0], i0[1], i0[2]) * (1 - t[2]) + at(i1[0], i0[1], i1[2]) * t[2];
    const double a11 = at(i1[0], i1[1], i0[2]) * (1 - t[2]) + at(i1[0], i1[1], i1[2]) * t[2];
    const double b0 = a00 * (1 - t[1]) + a01 * t[1], b1 = a10 * (1 - t[1]) + a11 * t[1];
    out[v] = (float)(b0 * (1 - t[0]) + b1 * t[0]);
  }
}

// bin_volume (preprocess.py:288-312): float32 sums over the B^3 strided
// sub-volumes in the reference's (i, j, k) order, then / B^3.
template <typename S>
__global__ void k_bin(const S* __restrict__ vol, int s0, int s1, int s2, int B, float* __restrict__ out) {
  const int o0 = s0 / B, o1 = s1 / B, o2 = s2 / B;
  const long long n = (long long)o0 * o1 * o2;
  const float inv = (float)(B * B * B);
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(v % o2);
    const long long r = v / o2;
    const int y = (int)(r % o1), x = (int)(r / o1);
    float acc = 0.f;
    for (int i = 0; i < B; ++i)
      for (int j = 0; j < B; ++j)
        for (int k = 0; k < B; ++k)
          acc = __fadd_rn(acc, (float)vol[((long long)(x * B + i) * s1 + (y * B + j)) * s2 + (z * B + k)]);
    out[v] = __fdiv_rn(acc, inv);
  }
}

// any() of (f > glt) & (g > glt) along the other two axes, per axis
__global__ void k_overlap_proj(const float* __restrict__ f, const float* __restrict__ g, int n0, int n1, int n2,
                               float glt, uint8_t* __restrict__ p0, uint8_t* __restrict__ p1,
                               uint8_t* __restrict__ p2) {
  const long long n = (long long)n0 * n1 * n2;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    if (!(f[v] > glt && g[v] > glt)) continue;
    const int k = (int)(v % n2);
    const long long r = v / n2;
    const int j = (int)(r % n1), i = (int)(r / n1);
    p0[i] = 1;  // every writer stores the same value
    p1[j] = 1;
    p2[k] = 1;
  }
}

}  // namespace vdvc

using namespace vdvc;

extern "C" {

int vdvc_warp_affine(const float* g, int gx, int gy, int gz, const double* A, const double* t, const double* c, int nx,
                     int ny, int nz, float* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(g && A && t && c && out && gx >= 1 && gy >= 1 && gz >= 1 && nx >= 1 && ny >= 1 && nz >= 1,
                 "bad arguments");
  Affine3 af;
  for (int q = 0; q < 9; ++q) af.A[q] = (float)A[q];
  for (int q = 0; q < 3; ++q) {
    af.c[q] = (float)c[q];
    af.t[q] = (float)t[q];
  }
  const long long n = (long long)nx * ny * nz;
  k_warp_affine<<<grid_blocks(n, 256, 152 * 32), 256, 0, (cudaStream_t)stream>>>(g, gx, gy, gz, af, nx, ny, nz, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_bin_volume(const void* vol, int dtype, int s0, int s1, int s2, int B, float* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(vol && out && B >= 1 && s0 >= B && s1 >= B && s2 >= B, "bad arguments");
  VDVC_CHECK_ARG(s0 % B == 0 && s1 % B == 0 && s2 % B == 0, "volume shape (%d,%d,%d) not divisible by %d", s0, s1,
                 s2, B);
  const long long n = (long long)(s0 / B) * (s1 / B) * (s2 / B);
  const int nb = grid_blocks(n, 256, 152 * 32);
  cudaStream_t s = (cudaStream_t)stream;
  switch (dtype) {
    case VDVC_F32: k_bin<float><<<nb, 256, 0, s>>>((const float*)vol, s0, s1, s2, B, out); break;
    case VDVC_U8: k_bin<uint8_t><<<nb, 256, 0, s>>>((const uint8_t*)vol, s0, s1, s2, B, out); break;
    case VDVC_U16: k_bin<uint16_t><<<nb, 256, 0, s>>>((const uint16_t*)vol, s0, s1, s2, B, out); break;
    case VDVC_I16: k_bin<int16_t><<<nb, 256, 0, s>>>((const int16_t*)vol, s0, s1, s2, B, out); break;
    default: return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
  }
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_overlap_projections(const float* f, const float* g, int n0, int n1, int n2, double glt, uint8_t* p0,
                             uint8_t* p1, uint8_t* p2, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f && g && p0 && p1 && p2 && n0 >= 1 && n1 >= 1 && n2 >= 1, "bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(p0, 0, n0, s));
  VDVC_CUDA(cudaMemsetAsync(p1, 0, n1, s));
  VDVC_CUDA(cudaMemsetAsync(p2, 0, n2, s));
  const long long n = (long long)n0 * n1 * n2;
  k_overlap_proj<<<grid_blocks(n, 256, 152 * 32), 256, 0, s>>>(f, g, n0, n1, n2, (float)glt, p0, p1, p2);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

}  // extern "C"
