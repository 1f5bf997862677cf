// Affine pre-alignment kernels (engine/correlate_gpu.py:417-825):
//   * warp + ZNCC sums of affine_prealign's cost (order-1 sampling of g at
//     A (x - c) + c + t, in-bounds voxels only),
//   * separable Gaussian smoothing with scipy.ndimage.gaussian_filter's
//     kernel (truncate 4) in modes 'nearest' and 'constant',
//   * the normalised-convolution division of _smooth_masked,
//   * the 12-parameter Gauss-Newton normal equations of affine_refine_gn and
//     its masked RMS.
// Images are vox layout (x fastest), float32.
//
// Normal equations.  With s(x) = x - M (x - c) - t_r, X~ = (x - c, 1) and
// gs = grad(f_s)(s), the Jacobian rows are J_(i,j) = -m gs_i X~_j, so
//   H_(i,j),(k,l) = sum m gs_i gs_k X~_j X~_l,   b_(i,j) = -sum m e gs_i X~_j.
// Along one x row X~_1, X~_2 and X~_3 = 1 are constant, so each row only
// needs the moments sum m gs_i gs_k X^p (p <= 2, 6 pairs) and
// sum m e gs_i X^p (p <= 1): 24 float sums per row, reduced over the warp
// that owns the row and expanded into the 90 distinct entries of (H, b) in
// float64 with the row's constants.
#include "ops.cuh"

namespace vdvc {

// ---- ZNCC cost ---------------------------------------------------------------

struct Affine9 {
  double A[9], t[3], c[3];
};

__device__ __forceinline__ float sample_lin(const float* __restrict__ g, int nx, int ny, int nz, double cx, double cy,
                                            double cz) {
  // order-1 interpolation at an in-bounds coordinate (float64 weights)
  const double fx = floor(cx), fy = floor(cy), fz = floor(cz);
  const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
  const int ix1 = min(ix + 1, nx - 1), iy1 = min(iy + 1, ny - 1), iz1 = min(iz + 1, nz - 1);
  const double tx = cx - fx, ty = cy - fy, tz = cz - fz;
  const long long sy = nx, sz = (long long)nx * ny;
  auto at = [&](int x, int y, int z) { return (double)g[(long long)x + y * sy + z * sz]; };
  const double a00 = at(ix, iy, iz) * (1 - tx) + at(ix1, iy, iz) * tx;
  const double a10 = at(ix, iy1, iz) * (1 - tx) + at(ix1, iy1, iz) * tx;
  const double a01 = at(ix, iy, iz1) * (1 - tx) + at(ix1, iy, iz1) * tx;
  const double a11 = at(ix, iy1, iz1) * (1 - tx) + at(ix1, iy1, iz1) * tx;
  const double b0 = a00 * (1 - ty) + a10 * ty, b1 = a01 * (1 - ty) + a11 * ty;
  return (float)(b0 * (1 - tz) + b1 * tz);
}

__global__ void __launch_bounds__(256) k_zncc_sums(const float* __restrict__ f, int nx, int ny, int nz,
                                                   const float* __restrict__ g, int gnx, int gny, int gnz, Affine9 P,
                                                   GridReduce red, double* __restrict__ out6) {
  __shared__ double s_red[8];
  double acc[6] = {0, 0, 0, 0, 0, 0};  // n, sum f, sum g, sum f^2, sum g^2, sum fg
  const long long n = (long long)nx * ny * nz;
  const double gxm = gnx - 1, gym = gny - 1, gzm = gnz - 1;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(v % nx);
    const long long r = v / nx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    const double X0 = x - P.c[0], X1 = y - P.c[1], X2 = z - P.c[2];
    const double px = P.A[0] * X0 + P.A[1] * X1 + P.A[2] * X2 + P.c[0] + P.t[0];
    const double py = P.A[3] * X0 + P.A[4] * X1 + P.A[5] * X2 + P.c[1] + P.t[1];
    const double pz = P.A[6] * X0 + P.A[7] * X1 + P.A[8] * X2 + P.c[2] + P.t[2];
    if (!(px >= 0 && px <= gxm && py >= 0 && py <= gym && pz >= 0 && pz <= gzm)) continue;
    const double fv = (double)f[v];
    const double gv = (double)sample_lin(g, gnx, gny, gnz, px, py, pz);
    acc[0] += 1.0;
    acc[1] += fv;
    acc[2] += gv;
    acc[3] += fv * fv;
    acc[4] += gv * gv;
    acc[5] += fv * gv;
  }
  double b6[6], o6[6];
  for (int q = 0; q < 6; ++q) b6[q] = block_sum(acc[q], s_red);
  if (grid_reduce_sum<6>(red, b6, o6, s_red) && threadIdx.x == 0)
    for (int q = 0; q < 6; ++q) out6[q] = o6[q];
}

// ---- Gaussian filter ------------------------------------------------------

struct GaussTaps {
  float w[129];
  int R;
};

// One axis of the separable filter.  mode 0: 'nearest' (clamp), mode 1:
// 'constant' (values beyond the edge are cval).  With `mul` the input is
// first multiplied elementwise by it (the numerator of _smooth_masked).
__global__ void k_gauss_axis(const float* __restrict__ in, float* __restrict__ out, int nx, int ny, int nz, int axis,
                             GaussTaps tp, int mode, float cval, const float* __restrict__ mul) {
  const long long n = (long long)nx * ny * nz;
  const long long stride = axis == 0 ? 1 : (axis == 1 ? (long long)nx : (long long)nx * ny);
  const int len = axis == 0 ? nx : (axis == 1 ? ny : nz);
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(v % nx);
    const long long r = v / nx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    const int c = axis == 0 ? x : (axis == 1 ? y : z);
    const long long base = v - (long long)c * stride;
    float s = 0.f;
    for (int k = -tp.R; k <= tp.R; ++k) {
      int q = c + k;
      float val;
      if ((q < 0 || q >= len) && mode == 1) {
        val = cval;
      } else {
        q = q < 0 ? 0 : (q >= len ? len - 1 : q);
        val = in[base + (long long)q * stride];
        if (mul) val *= mul[base + (long long)q * stride];
      }
      s += tp.w[k + tp.R] * val;
    }
    out[v] = s;
  }
}

__global__ void k_valid_f32(const float* __restrict__ g, long long n, float cval, float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (g[i] != cval) ? 1.f : 0.f;
}

__global__ void k_norm_div(const float* __restrict__ num, const float* __restrict__ den, const float* __restrict__ img,
                           long long n, float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = den[i] > 1e-6f ? num[i] / den[i] : img[i];
}

// ---- normal equations -----------------------------------------------------------

struct AffineGN {
  float M[9], tr[3], c[3];
  float cval;
  int nx, ny, nz;
};

// s(x) = x - M (x - c) - t_r in float32, as the reference forms it
// (engine/correlate_gpu.py:705-722)
__device__ __forceinline__ void gn_coords(const AffineGN& P, int x, int y, int z, float X[3], float s[3]) {
  X[0] = (float)x - P.c[0];
  X[1] = (float)y - P.c[1];
  X[2] = (float)z - P.c[2];
  const float base[3] = {(float)x, (float)y, (float)z};
#pragma unroll
  for (int i = 0; i < 3; ++i) s[i] = base[i] - (P.M[3 * i + 0] * X[0] + P.M[3 * i + 1] * X[1] + P.M[3 * i + 2] * X[2]) - P.tr[i];
}

__device__ __forceinline__ float lin3(const float* __restrict__ a, int stride, int comp, int nx, int ny, int nz,
                                      const float s[3]) {
  const float fx = floorf(s[0]), fy = floorf(s[1]), fz = floorf(s[2]);
  const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
  const int ix1 = min(ix + 1, nx - 1), iy1 = min(iy + 1, ny - 1), iz1 = min(iz + 1, nz - 1);
  const double tx = s[0] - fx, ty = s[1] - fy, tz = s[2] - fz;
  const long long sy = nx, sz = (long long)nx * ny;
  auto at = [&](int x, int y, int z) { return (double)a[((long long)x + y * sy + z * sz) * stride + comp]; };
  const double a00 = at(ix, iy, iz) * (1 - tx) + at(ix1, iy, iz) * tx;
  const double a10 = at(ix, iy1, iz) * (1 - tx) + at(ix1, iy1, iz) * tx;
  const double a01 = at(ix, iy, iz1) * (1 - tx) + at(ix1, iy, iz1) * tx;
  const double a11 = at(ix, iy1, iz1) * (1 - tx) + at(ix1, iy1, iz1) * tx;
  const double b0 = a00 * (1 - ty) + a10 * ty, b1 = a01 * (1 - ty) + a11 * ty;
  return (float)(b0 * (1 - tz) + b1 * tz);
}

// Entry q of the 90 distinct (H upper triangle in 12x12 parameter order
// M00..M22, t0..t2, then b) from the row moments.
// mu[pair][p]: pair (i<=k) index over (00,01,02,11,12,22), p = 0..2
// nu[i][p]: p = 0..1
__device__ __forceinline__ int pair_index(int i, int k) {
  if (i > k) { const int t = i; i = k; k = t; }
  return i == 0 ? k : (i == 1 ? 2 + k : 5);
}

// Parameter index P: 0..8 -> M_(i,j) with i = P/3, j = P%3; 9..11 -> t_i
// (j = 3, X~_3 = 1).
__device__ double expand_entry(int q, const float* mu, const float* nu, double Y, double Z) {
  if (q < 78) {
    // upper triangle (r <= c) enumeration
    int r = 0, c = 0, idx = q;
    for (r = 0; r < 12; ++r) {
      const int len = 12 - r;
      if (idx < len) { c = r + idx; break; }
      idx -= len;
    }
    const int i = r < 9 ? r / 3 : r - 9, j = r < 9 ? r % 3 : 3;
    const int k = c < 9 ? c / 3 : c - 9, l = c < 9 ? c % 3 : 3;
    const float* m = mu + 3 * pair_index(i, k);
    // X~_j X~_l with X~_0 = X (the row variable), X~_1 = Y, X~_2 = Z, X~_3 = 1
    int p = 0;
    double coef = 1.0;
    const int jl[2] = {j, l};
    for (int s = 0; s < 2; ++s) {
      if (jl[s] == 0) ++p;
      else if (jl[s] == 1) coef *= Y;
      else if (jl[s] == 2) coef *= Z;
    }
    return coef * (double)m[p];
  }
  const int P = q - 78;
  const int i = P < 9 ? P / 3 : P - 9, j = P < 9 ? P % 3 : 3;
  const float* n = nu + 2 * i;
  if (j == 0) return -(double)n[1];
  if (j == 1) return -Y * (double)n[0];
  if (j == 2) return -Z * (double)n[0];
  return -(double)n[0];
}

// One warp per (y, z) row; lanes stride over x.
__global__ void __launch_bounds__(256) k_affine_normal(const float* __restrict__ fs, const float* __restrict__ gradfs,
                                                       const float* __restrict__ gs_img,
                                                       const float* __restrict__ g_raw, AffineGN P, GridReduce red,
                                                       double* __restrict__ out90) {
  __shared__ double s_part[8][90];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int nx = P.nx, ny = P.ny, nz = P.nz;
  const float xm = nx - 1, ym = ny - 1, zm = nz - 1;
  const long long nrows = (long long)ny * nz;
  double accq[3] = {0.0, 0.0, 0.0};  // entries lane, lane+32, lane+64
  for (long long row = (long long)blockIdx.x * nwarp + warp; row < nrows; row += (long long)gridDim.x * nwarp) {
    const int y = (int)(row % ny), z = (int)(row / ny);
    float mu[18], nu[6];
#pragma unroll
    for (int q = 0; q < 18; ++q) mu[q] = 0.f;
#pragma unroll
    for (int q = 0; q < 6; ++q) nu[q] = 0.f;
    for (int x = lane; x < nx; x += 32) {
      float X[3], s[3];
      gn_coords(P, x, y, z, X, s);
      const bool inb = s[0] >= 0.f && s[0] <= xm && s[1] >= 0.f && s[1] <= ym && s[2] >= 0.f && s[2] <= zm;
      const long long v = (long long)x + (long long)y * nx + (long long)z * nx * ny;
      if (!inb || g_raw[v] == P.cval) continue;
      const float warped = lin3(fs, 1, 0, nx, ny, nz, s);
      const float e = gs_img[v] - warped;
      const float g0 = lin3(gradfs, 3, 0, nx, ny, nz, s);
      const float g1 = lin3(gradfs, 3, 1, nx, ny, nz, s);
      const float g2 = lin3(gradfs, 3, 2, nx, ny, nz, s);
      const float gsv[3] = {g0, g1, g2};
      const float Xx = X[0], Xx2 = X[0] * X[0];
      int pi = 0;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = i; k < 3; ++k) {
          const float gg = gsv[i] * gsv[k];
          mu[3 * pi + 0] += gg;
          mu[3 * pi + 1] += gg * Xx;
          mu[3 * pi + 2] += gg * Xx2;
          ++pi;
        }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float eg = e * gsv[i];
        nu[2 * i + 0] += eg;
        nu[2 * i + 1] += eg * Xx;
      }
    }
#pragma unroll
    for (int q = 0; q < 18; ++q)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) mu[q] += __shfl_xor_sync(0xffffffffu, mu[q], o);
#pragma unroll
    for (int q = 0; q < 6; ++q)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) nu[q] += __shfl_xor_sync(0xffffffffu, nu[q], o);
    const double Y = (double)((float)y - P.c[1]), Z = (double)((float)z - P.c[2]);
#pragma unroll
    for (int s3 = 0; s3 < 3; ++s3) {
      const int q = lane + 32 * s3;
      if (q < 90) accq[s3] += expand_entry(q, mu, nu, Y, Z);
    }
  }
#pragma unroll
  for (int s3 = 0; s3 < 3; ++s3) {
    const int q = lane + 32 * s3;
    if (q < 90) s_part[warp][q] = accq[s3];
  }
  __syncthreads();
  // block partial in fixed warp order, then the deterministic grid reduction
  __shared__ bool s_last;
  if (threadIdx.x < 90) {
    double t = 0.0;
    for (int w = 0; w < nwarp; ++w) t += s_part[w][threadIdx.x];
    red.partials[(size_t)blockIdx.x * 90 + threadIdx.x] = t;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(red.ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (threadIdx.x < 90) {
    double t = 0.0;
#pragma unroll 8  // unrolled; the summation order is unchanged
    for (unsigned int b = 0; b < gridDim.x; ++b) t += __ldcg(red.partials + (size_t)b * 90 + threadIdx.x);
    out90[threadIdx.x] = t;
  }
  if (threadIdx.x == 0) *red.ticket = 0u;
}

// masked RMS sums of e = g - f(s(x)), mode 'constant' sampling
__global__ void __launch_bounds__(256) k_affine_rms(const float* __restrict__ f, const float* __restrict__ g,
                                                    AffineGN P, GridReduce red, double* __restrict__ out2) {
  __shared__ double s_red[8];
  double se = 0.0, cnt = 0.0;
  const long long n = (long long)P.nx * P.ny * P.nz;
  const float xm = P.nx - 1, ym = P.ny - 1, zm = P.nz - 1;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(v % P.nx);
    const long long r = v / P.nx;
    const int y = (int)(r % P.ny), z = (int)(r / P.ny);
    float X[3], s[3];
    gn_coords(P, x, y, z, X, s);
    const bool inb = s[0] >= 0.f && s[0] <= xm && s[1] >= 0.f && s[1] <= ym && s[2] >= 0.f && s[2] <= zm;
    if (!inb || g[v] == P.cval) continue;
    const float e = g[v] - lin3(f, 1, 0, P.nx, P.ny, P.nz, s);
    se += (double)e * (double)e;
    cnt += 1.0;
  }
  double m2[2] = {block_sum(se, s_red), block_sum(cnt, s_red)}, o2[2];
  if (grid_reduce_sum<2>(red, m2, o2, s_red) && threadIdx.x == 0) {
    out2[0] = o2[0];
    out2[1] = o2[1];
  }
}

struct AffineWs {
  double* partials;
  unsigned int* ticket;
  double* out;
};

static int carve_affine(void* ws, size_t bytes, AffineWs* a) {
  Carve cv(ws, bytes);
  a->partials = cv.take<double>((size_t)kReduceBlocks * 90);
  a->ticket = cv.take<unsigned int>(1);
  a->out = cv.take<double>(96);
  if (!ws || !cv.fits()) return set_error(VDVC_ERR_WORKSPACE, "affine kernels need %zu bytes of workspace", cv.off);
  return VDVC_OK;
}

static AffineGN make_gn(const double* M, const double* tr, const double* c, double cval, int nx, int ny, int nz) {
  AffineGN P;
  for (int i = 0; i < 9; ++i) P.M[i] = (float)M[i];
  for (int i = 0; i < 3; ++i) {
    P.tr[i] = (float)tr[i];
    P.c[i] = (float)c[i];
  }
  P.cval = (float)cval;
  P.nx = nx;
  P.ny = ny;
  P.nz = nz;
  return P;
}

}  // namespace vdvc

using namespace vdvc;

extern "C" {

size_t vdvc_affine_workspace_bytes(void) {
  Carve cv(nullptr, 0);
  cv.take<double>((size_t)kReduceBlocks * 90);
  cv.take<unsigned int>(1);
  cv.take<double>(96);
  return cv.off + 256;
}

int vdvc_affine_zncc_sums(const float* f_vox, int nx, int ny, int nz, const float* g_vox, int gnx, int gny, int gnz,
                          const double* A9, const double* t3, const double* c3, double* out6_host, void* ws,
                          size_t ws_bytes, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f_vox && g_vox && A9 && t3 && c3 && out6_host, "null pointer");
  VDVC_CHECK_ARG(nx >= 1 && ny >= 1 && nz >= 1 && gnx >= 1 && gny >= 1 && gnz >= 1, "bad shapes");
  AffineWs a;
  int st = carve_affine(ws, ws_bytes, &a);
  if (st) return st;
  Affine9 P;
  for (int i = 0; i < 9; ++i) P.A[i] = A9[i];
  for (int i = 0; i < 3; ++i) {
    P.t[i] = t3[i];
    P.c[i] = c3[i];
  }
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(a.ticket, 0, sizeof(unsigned int), s));
  const long long n = (long long)nx * ny * nz;
  k_zncc_sums<<<grid_blocks(n, 256, kReduceBlocks), 256, 0, s>>>(f_vox, nx, ny, nz, g_vox, gnx, gny, gnz, P,
                                                                 GridReduce{a.partials, a.ticket}, a.out);
  VDVC_LAUNCHED();
  VDVC_CUDA(cudaMemcpyAsync(out6_host, a.out, 6 * sizeof(double), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaStreamSynchronize(s));
  return VDVC_OK;
}

int vdvc_gaussian_filter(const float* in, float* out, int nx, int ny, int nz, double sigma, int mode, double cval,
                         const float* mul, float* tmp, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(in && out && tmp && in != tmp && out != tmp, "bad pointers");
  VDVC_CHECK_ARG(sigma > 0.0 && mode >= 0 && mode <= 1, "sigma must be > 0 and mode 0 or 1");
  GaussTaps tp;
  tp.R = (int)(4.0 * sigma + 0.5);  // scipy's truncate = 4.0
  VDVC_CHECK_ARG(tp.R <= 64, "sigma too large (radius %d > 64)", tp.R);
  double sum = 0.0;
  double w[129];
  for (int k = -tp.R; k <= tp.R; ++k) sum += (w[k + tp.R] = exp(-0.5 / (sigma * sigma) * (double)k * k));
  for (int k = 0; k <= 2 * tp.R; ++k) tp.w[k] = (float)(w[k] / sum);
  cudaStream_t s = (cudaStream_t)stream;
  const long long n = (long long)nx * ny * nz;
  const int nb = grid_blocks(n, 256, 152 * 32);
  k_gauss_axis<<<nb, 256, 0, s>>>(in, out, nx, ny, nz, 0, tp, mode, (float)cval, mul);
  k_gauss_axis<<<nb, 256, 0, s>>>(out, tmp, nx, ny, nz, 1, tp, mode, (float)cval, nullptr);
  k_gauss_axis<<<nb, 256, 0, s>>>(tmp, out, nx, ny, nz, 2, tp, mode, (float)cval, nullptr);
  count_launch(3);
  VDVC_CUDA(cudaGetLastError());
  return VDVC_OK;
}

int vdvc_smooth_masked(const float* img, int nx, int ny, int nz, double sigma, double cval, float* out, float* tmp1,
                       float* tmp2, float* tmp3, vdvc_stream_t stream) {
  // num = G(img * valid), den = G(valid), mode 'constant' with 0 beyond the
  // edges; out = num / den where den > 1e-6, else img (_smooth_masked,
  // engine/correlate_gpu.py:585-597)
  VDVC_CHECK_ARG(img && out && tmp1 && tmp2 && tmp3, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  const long long n = (long long)nx * ny * nz;
  k_valid_f32<<<grid_blocks(n, 256, 152 * 32), 256, 0, s>>>(img, n, (float)cval, tmp2);  // valid = img != cval
  VDVC_LAUNCHED();
  int st = vdvc_gaussian_filter(img, tmp1, nx, ny, nz, sigma, 1, 0.0, tmp2, tmp3, stream);  // G(img * valid)
  if (st) return st;
  st = vdvc_gaussian_filter(tmp2, out, nx, ny, nz, sigma, 1, 0.0, nullptr, tmp3, stream);  // G(valid)
  if (st) return st;
  k_norm_div<<<grid_blocks(n, 256, 152 * 32), 256, 0, s>>>(tmp1, out, img, n, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_affine_normal_equations(const float* f_s, const float* grad_fs, const float* g_s, const float* g_raw, int nx,
                                 int ny, int nz, const double* M9, const double* tr3, const double* c3, double cval,
                                 double* H144_host, double* b12_host, void* ws, size_t ws_bytes,
                                 vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f_s && grad_fs && g_s && g_raw && M9 && tr3 && c3 && H144_host && b12_host, "null pointer");
  AffineWs a;
  int st = carve_affine(ws, ws_bytes, &a);
  if (st) return st;
  const AffineGN P = make_gn(M9, tr3, c3, cval, nx, ny, nz);
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(a.ticket, 0, sizeof(unsigned int), s));
  const long long rows = (long long)ny * nz;
  k_affine_normal<<<grid_blocks(rows, 8, kReduceBlocks), 256, 0, s>>>(f_s, grad_fs, g_s, g_raw, P,
                                                                     GridReduce{a.partials, a.ticket}, a.out);
  VDVC_LAUNCHED();
  double h90[90];
  VDVC_CUDA(cudaMemcpyAsync(h90, a.out, 90 * sizeof(double), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaStreamSynchronize(s));
  int q = 0;
  for (int r = 0; r < 12; ++r)
    for (int c = r; c < 12; ++c, ++q) H144_host[r * 12 + c] = H144_host[c * 12 + r] = h90[q];
  for (int i = 0; i < 12; ++i) b12_host[i] = h90[78 + i];
  return VDVC_OK;
}

int vdvc_affine_rms_sums(const float* f, const float* g, int nx, int ny, int nz, const double* M9, const double* tr3,
                         const double* c3, double cval, double* out2_host, void* ws, size_t ws_bytes,
                         vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f && g && M9 && tr3 && c3 && out2_host, "null pointer");
  AffineWs a;
  int st = carve_affine(ws, ws_bytes, &a);
  if (st) return st;
  const AffineGN P = make_gn(M9, tr3, c3, cval, nx, ny, nz);
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(a.ticket, 0, sizeof(unsigned int), s));
  const long long n = (long long)nx * ny * nz;
  k_affine_rms<<<grid_blocks(n, 256, kReduceBlocks), 256, 0, s>>>(f, g, P, GridReduce{a.partials, a.ticket}, a.out);
  VDVC_LAUNCHED();
  VDVC_CUDA(cudaMemcpyAsync(out2_host, a.out, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaStreamSynchronize(s));
  return VDVC_OK;
}

}  // extern "C"
