// Seeded synthetic workloads on the GPU (include/vdvc_synth.h): textures of
// blurred white noise plus bright cylinders, and analytically warped
// deformed images with additive Gaussian noise.
#include "ops.cuh"
#include "vdvc_synth.h"

namespace vdvc {

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// standard normal sample number i of stream `seed` (Box-Muller on a hash)
__device__ __forceinline__ float hash_normal(unsigned long long seed, unsigned long long i) {
  const unsigned long long r = splitmix64(seed * 0xD1B54A32D192ED03ull + i);
  const float u1 = ((float)(r >> 40) + 0.5f) * (1.0f / 16777216.0f);
  const float u2 = ((float)((r >> 16) & 0xFFFFFFull) + 0.5f) * (1.0f / 16777216.0f);
  return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

__global__ void k_noise(float* __restrict__ out, long long n, unsigned long long seed) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = hash_normal(seed, (unsigned long long)i);
}

struct Taps {
  float w[49];
  int R;
};

__global__ void k_blur(const float* __restrict__ in, float* __restrict__ out, int nx, int ny, int nz, int axis,
                       Taps tp) {
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
      q = q < 0 ? 0 : (q >= len ? len - 1 : q);
      s += tp.w[k + tp.R] * in[base + (long long)q * stride];
    }
    out[v] = s;
  }
}

__global__ void k_affine_map(float* __restrict__ a, long long n, float scale, float shift) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = shift + scale * a[i];
}

// One block per cylinder: soft-edged cylinder value written with max().
__global__ void k_cylinders(float* __restrict__ out, int nx, int ny, int nz, const float* __restrict__ cyl,
                            float value) {
  const float* c = cyl + 8 * (size_t)blockIdx.x;
  const float cx = c[0], cy = c[1], cz = c[2], dx = c[3], dy = c[4], dz = c[5], rad = c[6], hl = c[7];
  const float ex = hl * fabsf(dx) + rad + 1.f, ey = hl * fabsf(dy) + rad + 1.f, ez = hl * fabsf(dz) + rad + 1.f;
  const int x0 = max(0, (int)floorf(cx - ex)), x1 = min(nx - 1, (int)ceilf(cx + ex));
  const int y0 = max(0, (int)floorf(cy - ey)), y1 = min(ny - 1, (int)ceilf(cy + ey));
  const int z0 = max(0, (int)floorf(cz - ez)), z1 = min(nz - 1, (int)ceilf(cz + ez));
  if (x1 < x0 || y1 < y0 || z1 < z0) return;
  const int bx = x1 - x0 + 1, by = y1 - y0 + 1, bz = z1 - z0 + 1;
  const long long nb = (long long)bx * by * bz;
  for (long long t = threadIdx.x; t < nb; t += blockDim.x) {
    const int x = x0 + (int)(t % bx);
    const long long r = t / bx;
    const int y = y0 + (int)(r % by), z = z0 + (int)(r / by);
    const float px = x - cx, py = y - cy, pz = z - cz;
    const float ax = px * dx + py * dy + pz * dz;
    const float rho = sqrtf(fmaxf(px * px + py * py + pz * pz - ax * ax, 0.f));
    const float wr = fminf(fmaxf(rad + 0.5f - rho, 0.f), 1.f);
    const float wa = fminf(fmaxf(hl + 0.5f - fabsf(ax), 0.f), 1.f);
    const float val = value * wr * wa;
    if (val > 0.f) {
      const long long v = (long long)x + (long long)y * nx + (long long)z * nx * ny;
      atomicMax((int*)&out[v], __float_as_int(val));  // val > 0: int order == float order
    }
  }
}

__global__ void __launch_bounds__(256) k_minmax(const float* __restrict__ a, long long n, float* __restrict__ part) {
  __shared__ float smn[256], smx[256];
  float mn = 3.0e38f, mx = -3.0e38f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    mn = fminf(mn, a[i]);
    mx = fmaxf(mx, a[i]);
  }
  smn[threadIdx.x] = mn;
  smx[threadIdx.x] = mx;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      smn[threadIdx.x] = fminf(smn[threadIdx.x], smn[threadIdx.x + o]);
      smx[threadIdx.x] = fmaxf(smx[threadIdx.x], smx[threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = smn[0];
    part[2 * blockIdx.x + 1] = smx[0];
  }
}

__global__ void k_normalize(float* __restrict__ a, long long n, const float* __restrict__ part, int nparts) {
  __shared__ float s_mn, s_mx;
  if (threadIdx.x == 0) {
    float mn = part[0], mx = part[1];
    for (int b = 1; b < nparts; ++b) {
      mn = fminf(mn, part[2 * b]);
      mx = fmaxf(mx, part[2 * b + 1]);
    }
    s_mn = mn;
    s_mx = mx;
  }
  __syncthreads();
  const float mn = s_mn, inv = 1.0f / fmaxf(s_mx - s_mn, 1e-30f);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = (a[i] - mn) * inv;
}

constexpr int kMaxFieldParams = 64;

struct FieldParams {
  int kind;
  double p[kMaxFieldParams];
};

__device__ __forceinline__ void field_u(const FieldParams& fp, double x, double y, double z, double u[3]) {
  const double* p = fp.p;
  if (fp.kind == VDVC_FIELD_NECKING) {
    const double ez = p[0], a = p[1], zc = p[2], s = p[3], xc = p[4], yc = p[5], R = p[6];
    const double g = a * exp(-(z - zc) * (z - zc) / (2.0 * s * s)) / R;
    u[0] = -g * (x - xc);
    u[1] = -g * (y - yc);
    u[2] = ez * z;
    return;
  }
  // affine (+ sinusoid)
  const double X[3] = {x - p[12], y - p[13], z - p[14]};
  for (int k = 0; k < 3; ++k) u[k] = p[k] + p[3 + 3 * k] * X[0] + p[4 + 3 * k] * X[1] + p[5 + 3 * k] * X[2];
  if (fp.kind == VDVC_FIELD_AFFINE_SIN) {
    const double amp = p[15], wl = p[16];
    const double xs[3] = {x, y, z};
    for (int k = 0; k < 3; ++k) u[k] += amp * sin(2.0 * 3.14159265358979323846 * xs[(k + 1) % 3] / wl);
  }
  if (fp.kind == VDVC_FIELD_BUMPS) {
    const int nb = (int)p[15];
    for (int b = 0; b < nb; ++b) {
      const double* q = p + 16 + 7 * b;  // centre[3], width, amplitude[3]
      const double dx = x - q[0], dy = y - q[1], dz = z - q[2];
      const double e = exp(-(dx * dx + dy * dy + dz * dz) / (2.0 * q[3] * q[3]));
      u[0] += q[4] * e;
      u[1] += q[5] * e;
      u[2] += q[6] * e;
    }
  }
}

// u at the grid points (i, j, k) * stride, FP32 [point][3]
__global__ void k_field_grid(FieldParams fp, int gx, int gy, int gz, double stride, float* __restrict__ out) {
  const long long n = (long long)gx * gy * gz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % gx);
    const long long r = i / gx;
    const int y = (int)(r % gy), z = (int)(r / gy);
    double u[3];
    field_u(fp, x * stride, y * stride, z * stride, u);
    out[3 * i] = (float)u[0];
    out[3 * i + 1] = (float)u[1];
    out[3 * i + 2] = (float)u[2];
  }
}

// Trilinear sample of f at (cx, cy, cz), coordinates clamped to the volume.
__device__ __forceinline__ float sample_clamped(const float* __restrict__ f, int nx, int ny, int nz, float cx,
                                                float cy, float cz) {
  const float c[3] = {cx, cy, cz};
  const int dims[3] = {nx, ny, nz};
  int i0[3], i1[3];
  float t[3];
  for (int k = 0; k < 3; ++k) {
    const float cc = fminf(fmaxf(c[k], 0.f), (float)(dims[k] - 1));
    const float fl = floorf(cc);
    i0[k] = (int)fl;
    i1[k] = min(i0[k] + 1, dims[k] - 1);
    t[k] = cc - fl;
  }
  auto at = [&](int xx, int yy, int zz) { return f[(long long)xx + (long long)yy * nx + (long long)zz * nx * ny]; };
  const float a00 = at(i0[0], i0[1], i0[2]) + t[0] * (at(i1[0], i0[1], i0[2]) - at(i0[0], i0[1], i0[2]));
  const float a10 = at(i0[0], i1[1], i0[2]) + t[0] * (at(i1[0], i1[1], i0[2]) - at(i0[0], i1[1], i0[2]));
  const float a01 = at(i0[0], i0[1], i1[2]) + t[0] * (at(i1[0], i0[1], i1[2]) - at(i0[0], i0[1], i1[2]));
  const float a11 = at(i0[0], i1[1], i1[2]) + t[0] * (at(i1[0], i1[1], i1[2]) - at(i0[0], i1[1], i1[2]));
  const float b0 = a00 + t[1] * (a10 - a00), b1 = a01 + t[1] * (a11 - a01);
  return b0 + t[2] * (b1 - b0);
}

__global__ void k_warp(const float* __restrict__ f, int nx, int ny, int nz, FieldParams fp, float sigma,
                       unsigned long long seed, float* __restrict__ g) {
  const long long n = (long long)nx * ny * nz;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(v % nx);
    const long long r = v / nx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    double u[3];
    field_u(fp, x, y, z, u);
    float val = sample_clamped(f, nx, ny, nz, (float)(x - u[0]), (float)(y - u[1]), (float)(z - u[2]));
    if (sigma > 0.f) val += sigma * hash_normal(seed, (unsigned long long)v);
    g[v] = val;
  }
}

// ---- free-form deformation: affine + cubic B-spline ---------------------------

struct Ffd {
  float G[9], t[3], c[3];  // affine part u = t + G (x - c)
  const float* ctrl;       // [nc^3][3], first index fastest
  int nc;
  float inv_d[3];          // 1 / control spacing per axis
};

__device__ __forceinline__ void bspline3(float t, float (&b)[4]) {
  const float t2 = t * t, t3 = t2 * t, s = 1.f - t;
  b[0] = s * s * s * (1.f / 6.f);
  b[1] = (3.f * t3 - 6.f * t2 + 4.f) * (1.f / 6.f);
  b[2] = (-3.f * t3 + 3.f * t2 + 3.f * t + 1.f) * (1.f / 6.f);
  b[3] = t3 * (1.f / 6.f);
}

// u(x): the affine part plus the sum over the 4^3 control points of the cell
// around x of B(tx) B(ty) B(tz) ctrl; the cell index is clamped to
// [0, nc - 4], so a point outside the volume sees the border cells'
// polynomial.
__device__ __forceinline__ void ffd_u(const Ffd& F, float x, float y, float z, float (&u)[3]) {
  const float X[3] = {x - F.c[0], y - F.c[1], z - F.c[2]};
  for (int k = 0; k < 3; ++k) u[k] = F.t[k] + F.G[3 * k] * X[0] + F.G[3 * k + 1] * X[1] + F.G[3 * k + 2] * X[2];
  const float p[3] = {x, y, z};
  int cell[3];
  float b[3][4];
  for (int k = 0; k < 3; ++k) {
    const float sp = p[k] * F.inv_d[k];
    const float fl = fminf(fmaxf(floorf(sp), 0.f), (float)(F.nc - 4));
    cell[k] = (int)fl;
    bspline3(sp - fl, b[k]);
  }
  float acc[3] = {0.f, 0.f, 0.f};
  for (int cz = 0; cz < 4; ++cz)
    for (int cy = 0; cy < 4; ++cy) {
      const float wyz = b[2][cz] * b[1][cy];
      const float* row = F.ctrl + 3 * ((long long)(cell[0]) + (long long)(cell[1] + cy) * F.nc +
                                       (long long)(cell[2] + cz) * F.nc * F.nc);
#pragma unroll
      for (int cx = 0; cx < 4; ++cx) {
        const float w = wyz * b[0][cx];
        acc[0] += w * __ldg(row + 3 * cx);
        acc[1] += w * __ldg(row + 3 * cx + 1);
        acc[2] += w * __ldg(row + 3 * cx + 2);
      }
    }
  for (int k = 0; k < 3; ++k) u[k] += acc[k];
}

__global__ void k_warp_ffd(const float* __restrict__ f, int nx, int ny, int nz, Ffd F, float sigma,
                           unsigned long long seed, float* __restrict__ g) {
  const long long n = (long long)nx * ny * nz;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(v % nx);
    const long long r = v / nx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    float u[3];
    ffd_u(F, (float)x, (float)y, (float)z, u);
    float val = sample_clamped(f, nx, ny, nz, x - u[0], y - u[1], z - u[2]);
    if (sigma > 0.f) val += sigma * hash_normal(seed, (unsigned long long)v);
    g[v] = val;
  }
}

// U = u(X + U) at X = (i, j, k) * stride by `iters` fixed-point steps
__global__ void k_ffd_inverse_grid(Ffd F, int gx, int gy, int gz, float stride, int iters, float* __restrict__ out) {
  const long long n = (long long)gx * gy * gz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % gx);
    const long long r = i / gx;
    const int y = (int)(r % gy), z = (int)(r / gy);
    const float X[3] = {x * stride, y * stride, z * stride};
    float U[3] = {0.f, 0.f, 0.f};
    for (int it = 0; it < iters; ++it) {
      float u[3];
      ffd_u(F, X[0] + U[0], X[1] + U[1], X[2] + U[2], u);
      U[0] = u[0];
      U[1] = u[1];
      U[2] = u[2];
    }
    out[3 * i] = U[0];
    out[3 * i + 1] = U[1];
    out[3 * i + 2] = U[2];
  }
}

inline int gblocks(long long n) { return grid_blocks(n, 256, 152 * 32); }

}  // namespace vdvc

using namespace vdvc;

extern "C" {

size_t vdvc_synth_workspace_bytes(int nx, int ny, int nz) {
  Carve cv(nullptr, 0);
  cv.take<float>((size_t)nx * ny * nz);
  cv.take<float>(2 * kReduceBlocks);
  return cv.off + 256;
}

int vdvc_synth_texture(float* out, int nx, int ny, int nz, unsigned long long seed, double sigma, double noise_amp,
                       const float* cylinders, int n_cyl, double cyl_value, void* ws, size_t ws_bytes,
                       vdvc_stream_t stream) {
  VDVC_CHECK_ARG(out && nx >= 1 && ny >= 1 && nz >= 1, "bad arguments");
  VDVC_CHECK_ARG(sigma > 0.0 && sigma <= 6.0, "sigma must be in (0, 6]");
  VDVC_CHECK_ARG(n_cyl == 0 || cylinders, "cylinders is null");
  const long long n = (long long)nx * ny * nz;
  Carve cv(ws, ws_bytes);
  float* tmp = cv.take<float>(n);
  float* part = cv.take<float>(2 * kReduceBlocks);
  if (!ws || !cv.fits()) return set_error(VDVC_ERR_WORKSPACE, "synth_texture needs %zu bytes", cv.off);
  cudaStream_t s = (cudaStream_t)stream;
  Taps tp{};
  tp.R = (int)ceil(4.0 * sigma);
  double sum = 0.0, sq = 0.0;
  for (int k = -tp.R; k <= tp.R; ++k) sum += exp(-0.5 * k * k / (sigma * sigma));
  for (int k = -tp.R; k <= tp.R; ++k) {
    const double w = exp(-0.5 * k * k / (sigma * sigma)) / sum;
    tp.w[k + tp.R] = (float)w;
    sq += w * w;
  }
  const double std3 = pow(sq, 1.5);  // std of the 3-D blurred unit white noise
  const int nb = gblocks(n);
  k_noise<<<nb, 256, 0, s>>>(out, n, seed);
  k_blur<<<nb, 256, 0, s>>>(out, tmp, nx, ny, nz, 0, tp);
  k_blur<<<nb, 256, 0, s>>>(tmp, out, nx, ny, nz, 1, tp);
  k_blur<<<nb, 256, 0, s>>>(out, tmp, nx, ny, nz, 2, tp);
  k_affine_map<<<nb, 256, 0, s>>>(tmp, n, (float)(noise_amp / std3), 0.5f);
  count_launch(5);
  if (n_cyl > 0) {
    k_cylinders<<<n_cyl, 256, 0, s>>>(tmp, nx, ny, nz, cylinders, (float)cyl_value);
    count_launch();
  }
  const int rb = grid_blocks(n, 256, kReduceBlocks);
  k_minmax<<<rb, 256, 0, s>>>(tmp, n, part);
  k_normalize<<<nb, 256, 0, s>>>(tmp, n, part, rb);
  count_launch(2);
  VDVC_CUDA(cudaMemcpyAsync(out, tmp, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
  VDVC_CUDA(cudaGetLastError());
  return VDVC_OK;
}

static int field_params(int field, const double* params, int n_params, FieldParams* fp) {
  VDVC_CHECK_ARG(field >= VDVC_FIELD_AFFINE && field <= VDVC_FIELD_BUMPS, "unknown field %d", field);
  VDVC_CHECK_ARG(params && n_params >= 0 && n_params <= kMaxFieldParams, "bad params");
  if (field == VDVC_FIELD_BUMPS)
    VDVC_CHECK_ARG(n_params >= 16 && params[15] >= 0 && params[15] <= 6 && n_params >= 16 + 7 * (int)params[15],
                   "bumps field needs 16 + 7 * n_bumps params (n_bumps <= 6)");
  *fp = FieldParams{};
  fp->kind = field;
  for (int i = 0; i < n_params; ++i) fp->p[i] = params[i];
  return VDVC_OK;
}

int vdvc_synth_field_grid(int field, const double* params, int n_params, int gx, int gy, int gz, double stride,
                          float* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(out && gx >= 1 && gy >= 1 && gz >= 1 && stride > 0.0, "bad arguments");
  FieldParams fp;
  int st = field_params(field, params, n_params, &fp);
  if (st) return st;
  k_field_grid<<<gblocks((long long)gx * gy * gz), 256, 0, (cudaStream_t)stream>>>(fp, gx, gy, gz, stride, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_synth_warp(const float* f, int nx, int ny, int nz, int field, const double* params, int n_params,
                    double noise_sigma, unsigned long long seed, float* g, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f && g && f != g && nx >= 1 && ny >= 1 && nz >= 1, "bad arguments");
  FieldParams fp;
  int st = field_params(field, params, n_params, &fp);
  if (st) return st;
  const long long n = (long long)nx * ny * nz;
  k_warp<<<gblocks(n), 256, 0, (cudaStream_t)stream>>>(f, nx, ny, nz, fp, (float)noise_sigma, seed, g);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

static int make_ffd(const double* affine, const float* ctrl, int nc, int nx, int ny, int nz, Ffd* F) {
  VDVC_CHECK_ARG(affine && ctrl && nc >= 4 && nc <= 64, "bad free-form deformation (nc in [4, 64])");
  VDVC_CHECK_ARG(nx >= 2 && ny >= 2 && nz >= 2, "volume too small");
  for (int k = 0; k < 3; ++k) F->t[k] = (float)affine[k];
  for (int k = 0; k < 9; ++k) F->G[k] = (float)affine[3 + k];
  for (int k = 0; k < 3; ++k) F->c[k] = (float)affine[12 + k];
  F->ctrl = ctrl;
  F->nc = nc;
  const int dims[3] = {nx, ny, nz};
  for (int k = 0; k < 3; ++k) F->inv_d[k] = (float)((double)(nc - 3) / (double)(dims[k] - 1));
  return VDVC_OK;
}

int vdvc_synth_warp_ffd(const float* f, int nx, int ny, int nz, const double* affine, const float* ctrl, int nc,
                        double noise_sigma, unsigned long long seed, float* g, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f && g && f != g, "bad arguments");
  Ffd F;
  int st = make_ffd(affine, ctrl, nc, nx, ny, nz, &F);
  if (st) return st;
  const long long n = (long long)nx * ny * nz;
  k_warp_ffd<<<gblocks(n), 256, 0, (cudaStream_t)stream>>>(f, nx, ny, nz, F, (float)noise_sigma, seed, g);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_synth_ffd_inverse_grid(const double* affine, const float* ctrl, int nc, int nx, int ny, int nz, int gx,
                                int gy, int gz, double stride, int iters, float* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(out && gx >= 1 && gy >= 1 && gz >= 1 && stride > 0.0 && iters >= 1 && iters <= 200,
                 "bad arguments");
  Ffd F;
  int st = make_ffd(affine, ctrl, nc, nx, ny, nz, &F);
  if (st) return st;
  k_ffd_inverse_grid<<<gblocks((long long)gx * gy * gz), 256, 0, (cudaStream_t)stream>>>(F, gx, gy, gz,
                                                                                         (float)stride, iters, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

}  // extern "C"
