// Kernels of the learned initial guess (include/vdvc_cnn.h): BF16 3x3x3
// convolutions as implicit GEMMs on the tensor cores -- the tcgen05 forms
// live in conv_tc.cu; here the mma.sync m16n8k16 form (FP32 accumulation)
// for the layers those do not take -- their weight gradients, and the small
// elementwise pieces of training and inference.
//
// Convolution = gather GEMM.  Output positions are the GEMM rows (M), output
// channels the columns (N), and (tap, input channel) the reduction (K).  A
// warp owns 16 consecutive output positions and all N channels; its A
// fragments come straight from the channels-last source (the 16 channels of
// one tap are 32 contiguous bytes), its B fragments from the packed weights,
// both through L1 -- the same source positions are read by 27 taps and by
// neighbouring warps.  The input gradient is the same kernel on the
// transposed weights with the adjoint geometry, so one kernel serves both
// directions.  Every load is bounds-checked against the grids; outside the
// source volume the operand is zero (padding).
//
// Weight gradient = GEMM with the positions as reduction: for tap t,
// dW_t[n][k] = sum_p dy[p][n] x[q(p,t)][k].  Blocks split the positions;
// each warp keeps its own FP32 partial, and a second pass sums the partials
// in a fixed order, so the result is deterministic.
#include <cuda_bf16.h>

#include <cstdint>
#include <map>
#include <mutex>

#include "ops.cuh"
#include "vdvc_cnn.h"

namespace vdvc {

typedef __nv_bfloat16 bf16;

int launch_conv_tc(const void* src, int scs, int scoff, int cin, const void* w, int wrows, const float* bias,
                   int n_out, int relu, void* out, int out_f32, int ocs, int ocoff, int accumulate,
                   const vdvc_conv_geom* geom, int* err, cudaStream_t s);
int launch_conv_tma(const void* src, int scs, int scoff, int cin, const void* w, int wrows, const float* bias,
                    int n_out, int relu, void* out, int out_f32, int ocs, int ocoff, int accumulate,
                    const vdvc_conv_geom* geom, int* err, cudaStream_t s);
int launch_conv_first(const void* src, int scs, int scoff, const void* w, int wrows, const float* bias, int n_out,
                      int relu, void* out, int out_f32, int ocs, int ocoff, int accumulate, const vdvc_conv_geom* g,
                      int* err, cudaStream_t s);

struct Geo {
  int nx, ny, nz, sx, sy, sz, a, b, c, d;
};

__device__ __forceinline__ int map_src(int p, int t, const Geo& g, int S) {
  int num = p * g.a + g.b + t * g.c;
  if (num < 0) return -1;
  if (g.d != 1) {
    if (num % g.d) return -1;
    num /= g.d;
  }
  return num < S ? num : -1;
}

// source voxel index of output position (x,y,z) for tap t, or -1
__device__ __forceinline__ long long src_index(int x, int y, int z, int t, const Geo& g) {
  const int tx = t % 3, ty = (t / 3) % 3, tz = t / 9;
  const int qx = map_src(x, tx, g, g.sx), qy = map_src(y, ty, g, g.sy), qz = map_src(z, tz, g, g.sz);
  if (qx < 0 || qy < 0 || qz < 0) return -1;
  return ((long long)qz * g.sy + qy) * g.sx + qx;
}

// Timeout flag of the tensor-core convolutions (conv_tc.cu), one per device
// that loads the library; its address is looked up once per device.
__device__ int g_conv_err;

int conv_error_flag(int** out) {
  static std::mutex mu;
  static std::map<int, int*> addr;
  int dev = 0;
  VDVC_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  auto it = addr.find(dev);
  if (it == addr.end()) {
    void* p = nullptr;
    VDVC_CUDA(cudaGetSymbolAddress(&p, g_conv_err));
    it = addr.emplace(dev, (int*)p).first;
  }
  *out = it->second;
  return VDVC_OK;
}

__device__ __forceinline__ uint32_t ld32(const bf16* p) { return __ldg((const unsigned int*)p); }
__device__ __forceinline__ uint32_t ld16(const bf16* p) { return (uint32_t)__ldg((const unsigned short*)p); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ---- convolution (forward and input gradient) -------------------------------

// Fragment layout of m16n8k16 (PTX ISA): lane = 4*gid + tig.
//   A regs: 0 = (row gid,   k 2tig..+1), 1 = (row gid+8, k 2tig..+1),
//           2 = (row gid,   k 2tig+8..), 3 = (row gid+8, k 2tig+8..)
//   B regs: 0 = (k 2tig..+1, col gid),   1 = (k 2tig+8..,  col gid)
//   C: c0,c1 = (row gid, cols 2tig, 2tig+1), c2,c3 = (row gid+8, same cols)
template <int NF, bool SMALLC>
__global__ void __launch_bounds__(128) k_conv(const bf16* __restrict__ src, int scs, int scoff, int cin,
                                              const bf16* __restrict__ w, const float* __restrict__ bias, int n_out,
                                              int relu, void* __restrict__ out, int out_f32, int ocs, int ocoff,
                                              int accumulate, Geo g) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gid = lane >> 2, tig = lane & 3;
  const long long npos = (long long)g.nx * g.ny * g.nz;
  const long long p0 = ((long long)blockIdx.x * 4 + warp) * 16;
  if (p0 >= npos) return;  // warp-uniform
  long long pr[2];
  int px[2], py[2], pz[2];
  bool pv[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    pr[r] = p0 + gid + 8 * r;
    pv[r] = pr[r] < npos;
    const long long q = pv[r] ? pr[r] : 0;
    px[r] = (int)(q % g.nx);
    const long long rr = q / g.nx;
    py[r] = (int)(rr % g.ny);
    pz[r] = (int)(rr / g.ny);
  }
  float acc[NF][4];
#pragma unroll
  for (int j = 0; j < NF; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;

  if constexpr (SMALLC) {
    // cin == 2: K = (tap, channel) pairs, k = 2t + ci, padded to 64
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      uint32_t a[4];
#pragma unroll
      for (int hk = 0; hk < 2; ++hk) {
        const int t = ks * 8 + hk * 4 + tig;
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          uint32_t val = 0u;
          if (t < 27 && pv[r]) {
            const long long si = src_index(px[r], py[r], pz[r], t, g);
            if (si >= 0) val = ld32(src + si * scs + scoff);
          }
          a[hk * 2 + r] = val;
        }
      }
#pragma unroll
      for (int j = 0; j < NF; ++j) {
        const bf16* wr = w + (size_t)(j * 8 + gid) * 64 + ks * 16 + tig * 2;
        mma_bf16(acc[j], a, ld32(wr), ld32(wr + 8));
      }
    }
  } else {
#pragma unroll 1
    for (int t = 0; t < 27; ++t) {
      long long si[2];
#pragma unroll
      for (int r = 0; r < 2; ++r) si[r] = pv[r] ? src_index(px[r], py[r], pz[r], t, g) : -1;
      const bf16* s0 = src + (si[0] >= 0 ? si[0] : 0) * scs + scoff + tig * 2;
      const bf16* s1 = src + (si[1] >= 0 ? si[1] : 0) * scs + scoff + tig * 2;
      const bf16* wt = w + (size_t)t * cin + tig * 2;
#pragma unroll 1
      for (int kc = 0; kc < cin; kc += 16) {
        uint32_t a[4];
        a[0] = si[0] >= 0 ? ld32(s0 + kc) : 0u;
        a[1] = si[1] >= 0 ? ld32(s1 + kc) : 0u;
        a[2] = si[0] >= 0 ? ld32(s0 + kc + 8) : 0u;
        a[3] = si[1] >= 0 ? ld32(s1 + kc + 8) : 0u;
#pragma unroll
        for (int j = 0; j < NF; ++j) {
          const bf16* wr = wt + (size_t)(j * 8 + gid) * 27 * cin + kc;
          mma_bf16(acc[j], a, ld32(wr), ld32(wr + 8));
        }
      }
    }
  }

#pragma unroll
  for (int j = 0; j < NF; ++j)
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      if (!pv[r]) continue;
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int n = j * 8 + tig * 2 + e;
        if (n >= n_out) continue;
        float v = acc[j][2 * r + e];
        if (bias) v += bias[n];
        if (relu) v = fmaxf(v, 0.f);
        const long long o = pr[r] * ocs + ocoff + n;
        if (out_f32) {
          ((float*)out)[o] = v;
        } else {
          bf16* op = (bf16*)out;
          if (accumulate) v += __bfloat162float(op[o]);
          op[o] = __float2bfloat16_rn(v);
        }
      }
    }
}

// ---- weight gradient --------------------------------------------------------

// grid (27 taps, splits), 4 warps; warp (split, w) writes its partial
// part[(split*4 + w)][n][t][k] for n < n_out, k < cin.
// blockIdx.z selects the block of 32 output channels x 64 input channels
// this block computes (larger layers tile over it).
template <int MF, int NFC>
__global__ void __launch_bounds__(128) k_wgrad(const bf16* __restrict__ dy, int dcs, int dcoff, int n_out,
                                               const bf16* __restrict__ x, int xcs, int xcoff, int cin, Geo g,
                                               long long chunk, float* __restrict__ part) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gid = lane >> 2, tig = lane & 3;
  const int t = blockIdx.x, split = blockIdx.y;
  const int kblocks = (cin + 63) / 64;
  const int n0 = (int)(blockIdx.z / kblocks) * 32, c0 = (int)(blockIdx.z % kblocks) * 64;
  const long long npos = (long long)g.nx * g.ny * g.nz;
  const long long pbeg = (long long)split * chunk;
  const long long pend = min(npos, pbeg + chunk);
  float acc[MF][NFC][4];
#pragma unroll
  for (int mt = 0; mt < MF; ++mt)
#pragma unroll
    for (int j = 0; j < NFC; ++j) acc[mt][j][0] = acc[mt][j][1] = acc[mt][j][2] = acc[mt][j][3] = 0.f;

  for (long long p0 = pbeg + warp * 16; p0 < pend; p0 += 64) {
    // this lane's reduction positions: p0 + 2tig + {0, 1, 8, 9}
    long long kp[4], si[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      kp[q] = p0 + tig * 2 + (q & 1) + (q >> 1) * 8;
      si[q] = -1;
      if (kp[q] < pend) {
        const int xx = (int)(kp[q] % g.nx);
        const long long rr = kp[q] / g.nx;
        si[q] = src_index(xx, (int)(rr % g.ny), (int)(rr / g.ny), t, g);
      }
    }
    uint32_t a[MF][4];
#pragma unroll
    for (int mt = 0; mt < MF; ++mt) {
      uint32_t v[2][4];
#pragma unroll
      for (int hr = 0; hr < 2; ++hr) {
        const int n = n0 + mt * 16 + gid + 8 * hr;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          v[hr][q] = (kp[q] < pend && n < n_out) ? ld16(dy + kp[q] * dcs + dcoff + n) : 0u;
      }
      a[mt][0] = v[0][0] | (v[0][1] << 16);
      a[mt][1] = v[1][0] | (v[1][1] << 16);
      a[mt][2] = v[0][2] | (v[0][3] << 16);
      a[mt][3] = v[1][2] | (v[1][3] << 16);
    }
#pragma unroll
    for (int j = 0; j < NFC; ++j) {
      const int k = c0 + j * 8 + gid;
      uint32_t xv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) xv[q] = (si[q] >= 0 && k < cin) ? ld16(x + si[q] * xcs + xcoff + k) : 0u;
      const uint32_t b0 = xv[0] | (xv[1] << 16), b1 = xv[2] | (xv[3] << 16);
#pragma unroll
      for (int mt = 0; mt < MF; ++mt) mma_bf16(acc[mt][j], a[mt], b0, b1);
    }
  }
  float* pw = part + (size_t)(split * 4 + warp) * n_out * 27 * cin;
#pragma unroll
  for (int mt = 0; mt < MF; ++mt)
#pragma unroll
    for (int j = 0; j < NFC; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int n = n0 + mt * 16 + gid + 8 * (e >> 1), k = c0 + j * 8 + tig * 2 + (e & 1);
        if (n < n_out && k < cin) pw[((size_t)n * 27 + t) * cin + k] = acc[mt][j][e];
      }
}

__global__ void k_sum_parts(const float* __restrict__ part, int nparts, long long n, float* __restrict__ out,
                            int accumulate) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int q = 0; q < nparts; ++q) s += part[(size_t)q * n + i];
    out[i] = accumulate ? out[i] + s : s;
  }
}

// db partials: block (32 channels x 8 rows) over a position range
__global__ void k_bias_part(const bf16* __restrict__ dy, int dcs, int dcoff, int n_out, long long npos,
                            long long chunk, float* __restrict__ part) {
  __shared__ float s[8][33];
  const int c = threadIdx.x, ty = threadIdx.y;
  const long long pbeg = (long long)blockIdx.x * chunk, pend = min(npos, pbeg + chunk);
  float acc = 0.f;
  if (c < n_out)
    for (long long p = pbeg + ty; p < pend; p += 8) acc += __bfloat162float(dy[p * dcs + dcoff + c]);
  s[ty][c] = acc;
  __syncthreads();
  if (ty == 0 && c < n_out) {
    float v = 0.f;
    for (int q = 0; q < 8; ++q) v += s[q][c];
    part[(size_t)blockIdx.x * n_out + c] = v;
  }
}

// ---- elementwise pieces -------------------------------------------------------

__global__ void k_relu_bwd(bf16* __restrict__ dy, const bf16* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    if (!(__bfloat162float(y[i]) > 0.f)) dy[i] = __float2bfloat16_rn(0.f);
}

// per-axis taps of fine index p: coarse lo/hi and weights
__device__ __forceinline__ void up_taps(int p, int m, int& lo, int& hi, float& wlo, float& whi) {
  if ((p & 1) == 0) {
    lo = hi = p >> 1;
    wlo = 1.f;
    whi = 0.f;
  } else {
    lo = (p - 1) >> 1;
    hi = min((p + 1) >> 1, m - 1);
    wlo = 0.5f;
    whi = 0.5f;
  }
}

__global__ void k_upsample2(const bf16* __restrict__ cz, int ccs, int ccoff, int mx, int my, int mz,
                            bf16* __restrict__ fz, int fcs, int fcoff, int nx, int ny, int nz, int C) {
  const long long n = (long long)nx * ny * nz * C;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int ch = (int)(i % C);
    const long long p = i / C;
    const int x = (int)(p % nx);
    const long long rr = p / nx;
    const int y = (int)(rr % ny), z = (int)(rr / ny);
    int xl, xh, yl, yh, zl, zh;
    float wxl, wxh, wyl, wyh, wzl, wzh;
    up_taps(x, mx, xl, xh, wxl, wxh);
    up_taps(y, my, yl, yh, wyl, wyh);
    up_taps(z, mz, zl, zh, wzl, wzh);
    auto at = [&](int xx, int yy, int zz) {
      return __bfloat162float(cz[(((long long)zz * my + yy) * mx + xx) * ccs + ccoff + ch]);
    };
    float v = 0.f;
    const int X[2] = {xl, xh}, Y[2] = {yl, yh}, Z[2] = {zl, zh};
    const float WX[2] = {wxl, wxh}, WY[2] = {wyl, wyh}, WZ[2] = {wzl, wzh};
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const float wgt = WZ[a] * WY[b] * WX[c];
          if (wgt != 0.f) v += wgt * at(X[c], Y[b], Z[a]);
        }
    fz[p * fcs + fcoff + ch] = __float2bfloat16_rn(v);
  }
}

// weight of fine index p on coarse index q along one axis
__device__ __forceinline__ float up_weight(int p, int q, int m) {
  int lo, hi;
  float wlo, whi;
  up_taps(p, m, lo, hi, wlo, whi);
  return (lo == q ? wlo : 0.f) + (hi == q ? whi : 0.f);
}

// The same with one thread per 8-channel group: 16-byte loads of each
// corner's 8 channels and one 16-byte store, the per-channel arithmetic of
// k_upsample2 in the same order (bit-identical).  Channel strides, offsets
// and C multiples of 8, 16-byte aligned tensors.
__global__ void k_upsample2_v8(const bf16* __restrict__ cz, int ccs, int ccoff, int mx, int my, int mz,
                               bf16* __restrict__ fz, int fcs, int fcoff, int nx, int ny, int nz, int C) {
  const int G = C >> 3;
  const long long n = (long long)nx * ny * nz * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int gq = (int)(i % G);
    const long long p = i / G;
    const int x = (int)(p % nx);
    const long long rr = p / nx;
    const int y = (int)(rr % ny), z = (int)(rr / ny);
    int xl, xh, yl, yh, zl, zh;
    float wxl, wxh, wyl, wyh, wzl, wzh;
    up_taps(x, mx, xl, xh, wxl, wxh);
    up_taps(y, my, yl, yh, wyl, wyh);
    up_taps(z, mz, zl, zh, wzl, wzh);
    const int X[2] = {xl, xh}, Y[2] = {yl, yh}, Z[2] = {zl, zh};
    const float WX[2] = {wxl, wxh}, WY[2] = {wyl, wyh}, WZ[2] = {wzl, wzh};
    float v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] = 0.f;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const float wgt = WZ[a] * WY[b] * WX[c];
          if (wgt == 0.f) continue;
          const uint4 q = __ldg(
              (const uint4*)(cz + (((long long)Z[a] * my + Y[b]) * mx + X[c]) * ccs + ccoff + 8 * gq));
          const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            v[2 * k] += wgt * __uint_as_float(w[k] << 16);
            v[2 * k + 1] += wgt * __uint_as_float(w[k] & 0xFFFF0000u);
          }
        }
    uint32_t o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const __nv_bfloat162 b2 = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
      o[k] = *reinterpret_cast<const uint32_t*>(&b2);
    }
    *(uint4*)(fz + p * fcs + fcoff + 8 * gq) = make_uint4(o[0], o[1], o[2], o[3]);
  }
}

__global__ void k_upsample2_bwd(const bf16* __restrict__ df, int fcs, int fcoff, int nx, int ny, int nz,
                                bf16* __restrict__ dc, int ccs, int ccoff, int mx, int my, int mz, int C) {
  const long long n = (long long)mx * my * mz * C;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int ch = (int)(i % C);
    const long long q = i / C;
    const int x = (int)(q % mx);
    const long long rr = q / mx;
    const int y = (int)(rr % my), z = (int)(rr / my);
    float v = 0.f;
    for (int dz = -1; dz <= 1; ++dz) {
      const int pz = 2 * z + dz;
      if (pz < 0 || pz >= nz) continue;
      const float wz = up_weight(pz, z, mz);
      if (wz == 0.f) continue;
      for (int dyy = -1; dyy <= 1; ++dyy) {
        const int py = 2 * y + dyy;
        if (py < 0 || py >= ny) continue;
        const float wy = up_weight(py, y, my);
        if (wy == 0.f) continue;
        for (int dx = -1; dx <= 1; ++dx) {
          const int px = 2 * x + dx;
          if (px < 0 || px >= nx) continue;
          const float wx = up_weight(px, x, mx);
          if (wx == 0.f) continue;
          v += wz * wy * wx * __bfloat162float(df[(((long long)pz * ny + py) * nx + px) * fcs + fcoff + ch]);
        }
      }
    }
    dc[q * ccs + ccoff + ch] = __float2bfloat16_rn(v);
  }
}

// Mean and 1/std of an image from its sums (s, s2) over n voxels, as the
// host computes them: mean = s / n, var = s2 / n - mean^2, std = sqrt(var)
// (1 where var <= 0).
__device__ __forceinline__ void standardise_from_sums(double s, double s2, double n, float& mean, float& inv_std) {
  const double m = s / n;
  const double var = __dsub_rn(s2 / n, __dmul_rn(m, m));  // no FMA contraction: the host's rounding
  mean = (float)m;
  inv_std = (float)(1.0 / (var > 0.0 ? sqrt(var) : 1.0));
}

// flip (bit 0 x, 1 y, 2 z): pool the image mirrored along those axes.
// sums (device {sum f, sum f^2, sum g, sum g^2}, or null): the standardising
// statistics are computed from them instead of taken from mf..isg.
__global__ void k_pool_input(const float* __restrict__ f, const float* __restrict__ gimg, int nx, int ny, int nz,
                             int gx, int gy, int gz, float mf, float isf, float mg, float isg, int flip,
                             const double* __restrict__ sums, bf16* __restrict__ out) {
  const long long n = (long long)gx * gy * gz;
  if (sums) {
    // once per block (FP64 division and square root on GB300's narrow FP64 pipe)
    __shared__ float s_std[4];
    if (threadIdx.x == 0) {
      const double nv = (double)nx * ny * nz;
      standardise_from_sums(sums[0], sums[1], nv, s_std[0], s_std[1]);
      standardise_from_sums(sums[2], sums[3], nv, s_std[2], s_std[3]);
    }
    __syncthreads();
    mf = s_std[0];
    isf = s_std[1];
    mg = s_std[2];
    isg = s_std[3];
  }
  const float tw[5] = {1.f, 2.f, 2.f, 2.f, 1.f};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % gx);
    const long long rr = i / gx;
    const int y = (int)(rr % gy), z = (int)(rr / gy);
    // per axis the 5 taps' (mirrored) source indices and weights; a tap
    // outside the volume gets weight 0 at a clamped index, so the window is
    // walked without branches (adding +0 leaves the sums unchanged)
    int ox[5];
    long long oy[5], oz[5];
    float wx[5], wy[5], wz[5];
#pragma unroll
    for (int d = 0; d < 5; ++d) {
      const int vx = 4 * x + d - 2, vy = 4 * y + d - 2, vz = 4 * z + d - 2;
      const bool ix = vx >= 0 && vx < nx, iy = vy >= 0 && vy < ny, iz = vz >= 0 && vz < nz;
      const int cx = ix ? vx : 0, cy = iy ? vy : 0, cz = iz ? vz : 0;
      ox[d] = (flip & 1) ? nx - 1 - cx : cx;
      oy[d] = (long long)((flip & 2) ? ny - 1 - cy : cy) * nx;
      oz[d] = (long long)((flip & 4) ? nz - 1 - cz : cz) * nx * ny;
      wx[d] = ix ? tw[d] : 0.f;
      wy[d] = iy ? tw[d] : 0.f;
      wz[d] = iz ? tw[d] : 0.f;
    }
    float sf = 0.f, sg = 0.f, sw = 0.f;
#pragma unroll
    for (int dz = 0; dz < 5; ++dz) {
#pragma unroll
      for (int dyy = 0; dyy < 5; ++dyy) {
        const float wzy = wz[dz] * wy[dyy];
        const long long row = oz[dz] + oy[dyy];
#pragma unroll
        for (int dx = 0; dx < 5; ++dx) {
          const float wgt = wzy * wx[dx];
          sf += wgt * __ldg(f + row + ox[dx]);
          sg += wgt * __ldg(gimg + row + ox[dx]);
          sw += wgt;
        }
      }
    }
    out[2 * i] = __float2bfloat16_rn((sf / sw - mf) * isf);
    out[2 * i + 1] = __float2bfloat16_rn((sg / sw - mg) * isg);
  }
}

// Sums of f, f^2, g and g^2 in one read of each image: float4 loads, four
// grid strides per trip, FP32 partials over eight trips (128 elements per
// image), then one FP64 add per quantity -- GB300's FP64 pipe is narrow: one
// FP64 add and conversion per float4 made this pass FP64-bound (0.62 ms for
// 2 x 513^3 voxels), one per trip still 0.35 ms.
__global__ void __launch_bounds__(256) k_moments2(const float* __restrict__ f, const float* __restrict__ g, long long n,
                                                  bool vec4, GridReduce red, double* __restrict__ out) {
  __shared__ double s_red[8];
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  const long long gtid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i0 = 0;
  if (vec4) {
    // four grid strides per trip: eight 16-byte loads in flight per thread
    const long long n4 = n >> 2;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int trips = 0;
    for (long long q0 = gtid; q0 < n4; q0 += 4 * stride) {
      float4 x[4], y[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const long long q = q0 + u * stride;
        if (q < n4) {
          x[u] = __ldg((const float4*)f + q);
          y[u] = __ldg((const float4*)g + q);
        } else {
          x[u] = y[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        s0 += (x[u].x + x[u].y) + (x[u].z + x[u].w);
        s1 += x[u].x * x[u].x + x[u].y * x[u].y + x[u].z * x[u].z + x[u].w * x[u].w;
        s2 += (y[u].x + y[u].y) + (y[u].z + y[u].w);
        s3 += y[u].x * y[u].x + y[u].y * y[u].y + y[u].z * y[u].z + y[u].w * y[u].w;
      }
      if (++trips == 8) {
        a0 += (double)s0;
        a1 += (double)s1;
        a2 += (double)s2;
        a3 += (double)s3;
        s0 = s1 = s2 = s3 = 0.f;
        trips = 0;
      }
    }
    a0 += (double)s0;
    a1 += (double)s1;
    a2 += (double)s2;
    a3 += (double)s3;
    i0 = n4 << 2;
  }
  for (long long i = i0 + gtid; i < n; i += stride) {
    const double x = (double)f[i], y = (double)g[i];
    a0 += x;
    a1 += x * x;
    a2 += y;
    a3 += y * y;
  }
  double mine[4] = {block_sum(a0, s_red), block_sum(a1, s_red), block_sum(a2, s_red), block_sum(a3, s_red)}, o[4];
  if (grid_reduce_sum<4>(red, mine, o, s_red) && threadIdx.x == 0)
    for (int k = 0; k < 4; ++k) out[k] = o[k];
}

// out = x mirrored along the axes of flip; one position = two BF16
// channels = one 32-bit word.
__global__ void k_mirror_input(const uint32_t* __restrict__ x, int gx, int gy, int gz, int flip,
                               uint32_t* __restrict__ out) {
  const long long n = (long long)gx * gy * gz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int px = (int)(i % gx);
    const long long rr = i / gx;
    const int py = (int)(rr % gy), pz = (int)(rr / gy);
    const int sx = (flip & 1) ? gx - 1 - px : px, sy = (flip & 2) ? gy - 1 - py : py, sz = (flip & 4) ? gz - 1 - pz : pz;
    out[i] = x[((long long)sz * gy + sy) * gx + sx];
  }
}

__global__ void __launch_bounds__(256) k_mse(const float* __restrict__ pred, int pcs, const float* __restrict__ tgt,
                                             long long npos, double scale, bf16* __restrict__ dpred, int dcs,
                                             double* loss, GridReduce red) {
  __shared__ double s_red[8];
  const double inv = 1.0 / (3.0 * (double)npos);
  double acc = 0.0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npos;
       p += (long long)gridDim.x * blockDim.x) {
    for (int c = 0; c < 3; ++c) {
      const double d = (double)pred[p * pcs + c] - (double)tgt[3 * p + c];
      acc += d * d;
      if (dpred) dpred[p * dcs + c] = __float2bfloat16_rn((float)(scale * 2.0 * d * inv));
    }
    if (dpred)
      for (int c = 3; c < dcs; ++c) dpred[p * dcs + c] = __float2bfloat16_rn(0.f);
  }
  double mine[1] = {block_sum(acc, s_red)}, out[1];
  if (grid_reduce_sum<1>(red, mine, out, s_red) && threadIdx.x == 0) *loss = out[0] * inv;
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void k_pack(const float* __restrict__ w, int n_out, int cin, int npad8, bf16* __restrict__ wf,
                       bf16* __restrict__ wb, int kpad8, int npad16) {
  const bool small = (cin == 2);
  const long long nf = small ? (long long)npad8 * 64 : (long long)npad8 * 27 * cin;
  const long long nb = wb ? (long long)kpad8 * 27 * npad16 : 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nf + nb;
       i += (long long)gridDim.x * blockDim.x) {
    if (i < nf) {
      float v = 0.f;
      if (small) {
        const int n = (int)(i / 64), kk = (int)(i % 64);
        if (n < n_out && kk < 54) v = w[((size_t)n * 27 + kk / 2) * 2 + (kk & 1)];
      } else {
        const int n = (int)(i / (27 * cin));
        if (n < n_out) v = w[i];
      }
      wf[i] = __float2bfloat16_rn(v);
    } else {
      const long long j = i - nf;
      const int n = (int)(j % npad16);
      const long long r = j / npad16;
      const int t = (int)(r % 27), k = (int)(r / 27);
      float v = 0.f;
      if (n < n_out && k < cin) v = w[((size_t)n * 27 + t) * cin + k];
      wb[j] = __float2bfloat16_rn(v);
    }
  }
}

// flip (bit 0 x, 1 y, 2 z): pred is the network's output for the pair
// mirrored along those axes; it is read at the mirrored positions with the
// mirrored components negated.  U = (accumulate ? U : 0) + weight * sample.
__global__ void k_seed_nodes(const float* __restrict__ pred, int pcs, int px, int py, int pz, int h, int Nnx, int Nny,
                             int Nnz, int flip, double weight, int accumulate, double* __restrict__ U) {
  const long long n = (long long)Nnx * Nny * Nnz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int ni = (int)(i % Nnx);
    const long long rr = i / Nnx;
    const int nj = (int)(rr % Nny), nk = (int)(rr / Nny);
    const int dims[3] = {px, py, pz};
    double c[3] = {ni * (double)h / 8.0, nj * (double)h / 8.0, nk * (double)h / 8.0};
    for (int k = 0; k < 3; ++k)
      if (flip & (1 << k)) c[k] = (double)(dims[k] - 1) - c[k];
    int lo[3], hi[3];
    double t[3];
    for (int k = 0; k < 3; ++k) {
      const double cc = fmin(fmax(c[k], 0.0), (double)(dims[k] - 1));
      lo[k] = (int)floor(cc);
      hi[k] = min(lo[k] + 1, dims[k] - 1);
      t[k] = cc - lo[k];
    }
    for (int ch = 0; ch < 3; ++ch) {
      double v = 0.0;
      for (int a = 0; a < 8; ++a) {
        const int X = (a & 1) ? hi[0] : lo[0], Y = (a & 2) ? hi[1] : lo[1], Z = (a & 4) ? hi[2] : lo[2];
        const double wgt = ((a & 1) ? t[0] : 1.0 - t[0]) * ((a & 2) ? t[1] : 1.0 - t[1]) * ((a & 4) ? t[2] : 1.0 - t[2]);
        if (wgt != 0.0) v += wgt * (double)pred[(((long long)Z * py + Y) * px + X) * pcs + ch];
      }
      if (flip & (1 << ch)) v = -v;
      U[3 * i + ch] = (accumulate ? U[3 * i + ch] : 0.0) + weight * v;
    }
  }
}

inline int eblocks(long long n) { return grid_blocks(n, 256, 152 * 32); }

template <int NF>
static void launch_conv_nf(bool small, dim3 grid, const bf16* src, int scs, int scoff, int cin, const bf16* w,
                           const float* bias, int n_out, int relu, void* out, int out_f32, int ocs, int ocoff, int acc,
                           Geo g, cudaStream_t s) {
  if constexpr (NF <= 4) {
    if (small) {
      k_conv<NF, true><<<grid, 128, 0, s>>>(src, scs, scoff, cin, w, bias, n_out, relu, out, out_f32, ocs, ocoff, acc,
                                            g);
      return;
    }
  }
  k_conv<NF, false><<<grid, 128, 0, s>>>(src, scs, scoff, cin, w, bias, n_out, relu, out, out_f32, ocs, ocoff, acc, g);
}

template <int MF, int NFC>
static void launch_wgrad_t(dim3 grid, const bf16* dy, int dcs, int dcoff, int n_out, const bf16* x, int xcs, int xcoff,
                           int cin, Geo g, long long chunk, float* part, cudaStream_t s) {
  k_wgrad<MF, NFC><<<grid, 128, 0, s>>>(dy, dcs, dcoff, n_out, x, xcs, xcoff, cin, g, chunk, part);
}

template <int MF>
static int launch_wgrad_m(int nfc, dim3 grid, const bf16* dy, int dcs, int dcoff, int n_out, const bf16* x, int xcs,
                          int xcoff, int cin, Geo g, long long chunk, float* part, cudaStream_t s) {
  switch (nfc) {
    case 1: launch_wgrad_t<MF, 1>(grid, dy, dcs, dcoff, n_out, x, xcs, xcoff, cin, g, chunk, part, s); break;
    case 2: launch_wgrad_t<MF, 2>(grid, dy, dcs, dcoff, n_out, x, xcs, xcoff, cin, g, chunk, part, s); break;
    case 3: launch_wgrad_t<MF, 3>(grid, dy, dcs, dcoff, n_out, x, xcs, xcoff, cin, g, chunk, part, s); break;
    case 4: launch_wgrad_t<MF, 4>(grid, dy, dcs, dcoff, n_out, x, xcs, xcoff, cin, g, chunk, part, s); break;
    case 5: launch_wgrad_t<MF, 5>(grid, dy, dcs, dcoff, n_out, x, xcs, xcoff, cin, g, chunk, part, s); break;
    case 6: launch_wgrad_t<MF, 6>(grid, dy, dcs, dcoff, n_out, x, xcs, xcoff, cin, g, chunk, part, s); break;
    case 7: launch_wgrad_t<MF, 7>(grid, dy, dcs, dcoff, n_out, x, xcs, xcoff, cin, g, chunk, part, s); break;
    case 8: launch_wgrad_t<MF, 8>(grid, dy, dcs, dcoff, n_out, x, xcs, xcoff, cin, g, chunk, part, s); break;
    default: return VDVC_ERR_UNSUPPORTED;
  }
  return VDVC_OK;
}

constexpr int kWgradSplits = 24;  // position splits per tap (x 4 warps = partials)

static bool geo_ok(const vdvc_conv_geom* g) {
  return g && g->nx >= 1 && g->ny >= 1 && g->nz >= 1 && g->sx >= 1 && g->sy >= 1 && g->sz >= 1 && g->d >= 1 &&
         g->a >= 0 && (g->c == 1 || g->c == -1) && g->b >= -2 && g->b <= 2 && g->a <= 4 && g->d <= 4;
}

static Geo to_geo(const vdvc_conv_geom* g) {
  return Geo{g->nx, g->ny, g->nz, g->sx, g->sy, g->sz, g->a, g->b, g->c, g->d};
}

static bool al4(const void* p) { return ((uintptr_t)p & 3u) == 0; }

}  // namespace vdvc

using namespace vdvc;

extern "C" {

int vdvc_cnn_conv(const void* src, int src_cstride, int src_coff, int cin, const void* w, const float* bias, int n_out,
                  int relu, void* out, int out_f32, int out_cstride, int out_coff, int accumulate,
                  const vdvc_conv_geom* geom, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(src && w && out && geo_ok(geom), "bad arguments");
  VDVC_CHECK_ARG(cin == 2 || (cin >= 16 && cin % 16 == 0), "cin must be 2 or a multiple of 16 (got %d)", cin);
  VDVC_CHECK_ARG(n_out >= 1 && n_out <= 256, "n_out must be in [1, 256]");
  VDVC_CHECK_ARG(src_cstride % 2 == 0 && src_coff % 2 == 0 && src_coff >= 0 && src_coff + cin <= src_cstride,
                 "source channel range [%d, %d) does not fit stride %d (even offsets required)", src_coff,
                 src_coff + cin, src_cstride);
  VDVC_CHECK_ARG(out_coff >= 0 && out_coff + n_out <= out_cstride, "output channel range does not fit its stride");
  VDVC_CHECK_ARG(al4(src) && al4(w), "src and w must be 4-byte aligned");
  VDVC_CHECK_ARG(!(accumulate && out_f32), "accumulate needs a BF16 output");
  cudaStream_t s = (cudaStream_t)stream;
  // the tensor-core forms wherever the channel chunks are 16-byte aligned
  if (cin == 2) {
    int* err = nullptr;
    int st = conv_error_flag(&err);
    if (st) return st;
    st = launch_conv_first(src, src_cstride, src_coff, w, (n_out + 7) / 8 * 8, bias, n_out, relu, out, out_f32,
                           out_cstride, out_coff, accumulate, geom, err, s);
    if (st != VDVC_ERR_UNSUPPORTED) return st;
  } else {
    int* err = nullptr;
    int st = conv_error_flag(&err);
    if (st) return st;
    st = launch_conv_tma(src, src_cstride, src_coff, cin, w, (n_out + 7) / 8 * 8, bias, n_out, relu, out, out_f32,
                         out_cstride, out_coff, accumulate, geom, err, s);
    if (st != VDVC_ERR_UNSUPPORTED) return st;
    st = launch_conv_tc(src, src_cstride, src_coff, cin, w, (n_out + 7) / 8 * 8, bias, n_out, relu, out, out_f32,
                        out_cstride, out_coff, accumulate, geom, err, s);
    if (st != VDVC_ERR_UNSUPPORTED) return st;
  }
  VDVC_CHECK_ARG(n_out <= 80, "n_out must be in [1, 80] unless the layer fits the tensor-core form "
                              "(channel strides and offsets multiples of 8, 16-byte aligned tensors)");
  const int nf = (n_out + 7) / 8;
  if (cin == 2) VDVC_CHECK_ARG(nf <= 4, "cin == 2 supports n_out <= 32");
  const Geo g = to_geo(geom);
  const long long npos = (long long)g.nx * g.ny * g.nz;
  const long long nb = (npos + 63) / 64;
  VDVC_CHECK_ARG(nb < 0x7fffffffLL, "grid too large");
  dim3 grid((unsigned)nb);
  const bf16* sp = (const bf16*)src;
  const bf16* wp = (const bf16*)w;
  const bool small = cin == 2;
  switch (nf) {
    case 1: launch_conv_nf<1>(small, grid, sp, src_cstride, src_coff, cin, wp, bias, n_out, relu, out, out_f32, out_cstride, out_coff, accumulate, g, s); break;
    case 2: launch_conv_nf<2>(small, grid, sp, src_cstride, src_coff, cin, wp, bias, n_out, relu, out, out_f32, out_cstride, out_coff, accumulate, g, s); break;
    case 3: launch_conv_nf<3>(small, grid, sp, src_cstride, src_coff, cin, wp, bias, n_out, relu, out, out_f32, out_cstride, out_coff, accumulate, g, s); break;
    case 4: launch_conv_nf<4>(small, grid, sp, src_cstride, src_coff, cin, wp, bias, n_out, relu, out, out_f32, out_cstride, out_coff, accumulate, g, s); break;
    case 5: launch_conv_nf<5>(small, grid, sp, src_cstride, src_coff, cin, wp, bias, n_out, relu, out, out_f32, out_cstride, out_coff, accumulate, g, s); break;
    case 6: launch_conv_nf<6>(small, grid, sp, src_cstride, src_coff, cin, wp, bias, n_out, relu, out, out_f32, out_cstride, out_coff, accumulate, g, s); break;
    case 7: launch_conv_nf<7>(small, grid, sp, src_cstride, src_coff, cin, wp, bias, n_out, relu, out, out_f32, out_cstride, out_coff, accumulate, g, s); break;
    case 8: launch_conv_nf<8>(small, grid, sp, src_cstride, src_coff, cin, wp, bias, n_out, relu, out, out_f32, out_cstride, out_coff, accumulate, g, s); break;
    case 9: launch_conv_nf<9>(small, grid, sp, src_cstride, src_coff, cin, wp, bias, n_out, relu, out, out_f32, out_cstride, out_coff, accumulate, g, s); break;
    case 10: launch_conv_nf<10>(small, grid, sp, src_cstride, src_coff, cin, wp, bias, n_out, relu, out, out_f32, out_cstride, out_coff, accumulate, g, s); break;
  }
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cnn_status(vdvc_stream_t stream) {
  int* err = nullptr;
  int st = conv_error_flag(&err);
  if (st) return st;
  int h = 0;
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaStreamSynchronize(s));
  if (h) {
    VDVC_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    VDVC_CUDA(cudaStreamSynchronize(s));
    return set_error(VDVC_ERR_TIMEOUT, "a tensor-core convolution gave up a bounded wait; its output is incomplete");
  }
  return VDVC_OK;
}

size_t vdvc_cnn_wgrad_workspace_bytes(int n_out, int cin) {
  if (n_out < 1 || cin < 1) return 0;
  return (size_t)kWgradSplits * 4 * n_out * 27 * (cin < 16 ? 16 : cin) * sizeof(float) + 256;
}

int vdvc_cnn_conv_wgrad(const void* dy, int dy_cstride, int dy_coff, int n_out, const void* x, int x_cstride,
                        int x_coff, int cin, const vdvc_conv_geom* geom, float* dw, int accumulate, void* ws,
                        size_t ws_bytes, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(dy && x && dw && geo_ok(geom), "bad arguments");
  VDVC_CHECK_ARG(n_out >= 1 && n_out <= 256, "wgrad supports n_out <= 256");
  VDVC_CHECK_ARG(cin >= 1 && cin <= 256, "wgrad supports cin <= 256");
  VDVC_CHECK_ARG(dy_coff >= 0 && dy_coff + n_out <= dy_cstride && x_coff >= 0 && x_coff + cin <= x_cstride,
                 "channel ranges do not fit their strides");
  const size_t need = vdvc_cnn_wgrad_workspace_bytes(n_out, cin);
  VDVC_CHECK_ARG(ws && ws_bytes >= need, "wgrad needs %zu bytes of workspace", need);
  const Geo g = to_geo(geom);
  const long long npos = (long long)g.nx * g.ny * g.nz;
  const long long chunk = (npos + kWgradSplits - 1) / kWgradSplits;
  dim3 grid(27, kWgradSplits, ((n_out + 31) / 32) * ((cin + 63) / 64));
  cudaStream_t s = (cudaStream_t)stream;
  float* part = (float*)ws;
  const int mf = n_out > 16 ? 2 : 1, nfc = cin >= 64 ? 8 : (cin + 7) / 8;
  int st = (mf == 1) ? launch_wgrad_m<1>(nfc, grid, (const bf16*)dy, dy_cstride, dy_coff, n_out, (const bf16*)x,
                                         x_cstride, x_coff, cin, g, chunk, part, s)
                     : launch_wgrad_m<2>(nfc, grid, (const bf16*)dy, dy_cstride, dy_coff, n_out, (const bf16*)x,
                                         x_cstride, x_coff, cin, g, chunk, part, s);
  if (st) return set_error(st, "wgrad: unsupported shape");
  count_launch();
  const long long n = (long long)n_out * 27 * cin;
  k_sum_parts<<<eblocks(n), 256, 0, s>>>(part, kWgradSplits * 4, n, dw, accumulate);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cnn_bias_grad(const void* dy, int dy_cstride, int dy_coff, int n_out, long long npos, float* db,
                       int accumulate, void* ws, size_t ws_bytes, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(dy && db && npos >= 1 && n_out >= 1 && n_out <= 256 && dy_coff >= 0 &&
                     dy_coff + n_out <= dy_cstride,
                 "bad arguments");
  const int nblk = 256;
  VDVC_CHECK_ARG(ws && ws_bytes >= (size_t)nblk * 32 * sizeof(float), "bias_grad workspace too small");
  const long long chunk = (npos + nblk - 1) / nblk;
  cudaStream_t s = (cudaStream_t)stream;
  // groups of 32 channels, one after another through the same partials
  for (int c0 = 0; c0 < n_out; c0 += 32) {
    const int ng = n_out - c0 < 32 ? n_out - c0 : 32;
    k_bias_part<<<nblk, dim3(32, 8), 0, s>>>((const bf16*)dy, dy_cstride, dy_coff + c0, ng, npos, chunk,
                                             (float*)ws);
    count_launch();
    k_sum_parts<<<1, 32, 0, s>>>((const float*)ws, nblk, ng, db + c0, accumulate);
    VDVC_LAUNCHED();
  }
  return VDVC_OK;
}

int vdvc_cnn_relu_bwd(void* dy, const void* y, long long n, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(dy && y && n >= 0, "bad arguments");
  if (n == 0) return VDVC_OK;
  k_relu_bwd<<<eblocks(n), 256, 0, (cudaStream_t)stream>>>((bf16*)dy, (const bf16*)y, n);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cnn_upsample2(const void* coarse, int c_cstride, int ccoff, int mx, int my, int mz, void* fine, int f_cstride,
                       int fcoff, int nx, int ny, int nz, int C, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(coarse && fine && C >= 1 && mx >= 1 && my >= 1 && mz >= 1, "bad arguments");
  VDVC_CHECK_ARG(nx <= 2 * mx && ny <= 2 * my && nz <= 2 * mz && nx >= 2 * mx - 1 && ny >= 2 * my - 1 &&
                     nz >= 2 * mz - 1,
                 "fine grid must be 2m-1 or 2m per axis");
  VDVC_CHECK_ARG(ccoff >= 0 && ccoff + C <= c_cstride && fcoff >= 0 && fcoff + C <= f_cstride, "channel ranges");
  const long long n = (long long)nx * ny * nz * C;
  if (C % 8 == 0 && c_cstride % 8 == 0 && ccoff % 8 == 0 && f_cstride % 8 == 0 && fcoff % 8 == 0 &&
      (((uintptr_t)coarse | (uintptr_t)fine) & 15) == 0) {
    k_upsample2_v8<<<eblocks(n / 8), 256, 0, (cudaStream_t)stream>>>((const bf16*)coarse, c_cstride, ccoff, mx, my,
                                                                     mz, (bf16*)fine, f_cstride, fcoff, nx, ny, nz,
                                                                     C);
    VDVC_LAUNCHED();
    return VDVC_OK;
  }
  k_upsample2<<<eblocks(n), 256, 0, (cudaStream_t)stream>>>((const bf16*)coarse, c_cstride, ccoff, mx, my, mz,
                                                            (bf16*)fine, f_cstride, fcoff, nx, ny, nz, C);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cnn_upsample2_bwd(const void* dfine, int f_cstride, int fcoff, int nx, int ny, int nz, void* dcoarse,
                           int c_cstride, int ccoff, int mx, int my, int mz, int C, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(dfine && dcoarse && C >= 1 && mx >= 1 && my >= 1 && mz >= 1, "bad arguments");
  VDVC_CHECK_ARG(nx <= 2 * mx && ny <= 2 * my && nz <= 2 * mz && nx >= 2 * mx - 1 && ny >= 2 * my - 1 &&
                     nz >= 2 * mz - 1,
                 "fine grid must be 2m-1 or 2m per axis");
  VDVC_CHECK_ARG(ccoff >= 0 && ccoff + C <= c_cstride && fcoff >= 0 && fcoff + C <= f_cstride, "channel ranges");
  const long long n = (long long)mx * my * mz * C;
  k_upsample2_bwd<<<eblocks(n), 256, 0, (cudaStream_t)stream>>>((const bf16*)dfine, f_cstride, fcoff, nx, ny, nz,
                                                                (bf16*)dcoarse, c_cstride, ccoff, mx, my, mz, C);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cnn_pool_input(const float* f_vox, const float* g_vox, int nx, int ny, int nz, const double* mean_std,
                        void* out, vdvc_stream_t stream) {
  return vdvc_cnn_pool_input_mirrored(f_vox, g_vox, nx, ny, nz, mean_std, 0, out, stream);
}

int vdvc_cnn_pool_input_mirrored(const float* f_vox, const float* g_vox, int nx, int ny, int nz,
                                 const double* mean_std, int flip, void* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f_vox && g_vox && out && mean_std && nx >= 1 && ny >= 1 && nz >= 1, "bad arguments");
  VDVC_CHECK_ARG(flip >= 0 && flip <= 7, "flip is a bit mask of the axes x (1), y (2), z (4)");
  VDVC_CHECK_ARG(mean_std[1] > 0.0 && mean_std[3] > 0.0, "image std must be positive");
  const int gx = (nx - 1) / 4 + 1, gy = (ny - 1) / 4 + 1, gz = (nz - 1) / 4 + 1;
  const long long n = (long long)gx * gy * gz;
  k_pool_input<<<eblocks(n), 256, 0, (cudaStream_t)stream>>>(f_vox, g_vox, nx, ny, nz, gx, gy, gz, (float)mean_std[0],
                                                             (float)(1.0 / mean_std[1]), (float)mean_std[2],
                                                             (float)(1.0 / mean_std[3]), flip, nullptr, (bf16*)out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cnn_input_moments(const float* f_vox, const float* g_vox, long long n, double* sums, void* ws,
                           size_t ws_bytes, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f_vox && g_vox && sums && n >= 1, "bad arguments");
  Carve cv(ws, ws_bytes);
  GridReduce red;
  red.partials = cv.take<double>(4 * kReduceBlocks);
  red.ticket = cv.take<unsigned int>(1);
  VDVC_CHECK_ARG(ws && cv.fits(), "input moments need %zu bytes of workspace", cv.off);
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(red.ticket, 0, sizeof(unsigned int), s));
  const bool vec4 = (((uintptr_t)f_vox | (uintptr_t)g_vox) & 15u) == 0;
  k_moments2<<<grid_blocks(vec4 ? (n + 3) / 4 : n, 256, kReduceBlocks), 256, 0, s>>>(f_vox, g_vox, n, vec4, red, sums);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cnn_pool_input_dev(const float* f_vox, const float* g_vox, int nx, int ny, int nz, const double* sums,
                            int flip, void* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(f_vox && g_vox && out && sums && nx >= 1 && ny >= 1 && nz >= 1, "bad arguments");
  VDVC_CHECK_ARG(flip >= 0 && flip <= 7, "flip is a bit mask of the axes x (1), y (2), z (4)");
  const int gx = (nx - 1) / 4 + 1, gy = (ny - 1) / 4 + 1, gz = (nz - 1) / 4 + 1;
  const long long n = (long long)gx * gy * gz;
  k_pool_input<<<eblocks(n), 256, 0, (cudaStream_t)stream>>>(f_vox, g_vox, nx, ny, nz, gx, gy, gz, 0.f, 1.f, 0.f, 1.f,
                                                             flip, sums, (bf16*)out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cnn_mirror_input(const void* x, int gx, int gy, int gz, int flip, void* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(x && out && x != out && gx >= 1 && gy >= 1 && gz >= 1, "bad arguments");
  VDVC_CHECK_ARG(flip >= 0 && flip <= 7, "flip is a bit mask of the axes x (1), y (2), z (4)");
  VDVC_CHECK_ARG(al4(x) && al4(out), "x and out must be 4-byte aligned");
  const long long n = (long long)gx * gy * gz;
  k_mirror_input<<<eblocks(n), 256, 0, (cudaStream_t)stream>>>((const uint32_t*)x, gx, gy, gz, flip, (uint32_t*)out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cnn_mse(const float* pred, int pred_cstride, const float* target, long long npos, double* loss, void* dpred,
                 int dp_cstride, double scale, void* ws, size_t ws_bytes, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(pred && target && loss && npos >= 1 && pred_cstride >= 3, "bad arguments");
  VDVC_CHECK_ARG(!dpred || dp_cstride >= 3, "dpred stride must be >= 3");
  Carve cv(ws, ws_bytes);
  GridReduce red;
  red.partials = cv.take<double>(kReduceBlocks);
  red.ticket = cv.take<unsigned int>(1);
  VDVC_CHECK_ARG(ws && cv.fits(), "mse needs %zu bytes of workspace", cv.off);
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(red.ticket, 0, sizeof(unsigned int), s));
  k_mse<<<grid_blocks(npos, 256, kReduceBlocks), 256, 0, s>>>(pred, pred_cstride, target, npos, scale, (bf16*)dpred,
                                                              dp_cstride, loss, red);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cnn_adam(float* w, const float* grad, float* m, float* v, long long n, double lr, double beta1, double beta2,
                  double eps, int step, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(w && grad && m && v && n >= 1 && step >= 1, "bad arguments");
  const float c1 = (float)(1.0 - pow(beta1, step)), c2 = (float)(1.0 - pow(beta2, step));
  k_adam<<<eblocks(n), 256, 0, (cudaStream_t)stream>>>(w, grad, m, v, n, (float)lr, (float)beta1, (float)beta2,
                                                       (float)eps, c1, c2);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cnn_pack_weights(const float* w, int n_out, int cin, void* wf, void* wb, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(w && wf && n_out >= 1 && n_out <= 256 && cin >= 1 && cin <= 256, "bad arguments");
  VDVC_CHECK_ARG(cin == 2 || cin % 16 == 0, "cin must be 2 or a multiple of 16");
  const int npad8 = (n_out + 7) / 8 * 8, npad16 = (n_out + 15) / 16 * 16, kpad8 = (cin + 7) / 8 * 8;
  const long long nf = cin == 2 ? (long long)npad8 * 64 : (long long)npad8 * 27 * cin;
  const long long nb = wb ? (long long)kpad8 * 27 * npad16 : 0;
  k_pack<<<eblocks(nf + nb), 256, 0, (cudaStream_t)stream>>>(w, n_out, cin, npad8, (bf16*)wf, (bf16*)wb, kpad8, npad16);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cnn_seed_nodes(const float* pred, int pred_cstride, int px, int py, int pz, int h, int Nx, int Ny, int Nz,
                        double* U, vdvc_stream_t stream) {
  return vdvc_cnn_seed_nodes_acc(pred, pred_cstride, px, py, pz, h, Nx, Ny, Nz, 0, 1.0, 0, U, stream);
}

int vdvc_cnn_seed_nodes_acc(const float* pred, int pred_cstride, int px, int py, int pz, int h, int Nx, int Ny,
                            int Nz, int flip, double weight, int accumulate, double* U, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(pred && U && pred_cstride >= 3 && px >= 1 && py >= 1 && pz >= 1 && h >= 1, "bad arguments");
  VDVC_CHECK_ARG(Nx >= 1 && Ny >= 1 && Nz >= 1, "bad mesh");
  VDVC_CHECK_ARG(flip >= 0 && flip <= 7, "flip is a bit mask of the axes x (1), y (2), z (4)");
  const int N[3] = {Nx, Ny, Nz}, P[3] = {px, py, pz};
  for (int k = 0; k < 3; ++k)
    VDVC_CHECK_ARG(!(flip & (1 << k)) || (long long)(P[k] - 1) * 8 == (long long)N[k] * h,
                   "a mirrored seed needs the mesh to span the output grid along each mirrored axis");
  const long long n = (long long)(Nx + 1) * (Ny + 1) * (Nz + 1);
  k_seed_nodes<<<eblocks(n), 256, 0, (cudaStream_t)stream>>>(pred, pred_cstride, px, py, pz, h, Nx + 1, Ny + 1, Nz + 1,
                                                             flip, weight, accumulate, U);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

}  // extern "C"
