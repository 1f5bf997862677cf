// Float32 Hessian element pass (H v and its PCG form) with one thread per
// element, for small element edges.  Same quadrature, ownership and outputs
// as the strip kernels (strip.cuh): element (i,j,k) owns the voxels
// [iH, iH+H) x [jH, jH+H) x [kH, kH+H), plus the mesh's last voxel plane on
// the last element of each axis, with weight 1/2 per axis on the outer
// voxel planes.
//
// At h <= 4 an element owns at most 64 voxels, too little work to amortise
// the strip kernels' per-block staging and shared-memory reduction (measured
// on 64^3 elements: 23 vs 43 us at h = 2, 82 vs 88 us at h = 4, H v with
// its gather); here each thread
// holds its element's 24 nodal values and 24 sums in registers, walks its
// voxels row by row (x fastest; a warp reads 32 consecutive elements' voxels
// of a row, one contiguous span) and writes the 24 element sums, coalesced,
// to the [24][Ne] element-vector buffer.  Per (qy,qz) row the nodal field is
// reduced to its two x-lines and the row's sums are spread back to the four
// (y,z) corners, so a voxel costs ~20 FMAs.
#include "ops.cuh"
#include "pcg.cuh"

namespace vdvc {

// Element e's 24 sums of H v (+ regularizer); PCG: v = a.v + beta a.p_old.
template <int H, bool PCG>
__device__ __forceinline__ void elem_hv_body(const StripArgs<float>& a, const Kpair<float>* __restrict__ kp,
                                             long long e, float beta) {
  const Mesh& m = a.m;
  int i, j, k;
  elem_ijk(m, e, i, j, k);

  // nodal values u[dz][dy][dx][c] (PCG: p_new = z + beta p_old)
  float u[2][2][2][3];
#pragma unroll
  for (int dz = 0; dz < 2; ++dz)
#pragma unroll
    for (int dy = 0; dy < 2; ++dy) {
      const long long n0 = (long long)i + (long long)(j + dy) * m.Nnx + (long long)(k + dz) * m.NnxNny;
#pragma unroll
      for (int dx = 0; dx < 2; ++dx)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const long long q = 3 * (n0 + dx) + c;
          float val = __ldg(a.v + q);
          if constexpr (PCG) val += beta * __ldg(a.p_old + q);
          u[dz][dy][dx][c] = val;
        }
    }
  float o[2][2][2][3];
#pragma unroll
  for (int q = 0; q < 24; ++q) (&o[0][0][0][0])[q] = 0.f;

  const bool x_last = (i == m.Nx - 1), y_last = (j == m.Ny - 1), z_last = (k == m.Nz - 1);
  const float wx_first = (i == 0) ? 0.5f : 1.f;
  const float wy_first = (j == 0) ? 0.5f : 1.f;
  const float wz_first = (k == 0) ? 0.5f : 1.f;
#pragma unroll
  for (int qz = 0; qz <= H; ++qz) {
    if (qz == H && !z_last) break;
    const float fz1 = (float)qz / (float)H, fz0 = 1.f - fz1;
    const float wz = (qz == 0) ? wz_first : (qz == H ? 0.5f : 1.f);
#pragma unroll
    for (int qy = 0; qy <= H; ++qy) {
      if (qy == H && !y_last) break;
      const float fy1 = (float)qy / (float)H, fy0 = 1.f - fy1;
      const float wyz = wz * ((qy == 0) ? wy_first : (qy == H ? 0.5f : 1.f));
      // the nodal field on the row's two x-lines
      float ul[2][3];
#pragma unroll
      for (int dx = 0; dx < 2; ++dx)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          ul[dx][c] = fz0 * (fy0 * u[0][0][dx][c] + fy1 * u[0][1][dx][c]) +
                      fz1 * (fy0 * u[1][0][dx][c] + fy1 * u[1][1][dx][c]);
      const long long vrow = (long long)i * H + (long long)(j * H + qy) * m.Nvx + (long long)(k * H + qz) * m.NvxNvy;
      const float* __restrict__ gp = a.grad + 3 * vrow;
      const uint8_t* __restrict__ mp = a.mask + vrow;
      float A[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
      for (int qx = 0; qx <= H; ++qx) {
        if (qx == H && !x_last) break;
        const float fx1 = (float)qx / (float)H, fx0 = 1.f - fx1;
        const float wx = (qx == 0) ? wx_first : (qx == H ? 0.5f : 1.f);
        const float g0 = __ldg(gp + 3 * qx), g1 = __ldg(gp + 3 * qx + 1), g2 = __ldg(gp + 3 * qx + 2);
        const bool mk = __ldg(mp + qx) != 0;
        const float u0 = fx0 * ul[0][0] + fx1 * ul[1][0];
        const float u1 = fx0 * ul[0][1] + fx1 * ul[1][1];
        const float u2 = fx0 * ul[0][2] + fx1 * ul[1][2];
        float d = (g0 * u0 + g1 * u1 + g2 * u2) * (wx * wyz);
        d = mk ? d : 0.f;
        const float t0 = d * g0, t1 = d * g1, t2 = d * g2;
        A[0][0] += fx0 * t0; A[0][1] += fx0 * t1; A[0][2] += fx0 * t2;
        A[1][0] += fx1 * t0; A[1][1] += fx1 * t1; A[1][2] += fx1 * t2;
      }
#pragma unroll
      for (int dx = 0; dx < 2; ++dx)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          o[0][0][dx][c] += (fz0 * fy0) * A[dx][c];
          o[0][1][dx][c] += (fz0 * fy1) * A[dx][c];
          o[1][0][dx][c] += (fz1 * fy0) * A[dx][c];
          o[1][1][dx][c] += (fz1 * fy1) * A[dx][c];
        }
    }
  }

  // regularizer: c1 K1 u_e (+ c2 K2 w_e), then the 24 coalesced stores
#pragma unroll
  for (int ca = 0; ca < 8; ++ca) {
    const int adx = corner_dx(ca), ady = corner_dy(ca), adz = corner_dz(ca);
    float s[3] = {o[adz][ady][adx][0], o[adz][ady][adx][1], o[adz][ady][adx][2]};
    if (a.nreg >= 1) {
      if (a.k1_blockdiag) {
#pragma unroll
        for (int cb = 0; cb < 8; ++cb) {
          const float l = a.c1 * a.L8[ca * 8 + cb];
#pragma unroll
          for (int c = 0; c < 3; ++c) s[c] += l * u[corner_dz(cb)][corner_dy(cb)][corner_dx(cb)][c];
        }
      } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float k1 = 0.f;
#pragma unroll
          for (int b = 0; b < 24; ++b) {
            const int cb = b / 3;
            k1 += __ldg(kp->K1 + (3 * ca + c) * 24 + b) * u[corner_dz(cb)][corner_dy(cb)][corner_dx(cb)][b % 3];
          }
          s[c] += a.c1 * k1;
        }
      }
      if (a.nreg == 2) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float k2 = 0.f;
#pragma unroll 4
          for (int b = 0; b < 24; ++b) {
            const int cb = b / 3;
            const long long node = (long long)(i + corner_dx(cb)) + (long long)(j + corner_dy(cb)) * m.Nnx +
                                   (long long)(k + corner_dz(cb)) * m.NnxNny;
            k2 += __ldg(kp->K2 + (3 * ca + c) * 24 + b) * __ldg(a.w + 3 * node + b % 3);
          }
          s[c] += a.c2 * k2;
        }
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) a.evA[(long long)(3 * ca + c) * m.Ne + e] = s[c];
  }
}

template <int H, bool PCG>
// 128-thread blocks; at H <= 2 capped at 96 registers, 5 blocks (20 warps)
// per SM without spills, against 16 warps at 128 registers (H >= 3 spills
// under that cap and keeps 128).
__global__ void __launch_bounds__(128, H <= 2 ? 5 : 4) k_elem_hv(const StripArgs<float> a, const Kpair<float>* __restrict__ kp) {
  if constexpr (PCG) {
    if (a.st->done) return;
  }
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= a.m.Ne) return;
  float beta = 0.f;
  if constexpr (PCG) beta = (float)a.st->beta;
  elem_hv_body<H, PCG>(a, kp, e, beta);
}

template <int H, bool PCG>
static int launch_e(const StripArgs<float>& args, const Kpair<float>* kp, cudaStream_t s) {
  const long long nb = (args.m.Ne + 127) / 128;
  if (nb > 0x7fffffffLL) return set_error(VDVC_ERR_ARG, "too many elements");
  k_elem_hv<H, PCG><<<(unsigned)nb, 128, 0, s>>>(args, kp);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

// VDVC_ERR_UNSUPPORTED (error text untouched) when h has no specialisation.
template <bool PCG>
int launch_elem_fast(const StripArgs<float>& args, const Kpair<float>* kp, cudaStream_t s) {
  switch (args.m.h) {
    case 1: return launch_e<1, PCG>(args, kp, s);
    case 2: return launch_e<2, PCG>(args, kp, s);
    case 3: return launch_e<3, PCG>(args, kp, s);
    case 4: return launch_e<4, PCG>(args, kp, s);
  }
  return VDVC_ERR_UNSUPPORTED;
}

template int launch_elem_fast<false>(const StripArgs<float>&, const Kpair<float>*, cudaStream_t);
template int launch_elem_fast<true>(const StripArgs<float>&, const Kpair<float>*, cudaStream_t);

}  // namespace vdvc
