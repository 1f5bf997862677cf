// Float32 Hessian element pass (H v and its PCG form) specialised on a
// compile-time element edge H.  Same strip decomposition and results as
// k_strip<float, kModeHv> (strip.cu); the specialisation is about issue
// rate: with H known, the voxel loop along y is fully unrolled, the shape
// function weights phi_1(qy) = qy/H are constants, the outer-face weight of
// the first and last voxel plane is applied once per block instead of being
// tested per voxel, and all H (or H+1) rows of a voxel column are loaded
// back to back, which keeps 4(H+1) independent loads in flight per thread.
#include "ops.cuh"
#include "pcg.cuh"

namespace vdvc {

template <int H, bool PCG>
__global__ void __launch_bounds__(128, 8) k_strip_hv_fast(const StripArgs<float> a, const Kpair<float>* __restrict__ kp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int EX = (H >= 128) ? 1 : 128 / H;
  const int nthr = blockDim.x;
  float* s_acc = (float*)smem_raw;            // nthr*25
  // Unique nodes of the strip: 4 node lines (dy,dz) of EX+1 nodes x 3
  // components, so adjacent elements share their common face instead of each
  // loading all 8 corners.  Corner (dx,dy,dz) of strip element e is
  // s_v[((dy*2+dz)*NL + e + dx)*3 + c].
  constexpr int NL = EX + 1;
  float* s_v = s_acc + (size_t)nthr * 25;     // 12*NL
  float* s_w = s_v + 12 * NL;                 // 12*NL
  float* s_K = s_w + 12 * NL;                 // 2*576
  const Mesh& m = a.m;

  if constexpr (PCG) {
    if (a.st->done) return;
  }
  const int t = threadIdx.x;
  const int el = t / H, qx = t - el * H;
  const int i0 = blockIdx.x * EX, i = i0 + el;
  const int j = blockIdx.y, k = blockIdx.z;
  const int nel = min(EX, m.Nx - i0);
  const bool active = el < nel;
  const bool y_last = (j == m.Ny - 1), z_last = (k == m.Nz - 1);
  const int nz_e = H + (z_last ? 1 : 0);
  const int ncol = active ? ((i == m.Nx - 1 && qx == H - 1) ? 2 : 1) : 0;
  // outer-face weight of the first voxel row of this element row (y) -- the
  // extra last row (y_last) is the other outer face and gets 1/2 as well
  const float wy_first = (j == 0) ? 0.5f : 1.f;

  {
    float beta = 0.f;
    if constexpr (PCG) beta = (float)a.st->beta;
    const int line = (nel + 1) * 3;
    for (int idx = t; idx < 4 * line; idx += nthr) {
      const int dyz = idx / line, rem = idx - dyz * line, ii = rem / 3, c = rem - ii * 3;
      const long long node = (long long)(i0 + ii) + (long long)(j + (dyz >> 1)) * m.Nnx +
                             (long long)(k + (dyz & 1)) * m.NnxNny;
      float val = a.v[3 * node + c];
      if constexpr (PCG) val = val + beta * a.p_old[3 * node + c];
      s_v[(dyz * NL + ii) * 3 + c] = val;
      if (a.nreg == 2) s_w[(dyz * NL + ii) * 3 + c] = a.w[3 * node + c];
    }
    // dense K rows are staged only when needed: K1 unless it is the
    // block-diagonal Laplacian (then its 8x8 block rides in the parameters)
    if (a.nreg >= 1) {
      const int k_lo = a.k1_blockdiag ? 576 : 0, k_hi = 576 * a.nreg;
      for (int q = k_lo + t; q < k_hi; q += nthr) s_K[q] = (q < 576) ? kp->K1[q] : kp->K2[q - 576];
    }
    for (int r = 0; r < 25; ++r) s_acc[t * 25 + r] = 0.f;
  }
  __syncthreads();

  const long long row_stride = m.Nvx;  // voxels between consecutive y rows
  for (int col = 0; col < ncol; ++col) {
    const int qxc = qx + col;
    const long long x = (long long)i * H + qxc;
    const float fx1 = (float)qxc / (float)H, fx0 = 1.f - fx1;
    const float wx = (x == 0 || x == (long long)m.Nvx - 1) ? 0.5f : 1.f;
    float ux[12];
#pragma unroll
    for (int ay = 0; ay < 2; ++ay)
#pragma unroll
      for (int az = 0; az < 2; ++az)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          ux[ay * 6 + az * 3 + c] = fx0 * s_v[((ay * 2 + az) * NL + el) * 3 + c] +
                                    fx1 * s_v[((ay * 2 + az) * NL + el + 1) * 3 + c];
    float acc[12];
#pragma unroll
    for (int r = 0; r < 12; ++r) acc[r] = 0.f;

#pragma unroll 1
    for (int qz = 0; qz <= H; ++qz) {
      if (qz == H && !z_last) break;  // the outer-face plane exists on the last element layer only
      const float fz1 = (float)qz / (float)H, fz0 = 1.f - fz1;
      const long long vz = (long long)k * H + qz;
      const float wz = (vz == 0 || vz == m.Nvz - 1) ? 0.5f : 1.f;
      float u0[3], du[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        u0[c] = fz0 * ux[0 * 6 + 0 * 3 + c] + fz1 * ux[0 * 6 + 1 * 3 + c];
        du[c] = fz0 * ux[1 * 6 + 0 * 3 + c] + fz1 * ux[1 * 6 + 1 * 3 + c] - u0[c];
      }
      const long long v0 = x + (long long)j * H * row_stride + vz * m.NvxNvy;
      const float* __restrict__ gp = a.grad + 3 * v0;
      const uint8_t* __restrict__ mp = a.mask + v0;
      // load the column's H rows (plus the outer-face row) up front
      float g[H + 1][3];
      bool mk[H + 1];
#pragma unroll
      for (int qy = 0; qy < H; ++qy) {
        g[qy][0] = __ldg(gp + 3 * qy * row_stride + 0);
        g[qy][1] = __ldg(gp + 3 * qy * row_stride + 1);
        g[qy][2] = __ldg(gp + 3 * qy * row_stride + 2);
        mk[qy] = __ldg(mp + qy * row_stride) != 0;
      }
      if (y_last) {
        g[H][0] = __ldg(gp + 3 * H * row_stride + 0);
        g[H][1] = __ldg(gp + 3 * H * row_stride + 1);
        g[H][2] = __ldg(gp + 3 * H * row_stride + 2);
        mk[H] = __ldg(mp + H * row_stride) != 0;
      } else {
        g[H][0] = g[H][1] = g[H][2] = 0.f;
        mk[H] = false;
      }
      float S[3] = {0.f, 0.f, 0.f}, S1[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int qy = 0; qy <= H; ++qy) {
        const float fy1 = (float)qy / (float)H;
        const float uu0 = u0[0] + fy1 * du[0], uu1 = u0[1] + fy1 * du[1], uu2 = u0[2] + fy1 * du[2];
        float d = g[qy][0] * uu0 + g[qy][1] * uu1 + g[qy][2] * uu2;
        if (qy == 0) d *= wy_first;
        if (qy == H) d *= 0.5f;  // only loaded (non-zero) on the outer face
        d = mk[qy] ? d : 0.f;
        const float t0 = d * g[qy][0], t1 = d * g[qy][1], t2 = d * g[qy][2];
        S[0] += t0;
        S[1] += t1;
        S[2] += t2;
        if (qy > 0) {
          S1[0] += fy1 * t0;
          S1[1] += fy1 * t1;
          S1[2] += fy1 * t2;
        }
      }
      const float gz0 = wz * fz0, gz1 = wz * fz1;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float s0 = S[c] - S1[c];
        acc[0 * 6 + 0 * 3 + c] += gz0 * s0;
        acc[0 * 6 + 1 * 3 + c] += gz1 * s0;
        acc[1 * 6 + 0 * 3 + c] += gz0 * S1[c];
        acc[1 * 6 + 1 * 3 + c] += gz1 * S1[c];
      }
    }
    const float gx0 = wx * fx0, gx1 = wx * fx1;
#pragma unroll
    for (int r = 0; r < 12; ++r) {
      s_acc[t * 25 + r] += gx0 * acc[r];
      s_acc[t * 25 + 12 + r] += gx1 * acc[r];
    }
  }
  __syncthreads();

  const long long e_base = (long long)i0 + (long long)j * m.Nx + (long long)k * m.Nx * m.Ny;
  for (int idx = t; idx < nel * 24; idx += nthr) {
    const int r = idx / nel, e = idx - r * nel;
    const int ax = r / 12, ay = (r / 6) & 1, az = (r / 3) & 1, c = r % 3;
    const int row = 3 * corner_of(ax, ay, az) + c;
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < H; ++q) s += s_acc[(e * H + q) * 25 + r];
    if (a.nreg >= 1) {
      const int acorner = corner_of(ax, ay, az);
      float k1 = 0.f;
      if (a.k1_blockdiag) {
        // K1 couples equal displacement components only (vector Laplacian):
        // its 8x8 block, read from the kernel parameters (warp-uniform)
#pragma unroll
        for (int b = 0; b < 8; ++b)
          k1 += a.L8[acorner * 8 + b] *
                s_v[(((corner_dy(b) << 1) | corner_dz(b)) * NL + e + corner_dx(b)) * 3 + c];
      } else {
#pragma unroll 8
        for (int b = 0; b < 24; ++b) {
          const int bn = b / 3;
          k1 += s_K[row * 24 + b] * s_v[(((corner_dy(bn) << 1) | corner_dz(bn)) * NL + e + corner_dx(bn)) * 3 + b % 3];
        }
      }
      s += a.c1 * k1;
      if (a.nreg == 2) {
        float k2 = 0.f;
#pragma unroll 8
        for (int b = 0; b < 24; ++b) {
          const int bn = b / 3;
          k2 += s_K[576 + row * 24 + b] *
                s_w[(((corner_dy(bn) << 1) | corner_dz(bn)) * NL + e + corner_dx(bn)) * 3 + b % 3];
        }
        s += a.c2 * k2;
      }
    }
    a.evA[(long long)row * m.Ne + e_base + e] = s;
  }
}

template <int H, bool PCG>
static int launch_h(const StripArgs<float>& args, const Kpair<float>* kp, cudaStream_t s) {
  constexpr int EX = (H >= 128) ? 1 : 128 / H;
  const int threads = (EX * H + 31) / 32 * 32;
  const size_t smem = ((size_t)threads * 25 + 24 * (EX + 1) + 1152) * sizeof(float);
  if (smem > 48 * 1024)
    if (int st = ensure_dyn_smem((const void*)k_strip_hv_fast<H, PCG>, (int)smem)) return st;
  dim3 grid((args.m.Nx + EX - 1) / EX, args.m.Ny, args.m.Nz);
  StripArgs<float> a = args;
  a.EX = EX;
  k_strip_hv_fast<H, PCG><<<grid, threads, smem, s>>>(a, kp);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

// Returns VDVC_ERR_UNSUPPORTED (without touching the error text) when no
// specialisation exists for this h; the caller then uses the generic pass.
template <bool PCG>
int launch_strip_fast(const StripArgs<float>& args, const Kpair<float>* kp, cudaStream_t s) {
  switch (args.m.h) {
    case 6: return launch_h<6, PCG>(args, kp, s);
    case 8: return launch_h<8, PCG>(args, kp, s);
    case 12: return launch_h<12, PCG>(args, kp, s);
    case 16: return launch_h<16, PCG>(args, kp, s);
  }
  return VDVC_ERR_UNSUPPORTED;
}

template int launch_strip_fast<false>(const StripArgs<float>&, const Kpair<float>*, cudaStream_t);
template int launch_strip_fast<true>(const StripArgs<float>&, const Kpair<float>*, cudaStream_t);

}  // namespace vdvc
