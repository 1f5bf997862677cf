// Float32 right-hand-side pass of the Gauss-Newton iteration (residual, b
// and optionally diag H) specialised on a compile-time element edge H.
// Same strip decomposition, arithmetic and outputs as k_strip<float,
// kModeB | kModeRes [| kModeDiag]> (strip.cu): with H known, the loops are
// unrolled, the shape-function weights are constants, the voxel rows are
// processed in groups whose loads (gradient, f, g(x+u) and the two masks:
// 7 per row) are issued together, and the register budget is capped at 80
// so that 6 blocks of 128 threads stay resident per SM.  Element edges up
// to 4 voxels take a thread-per-element form of the same pass (k_elem_rhs).
//
// Residual (engine/correlate_gpu.py:1091-1105):
//   res = (f - mean0) - (std0/std1)(g - mean1) on the b mask, 0 elsewhere,
// in the reference's float32 operation order (round-to-nearest intrinsics,
// no contraction); b accumulates w m res N (x) grad as in compute_b_gpu
// (:341-378), diag H accumulates w m N^2 grad_k^2 (kernels_dvc.py:509-543).
// The displayed std(res) sums go through a deterministic grid reduction.
#include <stdlib.h>

#include "ops.cuh"

namespace vdvc {

__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }

// Residual scalars from the stats of g over the b mask: mean of g, -std0/sd
// and the reference mean, computed once per block by thread 0 (float64
// division and square root run on GB300's narrow FP64 pipe) and shared.
// The whole block must call this.
__device__ __forceinline__ void residual_scalars(const StripArgs<float>& a, float& gm, float& ratio, float& mean0) {
  __shared__ float s_sc[3];
  if (threadIdx.x == 0) {
    const double c = a.gstats[0];
    double mean = 0.0, sd = 0.0;
    if (c >= 1.0) {
      mean = a.gstats[1] / c;
      const double var = a.gstats[2] / c - mean * mean;
      sd = sqrt(var > 0.0 ? var : 0.0);
    }
    if (sd == 0.0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) *a.status = VDVC_ERR_ZERO_DIVISION;
    s_sc[0] = (float)mean;
    s_sc[1] = (float)(-(a.std0 / sd));
    s_sc[2] = (float)a.mean0;
  }
  __syncthreads();
  gm = s_sc[0];
  ratio = s_sc[1];
  mean0 = s_sc[2];
}

template <int H, bool DG>
__global__ void __launch_bounds__(128, 6) k_strip_rhs_fast(const StripArgs<float> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int EX = (H >= 128) ? 1 : 128 / H;
  constexpr int RB = DG ? 2 : 4;  // voxel rows loaded per group
  const int nthr = blockDim.x;
  float* s_accA = (float*)smem_raw;           // nthr*25
  float* s_accD = s_accA + (size_t)nthr * 25;  // nthr*25 (diag)
  __shared__ double s_red[4];
  const Mesh& m = a.m;

  const int t = threadIdx.x;
  const int el = t / H, qx = t - el * H;
  const int i0 = blockIdx.x * EX, i = i0 + el;
  const int j = blockIdx.y, k = blockIdx.z;
  const int nel = min(EX, m.Nx - i0);
  const bool active = el < nel;
  const bool y_last = (j == m.Ny - 1), z_last = (k == m.Nz - 1);
  const int ncol = active ? ((i == m.Nx - 1 && qx == H - 1) ? 2 : 1) : 0;
  const float wy_first = (j == 0) ? 0.5f : 1.f;

  // residual scalars from the stats of g over the b mask
  float gm, ratio, mean0;
  residual_scalars(a, gm, ratio, mean0);
  for (int r = 0; r < 25; ++r) {
    s_accA[t * 25 + r] = 0.f;
    if constexpr (DG) s_accD[t * 25 + r] = 0.f;
  }
  __syncthreads();

  double dsum[3] = {0.0, 0.0, 0.0};
  float dcol[3] = {0.f, 0.f, 0.f};  // float over the thread's columns (<= 2 x 81 voxels), float64 once
  const long long row_stride = m.Nvx;
  for (int col = 0; col < ncol; ++col) {
    const int qxc = qx + col;
    const long long x = (long long)i * H + qxc;
    const float fx1 = (float)qxc / (float)H, fx0 = 1.f - fx1;
    const int mx = (qxc == 0 && i > 0) ? 2 : 1;
    const float wx = (x == 0 || x == (long long)m.Nvx - 1) ? 0.5f : 1.f;
    float accA[12], accD[12];
#pragma unroll
    for (int r = 0; r < 12; ++r) accA[r] = accD[r] = 0.f;

#pragma unroll 1
    for (int qz = 0; qz <= H; ++qz) {
      if (qz == H && !z_last) break;
      const float fz1 = (float)qz / (float)H, fz0 = 1.f - fz1;
      const int mxz = mx * ((qz == 0 && k > 0) ? 2 : 1);
      const long long vz = (long long)k * H + qz;
      const float wz = (vz == 0 || vz == m.Nvz - 1) ? 0.5f : 1.f;
      const long long v0 = x + (long long)j * H * row_stride + vz * m.NvxNvy;
      const int nrows = H + (y_last ? 1 : 0);
      float S[3] = {0.f, 0.f, 0.f}, S1[3] = {0.f, 0.f, 0.f};
      float D0[3] = {0.f, 0.f, 0.f}, D1[3] = {0.f, 0.f, 0.f};
      float ds0 = 0.f, ds1 = 0.f, ds2 = 0.f;
      // rows in groups of RB: the group's loads are issued back to back
#pragma unroll 1
      for (int q0 = 0; q0 < nrows; q0 += RB) {
        float g[RB][3], fv[RB], gv[RB];
        bool mk[RB], lv[RB];
#pragma unroll
        for (int u = 0; u < RB; ++u) {
          if (q0 + u < nrows) {
            const long long vv = v0 + (long long)(q0 + u) * row_stride;
            g[u][0] = __ldg(a.grad + 3 * vv);
            g[u][1] = __ldg(a.grad + 3 * vv + 1);
            g[u][2] = __ldg(a.grad + 3 * vv + 2);
            fv[u] = __ldg(a.f + vv);
            gv[u] = __ldg(a.gvals + vv);
            mk[u] = __ldg(a.mask + vv) != 0;
            lv[u] = __ldg(a.live + vv) != 0;
          } else {
            g[u][0] = g[u][1] = g[u][2] = fv[u] = gv[u] = 0.f;
            mk[u] = lv[u] = false;
          }
        }
#pragma unroll
        for (int u = 0; u < RB; ++u) {
          const int qy = q0 + u;
          if (qy >= nrows) break;
          const float fy1 = (float)qy / (float)H;
          const float wy = (qy == 0) ? wy_first : (qy == H ? 0.5f : 1.f);
          const float fc = rsub(fv[u], mean0);
          const float rv = radd(rmul(rsub(gv[u], gm), ratio), fc);
          float r = mk[u] ? rv : 0.f;
          a.res_out[v0 + (long long)qy * row_stride] = r;
          if (lv[u]) {
            const float mf = (float)(mxz * ((qy == 0 && j > 0) ? 2 : 1));
            ds0 += mf;
            ds1 += mf * r;
            ds2 += mf * r * r;
          }
          r *= wy;
          const float t0 = r * g[u][0], t1 = r * g[u][1], t2 = r * g[u][2];
          S[0] += t0; S[1] += t1; S[2] += t2;
          S1[0] += fy1 * t0; S1[1] += fy1 * t1; S1[2] += fy1 * t2;
          if constexpr (DG) {
            const float fy0 = 1.f - fy1;
            const float w0 = wy * fy0 * fy0, w1 = wy * fy1 * fy1;
            const float d0 = mk[u] ? g[u][0] * g[u][0] : 0.f;
            const float d1 = mk[u] ? g[u][1] * g[u][1] : 0.f;
            const float d2 = mk[u] ? g[u][2] * g[u][2] : 0.f;
            D0[0] += w0 * d0; D0[1] += w0 * d1; D0[2] += w0 * d2;
            D1[0] += w1 * d0; D1[1] += w1 * d1; D1[2] += w1 * d2;
          }
        }
      }
      dcol[0] += ds0;
      dcol[1] += ds1;
      dcol[2] += ds2;
      const float gz0 = wz * fz0, gz1 = wz * fz1;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float s0 = S[c] - S1[c];
        accA[0 * 6 + 0 * 3 + c] += gz0 * s0;
        accA[0 * 6 + 1 * 3 + c] += gz1 * s0;
        accA[1 * 6 + 0 * 3 + c] += gz0 * S1[c];
        accA[1 * 6 + 1 * 3 + c] += gz1 * S1[c];
      }
      if constexpr (DG) {
        const float z0 = wz * fz0 * fz0, z1 = wz * fz1 * fz1;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          accD[0 * 6 + 0 * 3 + c] += z0 * D0[c];
          accD[0 * 6 + 1 * 3 + c] += z1 * D0[c];
          accD[1 * 6 + 0 * 3 + c] += z0 * D1[c];
          accD[1 * 6 + 1 * 3 + c] += z1 * D1[c];
        }
      }
    }
    const float gx0 = wx * fx0, gx1 = wx * fx1;
#pragma unroll
    for (int r = 0; r < 12; ++r) {
      s_accA[t * 25 + r] += gx0 * accA[r];
      s_accA[t * 25 + 12 + r] += gx1 * accA[r];
    }
    if constexpr (DG) {
      const float x0 = wx * fx0 * fx0, x1 = wx * fx1 * fx1;
#pragma unroll
      for (int r = 0; r < 12; ++r) {
        s_accD[t * 25 + r] += x0 * accD[r];
        s_accD[t * 25 + 12 + r] += x1 * accD[r];
      }
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
    for (int q = 0; q < H; ++q) s += s_accA[(e * H + q) * 25 + r];
    a.evA[(long long)row * m.Ne + e_base + e] = s;
    if constexpr (DG) {
      float d = 0.f;
#pragma unroll
      for (int q = 0; q < H; ++q) d += s_accD[(e * H + q) * 25 + r];
      a.evD[(long long)row * m.Ne + e_base + e] = d;
    }
  }

  for (int q = 0; q < 3; ++q) dsum[q] += dcol[q];
  double b3[3], out[3];
  for (int q = 0; q < 3; ++q) b3[q] = block_sum(dsum[q], s_red);
  if (grid_reduce_sum<3>(a.red, b3, out, s_red) && t == 0)
    for (int q = 0; q < 3; ++q) a.dstats[q] = out[q];
}

// Thread-per-element form of the same pass for small element edges (H <= 4),
// where an element's few voxels cannot amortise a strip block's staging and
// shared-memory reduction (the Hessian pass splits the same way,
// elem_fast.cu).  Element (i,j,k) owns the voxels of elem_fast.cu; a thread
// keeps its element's 24 b sums (and 24 diag sums) in registers, walks the
// voxels row by row (x fastest) and writes the sums coalesced to [24][Ne].
// Residual values are computed exactly as above; the per-element float
// partials of the displayed sums are folded into float64 per element.
template <int H, bool DG>
__global__ void __launch_bounds__(256) k_elem_rhs(const StripArgs<float> a) {
  __shared__ double s_red[8];
  const Mesh& m = a.m;
  float gm, ratio, mean0;
  residual_scalars(a, gm, ratio, mean0);
  double dsum[3] = {0.0, 0.0, 0.0};
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m.Ne;
       e += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    elem_ijk(m, e, i, j, k);
    float o[2][2][2][3], od[2][2][2][3];
#pragma unroll
    for (int q = 0; q < 24; ++q) {
      (&o[0][0][0][0])[q] = 0.f;
      (&od[0][0][0][0])[q] = 0.f;
    }
    const bool x_last = (i == m.Nx - 1), y_last = (j == m.Ny - 1), z_last = (k == m.Nz - 1);
    const float wx_first = (i == 0) ? 0.5f : 1.f;
    const float wy_first = (j == 0) ? 0.5f : 1.f;
    const float wz_first = (k == 0) ? 0.5f : 1.f;
    float ds0 = 0.f, ds1 = 0.f, ds2 = 0.f;
#pragma unroll(H <= 2 ? H + 1 : 1)
    for (int qz = 0; qz <= H; ++qz) {
      if (qz == H && !z_last) break;
      const float fz1 = (float)qz / (float)H, fz0 = 1.f - fz1;
      const float wz = (qz == 0) ? wz_first : (qz == H ? 0.5f : 1.f);
      const int mz = (qz == 0 && k > 0) ? 2 : 1;
#pragma unroll
      for (int qy = 0; qy <= H; ++qy) {
        if (qy == H && !y_last) break;
        const float fy1 = (float)qy / (float)H, fy0 = 1.f - fy1;
        const float wyz = wz * ((qy == 0) ? wy_first : (qy == H ? 0.5f : 1.f));
        const int myz = mz * ((qy == 0 && j > 0) ? 2 : 1);
        const long long vrow =
            (long long)i * H + (long long)(j * H + qy) * m.Nvx + (long long)(k * H + qz) * m.NvxNvy;
        float A[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
        float Dd[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
        for (int qx = 0; qx <= H; ++qx) {
          if (qx == H && !x_last) break;
          const float fx1 = (float)qx / (float)H, fx0 = 1.f - fx1;
          const float w = wyz * ((qx == 0) ? wx_first : (qx == H ? 0.5f : 1.f));
          const long long vv = vrow + qx;
          const float g0 = __ldg(a.grad + 3 * vv), g1 = __ldg(a.grad + 3 * vv + 1), g2 = __ldg(a.grad + 3 * vv + 2);
          const float fv = __ldg(a.f + vv), gv = __ldg(a.gvals + vv);
          const bool mk = __ldg(a.mask + vv) != 0, lv = __ldg(a.live + vv) != 0;
          const float fc = rsub(fv, mean0);
          const float rv = radd(rmul(rsub(gv, gm), ratio), fc);
          const float r = mk ? rv : 0.f;
          a.res_out[vv] = r;
          if (lv) {
            const float mf = (float)(myz * ((qx == 0 && i > 0) ? 2 : 1));
            ds0 += mf;
            ds1 += mf * r;
            ds2 += mf * r * r;
          }
          const float rw = r * w;
          const float t0 = rw * g0, t1 = rw * g1, t2 = rw * g2;
          A[0][0] += fx0 * t0; A[0][1] += fx0 * t1; A[0][2] += fx0 * t2;
          A[1][0] += fx1 * t0; A[1][1] += fx1 * t1; A[1][2] += fx1 * t2;
          if constexpr (DG) {
            const float w0 = w * fx0 * fx0, w1 = w * fx1 * fx1;
            const float d0 = mk ? g0 * g0 : 0.f, d1 = mk ? g1 * g1 : 0.f, d2 = mk ? g2 * g2 : 0.f;
            Dd[0][0] += w0 * d0; Dd[0][1] += w0 * d1; Dd[0][2] += w0 * d2;
            Dd[1][0] += w1 * d0; Dd[1][1] += w1 * d1; Dd[1][2] += w1 * d2;
          }
        }
#pragma unroll
        for (int dx = 0; dx < 2; ++dx)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            o[0][0][dx][c] += (fz0 * fy0) * A[dx][c];
            o[0][1][dx][c] += (fz0 * fy1) * A[dx][c];
            o[1][0][dx][c] += (fz1 * fy0) * A[dx][c];
            o[1][1][dx][c] += (fz1 * fy1) * A[dx][c];
            if constexpr (DG) {
              od[0][0][dx][c] += (fz0 * fz0 * fy0 * fy0) * Dd[dx][c];
              od[0][1][dx][c] += (fz0 * fz0 * fy1 * fy1) * Dd[dx][c];
              od[1][0][dx][c] += (fz1 * fz1 * fy0 * fy0) * Dd[dx][c];
              od[1][1][dx][c] += (fz1 * fz1 * fy1 * fy1) * Dd[dx][c];
            }
          }
      }
    }
    dsum[0] += (double)ds0;
    dsum[1] += (double)ds1;
    dsum[2] += (double)ds2;
#pragma unroll
    for (int ca = 0; ca < 8; ++ca) {
      const int adx = corner_dx(ca), ady = corner_dy(ca), adz = corner_dz(ca);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        a.evA[(long long)(3 * ca + c) * m.Ne + e] = o[adz][ady][adx][c];
        if constexpr (DG) a.evD[(long long)(3 * ca + c) * m.Ne + e] = od[adz][ady][adx][c];
      }
    }
  }
  double b3[3], out[3];
  for (int q = 0; q < 3; ++q) b3[q] = block_sum(dsum[q], s_red);
  if (grid_reduce_sum<3>(a.red, b3, out, s_red) && threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) a.dstats[q] = out[q];
}

// Element edges up to this one take the thread-per-element form.
constexpr int kElemRhsMaxH = 4;

// Without the diagonal (the element-Hessian forms, whose diagonal comes
// from the element Hessians) the thread-per-element form also serves h = 8
// (128 registers; measured on the 513^3 learned + precision solve, 3 GN
// rhs calls: 25.8 -> 25.3 ms).  With the diagonal its 48 register sums
// take 216 registers; that form keeps the strip kernel.
constexpr int kElemRhsMaxHNoDiag = 8;

template <int H, bool DG>
static int launch_rh(const StripArgs<float>& args, cudaStream_t s) {
  if constexpr (H <= kElemRhsMaxH || (!DG && H == kElemRhsMaxHNoDiag)) {
    // at most kReduceBlocks blocks: the reduction partials hold that many
    long long nb = (args.m.Ne + 255) / 256;
    if (nb > kReduceBlocks) nb = kReduceBlocks;
    k_elem_rhs<H, DG><<<(unsigned)nb, 256, 0, s>>>(args);
    VDVC_LAUNCHED();
    return VDVC_OK;
  } else {
    constexpr int EX = (H >= 128) ? 1 : 128 / H;
    const int threads = (EX * H + 31) / 32 * 32;
    const size_t smem = (size_t)threads * 25 * (DG ? 2 : 1) * sizeof(float);
    dim3 grid((args.m.Nx + EX - 1) / EX, args.m.Ny, args.m.Nz);
    k_strip_rhs_fast<H, DG><<<grid, threads, smem, s>>>(args);
    VDVC_LAUNCHED();
    return VDVC_OK;
  }
}

// VDVC_ERR_UNSUPPORTED (error text untouched) when h has no specialisation.
template <bool DG>
int launch_rhs_fast(const StripArgs<float>& args, cudaStream_t s) {
  switch (args.m.h) {
    case 1: return launch_rh<1, DG>(args, s);
    case 2: return launch_rh<2, DG>(args, s);
    case 3: return launch_rh<3, DG>(args, s);
    case 4: return launch_rh<4, DG>(args, s);
    case 6: return launch_rh<6, DG>(args, s);
    case 8: return launch_rh<8, DG>(args, s);
    case 12: return launch_rh<12, DG>(args, s);
    case 16: return launch_rh<16, DG>(args, s);
  }
  return VDVC_ERR_UNSUPPORTED;
}

template int launch_rhs_fast<false>(const StripArgs<float>&, cudaStream_t);
template int launch_rhs_fast<true>(const StripArgs<float>&, cudaStream_t);

}  // namespace vdvc
