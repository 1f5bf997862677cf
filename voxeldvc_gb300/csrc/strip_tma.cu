// Float32 Hessian element pass (H v, optionally the PCG form with the fused
// regularizer) with TMA staging: the strip decomposition of strip.cuh, but
// each voxel plane z of the strip -- its (h or h+1) rows of gradient and
// mask -- is fetched into shared memory by bulk copies (cp.async.bulk) issued
// by one thread, into a two-stage ring tracked by mbarriers.  While the CTA
// works on plane z, plane z+1 is in flight: tens of kilobytes per SM in
// flight with a few hundred threads, instead of a handful of loads per
// thread.
//
// Row copies start at the 16-byte boundary at or below the row start (the
// voxel grid has odd row lengths, so rows are not 16-byte aligned) and end
// at the boundary at or above the row end, clamped to the last 16-byte
// boundary inside the buffer; the few voxels of a row that fall past the
// clamp (only ever the last row of the volume) are read from global memory.
#include "ops.cuh"
#include "pcg.cuh"
#include "tma.cuh"

namespace vdvc {

struct TmaGeom {
  int L_max;        // longest staged row, voxels (EX*h + 1)
  int rows;         // rows per plane, h + 1
  int gpitch;       // bytes per staged gradient row
  int mpitch;       // bytes per staged mask row
  int stage_bytes;  // one plane
};

inline TmaGeom tma_geom(int h, int EX) {
  TmaGeom g;
  g.L_max = EX * h + 1;
  g.rows = h + 1;
  g.gpitch = (12 * g.L_max + 30 + 15) & ~15;
  g.mpitch = (g.L_max + 30 + 15) & ~15;
  g.stage_bytes = g.rows * (g.gpitch + g.mpitch);
  return g;
}

// [0,16) mbarriers | stage 0 | stage 1 | accA (nthr*25 f) | s_v | s_w | phi | K pair
inline size_t tma_smem_bytes(int h, int EX, int nthr) {
  TmaGeom g = tma_geom(h, EX);
  size_t b = 128 + 2 * (size_t)g.stage_bytes;
  b += ((size_t)nthr * 25 + (size_t)EX * 48 + (size_t)((h + 2) & ~1) + 1152) * sizeof(float);
  return b;
}

struct RowSpan {
  long long a0;   // first byte copied (16-aligned)
  int bytes;      // bytes copied (multiple of 16)
  int off;        // byte offset of the row's first voxel inside the copy
};

__device__ __forceinline__ RowSpan row_span(long long vidx, int esize, int L, long long total_bytes) {
  RowSpan r;
  const long long s = vidx * esize;
  r.a0 = s & ~15LL;
  long long a1 = (s + (long long)esize * L + 15) & ~15LL;
  const long long lim = total_bytes & ~15LL;
  if (a1 > lim) a1 = lim;
  r.bytes = a1 > r.a0 ? (int)(a1 - r.a0) : 0;
  r.off = (int)(s - r.a0);
  return r;
}

template <bool PCG>
__global__ void __launch_bounds__(128) k_strip_tma(const StripArgs<float> a, const Kpair<float>* __restrict__ kp,
                                                   const TmaGeom G) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bars = (uint64_t*)smem_raw;
  unsigned char* stage0 = smem_raw + 128;
  float* s_acc = (float*)(stage0 + 2 * (size_t)G.stage_bytes);
  const int nthr = blockDim.x;
  const Mesh& m = a.m;
  const int h = m.h, EX = a.EX;
  float* s_v = s_acc + (size_t)nthr * 25;
  float* s_w = s_v + (size_t)EX * 24;
  float* s_phi = s_w + (size_t)EX * 24;
  float* s_K = s_phi + ((h + 2) & ~1);
  __shared__ int s_fail;

  if constexpr (PCG) {
    if (a.st->done) return;
  }
  const int t = threadIdx.x;
  const int el = t / h, qx = t - el * h;
  const int i0 = blockIdx.x * EX, i = i0 + el;
  const int j = blockIdx.y, k = blockIdx.z;
  const int nel = min(EX, m.Nx - i0);
  const bool last_strip = (i0 + nel == m.Nx);
  const int L = nel * h + (last_strip ? 1 : 0);  // staged row length (voxels)
  const bool active = el < nel;
  const int ny_e = h + (j == m.Ny - 1), nz_e = h + (k == m.Nz - 1);
  const int ncol = active ? ((i == m.Nx - 1 && qx == h - 1) ? 2 : 1) : 0;
  const long long x0 = (long long)i0 * h;
  const long long gbytes = 12 * m.Nvox, mbytes = m.Nvox;

  // producer: stage plane qz of this strip into stage buffer sb
  auto issue = [&](int qz, int sb) {
    unsigned char* st = stage0 + (size_t)sb * G.stage_bytes;
    const long long vz = (long long)k * h + qz;
    uint32_t total = 0;
    for (int r = 0; r < ny_e; ++r) {
      const long long v = x0 + ((long long)j * h + r) * m.Nvx + vz * m.NvxNvy;
      total += row_span(v, 12, L, gbytes).bytes + row_span(v, 1, L, mbytes).bytes;
    }
    mbar_arrive_expect_tx(&bars[sb], total);
    for (int r = 0; r < ny_e; ++r) {
      const long long v = x0 + ((long long)j * h + r) * m.Nvx + vz * m.NvxNvy;
      const RowSpan g = row_span(v, 12, L, gbytes);
      const RowSpan mk = row_span(v, 1, L, mbytes);
      if (g.bytes) bulk_g2s(st + (size_t)r * G.gpitch, (const unsigned char*)a.grad + g.a0, g.bytes, &bars[sb]);
      if (mk.bytes)
        bulk_g2s(st + (size_t)G.rows * G.gpitch + (size_t)r * G.mpitch, a.mask + mk.a0, mk.bytes, &bars[sb]);
    }
  };

  if (t == 0) {
    s_fail = 0;
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (t == 0) {
    issue(0, 0);
    if (nz_e > 1) issue(1, 1);
  }

  // prologue overlapping the first copies: phi table, nodal strip vector, K
  for (int q = t; q <= h; q += nthr) s_phi[q] = (float)q / (float)h;
  {
    float beta = 0.f;
    if constexpr (PCG) beta = (float)a.st->beta;
    for (int idx = t; idx < nel * 24; idx += nthr) {
      const int e = idx / 24, r = idx - e * 24, c = r % 3, cn = r / 3;
      const long long node = (long long)(i0 + e + corner_dx(cn)) + (long long)(j + corner_dy(cn)) * m.Nnx +
                             (long long)(k + corner_dz(cn)) * m.NnxNny;
      float val = a.v[3 * node + c];
      if constexpr (PCG) val = val + beta * a.p_old[3 * node + c];
      s_v[idx] = val;
      if (a.nreg == 2) s_w[idx] = a.w[3 * node + c];
    }
    if (a.nreg >= 1)
      for (int q = t; q < 576 * a.nreg; q += nthr) s_K[q] = (q < 576) ? kp->K1[q] : kp->K2[q - 576];
  }
  __syncthreads();

  // per-column constants
  float ux[2][12], acc[2][12], wxs[2], fx0s[2], fx1s[2];
  int ccol[2];
#pragma unroll
  for (int col = 0; col < 2; ++col) {
    const int qxc = qx + col;
    ccol[col] = el * h + qxc;
    const long long x = x0 + ccol[col];
    const float fx1 = (col < ncol) ? s_phi[qxc] : 0.f, fx0 = 1.f - fx1;
    fx0s[col] = fx0;
    fx1s[col] = fx1;
    wxs[col] = (x == 0 || x == (long long)m.Nvx - 1) ? 0.5f : 1.f;
#pragma unroll
    for (int ay = 0; ay < 2; ++ay)
#pragma unroll
      for (int az = 0; az < 2; ++az)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          ux[col][ay * 6 + az * 3 + c] =
              (col < ncol) ? fx0 * s_v[el * 24 + 3 * corner_of(0, ay, az) + c] +
                                 fx1 * s_v[el * 24 + 3 * corner_of(1, ay, az) + c]
                           : 0.f;
#pragma unroll
    for (int r = 0; r < 12; ++r) acc[col][r] = 0.f;
  }

  for (int qz = 0; qz < nz_e; ++qz) {
    const int sb = qz & 1;
    const uint32_t parity = (uint32_t)((qz >> 1) & 1);
    const bool ok = mbar_wait_bounded(&bars[sb], parity);
    if (__syncthreads_or(!ok)) {
      if (t == 0) {
        s_fail = 1;
        if (a.status) atomicExch(a.status, VDVC_ERR_CUDA);
        // let the copies still in flight land before the CTA exits
        mbar_wait_bounded(&bars[0], 0, 1 << 20);
        mbar_wait_bounded(&bars[1], 0, 1 << 20);
      }
      __syncthreads();
      return;
    }
    const unsigned char* st = stage0 + (size_t)sb * G.stage_bytes;
    const unsigned char* stm = st + (size_t)G.rows * G.gpitch;
    const float fz1 = s_phi[qz], fz0 = 1.f - fz1;
    const long long vz = (long long)k * h + qz;
    const float wz = (vz == 0 || vz == m.Nvz - 1) ? 0.5f : 1.f;
#pragma unroll
    for (int col = 0; col < 2; ++col) {
      if (col >= ncol) break;
      float u0[3], du[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        u0[c] = fz0 * ux[col][0 * 6 + 0 * 3 + c] + fz1 * ux[col][0 * 6 + 1 * 3 + c];
        du[c] = fz0 * ux[col][1 * 6 + 0 * 3 + c] + fz1 * ux[col][1 * 6 + 1 * 3 + c] - u0[c];
      }
      float S[3] = {0.f, 0.f, 0.f}, S1[3] = {0.f, 0.f, 0.f};
      const int cc = ccol[col];
#pragma unroll 4
      for (int qy = 0; qy < ny_e; ++qy) {
        const long long v = x0 + ((long long)j * h + qy) * m.Nvx + vz * m.NvxNvy;
        const RowSpan g = row_span(v, 12, L, gbytes);
        const int go = g.off + 12 * cc;
        float g0, g1, g2;
        if (go + 12 <= g.bytes) {
          const float* gp = (const float*)(st + (size_t)qy * G.gpitch + go);
          g0 = gp[0];
          g1 = gp[1];
          g2 = gp[2];
        } else {
          const float* gp = a.grad + 3 * (v + cc);
          g0 = gp[0];
          g1 = gp[1];
          g2 = gp[2];
        }
        const RowSpan mk = row_span(v, 1, L, mbytes);
        const int mo = mk.off + cc;
        const bool mm = (mo < mk.bytes) ? (stm[(size_t)qy * G.mpitch + mo] != 0) : (a.mask[v + cc] != 0);
        const float fy1 = s_phi[qy];
        const long long vy = (long long)j * h + qy;
        const float wy = (vy == 0 || vy == m.Nvy - 1) ? 0.5f : 1.f;
        const float uu0 = u0[0] + fy1 * du[0], uu1 = u0[1] + fy1 * du[1], uu2 = u0[2] + fy1 * du[2];
        float d = g0 * uu0 + g1 * uu1 + g2 * uu2;
        d = mm ? d * wy : 0.f;
        const float t0 = d * g0, t1 = d * g1, t2 = d * g2;
        S[0] += t0;
        S[1] += t1;
        S[2] += t2;
        S1[0] += fy1 * t0;
        S1[1] += fy1 * t1;
        S1[2] += fy1 * t2;
      }
      const float gz0 = wz * fz0, gz1 = wz * fz1;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float s0 = S[c] - S1[c];
        acc[col][0 * 6 + 0 * 3 + c] += gz0 * s0;
        acc[col][0 * 6 + 1 * 3 + c] += gz1 * s0;
        acc[col][1 * 6 + 0 * 3 + c] += gz0 * S1[c];
        acc[col][1 * 6 + 1 * 3 + c] += gz1 * S1[c];
      }
    }
    __syncthreads();  // every thread is done with stage sb
    if (t == 0 && qz + 2 < nz_e) {
      fence_proxy_async_smem();
      issue(qz + 2, sb);
    }
  }

  // column weights and the shared-memory reduction over each element's columns
#pragma unroll
  for (int r = 0; r < 25; ++r) s_acc[t * 25 + r] = 0.f;
#pragma unroll
  for (int col = 0; col < 2; ++col) {
    if (col >= ncol) break;
    const float gx0 = wxs[col] * fx0s[col], gx1 = wxs[col] * fx1s[col];
#pragma unroll
    for (int r = 0; r < 12; ++r) {
      s_acc[t * 25 + r] += gx0 * acc[col][r];
      s_acc[t * 25 + 12 + r] += gx1 * acc[col][r];
    }
  }
  __syncthreads();
  const long long e_base = (long long)i0 + (long long)j * m.Nx + (long long)k * m.Nx * m.Ny;
  for (int idx = t; idx < nel * 24; idx += nthr) {
    const int r = idx / nel, e = idx - r * nel;
    const int ax = r / 12, ay = (r / 6) & 1, az = (r / 3) & 1, c = r % 3;
    const int row = 3 * corner_of(ax, ay, az) + c;
    float s = 0.f;
    for (int q = 0; q < h; ++q) s += s_acc[(e * h + q) * 25 + r];
    if (a.nreg >= 1) {
      float k1 = 0.f;
#pragma unroll 8
      for (int b = 0; b < 24; ++b) k1 += s_K[row * 24 + b] * s_v[e * 24 + b];
      s += a.c1 * k1;
      if (a.nreg == 2) {
        float k2 = 0.f;
#pragma unroll 8
        for (int b = 0; b < 24; ++b) k2 += s_K[576 + row * 24 + b] * s_w[e * 24 + b];
        s += a.c2 * k2;
      }
    }
    a.evA[(long long)row * m.Ne + e_base + e] = s;
  }
}

template <bool PCG>
int launch_strip_tma(const StripArgs<float>& args, const Kpair<float>* kp, cudaStream_t s) {
  const Mesh& m = args.m;
  if (m.h > 128) return set_error(VDVC_ERR_UNSUPPORTED, "element edge h=%d > 128 not supported", m.h);
  StripShape sh = strip_shape(m.h);
  const TmaGeom G = tma_geom(m.h, sh.EX);
  const size_t smem = tma_smem_bytes(m.h, sh.EX, sh.threads);
  if (smem > 200 * 1024) return set_error(VDVC_ERR_UNSUPPORTED, "TMA strip stage of %zu bytes too large", smem);
  static bool attr_set = false;
  if (!attr_set) {
    VDVC_CUDA(cudaFuncSetAttribute(k_strip_tma<PCG>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr_set = true;
  }
  dim3 grid((m.Nx + sh.EX - 1) / sh.EX, m.Ny, m.Nz);
  StripArgs<float> a = args;
  a.EX = sh.EX;
  k_strip_tma<PCG><<<grid, sh.threads, smem, s>>>(a, kp, G);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

template int launch_strip_tma<false>(const StripArgs<float>&, const Kpair<float>*, cudaStream_t);
template int launch_strip_tma<true>(const StripArgs<float>&, const Kpair<float>*, cudaStream_t);

}  // namespace vdvc
