// Voxel passes that do not assemble element vectors:
//   * multiplicity-weighted masked statistics (masked_quadpoint_mean_std),
//   * g(x + u(x)) sampling with the dynamic mask (sample_deformed_field),
//     optionally with the GN stats of g over the b mask fused in,
//   * u(x) at every voxel (interp_field_vox).
// The sampling kernels use the element-strip decomposition of strip.cuh so
// the nodal field of a strip is staged once in shared memory and
// interpolated separably per voxel column; the GN form at element edges up
// to 4 voxels runs one thread per element instead (k_elem_sample).
#include <stdlib.h>
#include <type_traits>

#include "ops.cuh"

namespace vdvc {

// ---- masked statistics -----------------------------------------------------

// Rows (y,z) are distributed over blocks, x over threads, so the y/z
// multiplicities are uniform per row; per-row float partials are folded into
// float sums of 16 trips and then into float64 accumulators (GB300's FP64
// pipe is narrow).  A block takes kStatsRows of its rows per trip with every
// mask byte and value loaded before any is used (the loads of a row would
// otherwise wait on one another through the mask test).
constexpr int kStatsRows = 4;

template <typename T>
__global__ void __launch_bounds__(256) k_masked_stats(const T* __restrict__ field, const uint8_t* __restrict__ mask,
                                                      const Mesh m, GridReduce red, double* __restrict__ out3) {
  __shared__ double s_red[8];
  double acc[3] = {0.0, 0.0, 0.0};
  float fac[3] = {0.f, 0.f, 0.f};  // float sums of 16 trips per float64 add (narrow FP64 pipe)
  int trips = 0;
  const long long nrows = (long long)m.Nvy * m.Nvz;
  for (long long row0 = blockIdx.x; row0 < nrows; row0 += (long long)kStatsRows * gridDim.x) {
    float c[kStatsRows], s1[kStatsRows], s2[kStatsRows];
    int myz[kStatsRows];
    long long base[kStatsRows];
#pragma unroll
    for (int r = 0; r < kStatsRows; ++r) {
      const long long row = row0 + (long long)r * gridDim.x;
      const int y = (int)(row % m.Nvy), z = (int)(row / m.Nvy);
      myz[r] = row < nrows ? axis_multiplicity(y, m.h, m.Ny) * axis_multiplicity(z, m.h, m.Nz) : 0;
      base[r] = row < nrows ? row * m.Nvx : 0;
      c[r] = s1[r] = s2[r] = 0.f;
    }
    for (int x = threadIdx.x; x < m.Nvx; x += blockDim.x) {
      uint8_t mk[kStatsRows];
      float v[kStatsRows];
#pragma unroll
      for (int r = 0; r < kStatsRows; ++r) {
        mk[r] = myz[r] ? __ldg(mask + base[r] + x) : (uint8_t)0;
        v[r] = myz[r] ? (float)__ldg(field + base[r] + x) : 0.f;
      }
      const int mx = axis_multiplicity(x, m.h, m.Nx);
#pragma unroll
      for (int r = 0; r < kStatsRows; ++r) {
        if (!mk[r]) continue;
        const float mult = (float)(myz[r] * mx);
        c[r] += mult;
        s1[r] += mult * v[r];
        s2[r] += mult * v[r] * v[r];
      }
    }
#pragma unroll
    for (int r = 0; r < kStatsRows; ++r) {
      fac[0] += c[r];
      fac[1] += s1[r];
      fac[2] += s2[r];
    }
    if (++trips == 16) {
      for (int q = 0; q < 3; ++q) {
        acc[q] += fac[q];
        fac[q] = 0.f;
      }
      trips = 0;
    }
  }
  for (int q = 0; q < 3; ++q) acc[q] += fac[q];
  double b3[3], o3[3];
  for (int q = 0; q < 3; ++q) b3[q] = block_sum(acc[q], s_red);
  if (grid_reduce_sum<3>(red, b3, o3, s_red) && threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) out3[q] = o3[q];
}

// float64 fields keep float64 per-row partials.
template <>
__global__ void __launch_bounds__(256) k_masked_stats<double>(const double* __restrict__ field,
                                                              const uint8_t* __restrict__ mask, const Mesh m,
                                                              GridReduce red, double* __restrict__ out3) {
  __shared__ double s_red[8];
  double acc[3] = {0.0, 0.0, 0.0};
  const long long nrows = (long long)m.Nvy * m.Nvz;
  for (long long row = blockIdx.x; row < nrows; row += gridDim.x) {
    const int y = (int)(row % m.Nvy), z = (int)(row / m.Nvy);
    const int myz = axis_multiplicity(y, m.h, m.Ny) * axis_multiplicity(z, m.h, m.Nz);
    const long long base = row * m.Nvx;
    for (int x = threadIdx.x; x < m.Nvx; x += blockDim.x) {
      if (!mask[base + x]) continue;
      const double mult = (double)(myz * axis_multiplicity(x, m.h, m.Nx));
      const double v = field[base + x];
      acc[0] += mult;
      acc[1] += mult * v;
      acc[2] += mult * v * v;
    }
  }
  double b3[3], o3[3];
  for (int q = 0; q < 3; ++q) b3[q] = block_sum(acc[q], s_red);
  if (grid_reduce_sum<3>(red, b3, o3, s_red) && threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) out3[q] = o3[q];
}

// ---- deformed-image sampling ------------------------------------------------


// Trilinear sample at a clipped coordinate c in [0, n-1] per axis
// (scipy.ndimage.map_coordinates order=1, mode='nearest').
template <typename T>
__device__ __forceinline__ T trilinear(const T* __restrict__ g, int nx, int ny, int nz, T cx, T cy, T cz) {
  const T fx = tfloor(cx), fy = tfloor(cy), fz = tfloor(cz);
  const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
  const T tx = cx - fx, ty = cy - fy, tz = cz - fz;
  // 32-bit offsets (the launcher rejects volumes of 2^32 voxels or more);
  // the upper neighbour is the sample itself on the last plane of an axis
  const unsigned sy = (unsigned)nx, sz = (unsigned)nx * (unsigned)ny;
  const unsigned o = (unsigned)ix + (unsigned)iy * sy + (unsigned)iz * sz;
  const unsigned dx = ix < nx - 1 ? 1u : 0u, dy = iy < ny - 1 ? sy : 0u, dz = iz < nz - 1 ? sz : 0u;
  const T v000 = __ldg(g + o), v100 = __ldg(g + o + dx);
  const T v010 = __ldg(g + o + dy), v110 = __ldg(g + o + dy + dx);
  const T v001 = __ldg(g + o + dz), v101 = __ldg(g + o + dz + dx);
  const T v011 = __ldg(g + o + dz + dy), v111 = __ldg(g + o + dz + dy + dx);
  const T a00 = v000 + tx * (v100 - v000), a10 = v010 + tx * (v110 - v010);
  const T a01 = v001 + tx * (v101 - v001), a11 = v011 + tx * (v111 - v011);
  const T b0 = a00 + ty * (a10 - a00), b1 = a01 + ty * (a11 - a01);
  return b0 + tz * (b1 - b0);
}

// HH > 0: the element edge is the compile-time constant HH (the row loop is
// unrolled four-fold and the strip shape folds into the index arithmetic);
// HH == 0: h from the mesh.
template <typename T, bool STATS, bool INTERP, int HH>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? (STATS ? 6 : 6) : 3) k_sample(const SampleArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double s_red[4];
  const Mesh& m = a.m;
  const int h = HH > 0 ? HH : m.h;
  const int EX = HH > 0 ? (HH >= 128 ? 1 : 128 / HH) : a.EX;
  const int nthr = blockDim.x;
  T* s_v = (T*)smem_raw;          // EX*24
  T* s_phi = s_v + (size_t)EX * 24;  // h+1

  const int t = threadIdx.x;
  const int el = t / h, qx = t - el * h;
  const int i0 = blockIdx.x * EX, i = i0 + el;
  const int j = blockIdx.y, k = blockIdx.z;
  const int nel = min(EX, m.Nx - i0);
  const bool active = el < nel;
  const int ny_e = h + (j == m.Ny - 1), nz_e = h + (k == m.Nz - 1);
  const int ncol = active ? ((i == m.Nx - 1 && qx == h - 1) ? 2 : 1) : 0;

  for (int q = t; q <= h; q += nthr) s_phi[q] = (T)q / (T)h;
  for (int idx = t; idx < nel * 24; idx += nthr) {
    const int e = idx / 24, r = idx - e * 24, c = r % 3, cn = r / 3;
    const long long node = (long long)(i0 + e + corner_dx(cn)) + (long long)(j + corner_dy(cn)) * m.Nnx +
                           (long long)(k + corner_dz(cn)) * m.NnxNny;
    s_v[idx] = a.U[3 * node + c];
  }
  __syncthreads();

  // float partials per voxel plane of the column, summed in float over the
  // thread's columns (at most 2 x 81 voxels) and added to float64 once:
  // GB300's FP64 pipe is narrow
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  float c4[4] = {0.f, 0.f, 0.f, 0.f};
  const T gxmax = (T)(a.gnx - 1), gymax = (T)(a.gny - 1), gzmax = (T)(a.gnz - 1);

  for (int col = 0; col < ncol; ++col) {
    const int qxc = qx + col;
    const int x = i * h + qxc;
    const T fx1 = s_phi[qxc], fx0 = T(1) - fx1;
    const int mx = (qxc == 0 && i > 0) ? 2 : 1;
    T ux[12];
#pragma unroll
    for (int ay = 0; ay < 2; ++ay)
#pragma unroll
      for (int az = 0; az < 2; ++az)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          ux[ay * 6 + az * 3 + c] = fx0 * s_v[el * 24 + 3 * corner_of(0, ay, az) + c] +
                                    fx1 * s_v[el * 24 + 3 * corner_of(1, ay, az) + c];
    const T vxf = (T)x;
    for (int qz = 0; qz < nz_e; ++qz) {
      const T fz1 = s_phi[qz], fz0 = T(1) - fz1;
      const int mxz = mx * ((qz == 0 && k > 0) ? 2 : 1);
      T u0[3], du[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        u0[c] = fz0 * ux[0 * 6 + 0 * 3 + c] + fz1 * ux[0 * 6 + 1 * 3 + c];
        du[c] = fz0 * ux[1 * 6 + 0 * 3 + c] + fz1 * ux[1 * 6 + 1 * 3 + c] - u0[c];
      }
      const int vz = k * h + qz;
      const T vzf = (T)vz;
      float r0 = 0.f, r1 = 0.f, r2 = 0.f, r3 = 0.f;
#pragma unroll(HH > 0 ? 4 : 1)
      for (int qy = 0; qy < ny_e; ++qy) {
        const T fy1 = s_phi[qy];
        const int vy = j * h + qy;
        const unsigned vv = (unsigned)x + (unsigned)vy * (unsigned)m.Nvx + (unsigned)vz * (unsigned)m.NvxNvy;
        const T ua = u0[0] + fy1 * du[0], ub = u0[1] + fy1 * du[1], uc = u0[2] + fy1 * du[2];
        if constexpr (INTERP) {
          if (a.channels_first) {
            a.uvox[vv] = ua;
            a.uvox[m.Nvox + vv] = ub;
            a.uvox[2 * m.Nvox + vv] = uc;
          } else {
            a.uvox[3 * (size_t)vv + 0] = ua;
            a.uvox[3 * (size_t)vv + 1] = ub;
            a.uvox[3 * (size_t)vv + 2] = uc;
          }
        } else {
          // (u + x) - g_origin, then bounds, clip and order-1 sampling
          // (engine/correlate_gpu.py:259-276)
          const T cx = (ua + vxf) - a.gx0, cy = (ub + (T)vy) - a.gy0, cz = (uc + vzf) - a.gz0;
          // clipped coordinates; in bounds iff clipping changed nothing
          // (NaN: clipped to a bound, so out of bounds as in the reference)
          const T ccx = tmin(tmax(cx, T(0)), gxmax), ccy = tmin(tmax(cy, T(0)), gymax);
          const T ccz = tmin(tmax(cz, T(0)), gzmax);
          const bool inb = (ccx == cx) & (ccy == cy) & (ccz == cz);
          const T gv = trilinear(a.g, a.gnx, a.gny, a.gnz, ccx, ccy, ccz);
          const bool m0 = a.mask0 ? (__ldg(a.mask0 + vv) != 0) : true;
          const bool mk = inb && m0 && (gv > a.glt);
          a.gvals[vv] = gv;
          a.mask_out[vv] = mk ? 1 : 0;
          if constexpr (STATS) {
            const bool bm = a.bmask_frozen ? (__ldg(a.bmask_frozen + vv) != 0) : mk;
            if (bm) {
              const float mult = (float)(mxz * ((qy == 0 && j > 0) ? 2 : 1));
              const float gf = (float)gv;
              r0 += mult;
              r1 += mult * gf;
              r2 += mult * gf * gf;
            }
            r3 += mk ? 1.f : 0.f;
          }
        }
      }
      if constexpr (STATS) {
        c4[0] += r0;
        c4[1] += r1;
        c4[2] += r2;
        c4[3] += r3;
      }
    }
  }
  if constexpr (STATS) {
    for (int q = 0; q < 4; ++q) acc[q] += c4[q];
    double b4[4], o4[4];
    for (int q = 0; q < 4; ++q) b4[q] = block_sum(acc[q], s_red);
    if (grid_reduce_sum<4>(a.red, b4, o4, s_red) && t == 0)
      for (int q = 0; q < 4; ++q) a.stats[q] = o4[q];
  }
}

// Thread-per-element form of the GN sampling pass (float32, stats fused) for
// small element edges (H <= 4), where an element's few voxels cannot
// amortise a strip block's staging: a thread holds its element's 24 nodal
// values, interpolates u with the strip kernel's operation order (x first,
// then z, then y in difference form) and walks the owned voxels (the
// ownership of elem_fast.cu).  Per-element float partials of the stats are
// folded into float64 per element.
template <int H>
__global__ void __launch_bounds__(256) k_elem_sample(const SampleArgs<float> a) {
  __shared__ double s_red[8];
  const Mesh& m = a.m;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const float gxmax = (float)(a.gnx - 1), gymax = (float)(a.gny - 1), gzmax = (float)(a.gnz - 1);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m.Ne;
       e += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    elem_ijk(m, e, i, j, k);
    float uc[2][2][2][3];  // [dx][dy][dz][c]
#pragma unroll
    for (int dz = 0; dz < 2; ++dz)
#pragma unroll
      for (int dy = 0; dy < 2; ++dy) {
        const long long n0 = (long long)i + (long long)(j + dy) * m.Nnx + (long long)(k + dz) * m.NnxNny;
#pragma unroll
        for (int dx = 0; dx < 2; ++dx)
#pragma unroll
          for (int c = 0; c < 3; ++c) uc[dx][dy][dz][c] = __ldg(a.U + 3 * (n0 + dx) + c);
      }
    const int nx_e = H + (i == m.Nx - 1), ny_e = H + (j == m.Ny - 1), nz_e = H + (k == m.Nz - 1);
    float r0 = 0.f, r1 = 0.f, r2 = 0.f, r3 = 0.f;
#pragma unroll 1
    for (int qx = 0; qx < nx_e; ++qx) {
      const int x = i * H + qx;
      const float fx1 = (float)qx / (float)H, fx0 = 1.f - fx1;
      const int mx = (qx == 0 && i > 0) ? 2 : 1;
      float ux[12];
#pragma unroll
      for (int ay = 0; ay < 2; ++ay)
#pragma unroll
        for (int az = 0; az < 2; ++az)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            ux[ay * 6 + az * 3 + c] = fx0 * uc[0][ay][az][c] + fx1 * uc[1][ay][az][c];
      const float vxf = (float)x;
#pragma unroll
      for (int qz = 0; qz <= H; ++qz) {
        if (qz == nz_e) break;
        const float fz1 = (float)qz / (float)H, fz0 = 1.f - fz1;
        const int mxz = mx * ((qz == 0 && k > 0) ? 2 : 1);
        float u0[3], du[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          u0[c] = fz0 * ux[0 * 6 + 0 * 3 + c] + fz1 * ux[0 * 6 + 1 * 3 + c];
          du[c] = fz0 * ux[1 * 6 + 0 * 3 + c] + fz1 * ux[1 * 6 + 1 * 3 + c] - u0[c];
        }
        const int vz = k * H + qz;
        const float vzf = (float)vz;
#pragma unroll
        for (int qy = 0; qy <= H; ++qy) {
          if (qy == ny_e) break;
          const float fy1 = (float)qy / (float)H;
          const int vy = j * H + qy;
          const unsigned vv = (unsigned)x + (unsigned)vy * (unsigned)m.Nvx + (unsigned)vz * (unsigned)m.NvxNvy;
          const float ua = u0[0] + fy1 * du[0], ub = u0[1] + fy1 * du[1], ucz = u0[2] + fy1 * du[2];
          // (u + x) - g_origin, then bounds, clip and order-1 sampling
          // (engine/correlate_gpu.py:259-276), as in k_sample
          const float cx = (ua + vxf) - a.gx0, cy = (ub + (float)vy) - a.gy0, cz = (ucz + vzf) - a.gz0;
          const float ccx = fminf(fmaxf(cx, 0.f), gxmax), ccy = fminf(fmaxf(cy, 0.f), gymax);
          const float ccz = fminf(fmaxf(cz, 0.f), gzmax);
          const bool inb = (ccx == cx) & (ccy == cy) & (ccz == cz);
          const float gv = trilinear(a.g, a.gnx, a.gny, a.gnz, ccx, ccy, ccz);
          const bool m0 = a.mask0 ? (__ldg(a.mask0 + vv) != 0) : true;
          const bool mk = inb && m0 && (gv > a.glt);
          a.gvals[vv] = gv;
          a.mask_out[vv] = mk ? 1 : 0;
          const bool bm = a.bmask_frozen ? (__ldg(a.bmask_frozen + vv) != 0) : mk;
          if (bm) {
            const float mult = (float)(mxz * ((qy == 0 && j > 0) ? 2 : 1));
            r0 += mult;
            r1 += mult * gv;
            r2 += mult * gv * gv;
          }
          r3 += mk ? 1.f : 0.f;
        }
      }
    }
    acc[0] += r0;
    acc[1] += r1;
    acc[2] += r2;
    acc[3] += r3;
  }
  double b4[4], o4[4];
  for (int q = 0; q < 4; ++q) b4[q] = block_sum(acc[q], s_red);
  if (grid_reduce_sum<4>(a.red, b4, o4, s_red) && threadIdx.x == 0)
    for (int q = 0; q < 4; ++q) a.stats[q] = o4[q];
}

// Element edges up to this one take the thread-per-element GN sampler.
constexpr int kElemSampleMaxH = 4;

template <int H>
static int launch_elem_sample(const SampleArgs<float>& a, cudaStream_t s) {
  // at most kReduceBlocks blocks: the reduction partials hold that many
  long long nb = (a.m.Ne + 255) / 256;
  if (nb > kReduceBlocks) nb = kReduceBlocks;
  k_elem_sample<H><<<(unsigned)nb, 256, 0, s>>>(a);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

template <typename T, bool STATS, bool INTERP>
int launch_sample(const SampleArgs<T>& args, cudaStream_t s) {
  if (args.m.h > 128) return set_error(VDVC_ERR_UNSUPPORTED, "element edge h=%d > 128 not supported", args.m.h);
  if ((unsigned long long)args.gnx * args.gny * args.gnz >= (1ull << 32))
    return set_error(VDVC_ERR_UNSUPPORTED, "deformed image of 2^32 voxels or more");
  StripShape sh = strip_shape(args.m.h);
  dim3 grid((args.m.Nx + sh.EX - 1) / sh.EX, args.m.Ny, args.m.Nz);
  const size_t smem = ((size_t)sh.EX * 24 + args.m.h + 2) * sizeof(T);
  SampleArgs<T> a = args;
  a.EX = sh.EX;
  if constexpr (std::is_same<T, float>::value && STATS && !INTERP) {
    if (args.m.h <= kElemSampleMaxH) {
      switch (args.m.h) {
        case 1: return launch_elem_sample<1>(a, s);
        case 2: return launch_elem_sample<2>(a, s);
        case 3: return launch_elem_sample<3>(a, s);
        case 4: return launch_elem_sample<4>(a, s);
      }
    }
  }
  if constexpr (std::is_same<T, float>::value) {
    switch (args.m.h) {
      case 2: k_sample<T, STATS, INTERP, 2><<<grid, sh.threads, smem, s>>>(a); VDVC_LAUNCHED(); return VDVC_OK;
      case 4: k_sample<T, STATS, INTERP, 4><<<grid, sh.threads, smem, s>>>(a); VDVC_LAUNCHED(); return VDVC_OK;
      case 8: k_sample<T, STATS, INTERP, 8><<<grid, sh.threads, smem, s>>>(a); VDVC_LAUNCHED(); return VDVC_OK;
      case 16: k_sample<T, STATS, INTERP, 16><<<grid, sh.threads, smem, s>>>(a); VDVC_LAUNCHED(); return VDVC_OK;
    }
  }
  k_sample<T, STATS, INTERP, 0><<<grid, sh.threads, smem, s>>>(a);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

template <typename T>
int launch_masked_stats(const T* field, const uint8_t* mask, const Mesh& m, GridReduce red, double* out3,
                        cudaStream_t s) {
  const long long rows = (long long)m.Nvy * m.Nvz;
  const int blocks = grid_blocks(rows, 1, kReduceBlocks);
  k_masked_stats<T><<<blocks, 256, 0, s>>>(field, mask, m, red, out3);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

template int launch_sample<float, true, false>(const SampleArgs<float>&, cudaStream_t);
template int launch_sample<double, true, false>(const SampleArgs<double>&, cudaStream_t);
template int launch_masked_stats<float>(const float*, const uint8_t*, const Mesh&, GridReduce, double*, cudaStream_t);
template int launch_masked_stats<double>(const double*, const uint8_t*, const Mesh&, GridReduce, double*,
                                         cudaStream_t);

}  // namespace vdvc

using namespace vdvc;

extern "C" {

int vdvc_masked_stats(const void* field, int dtype, const uint8_t* mask, int h, int Nx, int Ny, int Nz, double* out3,
                      void* ws, size_t ws_bytes, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(h, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(field && mask && out3, "null pointer");
  Carve cv(ws, ws_bytes);
  double* partials = cv.take<double>((size_t)kReduceBlocks * 3);
  unsigned int* ticket = cv.take<unsigned int>(1);
  if (!ws || !cv.fits()) return set_error(VDVC_ERR_WORKSPACE, "masked_stats needs %zu bytes of workspace", cv.off);
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s));
  GridReduce red{partials, ticket};
  if (dtype == VDVC_F32) return launch_masked_stats<float>((const float*)field, mask, m, red, out3, s);
  if (dtype == VDVC_F64) return launch_masked_stats<double>((const double*)field, mask, m, red, out3, s);
  return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
}

int vdvc_sample_deformed(const void* U, const void* g_vox, int dtype, int gnx, int gny, int gnz, double gx0,
                         double gy0, double gz0, const uint8_t* mask0, double glt, int h, int Nx, int Ny, int Nz,
                         void* g_vals, uint8_t* mask_out, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(h, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(U && g_vox && g_vals && mask_out, "null pointer");
  VDVC_CHECK_ARG(gnx >= 1 && gny >= 1 && gnz >= 1, "bad g shape");
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == VDVC_F32) {
    SampleArgs<float> a{};
    a.m = m; a.U = (const float*)U; a.g = (const float*)g_vox; a.gnx = gnx; a.gny = gny; a.gnz = gnz;
    a.gx0 = (float)gx0; a.gy0 = (float)gy0; a.gz0 = (float)gz0; a.mask0 = mask0; a.glt = (float)glt;
    a.gvals = (float*)g_vals; a.mask_out = mask_out;
    return launch_sample<float, false, false>(a, s);
  }
  if (dtype == VDVC_F64) {
    SampleArgs<double> a{};
    a.m = m; a.U = (const double*)U; a.g = (const double*)g_vox; a.gnx = gnx; a.gny = gny; a.gnz = gnz;
    a.gx0 = gx0; a.gy0 = gy0; a.gz0 = gz0; a.mask0 = mask0; a.glt = glt;
    a.gvals = (double*)g_vals; a.mask_out = mask_out;
    return launch_sample<double, false, false>(a, s);
  }
  return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
}

int vdvc_interp_field(const void* U, int dtype, int h, int Nx, int Ny, int Nz, int channels_first, void* out,
                      vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(h, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(U && out, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == VDVC_F32) {
    SampleArgs<float> a{};
    a.m = m; a.U = (const float*)U; a.uvox = (float*)out; a.channels_first = channels_first;
    return launch_sample<float, false, true>(a, s);
  }
  if (dtype == VDVC_F64) {
    SampleArgs<double> a{};
    a.m = m; a.U = (const double*)U; a.uvox = (double*)out; a.channels_first = channels_first;
    return launch_sample<double, false, true>(a, s);
  }
  return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
}

}  // extern "C"
