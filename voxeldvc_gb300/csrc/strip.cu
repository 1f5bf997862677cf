// Element-strip quadrature kernels (see strip.cuh for the decomposition) and
// the node gather that assembles element vectors into dof vectors.
#include <cstdlib>
#include <type_traits>

#include "ops.cuh"
#include "pcg.cuh"

namespace vdvc {

template <typename T> __device__ __forceinline__ T rn_add(T a, T b);
template <typename T> __device__ __forceinline__ T rn_sub(T a, T b);
template <typename T> __device__ __forceinline__ T rn_mul(T a, T b);
template <> __device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
template <> __device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }

// Accumulator index r = ax*12 + ay*6 + az*3 + c  ->  element-vector row 3a+c.
__device__ __forceinline__ int acc_row(int r) {
  const int ax = r / 12, ay = (r / 6) & 1, az = (r / 3) & 1, c = r % 3;
  return 3 * corner_of(ax, ay, az) + c;
}

template <typename T, int MODE>
__global__ void __launch_bounds__(128) k_strip(const StripArgs<T> a, const Kpair<T>* __restrict__ kp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Mesh& m = a.m;
  const int h = m.h, EX = a.EX;
  const int nthr = blockDim.x;
  T* s_accA = (T*)smem_raw;                              // nthr*25
  T* s_accD = s_accA + (size_t)nthr * 25;                // nthr*25 (diag)
  T* s_v = s_accD + ((MODE & kModeDiag) ? (size_t)nthr * 25 : 0);  // EX*24
  T* s_w = s_v + (size_t)EX * 24;                        // EX*24 (K2 input)
  T* s_phi = s_w + (size_t)EX * 24;                      // h+1
  T* s_K = s_phi + ((h + 2) & ~1);                       // 2*576
  __shared__ double s_red[4];

  constexpr bool HV = (MODE & kModeHv) != 0;
  constexpr bool BB = (MODE & kModeB) != 0;
  constexpr bool DG = (MODE & kModeDiag) != 0;
  constexpr bool RS = (MODE & kModeRes) != 0;
  constexpr bool PC = (MODE & kModePcg) != 0;

  if constexpr (PC) {
    if (a.st->done) return;
  }

  const int t = threadIdx.x;
  const int el = t / h, qx = t - el * h;
  const int i0 = blockIdx.x * EX;
  const int i = i0 + el;
  const int j = blockIdx.y, k = blockIdx.z;
  const int nel = min(EX, m.Nx - i0);
  const bool active = el < nel;
  const int ny_e = h + (j == m.Ny - 1), nz_e = h + (k == m.Nz - 1);
  const int ncol = active ? ((i == m.Nx - 1 && qx == h - 1) ? 2 : 1) : 0;

  // ---- block prologue: phi table, nodal strip vectors, regularizer K ----
  for (int q = t; q <= h; q += nthr) s_phi[q] = (T)q / (T)h;
  if constexpr (HV) {
    T beta = T(0);
    if constexpr (PC) beta = (T)a.st->beta;
    for (int idx = t; idx < nel * 24; idx += nthr) {
      const int e = idx / 24, r = idx - e * 24, c = r % 3, cn = r / 3;
      const long long node = (long long)(i0 + e + corner_dx(cn)) + (long long)(j + corner_dy(cn)) * m.Nnx +
                             (long long)(k + corner_dz(cn)) * m.NnxNny;
      T val = a.v[3 * node + c];
      if constexpr (PC) val = val + beta * a.p_old[3 * node + c];
      s_v[idx] = val;
      if (a.nreg == 2) s_w[idx] = a.w[3 * node + c];
    }
    if (a.nreg >= 1)
      for (int q = t; q < 576 * a.nreg; q += nthr) s_K[q] = (q < 576) ? kp->K1[q] : kp->K2[q - 576];
  }
  for (int r = 0; r < 25; ++r) {
    s_accA[t * 25 + r] = T(0);
    if constexpr (DG) s_accD[t * 25 + r] = T(0);
  }
  // GN residual scalars
  T gm = T(0), ratio = T(0), mean0 = T(0);
  if constexpr (RS) {
    const double c = a.gstats[0];
    double mean = 0.0, sd = 0.0;
    if (c >= 1.0) {
      mean = a.gstats[1] / c;
      const double var = a.gstats[2] / c - mean * mean;
      sd = sqrt(var > 0.0 ? var : 0.0);
    }
    if (sd == 0.0) {
      if (t == 0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) *a.status = VDVC_ERR_ZERO_DIVISION;
    }
    gm = (T)mean;
    ratio = (T)(-(a.std0 / sd));
    mean0 = (T)a.mean0;
  }
  __syncthreads();

  double dsum[3] = {0.0, 0.0, 0.0};  // display stats (RS)

  for (int col = 0; col < ncol; ++col) {
    const int qxc = qx + col;
    const long long x = (long long)i * h + qxc;
    const T fx1 = s_phi[qxc], fx0 = T(1) - fx1;
    const int mx = (qxc == 0 && i > 0) ? 2 : 1;
    // outer-face quadrature weight along x (1/2 on the first and last plane)
    const T wx = (x == 0 || x == (long long)m.Nvx - 1) ? T(0.5) : T(1);
    T ux[12];
    if constexpr (HV) {
#pragma unroll
      for (int ay = 0; ay < 2; ++ay)
#pragma unroll
        for (int az = 0; az < 2; ++az)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            ux[ay * 6 + az * 3 + c] = fx0 * s_v[el * 24 + 3 * corner_of(0, ay, az) + c] +
                                      fx1 * s_v[el * 24 + 3 * corner_of(1, ay, az) + c];
    }
    T accA[12], accD[12];
#pragma unroll
    for (int r = 0; r < 12; ++r) { accA[r] = T(0); accD[r] = T(0); }

    for (int qz = 0; qz < nz_e; ++qz) {
      const T fz1 = s_phi[qz], fz0 = T(1) - fz1;
      const int mxz = mx * ((qz == 0 && k > 0) ? 2 : 1);
      const int vz = k * h + qz;
      const T wz = (vz == 0 || vz == m.Nvz - 1) ? T(0.5) : T(1);
      T u0[3], du[3];
      if constexpr (HV) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          u0[c] = fz0 * ux[0 * 6 + 0 * 3 + c] + fz1 * ux[0 * 6 + 1 * 3 + c];
          const T u1 = fz0 * ux[1 * 6 + 0 * 3 + c] + fz1 * ux[1 * 6 + 1 * 3 + c];
          du[c] = u1 - u0[c];
        }
      }
      T S[3] = {T(0), T(0), T(0)}, S1[3] = {T(0), T(0), T(0)};
      T D0[3] = {T(0), T(0), T(0)}, D1[3] = {T(0), T(0), T(0)};
      float ds0 = 0.f, ds1 = 0.f, ds2 = 0.f;
      const long long vbase = x + (long long)j * h * m.Nvx + ((long long)k * h + qz) * m.NvxNvy;
#pragma unroll 4
      for (int qy = 0; qy < ny_e; ++qy) {
        const T fy1 = s_phi[qy];
        const long long vv = vbase + (long long)qy * m.Nvx;
        const int vy = j * h + qy;
        const T wy = (vy == 0 || vy == m.Nvy - 1) ? T(0.5) : T(1);
        // read-only inputs through the non-coherent path: the residual's
        // store below would otherwise keep them from being hoisted
        const T g0 = __ldg(a.grad + 3 * vv), g1 = __ldg(a.grad + 3 * vv + 1), g2 = __ldg(a.grad + 3 * vv + 2);
        const bool mm = __ldg(a.mask + vv) != 0;
        if constexpr (HV) {
          const T uu0 = u0[0] + fy1 * du[0], uu1 = u0[1] + fy1 * du[1], uu2 = u0[2] + fy1 * du[2];
          T d = g0 * uu0 + g1 * uu1 + g2 * uu2;
          d = mm ? d * wy : T(0);
          const T t0 = d * g0, t1 = d * g1, t2 = d * g2;
          S[0] += t0; S[1] += t1; S[2] += t2;
          S1[0] += fy1 * t0; S1[1] += fy1 * t1; S1[2] += fy1 * t2;
        }
        if constexpr (BB) {
          T r;
          if constexpr (RS) {
            const T fc = rn_sub(__ldg(a.f + vv), mean0);
            const T rv = rn_add(rn_mul(rn_sub(__ldg(a.gvals + vv), gm), ratio), fc);
            r = mm ? rv : T(0);
            a.res_out[vv] = r;
            if (__ldg(a.live + vv)) {
              const int mult = mxz * ((qy == 0 && j > 0) ? 2 : 1);
              const float rf = (float)r, mf = (float)mult;
              ds0 += mf;
              ds1 += mf * rf;
              ds2 += mf * rf * rf;
            }
          } else {
            r = mm ? __ldg(a.res_in + vv) : T(0);
          }
          r *= wy;
          const T t0 = r * g0, t1 = r * g1, t2 = r * g2;
          S[0] += t0; S[1] += t1; S[2] += t2;
          S1[0] += fy1 * t0; S1[1] += fy1 * t1; S1[2] += fy1 * t2;
        }
        if constexpr (DG) {
          const T fy0 = T(1) - fy1;
          const T w0 = wy * fy0 * fy0, w1 = wy * fy1 * fy1;
          const T d0 = mm ? g0 * g0 : T(0), d1 = mm ? g1 * g1 : T(0), d2 = mm ? g2 * g2 : T(0);
          D0[0] += w0 * d0; D0[1] += w0 * d1; D0[2] += w0 * d2;
          D1[0] += w1 * d0; D1[1] += w1 * d1; D1[2] += w1 * d2;
        }
      }
      if constexpr (RS) {
        dsum[0] += (double)ds0;
        dsum[1] += (double)ds1;
        dsum[2] += (double)ds2;
      }
      if constexpr (HV || BB) {
        const T gz0 = wz * fz0, gz1 = wz * fz1;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const T s0 = S[c] - S1[c];
          accA[0 * 6 + 0 * 3 + c] += gz0 * s0;
          accA[0 * 6 + 1 * 3 + c] += gz1 * s0;
          accA[1 * 6 + 0 * 3 + c] += gz0 * S1[c];
          accA[1 * 6 + 1 * 3 + c] += gz1 * S1[c];
        }
      }
      if constexpr (DG) {
        const T z0 = wz * fz0 * fz0, z1 = wz * fz1 * fz1;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          accD[0 * 6 + 0 * 3 + c] += z0 * D0[c];
          accD[0 * 6 + 1 * 3 + c] += z1 * D0[c];
          accD[1 * 6 + 0 * 3 + c] += z0 * D1[c];
          accD[1 * 6 + 1 * 3 + c] += z1 * D1[c];
        }
      }
    }
    if constexpr (HV || BB) {
      const T gx0 = wx * fx0, gx1 = wx * fx1;
#pragma unroll
      for (int r = 0; r < 12; ++r) {
        s_accA[t * 25 + r] += gx0 * accA[r];
        s_accA[t * 25 + 12 + r] += gx1 * accA[r];
      }
    }
    if constexpr (DG) {
      const T x0 = wx * fx0 * fx0, x1 = wx * fx1 * fx1;
#pragma unroll
      for (int r = 0; r < 12; ++r) {
        s_accD[t * 25 + r] += x0 * accD[r];
        s_accD[t * 25 + 12 + r] += x1 * accD[r];
      }
    }
  }
  __syncthreads();

  // ---- reduce the columns of each element and write element vectors ----
  const long long e_base = (long long)i0 + (long long)j * m.Nx + (long long)k * m.Nx * m.Ny;
  for (int idx = t; idx < nel * 24; idx += nthr) {
    const int r = idx / nel, e = idx - r * nel;  // element fastest: coalesced stores
    const int row = acc_row(r);
    if constexpr (HV || BB) {
      T s = T(0);
      for (int q = 0; q < h; ++q) s += s_accA[(e * h + q) * 25 + r];
      if constexpr (HV) {
        if (a.nreg >= 1) {
          T k1 = T(0);
#pragma unroll 8
          for (int b = 0; b < 24; ++b) k1 += s_K[row * 24 + b] * s_v[e * 24 + b];
          s += a.c1 * k1;
          if (a.nreg == 2) {
            T k2 = T(0);
#pragma unroll 8
            for (int b = 0; b < 24; ++b) k2 += s_K[576 + row * 24 + b] * s_w[e * 24 + b];
            s += a.c2 * k2;
          }
        }
      }
      a.evA[(long long)row * m.Ne + e_base + e] = s;
    }
    if constexpr (DG) {
      T s = T(0);
      for (int q = 0; q < h; ++q) s += s_accD[(e * h + q) * 25 + r];
      a.evD[(long long)row * m.Ne + e_base + e] = s;
    }
  }

  if constexpr (RS) {
    // display stats of res over the live mask (deterministic grid reduction)
    double b3[3], out[3];
    for (int q = 0; q < 3; ++q) b3[q] = block_sum(dsum[q], s_red);
    if (grid_reduce_sum<3>(a.red, b3, out, s_red) && t == 0)
      for (int q = 0; q < 3; ++q) a.dstats[q] = out[q];
  }
}

// Node gather: out[3n+c] = sum over the (up to 8) elements containing node
// n of ev[(3a+c)*Ne + e], a = n's corner in e.  Fixed summation order.
template <typename T>
__device__ __forceinline__ void gather_node(const Mesh& m, const T* __restrict__ ev, long long n, T out[3]) {
  // 32-bit node coordinates (the launcher rejects 2^32 nodes or more): a
  // 64-bit division costs tens of instructions per node
  const unsigned int nu = (unsigned int)n, nnx = (unsigned int)m.Nnx, rr = nu / nnx;
  const int ni = (int)(nu - rr * nnx), nj = (int)(rr % (unsigned int)m.Nny), nk = (int)(rr / (unsigned int)m.Nny);
  out[0] = out[1] = out[2] = T(0);
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int ei = ni - corner_dx(a), ej = nj - corner_dy(a), ek = nk - corner_dz(a);
    if (ei < 0 || ej < 0 || ek < 0 || ei >= m.Nx || ej >= m.Ny || ek >= m.Nz) continue;
    const long long e = (long long)ei + (long long)ej * m.Nx + (long long)ek * m.Nx * m.Ny;
#pragma unroll
    for (int c = 0; c < 3; ++c) out[c] += ev[(long long)(3 * a + c) * m.Ne + e];
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_gather(const Mesh m, const T* __restrict__ ev, T* __restrict__ out) {
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < m.Nnodes;
       n += (long long)gridDim.x * blockDim.x) {
    T s[3];
    gather_node(m, ev, n, s);
    out[3 * n + 0] = s[0];
    out[3 * n + 1] = s[1];
    out[3 * n + 2] = s[2];
  }
}

// ---- host-side launch helpers ---------------------------------------------

size_t strip_smem_bytes(int h, int mode, size_t tsize) {
  StripShape s = strip_shape(h);
  size_t n = (size_t)s.threads * 25;                 // accA
  if (mode & kModeDiag) n += (size_t)s.threads * 25; // accD
  n += (size_t)s.EX * 24 * 2;                        // s_v, s_w
  n += (size_t)((h + 2) & ~1);                       // phi
  n += 2 * 576;                                      // K1, K2
  return n * tsize;
}

// Kernel selection for the float32 passes: thread per element for
// h <= kElemMaxH (elem_fast.cu, rhs_fast.cu), else the compile-time-h strip
// specialisations (strip_fast.cu, rhs_fast.cu); the generic strip kernel of
// this file (runtime h) serves every other h and the float64 solve.
constexpr int kElemMaxH = 4;

template <typename T, int MODE>
int launch_strip(const StripArgs<T>& args, const Kpair<T>* kp, cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value && (MODE == kModeHv || MODE == (kModeHv | kModePcg))) {
    constexpr bool pcg = (MODE & kModePcg) != 0;
    const int st = args.m.h <= kElemMaxH ? launch_elem_fast<pcg>(args, kp, s) : launch_strip_fast<pcg>(args, kp, s);
    if (st != VDVC_ERR_UNSUPPORTED) return st;
  }
  if constexpr (std::is_same<T, float>::value &&
                (MODE == (kModeB | kModeRes) || MODE == (kModeB | kModeRes | kModeDiag))) {
    const int st = launch_rhs_fast<(MODE & kModeDiag) != 0>(args, s);
    if (st != VDVC_ERR_UNSUPPORTED) return st;
  }
  StripShape sh = strip_shape(args.m.h);
  if (args.m.h > 128) return set_error(VDVC_ERR_UNSUPPORTED, "element edge h=%d > 128 not supported", args.m.h);
  if (args.m.Ny > 65535 || args.m.Nz > 65535) return set_error(VDVC_ERR_ARG, "Ny/Nz > 65535");
  dim3 grid((args.m.Nx + sh.EX - 1) / sh.EX, args.m.Ny, args.m.Nz);
  size_t smem = strip_smem_bytes(args.m.h, MODE, sizeof(T));
  if (int st = ensure_dyn_smem((const void*)k_strip<T, MODE>, 96 * 1024)) return st;
  StripArgs<T> a = args;
  a.EX = sh.EX;
  k_strip<T, MODE><<<grid, sh.threads, smem, s>>>(a, kp);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

long long strip_grid_blocks(const Mesh& m) {
  StripShape sh = strip_shape(m.h);
  return (long long)((m.Nx + sh.EX - 1) / sh.EX) * m.Ny * m.Nz;
}

template <typename T>
int launch_gather(const Mesh& m, const T* ev, T* out, cudaStream_t s) {
  if (m.Nnodes >= (1ll << 32)) return set_error(VDVC_ERR_UNSUPPORTED, "2^32 nodes or more");
  long long b = (m.Nnodes + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  k_gather<T><<<(int)b, 256, 0, s>>>(m, ev, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

// explicit instantiations used by the entry points
#define VDVC_INST_STRIP(T, MODE) template int launch_strip<T, MODE>(const StripArgs<T>&, const Kpair<T>*, cudaStream_t);
VDVC_INST_STRIP(float, kModeHv)
VDVC_INST_STRIP(double, kModeHv)
VDVC_INST_STRIP(float, kModeB)
VDVC_INST_STRIP(double, kModeB)
VDVC_INST_STRIP(float, kModeDiag)
VDVC_INST_STRIP(double, kModeDiag)
VDVC_INST_STRIP(float, kModeB | kModeRes)
VDVC_INST_STRIP(float, kModeB | kModeRes | kModeDiag)
VDVC_INST_STRIP(double, kModeB | kModeRes)
VDVC_INST_STRIP(double, kModeB | kModeRes | kModeDiag)
VDVC_INST_STRIP(float, kModeHv | kModePcg)
VDVC_INST_STRIP(double, kModeHv | kModePcg)
template int launch_gather<float>(const Mesh&, const float*, float*, cudaStream_t);
template int launch_gather<double>(const Mesh&, const double*, double*, cudaStream_t);

}  // namespace vdvc
