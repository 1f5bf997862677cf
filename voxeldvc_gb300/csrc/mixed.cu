// Element-Hessian form of the Hessian: element Hessians formed once per
// Gauss-Newton iteration with FP32 accumulation, FP32 element-Hessian
// matvecs in the PCG.  The gradient is either the float32 gradient itself
// (VDVC_PREC_ELEMENT: the plain solve's arithmetic in another summation
// order) or its BF16 rounding (VDVC_PREC_MIXED, the precision form).  The
// precision form's GN solver also stores the 162 entries in BF16 (rounded
// once from their FP32 sums; the matvec accumulates in FP32): half the bytes
// of the PCG's dominant stream.  The fixed point of the GN iteration is set
// by the FP32 residual and right-hand side, not by H.  Under the
// equilibrium-gap regularizer the entries stay FP32 (gn.cu).
//
// Element Hessian structure.  With owner-computes quadrature (strip.cuh),
//   K_e[(a,k),(b,l)] = sum_q w_q m_q N_a(q) N_b(q) g_k(q) g_l(q),
// N_a = phi_ax phi_ay phi_az.  Per axis, phi_ax phi_bx takes one of three
// values psi_s (s = ax + bx: phi0^2, phi0 phi1, phi1^2), and g_k g_l is
// symmetric, so K_e has 27 x 6 = 162 distinct entries
//   T[sx][sy][sz][kl] = sum_q w m psi_sx(qx) psi_sy(qy) psi_sz(qz) G_kl(q),
// G = (g0g0, g0g1, g0g2, g1g1, g1g2, g2g2).  T is formed separably (per
// voxel 18 FMAs along y, 54 per z plane, the x sum as a shared-memory
// reduction over the element's voxel columns) and stored tile-major
// [Ne / 64][162][64] (see the matvec below).
// A BF16 x BF16 product is exact in FP32, so G carries no rounding beyond
// the BF16 gradient itself; from the float32 gradient G is rounded once, as
// the matrix-free pass rounds its products.
#include <cuda_bf16.h>

#include <type_traits>

#include "ops.cuh"
#include "pcg.cuh"
#include "tma.cuh"

namespace vdvc {

__global__ void k_grad_to_bf16(const float* __restrict__ g, long long n, __nv_bfloat16* __restrict__ out,
                               unsigned int* __restrict__ amax) {
  float mx = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const __nv_bfloat16 b = __float2bfloat16_rn(g[i]);
    out[i] = b;
    mx = fmaxf(mx, fabsf(__bfloat162float(b)));
  }
  // non-negative floats order like their bit patterns: one atomic per warp
  for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (amax && (threadIdx.x & 31) == 0) atomicMax(amax, __float_as_uint(mx));
}


constexpr int kRP = 55;  // shared-memory pitch of a column's 54 partial sums (odd: no bank conflicts)

__device__ __forceinline__ float grad_comp(const __nv_bfloat16* g, long long i) { return __bfloat162float(g[i]); }
__device__ __forceinline__ float grad_comp(const float* g, long long i) { return __ldg(g + i); }

template <int H, typename GT>
__global__ void __launch_bounds__(128) k_eh_form(const EhFormArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int EX = (H >= 128) ? 1 : 128 / H;
  float* s_R = (float*)smem_raw;  // (nthr + 1) * kRP: one row per column, +1 for the mesh's last column
  const Mesh& m = a.m;
  const int nthr = blockDim.x;
  const int t = threadIdx.x;
  const int el = t / H, qx = t - el * H;
  const int i0 = blockIdx.x * EX, i = i0 + el;
  const int j = blockIdx.y, k = blockIdx.z;
  const int nel = min(EX, m.Nx - i0);
  const bool active = el < nel;
  const bool y_last = (j == m.Ny - 1), z_last = (k == m.Nz - 1);
  const int ncol = active ? ((i == m.Nx - 1 && qx == H - 1) ? 2 : 1) : 0;
  const float wy_first = (j == 0) ? 0.5f : 1.f;
  const long long row_stride = m.Nvx;

  for (int r = 0; r < kRP; ++r) s_R[t * kRP + r] = 0.f;
  if (t == 0)
    for (int r = 0; r < kRP; ++r) s_R[nthr * kRP + r] = 0.f;
  __syncthreads();

  for (int col = 0; col < ncol; ++col) {
    const int qxc = qx + col;
    const long long x = (long long)i * H + qxc;
    float R[54];  // [sy][sz][kl]
#pragma unroll
    for (int q = 0; q < 54; ++q) R[q] = 0.f;
#pragma unroll 1
    for (int qz = 0; qz <= H; ++qz) {
      if (qz == H && !z_last) break;
      const float fz1 = (float)qz / (float)H, fz0 = 1.f - fz1;
      const long long vz = (long long)k * H + qz;
      const float wz = (vz == 0 || vz == m.Nvz - 1) ? 0.5f : 1.f;
      const float pz[3] = {wz * fz0 * fz0, wz * fz0 * fz1, wz * fz1 * fz1};
      const long long v0 = x + (long long)j * H * row_stride + vz * m.NvxNvy;
      float S[18];  // [sy][kl]
#pragma unroll
      for (int q = 0; q < 18; ++q) S[q] = 0.f;
#pragma unroll
      for (int qy = 0; qy <= H; ++qy) {
        if (qy == H && !y_last) break;
        const long long v = v0 + (long long)qy * row_stride;
        const GT* gb = (const GT*)a.grad + 3 * v;
        const float g0 = grad_comp(gb, 0);
        const float g1 = grad_comp(gb, 1);
        const float g2 = grad_comp(gb, 2);
        float W = a.mask[v] ? 1.f : 0.f;
        if (qy == 0) W *= wy_first;
        if (qy == H) W *= 0.5f;
        const float fy1 = (float)qy / (float)H, fy0 = 1.f - fy1;
        const float py[3] = {W * fy0 * fy0, W * fy0 * fy1, W * fy1 * fy1};
        const float G[6] = {g0 * g0, g0 * g1, g0 * g2, g1 * g1, g1 * g2, g2 * g2};
#pragma unroll
        for (int sy = 0; sy < 3; ++sy)
#pragma unroll
          for (int kl = 0; kl < 6; ++kl) S[sy * 6 + kl] += py[sy] * G[kl];
      }
#pragma unroll
      for (int sy = 0; sy < 3; ++sy)
#pragma unroll
        for (int sz = 0; sz < 3; ++sz)
#pragma unroll
          for (int kl = 0; kl < 6; ++kl) R[(sy * 3 + sz) * 6 + kl] += pz[sz] * S[sy * 6 + kl];
    }
    const float wx = (x == 0 || x == (long long)m.Nvx - 1) ? 0.5f : 1.f;
    float* row = s_R + (size_t)(col == 0 ? t : nthr) * kRP;
#pragma unroll
    for (int q = 0; q < 54; ++q) row[q] = wx * R[q];
  }
  __syncthreads();

  // x reduction: T[sx][sy][sz][kl] = sum over the element's columns of psi_sx(qx) R
  const bool last_strip = (i0 + nel == m.Nx);
  const long long e_base = (long long)i0 + (long long)j * m.Nx + (long long)k * m.Nx * m.Ny;
  for (int idx = t; idx < nel * 162; idx += nthr) {
    const int o = idx / nel, e = idx - o * nel;  // element fastest: coalesced stores
    const int sx = o / 54, rest = o - sx * 54;    // rest = (sy*3+sz)*6 + kl
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < H; ++q) {
      const float f1 = (float)q / (float)H, f0 = 1.f - f1;
      const float px = sx == 0 ? f0 * f0 : (sx == 1 ? f0 * f1 : f1 * f1);
      s += px * s_R[(e * H + q) * kRP + rest];
    }
    if (last_strip && e == nel - 1 && sx == 2) s += s_R[nthr * kRP + rest];  // column x = Nx*h: psi = (0,0,1)
    const long long eg = e_base + e;  // tile-major: [tile][162][kEhTile]
    const long long ti = ((eg / kEhTile) * 162 + o) * kEhTile + (eg % kEhTile);
    if (a.Tb)
      ((__nv_bfloat16*)a.Tb)[ti] = __float2bfloat16_rn(s);
    else
      a.T[ti] = s;
    // diagonal of K_e: a = (sx/2, sy/2, sz/2) with sx,sy,sz in {0,2}, kl in {00,11,22}
    const int sy = rest / 18, sz = (rest / 6) % 3, kl = rest % 6;
    if ((sx & 1) == 0 && (sy & 1) == 0 && (sz & 1) == 0 && (kl == 0 || kl == 3 || kl == 5)) {
      const int corner = corner_of(sx >> 1, sy >> 1, sz >> 1);
      const int kk = kl == 0 ? 0 : (kl == 3 ? 1 : 2);
      a.evD[(long long)(3 * corner + kk) * m.Ne + e_base + e] = s;
    }
  }
}

// kl index of the unordered component pair (k,l): (0,0) 0, (0,1) 1,
// (0,2) 2, (1,1) 3, (1,2) 4, (2,2) 5.  Not recursive, so that it folds to a
// constant in unrolled loops (a runtime index into a register array would
// move the array to local memory).
__host__ __device__ constexpr int kl_index(int k, int l) {
  return k <= l ? (k == 0 ? l : (k == 1 ? 2 + l : 5)) : (l == 0 ? k : (l == 1 ? 2 + k : 5));
}


template <int H>
static int launch_form(const EhFormArgs& args, cudaStream_t s) {
  constexpr int EX = (H >= 128) ? 1 : 128 / H;
  const int threads = (EX * H + 31) / 32 * 32;
  const size_t smem = (size_t)(threads + 1) * kRP * sizeof(float);
  dim3 grid((args.m.Nx + EX - 1) / EX, args.m.Ny, args.m.Nz);
  if (args.grad_f32)
    k_eh_form<H, float><<<grid, threads, smem, s>>>(args);
  else
    k_eh_form<H, __nv_bfloat16><<<grid, threads, smem, s>>>(args);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int launch_eh_form(const EhFormArgs& a, cudaStream_t s) {
  if (!a.grad_f32 && !a.Tb) {
    const int tc = launch_eh_form_tc(a, s);  // tcgen05 formation where it is built (h = 6, 8)
    if (tc != VDVC_ERR_UNSUPPORTED) return tc;
  }
  switch (a.m.h) {
    case 1: return launch_form<1>(a, s);
    case 2: return launch_form<2>(a, s);
    case 3: return launch_form<3>(a, s);
    case 4: return launch_form<4>(a, s);
    case 6: return launch_form<6>(a, s);
    case 8: return launch_form<8>(a, s);
    case 12: return launch_form<12>(a, s);
    case 16: return launch_form<16>(a, s);
  }
  return set_error(VDVC_ERR_UNSUPPORTED, "element Hessians for h=%d are not built (h in {1,2,3,4,6,8,12,16})", a.m.h);
}

// ---- TMA-staged element-Hessian matvec --------------------------------------
//
// T is stored tile-major, [tile][162][kEhTile]: a tile's 162 entry rows of
// kEhTile elements are one contiguous 41.5 KB span (20.7 KB for the BF16
// entries of the precision form, read into FP32 arithmetic).  A block owns one tile:
// one thread arms an mbarrier and issues a single bulk copy (cp.async.bulk)
// of the span into shared memory while every thread loads its element's
// nodal values; after the barrier each thread applies its element Hessian
// from shared memory (consecutive threads, consecutive words: no bank
// conflicts).  Five tiles in flight per SM keep the HBM stream of T deep
// without registers holding loads.  The wait is bounded; on a timeout the
// block raises *a.err, waits once more (bounded) for its copy and returns.
constexpr int kTile = kEhTile;

__device__ __forceinline__ float entry(const float* p) { return *p; }
__device__ __forceinline__ float entry(const __nv_bfloat16* p) { return __bfloat162float(*p); }

template <bool PCG, typename TT>
__global__ void __launch_bounds__(kTile) k_eh_matvec_tma(const EhMatvecArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TT* sT = (TT*)smem_raw;  // [162][kTile]
  const TT* Tg = std::is_same<TT, float>::value ? (const TT*)a.T : (const TT*)a.Tb;
  __shared__ __align__(8) uint64_t bar;
  if constexpr (PCG) {
    if (a.st->done) return;
  }
  const Mesh& m = a.m;
  const int t = threadIdx.x;
  const long long e0 = (long long)blockIdx.x * kTile;
  const int n_el = (int)min((long long)kTile, m.Ne - e0);
  constexpr uint32_t tile_bytes = 162u * kTile * sizeof(TT);
  if (t == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    mbar_arrive_expect_tx(&bar, tile_bytes);
    bulk_g2s(sT, Tg + (long long)blockIdx.x * 162 * kTile, tile_bytes, &bar);
  }
  __syncthreads();
  const long long e = e0 + t;
  const bool active = t < n_el;
  float vl[24];
  float beta = 0.f;
  if constexpr (PCG) beta = (float)a.st->beta;
  int ei = 0, ej = 0, ek = 0;
  if (active) {
    elem_ijk(m, e, ei, ej, ek);
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const long long node = (long long)(ei + corner_dx(b)) + (long long)(ej + corner_dy(b)) * m.Nnx +
                             (long long)(ek + corner_dz(b)) * m.NnxNny;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float val = __ldg(a.v + 3 * node + c);
        if constexpr (PCG) val += beta * __ldg(a.p_old + 3 * node + c);
        vl[3 * b + c] = val;
      }
    }
  }
  if (!mbar_wait_bounded(&bar, 0)) {
    if (t == 0) atomicExch(a.err, VDVC_ERR_TIMEOUT);
    mbar_wait_bounded(&bar, 0);
    return;
  }
  if (!active) return;
  float out[24];
#pragma unroll
  for (int r = 0; r < 24; ++r) out[r] = 0.f;
#pragma unroll
  for (int sx = 0; sx < 3; ++sx)
#pragma unroll
    for (int sy = 0; sy < 3; ++sy)
#pragma unroll
      for (int sz = 0; sz < 3; ++sz) {
        const int type = (sx * 3 + sy) * 3 + sz;
        float tv[6];
#pragma unroll
        for (int kl = 0; kl < 6; ++kl) tv[kl] = entry(sT + (type * 6 + kl) * kTile + t);
#pragma unroll
        for (int aa = 0; aa < 8; ++aa)
#pragma unroll
          for (int bb = 0; bb < 8; ++bb) {
            if (corner_dx(aa) + corner_dx(bb) != sx || corner_dy(aa) + corner_dy(bb) != sy ||
                corner_dz(aa) + corner_dz(bb) != sz)
              continue;
#pragma unroll
            for (int kk = 0; kk < 3; ++kk)
#pragma unroll
              for (int ll = 0; ll < 3; ++ll) out[3 * aa + kk] += tv[kl_index(kk, ll)] * vl[3 * bb + ll];
          }
      }
  if (a.nreg >= 1) {
#pragma unroll
    for (int aa = 0; aa < 8; ++aa)
#pragma unroll
      for (int bb = 0; bb < 8; ++bb) {
        const float lw = a.c1 * a.L8[aa * 8 + bb];
#pragma unroll
        for (int c = 0; c < 3; ++c) out[3 * aa + c] += lw * vl[3 * bb + c];
      }
    if (a.nreg == 2) {
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const long long node = (long long)(ei + corner_dx(b)) + (long long)(ej + corner_dy(b)) * m.Nnx +
                               (long long)(ek + corner_dz(b)) * m.NnxNny;
#pragma unroll
        for (int c = 0; c < 3; ++c) vl[3 * b + c] = a.w[3 * node + c];
      }
      // fully unrolled: a runtime row index would put out[] in local memory
#pragma unroll
      for (int r = 0; r < 24; ++r) {
        float s2 = 0.f;
#pragma unroll
        for (int q = 0; q < 24; ++q) s2 += __ldg(a.K2 + r * 24 + q) * vl[q];
        out[r] += a.c2 * s2;
      }
    }
  }
#pragma unroll
  for (int r = 0; r < 24; ++r) a.ev[(long long)r * m.Ne + e] = out[r];
}

// Elements rounded up to whole tiles (the T array holds 162 * eh_pitch floats).
long long eh_pitch(long long Ne) { return (Ne + kTile - 1) / kTile * kTile; }

template <bool PCG, typename TT>
static int launch_eh_matvec_t(const EhMatvecArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)162 * kTile * sizeof(TT);
  if (int st = ensure_dyn_smem((const void*)k_eh_matvec_tma<PCG, TT>, (int)smem)) return st;
  const long long nb = (a.m.Ne + kTile - 1) / kTile;
  k_eh_matvec_tma<PCG, TT><<<(unsigned)nb, kTile, smem, s>>>(a);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

template <bool PCG>
int launch_eh_matvec(const EhMatvecArgs& a, cudaStream_t s) {
  if ((((uintptr_t)a.T | (uintptr_t)a.Tb) & 15u)) return set_error(VDVC_ERR_ARG, "element Hessians misaligned");
  return a.Tb ? launch_eh_matvec_t<PCG, __nv_bfloat16>(a, s) : launch_eh_matvec_t<PCG, float>(a, s);
}
template int launch_eh_matvec<false>(const EhMatvecArgs&, cudaStream_t);
template int launch_eh_matvec<true>(const EhMatvecArgs&, cudaStream_t);

int launch_grad_bf16(const float* g, long long n, void* out, float* gmax, cudaStream_t s) {
  if (gmax) VDVC_CUDA(cudaMemsetAsync(gmax, 0, sizeof(float), s));
  k_grad_to_bf16<<<grid_blocks(n, 256, 152 * 32), 256, 0, s>>>(g, n, (__nv_bfloat16*)out, (unsigned int*)gmax);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

}  // namespace vdvc

using namespace vdvc;

extern "C" {

size_t vdvc_eh_workspace_bytes(int h, int Nx, int Ny, int Nz) {
  Mesh m;
  if (make_mesh(h, Nx, Ny, Nz, &m)) return 0;
  Carve cv(nullptr, 0);
  cv.take<float>((size_t)162 * eh_pitch(m.Ne));
  cv.take<float>((size_t)24 * m.Ne);
  cv.take<float>((size_t)24 * m.Ne);
  cv.take<int>(4);
  cv.take<uint16_t>((size_t)3 * m.Nvox);
  cv.take<float>(4);
  return cv.off + 256;
}

size_t vdvc_gn_eh_workspace_bytes(int precision, int h, int Nx, int Ny, int Nz) {
  Mesh m;
  if (make_mesh(h, Nx, Ny, Nz, &m)) return 0;
  if (precision != VDVC_PREC_MIXED && precision != VDVC_PREC_ELEMENT) return 0;
  // the solver's carve order: T, gmax, [BF16 gradient]
  Carve cv(nullptr, 0);
  cv.take<float>((size_t)162 * eh_pitch(m.Ne));
  cv.take<float>(4);
  if (precision == VDVC_PREC_MIXED) cv.take<uint16_t>((size_t)3 * m.Nvox);
  return cv.off + 256;
}

size_t vdvc_eh_bytes(int h, int Nx, int Ny, int Nz) {
  Mesh m;
  if (make_mesh(h, Nx, Ny, Nz, &m)) return 0;
  return (size_t)162 * eh_pitch(m.Ne) * sizeof(float);
}

size_t vdvc_eh_op_workspace_bytes(int h, int Nx, int Ny, int Nz) {
  Mesh m;
  if (make_mesh(h, Nx, Ny, Nz, &m)) return 0;
  Carve cv(nullptr, 0);
  cv.take<float>((size_t)24 * m.Ne);
  cv.take<int>(4);
  cv.take<float>(4);
  return cv.off + 256;
}

int vdvc_eh_form(const float* grad, int grad_bf16, const uint8_t* mask, int h, int Nx, int Ny, int Nz, float* T,
                 void* ws, size_t ws_bytes, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(h, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(grad && mask && T, "null pointer");
  VDVC_CHECK_ARG(grad_bf16 == 0 || grad_bf16 == 1, "grad_bf16 must be 0 or 1");
  VDVC_CHECK_ARG(((uintptr_t)T & 15u) == 0, "T must be 16-byte aligned");
  Carve cv(ws, ws_bytes);
  float* evD = cv.take<float>((size_t)24 * m.Ne);
  int* err = cv.take<int>(4);
  float* gmax = cv.take<float>(4);
  if (!ws || !cv.fits()) return set_error(VDVC_ERR_WORKSPACE, "eh_form needs %zu bytes of workspace", cv.off);
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  if (grad_bf16) VDVC_CUDA(cudaMemsetAsync(gmax, 0, sizeof(float), s));
  // the tensor-core formation needs max |g|, which only the solver's BF16
  // conversion records: this entry takes the CUDA-core formation
  EhFormArgs fa{m, grad, mask, T, evD, eh_pitch(m.Ne), nullptr, err, grad_bf16 ? 0 : 1};
  return launch_eh_form(fa, s);
}

int vdvc_eh_apply(const float* T, const float* v, int h, int Nx, int Ny, int Nz, float* out, void* ws,
                  size_t ws_bytes, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(h, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(T && v && out, "null pointer");
  VDVC_CHECK_ARG(((uintptr_t)T & 15u) == 0, "T must be 16-byte aligned");
  Carve cv(ws, ws_bytes);
  float* ev = cv.take<float>((size_t)24 * m.Ne);
  int* err = cv.take<int>(4);
  if (!ws || !cv.fits()) return set_error(VDVC_ERR_WORKSPACE, "eh_apply needs %zu bytes of workspace", cv.off);
  cudaStream_t s = (cudaStream_t)stream;
  EhMatvecArgs ma{};
  ma.m = m;
  ma.T = T;
  ma.pitch = eh_pitch(m.Ne);
  ma.err = err;
  ma.v = v;
  ma.ev = ev;
  if ((st = launch_eh_matvec<false>(ma, s))) return st;
  return launch_gather<float>(m, ev, out, s);
}

int vdvc_eh_status(void* ws, size_t ws_bytes, int h, int Nx, int Ny, int Nz, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(h, Nx, Ny, Nz, &m);
  if (st) return st;
  Carve cv(ws, ws_bytes);
  cv.take<float>((size_t)24 * m.Ne);
  int* err = cv.take<int>(4);
  if (!ws || !cv.fits()) return set_error(VDVC_ERR_WORKSPACE, "workspace of %zu bytes expected", cv.off);
  int h_err = 0;
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaStreamSynchronize(s));
  VDVC_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  if (h_err) return set_error(VDVC_ERR_TIMEOUT, "element-Hessian matvec: a bulk-copy wait timed out");
  return VDVC_OK;
}

int vdvc_matvec_H_mixed(const float* v, const float* grad, const uint8_t* mask, int h, int Nx, int Ny, int Nz,
                        float* out, void* ws, size_t ws_bytes, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(h, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(v && grad && mask && out, "null pointer");
  Carve cv(ws, ws_bytes);
  const long long pitch = eh_pitch(m.Ne);
  float* T = cv.take<float>((size_t)162 * pitch);
  float* evD = cv.take<float>((size_t)24 * m.Ne);
  float* ev = cv.take<float>((size_t)24 * m.Ne);
  int* err = cv.take<int>(4);
  uint16_t* gb = cv.take<uint16_t>((size_t)3 * m.Nvox);
  float* gmax = cv.take<float>(4);
  if (!ws || !cv.fits()) return set_error(VDVC_ERR_WORKSPACE, "mixed matvec needs %zu bytes of workspace", cv.off);
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  if ((st = launch_grad_bf16(grad, 3 * m.Nvox, gb, gmax, s))) return st;
  EhFormArgs fa{m, (const __nv_bfloat16*)gb, mask, T, evD, pitch, gmax, err, 0};
  if ((st = launch_eh_form(fa, s))) return st;
  EhMatvecArgs ma{};
  ma.m = m;
  ma.T = T;
  ma.pitch = pitch;
  ma.err = err;
  ma.v = v;
  ma.ev = ev;
  if ((st = launch_eh_matvec<false>(ma, s))) return st;
  if ((st = launch_gather<float>(m, ev, out, s))) return st;
  // the bulk-copy waits are bounded: report a timeout (never seen in practice)
  int h_err = 0;
  VDVC_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaStreamSynchronize(s));
  if (h_err) return set_error(VDVC_ERR_TIMEOUT, "element-Hessian matvec: a bulk-copy wait timed out");
  return VDVC_OK;
}

}  // extern "C"
