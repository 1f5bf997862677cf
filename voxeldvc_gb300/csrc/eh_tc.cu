// Element-Hessian formation of the precision form on the 5th-generation
// tensor cores (tcgen05 / TMEM), for h in {6, 8}.
//
// The 162 distinct entries of an element's 24x24 Hessian (mixed.cu) are
//   T_e[s][kl] = sum_q P[s][q] A_e[kl][q],   s = (sx, sy, sz) in 3^3,
// a contraction over the element's (h+1)^3 voxel-centre points q with
//   P[s][q]    = psi_sx(qx) psi_sy(qy) psi_sz(qz)        (the same for all elements)
//   A_e[kl][q] = w_q m_q g_k(q) g_l(q)                   (the element's data).
// Stacking 21 elements x 6 pairs kl as the 128 rows of A (126 used) gives one
// UMMA GEMM per tile: D[128 x 32] += A[128 x 64] B[64 x 32] per K-block of 64
// points, B = P^T (27 of 32 columns used), FP16 operands, FP32 accumulation
// in TMEM.  A point q of an element's block that another element owns
// (owner-computes: a shared face belongs to the element beyond it) and the
// padding points carry A = 0, so the per-element sums are those of the
// CUDA-core formation.
//
// Scaling: P is stored x 256 (its smallest non-zero value leaves the FP16
// subnormal range) and A x 2^(13 - floor(log2 max g^2)) (the largest g_k g_l
// becomes < 2^14); both are powers of two and undone exactly in the epilogue.
// A BF16 x BF16 product is exact in FP32; the FP16 rounding of A and P is
// the precision form's only extra rounding (2^-11 relative).
//
// Pipeline per CTA (256 threads, persistent over tiles): B resident in shared
// memory; A double-buffered; all threads build A[buf] from the BF16 gradient,
// fence it to the async proxy and sync; one thread issues the four K=16 MMAs
// and commits them to the buffer's mbarrier; a buffer is refilled only after
// its previous MMAs completed.  After a tile's last K-block every warp reads
// its TMEM lane quarter (tcgen05.ld 32x32b) and stores T.  Every mbarrier
// wait is bounded; on a timeout the CTA raises *err, waits (bounded) for its
// MMAs, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdlib>
#include <cstring>

#include "ops.cuh"
#include "tma.cuh"

namespace vdvc {

namespace {

__device__ __forceinline__ void tc_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] B[smem], kind::f16 (FP16 x FP16 -> FP32)
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// arrive on `bar` once every tcgen05 operation this thread issued so far has completed
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int c = 0; c < 16; ++c) v[c] = __uint_as_float(r[c]);
}

// Shared-memory matrix descriptor, no swizzle, K-major canonical layout:
// 8-row x 16-byte core matrices stored as 128 contiguous bytes; `lbo` = byte
// stride between core matrices adjacent along K, `sbo` = along M/N.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of the sm_100 family; base offset 0, no swizzle
  return d;
}

// Instruction descriptor of kind::f16: FP32 D, FP16 A and B, both K-major.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

constexpr int kThreads = 256;
constexpr int kElems = 21;  // elements per tile: 6 rows each in M = 128
constexpr int kRP = (kElems * 64 + kThreads - 1) / kThreads;  // points per thread per K-block
constexpr int kM = 128, kN = 32, kKB = 64;
constexpr uint32_t kAbytes = kM * kKB * 2;  // one A buffer: 16 KB
constexpr uint32_t kA_LBO = (kM / 8) * 128, kA_SBO = 128;
constexpr uint32_t kB_LBO = (kN / 8) * 128, kB_SBO = 128;

// byte offset of element (row, col) in a K-major no-swizzle tile with `groups` 8-row groups
__device__ __forceinline__ uint32_t kmajor_off(int row, int col, int groups) {
  return (uint32_t)((((col >> 3) * groups + (row >> 3)) << 7) + ((row & 7) << 4) + ((col & 7) << 1));
}

__device__ __forceinline__ float psi(int s, int q, float inv_h) {
  const float f1 = (float)q * inv_h, f0 = 1.f - f1;
  return s == 0 ? f0 * f0 : (s == 1 ? f0 * f1 : f1 * f1);
}

template <int H>
struct TcShape {
  static constexpr int Q1 = H + 1, NQ = Q1 * Q1 * Q1;
  static constexpr int NKB = (NQ + kKB - 1) / kKB, KPAD = NKB * kKB;
  static constexpr uint32_t Bbytes = (uint32_t)kN * KPAD * 2;
  // [A0][A1][B][q table: int2 per point][element table][2 mbarriers][TMEM address]
  static constexpr uint32_t offB = 2 * kAbytes, offQ = offB + Bbytes, offE = offQ + KPAD * 8;
  static constexpr uint32_t offBar = offE + kElems * 16, offTm = offBar + 16, smem = offTm + 16;
};

struct ElemInfo {
  long long vbase;  // voxel index of the element's q = 0 point, -1: past the mesh
  int flags;        // bit 0/1/2: last along x/y/z; bit 3/4/5: first along x/y/z
  int pad;
};

template <int H>
__global__ void __launch_bounds__(kThreads) k_eh_form_tc(const EhFormArgs a, long long ntiles) {
  using S = TcShape<H>;
  extern __shared__ __align__(1024) unsigned char smem[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const Mesh& m = a.m;
  int2* qtab = (int2*)(smem + S::offQ);
  ElemInfo* einfo = (ElemInfo*)(smem + S::offE);
  uint64_t* bar = (uint64_t*)(smem + S::offBar);
  uint32_t* tm_slot = (uint32_t*)(smem + S::offTm);
  const uint32_t sbase = smem_addr(smem);
  const float inv_h = 1.f / (float)H;

  // scale of A from the level's max |g| (device), undone in the epilogue
  const float gm = a.gmax ? *a.gmax : 0.f;
  const float g2 = gm * gm;
  int e2 = (g2 > 0.f && g2 < 3.0e38f) ? ilogbf(g2) : 0;
  e2 = max(-100, min(100, e2));
  const float scaleA = ldexpf(1.f, 13 - e2);
  const float unscale = ldexpf(1.f, e2 - 13 - 8);

  // B = 256 P^T, zero A buffers (rows 126, 127 stay zero), point table
  for (int idx = tid; idx < kN * S::KPAD; idx += kThreads) {
    const int n = idx / S::KPAD, q = idx - n * S::KPAD;
    float val = 0.f;
    if (n < 27 && q < S::NQ) {
      const int qx = q % S::Q1, qy = (q / S::Q1) % S::Q1, qz = q / (S::Q1 * S::Q1);
      val = 256.f * psi(n / 9, qx, inv_h) * psi((n / 3) % 3, qy, inv_h) * psi(n % 3, qz, inv_h);
    }
    *(__half*)(smem + S::offB + kmajor_off(n, q, kN / 8)) = __float2half_rn(val);
  }
  for (uint32_t o = tid * 16; o < 2 * kAbytes; o += kThreads * 16) *(uint4*)(smem + o) = make_uint4(0, 0, 0, 0);
  for (int q = tid; q < S::KPAD; q += kThreads) {
    int2 t{0, 0};
    if (q < S::NQ) {
      const int qx = q % S::Q1, qy = (q / S::Q1) % S::Q1, qz = q / (S::Q1 * S::Q1);
      t.x = (int)(qx + (long long)qy * m.Nvx + (long long)qz * m.NvxNvy);
      // face code: bit 0/1/2 on the far face (q = h) along x/y/z, bit 3/4/5 on the near face (q = 0)
      t.y = (qx == H) | ((qy == H) << 1) | ((qz == H) << 2) | ((qx == 0) << 3) | ((qy == 0) << 4) |
            ((qz == 0) << 5) | (1 << 15);
    }
    qtab[q] = t;
  }
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tc_alloc(tm_slot, 32);
    tc_relinquish();
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tm_slot;
  const uint32_t idesc = idesc_f16(kM, kN);
  const __nv_bfloat16* __restrict__ grad = (const __nv_bfloat16*)a.grad;

  int issued[2] = {0, 0};
  bool failed = false;
  long long kcount = 0;
  for (long long tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
    const long long e0 = tile * kElems;
    if (tid < kElems) {
      const long long e = e0 + tid;
      ElemInfo ei{-1, 0, 0};
      if (e < m.Ne) {
        const int i = (int)(e % m.Nx);
        const long long r = e / m.Nx;
        const int j = (int)(r % m.Ny), k = (int)(r / m.Ny);
        ei.vbase = (long long)i * H + (long long)j * H * m.Nvx + (long long)k * H * m.NvxNvy;
        ei.flags = (i == m.Nx - 1) | ((j == m.Ny - 1) << 1) | ((k == m.Nz - 1) << 2) | ((i == 0) << 3) |
                   ((j == 0) << 4) | ((k == 0) << 5);
      }
      einfo[tid] = ei;
    }
    __syncthreads();
    // A is filled in tasks of one element x one 8-point K chunk (a 16-byte
    // row segment per pair kl): thread t < 168 owns element t / 8, chunk t % 8
    // of every K-block.  Its 8 points' loads for the next K-block are issued
    // right after this block's stores, so they are in flight across the
    // barrier and the MMA issue.
    const bool tact = tid < kElems * 8;
    const int tel = tid >> 3, tch = tid & 7;
    const ElemInfo tei = tact ? einfo[tel] : ElemInfo{-1, 0, 0};
    const int kill = ~tei.flags & 7, half = tei.flags;
    float ng[8][3], nw[8];
    auto gather = [&](int kb) {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        ng[u][0] = ng[u][1] = ng[u][2] = 0.f;
        nw[u] = 0.f;
        const int2 tq = qtab[kb * kKB + tch * 8 + u];
        if (tei.vbase >= 0 && (tq.y >> 15) && !(tq.y & kill)) {
          const long long v = tei.vbase + tq.x;
          // scaleA / 2^(number of domain faces the point lies on): exponent decrement
          const float w = __int_as_float(__float_as_int(scaleA) - (__popc(tq.y & half & 63) << 23));
          nw[u] = a.mask[v] ? w : 0.f;
          const __nv_bfloat16* gp = grad + 3 * v;
          ng[u][0] = __bfloat162float(gp[0]);
          ng[u][1] = __bfloat162float(gp[1]);
          ng[u][2] = __bfloat162float(gp[2]);
        }
      }
    };
    gather(0);
    int last_buf = 0;
    for (int kb = 0; kb < S::NKB; ++kb, ++kcount) {
      const int buf = (int)(kcount & 1);
      if (issued[buf] > 0) {
        const bool ok = mbar_wait_bounded(&bar[buf], (uint32_t)((issued[buf] - 1) & 1));
        if (__syncthreads_or(!ok)) {
          failed = true;
          break;
        }
      }
      unsigned char* A = smem + buf * kAbytes;
      if (tact) {
#pragma unroll
        for (int kl = 0; kl < 6; ++kl) {
          const int k0 = kl < 3 ? 0 : (kl < 5 ? 1 : 2);
          const int k1 = kl == 0 ? 0 : (kl == 1 || kl == 3 ? 1 : 2);
          uint32_t pk[4];
#pragma unroll
          for (int u = 0; u < 8; u += 2) {
            const __half2 h2 = __floats2half2_rn(nw[u] * (ng[u][k0] * ng[u][k1]),
                                                 nw[u + 1] * (ng[u + 1][k0] * ng[u + 1][k1]));
            pk[u >> 1] = *(const uint32_t*)&h2;
          }
          *(uint4*)(A + kmajor_off(6 * tel + kl, tch * 8, kM / 8)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
      if (kb + 1 < S::NKB && tact) gather(kb + 1);
      fence_proxy_async_smem();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint32_t a_addr = sbase + buf * kAbytes, b_addr = sbase + S::offB;
#pragma unroll
        for (int t = 0; t < kKB / 16; ++t) {
          const uint64_t ad = smem_desc(a_addr + t * 2 * kA_LBO, kA_LBO, kA_SBO);
          const uint64_t bd = smem_desc(b_addr + (kb * (kKB / 8) + 2 * t) * kB_LBO, kB_LBO, kB_SBO);
          tc_mma(tmem, ad, bd, idesc, (kb > 0 || t > 0) ? 1u : 0u);
        }
        tc_commit(&bar[buf]);
      }
      ++issued[buf];
      last_buf = buf;
    }
    if (failed) break;
    // tile epilogue: wait for the accumulator, read this warp's lane quarter
    const bool ok = mbar_wait_bounded(&bar[last_buf], (uint32_t)((issued[last_buf] - 1) & 1));
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    tc_fence_after();
    const int row = 32 * (warp & 3) + lane, c0 = 16 * (warp >> 2);
    float d[16];
    tc_ld16(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)c0, d);
    tc_fence_before();
    const int el = row / 6, kl = row - 6 * (row / 6);
    const long long eg = e0 + el;
    if (el < kElems && eg < m.Ne) {
      const long long tbase = (eg / kEhTile) * 162 * kEhTile + (eg % kEhTile);
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int s = c0 + c;
        if (s < 27) {
          const float val = d[c] * unscale;
          a.T[tbase + (long long)(s * 6 + kl) * kEhTile] = val;
          const int sx = s / 9, sy = (s / 3) % 3, sz = s % 3;
          if (!(sx & 1) && !(sy & 1) && !(sz & 1) && (kl == 0 || kl == 3 || kl == 5)) {
            const int corner = corner_of(sx >> 1, sy >> 1, sz >> 1);
            const int kk = kl == 0 ? 0 : (kl == 3 ? 1 : 2);
            a.evD[(long long)(3 * corner + kk) * m.Ne + eg] = val;
          }
        }
      }
    }
  }
  if (failed) {
    if (tid == 0) atomicExch(a.err, (int)VDVC_ERR_TIMEOUT);
    // let any MMA still in flight finish before the TMEM is released
    for (int b = 0; b < 2; ++b)
      if (issued[b] > 0) mbar_wait_bounded(&bar[b], (uint32_t)((issued[b] - 1) & 1));
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tc_dealloc(tmem, 32);
  }
}

template <int H>
int launch_tc(const EhFormArgs& a, cudaStream_t s) {
  using S = TcShape<H>;
  if (int st = ensure_dyn_smem((const void*)k_eh_form_tc<H>, (int)S::smem)) return st;
  const long long ntiles = (a.m.Ne + kElems - 1) / kElems;
  const long long grid = ntiles < 2 * 152 ? ntiles : 2 * 152;
  k_eh_form_tc<H><<<(unsigned)grid, kThreads, S::smem, s>>>(a, ntiles);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

}  // namespace

// Tensor-core formation when selected (VDVC_EH_FORM=tc) and built for the
// element size (h in {6, 8}); returns VDVC_ERR_UNSUPPORTED otherwise so the
// caller runs the CUDA-core formation.  The CUDA-core formation is the
// default: it reads each voxel once, coalesced, in one pass, while this
// kernel's per-point gathers into the A tiles are latency bound (at 513^3,
// h = 8: about 2.2 ms against 0.65 ms per formation on a GB300).
int launch_eh_form_tc(const EhFormArgs& a, cudaStream_t s) {
  const char* env = getenv("VDVC_EH_FORM");
  if (!env || strcmp(env, "tc") != 0 || !a.gmax || !a.err) return VDVC_ERR_UNSUPPORTED;
  if (a.m.h == 8) return launch_tc<8>(a, s);
  if (a.m.h == 6) return launch_tc<6>(a, s);
  return VDVC_ERR_UNSUPPORTED;
}

}  // namespace vdvc
