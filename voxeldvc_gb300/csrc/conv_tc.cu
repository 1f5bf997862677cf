// 3x3x3 gather convolutions (include/vdvc_cnn.h) on the 5th-generation
// tensor cores: tcgen05.mma kind::f16 (BF16 x BF16 -> FP32 in TMEM).
//
// GEMM view: D[p][n] = sum_K A[p][K] B[n][K], with p the output positions
// (M = 128 per CTA), n the output channels (N = n_out rounded up to 16) and
// K = (tap t, input channel c) in the order t * cin + c -- the order of the
// packed forward weights [n_pad][27][cin] and of the input-gradient weights
// [cin_pad][27][n_pad16], so both read unchanged.
//
// The kernels share the epilogue (TMEM -> registers, bias, ReLU, BF16 or
// FP32 stores, each warp its 32 lanes = 32 positions):
//
// k_conv_tma, k_conv_tma_p -- geometries with a unit source step (d = 1:
// every forward convolution, stride 1 or 2, and the input gradient of a
// stride-1 one).
// The CTA's 128 positions are an 8 x 4 x 4 brick of the output grid, so for
// tap t and a block of CB input channels the A operand is one box of a 4-D
// tensor map over the channels-last source (channel, x, y, z): the box starts
// at q = a * brick origin + b + c * t per axis, walks the source with element
// step a (the convolution stride), and TMA fills positions outside the
// source with zeros -- the padding.  B is a box of the packed weights.  Both
// land in the 128-byte (CB = 64) or 64-byte (CB = 32) swizzled K-major
// layout the MMA descriptors name.  One thread issues the copies, another
// the MMAs; full/empty mbarriers per stage, no CTA-wide barrier in the main
// loop.  k_conv_tma_p is the persistent form (two CTAs per SM walking the
// bricks, two TMEM accumulators so that a brick's epilogue runs under the
// next brick's main loop), used for N >= 32.
//
// k_conv_first -- the 2-channel first layer (K = 54), its A tile built in
// shared memory from the brick's source halo (below).
//
// k_conv_tc -- the other geometries (input gradients of stride-2 layers,
// d = 2) and channel counts that are multiples of 8 but not of 32.  A K-block
// is 64 K values = eight 16-byte chunks of 8 channels; a chunk of row p is
// 16 contiguous bytes of the source at position q(p, t) (zero when q falls
// outside), copied by cp.async into the no-swizzle K-major layout (8-row x
// 16-byte core matrices); B rows past the packed rows and K past 27 * cin
// are zero-filled the same way (src-size 0).  kStages stages; every thread
// copies its own A row and a share of B, the CTA syncs, one thread issues
// the MMAs and commits them to the stage's mbarrier.
//
// Every mbarrier wait is bounded: on a timeout the CTA sets *err, skips its
// stores, waits (bounded) for its copies and MMAs in flight, frees its TMEM
// and returns; the host reports VDVC_ERR_TIMEOUT.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <mutex>

#include "ops.cuh"
#include "tma.cuh"
#include "vdvc_cnn.h"

namespace vdvc {
namespace {

typedef __nv_bfloat16 bf16;

constexpr int kThreads = 128;
constexpr int kM = 128;
constexpr int kStages = 3;  // 3 stages: 8 % faster network than 4 (more CTAs per SM), same as 2 within 3 %
constexpr uint32_t kAStage = kM * 64 * 2;  // 16 KB

struct TcGeo {
  int nx, ny, nz, sx, sy, sz, a, b, c, d;
};

__device__ __forceinline__ int tap_src(int p, int t, int a, int b, int c, int d, int S) {
  int num = p * a + b + t * c;
  if (num < 0) return -1;
  if (d != 1) {
    if (num % d) return -1;
    num /= d;
  }
  return num < S ? num : -1;
}

__device__ __forceinline__ void cp16(uint32_t dst, const void* src, uint32_t nbytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(nbytes) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

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

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

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

// no-swizzle K-major shared-memory descriptor (sm_100 family, version 1)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// kind::f16 instruction descriptor: FP32 D, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of 16-byte chunk `ch` (0..7) of row `row` in a K-major tile of
// `rows` rows: core matrix (row / 8, ch) at (ch * rows / 8 + row / 8) * 128
__device__ __forceinline__ uint32_t chunk_off(int row, int ch, int rows) {
  return (uint32_t)(((ch * (rows >> 3) + (row >> 3)) << 7) + ((row & 7) << 4));
}

// epilogue parameters (both kernels)
struct Epi {
  const float* bias;
  int n_out, NT;  // NT: n_out rounded up to 16
  int relu, out_f32, ocs, ocoff, accumulate;
  void* out;
};

// Reads this warp's 32 accumulator rows (lane = row) and stores row `pr`
// (when `valid`): bias, ReLU, then BF16 (optionally added to the output) or
// FP32.  Every lane of the warp calls it (tcgen05.ld is warp-collective).
__device__ __forceinline__ void store_rows(uint32_t tmem, int warp, bool valid, long long pr, const Epi& E) {
  // BF16 output in 16-byte pieces where a 16-channel group is whole and
  // aligned (channel stride and offset multiples of 8: every layer here)
  const bool vec_out = !E.out_f32 && (E.ocs % 8) == 0 && (E.ocoff % 8) == 0 && ((uintptr_t)E.out & 15) == 0;
  for (int c0 = 0; c0 < E.NT; c0 += 16) {
    float v[16];
    tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
    if (!valid) continue;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const int n = c0 + c;
      float x = v[c];
      if (E.bias && n < E.n_out) x += E.bias[n];
      if (E.relu) x = fmaxf(x, 0.f);
      v[c] = x;
    }
    const long long o = pr * E.ocs + E.ocoff + c0;
    // fixed trip counts with a predicate: a data-dependent bound would
    // index v[] at run time and move it to local memory
    if (E.out_f32) {
      float* op = (float*)E.out + o;
#pragma unroll
      for (int c = 0; c < 16; ++c)
        if (c0 + c < E.n_out) op[c] = v[c];
    } else if (vec_out && c0 + 16 <= E.n_out) {
      uint4* op = (uint4*)((bf16*)E.out + o);
      uint32_t w[8];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        if (E.accumulate) {
          const uint4 old = op[q];
          const uint32_t ow[4] = {old.x, old.y, old.z, old.w};
#pragma unroll
          for (int c = 0; c < 8; c += 2) {
            v[8 * q + c] += __uint_as_float(ow[c / 2] << 16);
            v[8 * q + c + 1] += __uint_as_float(ow[c / 2] & 0xFFFF0000u);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < 16; c += 2) {
        const __nv_bfloat162 b2 = __floats2bfloat162_rn(v[c], v[c + 1]);
        w[c / 2] = *reinterpret_cast<const uint32_t*>(&b2);
      }
      op[0] = make_uint4(w[0], w[1], w[2], w[3]);
      op[1] = make_uint4(w[4], w[5], w[6], w[7]);
    } else {
      bf16* op = (bf16*)E.out + o;
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        if (c0 + c >= E.n_out) continue;
        float x = v[c];
        if (E.accumulate) x += __bfloat162float(op[c]);
        op[c] = __float2bfloat16_rn(x);
      }
    }
  }
}

struct ConvTcArgs {
  const bf16* src;
  int scs, scoff, cin;
  const bf16* w;  // [wrows][27 * cin]
  int wrows;      // packed weight rows (>= n_out)
  Epi e;
  TcGeo g;
  int* err;
};

__global__ void __launch_bounds__(kThreads) k_conv_tc(const ConvTcArgs A) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int NT = A.e.NT;
  const uint32_t bstage = (uint32_t)NT * 128;
  unsigned char* sA = smem;
  unsigned char* sB = smem + kStages * kAStage;
  uint64_t* bars = (uint64_t*)(sB + kStages * bstage);  // kStages mbarriers
  uint32_t* s_tmem = (uint32_t*)(bars + kStages);
  int* s_fail = (int*)(s_tmem + 1);
  int* s_last = s_fail + 1;  // last K-block whose MMAs were committed

  const TcGeo& g = A.g;
  const long long npos = (long long)g.nx * g.ny * g.nz;
  const long long p = (long long)blockIdx.x * kM + tid;  // this thread's A row
  const bool prow = p < npos;
  int px = 0, py = 0, pz = 0;
  if (prow) {
    px = (int)(p % g.nx);
    const long long r = p / g.nx;
    py = (int)(r % g.ny);
    pz = (int)(r / g.ny);
  }
  const int cpt = A.cin >> 3;           // 16-byte chunks per tap
  const int nchunks = 27 * cpt;         // K chunks with data
  const int nkb = (nchunks + 7) >> 3;   // K-blocks of 64
  const long long krow = 27LL * A.cin;  // packed weight row length

  uint32_t ncols = 32;
  while ((int)ncols < NT) ncols <<= 1;
  if (warp == 0) {
    tc_alloc(s_tmem, ncols);
    tc_relinquish();
  }
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
    *s_fail = 0;
    *s_last = -1;
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *s_tmem;
  const uint32_t idesc = idesc_bf16(kM, NT);
  const uint32_t aLBO = (kM / 8) * 128, bLBO = (uint32_t)(NT / 8) * 128;

  // issue the copies of K-block kb into stage st
  auto load_stage = [&](int kb, int st) {
    const uint32_t a0 = smem_addr(sA + st * kAStage);
    int last_t = -1;
    long long si = -1;
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
      const int kc = kb * 8 + ch;
      const bf16* srcp = A.src;
      uint32_t nb = 0;
      if (prow && kc < nchunks) {
        const int t = kc / cpt;
        if (t != last_t) {
          last_t = t;
          const int qx = tap_src(px, t % 3, g.a, g.b, g.c, g.d, g.sx);
          const int qy = tap_src(py, (t / 3) % 3, g.a, g.b, g.c, g.d, g.sy);
          const int qz = tap_src(pz, t / 9, g.a, g.b, g.c, g.d, g.sz);
          si = (qx < 0 || qy < 0 || qz < 0) ? -1 : ((long long)qz * g.sy + qy) * g.sx + qx;
        }
        if (si >= 0) {
          srcp = A.src + si * A.scs + A.scoff + (kc - t * cpt) * 8;
          nb = 16;
        }
      }
      cp16(a0 + chunk_off(tid, ch, kM), srcp, nb);
    }
    const uint32_t b0 = smem_addr(sB + st * bstage);
    for (int q = tid; q < NT * 8; q += kThreads) {
      const int n = q >> 3, ch = q & 7;
      const int kc = kb * 8 + ch;
      const bf16* srcp = A.w;
      uint32_t nb = 0;
      if (n < A.wrows && kc < nchunks) {
        srcp = A.w + (long long)n * krow + (long long)kc * 8;
        nb = 16;
      }
      cp16(b0 + chunk_off(n, ch, NT), srcp, nb);
    }
  };

  bool ok = true;
  // prologue: kStages - 1 K-blocks in flight
  for (int kb = 0; kb < kStages - 1; ++kb) {
    if (kb < nkb) load_stage(kb, kb);
    cp_commit();
  }
  for (int kb = 0; kb < nkb; ++kb) {
    // refill: K-block kb + kStages - 1 into the stage K-block kb - 1 used
    const int nk = kb + kStages - 1;
    if (nk < nkb) {
      const int st = nk % kStages;
      if (nk >= kStages) {
        // that stage's previous MMAs (K-block nk - kStages) must be done
        if (!mbar_wait_bounded(&bars[st], (uint32_t)((nk / kStages - 1) & 1))) ok = false;
      }
      load_stage(nk, st);
    }
    cp_commit();
    cp_wait<kStages - 1>();  // this thread's copies of K-block kb have landed
    fence_proxy_async_smem();
    __syncthreads();
    if (__syncthreads_or(!ok)) {
      if (tid == 0) *s_fail = 1;
      break;
    }
    if (tid == 0) {
      tc_fence_after();
      const int st = kb % kStages;
      const uint32_t a0 = smem_addr(sA + st * kAStage), b0 = smem_addr(sB + st * bstage);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const uint64_t ad = smem_desc(a0 + kk * 2 * aLBO, aLBO, 128);
        const uint64_t bd = smem_desc(b0 + kk * 2 * bLBO, bLBO, 128);
        tc_mma(tmem, ad, bd, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
      }
      tc_commit(&bars[st]);
      *s_last = kb;
    }
  }
  cp_wait<0>();
  __syncthreads();
  // the last commit covers every MMA issued before it
  const int lastkb = *s_last;
  if (lastkb < nkb - 1) ok = false;
  if (lastkb >= 0 && !mbar_wait_bounded(&bars[lastkb % kStages], (uint32_t)((lastkb / kStages) & 1))) ok = false;
  tc_fence_after();
  __syncthreads();
  const bool fail = __syncthreads_or(!ok) || *s_fail;
  if (!fail) {
    const long long pr = (long long)blockIdx.x * kM + warp * 32 + lane;
    store_rows(tmem, warp, pr < npos, pr, A.e);
  } else if (tid == 0) {
    atomicExch(A.err, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tc_dealloc(tmem, ncols);
  }
}

// ---------------------------------------------------------------------------
// k_conv_tma

constexpr int kBX = 8, kBY = 4, kBZ = 4;  // output brick = the 128 GEMM rows
static_assert(kBX * kBY * kBZ == kM, "a brick is one M tile");
constexpr int kTmaMaxStages = 8;
constexpr uint32_t kTmaStageBudget = 96 * 1024;  // stages of two CTAs fit one SM

struct ConvTmaArgs {
  int nx, ny, nz;  // output grid
  int nbx, nby;    // bricks along x and y
  int a, b, c;     // source coordinate a * p + b + c * tap, per axis
  int cin, scoff;  // input channels, their offset in the source's channel stride
  int ncb, nkb;    // channel blocks per tap, K-blocks (27 * ncb)
  int stages;
  Epi e;
  int* err;
};

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}

// K-major descriptor of rows of CB * 2 bytes in the swizzled layout TMA
// writes (8-row atoms: 1024 B for the 128-byte swizzle, 512 B for 64-byte);
// the leading-byte offset is unused for swizzled K-major operands.
template <int CB>
__device__ __forceinline__ uint64_t sw_desc(uint32_t saddr) {
  constexpr uint32_t sbo = 8u * CB * 2u;
  constexpr uint64_t layout = CB == 64 ? 2 : 4;  // SWIZZLE_128B : SWIZZLE_64B
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= layout << 61;
  return d;
}

// Bounded wait (at most 2^22 polls).  Every 256 polls it also gives up once
// the CTA's other role thread has aborted (`abort`, when given) or -- after
// `patience` polls -- once any CTA of the launch has reported a failure in
// *gerr, so that one stuck CTA does not make every other one sit out its
// own full limit.
__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, uint32_t parity, volatile int* abort, volatile int* gerr,
                                              long long patience) {
  for (long long i = 0; i < (1LL << 22); ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255) == 255 && ((abort && *abort) || (i >= patience && *gerr))) return false;
  }
  return false;
}

template <int CB>
__global__ void __launch_bounds__(kThreads) k_conv_tma(const __grid_constant__ CUtensorMap tmA,
                                                       const __grid_constant__ CUtensorMap tmB, const ConvTmaArgs P) {
  extern __shared__ unsigned char smem_raw[];
  // the swizzle atoms need 1024-byte aligned stages
  const uint32_t raw = smem_addr(smem_raw);
  unsigned char* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int S = P.stages, NT = P.e.NT;
  volatile int* gerr = P.err;
  constexpr uint32_t aBytes = (uint32_t)kM * CB * 2;
  const uint32_t stageBytes = aBytes + (uint32_t)NT * CB * 2;
  uint64_t* full = (uint64_t*)(smem + S * stageBytes);
  uint64_t* empty = full + S;
  uint64_t* done = empty + S;
  uint32_t* s_tmem = (uint32_t*)(done + 1);
  volatile int* s_abort = (volatile int*)(s_tmem + 1);
  int* s_cnt = (int*)(s_tmem + 2);  // [0] K-blocks whose copies were issued, [1] consumed by MMAs

  uint32_t ncols = 32;
  while ((int)ncols < NT) ncols <<= 1;
  if (warp == 0) {
    tc_alloc(s_tmem, ncols);
    tc_relinquish();
  }
  if (tid == 32) {
    for (int st = 0; st < S; ++st) {
      mbar_init(&full[st], 1);
      mbar_init(&empty[st], 1);
    }
    mbar_init(done, 1);
    *s_abort = 0;
    s_cnt[0] = s_cnt[1] = 0;
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *s_tmem;

  const int bid = blockIdx.x;
  const int x0 = (bid % P.nbx) * kBX, y0 = ((bid / P.nbx) % P.nby) * kBY, z0 = (bid / (P.nbx * P.nby)) * kBZ;

  if (tid == 0) {
    // producer: the A box and the B box of each K-block into its stage
    int kb = 0;
    for (; kb < P.nkb; ++kb) {
      const int st = kb % S;
      if (kb >= S && !wait_or_abort(&empty[st], (uint32_t)((kb / S - 1) & 1), s_abort, gerr, 0)) {
        *s_abort = 1;
        atomicExch(P.err, 1);
        break;
      }
      const int t = kb / P.ncb, cb = kb - t * P.ncb;
      const int tx = t % 3, ty = (t / 3) % 3, tz = t / 9;
      const uint32_t sa = smem_addr(smem + st * stageBytes), fb = smem_addr(&full[st]);
      mbar_arrive_expect_tx(&full[st], stageBytes);
      tma_load_4d(sa, &tmA, P.scoff + cb * CB, P.a * x0 + P.b + P.c * tx, P.a * y0 + P.b + P.c * ty,
                  P.a * z0 + P.b + P.c * tz, fb);
      tma_load_2d(sa + aBytes, &tmB, t * P.cin + cb * CB, 0, fb);
    }
    s_cnt[0] = kb;
  } else if (tid == 32) {
    // MMA issuer: CB / 16 MMAs of K = 16 per K-block, the stage released by
    // the commit once they have read it
    const uint32_t idesc = idesc_bf16(kM, NT);
    int kb = 0;
    for (; kb < P.nkb; ++kb) {
      const int st = kb % S;
      if (!wait_or_abort(&full[st], (uint32_t)((kb / S) & 1), s_abort, gerr, 0)) {
        *s_abort = 1;
        atomicExch(P.err, 1);
        break;
      }
      tc_fence_after();
      const uint32_t sa = smem_addr(smem + st * stageBytes);
#pragma unroll
      for (int kk = 0; kk < CB / 16; ++kk)
        tc_mma(tmem, sw_desc<CB>(sa + kk * 32), sw_desc<CB>(sa + aBytes + kk * 32), idesc,
               (kb > 0 || kk > 0) ? 1u : 0u);
      tc_commit(&empty[st]);
    }
    s_cnt[1] = kb;
    tc_commit(done);  // tracks every MMA issued before it
  }
  __syncwarp();
  // the MMAs issued so far always complete: no early exit on *gerr
  bool ok = wait_or_abort(done, 0, nullptr, gerr, 1LL << 22);
  tc_fence_after();
  __syncthreads();
  // after an abort: copies issued but never consumed must land before exit
  // (a copy lands within microseconds; past 2^14 polls with a failure
  // reported it is taken as stuck)
  if (tid == 0)
    for (int kb = s_cnt[1]; kb < s_cnt[0]; ++kb)
      if (!wait_or_abort(&full[kb % S], (uint32_t)((kb / S) & 1), nullptr, gerr, 1LL << 14)) ok = false;
  const bool fail = __syncthreads_or(!ok || *s_abort != 0 || s_cnt[1] < P.nkb);
  if (!fail) {
    const int r = warp * 32 + lane;
    const int x = x0 + r % kBX, y = y0 + (r / kBX) % kBY, z = z0 + r / (kBX * kBY);
    store_rows(tmem, warp, x < P.nx && y < P.ny && z < P.nz, ((long long)z * P.ny + y) * P.nx + x, P.e);
  } else if (tid == 0) {
    atomicExch(P.err, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tc_dealloc(tmem, ncols);
  }
}

// ---------------------------------------------------------------------------
// k_conv_tma_p: the same convolution as a persistent kernel, two CTAs per SM
// each walking bricks blockIdx.x, blockIdx.x + gridDim.x, ...  Warp 0's lane 0
// issues the copies of every K-block of every brick through a ring of S
// stages (it never waits for a brick to finish), warp 1's lane 0 issues the
// MMAs into one of two TMEM accumulators (alternating per brick), and warps
// 2-5 (one per TMEM lane quarter) read a finished accumulator, store it and
// hand it back -- a brick's epilogue runs under the next brick's main loop.
// Barriers: full/empty per stage, accumulator full (MMA commit) / empty (one
// arrival per epilogue warp) per accumulator.  Every wait is bounded and
// gives up once the CTA or the launch has reported a failure; copies and
// MMAs in flight are drained (bounded) before the TMEM is freed.

constexpr int kPThreads = 192;
constexpr uint32_t kPStageBudget = 96 * 1024;
constexpr int kPMaxStages = 12;

template <int CB>
__global__ void __launch_bounds__(kPThreads, 2) k_conv_tma_p(const __grid_constant__ CUtensorMap tmA,
                                                             const __grid_constant__ CUtensorMap tmB,
                                                             const ConvTmaArgs P, int ntiles) {
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = smem_addr(smem_raw);
  unsigned char* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int S = P.stages, NT = P.e.NT;
  volatile int* gerr = P.err;
  constexpr uint32_t aBytes = (uint32_t)kM * CB * 2;
  const uint32_t stageBytes = aBytes + (uint32_t)NT * CB * 2;
  uint64_t* full = (uint64_t*)(smem + S * stageBytes);
  uint64_t* empty = full + S;
  uint64_t* accf = empty + S;  // [2]
  uint64_t* acce = accf + 2;   // [2]
  uint64_t* done = acce + 2;
  uint32_t* s_tmem = (uint32_t*)(done + 1);
  volatile int* s_abort = (volatile int*)(s_tmem + 1);
  int* s_cnt = (int*)(s_tmem + 2);  // [0] K-blocks whose copies were issued, [1] consumed by MMAs

  uint32_t ncols = 32;
  while ((int)ncols < 2 * NT) ncols <<= 1;
  if (warp == 0) {
    tc_alloc(s_tmem, ncols);
    tc_relinquish();
  }
  if (tid == 32) {
    for (int st = 0; st < S; ++st) {
      mbar_init(&full[st], 1);
      mbar_init(&empty[st], 1);
    }
    for (int q = 0; q < 2; ++q) {
      mbar_init(&accf[q], 1);
      mbar_init(&acce[q], 4);
    }
    mbar_init(done, 1);
    *s_abort = 0;
    s_cnt[0] = s_cnt[1] = 0;
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *s_tmem;
  const int nkb = P.nkb;

  if (tid == 0) {
    // producer
    int g = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
      const int x0 = (tile % P.nbx) * kBX, y0 = ((tile / P.nbx) % P.nby) * kBY, z0 = (tile / (P.nbx * P.nby)) * kBZ;
      for (int kb = 0; kb < nkb; ++kb, ++g) {
        const int st = g % S;
        if (g >= S && !wait_or_abort(&empty[st], (uint32_t)((g / S - 1) & 1), s_abort, gerr, 0)) {
          *s_abort = 1;
          atomicExch(P.err, 1);
          ok = false;
          break;
        }
        const int t = kb / P.ncb, cb = kb - t * P.ncb;
        const int tx = t % 3, ty = (t / 3) % 3, tz = t / 9;
        const uint32_t sa = smem_addr(smem + st * stageBytes), fb = smem_addr(&full[st]);
        mbar_arrive_expect_tx(&full[st], stageBytes);
        tma_load_4d(sa, &tmA, P.scoff + cb * CB, P.a * x0 + P.b + P.c * tx, P.a * y0 + P.b + P.c * ty,
                    P.a * z0 + P.b + P.c * tz, fb);
        tma_load_2d(sa + aBytes, &tmB, t * P.cin + cb * CB, 0, fb);
      }
    }
    s_cnt[0] = g;
  } else if (tid == 32) {
    // MMA issuer
    const uint32_t idesc = idesc_bf16(kM, NT);
    int g = 0, it = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++it) {
      const int acc = it & 1;
      if (it >= 2 && !wait_or_abort(&acce[acc], (uint32_t)((it / 2 - 1) & 1), s_abort, gerr, 0)) {
        *s_abort = 1;
        atomicExch(P.err, 1);
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)(acc * NT);
      for (int kb = 0; kb < nkb; ++kb, ++g) {
        const int st = g % S;
        if (!wait_or_abort(&full[st], (uint32_t)((g / S) & 1), s_abort, gerr, 0)) {
          *s_abort = 1;
          atomicExch(P.err, 1);
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t sa = smem_addr(smem + st * stageBytes);
#pragma unroll
        for (int kk = 0; kk < CB / 16; ++kk)
          tc_mma(d, sw_desc<CB>(sa + kk * 32), sw_desc<CB>(sa + aBytes + kk * 32), idesc,
                 (kb > 0 || kk > 0) ? 1u : 0u);
        tc_commit(&empty[st]);
      }
      if (ok) tc_commit(&accf[acc]);
    }
    s_cnt[1] = g;
    tc_commit(done);  // tracks every MMA issued before it
  } else if (warp >= 2) {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31
    const int q = warp & 3;
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
      const int acc = it & 1;
      if (!wait_or_abort(&accf[acc], (uint32_t)((it / 2) & 1), s_abort, gerr, 0)) break;
      tc_fence_after();
      const int x0 = (tile % P.nbx) * kBX, y0 = ((tile / P.nbx) % P.nby) * kBY, z0 = (tile / (P.nbx * P.nby)) * kBZ;
      const int r = q * 32 + lane;
      const int x = x0 + r % kBX, y = y0 + (r / kBX) % kBY, z = z0 + r / (kBX * kBY);
      store_rows(tmem + (uint32_t)(acc * NT), q, x < P.nx && y < P.ny && z < P.nz,
                 ((long long)z * P.ny + y) * P.nx + x, P.e);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[acc]);
    }
  }
  __syncwarp();
  // MMAs issued so far always complete: no early exit on *gerr
  bool ok = wait_or_abort(done, 0, nullptr, gerr, 1LL << 22);
  tc_fence_after();
  __syncthreads();
  if (tid == 0)
    for (int g = s_cnt[1]; g < s_cnt[0]; ++g)
      if (!wait_or_abort(&full[g % S], (uint32_t)((g / S) & 1), nullptr, gerr, 1LL << 14)) ok = false;
  const bool fail = __syncthreads_or(!ok || *s_abort != 0);
  if (fail && tid == 0) atomicExch(P.err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tc_dealloc(tmem, ncols);
  }
}

// ---------------------------------------------------------------------------
// k_conv_first: the 2-channel first layer (stride 1, K = 27 taps x 2
// channels = 54, padded to 64) on the tensor cores.  Per CTA one 8 x 4 x 4
// brick: the brick's 10 x 6 x 6 source halo (2 BF16 channels = one 32-bit
// word per position, zero outside the volume: the padding) is loaded once
// into shared memory, the 128 x 64 A tile is built from it there (row =
// position, K = 2 t + c as the packed first-layer weights [n_pad8][64]
// order it; one 16-byte chunk = 4 taps), B (<= 64 x 64) is staged from the
// packed weights, and one thread issues the four K = 16 MMAs into TMEM.
// No per-row or per-tap copies: the layer's whole input footprint is read
// about once per brick instead of 27 times.

constexpr int kHX = kBX + 2, kHY = kBY + 2, kHZ = kBZ + 2;  // halo of a brick
constexpr int kHalo = kHX * kHY * kHZ;                      // 360 positions

struct ConvFirstArgs {
  const uint32_t* src;  // 2 BF16 channels per position (channel stride 2)
  const bf16* w;        // [wrows][64]
  int wrows;
  int nx, ny, nz, nbx, nby;
  Epi e;
  int* err;
};

__global__ void __launch_bounds__(kThreads) k_conv_first(const ConvFirstArgs P) {
  __shared__ __align__(128) unsigned char sA[kM * 64 * 2];  // 16 KB, no-swizzle K-major
  __shared__ __align__(128) unsigned char sB[64 * 64 * 2];  // up to 64 rows
  __shared__ uint32_t sH[kHalo];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int NT = P.e.NT;
  uint32_t ncols = 32;
  while ((int)ncols < NT) ncols <<= 1;
  if (warp == 0) {
    tc_alloc(&s_tmem, ncols);
    tc_relinquish();
  }
  if (tid == 32) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  const int bid = blockIdx.x;
  const int x0 = (bid % P.nbx) * kBX, y0 = ((bid / P.nbx) % P.nby) * kBY, z0 = (bid / (P.nbx * P.nby)) * kBZ;
  // halo: positions (x0 - 1 .. x0 + 8, y0 - 1 .. y0 + 4, z0 - 1 .. z0 + 4)
  for (int i = tid; i < kHalo; i += kThreads) {
    const int hx = i % kHX, hy = (i / kHX) % kHY, hz = i / (kHX * kHY);
    const int x = x0 - 1 + hx, y = y0 - 1 + hy, z = z0 - 1 + hz;
    uint32_t v = 0u;
    if (x >= 0 && y >= 0 && z >= 0 && x < P.nx && y < P.ny && z < P.nz)
      v = __ldg(P.src + ((size_t)z * P.ny + y) * P.nx + x);
    sH[i] = v;
  }
  // B: NT rows of 8 chunks (zero past the packed rows)
  for (int q = tid; q < NT * 8; q += kThreads) {
    const int n = q >> 3, c = q & 7;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (n < P.wrows) v = __ldg((const uint4*)(P.w + (size_t)n * 64) + c);
    *(uint4*)(sB + c * (NT * 16) + (n >> 3) * 128 + (n & 7) * 16) = v;
  }
  __syncthreads();
  // A: row r = this thread's position in the brick; chunk c = taps 4c .. 4c+3
  {
    const int r = tid;
    const int rx = r % kBX, ry = (r / kBX) % kBY, rz = r / (kBX * kBY);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      uint32_t wv[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int t = 4 * c + j;
        wv[j] = 0u;
        if (t < 27) {
          const int dx = t % 3, dy = (t / 3) % 3, dz = t / 9;
          wv[j] = sH[(rx + dx) + kHX * ((ry + dy) + kHY * (rz + dz))];
        }
      }
      *(uint4*)(sA + c * 2048 + (r >> 3) * 128 + (r & 7) * 16) = make_uint4(wv[0], wv[1], wv[2], wv[3]);
    }
  }
  fence_proxy_async_smem();  // the tiles' generic stores before the tensor core reads them
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  if (tid == 0) {
    const uint32_t a0 = smem_addr(sA), b0 = smem_addr(sB), bL = (uint32_t)NT * 16;
    const uint32_t idesc = idesc_bf16(kM, NT);
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
      tc_mma(tmem, smem_desc(a0 + kk * 2 * 2048, 2048, 128), smem_desc(b0 + kk * 2 * bL, bL, 128), idesc,
             kk > 0 ? 1u : 0u);
    tc_commit(&bar);
  }
  __syncwarp();
  const bool ok = mbar_wait_bounded(&bar, 0);
  tc_fence_after();
  if (__syncthreads_or(!ok)) {
    if (tid == 0) atomicExch(P.err, 1);
  } else {
    const int r = warp * 32 + lane;
    const int x = x0 + r % kBX, y = y0 + (r / kBX) % kBY, z = z0 + r / (kBX * kBY);
    store_rows(tmem, warp, x < P.nx && y < P.ny && z < P.nz, ((long long)z * P.ny + y) * P.nx + x, P.e);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tc_dealloc(tmem, ncols);
  }
}

}  // namespace

size_t conv_tc_smem_bytes(int n_out) {
  const int NT = (n_out + 15) / 16 * 16;
  return (size_t)kStages * (kAStage + (size_t)NT * 128) + kStages * 8 + 32;
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

template <int CB>
int launch_tma_cb(const CUtensorMap& ta, const CUtensorMap& tb, const ConvTmaArgs& a, unsigned nb, size_t smem,
                  cudaStream_t s) {
  if (int st = ensure_dyn_smem((const void*)k_conv_tma<CB>, (int)smem)) return st;
  k_conv_tma<CB><<<nb, kThreads, smem, s>>>(ta, tb, a);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

template <int CB>
int launch_tma_p(const CUtensorMap& ta, const CUtensorMap& tb, ConvTmaArgs a, long long ntiles, cudaStream_t s) {
  int dev = 0, sms = 0;
  VDVC_CUDA(cudaGetDevice(&dev));
  VDVC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint32_t stage = (uint32_t)(kM + a.e.NT) * CB * 2;
  a.stages = (int)(kPStageBudget / stage);
  if (a.stages > kPMaxStages) a.stages = kPMaxStages;
  if (a.stages < 2) return VDVC_ERR_UNSUPPORTED;
  const size_t smem = (size_t)a.stages * stage + 1024 + (2 * a.stages + 5) * 8 + 16;
  if (int st = ensure_dyn_smem((const void*)k_conv_tma_p<CB>, (int)smem)) return st;
  const long long nb = ntiles < 2LL * sms ? ntiles : 2LL * sms;
  k_conv_tma_p<CB><<<(unsigned)nb, kPThreads, smem, s>>>(ta, tb, a, (int)ntiles);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

}  // namespace

// The TMA form: unit source step (d = 1), |c| = 1, 1 <= a <= 4, cin a
// multiple of 32 with a 16-byte aligned channel range.  VDVC_ERR_UNSUPPORTED
// (error text untouched) otherwise, and the caller takes k_conv_tc.
int launch_conv_tma(const void* src, int scs, int scoff, int cin, const void* w, int wrows, const float* bias,
                    int n_out, int relu, void* out, int out_f32, int ocs, int ocoff, int accumulate,
                    const vdvc_conv_geom* g, int* err, cudaStream_t s) {
  if (g->d != 1 || (g->c != 1 && g->c != -1) || g->a < 1 || g->a > 4) return VDVC_ERR_UNSUPPORTED;
  if (cin < 32 || cin % 32 || scs % 8 || scoff % 8 || n_out > 256 || wrows < n_out) return VDVC_ERR_UNSUPPORTED;
  if (((uintptr_t)src | (uintptr_t)w) & 15) return VDVC_ERR_UNSUPPORTED;
  PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if (!encode) return VDVC_ERR_UNSUPPORTED;
  const int CB = cin % 64 == 0 ? 64 : 32;
  const int NT = (n_out + 15) / 16 * 16;
  const CUtensorMapSwizzle sw = CB == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
  const cuuint32_t A = (cuuint32_t)g->a;
  alignas(64) CUtensorMap ta, tb;
  {
    const cuuint64_t dim[4] = {(cuuint64_t)scs, (cuuint64_t)g->sx, (cuuint64_t)g->sy, (cuuint64_t)g->sz};
    const cuuint64_t stride[3] = {(cuuint64_t)scs * 2, (cuuint64_t)scs * 2 * g->sx,
                                  (cuuint64_t)scs * 2 * g->sx * g->sy};
    const cuuint32_t box[4] = {(cuuint32_t)CB, kBX * A, kBY * A, kBZ * A};
    const cuuint32_t step[4] = {1, A, A, A};
    if (encode(&ta, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(src), dim, stride, box, step,
               CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return set_error(VDVC_ERR_CUDA, "cuTensorMapEncodeTiled (convolution source) failed");
  }
  {
    const cuuint64_t dim[2] = {(cuuint64_t)27 * cin, (cuuint64_t)wrows};
    const cuuint64_t stride[1] = {(cuuint64_t)27 * cin * 2};
    const cuuint32_t box[2] = {(cuuint32_t)CB, (cuuint32_t)NT};
    const cuuint32_t step[2] = {1, 1};
    if (encode(&tb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(w), dim, stride, box, step,
               CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return set_error(VDVC_ERR_CUDA, "cuTensorMapEncodeTiled (convolution weights) failed");
  }
  ConvTmaArgs a{};
  a.nx = g->nx;
  a.ny = g->ny;
  a.nz = g->nz;
  a.nbx = (g->nx + kBX - 1) / kBX;
  a.nby = (g->ny + kBY - 1) / kBY;
  const long long nbz = (g->nz + kBZ - 1) / kBZ;
  a.a = g->a;
  a.b = g->b;
  a.c = g->c;
  a.cin = cin;
  a.scoff = scoff;
  a.ncb = cin / CB;
  a.nkb = 27 * a.ncb;
  const uint32_t stage = (uint32_t)(kM + NT) * CB * 2;
  a.stages = (int)(kTmaStageBudget / stage);
  if (a.stages > kTmaMaxStages) a.stages = kTmaMaxStages;
  if (a.stages < 2) return VDVC_ERR_UNSUPPORTED;
  a.e = Epi{bias, n_out, NT, relu, out_f32, ocs, ocoff, accumulate, out};
  a.err = err;
  const long long nb = (long long)a.nbx * a.nby * nbz;
  if (nb >= 0x7fffffffLL) return set_error(VDVC_ERR_ARG, "grid too large");
  // stages + 1 KB of alignment slack + barriers and flags
  const size_t smem = (size_t)a.stages * stage + 1024 + (2 * a.stages + 1) * 8 + 16;
  // the persistent form where a brick's stages are large (N >= 32: at most
  // two one-brick CTAs would fit an SM anyway); with N = 16 the one-brick
  // form keeps three CTAs per SM and is faster (513^3 output layer 78 vs
  // 108 us; e2b 140 vs 113 us the other way round)
  if (NT >= 32) return CB == 64 ? launch_tma_p<64>(ta, tb, a, nb, s) : launch_tma_p<32>(ta, tb, a, nb, s);
  return CB == 64 ? launch_tma_cb<64>(ta, tb, a, (unsigned)nb, smem, s)
                  : launch_tma_cb<32>(ta, tb, a, (unsigned)nb, smem, s);
}

// The first-layer form: cin = 2 (packed [wrows][64] weights), forward
// stride 1 (a = 1, b = -1, c = 1, d = 1, source grid = output grid),
// n_out <= 64, a contiguous 2-channel source, 4-byte aligned.
// VDVC_ERR_UNSUPPORTED otherwise (the caller keeps the mma.sync kernel).
int launch_conv_first(const void* src, int scs, int scoff, const void* w, int wrows, const float* bias, int n_out,
                      int relu, void* out, int out_f32, int ocs, int ocoff, int accumulate, const vdvc_conv_geom* g,
                      int* err, cudaStream_t s) {
  if (g->a != 1 || g->b != -1 || g->c != 1 || g->d != 1 || g->sx != g->nx || g->sy != g->ny || g->sz != g->nz)
    return VDVC_ERR_UNSUPPORTED;
  if (scs != 2 || scoff != 0 || n_out > 64 || (((uintptr_t)src | (uintptr_t)w) & 15)) return VDVC_ERR_UNSUPPORTED;
  ConvFirstArgs a{};
  a.src = (const uint32_t*)src;
  a.w = (const bf16*)w;
  a.wrows = wrows;
  a.nx = g->nx;
  a.ny = g->ny;
  a.nz = g->nz;
  a.nbx = (g->nx + kBX - 1) / kBX;
  a.nby = (g->ny + kBY - 1) / kBY;
  a.e = Epi{bias, n_out, (n_out + 15) / 16 * 16, relu, out_f32, ocs, ocoff, accumulate, out};
  a.err = err;
  const long long nb = (long long)a.nbx * a.nby * ((g->nz + kBZ - 1) / kBZ);
  if (nb >= 0x7fffffffLL) return set_error(VDVC_ERR_ARG, "grid too large");
  k_conv_first<<<(unsigned)nb, kThreads, 0, s>>>(a);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

// VDVC_ERR_UNSUPPORTED (error text untouched) when the layer does not fit
// the tensor-core form: cin a multiple of 8 with 16-byte aligned channel
// chunks (strides and offsets multiples of 8 channels), n_out <= 256.
int launch_conv_tc(const void* src, int scs, int scoff, int cin, const void* w, int wrows, const float* bias,
                   int n_out, int relu, void* out, int out_f32, int ocs, int ocoff, int accumulate,
                   const vdvc_conv_geom* geom, int* err, cudaStream_t s) {
  if (cin < 8 || cin % 8 || scs % 8 || scoff % 8 || n_out > 256 || wrows < n_out) return VDVC_ERR_UNSUPPORTED;
  if (((uintptr_t)src | (uintptr_t)w) & 15) return VDVC_ERR_UNSUPPORTED;
  ConvTcArgs a{};
  a.src = (const bf16*)src;
  a.scs = scs;
  a.scoff = scoff;
  a.cin = cin;
  a.w = (const bf16*)w;
  a.wrows = wrows;
  a.e = Epi{bias, n_out, (n_out + 15) / 16 * 16, relu, out_f32, ocs, ocoff, accumulate, out};
  a.g = TcGeo{geom->nx, geom->ny, geom->nz, geom->sx, geom->sy, geom->sz, geom->a, geom->b, geom->c, geom->d};
  a.err = err;
  const long long npos = (long long)geom->nx * geom->ny * geom->nz;
  const long long nb = (npos + kM - 1) / kM;
  if (nb >= 0x7fffffffLL) return set_error(VDVC_ERR_ARG, "grid too large");
  const size_t smem = conv_tc_smem_bytes(n_out);
  if (int st = ensure_dyn_smem((const void*)k_conv_tc, (int)smem)) return st;
  k_conv_tc<<<(unsigned)nb, kThreads, smem, s>>>(a);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

}  // namespace vdvc
