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
// COHERENT: v and p_old are read through L2 (they were written by other
// blocks of the same persistent kernel, so the read-only path may be stale).
template <int H, bool PCG, bool COHERENT = false>
__device__ __forceinline__ void elem_hv_body(const StripArgs<float>& a, const Kpair<float>* __restrict__ kp,
                                             long long e, float beta) {
  const Mesh& m = a.m;
  const int i = (int)(e % m.Nx);
  const long long rr = e / m.Nx;
  const int j = (int)(rr % m.Ny), k = (int)(rr / m.Ny);

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
          float val = COHERENT ? __ldcg(a.v + q) : __ldg(a.v + q);
          if constexpr (PCG) val += beta * (COHERENT ? __ldcg(a.p_old + q) : __ldg(a.p_old + q));
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

// ---- persistent fused PCG -------------------------------------------------
//
// The whole Jacobi PCG of one GN iteration in one cooperative launch, for the
// small levels where a PCG iteration's separate launches (element pass,
// gather, update), their grid-reduction tails and the graph's per-node
// overhead cost several times the iteration's data movement (at 129^3 voxels
// the working set -- gradient, mask, element vectors, six nodal vectors --
// is ~70 MB and stays in the 129 MB L2).  Per iteration, in every block:
//   A  element pass, p_new = z + beta p on the fly       | grid barrier
//   B  gather: p <- p_new, Ap = sum ev, block p.Ap         | grid barrier
//      alpha = rz / (sum of the block partials + 1e-30)
//   C  x += alpha p, r -= alpha Ap, z = M r, block r.r, r.z | grid barrier
//      res, convergence, beta = rz_new / (rz + 1e-30)
// Every block sums the partials itself in the same fixed order, so all
// blocks hold identical scalars and leave the loop together.  The arithmetic
// is that of the graph-replayed kernels (k_pcg_gather, k_pcg_update).
// Barriers spin on a generation counter with a bounded wait: on a timeout
// the kernel raises an error flag, every block leaves, and the host reports
// the failure.  Data written by other blocks is read through L2 (ld.cg).

// Spin bound of a barrier wait: tens of millions of polls (seconds, with or
// without the optional sleep) -- far beyond any healthy barrier.
constexpr long long kBarrierSpins = 20000000;

__device__ __forceinline__ bool grid_barrier(unsigned int* bar, int* err, unsigned int nblocks, int sleep_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* vgen = bar + 1;
    volatile int* verr = err;
    const unsigned int g = *vgen;
    __threadfence();
    int ok = 1;
    if (atomicAdd(bar, 1u) == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long spins = 0;
      while (*vgen == g) {
        if (*verr) {
          ok = 0;
          break;
        }
        if (++spins > kBarrierSpins) {
          atomicExch(err, 1);
          ok = 0;
          break;
        }
        if (sleep_ns > 0) __nanosleep(sleep_ns);
      }
    }
    __threadfence();
    if (*verr) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Sum of partials[slot*nb + b] over all blocks b, fixed order, in every thread.
__device__ __forceinline__ double all_blocks_sum(const double* partials, int slot, unsigned int nb, double* s_red,
                                                 double* s_bc) {
  double v = 0.0;
#pragma unroll 4
  for (unsigned int b = threadIdx.x; b < nb; b += blockDim.x) v += __ldcg(partials + (size_t)slot * nb + b);
  v = block_sum(v, s_red);
  if (threadIdx.x == 0) *s_bc = v;
  __syncthreads();
  v = *s_bc;
  __syncthreads();
  return v;
}

template <int H>
__global__ void __launch_bounds__(256, 2) k_pcg_persistent(const PcgPersistArgs A) {
  __shared__ double s_red[8];
  __shared__ double s_bc;
  const unsigned int nb = gridDim.x;
  const Mesh& m = A.sa.m;
  const long long gtid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)nb * blockDim.x;
  double rz = A.st->rz, beta = A.st->beta, alpha = A.st->alpha, res = A.st->res, rr = A.st->rr;
  const double r0 = A.st->r0, tol = A.st->tol;
  int iter = A.st->iter, done = A.st->done, status = A.st->status;
  const int max_iter = A.st->max_iter;
  bool ok = true;
  while (!done) {
    // A: element vectors of H p_new (+ regularizer)
    const float bf = (float)beta;
    for (long long e = gtid; e < m.Ne; e += stride) elem_hv_body<H, true, true>(A.sa, A.kp, e, bf);
    if (!(ok = grid_barrier(A.bar, A.err, nb, A.sleep_ns))) break;
    // B: p <- p_new, Ap, p.Ap
    float pap = 0.f;
    for (long long n = gtid; n < m.Nnodes; n += stride) {
      const int ni = (int)(n % m.Nnx);
      const long long rn = n / m.Nnx;
      const int nj = (int)(rn % m.Nny), nk = (int)(rn / m.Nny);
      float sacc[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        const int ei = ni - corner_dx(a), ej = nj - corner_dy(a), ek = nk - corner_dz(a);
        if (ei < 0 || ej < 0 || ek < 0 || ei >= m.Nx || ej >= m.Ny || ek >= m.Nz) continue;
        const long long e = (long long)ei + (long long)ej * m.Nx + (long long)ek * m.Nx * m.Ny;
#pragma unroll
        for (int c = 0; c < 3; ++c) sacc[c] += __ldcg(A.sa.evA + (long long)(3 * a + c) * m.Ne + e);
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const long long d = 3 * n + c;
        const float pn = __ldcg(A.z + d) + bf * __ldcg(A.p + d);
        A.p[d] = pn;
        A.Ap[d] = sacc[c];
        pap += pn * sacc[c];
      }
    }
    {
      const double bs = block_sum_f(pap, s_red);
      if (threadIdx.x == 0) A.partials[blockIdx.x] = bs;
    }
    if (!(ok = grid_barrier(A.bar, A.err, nb, A.sleep_ns))) break;
    alpha = rz / (all_blocks_sum(A.partials, 0, nb, s_red, &s_bc) + 1e-30);
    // C: x, r, z and r.r, r.z
    const float af = (float)alpha;
    float rrf = 0.f, rzf = 0.f;
    for (long long i = gtid; i < m.Ndof; i += stride) {
      const float pi = __ldcg(A.p + i), api = __ldcg(A.Ap + i);
      A.x[i] = __ldcg(A.x + i) + af * pi;
      const float ri = __ldcg(A.r + i) - af * api;
      const float zi = A.Minv[i] * ri;
      A.r[i] = ri;
      A.z[i] = zi;
      rrf += ri * ri;
      rzf += ri * zi;
    }
    {
      const double b1 = block_sum_f(rrf, s_red);
      const double b2 = block_sum_f(rzf, s_red);
      if (threadIdx.x == 0) {
        A.partials[(size_t)nb + blockIdx.x] = b1;
        A.partials[(size_t)2 * nb + blockIdx.x] = b2;
      }
    }
    if (!(ok = grid_barrier(A.bar, A.err, nb, A.sleep_ns))) break;
    rr = all_blocks_sum(A.partials, 1, nb, s_red, &s_bc);
    const double rz_new = all_blocks_sum(A.partials, 2, nb, s_red, &s_bc);
    res = sqrt(rr / r0);
    iter += 1;
    if (!(res == res) || !isfinite(alpha)) {
      status = VDVC_ERR_NONFINITE;
      done = 1;
    } else if (res < tol || iter >= max_iter) {
      done = 1;
    }
    beta = rz_new / (rz + 1e-30);
    rz = rz_new;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    A.st->rz = rz;
    A.st->beta = beta;
    A.st->alpha = alpha;
    A.st->res = res;
    A.st->rr = rr;
    A.st->iter = iter;
    A.st->done = 1;
    A.st->status = ok ? status : VDVC_ERR_CUDA;
  }
}

template <int H>
static int launch_persist_h(const PcgPersistArgs& a, int max_blocks, cudaStream_t s) {
  int per_sm = 0, dev = 0, nsm = 0;
  VDVC_CUDA(cudaGetDevice(&dev));
  VDVC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  VDVC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_persistent<H>, 256, 0));
  if (per_sm < 1) return VDVC_ERR_UNSUPPORTED;
  int grid = per_sm * nsm;
  if (grid > max_blocks) grid = max_blocks;
  PcgPersistArgs args = a;
  void* params[] = {(void*)&args};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_pcg_persistent<H>, dim3(grid), dim3(256), params, 0, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(VDVC_ERR_CUDA, "persistent PCG launch: %s", cudaGetErrorString(e));
  }
  count_launch();
  return VDVC_OK;
}

// h <= 2 only: at h = 4 the element pass alone (~75 us at 64^3 elements)
// dominates the iteration, and the fused kernel's register demand (one block
// per SM) would slow it down more than the launches it saves.
int launch_pcg_persistent(const PcgPersistArgs& a, int max_blocks, cudaStream_t s) {
  switch (a.sa.m.h) {
    case 1: return launch_persist_h<1>(a, max_blocks, s);
    case 2: return launch_persist_h<2>(a, max_blocks, s);
  }
  return VDVC_ERR_UNSUPPORTED;
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
