// Jacobi-preconditioned CG (engine/kernels_dvc.py:550-583) as device
// kernels with float64 dot products and device-resident scalars.
//
// Iteration it (p_old from the previous iteration, beta in the state):
//   [eq. gap]  w      = P_i (h K_el p_new)                 (stencil, reg.cu)
//   strip      ev     = H_e p_new + c1 K1 p_new,e + c2 K2 w_e
//   gather     p      = p_new = z + beta p_old ; Ap = sum ev ; alpha = rz/(p.Ap + 1e-30)
//   update     x += alpha p ; r -= alpha Ap ; z = M r ; res = sqrt(r.r / r0)
//              done if res < tol or it+1 == max_iter ; beta = r.z_new/(rz + 1e-30)
// p_new is formed on the fly from z and p_old by the kernels that need it,
// so there is no separate p-update pass.
//
// Dot products: each thread sums its few products in the vector type (FP32
// for float vectors: the products' own rounding), converts once, and the
// block and grid sums run in float64 in a fixed order.  FP64 arithmetic per
// vector entry would run on GB300's much narrower FP64 pipe.  Every kernel returns at once when
// state.done is set, which makes a captured chunk of iterations safe to
// replay past convergence.
#include <cstdint>
#include <type_traits>

#include "ops.cuh"
#include "pcg.cuh"

namespace vdvc {

// r = b - Ax ; z = M r ; p = z (or 0 for the fused form with beta = 0) ;
// rz = r.z ; r0 = b.b + 1e-30.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_init(const T* __restrict__ b, const T* __restrict__ Ax,
                                                  const T* __restrict__ Minv, long long n, T* __restrict__ r,
                                                  T* __restrict__ z, T* __restrict__ p, bool p_is_z,
                                                  T* __restrict__ x0, PcgState* st, GridReduce red, int max_iter,
                                                  double tol) {
  __shared__ double s_red[8];
  T rz = T(0), bb = T(0);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (x0) x0[i] = T(0);
    const T bi = b[i];
    const T ri = Ax ? (T)(bi - Ax[i]) : bi;
    const T zi = Minv[i] * ri;
    r[i] = ri;
    z[i] = zi;
    p[i] = p_is_z ? zi : T(0);
    rz += ri * zi;
    bb += bi * bi;
  }
  double mine[2] = {block_sum_f(rz, s_red), block_sum_f(bb, s_red)}, out[2];
  if (grid_reduce_sum<2>(red, mine, out, s_red) && threadIdx.x == 0) {
    st->rz = out[0];
    st->r0 = out[1] + 1e-30;
    st->alpha = 0.0;
    st->beta = 0.0;
    st->res = 0.0;
    st->rr = 0.0;
    st->iter = 0;
    st->done = max_iter <= 0 ? 1 : 0;
    st->status = VDVC_OK;
    st->max_iter = max_iter;
    st->tol = tol;
  }
}

// Fused gather: p <- z + beta p ; Ap <- sum of element vectors ; alpha.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_gather(const Mesh m, const T* __restrict__ ev,
                                                    const T* __restrict__ z, T* __restrict__ p,
                                                    T* __restrict__ Ap, PcgState* st, GridReduce red) {
  __shared__ double s_red[8];
  if (st->done) return;
  const T beta = (T)st->beta;
  T pap = T(0);
  // 32-bit node coordinates (the launcher rejects 2^32 nodes or more)
  const unsigned int nnx = (unsigned int)m.Nnx, nny = (unsigned int)m.Nny;
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < m.Nnodes;
       n += (long long)gridDim.x * blockDim.x) {
    const unsigned int nu = (unsigned int)n, rr = nu / nnx;
    const int ni = (int)(nu - rr * nnx), nj = (int)(rr % nny), nk = (int)(rr / nny);
    T s[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const int ei = ni - corner_dx(a), ej = nj - corner_dy(a), ek = nk - corner_dz(a);
      if (ei < 0 || ej < 0 || ek < 0 || ei >= m.Nx || ej >= m.Ny || ek >= m.Nz) continue;
      const long long e = (long long)ei + (long long)ej * m.Nx + (long long)ek * m.Nx * m.Ny;
#pragma unroll
      for (int c = 0; c < 3; ++c) s[c] += ev[(long long)(3 * a + c) * m.Ne + e];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long long d = 3 * n + c;
      const T pn = z[d] + beta * p[d];
      p[d] = pn;
      Ap[d] = s[c];
      pap += pn * s[c];
    }
  }
  double mine[1] = {block_sum_f(pap, s_red)}, out[1];
  if (grid_reduce_sum<1>(red, mine, out, s_red) && threadIdx.x == 0) st->alpha = st->rz / (out[0] + 1e-30);
}

// Generic form: alpha = rz / (p.Ap + 1e-30) for an externally computed Ap.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_alpha(const T* __restrict__ p, const T* __restrict__ Ap, long long n,
                                                   PcgState* st, GridReduce red) {
  __shared__ double s_red[8];
  if (st->done) return;
  T pap = T(0);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    pap += p[i] * Ap[i];
  double mine[1] = {block_sum_f(pap, s_red)}, out[1];
  if (grid_reduce_sum<1>(red, mine, out, s_red) && threadIdx.x == 0) st->alpha = st->rz / (out[0] + 1e-30);
}

template <typename T>
__global__ void __launch_bounds__(256) k_pcg_update(const T* __restrict__ p, const T* __restrict__ Ap,
                                                    const T* __restrict__ Minv, long long n, T* __restrict__ x,
                                                    T* __restrict__ r, T* __restrict__ z, PcgState* st,
                                                    GridReduce red, bool vec4) {
  __shared__ double s_red[8];
  if (st->done) return;
  const T alpha = (T)st->alpha;
  T rr = T(0), rz = T(0);
  const long long gtid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i0 = 0;
  if constexpr (std::is_same<T, float>::value) {
    if (vec4) {  // every pointer 16-byte aligned: float4 body, scalar tail
      const long long n4 = n >> 2;
      for (long long q = gtid; q < n4; q += stride) {
        const float4 pv = ((const float4*)p)[q], av = ((const float4*)Ap)[q], mv = ((const float4*)Minv)[q];
        float4 xv = ((float4*)x)[q], rv = ((float4*)r)[q], zv;
        xv.x += alpha * pv.x; xv.y += alpha * pv.y; xv.z += alpha * pv.z; xv.w += alpha * pv.w;
        rv.x -= alpha * av.x; rv.y -= alpha * av.y; rv.z -= alpha * av.z; rv.w -= alpha * av.w;
        zv.x = mv.x * rv.x; zv.y = mv.y * rv.y; zv.z = mv.z * rv.z; zv.w = mv.w * rv.w;
        ((float4*)x)[q] = xv;
        ((float4*)r)[q] = rv;
        ((float4*)z)[q] = zv;
        rr += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
        rz += rv.x * zv.x + rv.y * zv.y + rv.z * zv.z + rv.w * zv.w;
      }
      i0 = n4 << 2;
    }
  }
  for (long long i = i0 + gtid; i < n; i += stride) {
    x[i] = x[i] + alpha * p[i];
    const T ri = r[i] - alpha * Ap[i];
    const T zi = Minv[i] * ri;
    r[i] = ri;
    z[i] = zi;
    rr += ri * ri;
    rz += ri * zi;
  }
  double mine[2] = {block_sum_f(rr, s_red), block_sum_f(rz, s_red)}, out[2];
  if (grid_reduce_sum<2>(red, mine, out, s_red) && threadIdx.x == 0) {
    const double res = sqrt(out[0] / st->r0);
    st->rr = out[0];
    st->res = res;
    st->iter += 1;
    if (!(res == res) || !isfinite(st->alpha)) {
      st->status = VDVC_ERR_NONFINITE;
      st->done = 1;
    } else if (res < st->tol || st->iter >= st->max_iter) {
      st->done = 1;
    }
    st->beta = out[1] / (st->rz + 1e-30);
    st->rz = out[1];
  }
}

// Generic form: p = z + beta p.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_pupdate(const T* __restrict__ z, T* __restrict__ p, long long n,
                                                     const PcgState* st) {
  if (st->done) return;
  const T beta = (T)st->beta;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = z[i] + beta * p[i];
}

inline int vec_blocks(long long n) { return grid_blocks(n, 256, kReduceBlocks); }
inline bool aligned16(const void* q) { return ((uintptr_t)q & 15u) == 0; }

template <typename T>
int launch_pcg_init(const T* b, const T* Ax, const T* Minv, long long n, T* r, T* z, T* p, bool p_is_z, T* x0,
                    PcgState* st, GridReduce red, int max_iter, double tol, cudaStream_t s) {
  k_pcg_init<T><<<vec_blocks(n), 256, 0, s>>>(b, Ax, Minv, n, r, z, p, p_is_z, x0, st, red, max_iter, tol);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

template <typename T>
int launch_pcg_gather(const Mesh& m, const T* ev, const T* z, T* p, T* Ap, PcgState* st, GridReduce red,
                      cudaStream_t s, long long max_blocks) {
  if (m.Nnodes >= (1ll << 32)) return set_error(VDVC_ERR_UNSUPPORTED, "2^32 nodes or more");
  // one node per thread where the partials allow it: a capped grid leaves a
  // few threads with two nodes, which doubles the kernel's critical path
  k_pcg_gather<T><<<grid_blocks(m.Nnodes, 256, max_blocks > kReduceBlocks ? max_blocks : kReduceBlocks), 256, 0,
                    s>>>(m, ev, z, p, Ap, st, red);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

template <typename T>
int launch_pcg_update(const T* p, const T* Ap, const T* Minv, long long n, T* x, T* r, T* z, PcgState* st,
                      GridReduce red, cudaStream_t s) {
  const bool vec4 = aligned16(p) && aligned16(Ap) && aligned16(Minv) && aligned16(x) && aligned16(r) && aligned16(z);
  k_pcg_update<T><<<vec_blocks(vec4 ? (n + 3) / 4 : n), 256, 0, s>>>(p, Ap, Minv, n, x, r, z, st, red, vec4);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

template int launch_pcg_init<float>(const float*, const float*, const float*, long long, float*, float*, float*,
                                    bool, float*, PcgState*, GridReduce, int, double, cudaStream_t);
template int launch_pcg_init<double>(const double*, const double*, const double*, long long, double*, double*,
                                     double*, bool, double*, PcgState*, GridReduce, int, double, cudaStream_t);
template int launch_pcg_gather<float>(const Mesh&, const float*, const float*, float*, float*, PcgState*, GridReduce,
                                      cudaStream_t, long long);
template int launch_pcg_gather<double>(const Mesh&, const double*, const double*, double*, double*, PcgState*,
                                       GridReduce, cudaStream_t, long long);
template int launch_pcg_update<float>(const float*, const float*, const float*, long long, float*, float*, float*,
                                      PcgState*, GridReduce, cudaStream_t);
template int launch_pcg_update<double>(const double*, const double*, const double*, long long, double*, double*,
                                       double*, PcgState*, GridReduce, cudaStream_t);

// ---- generic PCG around an external matvec --------------------------------

struct GenericPcg {
  PcgState* st;
  GridReduce red;
};

static int carve_generic(void* ws, size_t ws_bytes, GenericPcg* g) {
  Carve cv(ws, ws_bytes);
  g->st = cv.take<PcgState>(1);
  g->red.partials = cv.take<double>((size_t)kReduceBlocks * 2);
  g->red.ticket = cv.take<unsigned int>(1);
  if (!ws || !cv.fits()) return set_error(VDVC_ERR_WORKSPACE, "pcg needs %zu bytes of workspace", cv.off);
  return VDVC_OK;
}

}  // namespace vdvc

using namespace vdvc;

extern "C" {

size_t vdvc_pcg_workspace_bytes(void) {
  Carve cv(nullptr, 0);
  cv.take<PcgState>(1);
  cv.take<double>((size_t)kReduceBlocks * 2);
  cv.take<unsigned int>(1);
  return cv.off + 256;
}

int vdvc_pcg_begin(const void* b, const void* Ax, const void* Minv, int dtype, long long n, void* r, void* z,
                   void* p, int max_iter, double tol, void* ws, size_t ws_bytes, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(b && Minv && r && z && p && n >= 1, "bad arguments");
  GenericPcg g;
  int st = carve_generic(ws, ws_bytes, &g);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  VDVC_CUDA(cudaMemsetAsync(g.red.ticket, 0, sizeof(unsigned int), s));
  if (dtype == VDVC_F32)
    return launch_pcg_init<float>((const float*)b, (const float*)Ax, (const float*)Minv, n, (float*)r, (float*)z,
                                  (float*)p, true, nullptr, g.st, g.red, max_iter, tol, s);
  if (dtype == VDVC_F64)
    return launch_pcg_init<double>((const double*)b, (const double*)Ax, (const double*)Minv, n, (double*)r,
                                   (double*)z, (double*)p, true, nullptr, g.st, g.red, max_iter, tol, s);
  return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
}

int vdvc_pcg_step(const void* Ap, const void* Minv, int dtype, long long n, void* x, void* r, void* z, void* p,
                  void* ws, size_t ws_bytes, double* res_out, int* done_out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(Ap && Minv && x && r && z && p && n >= 1, "bad arguments");
  GenericPcg g;
  int st = carve_generic(ws, ws_bytes, &g);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = vec_blocks(n);
  if (dtype == VDVC_F32) {
    k_pcg_alpha<float><<<nb, 256, 0, s>>>((const float*)p, (const float*)Ap, n, g.st, g.red);
    VDVC_LAUNCHED();
    if ((st = launch_pcg_update<float>((const float*)p, (const float*)Ap, (const float*)Minv, n, (float*)x,
                                       (float*)r, (float*)z, g.st, g.red, s)))
      return st;
  } else if (dtype == VDVC_F64) {
    k_pcg_alpha<double><<<nb, 256, 0, s>>>((const double*)p, (const double*)Ap, n, g.st, g.red);
    VDVC_LAUNCHED();
    if ((st = launch_pcg_update<double>((const double*)p, (const double*)Ap, (const double*)Minv, n, (double*)x,
                                        (double*)r, (double*)z, g.st, g.red, s)))
      return st;
  } else {
    return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
  }
  PcgState h;
  VDVC_CUDA(cudaMemcpyAsync(&h, g.st, sizeof(PcgState), cudaMemcpyDeviceToHost, s));
  VDVC_CUDA(cudaStreamSynchronize(s));
  if (res_out) *res_out = h.res;
  if (done_out) *done_out = h.done;
  return VDVC_OK;
}

int vdvc_pcg_direction(const void* z, void* p, int dtype, long long n, void* ws, size_t ws_bytes,
                       vdvc_stream_t stream) {
  VDVC_CHECK_ARG(z && p && n >= 1, "bad arguments");
  GenericPcg g;
  int st = carve_generic(ws, ws_bytes, &g);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  // the direction update runs even after `done`: the caller decides (the
  // reference breaks before it on convergence)
  if (dtype == VDVC_F32) {
    k_pcg_pupdate<float><<<vec_blocks(n), 256, 0, s>>>((const float*)z, (float*)p, n, g.st);
  } else if (dtype == VDVC_F64) {
    k_pcg_pupdate<double><<<vec_blocks(n), 256, 0, s>>>((const double*)z, (double*)p, n, g.st);
  } else {
    return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
  }
  VDVC_LAUNCHED();
  return VDVC_OK;
}

}  // extern "C"
