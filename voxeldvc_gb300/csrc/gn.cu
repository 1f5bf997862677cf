// Gauss-Newton DVC solver at one pyramid level (engine/correlate_gpu.py:
// 828-1140) as a device-resident object.  The host drives one GN iteration
// with four calls -- sample, rhs, pcg, update -- and reads back a handful of
// scalars once per iteration; everything between those calls stays on the
// GPU (scalars included).
//
// Per iteration, for T = float (the plain solve) or double:
//   sample : g(x+u), live mask, [freeze], stats of g over the b mask
//   rhs    : R U (regularizer stencils), res = f - (std0/std1)(g - mean) on the b
//            mask, element vectors of b and diag H, display stats of res;
//            gather b = sum - ll R U, diag = sum + ll diag_R, min diag; M^-1
//   pcg    : Jacobi PCG on (H + ll R) dU = b, replayed as a CUDA graph of
//            `chunk` iterations until the device state says done
//   update : U += dU (float64 master copy), |dU|^2, |U|^2
//
// Element-Hessian forms (float solver): rhs forms the element Hessians
// T[162][Ne] and the diagonal from them instead of the diag strip pass, and
// the PCG applies H from T.  Once the b mask is frozen (or with a fixed
// mask0), H, diag and M^-1 no longer change and are formed only once.
// VDVC_PREC_ELEMENT forms T from the float32 gradient; VDVC_PREC_MIXED (the
// precision form) from its BF16 rounding, made once at create, and keeps T
// in BF16 (FP32 under the equilibrium-gap regularizer).
#include <cstdlib>
#include <new>
#include <type_traits>
#include <vector>

#include "ops.cuh"
#include "pcg.cuh"

namespace vdvc {

struct GnScalars {
  double gstats[4];  // count, s1, s2 of g over the b mask; n_active
  double dstats[3];  // count, s1, s2 of res over the live mask
  double dmin;       // min diag
  double norms[2];   // |dU|^2, |U|^2
  int status;
  int pad;
};

template <typename T>
struct GnSolver {
  Mesh m;
  vdvc_gn_desc d;
  Kmat Klap, Kel;
  bool lap_blockdiag;  // K_lap = L8 on each displacement component
  float L8[64];
  // device buffers (carved from the caller's workspace)
  double* U64;
  T *U32, *x, *r, *z, *p, *Ap, *Minv, *b, *w, *ru, *t1, *gvals, *res, *evA, *evD;
  T* diag;
  double* diag_reg;  // h diag(K_lap) [+ equilibrium-gap diagonal], float64
  T* diag_reg_t;     // the same in the solve type
  uint8_t *live, *frozen;
  bool live_is_b;    // the last sampling pass wrote the live mask into the b mask buffer only
  double* partials;
  size_t n_partials;
  unsigned int* ticket;
  GnScalars* sc;
  PcgState* pcg;
  Kpair<T>* kp;
  bool frozen_set;
  // element-Hessian forms
  bool eh;           // the PCG applies H from element Hessians
  bool eh_bf16;      // ... formed from the BF16 gradient (precision form)
  bool eh_T_bf16;    // ... and stored in BF16 (precision form, no equilibrium-gap term)
  bool eh_fixed;     // T, diag and M^-1 are final (b mask frozen, or mask0)
  float* T_eh;       // [162][Ne] element Hessians
  void* grad_bf16;   // (Nvox,3) BF16 (precision form only)
  float* gmax;       // max |g| of grad_bf16 (the tensor-core formation's scale)
  // PCG graph
  cudaStream_t cap_stream;
  cudaStream_t side;              // element-Hessian formation beside the residual pass
  cudaEvent_t ev_fork, ev_join;
  cudaGraph_t graph;
  cudaGraphExec_t gexec;
  int chunk, kernels_per_iter;
  // pinned readback slots
  PcgState* h_pcg;
  GnScalars* h_sc;
  cudaEvent_t ev[2];
};

template <typename T>
static size_t carve_solver(const Mesh& m, GnSolver<T>* S, void* ws, size_t bytes) {
  Carve cv(ws, bytes);
  const size_t nd = (size_t)m.Ndof, nv = (size_t)m.Nvox;
  S->U64 = cv.take<double>(nd);
  S->U32 = cv.take<T>(nd);
  S->x = cv.take<T>(nd);
  S->r = cv.take<T>(nd);
  S->z = cv.take<T>(nd);
  S->p = cv.take<T>(nd);
  S->Ap = cv.take<T>(nd);
  S->Minv = cv.take<T>(nd);
  S->b = cv.take<T>(nd);
  S->w = cv.take<T>(nd);
  S->ru = cv.take<T>(nd);
  S->t1 = cv.take<T>(nd);
  S->diag = cv.take<T>(nd);
  S->diag_reg = cv.take<double>(nd);
  S->diag_reg_t = cv.take<T>(nd);
  S->gvals = cv.take<T>(nv);
  S->res = cv.take<T>(nv);
  S->live = cv.take<uint8_t>(nv);
  S->frozen = cv.take<uint8_t>(nv);
  S->evA = cv.take<T>((size_t)24 * m.Ne);
  S->evD = cv.take<T>((size_t)24 * m.Ne);
  const long long nb = strip_grid_blocks(m);
  S->n_partials = (size_t)(nb > kReduceBlocks ? nb : kReduceBlocks) * 4;
  S->partials = cv.take<double>(S->n_partials);
  S->ticket = cv.take<unsigned int>(4);
  S->sc = cv.take<GnScalars>(1);
  S->pcg = cv.take<PcgState>(1);
  S->kp = cv.take<Kpair<T>>(1);
  return cv.off;  // bytes used from ws
}

// ---- small kernels -----------------------------------------------------------

template <typename T>
__global__ void k_set_U(const double* __restrict__ U0, long long n, double* __restrict__ U64, T* __restrict__ U32) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double u = U0 ? U0[i] : 0.0;
    U64[i] = u;
    U32[i] = (T)u;
  }
}

// b = sum of element vectors - ll R U ; diag = sum + ll diag_R ; min diag
// -> sc->dmin.  In the solve type T: FP64 per entry would run on GB300's
// narrow FP64 pipe.
template <typename T>
__global__ void __launch_bounds__(256) k_gn_gather_rhs(const Mesh m, const T* __restrict__ evA,
                                                       const T* __restrict__ evD, const T* __restrict__ ru, double ll,
                                                       const T* __restrict__ diag_reg, T* __restrict__ b,
                                                       T* __restrict__ diag, GnScalars* sc, GridReduce red,
                                                       bool with_diag) {
  __shared__ double s_red[8];
  const T llT = (T)ll;
  T dmin = T(3.0e38);
  // 32-bit node coordinates (the solver rejects 2^32 nodes or more)
  const unsigned int nnx = (unsigned int)m.Nnx, nny = (unsigned int)m.Nny;
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < m.Nnodes;
       n += (long long)gridDim.x * blockDim.x) {
    const unsigned int nu = (unsigned int)n, rr = nu / nnx;
    const int ni = (int)(nu - rr * nnx), nj = (int)(rr % nny), nk = (int)(rr / nny);
    T sb[3] = {T(0), T(0), T(0)}, sd[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const int ei = ni - corner_dx(a), ej = nj - corner_dy(a), ek = nk - corner_dz(a);
      if (ei < 0 || ej < 0 || ek < 0 || ei >= m.Nx || ej >= m.Ny || ek >= m.Nz) continue;
      const long long e = (long long)ei + (long long)ej * m.Nx + (long long)ek * m.Nx * m.Ny;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sb[c] += evA[(long long)(3 * a + c) * m.Ne + e];
        if (with_diag) sd[c] += evD[(long long)(3 * a + c) * m.Ne + e];
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long long dof = 3 * n + c;
      b[dof] = ru ? sb[c] - llT * ru[dof] : sb[c];
      if (with_diag) {
        const T dg = sd[c] + (diag_reg ? llT * diag_reg[dof] : T(0));
        diag[dof] = dg;
        dmin = tmin(dmin, dg);
      }
    }
  }
  if (!with_diag) return;
  double bm = block_min((double)dmin, s_red);
  // grid min through the deterministic reduction slots (values, not sums)
  __shared__ bool s_last;
  const unsigned int nb = gridDim.x;
  if (threadIdx.x == 0) {
    red.partials[blockIdx.x] = bm;
    __threadfence();
    s_last = (atomicAdd(red.ticket, 1u) == nb - 1);
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    double v = 1.0e300;
#pragma unroll 4
    for (unsigned int q = threadIdx.x; q < nb; q += blockDim.x) v = fmin(v, __ldcg(red.partials + q));
    v = block_min(v, s_red);
    if (threadIdx.x == 0) {
      sc->dmin = v;
      *red.ticket = 0u;
    }
  }
}

template <typename T>
__global__ void k_gn_minv(const T* __restrict__ diag, long long n, const GnScalars* sc, T* __restrict__ Minv) {
  const T eps = (T)(1e-5 * sc->dmin);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    Minv[i] = T(1) / (diag[i] + eps);
}

template <typename T>
__global__ void __launch_bounds__(256) k_gn_update(const T* __restrict__ dU, long long n, double* __restrict__ U64,
                                                   T* __restrict__ U32, GnScalars* sc, GridReduce red) {
  __shared__ double s_red[8];
  // U is kept in float64; the norms of the convergence test are summed in T
  // per thread (one float64 add per thread)
  T dd = T(0), uu = T(0);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const T du = dU[i];
    const double u = U64[i] + (double)du;
    U64[i] = u;
    const T ut = (T)u;
    U32[i] = ut;
    dd += du * du;
    uu += ut * ut;
  }
  double mine[2] = {block_sum_f(dd, s_red), block_sum_f(uu, s_red)}, out[2];
  if (grid_reduce_sum<2>(red, mine, out, s_red) && threadIdx.x == 0) {
    sc->norms[0] = out[0];
    sc->norms[1] = out[1];
  }
}

template <typename T>
__global__ void k_copy_out(const T* __restrict__ src, long long n, void* __restrict__ dst, int dst_f64) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (dst_f64)
      ((double*)dst)[i] = (double)src[i];
    else
      ((float*)dst)[i] = (float)src[i];
  }
}

__global__ void k_add_scaled_f64(double* a, const double* b, double s, long long n) {  // a may alias b
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] += s * b[i];
}

inline int nblk(long long n) { return grid_blocks(n, 256, 152 * 16); }

// ---- the regularizer applied to a nodal vector (stencil chain) --------------

// out = R v with R = h K_lap (Laplacian) or h K_el P h K_el + eps h K_lap.
// With p_old != null the input is p_new = v + beta p_old (PCG).
template <typename T>
static int apply_reg(GnSolver<T>* S, const T* v, T* out, cudaStream_t s) {
  const vdvc_gn_desc& d = S->d;
  StencilArgs<T> a{};
  a.m = S->m;
  a.E = (double)d.h;
  a.scale = 1.0;
  if (d.reg_type == VDVC_REG_LAPLACIAN) {
    a.v = v;
    a.out = out;
    return launch_kref_apply<T>(a, S->Klap, s);
  }
  int st;
  a.v = v;
  a.interior = (const T*)d.interior;
  a.out = S->t1;
  if ((st = launch_kref_apply<T>(a, S->Kel, s))) return st;
  StencilArgs<T> b2 = a;  // eps h K_lap v
  b2.interior = nullptr;
  b2.v = v;
  b2.scale = d.eps_reg;
  b2.out = out;
  if ((st = launch_kref_apply<T>(b2, S->Klap, s))) return st;
  StencilArgs<T> c2 = a;  // + h K_el t1
  c2.interior = nullptr;
  c2.v = S->t1;
  c2.add_to = out;
  c2.out = out;
  return launch_kref_apply<T>(c2, S->Kel, s);
}

// ---- one PCG iteration (captured into the graph) ----------------------------

// The Hessian pass of a PCG iteration: input p_new = z + beta p, H mask, the
// regularizer fused in its epilogue.
template <typename T>
static StripArgs<T> pcg_strip_args(GnSolver<T>* S) {
  const vdvc_gn_desc& d = S->d;
  StripArgs<T> sa{};
  sa.m = S->m;
  sa.v = S->z;
  sa.p_old = S->p;
  sa.st = S->pcg;
  sa.grad = (const T*)d.grad;
  // H mask: the b mask buffer (dynamic_mask) or mask0 -- fixed pointers, so
  // the captured graph stays valid for the solver's lifetime
  sa.mask = d.dynamic_mask ? S->frozen : d.mask0;
  sa.evA = S->evA;
  sa.nreg = 0;
  // K1 is the vector Laplacian in both regularizers; pass its 8x8 block when
  // it has the block structure of build_K_ref_laplacian
  sa.k1_blockdiag = S->lap_blockdiag ? 1 : 0;
  for (int q = 0; q < 64; ++q) sa.L8[q] = S->L8[q];
  if (d.ll != 0.0 && d.reg_type == VDVC_REG_LAPLACIAN) {
    sa.nreg = 1;
    sa.c1 = (T)(d.ll * d.h);
  } else if (d.ll != 0.0 && d.reg_type == VDVC_REG_EQUILIBRIUM_GAP) {
    sa.nreg = 2;
    sa.c1 = (T)(d.ll * d.eps_reg * d.h);
    sa.c2 = (T)(d.ll * d.h);
    sa.w = S->w;
  }
  return sa;
}

// VDVC_PCG=eager: the PCG iterations are launched from the host instead of
// the graph (a profiling mode: every kernel is a separate stream launch).
static bool eager_pcg() {
  const char* e = getenv("VDVC_PCG");
  return e && e[0] == 'e';
}

// After the element pass: p, Ap and alpha (gather), then the x / r / z
// update with the convergence test.
template <typename T>
static int pcg_gather_update(GnSolver<T>* S, cudaStream_t s) {
  GridReduce red{S->partials, S->ticket};
  int st = launch_pcg_gather<T>(S->m, S->evA, S->z, S->p, S->Ap, S->pcg, red, s, (long long)S->n_partials);
  if (st) return st;
  return launch_pcg_update<T>(S->p, S->Ap, S->Minv, S->m.Ndof, S->x, S->r, S->z, S->pcg, red, s);
}

template <typename T>
static int pcg_iteration(GnSolver<T>* S, cudaStream_t s) {
  const vdvc_gn_desc& d = S->d;
  GridReduce red{S->partials, S->ticket};
  int st;
  if (d.reg_type == VDVC_REG_EQUILIBRIUM_GAP && d.ll != 0.0) {
    StencilArgs<T> a{};
    a.m = S->m;
    a.v = S->z;
    a.p_old = S->p;
    a.st = S->pcg;
    a.E = (double)d.h;
    a.scale = 1.0;
    a.interior = (const T*)d.interior;
    a.out = S->w;
    if ((st = launch_kref_apply<T>(a, S->Kel, s))) return st;
  }
  if constexpr (std::is_same<T, float>::value) {
    if (S->eh) {
      EhMatvecArgs ma{};
      ma.m = S->m;
      ma.T = S->T_eh;
      ma.Tb = S->eh_T_bf16 ? (const void*)S->T_eh : nullptr;  // the precision form keeps BF16 entries
      ma.pitch = eh_pitch(S->m.Ne);
      ma.err = &S->sc->status;  // read with the GN scalars after the iteration
      ma.v = S->z;
      ma.p_old = S->p;
      ma.st = S->pcg;
      ma.ev = S->evA;
      for (int q = 0; q < 64; ++q) ma.L8[q] = S->L8[q];
      if (d.ll != 0.0 && d.reg_type == VDVC_REG_LAPLACIAN) {
        ma.nreg = 1;
        ma.c1 = (float)(d.ll * d.h);
      } else if (d.ll != 0.0 && d.reg_type == VDVC_REG_EQUILIBRIUM_GAP) {
        ma.nreg = 2;
        ma.c1 = (float)(d.ll * d.eps_reg * d.h);
        ma.c2 = (float)(d.ll * d.h);
        ma.w = S->w;
        ma.K2 = S->kp->K2;  // device address of the float K_el copy
      }
      if ((st = launch_eh_matvec<true>(ma, s))) return st;
      return pcg_gather_update<T>(S, s);
    }
  }
  const StripArgs<T> sa = pcg_strip_args<T>(S);
  if ((st = launch_strip<T, kModeHv | kModePcg>(sa, S->kp, s))) return st;
  return pcg_gather_update<T>(S, s);
}

// Keeps the WHILE node of the PCG graph running until the state says done.
__global__ void k_pcg_continue(cudaGraphConditionalHandle h, const PcgState* st) {
  if (threadIdx.x == 0) cudaGraphSetConditional(h, st->done ? 0u : 1u);
}

// The whole PCG loop as one CUDA graph: a WHILE conditional node whose body
// is `chunk` captured iterations followed by k_pcg_continue, so the device
// itself decides when to stop and the host launches once per solve.
template <typename T>
static int build_graph(GnSolver<T>* S) {
  if (S->gexec) {
    cudaGraphExecDestroy(S->gexec);
    S->gexec = nullptr;
  }
  if (S->graph) {
    cudaGraphDestroy(S->graph);
    S->graph = nullptr;
  }
  cudaGraph_t g = nullptr;
  VDVC_CUDA(cudaGraphCreate(&g, 0));
  S->graph = g;
  cudaGraphConditionalHandle hnd;
  VDVC_CUDA(cudaGraphConditionalHandleCreate(&hnd, g, 1u, cudaGraphCondAssignDefault));
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = hnd;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  VDVC_CUDA(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np));
  cudaGraph_t body = np.conditional.phGraph_out[0];
  cudaStream_t cs = S->cap_stream;
  VDVC_CUDA(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  const long long before = vdvc_launch_count();
  int st = VDVC_OK;
  for (int it = 0; it < S->chunk && st == VDVC_OK; ++it) st = pcg_iteration<T>(S, cs);
  const long long captured = vdvc_launch_count() - before;
  count_launch(-captured);  // captured launches run (and are counted) at replay time
  if (st == VDVC_OK) {
    k_pcg_continue<<<1, 32, 0, cs>>>(hnd, S->pcg);
    if (cudaGetLastError() != cudaSuccess) st = set_error(VDVC_ERR_CUDA, "continue kernel capture failed");
  }
  cudaGraph_t body_out = nullptr;
  cudaError_t e = cudaStreamEndCapture(cs, &body_out);
  if (st) return st;
  if (e != cudaSuccess) return set_error(VDVC_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  S->kernels_per_iter = (int)(captured / S->chunk);
  VDVC_CUDA(cudaGraphInstantiate(&S->gexec, g, 0));
  return VDVC_OK;
}

template <typename T>
static size_t solver_bytes(const Mesh& m) {
  GnSolver<T> tmp{};
  return carve_solver<T>(m, &tmp, nullptr, 0) + 256;
}

template <typename T>
static int create(const vdvc_gn_desc* d, void* ws, size_t ws_bytes, void** out) {
  Mesh m;
  int st = make_mesh(d->h, d->Nx, d->Ny, d->Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(d->f_vox && d->g_vox && d->grad && d->mask0, "null input pointer");
  VDVC_CHECK_ARG(d->gnx >= 1 && d->gny >= 1 && d->gnz >= 1, "bad g shape");
  if (m.Nnodes >= (1ll << 32)) return set_error(VDVC_ERR_UNSUPPORTED, "2^32 nodes or more");
  VDVC_CHECK_ARG(d->reg_type >= VDVC_REG_NONE && d->reg_type <= VDVC_REG_EQUILIBRIUM_GAP, "bad reg_type");
  if (d->reg_type != VDVC_REG_NONE) VDVC_CHECK_ARG(d->K_lap != nullptr, "K_lap required");
  if (d->reg_type == VDVC_REG_EQUILIBRIUM_GAP)
    VDVC_CHECK_ARG(d->K_el && d->interior && d->diag_eqgap, "equilibrium gap needs K_el, interior, diag_eqgap");
  GnSolver<T>* S = new (std::nothrow) GnSolver<T>();
  if (!S) return set_error(VDVC_ERR_ARG, "host allocation failed");
  S->m = m;
  S->d = *d;
  size_t need = solver_bytes<T>(m);
  if (!ws || ws_bytes < need) {
    delete S;
    return set_error(VDVC_ERR_WORKSPACE, "solver needs %zu bytes of workspace (got %zu)", need, ws_bytes);
  }
  carve_solver<T>(m, S, ws, ws_bytes);
  S->eh = d->precision == VDVC_PREC_MIXED || d->precision == VDVC_PREC_ELEMENT;
  S->eh_bf16 = d->precision == VDVC_PREC_MIXED;
  // The equilibrium-gap system keeps FP32 entries: its PCG runs hundreds of
  // iterations on a stiff operator and, within a GN iteration cap, ends
  // where the rounding of H steers the Krylov trajectory.
  S->eh_T_bf16 = S->eh_bf16 && d->reg_type != VDVC_REG_EQUILIBRIUM_GAP;
  if (d->precision != VDVC_PREC_PLAIN && !S->eh) {
    delete S;
    return set_error(VDVC_ERR_ARG, "precision %d", d->precision);
  }
  if (S->eh) {
    Carve cv(d->eh_ws, d->eh_ws_bytes);
    S->T_eh = cv.take<float>((size_t)162 * eh_pitch(m.Ne));
    S->gmax = cv.take<float>(4);
    S->grad_bf16 = S->eh_bf16 ? cv.take<uint16_t>((size_t)3 * m.Nvox) : nullptr;
    const bool ok = std::is_same<T, float>::value;
    const bool h_ok = d->h == 1 || d->h == 2 || d->h == 3 || d->h == 4 || d->h == 6 || d->h == 8 || d->h == 12 ||
                      d->h == 16;
    if (!ok || !h_ok || !d->eh_ws || !cv.fits()) {
      delete S;
      if (!ok) return set_error(VDVC_ERR_ARG, "the element-Hessian forms are float32 solves");
      if (!h_ok)
        return set_error(VDVC_ERR_UNSUPPORTED, "element Hessians for h=%d (h in {1,2,3,4,6,8,12,16})", d->h);
      return set_error(VDVC_ERR_WORKSPACE, "element-Hessian form needs eh_ws of vdvc_gn_eh_workspace_bytes bytes");
    }
  }
  if (d->K_lap) load_K(d->K_lap, &S->Klap);
  if (d->K_el) load_K(d->K_el, &S->Kel);
  // K_lap[3a+c][3b+c'] == (c == c') * L8[a][b] ?
  S->lap_blockdiag = d->K_lap != nullptr;
  for (int r = 0; r < 24 && S->lap_blockdiag; ++r)
    for (int q = 0; q < 24; ++q) {
      const double v = S->Klap.k[r * 24 + q];
      const double ref = (r % 3 == q % 3) ? S->Klap.k[(r / 3) * 3 * 24 + (q / 3) * 3] : 0.0;
      if (v != ref) {
        S->lap_blockdiag = false;
        break;
      }
    }
  for (int a = 0; a < 8; ++a)
    for (int b = 0; b < 8; ++b) S->L8[a * 8 + b] = (float)S->Klap.k[(3 * a) * 24 + 3 * b];
  if (S->eh && d->reg_type != VDVC_REG_NONE && !S->lap_blockdiag) {
    delete S;
    return set_error(VDVC_ERR_UNSUPPORTED, "element-Hessian form needs K_lap = one 8x8 block per component");
  }
  S->chunk = d->pcg_chunk > 0 ? d->pcg_chunk : 4;
  cudaStream_t s = (cudaStream_t)d->stream;
  int e = VDVC_OK;
  static_assert(2 * sizeof(PcgState) + sizeof(GnScalars) <= kPinnedSlot, "pinned read-back slot too small");
  auto fail = [&](int code) {
    pool_stream_return(S->cap_stream);
    pool_stream_return(S->side);
    pool_event_return(S->ev[0]);
    pool_event_return(S->ev[1]);
    pool_event_return(S->ev_fork);
    pool_event_return(S->ev_join);
    pool_pinned_return(S->h_pcg);
    delete S;
    return code;
  };
  void* pin = nullptr;
  if (pool_stream(&S->cap_stream) || pool_pinned(&pin) || pool_event(&S->ev[0]) || pool_event(&S->ev[1]) ||
      (S->eh && (pool_stream(&S->side) || pool_event(&S->ev_fork) || pool_event(&S->ev_join)))) {
    S->h_pcg = (PcgState*)pin;
    return fail(set_error(VDVC_ERR_CUDA, "solver stream/event/pinned setup failed"));
  }
  S->h_pcg = (PcgState*)pin;
  S->h_sc = (GnScalars*)(S->h_pcg + 2);
  // device-side constants: the fused K pair, zeroed reduction tickets, scalars
  Kpair<T> kh;
  for (int q = 0; q < 576; ++q) {
    kh.K1[q] = (T)S->Klap.k[q];
    kh.K2[q] = (T)S->Kel.k[q];
  }
  if (cudaMemcpyAsync(S->kp, &kh, sizeof(kh), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemsetAsync(S->ticket, 0, 4 * sizeof(unsigned int), s) != cudaSuccess ||
      cudaMemsetAsync(S->sc, 0, sizeof(GnScalars), s) != cudaSuccess)
    return fail(set_error(VDVC_ERR_CUDA, "solver upload failed"));
  // regularizer diagonal in float64: h diag(K_lap) [+ eq. gap Hutchinson]
  if (d->reg_type != VDVC_REG_NONE) {
    if ((e = launch_kref_diag<double>(m, S->Klap, nullptr, (double)d->h, S->diag_reg, s))) return fail(e);
    if (d->reg_type == VDVC_REG_EQUILIBRIUM_GAP) {
      // diag_reg = diag_eqgap + eps * h diag(K_lap)
      const long long n = m.Ndof;
      k_add_scaled_f64<<<nblk(n), 256, 0, s>>>(S->diag_reg, S->diag_reg, d->eps_reg - 1.0, n);
      k_add_scaled_f64<<<nblk(n), 256, 0, s>>>(S->diag_reg, d->diag_eqgap, 1.0, n);
      count_launch(2);
    }
  }
  if (d->reg_type != VDVC_REG_NONE) {
    k_copy_out<double><<<nblk(m.Ndof), 256, 0, s>>>(S->diag_reg, m.Ndof, S->diag_reg_t,
                                                     std::is_same<T, double>::value ? 1 : 0);
    count_launch();
  }
  k_set_U<T><<<nblk(m.Ndof), 256, 0, s>>>(nullptr, m.Ndof, S->U64, S->U32);
  count_launch();
  if (S->eh_bf16 && (e = launch_grad_bf16((const float*)d->grad, 3 * m.Nvox, S->grad_bf16, S->gmax, s))) return fail(e);
  // sync before the graph (captured on a private stream) sees the buffers
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail(set_error(VDVC_ERR_CUDA, "solver setup sync failed"));
  *out = S;
  return VDVC_OK;
}

template <typename T>
static int set_U(GnSolver<T>* S, const double* U0, cudaStream_t s) {
  k_set_U<T><<<nblk(S->m.Ndof), 256, 0, s>>>(U0, S->m.Ndof, S->U64, S->U32);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

// Element-Hessian formation over `mask` from the solver's gradient (float32,
// or its BF16 rounding in the precision form).
template <typename T>
static EhFormArgs eh_form_args(GnSolver<T>* S, const uint8_t* mask) {
  EhFormArgs fa{S->m, S->eh_bf16 ? S->grad_bf16 : S->d.grad, mask, S->T_eh, (float*)S->evD, eh_pitch(S->m.Ne),
                S->eh_bf16 ? S->gmax : nullptr, &S->sc->status, S->eh_bf16 ? 0 : 1,
                S->eh_T_bf16 ? (void*)S->T_eh : nullptr};
  return fa;
}

// Frozen-H preconditioner (dynamic_mask == 0): diag H over mask0, built once.
template <typename T>
static int frozen_diag(GnSolver<T>* S, cudaStream_t s) {
  int st;
  if (S->eh) {
    if ((st = launch_eh_form(eh_form_args(S, S->d.mask0), s))) return st;
    S->eh_fixed = true;
  } else {
    StripArgs<T> a{};
    a.m = S->m;
    a.grad = (const T*)S->d.grad;
    a.mask = S->d.mask0;
    a.evD = S->evD;
    if ((st = launch_strip<T, kModeDiag>(a, nullptr, s))) return st;
  }
  GridReduce red{S->partials, S->ticket};
  k_gn_gather_rhs<T><<<grid_blocks(S->m.Nnodes, 256, (long long)S->n_partials), 256, 0, s>>>(
      S->m, S->evD, S->evD, nullptr, S->d.ll, S->d.reg_type != VDVC_REG_NONE ? S->diag_reg_t : nullptr, S->t1,
      S->diag, S->sc, red, true);
  VDVC_LAUNCHED();
  k_gn_minv<T><<<nblk(S->m.Ndof), 256, 0, s>>>(S->diag, S->m.Ndof, S->sc, S->Minv);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

template <typename T>
static int sample(GnSolver<T>* S, int freeze_now, cudaStream_t s) {
  const vdvc_gn_desc& d = S->d;
  SampleArgs<T> a{};
  a.m = S->m;
  a.U = S->U32;
  a.g = (const T*)d.g_vox;
  a.gnx = d.gnx; a.gny = d.gny; a.gnz = d.gnz;
  a.gx0 = (T)d.gx0; a.gy0 = (T)d.gy0; a.gz0 = (T)d.gz0;
  a.mask0 = d.mask0;
  a.glt = (T)d.glt;
  a.gvals = S->gvals;
  // S->frozen is the b mask buffer: it follows the live mask until the freeze
  // iteration (engine/correlate_gpu.py:1079-1081) and is kept after it.
  // Until then the live mask is written there alone (one byte stream per
  // voxel, not two), after it into S->live.
  a.mask_out = S->frozen_set ? S->live : S->frozen;
  a.bmask_frozen = S->frozen_set ? S->frozen : nullptr;
  S->live_is_b = !S->frozen_set;
  a.red = GridReduce{S->partials, S->ticket};
  a.stats = S->sc->gstats;
  int st = launch_sample<T, true, false>(a, s);
  if (st) return st;
  if (freeze_now && !S->frozen_set) S->frozen_set = true;
  return VDVC_OK;
}

template <typename T>
static int rhs(GnSolver<T>* S, cudaStream_t s) {
  const vdvc_gn_desc& d = S->d;
  int st;
  const bool reg = d.reg_type != VDVC_REG_NONE && d.ll != 0.0;
  if (reg && (st = apply_reg<T>(S, S->U32, S->ru, s))) return st;
  StripArgs<T> a{};
  a.m = S->m;
  a.grad = (const T*)d.grad;
  a.mask = S->frozen;  // b mask
  a.f = (const T*)d.f_vox;
  a.gvals = S->gvals;
  a.live = S->live_is_b ? S->frozen : S->live;
  a.gstats = S->sc->gstats;
  a.mean0 = d.mean0;
  a.std0 = d.std0;
  a.res_out = S->res;
  a.red = GridReduce{S->partials, S->ticket};
  a.dstats = S->sc->dstats;
  a.status = &S->sc->status;
  a.evA = S->evA;
  a.evD = S->evD;
  // diag H from the strip pass (matrix-free), from the element Hessians, or
  // not at all once it is final
  const bool with_diag = d.dynamic_mask && !S->eh_fixed;
  const bool form = with_diag && S->eh;
  if (form) {
    // The element Hessians (gradient and b mask) and the residual pass
    // (f, g values, b and live masks) are independent: the formation runs
    // on the solver's side stream, beside the residual pass, and the
    // gather below waits for both.
    VDVC_CUDA(cudaEventRecord(S->ev_fork, s));
    VDVC_CUDA(cudaStreamWaitEvent(S->side, S->ev_fork, 0));
    if ((st = launch_eh_form(eh_form_args(S, S->frozen), S->side))) return st;
    VDVC_CUDA(cudaEventRecord(S->ev_join, S->side));
  }
  if (with_diag && !S->eh)
    st = launch_strip<T, kModeB | kModeRes | kModeDiag>(a, nullptr, s);
  else
    st = launch_strip<T, kModeB | kModeRes>(a, nullptr, s);
  if (form) {
    // joined even when the residual launch failed: nothing is left pending
    // on the side stream behind the caller's stream
    VDVC_CUDA(cudaStreamWaitEvent(s, S->ev_join, 0));
    if (S->frozen_set) S->eh_fixed = true;
  }
  if (st) return st;
  GridReduce red{S->partials, S->ticket};
  k_gn_gather_rhs<T><<<grid_blocks(S->m.Nnodes, 256, (long long)S->n_partials), 256, 0, s>>>(
      S->m, S->evA, S->evD, reg ? S->ru : nullptr, d.ll, d.reg_type != VDVC_REG_NONE ? S->diag_reg_t : nullptr, S->b,
      S->diag, S->sc, red, with_diag);
  VDVC_LAUNCHED();
  if (with_diag) {
    k_gn_minv<T><<<nblk(S->m.Ndof), 256, 0, s>>>(S->diag, S->m.Ndof, S->sc, S->Minv);
    VDVC_LAUNCHED();
  }
  return VDVC_OK;
}

// PCG from dU = 0 on the stream: the graph (or, in the eager mode, the
// host-launched iterations) and the copy of the final state into the pinned
// read-back slot.  *graph_ran: whether the graph ran (its launches are
// counted once the final iteration count is known).
template <typename T>
static int pcg_enqueue(GnSolver<T>* S, int max_iter, double tol, cudaStream_t s, bool* graph_ran) {
  // A residual normalisation failure of the rhs pass (the reference raises
  // at engine/correlate_gpu.py:1095) leaves a non-finite b: the PCG stops on
  // it at once and vdvc_gn_update reports the rhs status, so the iteration
  // needs no extra synchronisation here.
  GridReduce red{S->partials, S->ticket};
  int st = launch_pcg_init<T>(S->b, nullptr, S->Minv, S->m.Ndof, S->r, S->z, S->p, false, S->x, S->pcg, red,
                              max_iter, tol, s);
  if (st) return st;
  *graph_ran = false;
  if (eager_pcg()) {
    // the same iteration kernels launched from the host, so that a profiler
    // sees each launch; the device state is read every 16 iterations
    for (int it = 0; it < max_iter; ++it) {
      if ((st = pcg_iteration<T>(S, s))) return st;
      if ((it & 15) == 15 || it == max_iter - 1) {
        VDVC_CUDA(cudaMemcpyAsync(S->h_pcg, S->pcg, sizeof(PcgState), cudaMemcpyDeviceToHost, s));
        VDVC_CUDA(cudaStreamSynchronize(s));
        if (S->h_pcg->done) break;
      }
    }
  } else {
    if (!S->gexec && (st = build_graph<T>(S))) return st;
    if (max_iter > 0) {
      VDVC_CUDA(cudaGraphLaunch(S->gexec, s));
      *graph_ran = true;
    }
  }
  VDVC_CUDA(cudaMemcpyAsync(S->h_pcg, S->pcg, sizeof(PcgState), cudaMemcpyDeviceToHost, s));
  return VDVC_OK;
}

// After the stream has synchronised: the final PCG state, and the graph's
// launches counted.
template <typename T>
static const PcgState& pcg_finish(GnSolver<T>* S, bool graph_ran) {
  const PcgState& fin = S->h_pcg[0];
  if (graph_ran) {
    // body executions = ceil(iter / chunk); each runs chunk iterations' kernels + the continue kernel
    const long long bodies = (fin.iter + S->chunk - 1) / S->chunk;
    count_launch(bodies * ((long long)S->chunk * S->kernels_per_iter + 1));
  }
  return fin;
}

template <typename T>
static int pcg(GnSolver<T>* S, int max_iter, double tol, int* iters, double* res, int* status, cudaStream_t s) {
  bool graph_ran = false;
  int st = pcg_enqueue<T>(S, max_iter, tol, s, &graph_ran);
  if (st) return st;
  VDVC_CUDA(cudaStreamSynchronize(s));
  const PcgState& fin = pcg_finish<T>(S, graph_ran);
  if (iters) *iters = fin.iter;
  if (res) *res = fin.res;
  if (status) *status = fin.status;
  return VDVC_OK;
}

// U += dU and the iteration scalars into the pinned read-back slots (no sync)
template <typename T>
static int update_enqueue(GnSolver<T>* S, cudaStream_t s) {
  GridReduce red{S->partials, S->ticket};
  k_gn_update<T><<<grid_blocks(S->m.Ndof, 256, kReduceBlocks), 256, 0, s>>>(S->x, S->m.Ndof, S->U64, S->U32, S->sc,
                                                                            red);
  VDVC_LAUNCHED();
  VDVC_CUDA(cudaMemcpyAsync(S->h_sc, S->sc, sizeof(GnScalars), cudaMemcpyDeviceToHost, s));
  return VDVC_OK;
}

template <typename T>
static int update(GnSolver<T>* S, double* out8, cudaStream_t s) {
  int st = update_enqueue<T>(S, s);
  if (st) return st;
  VDVC_CUDA(cudaStreamSynchronize(s));
  const GnScalars& h = *S->h_sc;
  if (out8) {
    out8[0] = h.norms[0];
    out8[1] = h.norms[1];
    out8[2] = h.dstats[0];
    out8[3] = h.dstats[1];
    out8[4] = h.dstats[2];
    out8[5] = h.gstats[3];
    out8[6] = h.gstats[0];
    out8[7] = (double)h.status;
  }
  if (h.status != VDVC_OK) {
    const int code = h.status;
    cudaMemsetAsync(&S->sc->status, 0, sizeof(int), s);
    return set_error(code, code == VDVC_ERR_ZERO_DIVISION ? "float division by zero (std of g over the mask is 0)"
                                                          : "solver status %d", code);
  }
  return VDVC_OK;
}

// One whole GN iteration with a single host synchronisation: sample, rhs,
// PCG, update, then every scalar of the iteration at once.  out12: the 8
// values of update(), PCG iterations, PCG relative residual, PCG status, the
// solver status.
template <typename T>
static int iterate(GnSolver<T>* S, int freeze_now, int max_iter, double tol, double* out12, cudaStream_t s) {
  int st;
  if ((st = sample<T>(S, freeze_now, s))) return st;
  if ((st = rhs<T>(S, s))) return st;
  bool graph_ran = false;
  if ((st = pcg_enqueue<T>(S, max_iter, tol, s, &graph_ran))) return st;
  if ((st = update_enqueue<T>(S, s))) return st;
  VDVC_CUDA(cudaStreamSynchronize(s));
  const PcgState& fin = pcg_finish<T>(S, graph_ran);
  const GnScalars& h = *S->h_sc;
  if (out12) {
    out12[0] = h.norms[0];
    out12[1] = h.norms[1];
    out12[2] = h.dstats[0];
    out12[3] = h.dstats[1];
    out12[4] = h.dstats[2];
    out12[5] = h.gstats[3];
    out12[6] = h.gstats[0];
    out12[7] = (double)h.status;
    out12[8] = (double)fin.iter;
    out12[9] = fin.res;
    out12[10] = (double)fin.status;
    out12[11] = (double)h.status;
  }
  if (h.status != VDVC_OK) {
    const int code = h.status;
    cudaMemsetAsync(&S->sc->status, 0, sizeof(int), s);
    return set_error(code, code == VDVC_ERR_ZERO_DIVISION ? "float division by zero (std of g over the mask is 0)"
                                                          : "solver status %d", code);
  }
  return VDVC_OK;
}

template <typename T>
static int read(GnSolver<T>* S, int which, void* dst, int dst_f64, cudaStream_t s) {
  const long long nd = S->m.Ndof, nv = S->m.Nvox;
  switch (which) {
    case VDVC_GN_U:
      if (dst_f64) {
        // dst may be device or (pinned, mapped) host memory
        VDVC_CUDA(cudaMemcpyAsync(dst, S->U64, nd * sizeof(double), cudaMemcpyDefault, s));
      } else {
        k_copy_out<double><<<nblk(nd), 256, 0, s>>>(S->U64, nd, dst, 0);
        VDVC_LAUNCHED();
      }
      return VDVC_OK;
    case VDVC_GN_DU:
      k_copy_out<T><<<nblk(nd), 256, 0, s>>>(S->x, nd, dst, dst_f64);
      VDVC_LAUNCHED();
      return VDVC_OK;
    case VDVC_GN_RES:
      k_copy_out<T><<<nblk(nv), 256, 0, s>>>(S->res, nv, dst, dst_f64);
      VDVC_LAUNCHED();
      return VDVC_OK;
    case VDVC_GN_LIVE_MASK:
      VDVC_CUDA(cudaMemcpyAsync(dst, S->live_is_b ? S->frozen : S->live, nv, cudaMemcpyDefault, s));
      return VDVC_OK;
  }
  return set_error(VDVC_ERR_ARG, "unknown buffer %d", which);
}

template <typename T>
static void destroy(GnSolver<T>* S) {
  if (!S) return;
  if (S->gexec) cudaGraphExecDestroy(S->gexec);
  if (S->graph) cudaGraphDestroy(S->graph);
  pool_stream_return(S->cap_stream);
  pool_stream_return(S->side);
  pool_event_return(S->ev[0]);
  pool_event_return(S->ev[1]);
  pool_event_return(S->ev_fork);
  pool_event_return(S->ev_join);
  pool_pinned_return(S->h_pcg);
  delete S;
}

// ---- batches of independent solves ------------------------------------------
//
// A series of deformed volumes (different ROIs, element sizes h, masks) are
// iterated in lockstep: one GN iteration of every active problem per call.
// Sampling, residual and PCG set-up run on one stream per problem (the small
// problems overlap on the GPU), then the PCG loops of all active problems
// run as ONE CUDA graph: a WHILE node whose body holds `chunk` iterations of
// every problem as parallel branches and a continue kernel that keeps the
// loop going while any problem's PCG state is not done (a problem that
// converged skips its kernels).  One host synchronisation per GN iteration
// reads every problem's scalars.  The graph holds every problem of the
// batch and is built once per schedule: a problem that left the lockstep
// keeps its PCG state at done, so its captured kernels return at once
// (rebuilding the graph whenever a problem converged cost a capture and an
// instantiation per convergence, more than the early returns).

__global__ void k_pcg_mark_done(PcgState* st) {
  if (threadIdx.x == 0) st->done = 1;
}

__global__ void k_batch_continue(cudaGraphConditionalHandle h, PcgState* const* states, int n) {
  if (threadIdx.x == 0) {
    unsigned int more = 0;
    for (int i = 0; i < n; ++i) more |= states[i]->done ? 0u : 1u;
    cudaGraphSetConditional(h, more);
  }
}

struct GnBatch {
  int n = 0;
  int chunk = 4;
  int concurrent = 1;  // 1: problems on their own streams (parallel graph branches)
  std::vector<GnSolver<float>*> S;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> done_ev;
  cudaEvent_t fork_ev = nullptr;
  cudaStream_t cap = nullptr;
  PcgState** d_states = nullptr;  // device array of the active problems' PCG states
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<char> graph_active;
  long long kernels_per_body = 0;
};

static void batch_free_graph(GnBatch* B) {
  if (B->exec) cudaGraphExecDestroy(B->exec);
  if (B->graph) cudaGraphDestroy(B->graph);
  B->exec = nullptr;
  B->graph = nullptr;
}

static cudaStream_t batch_stream(GnBatch* B, int i, cudaStream_t main) {
  return B->concurrent ? B->streams[i] : main;
}

static int batch_build_graph(GnBatch* B, const std::vector<char>& active) {
  batch_free_graph(B);
  std::vector<PcgState*> h_states;
  for (int i = 0; i < B->n; ++i)
    if (active[i]) h_states.push_back(B->S[i]->pcg);
  VDVC_CUDA(cudaMemcpy(B->d_states, h_states.data(), h_states.size() * sizeof(PcgState*), cudaMemcpyHostToDevice));
  cudaGraph_t g = nullptr;
  VDVC_CUDA(cudaGraphCreate(&g, 0));
  B->graph = g;
  cudaGraphConditionalHandle hnd;
  VDVC_CUDA(cudaGraphConditionalHandleCreate(&hnd, g, 1u, cudaGraphCondAssignDefault));
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = hnd;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  VDVC_CUDA(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np));
  cudaGraph_t body = np.conditional.phGraph_out[0];
  cudaStream_t cs = B->cap;
  VDVC_CUDA(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  const long long before = vdvc_launch_count();
  int st = VDVC_OK;
  if (cudaEventRecord(B->fork_ev, cs) != cudaSuccess) st = set_error(VDVC_ERR_CUDA, "batch fork record");
  for (int i = 0; i < B->n && st == VDVC_OK; ++i) {
    if (!active[i]) continue;
    cudaStream_t ps = B->concurrent ? B->streams[i] : cs;
    if (B->concurrent && cudaStreamWaitEvent(ps, B->fork_ev, 0) != cudaSuccess) {
      st = set_error(VDVC_ERR_CUDA, "batch fork wait");
      break;
    }
    for (int it = 0; it < B->chunk && st == VDVC_OK; ++it) st = pcg_iteration<float>(B->S[i], ps);
    if (st == VDVC_OK && B->concurrent) {
      if (cudaEventRecord(B->done_ev[i], ps) != cudaSuccess || cudaStreamWaitEvent(cs, B->done_ev[i], 0) != cudaSuccess)
        st = set_error(VDVC_ERR_CUDA, "batch join");
    }
  }
  const long long captured = vdvc_launch_count() - before;
  count_launch(-captured);
  if (st == VDVC_OK) {
    k_batch_continue<<<1, 32, 0, cs>>>(hnd, B->d_states, (int)h_states.size());
    if (cudaGetLastError() != cudaSuccess) st = set_error(VDVC_ERR_CUDA, "batch continue kernel capture failed");
  }
  cudaGraph_t body_out = nullptr;
  cudaError_t e = cudaStreamEndCapture(cs, &body_out);
  if (st) return st;
  if (e != cudaSuccess) return set_error(VDVC_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(e));
  B->kernels_per_body = captured + 1;
  VDVC_CUDA(cudaGraphInstantiate(&B->exec, g, 0));
  B->graph_active = active;
  return VDVC_OK;
}

// One GN iteration of every active problem.  out: 12 doubles per problem:
// the 8 values of vdvc_gn_update, PCG iterations, PCG residual, PCG status,
// residual status (VDVC_ERR_ZERO_DIVISION when std(g) over the b mask is 0).
static int batch_iterate(GnBatch* B, const int* active_in, const int* freeze_now, int max_iter, double tol,
                         double* out, cudaStream_t s) {
  std::vector<char> active(B->n);
  int n_active = 0;
  for (int i = 0; i < B->n; ++i) n_active += (active[i] = active_in[i] ? 1 : 0);
  if (n_active == 0) return VDVC_OK;
  int st;
  if (max_iter > 0 && !B->exec && (st = batch_build_graph(B, std::vector<char>(B->n, 1)))) return st;
  // problems outside the lockstep: their captured PCG kernels must return at once
  for (int i = 0; i < B->n; ++i)
    if (!active[i]) {
      k_pcg_mark_done<<<1, 32, 0, s>>>(B->S[i]->pcg);
      VDVC_LAUNCHED();
    }
  // sampling, residual, b, diag and the PCG start of every active problem
  VDVC_CUDA(cudaEventRecord(B->fork_ev, s));
  for (int i = 0; i < B->n; ++i) {
    if (!active[i]) continue;
    GnSolver<float>* S = B->S[i];
    cudaStream_t ps = batch_stream(B, i, s);
    if (B->concurrent) VDVC_CUDA(cudaStreamWaitEvent(ps, B->fork_ev, 0));
    if ((st = sample<float>(S, freeze_now ? freeze_now[i] : 0, ps))) return st;
    if ((st = rhs<float>(S, ps))) return st;
    GridReduce red{S->partials, S->ticket};
    if ((st = launch_pcg_init<float>(S->b, nullptr, S->Minv, S->m.Ndof, S->r, S->z, S->p, false, S->x, S->pcg, red,
                                     max_iter, tol, ps)))
      return st;
    if (B->concurrent) {
      VDVC_CUDA(cudaEventRecord(B->done_ev[i], ps));
      VDVC_CUDA(cudaStreamWaitEvent(s, B->done_ev[i], 0));
    }
  }
  if (max_iter > 0) VDVC_CUDA(cudaGraphLaunch(B->exec, s));
  VDVC_CUDA(cudaEventRecord(B->fork_ev, s));
  for (int i = 0; i < B->n; ++i) {
    if (!active[i]) continue;
    GnSolver<float>* S = B->S[i];
    cudaStream_t ps = batch_stream(B, i, s);
    if (B->concurrent) VDVC_CUDA(cudaStreamWaitEvent(ps, B->fork_ev, 0));
    if ((st = update_enqueue<float>(S, ps))) return st;
    VDVC_CUDA(cudaMemcpyAsync(S->h_pcg, S->pcg, sizeof(PcgState), cudaMemcpyDeviceToHost, ps));
    if (B->concurrent) {
      VDVC_CUDA(cudaEventRecord(B->done_ev[i], ps));
      VDVC_CUDA(cudaStreamWaitEvent(s, B->done_ev[i], 0));
    }
  }
  VDVC_CUDA(cudaStreamSynchronize(s));
  int max_it = 0;
  for (int i = 0; i < B->n; ++i) {
    if (!active[i]) continue;
    GnSolver<float>* S = B->S[i];
    const GnScalars& h = *S->h_sc;
    const PcgState& pc = S->h_pcg[0];
    double* o = out + 12 * (size_t)i;
    o[0] = h.norms[0];
    o[1] = h.norms[1];
    o[2] = h.dstats[0];
    o[3] = h.dstats[1];
    o[4] = h.dstats[2];
    o[5] = h.gstats[3];
    o[6] = h.gstats[0];
    o[7] = (double)h.status;
    o[8] = (double)pc.iter;
    o[9] = pc.res;
    o[10] = (double)pc.status;
    o[11] = (double)h.status;
    if (pc.iter > max_it) max_it = pc.iter;
    if (h.status != VDVC_OK) VDVC_CUDA(cudaMemsetAsync(&S->sc->status, 0, sizeof(int), s));
  }
  if (max_iter > 0) count_launch(((max_it + B->chunk - 1) / B->chunk) * B->kernels_per_body);
  return VDVC_OK;
}

static void batch_destroy(GnBatch* B) {
  if (!B) return;
  batch_free_graph(B);
  for (auto* S : B->S) destroy<float>(S);
  for (auto st : B->streams) pool_stream_return(st);
  for (auto ev : B->done_ev) pool_event_return(ev);
  pool_event_return(B->fork_ev);
  pool_stream_return(B->cap);
  if (B->d_states) cudaFree(B->d_states);
  delete B;
}

}  // namespace vdvc

using namespace vdvc;

struct vdvc_gn_solver {
  int dtype;
  void* impl;
  bool borrowed = false;  // owned by a batch
};

struct vdvc_gn_batch {
  GnBatch* impl;
  std::vector<vdvc_gn_solver*> handles;
};

extern "C" {

size_t vdvc_gn_workspace_bytes(int dtype, int h, int Nx, int Ny, int Nz) {
  Mesh m;
  if (make_mesh(h, Nx, Ny, Nz, &m)) return 0;
  if (dtype == VDVC_F32) return solver_bytes<float>(m);
  if (dtype == VDVC_F64) return solver_bytes<double>(m);
  return 0;
}

int vdvc_gn_create(const vdvc_gn_desc* desc, void* ws, size_t ws_bytes, vdvc_gn_solver** out) {
  VDVC_CHECK_ARG(desc && out, "null pointer");
  vdvc_gn_solver* h = new (std::nothrow) vdvc_gn_solver();
  if (!h) return set_error(VDVC_ERR_ARG, "host allocation failed");
  h->dtype = desc->dtype;
  int st;
  if (desc->dtype == VDVC_F32)
    st = create<float>(desc, ws, ws_bytes, &h->impl);
  else if (desc->dtype == VDVC_F64)
    st = create<double>(desc, ws, ws_bytes, &h->impl);
  else
    st = set_error(VDVC_ERR_ARG, "dtype %d", desc->dtype);
  if (st) {
    delete h;
    return st;
  }
  *out = h;
  return VDVC_OK;
}

#define VDVC_GN_DISPATCH(call_f, call_d)                                      \
  do {                                                                        \
    VDVC_CHECK_ARG(solver != nullptr, "null solver");                         \
    if (solver->dtype == VDVC_F32) {                                          \
      GnSolver<float>* S = (GnSolver<float>*)solver->impl;                    \
      return call_f;                                                          \
    } else {                                                                  \
      GnSolver<double>* S = (GnSolver<double>*)solver->impl;                  \
      return call_d;                                                          \
    }                                                                         \
  } while (0)

int vdvc_gn_set_U(vdvc_gn_solver* solver, const double* U0, vdvc_stream_t stream) {
  VDVC_GN_DISPATCH(set_U<float>(S, U0, (cudaStream_t)stream), set_U<double>(S, U0, (cudaStream_t)stream));
}

int vdvc_gn_frozen_diag(vdvc_gn_solver* solver, vdvc_stream_t stream) {
  VDVC_GN_DISPATCH(frozen_diag<float>(S, (cudaStream_t)stream), frozen_diag<double>(S, (cudaStream_t)stream));
}

int vdvc_gn_sample(vdvc_gn_solver* solver, int freeze_now, vdvc_stream_t stream) {
  VDVC_GN_DISPATCH(sample<float>(S, freeze_now, (cudaStream_t)stream),
                   sample<double>(S, freeze_now, (cudaStream_t)stream));
}

int vdvc_gn_rhs(vdvc_gn_solver* solver, vdvc_stream_t stream) {
  VDVC_GN_DISPATCH(rhs<float>(S, (cudaStream_t)stream), rhs<double>(S, (cudaStream_t)stream));
}

int vdvc_gn_pcg(vdvc_gn_solver* solver, int max_iter, double tol, int* iters, double* res, int* status,
                vdvc_stream_t stream) {
  VDVC_GN_DISPATCH(pcg<float>(S, max_iter, tol, iters, res, status, (cudaStream_t)stream),
                   pcg<double>(S, max_iter, tol, iters, res, status, (cudaStream_t)stream));
}

int vdvc_gn_update(vdvc_gn_solver* solver, double* out8, vdvc_stream_t stream) {
  VDVC_GN_DISPATCH(update<float>(S, out8, (cudaStream_t)stream), update<double>(S, out8, (cudaStream_t)stream));
}

int vdvc_gn_iterate(vdvc_gn_solver* solver, int freeze_now, int max_iter, double tol, double* out12,
                    vdvc_stream_t stream) {
  VDVC_GN_DISPATCH(iterate<float>(S, freeze_now, max_iter, tol, out12, (cudaStream_t)stream),
                   iterate<double>(S, freeze_now, max_iter, tol, out12, (cudaStream_t)stream));
}

int vdvc_gn_read(vdvc_gn_solver* solver, int which, void* dst, int dst_f64, vdvc_stream_t stream) {
  VDVC_GN_DISPATCH(read<float>(S, which, dst, dst_f64, (cudaStream_t)stream),
                   read<double>(S, which, dst, dst_f64, (cudaStream_t)stream));
}

void vdvc_gn_destroy(vdvc_gn_solver* solver) {
  if (!solver || solver->borrowed) return;
  if (solver->dtype == VDVC_F32)
    destroy<float>((GnSolver<float>*)solver->impl);
  else
    destroy<double>((GnSolver<double>*)solver->impl);
  delete solver;
}

int vdvc_gn_batch_create(const vdvc_gn_desc* descs, int n, void* const* ws, const size_t* ws_bytes, int pcg_chunk,
                         int concurrent, vdvc_gn_batch** out) {
  VDVC_CHECK_ARG(descs && ws && ws_bytes && out && n >= 1 && n <= 4096, "bad arguments");
  for (int i = 0; i < n; ++i)
    VDVC_CHECK_ARG(descs[i].dtype == VDVC_F32, "batched solves are float32 (problem %d)", i);
  GnBatch* B = new (std::nothrow) GnBatch();
  if (!B) return set_error(VDVC_ERR_ARG, "host allocation failed");
  B->n = n;
  B->chunk = pcg_chunk > 0 ? pcg_chunk : 4;
  B->concurrent = concurrent ? 1 : 0;
  auto fail = [&](int code) {
    batch_destroy(B);
    return code;
  };
  for (int i = 0; i < n; ++i) {
    void* impl = nullptr;
    int st = create<float>(&descs[i], ws[i], ws_bytes[i], &impl);
    if (st) return fail(st);
    B->S.push_back((GnSolver<float>*)impl);
  }
  if (pool_stream(&B->cap) || pool_event(&B->fork_ev) ||
      cudaMalloc((void**)&B->d_states, n * sizeof(PcgState*)) != cudaSuccess)
    return fail(set_error(VDVC_ERR_CUDA, "batch stream/event/state setup failed"));
  for (int i = 0; i < n; ++i) {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    if (pool_stream(&st)) return fail(set_error(VDVC_ERR_CUDA, "batch stream setup failed"));
    B->streams.push_back(st);
    if (pool_event(&ev)) return fail(set_error(VDVC_ERR_CUDA, "batch event setup failed"));
    B->done_ev.push_back(ev);
  }
  vdvc_gn_batch* h = new (std::nothrow) vdvc_gn_batch();
  if (!h) return fail(set_error(VDVC_ERR_ARG, "host allocation failed"));
  h->impl = B;
  for (int i = 0; i < n; ++i) {
    vdvc_gn_solver* sv = new (std::nothrow) vdvc_gn_solver();
    if (!sv) {
      for (auto* q : h->handles) delete q;
      delete h;
      return fail(set_error(VDVC_ERR_ARG, "host allocation failed"));
    }
    sv->dtype = VDVC_F32;
    sv->impl = B->S[i];
    sv->borrowed = true;
    h->handles.push_back(sv);
  }
  *out = h;
  return VDVC_OK;
}

int vdvc_gn_batch_solver(vdvc_gn_batch* batch, int i, vdvc_gn_solver** out) {
  VDVC_CHECK_ARG(batch && out && i >= 0 && i < batch->impl->n, "bad arguments");
  *out = batch->handles[i];
  return VDVC_OK;
}

int vdvc_gn_batch_iterate(vdvc_gn_batch* batch, const int* active, const int* freeze_now, int max_iter, double tol,
                          double* out12, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(batch && active && out12, "bad arguments");
  return batch_iterate(batch->impl, active, freeze_now, max_iter, tol, out12, (cudaStream_t)stream);
}

int vdvc_gn_batch_set_schedule(vdvc_gn_batch* batch, int pcg_chunk, int concurrent) {
  VDVC_CHECK_ARG(batch && pcg_chunk >= 1 && pcg_chunk <= 64, "bad arguments");
  GnBatch* B = batch->impl;
  if (B->chunk != pcg_chunk || B->concurrent != (concurrent ? 1 : 0)) {
    B->chunk = pcg_chunk;
    B->concurrent = concurrent ? 1 : 0;
    batch_free_graph(B);
  }
  return VDVC_OK;
}

void vdvc_gn_batch_destroy(vdvc_gn_batch* batch) {
  if (!batch) return;
  for (auto* q : batch->handles) delete q;
  batch_destroy(batch->impl);
  delete batch;
}

}  // extern "C"
