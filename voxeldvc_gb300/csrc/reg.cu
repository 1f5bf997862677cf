// Constant-element-operator kernels (the Laplacian / elastic regularizers):
// node-centric application of K = sum_e E_e P_e^T K_ref P_e, its diagonal,
// the equilibrium-gap composition K P_i K and the Hutchinson diagonal.
//
// Node-centric form: (K v)[3n+c] = sum over the elements e containing node n
// (n is corner a of e) of E_e * sum_{b,c'} K_ref[3a+c][3b+c'] v[3 node(e,b)+c'].
// Each thread owns one node, so the result is written once, deterministically,
// with no scatter (engine/kernels_dvc.py:349-374 scatters with add.at).
#include "ops.cuh"
#include "pcg.cuh"

namespace vdvc {

template <typename T>
__global__ void __launch_bounds__(256) k_kref_apply(const StencilArgs<T> a, const Kmat Kd) {
  __shared__ T sK[576];
  if (a.st && a.st->done) return;
  for (int q = threadIdx.x; q < 576; q += blockDim.x) sK[q] = (T)Kd.k[q];
  __syncthreads();
  const Mesh& m = a.m;
  T beta = T(0);
  if (a.p_old) beta = (T)a.st->beta;
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < m.Nnodes;
       n += (long long)gridDim.x * blockDim.x) {
    const int ni = (int)(n % m.Nnx);
    const long long rr = n / m.Nnx;
    const int nj = (int)(rr % m.Nny), nk = (int)(rr / m.Nny);
    T acc[3] = {T(0), T(0), T(0)};
#pragma unroll 1
    for (int a_ = 0; a_ < 8; ++a_) {
      const int ei = ni - corner_dx(a_), ej = nj - corner_dy(a_), ek = nk - corner_dz(a_);
      if (ei < 0 || ej < 0 || ek < 0 || ei >= m.Nx || ej >= m.Ny || ek >= m.Nz) continue;
      const long long e = (long long)ei + (long long)ej * m.Nx + (long long)ek * m.Nx * m.Ny;
      const T Ee = a.E_elem ? a.E_elem[e] : (T)a.E;
      T s[3] = {T(0), T(0), T(0)};
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const long long nb = (long long)(ei + corner_dx(b)) + (long long)(ej + corner_dy(b)) * m.Nnx +
                             (long long)(ek + corner_dz(b)) * m.NnxNny;
        T vb[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          vb[c] = a.v[3 * nb + c];
          if (a.p_old) vb[c] += beta * a.p_old[3 * nb + c];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const T* Kr = sK + (3 * a_ + c) * 24 + 3 * b;
          s[c] += Kr[0] * vb[0] + Kr[1] * vb[1] + Kr[2] * vb[2];
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[c] += Ee * s[c];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T r = (T)a.scale * acc[c];
      if (a.interior) r *= a.interior[3 * n + c];
      if (a.add_to) r += a.add_to[3 * n + c];
      a.out[3 * n + c] = r;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_kref_diag(const Mesh m, const Kmat Kd,
                                                   const T* __restrict__ E_elem, double E, T* __restrict__ out) {
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < m.Nnodes;
       n += (long long)gridDim.x * blockDim.x) {
    const int ni = (int)(n % m.Nnx);
    const long long rr = n / m.Nnx;
    const int nj = (int)(rr % m.Nny), nk = (int)(rr / m.Nny);
    T acc[3] = {T(0), T(0), T(0)};
    for (int a_ = 0; a_ < 8; ++a_) {
      const int ei = ni - corner_dx(a_), ej = nj - corner_dy(a_), ek = nk - corner_dz(a_);
      if (ei < 0 || ej < 0 || ek < 0 || ei >= m.Nx || ej >= m.Ny || ek >= m.Nz) continue;
      const long long e = (long long)ei + (long long)ej * m.Nx + (long long)ek * m.Nx * m.Ny;
      const T Ee = E_elem ? E_elem[e] : (T)E;
      for (int c = 0; c < 3; ++c) acc[c] += Ee * (T)Kd.k[(3 * a_ + c) * 25];
    }
    for (int c = 0; c < 3; ++c) out[3 * n + c] = acc[c];
  }
}

// diag_acc += z .* Rz for one int8 probe (float64 throughout).
__global__ void k_probe_to_f64(const int8_t* __restrict__ z, long long n, double* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (double)z[i];
}

__global__ void k_hutch_acc(const int8_t* __restrict__ z, const double* __restrict__ Rz, long long n,
                            double* __restrict__ acc) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc[i] = acc[i] + (double)z[i] * Rz[i];
}

// diag = acc / n_probes, then clip below at 1e-12 * max|diag|: two passes,
// the first finds max|diag| with a deterministic grid reduction.
__global__ void __launch_bounds__(256) k_hutch_max(const double* __restrict__ acc, long long n, int n_probes,
                                                   GridReduce red, double* __restrict__ maxout) {
  __shared__ double s_red[8];
  double mx = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    mx = fmax(mx, fabs(acc[i] / (double)n_probes));
  // block max via negated min
  double bm = -block_min(-mx, s_red);
  double mine[1] = {bm}, out[1];
  // grid max: sum-reduction slots reused, the last block takes the max of the partials
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    red.partials[blockIdx.x] = mine[0];
    __threadfence();
    unsigned int t = atomicAdd(red.ticket, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    double g = 0.0;
    for (unsigned int b = 0; b < gridDim.x; ++b) g = fmax(g, ((volatile double*)red.partials)[b]);
    *maxout = g;
    *red.ticket = 0u;
  }
  (void)out;
}

__global__ void k_hutch_clip(const double* __restrict__ acc, long long n, int n_probes,
                             const double* __restrict__ maxv, double* __restrict__ out) {
  const double lo = 1e-12 * (*maxv);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double d = acc[i] / (double)n_probes;
    out[i] = d < lo ? lo : d;
  }
}

inline int node_blocks(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

template <typename T>
int launch_kref_apply(const StencilArgs<T>& a, const Kmat& K, cudaStream_t s) {
  k_kref_apply<T><<<node_blocks(a.m.Nnodes), 256, 0, s>>>(a, K);
  VDVC_LAUNCHED();
  return VDVC_OK;
}
template int launch_kref_apply<float>(const StencilArgs<float>&, const Kmat&, cudaStream_t);
template int launch_kref_apply<double>(const StencilArgs<double>&, const Kmat&, cudaStream_t);

template <typename T>
int launch_kref_diag(const Mesh& m, const Kmat& K, const T* E_elem, double E, T* out, cudaStream_t s) {
  k_kref_diag<T><<<node_blocks(m.Nnodes), 256, 0, s>>>(m, K, E_elem, E, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}
template int launch_kref_diag<float>(const Mesh&, const Kmat&, const float*, double, float*, cudaStream_t);
template int launch_kref_diag<double>(const Mesh&, const Kmat&, const double*, double, double*, cudaStream_t);

int load_K(const double* K_host, Kmat* K) {
  VDVC_CHECK_ARG(K_host != nullptr, "K_ref is null");
  for (int q = 0; q < 576; ++q) K->k[q] = K_host[q];
  return VDVC_OK;
}

}  // namespace vdvc

using namespace vdvc;

extern "C" {

int vdvc_matvec_K_ref(const void* v, int dtype, const double* K_ref, const void* E_elem, double E, int Nx, int Ny,
                      int Nz, void* out, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(1, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(v && out && K_ref, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  Kmat Kd;
  if ((st = load_K(K_ref, &Kd))) return st;
  if (dtype == VDVC_F32) {
    StencilArgs<float> a{};
    a.m = m; a.v = (const float*)v; a.E_elem = (const float*)E_elem; a.E = E; a.scale = 1.0; a.out = (float*)out;
    st = launch_kref_apply<float>(a, Kd, s);
  } else if (dtype == VDVC_F64) {
    StencilArgs<double> a{};
    a.m = m; a.v = (const double*)v; a.E_elem = (const double*)E_elem; a.E = E; a.scale = 1.0; a.out = (double*)out;
    st = launch_kref_apply<double>(a, Kd, s);
  } else {
    st = set_error(VDVC_ERR_ARG, "dtype %d", dtype);
  }
  return st;
}

int vdvc_diag_K_ref(int dtype, const double* K_ref, const void* E_elem, double E, int Nx, int Ny, int Nz, void* out,
                    vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(1, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(out && K_ref, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  Kmat Kd;
  if ((st = load_K(K_ref, &Kd))) return st;
  if (dtype == VDVC_F32)
    st = launch_kref_diag<float>(m, Kd, (const float*)E_elem, E, (float*)out, s);
  else if (dtype == VDVC_F64)
    st = launch_kref_diag<double>(m, Kd, (const double*)E_elem, E, (double*)out, s);
  else
    st = set_error(VDVC_ERR_ARG, "dtype %d", dtype);
  return st;
}

int vdvc_matvec_equilibrium_gap(const void* v, int dtype, const double* K_el, const void* interior,
                                const void* E_elem, double E, int Nx, int Ny, int Nz, void* out, void* ws,
                                size_t ws_bytes, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(1, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(v && out && K_el && interior, "null pointer");
  const size_t ts = dtype_size(dtype);
  Carve cv(ws, ws_bytes);
  void* tmp = cv.take<char>((size_t)m.Ndof * ts);
  if (!ws || !cv.fits())
    return set_error(VDVC_ERR_WORKSPACE, "equilibrium gap needs %zu bytes of workspace", cv.off);
  cudaStream_t s = (cudaStream_t)stream;
  Kmat Kd;
  if ((st = load_K(K_el, &Kd))) return st;
  if (dtype == VDVC_F32) {
    StencilArgs<float> a{};
    a.m = m; a.v = (const float*)v; a.E_elem = (const float*)E_elem; a.E = E; a.scale = 1.0;
    a.interior = (const float*)interior; a.out = (float*)tmp;
    if ((st = launch_kref_apply<float>(a, Kd, s))) return st;
    a.v = (const float*)tmp; a.interior = nullptr; a.out = (float*)out;
    return launch_kref_apply<float>(a, Kd, s);
  } else if (dtype == VDVC_F64) {
    StencilArgs<double> a{};
    a.m = m; a.v = (const double*)v; a.E_elem = (const double*)E_elem; a.E = E; a.scale = 1.0;
    a.interior = (const double*)interior; a.out = (double*)tmp;
    if ((st = launch_kref_apply<double>(a, Kd, s))) return st;
    a.v = (const double*)tmp; a.interior = nullptr; a.out = (double*)out;
    return launch_kref_apply<double>(a, Kd, s);
  }
  return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
}

int vdvc_diag_equilibrium_gap(const int8_t* probes, int n_probes, const double* K_el, const double* interior,
                              const double* E_elem, double E, int Nx, int Ny, int Nz, double* out, void* ws,
                              size_t ws_bytes, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(1, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(probes && K_el && interior && out && n_probes >= 1, "bad arguments");
  Carve cv(ws, ws_bytes);
  double* z = cv.take<double>(m.Ndof);
  double* w = cv.take<double>(m.Ndof);
  double* Rz = cv.take<double>(m.Ndof);
  double* acc = cv.take<double>(m.Ndof);
  double* partials = cv.take<double>(kReduceBlocks);
  double* maxv = cv.take<double>(1);
  unsigned int* ticket = cv.take<unsigned int>(1);
  if (!ws || !cv.fits())
    return set_error(VDVC_ERR_WORKSPACE, "diag_equilibrium_gap needs %zu bytes of workspace", cv.off);
  cudaStream_t s = (cudaStream_t)stream;
  Kmat Kd;
  if ((st = load_K(K_el, &Kd))) return st;
  VDVC_CUDA(cudaMemsetAsync(acc, 0, m.Ndof * sizeof(double), s));
  VDVC_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s));
  const int nb = node_blocks(m.Ndof);
  for (int p = 0; p < n_probes; ++p) {
    const int8_t* zp = probes + (size_t)p * m.Ndof;
    k_probe_to_f64<<<nb, 256, 0, s>>>(zp, m.Ndof, z);
    VDVC_LAUNCHED();
    StencilArgs<double> a{};
    a.m = m; a.v = z; a.E_elem = E_elem; a.E = E; a.scale = 1.0; a.interior = interior; a.out = w;
    if ((st = launch_kref_apply<double>(a, Kd, s))) return st;
    a.v = w; a.interior = nullptr; a.out = Rz;
    if ((st = launch_kref_apply<double>(a, Kd, s))) return st;
    k_hutch_acc<<<nb, 256, 0, s>>>(zp, Rz, m.Ndof, acc);
    VDVC_LAUNCHED();
  }
  const int rb = nb < kReduceBlocks ? nb : kReduceBlocks;
  GridReduce red{partials, ticket};
  k_hutch_max<<<rb, 256, 0, s>>>(acc, m.Ndof, n_probes, red, maxv);
  VDVC_LAUNCHED();
  k_hutch_clip<<<nb, 256, 0, s>>>(acc, m.Ndof, n_probes, maxv, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

}  // extern "C"
