// C-ABI entry points of the correlation operator: H v, diag H, b, and the
// operator scratch-size query.
#include "ops.cuh"

namespace vdvc {

size_t operator_ws_bytes(const Mesh& m, size_t ts) {
  Carve cv(nullptr, 0);
  cv.take<char>((size_t)24 * m.Ne * ts);  // element vectors A
  cv.take<char>((size_t)24 * m.Ne * ts);  // element vectors D
  const long long nb = strip_grid_blocks(m);
  cv.take<double>((size_t)(nb > kReduceBlocks ? nb : kReduceBlocks) * 4);  // reduction partials
  cv.take<unsigned int>(4);
  return cv.off + 256;
}

template <typename T, int MODE>
int run_operator(const Mesh& m, const T* v, const T* grad, const uint8_t* mask, const T* res, T* out, void* ws,
                 size_t ws_bytes, cudaStream_t s) {
  Carve cv(ws, ws_bytes);
  T* evA = cv.take<T>((size_t)24 * m.Ne);
  T* evD = cv.take<T>((size_t)24 * m.Ne);
  if (!ws || !cv.fits())
    return set_error(VDVC_ERR_WORKSPACE, "operator needs %zu bytes of workspace (got %zu)",
                     operator_ws_bytes(m, sizeof(T)), ws_bytes);
  StripArgs<T> a{};
  a.m = m;
  a.v = v;
  a.grad = grad;
  a.mask = mask;
  a.res_in = res;
  a.evA = evA;
  a.evD = evD;
  int st = launch_strip<T, MODE>(a, nullptr, s);
  if (st) return st;
  return launch_gather<T>(m, (MODE & kModeDiag) ? evD : evA, out, s);
}

}  // namespace vdvc

using namespace vdvc;

extern "C" {

size_t vdvc_workspace_bytes(int dtype, int h, int Nx, int Ny, int Nz) {
  Mesh m;
  if (make_mesh(h, Nx, Ny, Nz, &m)) return 0;
  const size_t ts = dtype_size(dtype);
  if (ts == 0) return 0;
  const size_t a = operator_ws_bytes(m, ts);
  // equilibrium-gap temporaries and the Hutchinson accumulators (float64)
  const size_t b = (size_t)m.Ndof * 8 * 4 + (size_t)kReduceBlocks * 8 + 8 * 256;
  return a > b ? a : b;
}

int vdvc_matvec_H(const void* v, const void* grad, const uint8_t* mask, int dtype, int h, int Nx, int Ny, int Nz,
                  void* out, void* ws, size_t ws_bytes, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(h, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(v && grad && mask && out, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == VDVC_F32)
    return run_operator<float, kModeHv>(m, (const float*)v, (const float*)grad, mask, nullptr, (float*)out, ws,
                                        ws_bytes, s);
  if (dtype == VDVC_F64)
    return run_operator<double, kModeHv>(m, (const double*)v, (const double*)grad, mask, nullptr, (double*)out, ws,
                                         ws_bytes, s);
  return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
}

int vdvc_diag_H(const void* grad, const uint8_t* mask, int dtype, int h, int Nx, int Ny, int Nz, void* out, void* ws,
                size_t ws_bytes, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(h, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(grad && mask && out, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == VDVC_F32)
    return run_operator<float, kModeDiag>(m, nullptr, (const float*)grad, mask, nullptr, (float*)out, ws, ws_bytes,
                                          s);
  if (dtype == VDVC_F64)
    return run_operator<double, kModeDiag>(m, nullptr, (const double*)grad, mask, nullptr, (double*)out, ws,
                                           ws_bytes, s);
  return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
}

int vdvc_compute_b(const void* res, const uint8_t* mask, const void* grad, int dtype, int h, int Nx, int Ny, int Nz,
                   void* out, void* ws, size_t ws_bytes, vdvc_stream_t stream) {
  Mesh m;
  int st = make_mesh(h, Nx, Ny, Nz, &m);
  if (st) return st;
  VDVC_CHECK_ARG(res && grad && mask && out, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == VDVC_F32)
    return run_operator<float, kModeB>(m, nullptr, (const float*)grad, mask, (const float*)res, (float*)out, ws,
                                       ws_bytes, s);
  if (dtype == VDVC_F64)
    return run_operator<double, kModeB>(m, nullptr, (const double*)grad, mask, (const double*)res, (double*)out, ws,
                                        ws_bytes, s);
  return set_error(VDVC_ERR_ARG, "dtype %d", dtype);
}

}  // extern "C"
