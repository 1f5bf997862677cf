// Per-element (cell) output fields of `voxeldvc run` (engine/write_output.py
// :256-491): principal and equivalent strains at the element centroids, the
// material / safe cell masks and the material mask's one-cell erosion, the
// per-cell residual std and ZNCC over each element's active voxels, and the
// per-cell Gauss-Newton convergence ratio.  One thread per element, float64
// throughout (once per solve; the reference works in float64).  Element
// arrays are x-fastest, e = i + j Nx + k Nx Ny; a cell's voxels are its
// (h+1)^3 block, shared faces included, as in the reference.
#include <limits>

#include "ops.cuh"

namespace vdvc {

__device__ __forceinline__ double dnan() { return __longlong_as_double(0x7ff8000000000000ULL); }

// Eigenvalues of a symmetric 3x3 matrix by cyclic Jacobi rotations (Golub &
// Van Loan, Matrix Computations, 8.5), returned in descending order.
__device__ void sym3_eigvals_desc(double a[3][3], double ev[3]) {
  for (int sweep = 0; sweep < 12; ++sweep) {
    const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    const double scale = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2] + 2.0 * off;
    if (off <= 1e-36 * scale || off == 0.0) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        if (a[p][q] == 0.0) continue;
        const double tau = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        const double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        // A <- J^T A J with the rotation in the (p, q) plane
        for (int k = 0; k < 3; ++k) {
          const double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          const double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
      }
  }
  double e0 = a[0][0], e1 = a[1][1], e2 = a[2][2], tmp;
  if (e0 < e1) { tmp = e0; e0 = e1; e1 = tmp; }
  if (e1 < e2) { tmp = e1; e1 = e2; e2 = tmp; }
  if (e0 < e1) { tmp = e0; e0 = e1; e1 = tmp; }
  ev[0] = e0;
  ev[1] = e1;
  ev[2] = e2;
}

// principal strains at the centroid (shape-function gradients +-1/(4h)) and
// the von Mises equivalent strain sqrt(2)/3 sqrt(sum of squared differences)
__global__ void k_cell_strains(const double* __restrict__ U, int Nx, int Ny, int Nz, double h, double* __restrict__ ps,
                               double* __restrict__ eq) {
  const long long Ne = (long long)Nx * Ny * Nz;
  const int Nnx = Nx + 1, Nny = Ny + 1;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < Ne; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % Nx);
    const long long r = e / Nx;
    const int j = (int)(r % Ny), k = (int)(r / Ny);
    double g[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int a = 0; a < 8; ++a) {
      const int dx = corner_dx(a), dy = corner_dy(a), dz = corner_dz(a);
      const long long node = (long long)(i + dx) + (long long)(j + dy) * Nnx + (long long)(k + dz) * Nnx * Nny;
      const double s[3] = {dx ? 0.25 / h : -0.25 / h, dy ? 0.25 / h : -0.25 / h, dz ? 0.25 / h : -0.25 / h};
      for (int c = 0; c < 3; ++c) {
        const double u = U[3 * node + c];
        for (int d = 0; d < 3; ++d) g[c][d] += u * s[d];
      }
    }
    double eps[3][3];
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 3; ++d) eps[c][d] = 0.5 * (g[c][d] + g[d][c]);
    double ev[3];
    sym3_eigvals_desc(eps, ev);
    for (int q = 0; q < 3; ++q) ps[3 * e + q] = ev[q];
    if (eq) {
      const double a = ev[0] - ev[1], b = ev[1] - ev[2], c = ev[2] - ev[0];
      eq[e] = (sqrt(2.0) / 3.0) * sqrt(a * a + b * b + c * c);
    }
  }
}

// material mask (block mean of ref > glt), safe mask (no unsafe voxel in the
// block), residual std and ZNCC over the block's active voxels (res != 0).
// One warp per element: the lanes stride over the block's voxels (x fastest,
// coalesced), float64 sums are combined by a fixed shuffle tree; the ZNCC's
// centred second pass re-reads the block from L1.
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename TR>
__global__ void __launch_bounds__(256) k_cell_fields(const TR* __restrict__ ref, const double* __restrict__ res,
                                                     const uint8_t* __restrict__ unsafe, int h, int Nx, int Ny,
                                                     int Nz, double glt, uint8_t* __restrict__ material,
                                                     uint8_t* __restrict__ safe, double* __restrict__ rstd,
                                                     double* __restrict__ zncc) {
  const long long Ne = (long long)Nx * Ny * Nz;
  const long long Nvx = (long long)Nx * h + 1, NvxNvy = Nvx * ((long long)Ny * h + 1);
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const int q1 = h + 1, nq = q1 * q1 * q1;
  for (long long e = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); e < Ne; e += warps) {
    const int i = (int)(e % Nx);
    const long long r = e / Nx;
    const int j = (int)(r % Ny), k = (int)(r / Ny);
    const long long v0 = (long long)i * h + (long long)j * h * Nvx + (long long)k * h * NvxNvy;
    double sref = 0.0, cnt = 0.0, sr = 0.0, srr = 0.0, sf = 0.0, sg = 0.0;
    bool any_unsafe = false;
    for (int q = lane; q < nq; q += 32) {
      const int qx = q % q1, qy = (q / q1) % q1, qz = q / (q1 * q1);
      const long long v = v0 + qx + qy * Nvx + qz * NvxNvy;
      const double f = ref ? (double)ref[v] : 0.0;
      sref += f;
      if (unsafe && unsafe[v]) any_unsafe = true;
      if (res) {
        const double rv = res[v];
        if (rv != 0.0) {
          cnt += 1.0;
          sr += rv;
          srr += rv * rv;
          sf += f;
          sg += f - rv;
        }
      }
    }
    sref = warp_sum_d(sref);
    any_unsafe = __any_sync(0xffffffffu, any_unsafe);
    if (lane == 0) {
      const double nqd = (double)nq;
      if (material) material[e] = (sref / nqd) > glt ? 1 : 0;
      if (safe) safe[e] = any_unsafe ? 0 : 1;
    }
    if (!res) continue;
    cnt = warp_sum_d(cnt);
    sr = warp_sum_d(sr);
    srr = warp_sum_d(srr);
    sf = warp_sum_d(sf);
    sg = warp_sum_d(sg);
    const double dc = cnt > 1.0 ? cnt : 1.0;
    const double fm = sf / dc, gm = sg / dc;
    double num = 0.0, ff = 0.0, gg = 0.0;
    for (int q = lane; q < nq; q += 32) {
      const int qx = q % q1, qy = (q / q1) % q1, qz = q / (q1 * q1);
      const long long v = v0 + qx + qy * Nvx + qz * NvxNvy;
      const double rv = res[v];
      if (rv == 0.0) continue;
      const double f = (double)ref[v];
      const double fc = f - fm, gc = (f - rv) - gm;
      num += fc * gc;
      ff += fc * fc;
      gg += gc * gc;
    }
    num = warp_sum_d(num);
    ff = warp_sum_d(ff);
    gg = warp_sum_d(gg);
    if (lane == 0) {
      const double mr = sr / dc;
      const double var = srr / dc - mr * mr;
      rstd[e] = cnt < 8.0 ? dnan() : sqrt(var > 0.0 ? var : 0.0);
      const double den = sqrt(ff * gg);
      zncc[e] = (cnt < 8.0 || !(den > 0.0)) ? dnan() : num / den;
    }
  }
}

// one-cell erosion, 26-neighbourhood, outside the mesh counts as material
__global__ void k_cell_erode(const uint8_t* __restrict__ in, int Nx, int Ny, int Nz, uint8_t* __restrict__ out) {
  const long long Ne = (long long)Nx * Ny * Nz;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < Ne; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % Nx);
    const long long r = e / Nx;
    const int j = (int)(r % Ny), k = (int)(r / Ny);
    bool keep = in[e] != 0;
    for (int dk = -1; dk <= 1 && keep; ++dk)
      for (int dj = -1; dj <= 1 && keep; ++dj)
        for (int di = -1; di <= 1 && keep; ++di) {
          const int a = i + di, b = j + dj, c = k + dk;
          if (a < 0 || b < 0 || c < 0 || a >= Nx || b >= Ny || c >= Nz) continue;
          if (!in[(long long)a + (long long)b * Nx + (long long)c * Nx * Ny]) keep = false;
        }
    out[e] = keep ? 1 : 0;
  }
}

// ||dU|| / ||U|| over each element's 8 corner nodes (NaN where ||U|| = 0)
__global__ void k_cell_gn(const double* __restrict__ dU, const double* __restrict__ U, int Nx, int Ny, int Nz,
                          double* __restrict__ out) {
  const long long Ne = (long long)Nx * Ny * Nz;
  const int Nnx = Nx + 1, Nny = Ny + 1;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < Ne; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % Nx);
    const long long r = e / Nx;
    const int j = (int)(r % Ny), k = (int)(r / Ny);
    double nd = 0.0, nu = 0.0;
    for (int a = 0; a < 8; ++a) {
      const long long node = (long long)(i + corner_dx(a)) + (long long)(j + corner_dy(a)) * Nnx +
                             (long long)(k + corner_dz(a)) * Nnx * Nny;
      for (int c = 0; c < 3; ++c) {
        const double x = dU[3 * node + c], y = U[3 * node + c];
        nd += x * x;
        nu += y * y;
      }
    }
    const double den = sqrt(nu);
    out[e] = den > 0.0 ? sqrt(nd) / den : dnan();
  }
}

// von Mises equivalent strain of any (n, 3) principal-strain array
__global__ void k_equivalent_strain(const double* __restrict__ ps, long long n, double* __restrict__ eq) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const double a = ps[3 * e] - ps[3 * e + 1], b = ps[3 * e + 1] - ps[3 * e + 2], c = ps[3 * e + 2] - ps[3 * e];
    eq[e] = (sqrt(2.0) / 3.0) * sqrt(a * a + b * b + c * c);
  }
}

// Diagnostic masks of kernels_dvc.py:92-341.  Pass 1, per element over its
// voxel block: any inactive voxel; material (mask0) and lost (mask0 and not
// active) counts -> overlap-lost (lost / material > thr) and sparse
// (material / (h+1)^3 < min_frac) flags, fractions formed in float64.
enum : uint8_t { kInactive = 1, kLost = 2, kSparse = 4, kBoundary = 8 };

__global__ void k_elem_block_flags(const uint8_t* __restrict__ active, const uint8_t* __restrict__ mask0, int h,
                                   int Nx, int Ny, int Nz, double frac_threshold, double min_material_frac,
                                   uint8_t* __restrict__ flags) {
  const long long Ne = (long long)Nx * Ny * Nz;
  const long long Nvx = (long long)Nx * h + 1, NvxNvy = Nvx * ((long long)Ny * h + 1);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < Ne; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % Nx);
    const long long r = e / Nx;
    const int j = (int)(r % Ny), k = (int)(r / Ny);
    const long long v0 = (long long)i * h + (long long)j * h * Nvx + (long long)k * h * NvxNvy;
    int n_mat = 0, n_lost = 0;
    bool inactive = false;
    for (int qz = 0; qz <= h; ++qz)
      for (int qy = 0; qy <= h; ++qy)
        for (int qx = 0; qx <= h; ++qx) {
          const long long v = v0 + qx + qy * Nvx + qz * NvxNvy;
          const bool a = active[v] != 0;
          inactive |= !a;
          if (mask0 && mask0[v]) {
            ++n_mat;
            n_lost += a ? 0 : 1;
          }
        }
    uint8_t fl = inactive ? kInactive : 0;
    if (mask0) {
      if (n_mat > 0 && (double)n_lost / (double)n_mat > frac_threshold) fl |= kLost;
      if ((double)n_mat / ((double)(h + 1) * (h + 1) * (h + 1)) < min_material_frac) fl |= kSparse;
    }
    if (i == 0 || j == 0 || k == 0 || i == Nx - 1 || j == Ny - 1 || k == Nz - 1) fl |= kBoundary;
    flags[e] = fl;
  }
}

// Pass 2, per node over its up-to-8 elements: bit 0 = touched by an element
// with an inactive voxel, bit 1 = that or by a boundary-shell element (the
// returned unsafe node mask), bit 2 = touched by an overlap-lost element.
__global__ void k_node_flags(const uint8_t* __restrict__ ef, int Nx, int Ny, int Nz, uint8_t* __restrict__ nf) {
  const int Nnx = Nx + 1, Nny = Ny + 1;
  const long long Nn = (long long)Nnx * Nny * (Nz + 1);
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < Nn; n += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(n % Nnx);
    const long long r = n / Nnx;
    const int b = (int)(r % Nny), c = (int)(r / Nny);
    uint8_t o = 0;
    for (int dk = -1; dk <= 0; ++dk)
      for (int dj = -1; dj <= 0; ++dj)
        for (int di = -1; di <= 0; ++di) {
          const int i = a + di, j = b + dj, k = c + dk;
          if (i < 0 || j < 0 || k < 0 || i >= Nx || j >= Ny || k >= Nz) continue;
          const uint8_t f = ef[(long long)i + (long long)j * Nx + (long long)k * Nx * Ny];
          if (f & kInactive) o |= 1 | 2;
          if (f & kBoundary) o |= 2;
          if (f & kLost) o |= 4;
        }
    nf[n] = o;
  }
}

// Pass 3, per element over its 8 corner nodes: unsafe element (a corner
// touched by an inactive element, or the boundary shell) and the
// overlap-lost element mask (a corner touched by an overlap-lost element,
// or sparse, or the boundary shell).
__global__ void k_elem_node_flags(const uint8_t* __restrict__ ef, const uint8_t* __restrict__ nf, int Nx, int Ny,
                                  int Nz, uint8_t* __restrict__ elem_unsafe, uint8_t* __restrict__ overlap_lost) {
  const long long Ne = (long long)Nx * Ny * Nz;
  const int Nnx = Nx + 1, Nny = Ny + 1;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < Ne; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % Nx);
    const long long r = e / Nx;
    const int j = (int)(r % Ny), k = (int)(r / Ny);
    uint8_t any = 0;
    for (int a = 0; a < 8; ++a)
      any |= nf[(long long)(i + corner_dx(a)) + (long long)(j + corner_dy(a)) * Nnx +
                (long long)(k + corner_dz(a)) * Nnx * Nny];
    const uint8_t f = ef[e];
    const bool bnd = (f & kBoundary) != 0;
    if (elem_unsafe) elem_unsafe[e] = ((any & 1) || bnd) ? 1 : 0;
    if (overlap_lost) overlap_lost[e] = ((any & 4) || (f & kSparse) || bnd) ? 1 : 0;
  }
}

// Pass 4, per voxel over the elements whose (h+1)^3 block holds it (up to
// 2 per axis on shared faces): the unsafe voxel mask.
__global__ void k_vox_unsafe(const uint8_t* __restrict__ elem_unsafe, int h, int Nx, int Ny, int Nz,
                             uint8_t* __restrict__ out) {
  const int Nvx = Nx * h + 1, Nvy = Ny * h + 1;
  const long long Nv = (long long)Nvx * Nvy * (Nz * h + 1);
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < Nv; v += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(v % Nvx);
    const long long r = v / Nvx;
    const int y = (int)(r % Nvy), z = (int)(r / Nvy);
    const int e[3] = {x / h, y / h, z / h}, lim[3] = {Nx, Ny, Nz}, p[3] = {x, y, z};
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
      hi[d] = e[d] < lim[d] ? e[d] : lim[d] - 1;
      lo[d] = (p[d] % h == 0 && p[d] > 0) ? e[d] - 1 : hi[d];
    }
    uint8_t o = 0;
    for (int k = lo[2]; k <= hi[2] && !o; ++k)
      for (int j = lo[1]; j <= hi[1] && !o; ++j)
        for (int i = lo[0]; i <= hi[0] && !o; ++i) o = elem_unsafe[(long long)i + (long long)j * Nx + (long long)k * Nx * Ny];
    out[v] = o ? 1 : 0;
  }
}

__global__ void k_node_bit(const uint8_t* __restrict__ nf, long long n, int bit, uint8_t* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (nf[i] & bit) ? 1 : 0;
}

inline int cblocks(long long n) { return grid_blocks(n, 128, 152 * 32); }

}  // namespace vdvc

using namespace vdvc;

extern "C" {

int vdvc_cell_strains(const double* U, int h, int Nx, int Ny, int Nz, double* principal, double* equivalent,
                      vdvc_stream_t stream) {
  VDVC_CHECK_ARG(U && principal && h >= 1 && Nx >= 1 && Ny >= 1 && Nz >= 1, "bad arguments");
  const long long Ne = (long long)Nx * Ny * Nz;
  k_cell_strains<<<cblocks(Ne), 128, 0, (cudaStream_t)stream>>>(U, Nx, Ny, Nz, (double)h, principal, equivalent);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cell_fields(const void* ref, int ref_dtype, const double* res, const uint8_t* unsafe, int h, int Nx, int Ny,
                     int Nz, double glt, uint8_t* material, uint8_t* safe, double* residual_std, double* zncc,
                     vdvc_stream_t stream) {
  VDVC_CHECK_ARG(h >= 1 && Nx >= 1 && Ny >= 1 && Nz >= 1, "bad arguments");
  VDVC_CHECK_ARG(ref || (!material && !res), "material and res need ref");
  VDVC_CHECK_ARG(!res || (residual_std && zncc), "res needs residual_std and zncc outputs");
  VDVC_CHECK_ARG(!safe || unsafe, "safe needs the unsafe voxel mask");
  const long long Ne = (long long)Nx * Ny * Nz;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = grid_blocks(Ne, 8, 152 * 16);  // 8 elements (warps) per block
  if (ref_dtype == VDVC_F32)
    k_cell_fields<float><<<nb, 256, 0, s>>>((const float*)ref, res, unsafe, h, Nx, Ny, Nz, glt, material, safe,
                                            residual_std, zncc);
  else if (ref_dtype == VDVC_F64)
    k_cell_fields<double><<<nb, 256, 0, s>>>((const double*)ref, res, unsafe, h, Nx, Ny, Nz, glt, material, safe,
                                             residual_std, zncc);
  else
    return set_error(VDVC_ERR_ARG, "ref dtype %d", ref_dtype);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cell_erode(const uint8_t* in, int Nx, int Ny, int Nz, uint8_t* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(in && out && in != out && Nx >= 1 && Ny >= 1 && Nz >= 1, "bad arguments");
  const long long Ne = (long long)Nx * Ny * Nz;
  k_cell_erode<<<cblocks(Ne), 128, 0, (cudaStream_t)stream>>>(in, Nx, Ny, Nz, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_cell_gn_convergence(const double* dU, const double* U, int Nx, int Ny, int Nz, double* out,
                             vdvc_stream_t stream) {
  VDVC_CHECK_ARG(dU && U && out && Nx >= 1 && Ny >= 1 && Nz >= 1, "bad arguments");
  const long long Ne = (long long)Nx * Ny * Nz;
  k_cell_gn<<<cblocks(Ne), 128, 0, (cudaStream_t)stream>>>(dU, U, Nx, Ny, Nz, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_equivalent_strain(const double* principal, long long n, double* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(principal && out && n >= 0, "bad arguments");
  if (n == 0) return VDVC_OK;
  k_equivalent_strain<<<cblocks(n), 128, 0, (cudaStream_t)stream>>>(principal, n, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

size_t vdvc_unsafe_masks_workspace_bytes(int Nx, int Ny, int Nz) {
  const size_t Ne = (size_t)Nx * Ny * Nz, Nn = (size_t)(Nx + 1) * (Ny + 1) * (Nz + 1);
  return ((Ne + 255) & ~(size_t)255) + ((Nn + 255) & ~(size_t)255) + ((Ne + 255) & ~(size_t)255);
}

int vdvc_unsafe_masks(const uint8_t* active, const uint8_t* mask0, int h, int Nx, int Ny, int Nz,
                      double frac_threshold, double min_material_frac, uint8_t* unsafe_vox, uint8_t* unsafe_elem,
                      uint8_t* unsafe_node, uint8_t* overlap_lost, void* ws, size_t ws_bytes, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(active && h >= 1 && Nx >= 1 && Ny >= 1 && Nz >= 1, "bad arguments");
  VDVC_CHECK_ARG(!overlap_lost || mask0, "the overlap-lost mask needs mask0");
  const size_t need = vdvc_unsafe_masks_workspace_bytes(Nx, Ny, Nz);
  if (!ws || ws_bytes < need) return set_error(VDVC_ERR_WORKSPACE, "unsafe masks need %zu bytes", need);
  const long long Ne = (long long)Nx * Ny * Nz, Nn = (long long)(Nx + 1) * (Ny + 1) * (Nz + 1);
  uint8_t* ef = (uint8_t*)ws;
  uint8_t* nf = ef + ((Ne + 255) & ~255LL);
  uint8_t* eu = unsafe_elem ? unsafe_elem : nf + ((Nn + 255) & ~255LL);
  cudaStream_t s = (cudaStream_t)stream;
  k_elem_block_flags<<<cblocks(Ne), 128, 0, s>>>(active, mask0, h, Nx, Ny, Nz, frac_threshold, min_material_frac,
                                                 ef);
  k_node_flags<<<cblocks(Nn), 128, 0, s>>>(ef, Nx, Ny, Nz, nf);
  k_elem_node_flags<<<cblocks(Ne), 128, 0, s>>>(ef, nf, Nx, Ny, Nz, eu, overlap_lost);
  count_launch(3);
  if (unsafe_node) {
    // bit 1 of the node flags is the returned node mask
    k_node_bit<<<cblocks(Nn), 128, 0, s>>>(nf, Nn, 2, unsafe_node);
    count_launch(1);
  }
  if (unsafe_vox) {
    const long long Nv = ((long long)Nx * h + 1) * ((long long)Ny * h + 1) * ((long long)Nz * h + 1);
    k_vox_unsafe<<<cblocks(Nv), 128, 0, s>>>(eu, h, Nx, Ny, Nz, unsafe_vox);
    count_launch(1);
  }
  VDVC_CUDA(cudaGetLastError());
  return VDVC_OK;
}

}  // extern "C"
