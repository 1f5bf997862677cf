// Known-answer (ground-truth) harness kernels (ground_truth/
// prepare_ground_truth.py, ground_truth/analyse_ground_truth.py): the
// backward warp that makes the deformed image from the reference and a known
// displacement, the per-voxel recoverability mask, and the per-node
// out-of-bounds support fraction.  Volumes are numpy pix[x, y, z] arrays in
// C order (z fastest); displacements are channels-last (x, y, z, 3).
#include "ops.cuh"

namespace vdvc {

// deformed(x) = ref(x - u(x)) with scipy's RegularGridInterpolator
// (method 'linear', fill_value None: linear extrapolation past the edges).
// Per axis the cell is i = clamp(searchsorted(grid, p) - 1, 0, n - 2) and
// the weights 1 - t, t with t = p - i; the 8 corner terms are summed in the
// interpolator's order ((lo, hi) product, last axis fastest) with the weight
// products formed left to right, all in round-to-nearest float64 without
// contraction, so the result is the interpolator's to the last bit.
__global__ void k_gt_warp(const double* __restrict__ ref, const double* __restrict__ u, int nx, int ny, int nz,
                          double* __restrict__ out) {
  const long long n = (long long)nx * ny * nz;
  const int dims[3] = {nx, ny, nz};
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(v % nz);
    const long long r = v / nz;
    const int y = (int)(r % ny), x = (int)(r / ny);
    const int pos[3] = {x, y, z};
    int lo[3];
    double w[3][2];
    for (int a = 0; a < 3; ++a) {
      const double p = __dsub_rn((double)pos[a], u[3 * v + a]);
      // searchsorted(grid, p, 'left') - 1 on the integer grid 0..n-1: the
      // largest i with i < p, i.e. ceil(p) - 1, then clipped
      const double c = ceil(p) - 1.0;
      int i = c < 0.0 ? 0 : (c > (double)(dims[a] - 2) ? dims[a] - 2 : (int)c);
      if (dims[a] < 2) i = 0;
      lo[a] = i;
      const double t = __dsub_rn(p, (double)i);
      w[a][0] = __dsub_rn(1.0, t);
      w[a][1] = t;
    }
    double acc = 0.0;
    for (int b0 = 0; b0 < 2; ++b0)
      for (int b1 = 0; b1 < 2; ++b1)
        for (int b2 = 0; b2 < 2; ++b2) {
          const int i0 = min(lo[0] + b0, nx - 1), i1 = min(lo[1] + b1, ny - 1), i2 = min(lo[2] + b2, nz - 1);
          const double wt = __dmul_rn(__dmul_rn(w[0][b0], w[1][b1]), w[2][b2]);
          acc = __dadd_rn(acc, __dmul_rn(ref[((long long)i0 * ny + i1) * nz + i2], wt));
        }
    out[v] = acc;
  }
}

// voxel_in_bounds: x + u_gt(x) inside [0, g - 1] on every axis
__global__ void k_gt_in_bounds(const double* __restrict__ u, int nx, int ny, int nz, int gx, int gy, int gz,
                               uint8_t* __restrict__ out) {
  const long long n = (long long)nx * ny * nz;
  const int g[3] = {gx, gy, gz};
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(v % nz);
    const long long r = v / nz;
    const int y = (int)(r % ny), x = (int)(r / ny);
    const int pos[3] = {x, y, z};
    bool in = true;
    for (int a = 0; a < 3; ++a) {
      const double c = __dadd_rn((double)pos[a], u[3 * v + a]);
      in = in && c >= 0.0 && c <= (double)(g[a] - 1);
    }
    out[v] = in ? 1 : 0;
  }
}

// node_oob_fraction: 1 - mean of the in-bounds mask over the node's support
// box [v - h, v + h] (clamped to the image), v = crop_lo + (i, j, k) h
__global__ void k_gt_node_oob(const uint8_t* __restrict__ inb, int nx, int ny, int nz, int h, int nbx, int nby,
                              int nbz, int l0, int l1, int l2, double* __restrict__ out) {
  const long long nn = (long long)nbx * nby * nbz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nn; q += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(q % nbz);
    const long long r = q / nbz;
    const int j = (int)(r % nby), i = (int)(r / nby);
    const int c[3] = {l0 + i * h, l1 + j * h, l2 + k * h}, d[3] = {nx, ny, nz};
    int a[3], b[3];
    for (int s = 0; s < 3; ++s) {
      a[s] = max(c[s] - h, 0);
      b[s] = min(c[s] + h, d[s] - 1);
    }
    long long cnt = 0, tot = 0;
    for (int x = a[0]; x <= b[0]; ++x)
      for (int y = a[1]; y <= b[1]; ++y) {
        const uint8_t* row = inb + ((long long)x * ny + y) * nz;
        for (int z = a[2]; z <= b[2]; ++z) cnt += row[z];
        tot += b[2] >= a[2] ? b[2] - a[2] + 1 : 0;
      }
    out[q] = 1.0 - (double)cnt / (double)tot;
  }
}

}  // namespace vdvc

using namespace vdvc;

extern "C" {

int vdvc_gt_warp(const double* ref, const double* u_vox, int nx, int ny, int nz, double* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(ref && u_vox && out && nx >= 1 && ny >= 1 && nz >= 1, "bad arguments");
  const long long n = (long long)nx * ny * nz;
  k_gt_warp<<<grid_blocks(n, 256, 152 * 32), 256, 0, (cudaStream_t)stream>>>(ref, u_vox, nx, ny, nz, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_gt_voxel_in_bounds(const double* u_vox, int nx, int ny, int nz, int gx, int gy, int gz, uint8_t* out,
                            vdvc_stream_t stream) {
  VDVC_CHECK_ARG(u_vox && out && nx >= 1 && ny >= 1 && nz >= 1 && gx >= 1 && gy >= 1 && gz >= 1, "bad arguments");
  const long long n = (long long)nx * ny * nz;
  k_gt_in_bounds<<<grid_blocks(n, 256, 152 * 32), 256, 0, (cudaStream_t)stream>>>(u_vox, nx, ny, nz, gx, gy, gz, out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

int vdvc_gt_node_oob_fraction(const uint8_t* in_bounds, int nx, int ny, int nz, int h, int nbx, int nby, int nbz,
                              const long long* crop_lo, double* out, vdvc_stream_t stream) {
  VDVC_CHECK_ARG(in_bounds && crop_lo && out && h >= 1 && nbx >= 1 && nby >= 1 && nbz >= 1, "bad arguments");
  for (int s = 0; s < 3; ++s) {
    const int d = s == 0 ? nx : (s == 1 ? ny : nz), nb = s == 0 ? nbx : (s == 1 ? nby : nbz);
    // every node's support box must meet the image (the reference's slices
    // would otherwise be empty and its mean undefined)
    VDVC_CHECK_ARG(crop_lo[s] >= 0 && crop_lo[s] + (long long)(nb - 1) * h < d,
                   "nodes outside the image on axis %d", s);
  }
  const long long nn = (long long)nbx * nby * nbz;
  k_gt_node_oob<<<grid_blocks(nn, 128, 152 * 16), 128, 0, (cudaStream_t)stream>>>(
      in_bounds, nx, ny, nz, h, nbx, nby, nbz, (int)crop_lo[0], (int)crop_lo[1], (int)crop_lo[2], out);
  VDVC_LAUNCHED();
  return VDVC_OK;
}

}  // extern "C"
