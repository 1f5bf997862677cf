/*
 * vdvc_cnn.h -- kernels of the learned initial guess: a small BF16 3-D
 * convolutional network that predicts the displacement field on a stride-8
 * voxel grid from the (f, g) pair, with its training kernels.
 *
 * No counterpart in the reference: its multiscale solve seeds the finest
 * level from the coarse pyramid levels and an FFT shift
 * (engine/correlate_gpu.py:1143-1305); the learned seed replaces both, and
 * that solve stays its fallback.
 *
 * Activations are channels-last BF16 tensors: element (x, y, z, c) of a
 * tensor with channel stride C sits at ((z*ny + y)*nx + x)*C + c, x fastest
 * among positions.  A layer reads or writes channels [coff, coff + n) of
 * such a tensor, so a concatenation is two layers writing disjoint channel
 * ranges of one buffer.  All pointers are device pointers.
 *
 * Every convolution is 3x3x3 with a "gather" geometry: output position p
 * reads, per axis and tap t in {0,1,2}, source index
 *     q = (p*a + b + t*c) / d      (only when d divides p*a + b + t*c)
 * and contributes nothing when q falls outside [0, source extent).
 *   forward, stride s, padding 1       : a = s, b = -1, c = +1, d = 1
 *   input gradient of that convolution : a = 1, b = +1, c = -1, d = s
 * Tap t = (tz*3 + ty)*3 + tx.
 */
#ifndef VDVC_CNN_H
#define VDVC_CNN_H

#include "vdvc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vdvc_conv_geom {
  int nx, ny, nz;  /* output grid                          */
  int sx, sy, sz;  /* source grid                          */
  int a, b, c, d;  /* tap mapping, as above                */
} vdvc_conv_geom;

/* out[p][n] = act( sum_{t,k} src[q(p,t)][k] * w[n][t][k] + bias[n] ),
   on the tensor cores, BF16 x BF16 -> FP32: tcgen05.mma with the
   accumulator in TMEM when the channel chunks are 16-byte aligned (source
   channel stride and offset multiples of 8, src and w 16-byte aligned;
   n_out <= 256), else mma.sync m16n8k16 (n_out <= 80).
   cin: a multiple of 16, or 2 (then w is [n_pad][64] with k = 2t + ci and
   zero rows k >= 54; a forward stride-1 layer with n_out <= 64 on a
   contiguous 2-channel source runs on tcgen05 with its A tile built in
   shared memory from the brick's source halo, other 2-channel layers on
   mma.sync).  Otherwise w is BF16 [n_pad][27][cin].
   n_pad = n_out rounded up to 8; rows n >= n_out must be zero.
   bias: FP32 (n_out) or NULL.  relu: apply max(0, .).
   out_f32: store FP32 instead of BF16.  accumulate (BF16 output only):
   out += result (the input-gradient sum of two consumers). */
int vdvc_cnn_conv(const void* src, int src_cstride, int src_coff, int cin,
                  const void* w, const float* bias, int n_out, int relu,
                  void* out, int out_f32, int out_cstride, int out_coff,
                  int accumulate, const vdvc_conv_geom* geom,
                  vdvc_stream_t stream);

/* Synchronises the stream; VDVC_ERR_TIMEOUT (and clears the flag) when a
   tensor-core convolution launched since the last call gave up one of its
   bounded waits -- its output is then incomplete -- else VDVC_OK. */
int vdvc_cnn_status(vdvc_stream_t stream);

/* Weight gradient of a forward convolution (geom = its forward geometry):
   dw[n][t][k] (+)= sum_p dy[p][n] * x[q(p,t)][k], FP32 [n_out][27][cin],
   on the tensor cores (n_out, cin <= 256; blocks of 32 output x 64 input
   channels).  The positions are split over blocks; each block's partial
   goes to ws and a second pass sums the partials in a fixed order
   (deterministic).  accumulate: dw += instead of dw =.
   Workspace: vdvc_cnn_wgrad_workspace_bytes(n_out, cin). */
int vdvc_cnn_conv_wgrad(const void* dy, int dy_cstride, int dy_coff,
                        int n_out, const void* x, int x_cstride, int x_coff,
                        int cin, const vdvc_conv_geom* geom, float* dw,
                        int accumulate, void* ws, size_t ws_bytes,
                        vdvc_stream_t stream);
size_t vdvc_cnn_wgrad_workspace_bytes(int n_out, int cin);

/* db[n] (+)= sum over positions of dy[p][n] (deterministic).
   ws: vdvc_cnn_wgrad_workspace_bytes(n_out, 16) bytes suffice. */
int vdvc_cnn_bias_grad(const void* dy, int dy_cstride, int dy_coff,
                       int n_out, long long npos, float* db, int accumulate,
                       void* ws, size_t ws_bytes, vdvc_stream_t stream);

/* dy[i] = (y[i] > 0) ? dy[i] : 0 over n BF16 elements (ReLU backward, in
   place; dy and y share one layout). */
int vdvc_cnn_relu_bwd(void* dy, const void* y, long long n,
                      vdvc_stream_t stream);

/* Linear 2x upsampling, coarse (mx,my,mz) -> fine (nx,ny,nz): fine p reads
   coarse p/2 (p even) or the mean of (p-1)/2 and (p+1)/2 (p odd; the upper
   index clamped), per axis.  C channels from coarse channel offset ccoff
   to fine channel offset fcoff.  _bwd is its adjoint (a gather over the
   fine positions each coarse position feeds; overwrites dcoarse). */
int vdvc_cnn_upsample2(const void* coarse, int c_cstride, int ccoff, int mx,
                       int my, int mz, void* fine, int f_cstride, int fcoff,
                       int nx, int ny, int nz, int C, vdvc_stream_t stream);
int vdvc_cnn_upsample2_bwd(const void* dfine, int f_cstride, int fcoff,
                           int nx, int ny, int nz, void* dcoarse,
                           int c_cstride, int ccoff, int mx, int my, int mz,
                           int C, vdvc_stream_t stream);

/* Network input: f and g (FP32 vox layout, nx*ny*nz) low-passed with the
   separable [1 2 2 2 1]/8 filter (weights renormalised at the borders),
   sampled every 4 voxels (grid gx = (nx-1)/4 + 1, ...), standardised by
   (mean, std) of each image and written as 2 BF16 channels (cstride 2).
   mean_std: host {mean_f, std_f, mean_g, std_g}. */
int vdvc_cnn_pool_input(const float* f_vox, const float* g_vox, int nx,
                        int ny, int nz, const double* mean_std, void* out,
                        vdvc_stream_t stream);
/* The same of the pair mirrored along the axes of `flip` (bit 0 x, 1 y,
   2 z): the input of a mirrored network pass (test-time averaging). */
int vdvc_cnn_pool_input_mirrored(const float* f_vox, const float* g_vox,
                                 int nx, int ny, int nz,
                                 const double* mean_std, int flip, void* out,
                                 vdvc_stream_t stream);
/* Device-side statistics of the network input: sums[0..3] (device
   doubles) = {sum f, sum f^2, sum g, sum g^2} over the n voxels, one read of
   each image.  ws: >= 4 * 1024 * 8 + 64 bytes of device workspace. */
int vdvc_cnn_input_moments(const float* f_vox, const float* g_vox, long long n,
                           double* sums, void* ws, size_t ws_bytes,
                           vdvc_stream_t stream);
/* vdvc_cnn_pool_input_mirrored with the standardising mean and std taken
   on the device from vdvc_cnn_input_moments' sums over the nx*ny*nz
   voxels (mean = s / n, std = sqrt(s2 / n - mean^2), 1 where that is not
   positive): no host read-back between the statistics and the pooling. */
int vdvc_cnn_pool_input_dev(const float* f_vox, const float* g_vox, int nx,
                            int ny, int nz, const double* sums, int flip,
                            void* out, vdvc_stream_t stream);
/* out = the pooled input x (gx*gy*gz positions of 2 BF16 channels)
   mirrored along the axes of flip.  When (n - 1) % 4 == 0 along each
   mirrored axis (n the voxel count) the pooling grid is symmetric under the
   mirror, and this equals pooling the mirrored pair up to the FP32
   summation order of a window (an element may round to the neighbouring
   BF16 value) -- at a read of the pooled grid instead of the images. */
int vdvc_cnn_mirror_input(const void* x, int gx, int gy, int gz, int flip,
                          void* out, vdvc_stream_t stream);

/* Mean squared error of pred (FP32, channels [0,3) of stride pred_cstride)
   against target (FP32 [npos][3]); *loss (device double) = mean; dpred
   (BF16, stride dp_cstride, all channels written: 0 beyond 3) =
   scale * 2 (pred - target) / (3 npos).  ws >= 16 KiB. */
int vdvc_cnn_mse(const float* pred, int pred_cstride, const float* target,
                 long long npos, double* loss, void* dpred, int dp_cstride,
                 double scale, void* ws, size_t ws_bytes,
                 vdvc_stream_t stream);

/* Adam step on FP32 master weights (bias-corrected, step >= 1). */
int vdvc_cnn_adam(float* w, const float* grad, float* m, float* v,
                  long long n, double lr, double beta1, double beta2,
                  double eps, int step, vdvc_stream_t stream);

/* FP32 master weights [n_out][27][cin] -> the BF16 layouts of the forward
   convolution (wf: [n_pad8][27][cin], or [n_pad8][64] for cin == 2) and,
   when wb != NULL, of its input gradient (wb: [cin_pad8][27][n_pad16]:
   B[k][t][n] = W[n][t][k], zero padded). */
int vdvc_cnn_pack_weights(const float* w, int n_out, int cin, void* wf,
                          void* wb, vdvc_stream_t stream);

/* Nodal seed from the network output: U[3*node + c] = trilinear sample of
   the stride-8 FP32 field pred (channels [0,3) of stride pred_cstride, grid
   px*py*pz) at voxel position node*h, for the (Nx+1)(Ny+1)(Nz+1) mesh
   nodes; FP64 out. */
int vdvc_cnn_seed_nodes(const float* pred, int pred_cstride, int px, int py,
                        int pz, int h, int Nx, int Ny, int Nz, double* U,
                        vdvc_stream_t stream);
/* The same with U = (accumulate ? U : 0) + weight * sample, where pred is
   the output of the pass mirrored along the axes of `flip`: read at the
   mirrored positions, the mirrored components negated.  Mirroring an axis
   needs the mesh to span the output grid along it, (p - 1) * 8 = N h. */
int vdvc_cnn_seed_nodes_acc(const float* pred, int pred_cstride, int px,
                            int py, int pz, int h, int Nx, int Ny, int Nz,
                            int flip, double weight, int accumulate,
                            double* U, vdvc_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* VDVC_CNN_H */
