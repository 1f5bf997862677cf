/*
 * vdvc_synth.h -- seeded synthetic DVC workloads generated on the GPU.
 *
 * No counterpart in the reference (it ships no benchmark data); these build
 * the texture + warp pairs the benchmark and the large-size tests run on:
 * fiber-composite-like textures (Gaussian-filtered white noise plus bright
 * randomly oriented cylinders, normalised to [0,1]) and deformed images
 * g(x) = f(x - u(x)) + noise for analytic displacement fields u.
 * All arrays are vox layout (x fastest), float32, device pointers.
 */
#ifndef VDVC_SYNTH_H
#define VDVC_SYNTH_H

#include "vdvc.h"

#ifdef __cplusplus
extern "C" {
#endif

/* displacement fields of vdvc_synth_warp */
enum {
  VDVC_FIELD_AFFINE = 0,   /* u = t + G (x - c); params: t[3], G[9] row-major, c[3]            */
  VDVC_FIELD_NECKING = 1,  /* u_z = ez*z; radial contraction a*exp(-(z-zc)^2/(2 s^2)) r/R;
                              params: ez, a, zc, s, xc, yc, R                                  */
  VDVC_FIELD_AFFINE_SIN = 2, /* affine as above plus amp*sin(2 pi x_k / wl) on each component;
                              params: t[3], G[9], c[3], amp, wl                               */
  VDVC_FIELD_BUMPS = 3      /* affine as above plus n_b <= 6 Gaussian bumps
                              A_b exp(-|x - c_b|^2 / (2 w_b^2)); params: t[3], G[9], c[3],
                              n_b, then per bump c_b[3], w_b, A_b[3] (at most 64 params)     */
};

/* Bytes of scratch vdvc_synth_texture needs (one float volume + reductions). */
size_t vdvc_synth_workspace_bytes(int nx, int ny, int nz);

/* out = normalise01( 0.5 + noise_amp * blur_sigma(white noise)/std
                      max  cyl_value * smoothstep(cylinder interiors) )
   cylinders: n_cyl rows of 8 floats (cx, cy, cz, dx, dy, dz, radius,
   half_length) in voxel units, |d| = 1, device pointer. */
int vdvc_synth_texture(float* out, int nx, int ny, int nz,
                       unsigned long long seed, double sigma,
                       double noise_amp, const float* cylinders, int n_cyl,
                       double cyl_value, void* ws, size_t ws_bytes,
                       vdvc_stream_t stream);

/* u(x) at the grid points x = (i, j, k) * stride, FP32 (gx*gy*gz, 3),
   x fastest: training targets of the learned initial guess. */
int vdvc_synth_field_grid(int field, const double* params, int n_params,
                          int gx, int gy, int gz, double stride, float* out,
                          vdvc_stream_t stream);

/* g(x) = f(x - u(x)) (trilinear, clamped) + N(0, noise_sigma^2). */
int vdvc_synth_warp(const float* f, int nx, int ny, int nz, int field,
                    const double* params, int n_params, double noise_sigma,
                    unsigned long long seed, float* g, vdvc_stream_t stream);

/* Free-form deformation (the learned seed's training fields): the affine
   field of VDVC_FIELD_AFFINE (affine = t[3], G[9] row-major, c[3]) plus a
   uniform cubic B-spline displacement on an nc^3 control grid spanning the
   volume (spacing (n - 1) / (nc - 3) per axis; the 4^3 control points of
   the cell around x weigh in), control displacements ctrl: device FP32
   [nc^3][3], first index fastest.  Evaluated in FP32.
   vdvc_synth_warp_ffd: g(x) = f(x - u(x)) (trilinear, clamped) + noise.
   vdvc_synth_ffd_inverse_grid: U with U = u(X + U) -- the displacement a
   correlation of f against that g recovers -- at X = (i, j, k) * stride,
   `iters` fixed-point steps, FP32 (gx*gy*gz, 3), x fastest. */
int vdvc_synth_warp_ffd(const float* f, int nx, int ny, int nz,
                        const double* affine, const float* ctrl, int nc,
                        double noise_sigma, unsigned long long seed,
                        float* g, vdvc_stream_t stream);
int vdvc_synth_ffd_inverse_grid(const double* affine, const float* ctrl,
                                int nc, int nx, int ny, int nz, int gx,
                                int gy, int gz, double stride, int iters,
                                float* out, vdvc_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* VDVC_SYNTH_H */
