/*
 * vdvc.h -- C ABI of the GB300 (sm_103a) voxelDVC global Gauss-Newton path.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream,
 * enqueues its kernels on that stream and returns an int status
 * (VDVC_OK == 0).  Nothing here takes ownership of a pointer.  Outputs are
 * caller-allocated; scratch memory is passed in as (ws, ws_bytes) and its
 * required size is given by the matching *_workspace_bytes() query.
 *
 * Layouts (identical to the reference's xp arrays):
 *   voxel fields  : flat, x fastest, vidx = vx + vy*Nvx + vz*Nvx*Nvy,
 *                   Nv? = N?*h + 1 ("vox" layout = F-order ravel of pix[x,y,z])
 *   grad          : (Nvox, 3) interleaved, component fastest
 *   masks         : (Nvox) uint8, 0/1
 *   dof vectors   : (Ndof) with dof = 3*node + c, node = i + j*(Nx+1) + k*(Nx+1)*(Ny+1)
 *   element index : e = i + j*Nx + k*Nx*Ny
 *   images (pix)  : C-order (nx, ny, nz) arrays, z fastest, as numpy holds pix[x,y,z]
 *
 * `dtype` arguments select the floating type of every floating array of
 * the call: VDVC_F32 or VDVC_F64.
 *
 * Citations name the reference function each entry point replaces
 * (paths inside the voxelDVC project, src/voxeldvc/...).
 */
#ifndef VDVC_H
#define VDVC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* vdvc_stream_t; /* == cudaStream_t */

/* ---- status codes --------------------------------------------------- */
enum {
  VDVC_OK = 0,
  VDVC_ERR_ARG = 1,          /* invalid argument (size, pointer, dtype)          */
  VDVC_ERR_INDEX_RANGE = 2,  /* Nvox or Ndof beyond int32 (correlate_gpu.py:933) */
  VDVC_ERR_CUDA = 3,         /* CUDA runtime / launch error                      */
  VDVC_ERR_WORKSPACE = 4,    /* ws_bytes smaller than the query returned         */
  VDVC_ERR_NONFINITE = 5,    /* NaN/Inf met where a finite value is required     */
  VDVC_ERR_ZERO_DIVISION = 6,/* a normalisation std of zero (the reference raises
                                ZeroDivisionError at correlate_gpu.py:1095)      */
  VDVC_ERR_CUFFT = 7,        /* cuFFT plan/exec failure                          */
  VDVC_ERR_UNSUPPORTED = 8,  /* valid request this build does not implement      */
  VDVC_ERR_TIMEOUT = 9       /* a bounded device-side wait (mbarrier) ran
                                out; the kernel returned without finishing
                                and the context stays usable                */
};

/* element types for dtype / pix_dtype arguments */
enum {
  VDVC_F32 = 0,
  VDVC_F64 = 1,
  VDVC_U8 = 2,
  VDVC_U16 = 3,
  VDVC_I16 = 4,
  VDVC_I32 = 5
};

/* regularizer kinds (correlate_gpu.py:966-967, reg_type) */
enum {
  VDVC_REG_NONE = 0,
  VDVC_REG_LAPLACIAN = 1,
  VDVC_REG_EQUILIBRIUM_GAP = 2
};

/* ---- library info ---------------------------------------------------- */
int vdvc_abi_version(void);
const char* vdvc_status_string(int status);
/* Detail of the last non-OK status raised on the calling host thread. */
const char* vdvc_last_error(void);
/* Number of kernels this library has enqueued since load (graph nodes
   count once per replay). */
long long vdvc_launch_count(void);
/* 1 when kernels on `device` read ordinary (pageable, not registered) host
   memory in place through the host's page tables --
   cudaDevAttrPageableMemoryAccess and ...UsesHostPageTables, e.g. a Grace
   host over NVLink-C2C -- else 0.  Where it is 1,
   vdvc_pix_to_vox accepts a host pointer as `pix` (the transpose then reads
   the host array itself instead of a staged device copy). */
int vdvc_device_reads_pageable(int device);

/* ---- scratch size query -------------------------------------------- */
/* Bytes of scratch that any single operator call below needs for this mesh
   (element vectors + reduction partials).  Solver calls have their own
   queries further down. */
size_t vdvc_workspace_bytes(int dtype, int h, int Nx, int Ny, int Nz);

/* ---- image layout ---------------------------------------------------- */
/* pix (C-order nx*ny*nz of pix_dtype) -> vox (x fastest, dtype), with the
   cast.  Replaces xp.asarray(pix, dtype) + xp.ravel(order='F')
   (engine/correlate_gpu.py:59-60, :938-939). */
int vdvc_pix_to_vox(const void* pix, int pix_dtype, int nx, int ny, int nz,
                    void* vox, int dtype, vdvc_stream_t stream);
/* The same on every step-th voxel per axis: vox = the vox layout of
   pix[::step, ::step, ::step] (ceil(n / step) per axis), reading only those
   voxels: a pyramid level straight from the source image, as the reference
   takes it (xp.asarray(f_pix)[::s, ::s, ::s], engine/correlate_gpu.py:
   1257-1258).  max_blocks > 0 bounds the grid (blocks then walk the tiles):
   a copy from host memory run in the background of other kernels keeps its
   blocks, which mostly wait on the host link, off most of the SMs. */
int vdvc_pix_to_vox_strided(const void* pix, int pix_dtype, int nx, int ny,
                            int nz, int step, int max_blocks, void* vox,
                            int dtype, vdvc_stream_t stream);

/* Strided decimation in vox layout: out = in[::s, ::s, ::s]
   (engine/correlate_gpu.py:1257-1258).  out has ceil(n/s) per axis. */
int vdvc_decimate(const void* in, int dtype, int nx, int ny, int nz, int s,
                  void* out, vdvc_stream_t stream);

/* ---- reference-image preparation ------------------------------------ */
/* grad = per-axis xp.gradient (central differences, one-sided first order at
   the borders) of the vox field f (engine/correlate_gpu.py:49-72).  When
   mask0 != NULL also: mask0 = f > glt (:951) and grad zeroed where the
   6-neighbour erosion (mode 'nearest') of mask0 is false (:952-953,
   erode_mask0_vox :75-94). */
int vdvc_image_grad(const void* f_vox, int dtype, int Nvx, int Nvy, int Nvz,
                    double glt, void* grad, uint8_t* mask0,
                    vdvc_stream_t stream);

/* vdvc_image_grad (float32, with mask0) and, from the same read of f, the
   sums of vdvc_masked_stats over mask0 for the mesh (h, Nx, Ny, Nz) whose
   voxel grid f is: out3 (device) = count, sum f, sum f^2 -- the level
   set-up's reference statistics (engine/correlate_gpu.py:951-962).
   ws: >= 3 * 8192 * 8 + 512 bytes. */
int vdvc_image_grad_stats(const float* f_vox, int Nvx, int Nvy, int Nvz,
                          double glt, float* grad, uint8_t* mask0, int h,
                          int Nx, int Ny, int Nz, double* out3, void* ws,
                          size_t ws_bytes, vdvc_stream_t stream);

/* 6-neighbour minimum filter, mode 'nearest' (erode_mask0_vox,
   engine/correlate_gpu.py:75-94). */
int vdvc_erode_mask(const uint8_t* mask, int Nvx, int Nvy, int Nvz,
                    uint8_t* out, vdvc_stream_t stream);

/* ---- statistics ------------------------------------------------------ */
/* Multiplicity-weighted masked sums over the (element, stencil point)
   array: out3[0] = count, out3[1] = sum x, out3[2] = sum x^2 (float64, on
   the device).  masked_quadpoint_mean_std, engine/correlate_gpu.py:113-157. */
int vdvc_masked_stats(const void* field, int dtype, const uint8_t* mask,
                      int h, int Nx, int Ny, int Nz, double* out3,
                      void* ws, size_t ws_bytes, vdvc_stream_t stream);

/* ---- operators (engine/kernels_dvc.py) -------------------------------- */
/* out = H v, matrix-free correlation Hessian (matvec_H, kernels_dvc.py:452-506). */
int vdvc_matvec_H(const void* v, const void* grad, const uint8_t* mask,
                  int dtype, int h, int Nx, int Ny, int Nz, void* out,
                  void* ws, size_t ws_bytes, vdvc_stream_t stream);

/* out = H v in float32 for callers that cannot allocate device memory (a
   plugin whose host owns all device memory through its own pool, a
   latency-critical loop where cudaMalloc is not allowed).  No counterpart
   in the reference.  Same result as vdvc_matvec_H; the element-vector
   scratch is a fixed 32 MiB file-scope device array (meshes of at most
   vdvc_matvec_H_noalloc_max_elements() elements, larger ones are rejected
   with VDVC_ERR_ARG), held by every GPU that loads the library until exit.
   The first call on a device looks the array's address up
   (cudaGetSymbolAddress) and should come before any stream capture.  All
   calls share the array: calls whose kernels overlap on the GPU race. */
int vdvc_matvec_H_noalloc(const float* v, const float* grad,
                          const uint8_t* mask, int h, int Nx, int Ny, int Nz,
                          float* out, vdvc_stream_t stream);
size_t vdvc_matvec_H_noalloc_max_elements(void);

/* ---- failure detection -------------------------------------------------- */
/* Runs the library's bounded device-side wait -- the mbarrier wait of the
   bulk-copy and tensor-core pipelines (element-Hessian matvec and formation,
   tensor-core convolutions) -- and reports it the way those kernels do.
   which = 0: on a barrier nothing arrives at, so the wait gives up after
   max_polls polls (1 .. 2^24) and the call returns VDVC_ERR_TIMEOUT; 1: the
   same wait released normally, VDVC_OK.  The kernel always returns and the
   CUDA context stays usable; nothing faults or hangs.  Synchronises the
   stream.  No counterpart in the reference (which has no device-side
   waits). */
int vdvc_selftest_bounded_wait(int which, long long max_polls, vdvc_stream_t stream);

/* Precision form of matvec_H (kernels_dvc.py:452-506): the gradient is
   rounded to BF16, the 162 distinct entries of every 24x24 element Hessian
   are formed with FP32 accumulation, and out = H v is applied from them in
   FP32.  float32 v/grad/out; h in {1,2,3,4,6,8,12,16}.  The Gauss-Newton
   solver forms the element Hessians once per iteration and reuses them for
   every PCG step; this entry forms them on each call.  Workspace:
   vdvc_eh_workspace_bytes(h, Nx, Ny, Nz). */
int vdvc_matvec_H_mixed(const float* v, const float* grad,
                        const uint8_t* mask, int h, int Nx, int Ny, int Nz,
                        float* out, void* ws, size_t ws_bytes,
                        vdvc_stream_t stream);
size_t vdvc_eh_workspace_bytes(int h, int Nx, int Ny, int Nz);

/* The Hessian of matvec_H (kernels_dvc.py:452-506) as element Hessians,
   formed once and applied many times -- the operator the GN solver's PCG
   uses at element edges >= 6.  T holds the 162 distinct entries of every
   element's 24x24 block (FP32 accumulation), tile-major, vdvc_eh_bytes()
   bytes, 16-byte aligned.  vdvc_eh_form builds T from the float32 gradient
   (grad_bf16 = 0: the matrix-free pass's float32 products summed in another
   order) or from its BF16 rounding (grad_bf16 = 1: grad then points to
   (Nvox,3) BF16 values).  vdvc_eh_apply: out = H v from T.  Both take a
   workspace of vdvc_eh_op_workspace_bytes() bytes, zero-filled before its
   first use; its status word records a timed-out bulk-copy wait, which
   vdvc_eh_status reports (VDVC_ERR_TIMEOUT) and clears.  h in
   {1,2,3,4,6,8,12,16}. */
size_t vdvc_eh_bytes(int h, int Nx, int Ny, int Nz);
size_t vdvc_eh_op_workspace_bytes(int h, int Nx, int Ny, int Nz);
int vdvc_eh_form(const float* grad, int grad_bf16, const uint8_t* mask,
                 int h, int Nx, int Ny, int Nz, float* T, void* ws,
                 size_t ws_bytes, vdvc_stream_t stream);
int vdvc_eh_apply(const float* T, const float* v, int h, int Nx, int Ny,
                  int Nz, float* out, void* ws, size_t ws_bytes,
                  vdvc_stream_t stream);
int vdvc_eh_status(void* ws, size_t ws_bytes, int h, int Nx, int Ny, int Nz,
                   vdvc_stream_t stream);

/* out = diag(H) (build_diagonal_H, kernels_dvc.py:509-543). */
int vdvc_diag_H(const void* grad, const uint8_t* mask, int dtype, int h,
                int Nx, int Ny, int Nz, void* out, void* ws, size_t ws_bytes,
                vdvc_stream_t stream);

/* out = sum_e P_e^T sum_q w m res N (x) grad (compute_b_gpu,
   engine/correlate_gpu.py:341-378). */
int vdvc_compute_b(const void* res, const uint8_t* mask, const void* grad,
                   int dtype, int h, int Nx, int Ny, int Nz, void* out,
                   void* ws, size_t ws_bytes, vdvc_stream_t stream);

/* out = sum_e E_e P_e^T K_ref P_e v (matvec_K_ref, kernels_dvc.py:349-374).
   K_ref: host 24x24 row-major float64.  E_elem: device (Ne) array of dtype,
   or NULL to use the scalar E. */
int vdvc_matvec_K_ref(const void* v, int dtype, const double* K_ref,
                      const void* E_elem, double E, int Nx, int Ny, int Nz,
                      void* out, vdvc_stream_t stream);

/* out = diag of the operator above (build_diagonal_K_ref, kernels_dvc.py:377-392). */
int vdvc_diag_K_ref(int dtype, const double* K_ref, const void* E_elem,
                    double E, int Nx, int Ny, int Nz, void* out,
                    vdvc_stream_t stream);

/* out = K (P_i (K v)), K = sum_e E_e P_e^T K_el P_e
   (matvec_equilibrium_gap, kernels_dvc.py:402-417).  interior: device
   (Ndof) array of dtype (the P_i diagonal). */
int vdvc_matvec_equilibrium_gap(const void* v, int dtype, const double* K_el,
                                const void* interior, const void* E_elem,
                                double E, int Nx, int Ny, int Nz, void* out,
                                void* ws, size_t ws_bytes,
                                vdvc_stream_t stream);

/* Hutchinson estimate of diag(K P_i K) in float64 from n_probes Rademacher
   probes given as int8 (+1/-1), probe-major (n_probes x Ndof), then the
   clip at 1e-12*max|diag| (build_diagonal_equilibrium_gap,
   kernels_dvc.py:420-437). */
int vdvc_diag_equilibrium_gap(const int8_t* probes, int n_probes,
                              const double* K_el, const double* interior,
                              const double* E_elem, double E, int Nx, int Ny,
                              int Nz, double* out, void* ws, size_t ws_bytes,
                              vdvc_stream_t stream);

/* g(x + u(x)) at every voxel and the active mask in_bounds & mask0 & g>glt
   (sample_deformed_field, engine/correlate_gpu.py:201-281).  U: (Ndof) of
   dtype; g_vox: (gnx*gny*gnz) vox layout of dtype; mask0 may be NULL (all
   ones).  Voxels shared by elements take the highest element's u. */
int vdvc_sample_deformed(const void* U, const void* g_vox, int dtype,
                         int gnx, int gny, int gnz, double gx0, double gy0,
                         double gz0, const uint8_t* mask0, double glt, int h,
                         int Nx, int Ny, int Nz, void* g_vals,
                         uint8_t* mask_out, vdvc_stream_t stream);

/* u(x) at every voxel centre, (Nvox,3) or channels-first (3,Nvox)
   (interp_field_vox, engine/correlate_gpu.py:160-198). */
int vdvc_interp_field(const void* U, int dtype, int h, int Nx, int Ny,
                      int Nz, int channels_first, void* out,
                      vdvc_stream_t stream);

/* ---- post-solve voxel stages (engine/write_output.py) ------------------- */
/* sampling modes of vdvc_push_field (scipy.ndimage.map_coordinates) */
enum { VDVC_MODE_NEAREST = 0, VDVC_MODE_CONSTANT = 1 };

/* out(x) = field(x - u(x)) on the voxel grid (push_field_forward,
   engine/write_output.py:571-608): field and out in vox layout
   (nx*ny*nz) of dtype (VDVC_F32, VDVC_F64 or VDVC_U8 for label fields);
   u_cf: the displacement at every voxel, float64 channels-first (3, nvox)
   as vdvc_interp_field writes it; order 0 (nearest, ties upward) or 1
   (trilinear); mode NEAREST clamps to [0, n-1], CONSTANT writes cval where
   any coordinate is outside [0, n-1].  Coordinates in float64. */
int vdvc_push_field(const void* field, int dtype, const double* u_cf, int nx,
                    int ny, int nz, int order, int mode, double cval,
                    void* out, vdvc_stream_t stream);

/* float64 -> dtype (VDVC_F32, VDVC_U8, VDVC_U16, VDVC_I16, VDVC_I32) with
   scipy.ndimage's output conversion for integer fields: round half away from
   zero, saturate (the integer-field case of push_field_forward). */
int vdvc_cast_round(const double* in, long long n, int dtype, void* out,
                    vdvc_stream_t stream);
/* *out_host = zero-normalised cross-correlation of f and g over mask
   (compute_zncc, engine/write_output.py:658-690): float64 sums in two
   passes (means, then centred products); NaN for an empty mask or a zero
   denominator.  ws >= 32 KiB.  Synchronises the stream. */
int vdvc_zncc(const void* f, const void* g, int dtype, const uint8_t* mask,
              long long n, double* out_host, void* ws, size_t ws_bytes,
              vdvc_stream_t stream);

/* ---- preprocess glue (preprocess.py) ----------------------------------- */
/* out[i,j,k] (C order, nx*ny*nz) = g sampled at A (x - c) + c + t, x =
   (i,j,k), coordinates in float32 as the reference forms them, order-1
   interpolation, 0 outside [0, n-1] (warp_onto_ref_grid,
   preprocess.py:233-285).  g: C-order float32 (gx, gy, gz); A: host 3x3
   row-major; t, c: host 3-vectors. */
int vdvc_warp_affine(const float* g, int gx, int gy, int gz, const double* A,
                     const double* t, const double* c, int nx, int ny,
                     int nz, float* out, vdvc_stream_t stream);

/* float32 mean over B^3 blocks of a C-order volume of dtype (F32, U8, U16,
   I16), summed in the reference's order (bin_volume,
   preprocess.py:288-312); the shape must be divisible by B. */
int vdvc_bin_volume(const void* vol, int dtype, int s0, int s1, int s2, int B,
                    float* out, vdvc_stream_t stream);

/* Axis projections of the valid overlap (f > glt) & (g > glt) of two C-order
   float32 volumes (n0, n1, n2): p_a[i] = 1 where some voxel with index i on
   axis a is valid (compute_crop's bounding-box search,
   preprocess.py:315-367). */
int vdvc_overlap_projections(const float* f, const float* g, int n0, int n1,
                             int n2, double glt, uint8_t* p0, uint8_t* p1,
                             uint8_t* p2, vdvc_stream_t stream);

/* ---- per-element (cell) output fields ------------------------------------
   The element-scale stages of `voxeldvc run`'s outputs
   (engine/write_output.py:256-491, engine/kernels_dvc.py:92-341).  Element
   arrays are x-fastest (e = i + j Nx + k Nx Ny), voxel arrays x-fastest over
   (Nx h + 1, Ny h + 1, Nz h + 1), node vectors node-major with the component
   fastest (U[3 node + c]); an element's voxels are its (h+1)^3 block,
   shared faces included.  All float64 unless stated. */

/* Principal strains e1 >= e2 >= e3 (principal: Ne x 3) of the small-strain
   tensor at each element centroid from the Hex8 shape-function gradients
   scaled by 1/h (compute_principal_strains_cell, write_output.py:256-281);
   equivalent (may be NULL): the von Mises equivalent strain
   sqrt(2)/3 sqrt((e1-e2)^2 + (e2-e3)^2 + (e3-e1)^2)
   (compute_equivalent_strain, :284-310). */
int vdvc_cell_strains(const double* U, int h, int Nx, int Ny, int Nz,
                      double* principal, double* equivalent,
                      vdvc_stream_t stream);
/* compute_equivalent_strain of any (n, 3) principal-strain array. */
int vdvc_equivalent_strain(const double* principal, long long n, double* out,
                           vdvc_stream_t stream);

/* Block reductions per element over its voxels (NULL outputs are skipped):
     material      block mean of ref > glt (compute_material_cell_mask,
                   :313-338); ref VDVC_F32 or VDVC_F64
     safe          no voxel of the block flagged in unsafe (uint8)
                   (compute_safe_cell_mask, :358-381)
     residual_std, zncc   over the block's active voxels (res != 0): the
                   population std of res and the ZNCC of ref and ref - res,
                   NaN below 8 active voxels or for a zero denominator
                   (compute_correlation_quality_cell, :384-452); both are
                   written when res != NULL. */
int vdvc_cell_fields(const void* ref, int ref_dtype, const double* res,
                     const uint8_t* unsafe, int h, int Nx, int Ny, int Nz,
                     double glt, uint8_t* material, uint8_t* safe,
                     double* residual_std, double* zncc,
                     vdvc_stream_t stream);
/* One-cell erosion with the 26-neighbourhood, the mesh border counting as
   material (compute_material_cell_mask_eroded, :341-355).  in != out. */
int vdvc_cell_erode(const uint8_t* in, int Nx, int Ny, int Nz, uint8_t* out,
                    vdvc_stream_t stream);
/* ||dU|| / ||U|| over each element's 24 corner DOFs, NaN where ||U|| = 0
   (compute_gn_convergence_cell, :455-491). */
int vdvc_cell_gn_convergence(const double* dU, const double* U, int Nx,
                             int Ny, int Nz, double* out,
                             vdvc_stream_t stream);

/* Diagnostic masks of kernels_dvc.py:92-341 from the active voxel mask
   (uint8) and, for the overlap-lost mask, the material mask mask0 (uint8;
   may be NULL otherwise).  Outputs (uint8, NULL to skip):
     unsafe_vox   (Nvox)  compute_unsafe_voxel_mask
     unsafe_elem  (Ne)    compute_unsafe_element_mask
     unsafe_node  (Nnode) compute_unsafe_node_mask
     overlap_lost (Ne)    compute_overlap_lost_element_mask(frac_threshold,
                          min_material_frac)
   each including the outer element shell (boundary_element_mask). */
size_t vdvc_unsafe_masks_workspace_bytes(int Nx, int Ny, int Nz);
int vdvc_unsafe_masks(const uint8_t* active, const uint8_t* mask0, int h,
                      int Nx, int Ny, int Nz, double frac_threshold,
                      double min_material_frac, uint8_t* unsafe_vox,
                      uint8_t* unsafe_elem, uint8_t* unsafe_node,
                      uint8_t* overlap_lost, void* ws, size_t ws_bytes,
                      vdvc_stream_t stream);

/* ---- known-answer (ground-truth) harness --------------------------------
   ground_truth/prepare_ground_truth.py and analyse_ground_truth.py.
   Volumes are pix[x, y, z] C-order arrays, displacements (nx, ny, nz, 3)
   channels-last, float64. */
/* deformed(x) = ref(x - u(x)) by scipy RegularGridInterpolator (linear,
   linear extrapolation past the edges) (make_deformed_image,
   prepare_ground_truth.py:66-89); bit-identical to it. */
int vdvc_gt_warp(const double* ref, const double* u_vox, int nx, int ny,
                 int nz, double* out, vdvc_stream_t stream);
/* out = x + u(x) inside [0, g-1] on every axis (voxel_in_bounds,
   analyse_ground_truth.py:113-136), uint8. */
int vdvc_gt_voxel_in_bounds(const double* u_vox, int nx, int ny, int nz,
                            int gx, int gy, int gz, uint8_t* out,
                            vdvc_stream_t stream);
/* Per node (nbx, nby, nbz, C order) 1 - mean of in_bounds over the support
   box [v-h, v+h] clamped to the image, v = crop_lo + (i, j, k) h
   (node_oob_fraction, :139-174).  crop_lo: host, 3 values. */
int vdvc_gt_node_oob_fraction(const uint8_t* in_bounds, int nx, int ny,
                              int nz, int h, int nbx, int nby, int nbz,
                              const long long* crop_lo, double* out,
                              vdvc_stream_t stream);

/* ---- reductions and pre-alignment ------------------------------------- */
/* *out_host = sum a*b (b != NULL) or sum a, accumulated in float64;
   synchronises the stream (the xp.dot / .sum() calls of the lambda
   calibration, engine/correlate_gpu.py:1007-1025).  ws: >= 16 KiB. */
int vdvc_dot(const void* a, const void* b, int dtype, long long n,
             double* out_host, void* ws, size_t ws_bytes,
             vdvc_stream_t stream);
/* The same into device memory (*out_dev, one double), without a
   synchronisation: several sums can be read back at once. */
int vdvc_dot_device(const void* a, const void* b, int dtype, long long n,
                    double* out_dev, void* ws, size_t ws_bytes,
                    vdvc_stream_t stream);

/* Rigid voxel shift d (host, 3 doubles, pix axis order x,y,z) with
   g(x) ~= f(x - d) by phase correlation of the common corner crop
   (fft_rigid_shift, engine/correlate_gpu.py:381-414).  f_vox, g_vox: vox
   layout of dtype.  Synchronises the stream. */
int vdvc_fft_rigid_shift(const void* f_vox, int fnx, int fny, int fnz,
                         const void* g_vox, int gnx, int gny, int gnz,
                         int dtype, double* d_out3, vdvc_stream_t stream);
/* The same with the shift left on the device (d_dev3: 3 doubles) and no
   host synchronisation: a seed consumed by device work on the same stream. */
int vdvc_fft_rigid_shift_device(const void* f_vox, int fnx, int fny, int fnz,
                                const void* g_vox, int gnx, int gny, int gnz,
                                int dtype, double* d_dev3,
                                vdvc_stream_t stream);

/* ---- affine pre-alignment (engine/correlate_gpu.py:417-825) ------------ */
/* Scratch bytes of the affine entry points below. */
size_t vdvc_affine_workspace_bytes(void);

/* ZNCC sums of affine_prealign's cost (warp_and_cost, :523-536): over the
   voxels x of f whose warped position A (x - c) + c + t lies inside g,
   out6_host = {n, sum f, sum g, sum f^2, sum g^2, sum f g} (float64, g
   sampled at order 1).  A9 row-major; synchronises the stream. */
int vdvc_affine_zncc_sums(const float* f_vox, int nx, int ny, int nz,
                          const float* g_vox, int gnx, int gny, int gnz,
                          const double* A9, const double* t3, const double* c3,
                          double* out6_host, void* ws, size_t ws_bytes,
                          vdvc_stream_t stream);

/* scipy.ndimage.gaussian_filter(in, sigma, mode) with truncate 4 (_smooth_plain,
   :578-582): mode 0 'nearest', 1 'constant' (cval beyond the edges).  When
   mul != NULL the input is multiplied by it first.  tmp: one volume. */
int vdvc_gaussian_filter(const float* in, float* out, int nx, int ny, int nz,
                         double sigma, int mode, double cval, const float* mul,
                         float* tmp, vdvc_stream_t stream);

/* Normalised-convolution smoothing G(img valid)/G(valid), valid = img != cval,
   keeping img where G(valid) <= 1e-6 (_smooth_masked, :585-597).
   tmp1..tmp3: one volume each. */
int vdvc_smooth_masked(const float* img, int nx, int ny, int nz, double sigma,
                       double cval, float* out, float* tmp1, float* tmp2,
                       float* tmp3, vdvc_stream_t stream);

/* One Gauss-Newton system of affine_refine_gn (:757-791): H (12x12, host,
   row-major) and b (12) of the 12-parameter warp s(x) = x - M (x - c) - t_r
   over voxels with s in bounds and g_raw != cval, from the smoothed f_s, its
   (Nvox,3) gradient and the smoothed g_s.  Synchronises the stream. */
int vdvc_affine_normal_equations(const float* f_s, const float* grad_fs,
                                 const float* g_s, const float* g_raw, int nx,
                                 int ny, int nz, const double* M9,
                                 const double* tr3, const double* c3,
                                 double cval, double* H144_host,
                                 double* b12_host, void* ws, size_t ws_bytes,
                                 vdvc_stream_t stream);

/* Masked residual sums of _rms (:724-741): out2_host = {sum e^2, n}. */
int vdvc_affine_rms_sums(const float* f, const float* g, int nx, int ny,
                         int nz, const double* M9, const double* tr3,
                         const double* c3, double cval, double* out2_host,
                         void* ws, size_t ws_bytes, vdvc_stream_t stream);

/* ---- preconditioned CG around an external matvec ------------------------
   The pieces of pcg(matvec, b, M_inv, xp, x0, max_iter, tol)
   (engine/kernels_dvc.py:550-583) for a caller that applies A itself:
     begin      r = b - Ax (Ax may be NULL for x0 = 0), z = M r, p = z,
                rz = r.z, r0 = b.b + 1e-30
     step       alpha = rz / (p.Ap + 1e-30); x += alpha p; r -= alpha Ap;
                z = M r; *res_out = sqrt(r.r / r0) (synchronises the stream)
     direction  p = z + beta p
   Dot products are float64.  ws is vdvc_pcg_workspace_bytes() bytes and
   carries the scalar state between the calls of one solve. */
size_t vdvc_pcg_workspace_bytes(void);
int vdvc_pcg_begin(const void* b, const void* Ax, const void* Minv, int dtype,
                   long long n, void* r, void* z, void* p, int max_iter,
                   double tol, void* ws, size_t ws_bytes, vdvc_stream_t stream);
int vdvc_pcg_step(const void* Ap, const void* Minv, int dtype, long long n,
                  void* x, void* r, void* z, void* p, void* ws,
                  size_t ws_bytes, double* res_out, int* done_out,
                  vdvc_stream_t stream);
int vdvc_pcg_direction(const void* z, void* p, int dtype, long long n,
                       void* ws, size_t ws_bytes, vdvc_stream_t stream);

/* ---- Gauss-Newton solver of one pyramid level ----------------------------
   Device-resident form of the correlate_gpu iteration
   (engine/correlate_gpu.py:1065-1138).  One GN iteration is
     vdvc_gn_sample -> vdvc_gn_rhs -> vdvc_gn_pcg -> vdvc_gn_update.
   All inputs are device pointers that must outlive the solver; the
   workspace (vdvc_gn_workspace_bytes) holds every per-iteration buffer. */
typedef struct vdvc_gn_desc {
  int dtype;                 /* VDVC_F32 (plain solve) or VDVC_F64          */
  int h, Nx, Ny, Nz;
  int gnx, gny, gnz;         /* deformed image shape                          */
  double gx0, gy0, gz0;      /* g_origin                                      */
  double glt;                /* gray-level threshold                          */
  int reg_type;              /* VDVC_REG_*                                     */
  double ll;                 /* regularization weight lambda                  */
  double eps_reg;            /* Laplacian share of the equilibrium-gap R      */
  const double* K_lap;       /* host 24x24 (required when reg_type != NONE)    */
  const double* K_el;        /* host 24x24 (equilibrium gap)                  */
  int dynamic_mask;          /* 1: H and M follow the b mask each iteration   */
  int pcg_chunk;             /* PCG iterations per body of the graph's
                                device-driven WHILE loop (<= 0: 4)           */
  const void* f_vox;         /* reference values, vox layout, uncentred       */
  const void* g_vox;         /* deformed image, vox layout                    */
  const void* grad;          /* (Nvox,3) eroded gradient of f                 */
  const uint8_t* mask0;      /* f > glt                                       */
  const void* interior;      /* (Ndof) P_i diagonal (equilibrium gap)         */
  const double* diag_eqgap;  /* (Ndof) float64 Hutchinson diag of K P_i K     */
  double mean0, std0;        /* multiplicity-weighted stats of f over mask0   */
  vdvc_stream_t stream;      /* stream used for the set-up in vdvc_gn_create   */
  int precision;             /* VDVC_PREC_PLAIN: matrix-free H v from the
                                gradient every PCG step (kernels_dvc.py:
                                452-506).  VDVC_PREC_ELEMENT: element
                                Hessians formed from the float32 gradient
                                once per GN iteration (once per solve after
                                the b mask freezes), FP32 element-Hessian
                                matvecs in the PCG -- the same float32
                                products summed in another order.
                                VDVC_PREC_MIXED: the same from the BF16-
                                rounded gradient.  Both: dtype VDVC_F32,
                                Laplacian K_lap one 8x8 block per component */
  void* eh_ws;               /* ELEMENT / MIXED: device workspace of           */
  size_t eh_ws_bytes;        /*   vdvc_gn_eh_workspace_bytes(precision, ...)   */
} vdvc_gn_desc;

enum { VDVC_PREC_PLAIN = 0, VDVC_PREC_MIXED = 1, VDVC_PREC_ELEMENT = 2 };

/* Bytes of vdvc_gn_desc.eh_ws for a solver of this precision and mesh (0
   for VDVC_PREC_PLAIN or a bad mesh). */
size_t vdvc_gn_eh_workspace_bytes(int precision, int h, int Nx, int Ny, int Nz);

typedef struct vdvc_gn_solver vdvc_gn_solver;

/* buffers readable with vdvc_gn_read */
enum { VDVC_GN_U = 0, VDVC_GN_DU = 1, VDVC_GN_RES = 2, VDVC_GN_LIVE_MASK = 3 };

size_t vdvc_gn_workspace_bytes(int dtype, int h, int Nx, int Ny, int Nz);
int vdvc_gn_create(const vdvc_gn_desc* desc, void* ws, size_t ws_bytes,
                   vdvc_gn_solver** out);
/* U <- U0 (device float64, Ndof) or zeros when U0 == NULL. */
int vdvc_gn_set_U(vdvc_gn_solver* solver, const double* U0,
                  vdvc_stream_t stream);
/* dynamic_mask == 0: diag(H over mask0) + lambda diag(R) and M^-1, once. */
int vdvc_gn_frozen_diag(vdvc_gn_solver* solver, vdvc_stream_t stream);
/* g(x+u), live mask, stats of g over the b mask; freeze_now fixes the b
   mask to this iteration's live mask for the rest of the solve. */
int vdvc_gn_sample(vdvc_gn_solver* solver, int freeze_now,
                   vdvc_stream_t stream);
/* residual, b - lambda R U, diag and M^-1 (dynamic_mask). */
int vdvc_gn_rhs(vdvc_gn_solver* solver, vdvc_stream_t stream);
/* PCG from dU = 0; returns iterations, final relative residual and the
   device status (VDVC_OK or VDVC_ERR_NONFINITE). Synchronises the stream. */
int vdvc_gn_pcg(vdvc_gn_solver* solver, int max_iter, double tol, int* iters,
                double* res, int* status, vdvc_stream_t stream);
/* U += dU and the iteration scalars (synchronises the stream):
   out8 = {|dU|^2, |U|^2, count, sum, sum^2 of res over the live mask,
           active voxels, b-mask weight, status}. */
int vdvc_gn_update(vdvc_gn_solver* solver, double* out8, vdvc_stream_t stream);
/* One whole GN iteration -- sample, rhs, pcg, update -- with a single
   synchronisation of the stream.  out12: the 8 values of vdvc_gn_update,
   PCG iterations, PCG relative residual, PCG status, solver status; the
   return value is that of vdvc_gn_update (e.g. VDVC_ERR_ZERO_DIVISION). */
int vdvc_gn_iterate(vdvc_gn_solver* solver, int freeze_now, int max_iter,
                    double tol, double* out12, vdvc_stream_t stream);
/* Copy a solver buffer to dst (float64 when dst_f64, else float32; masks
   as uint8). */
int vdvc_gn_read(vdvc_gn_solver* solver, int which, void* dst, int dst_f64,
                 vdvc_stream_t stream);
void vdvc_gn_destroy(vdvc_gn_solver* solver);

/* ---- batches of independent solves ------------------------------------
   No counterpart in the reference (it solves one pair per call): a series
   of deformed volumes against one reference, with their own ROIs, element
   sizes and masks, iterated in lockstep.  Each call runs one GN iteration
   of every active problem: sampling, residual and PCG set-up on one stream
   per problem (concurrent = 1) or all on `stream` (concurrent = 0), then
   the PCG loops of all active problems as one CUDA graph (a device-driven
   WHILE loop whose body holds pcg_chunk iterations of every problem), then
   the updates, and one synchronisation.  float32 problems only; descs[i]
   and ws[i] as for vdvc_gn_create. */
typedef struct vdvc_gn_batch vdvc_gn_batch;
int vdvc_gn_batch_create(const vdvc_gn_desc* descs, int n, void* const* ws,
                         const size_t* ws_bytes, int pcg_chunk,
                         int concurrent, vdvc_gn_batch** out);
/* Problem i's solver (for vdvc_gn_set_U / frozen_diag / read; owned by the
   batch: vdvc_gn_destroy on it does nothing). */
int vdvc_gn_batch_solver(vdvc_gn_batch* batch, int i, vdvc_gn_solver** out);
/* One GN iteration of the problems with active[i] != 0 (freeze_now may be
   NULL).  out12: 12 doubles per problem: the 8 values of vdvc_gn_update,
   PCG iterations, PCG relative residual, PCG status, residual status
   (VDVC_ERR_ZERO_DIVISION when std(g) over the b mask is 0). */
int vdvc_gn_batch_iterate(vdvc_gn_batch* batch, const int* active,
                          const int* freeze_now, int max_iter, double tol,
                          double* out12, vdvc_stream_t stream);
/* Change the PCG graph's iterations per body (1..64) and the stream
   schedule; the graph is rebuilt at the next iteration (the autotuner's
   knobs). */
int vdvc_gn_batch_set_schedule(vdvc_gn_batch* batch, int pcg_chunk,
                               int concurrent);
void vdvc_gn_batch_destroy(vdvc_gn_batch* batch);

#ifdef __cplusplus
}
#endif
#endif /* VDVC_H */
