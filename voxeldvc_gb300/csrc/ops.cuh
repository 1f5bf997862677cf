// Declarations shared between the kernel translation units.
#pragma once

#include "common.cuh"
#include "strip.cuh"

namespace vdvc {

struct PcgState;

// Node-centric K application (reg.cu).
template <typename T>
struct StencilArgs {
  Mesh m;
  const T* v;          // nodal input
  const T* p_old;      // when non-null: input is v + beta * p_old (PCG p_new)
  const PcgState* st;  // beta source / done flag (with p_old)
  const T* E_elem;     // per-element scale, or null for scalar E
  double E;
  const T* interior;   // per-dof multiplier applied to the result, or null
  double scale;        // global multiplier
  T* out;
  const T* add_to;     // when non-null: out = add_to + result
};

template <typename T>
int launch_kref_apply(const StencilArgs<T>& a, const Kmat& K, cudaStream_t s);
template <typename T>
int launch_kref_diag(const Mesh& m, const Kmat& K, const T* E_elem, double E, T* out, cudaStream_t s);
int load_K(const double* K_host, Kmat* K);

// Element-strip passes and node gather (strip.cu).
template <typename T, int MODE>
int launch_strip(const StripArgs<T>& args, const Kpair<T>* kp, cudaStream_t s);
template <typename T>
int launch_gather(const Mesh& m, const T* ev, T* out, cudaStream_t s);
// Compile-time-h float32 Hessian pass (strip_fast.cu); VDVC_ERR_UNSUPPORTED
// when h has no specialisation.
template <bool PCG>
int launch_strip_fast(const StripArgs<float>& args, const Kpair<float>* kp, cudaStream_t s);
// Thread-per-element float32 Hessian pass for h <= 4 (elem_fast.cu);
// VDVC_ERR_UNSUPPORTED when h has no specialisation.
template <bool PCG>
int launch_elem_fast(const StripArgs<float>& args, const Kpair<float>* kp, cudaStream_t s);
// Compile-time-h float32 residual / b [/ diag H] pass (rhs_fast.cu);
// VDVC_ERR_UNSUPPORTED when h has no specialisation.
template <bool DG>
int launch_rhs_fast(const StripArgs<float>& args, cudaStream_t s);
long long strip_grid_blocks(const Mesh& m);

// PCG pieces (pcg.cu).
template <typename T>
int launch_pcg_init(const T* b, const T* Ax, const T* Minv, long long n, T* r, T* z, T* p, bool p_is_z, T* x0,
                    PcgState* st, GridReduce red, int max_iter, double tol, cudaStream_t s);
template <typename T>
// max_blocks: blocks the reduction partials of `red` hold (kReduceBlocks at least)
int launch_pcg_gather(const Mesh& m, const T* ev, const T* z, T* p, T* Ap, PcgState* st, GridReduce red,
                      cudaStream_t s, long long max_blocks = kReduceBlocks);
template <typename T>
int launch_pcg_update(const T* p, const T* Ap, const T* Minv, long long n, T* x, T* r, T* z, PcgState* st,
                      GridReduce red, cudaStream_t s);
// Sampling and statistics (sample.cu).
template <typename T>
struct SampleArgs {
  Mesh m;
  int EX;
  const T* U;             // nodal displacement (Ndof)
  const T* g;             // deformed image, vox layout (gnx*gny*gnz)
  int gnx, gny, gnz;
  T gx0, gy0, gz0;        // origin of g in f's voxel frame
  const uint8_t* mask0;   // may be null (all ones)
  T glt;
  T* gvals;               // out (Nvox)
  uint8_t* mask_out;      // out (Nvox)
  // GN extras (stats != null): stats of g over the b mask and the active count
  const uint8_t* bmask_frozen;  // null: b mask = live mask
  GridReduce red;
  double* stats;                // out: count, s1, s2 over the b mask, n_active
  // interp mode (uvox != null): write u(x) instead of sampling
  T* uvox;
  int channels_first;
};
template <typename T, bool STATS, bool INTERP>
int launch_sample(const SampleArgs<T>& args, cudaStream_t s);
template <typename T>
int launch_masked_stats(const T* field, const uint8_t* mask, const Mesh& m, GridReduce red, double* out3,
                        cudaStream_t s);

// Precision form (mixed.cu): BF16 gradient, element Hessians T stored
// tile-major [Ne / kEhTile][162][kEhTile].
constexpr int kEhTile = 64;
struct EhFormArgs {
  Mesh m;
  const void* grad;       // (Nvox,3) __nv_bfloat16, or float when grad_f32
  const uint8_t* mask;    // H mask
  float* T;               // [tiles][162][kEhTile]
  float* evD;             // [24][Ne] diagonal contributions
  long long pitch;        // eh_pitch(Ne): elements rounded up to whole tiles
  const float* gmax;      // max |g| of the BF16 gradient (device); the tensor-core formation's scale
  int* err;               // set to VDVC_ERR_CUDA if a tensor-core formation wait times out
  int grad_f32;           // 1: grad is the float32 gradient itself (no BF16 rounding)
  void* Tb;               // when set: the entries are stored here as BF16 (same layout) instead of in T
};

struct EhMatvecArgs {
  Mesh m;
  const float* T;      // [tiles][162][kEhTile]
  const void* Tb;      // when set: BF16 entries (same layout) read instead of T
  long long pitch;     // eh_pitch(Ne): elements rounded up to whole tiles
  int* err;            // set to VDVC_ERR_CUDA if a tile's bulk copies time out
  const float* v;      // nodal input (PCG: z)
  const float* p_old;  // PCG: p_new = z + beta p_old
  const PcgState* st;
  float* ev;           // [24][Ne]
  // regularizer: c1 * (L8 on each component) v_e + c2 * K2 w_e
  int nreg;
  float c1, c2;
  float L8[64];
  const float* w;
  const float* K2;     // 576 (device)
};

int launch_eh_form(const EhFormArgs& a, cudaStream_t s);
long long eh_pitch(long long Ne);  // elements rounded up to whole tiles
template <bool PCG>
int launch_eh_matvec(const EhMatvecArgs& a, cudaStream_t s);
// BF16 copy of the gradient and, when gmax != NULL, max |g| of the copy
int launch_grad_bf16(const float* g, long long n, void* out, float* gmax, cudaStream_t s);
int launch_eh_form_tc(const EhFormArgs& a, cudaStream_t s);

inline int grid_blocks(long long n, int threads, long long cap) {
  long long b = (n + threads - 1) / threads;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace vdvc
