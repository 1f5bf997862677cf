// Element-strip kernels: the voxel-centre quadrature passes of the
// correlation operator (H v, b, diag H) over implicit Hex8 connectivity.
//
// Decomposition ("owner computes").  Every voxel is visited exactly once, by
// the element with the highest index containing it, i.e. element
// (min(vx/h, Nx-1), ...).  The reference visits each voxel once per element
// containing it, with trapezoid weights 1/2 per axis on element end planes
// (engine/kernels_dvc.py:452-506, engine/geometry_dvc.py:26-51).  On an
// interior element plane the two halves of the two elements sharing the
// voxel add up to 1, and the Hex8 shape functions are continuous across the
// plane, so one visit with weight 1 assembles the same operator.  On the
// outer faces of the mesh only one element holds the voxel and its weight
// stays 1/2 per axis: the kernels apply w = prod over axes of (1/2 on the
// first/last voxel plane, 1 elsewhere).
//
// A CTA owns a strip of EX consecutive elements along x in element row
// (j,k).  Thread t owns voxel column x = i*h + qx (i = strip element t/h,
// qx = t%h) and walks its (qy,qz) plane; the last element of the mesh also
// owns the column x = Nx*h, walked by its qx = h-1 thread.  The shape
// functions are separable, N_a(q) = phi_ax(qx) phi_ay(qy) phi_az(qz), so the
// 24 element sums are accumulated separably: per voxel 6 FMAs on a qy run,
// per qz row 12 FMAs, per column a phi_ax weighting, and a shared-memory
// reduction over the columns of each element.  Element vectors go to a
// [24][Ne] buffer (row = 3*a + c), and a node-parallel gather sums the eight
// element contributions of every node in a fixed order -- deterministic,
// with no atomics.
#pragma once

#include "common.cuh"

namespace vdvc {

enum StripMode : int {
  kModeHv = 1,    // accumulate m (grad.u) grad with phi weights  (H v)
  kModeB = 2,     // accumulate m res grad with phi weights        (b)
  kModeDiag = 4,  // accumulate m grad^2 with phi^2 weights         (diag H)
  kModeRes = 8,   // compute res from f, g(x+u) and the stats, write it (GN)
  kModePcg = 16   // nodal input is p_new = z + beta p (PCG, reads state)
};

struct PcgState;  // pcg.cuh

// Largest strip used: EX*h <= 128 threads.
struct StripShape {
  int EX, threads;
};

inline StripShape strip_shape(int h) {
  StripShape s;
  s.EX = h >= 128 ? 1 : 128 / h;
  int t = s.EX * h;
  s.threads = (t + 31) / 32 * 32;
  return s;
}

// Dense 24x24 operators fused into the H element pass (regularizer terms).
template <typename T>
struct Kpair {
  T K1[576];
  T K2[576];
};

template <typename T>
struct StripArgs {
  Mesh m;
  int EX;
  // inputs
  const T* v;          // nodal vector (Hv), or z in PCG mode
  const T* p_old;      // PCG mode: p_new = z + beta * p_old
  const PcgState* st;  // PCG mode
  const T* grad;       // (Nvox,3)
  const uint8_t* mask; // H / b mask (Nvox)
  const T* res_in;     // b mode without kModeRes
  // GN residual inputs (kModeRes)
  const T* f;          // reference values (uncentred)
  const T* gvals;      // g(x+u)
  const uint8_t* live; // live mask for the displayed std(res)
  const double* gstats;// count, s1, s2 of g over the b mask (device)
  double mean0, std0;  // reference stats
  T* res_out;          // residual output (Nvox)
  GridReduce red;      // display stats of res over the live mask
  double* dstats;      // count, s1, s2 of res over live (device, written by the last block)
  int* status;         // device status word
  // outputs
  T* evA;  // [24][Ne] phi-weighted sums (Hv or b)
  T* evD;  // [24][Ne] phi^2-weighted sums (diag)
  // regularizer fusion (Hv only): ev += c1 K1 v_loc + c2 K2 w_loc
  const T* w;  // nodal vector for K2 (may be null)
  T c1, c2;
  int nreg;    // 0, 1 (K1) or 2 (K1 and K2)
  int k1_blockdiag;  // K1 = the same 8x8 block L8 on each component (vector Laplacian)
  float L8[64];      // that block, row-major over local corners (k1_blockdiag)
};

}  // namespace vdvc
