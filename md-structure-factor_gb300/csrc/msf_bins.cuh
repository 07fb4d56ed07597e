// msf_bins.cuh -- numpy.histogramdd bin search shared by the deposit kernels.
//
// Edges e[i] = i*(L/n), e[n] = L (numpy.linspace); bin = the largest i with
// e[i] <= x; x == e[n] goes to bin n-1; x < 0, x > L and NaN are dropped (-1).
// float32 inputs are searched in FP32 against flo[i] = smallest float >= e[i]
// and fhi[i] = largest float <= e[i], which gives the FP64 answer exactly.
#pragma once

#include "msf_internal.cuh"

namespace msf {

struct DepArgs {
  const void* pos;
  const int32_t* w;
  int64_t n_atoms;
  int64_t frame_stride;  // elements (float4 or double) between frames
  const double* scale;   // (nframes, 3) or null
  int flags;
  int n0, n1, n2;
  double L0, L1, L2;
  float inv0, inv1, inv2;
  const double* e0;
  const double* e1;
  const double* e2;
  const float* flo0;
  const float* flo1;
  const float* flo2;
  const float* fhi0;
  const float* fhi1;
  const float* fhi2;
  int32_t* grids;
  int64_t V;
};

// The estimate floor(x*n/L) is off by at most one bin; both neighbouring
// edges are loaded together (one dependent round trip) and the rare
// misestimate is corrected by the loops.
__device__ __forceinline__ int bin_f32(float x, int n, float inv, const float* __restrict__ flo,
                                       const float* __restrict__ fhi) {
  const float lo_edge = __ldg(flo), hi_edge = __ldg(fhi + n);
  int b = (int)(x * inv);
  b = b < 0 ? 0 : (b > n - 1 ? n - 1 : b);
  const float e0 = __ldg(flo + b), e1 = __ldg(flo + b + 1);
  if (!(x >= lo_edge) || !(x <= hi_edge)) return -1;  // also drops NaN
  if (x < e0) {
    --b;
    while (b > 0 && x < __ldg(flo + b)) --b;
  } else if (b < n - 1 && x >= e1) {
    ++b;
    while (b < n - 1 && x >= __ldg(flo + b + 1)) ++b;
  }
  return b;
}

// bin_f32 with the flo table in shared memory (plain loads) and the upper
// edge fhi[n] passed by value
__device__ __forceinline__ int bin_f32_tab(float x, int n, float inv, const float* flo, float hi_edge) {
  const float lo_edge = flo[0];
  int b = (int)(x * inv);
  b = b < 0 ? 0 : (b > n - 1 ? n - 1 : b);
  const float e0 = flo[b], e1 = flo[b + 1];
  if (!(x >= lo_edge) || !(x <= hi_edge)) return -1;  // also drops NaN
  if (x < e0) {
    --b;
    while (b > 0 && x < flo[b]) --b;
  } else if (b < n - 1 && x >= e1) {
    ++b;
    while (b < n - 1 && x >= flo[b + 1]) ++b;
  }
  return b;
}

__device__ __forceinline__ int bin_f64(double x, int n, float inv, const double* __restrict__ e) {
  const double lo_edge = __ldg(e), hi_edge = __ldg(e + n);
  int b = (int)((float)x * inv);
  b = b < 0 ? 0 : (b > n - 1 ? n - 1 : b);
  const double e0 = __ldg(e + b), e1 = __ldg(e + b + 1);
  if (!(x >= lo_edge) || !(x <= hi_edge)) return -1;
  if (x < e0) {
    --b;
    while (b > 0 && x < __ldg(e + b)) --b;
  } else if (b < n - 1 && x >= e1) {
    ++b;
    while (b < n - 1 && x >= __ldg(e + b + 1)) ++b;
  }
  return b;
}

// dens.py:52-58 (per-frame rescale) and dens.py:211-212 (wrap), in FP64.
__device__ __forceinline__ double prep(double x, const double* s, int axis, bool wrap, double L) {
  if (s) x = __dmul_rn(x, __ldg(s + axis));
  if (wrap) {
    x = (x < L) ? x : __dsub_rn(x, L);
    x = (x > 0.0) ? x : __dadd_rn(x, L);
  }
  return x;
}

inline DepArgs dep_args(const msf_plan* p) {
  DepArgs a;
  a.n0 = p->n0; a.n1 = p->n1; a.n2 = p->n2;
  a.L0 = p->box[0]; a.L1 = p->box[1]; a.L2 = p->box[2];
  a.inv0 = (float)(p->n0 / p->box[0]);
  a.inv1 = (float)(p->n1 / p->box[1]);
  a.inv2 = (float)(p->n2 / p->box[2]);
  const double* e = ws_ptr<double>(p, p->off_edges_d);
  const float* lo = ws_ptr<float>(p, p->off_edges_flo);
  const float* hi = ws_ptr<float>(p, p->off_edges_fhi);
  const int o1 = p->n0 + 1, o2 = p->n0 + p->n1 + 2;
  a.e0 = e; a.e1 = e + o1; a.e2 = e + o2;
  a.flo0 = lo; a.flo1 = lo + o1; a.flo2 = lo + o2;
  a.fhi0 = hi; a.fhi1 = hi + o1; a.fhi2 = hi + o2;
  a.V = grid_elems(p);
  return a;
}

// Bins (b0, b1, b2) and weight of atom i of `frame` for position layout MODE:
// 0 float4 FP32 search, 1 float4 FP64 rescale/wrap, 2 FP64 (N,3) + int32 w,
// 3 float (N,3) + int32 w FP32 search, 4 float (N,3) + int32 w FP64 rescale/wrap.
// Returns false when the atom is dropped.
template <int MODE>
__device__ __forceinline__ bool atom_bins(const DepArgs& a, int frame, int64_t i, int& b0, int& b1,
                                          int& b2, int& wgt) {
  const double* s = a.scale ? a.scale + 3 * frame : nullptr;
  const bool wrap = a.flags & MSF_WRAP;
  if (MODE == 2) {
    const double* r = static_cast<const double*>(a.pos) + frame * a.frame_stride + 3 * i;
    wgt = __ldg(a.w + i);
    b0 = bin_f64(prep(__ldg(r + 0), s, 0, wrap, a.L0), a.n0, a.inv0, a.e0);
    b1 = bin_f64(prep(__ldg(r + 1), s, 1, wrap, a.L1), a.n1, a.inv1, a.e1);
    b2 = bin_f64(prep(__ldg(r + 2), s, 2, wrap, a.L2), a.n2, a.inv2, a.e2);
  } else if (MODE >= 3) {
    const float* r = static_cast<const float*>(a.pos) + frame * a.frame_stride + 3 * i;
    wgt = __ldg(a.w + i);
    const float x = __ldg(r + 0), y = __ldg(r + 1), z = __ldg(r + 2);
    if (MODE == 3) {
      b0 = bin_f32(x, a.n0, a.inv0, a.flo0, a.fhi0);
      b1 = bin_f32(y, a.n1, a.inv1, a.flo1, a.fhi1);
      b2 = bin_f32(z, a.n2, a.inv2, a.flo2, a.fhi2);
    } else {
      b0 = bin_f64(prep((double)x, s, 0, wrap, a.L0), a.n0, a.inv0, a.e0);
      b1 = bin_f64(prep((double)y, s, 1, wrap, a.L1), a.n1, a.inv1, a.e1);
      b2 = bin_f64(prep((double)z, s, 2, wrap, a.L2), a.n2, a.inv2, a.e2);
    }
  } else {
    const float4 v = __ldg(static_cast<const float4*>(a.pos) + frame * a.frame_stride + i);
    wgt = __float2int_rn(v.w);
    if (MODE == 0) {
      b0 = bin_f32(v.x, a.n0, a.inv0, a.flo0, a.fhi0);
      b1 = bin_f32(v.y, a.n1, a.inv1, a.flo1, a.fhi1);
      b2 = bin_f32(v.z, a.n2, a.inv2, a.flo2, a.fhi2);
    } else {
      b0 = bin_f64(prep((double)v.x, s, 0, wrap, a.L0), a.n0, a.inv0, a.e0);
      b1 = bin_f64(prep((double)v.y, s, 1, wrap, a.L1), a.n1, a.inv1, a.e1);
      b2 = bin_f64(prep((double)v.z, s, 2, wrap, a.L2), a.n2, a.inv2, a.e2);
    }
  }
  return (b0 >= 0) & (b1 >= 0) & (b2 >= 0);
}

// atom_bins for the FP32-search modes (0, 3) with the three flo tables in
// shared memory (t: flo0 | flo1 | flo2, t_hi: the three fhi[n])
template <int MODE>
__device__ __forceinline__ bool atom_bins_tab(const DepArgs& a, int frame, int64_t i, const float* t,
                                              const float* t_hi, int& b0, int& b1, int& b2, int& wgt) {
  static_assert(MODE == 0 || MODE == 3, "FP32 search modes only");
  float x, y, z;
  if (MODE == 0) {
    const float4 v = __ldg(static_cast<const float4*>(a.pos) + frame * a.frame_stride + i);
    x = v.x; y = v.y; z = v.z;
    wgt = __float2int_rn(v.w);
  } else {
    const float* r = static_cast<const float*>(a.pos) + frame * a.frame_stride + 3 * i;
    wgt = __ldg(a.w + i);
    x = __ldg(r + 0); y = __ldg(r + 1); z = __ldg(r + 2);
  }
  b0 = bin_f32_tab(x, a.n0, a.inv0, t, t_hi[0]);
  b1 = bin_f32_tab(y, a.n1, a.inv1, t + a.n0 + 1, t_hi[1]);
  b2 = bin_f32_tab(z, a.n2, a.inv2, t + a.n0 + a.n1 + 2, t_hi[2]);
  return (b0 >= 0) & (b1 >= 0) & (b2 >= 0);
}

// MODE for a position layout and the presence of rescale/wrap.
inline int deposit_mode(int layout, bool fp64_prep) {
  if (layout == kLayoutF64) return 2;
  if (layout == kLayoutF32xyz) return fp64_prep ? 4 : 3;
  return fp64_prep ? 1 : 0;
}

}  // namespace msf
