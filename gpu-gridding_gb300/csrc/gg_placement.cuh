// Placement arithmetic shared by the gridding and degridding kernels.
//
// Reproduces the reference's placement exactly (oskar_grid_wproj.c:146-187
// for FP32, :57-98 for FP64): every product, difference, square root and
// rounding is an explicitly rounded IEEE operation (no contraction), so the
// cell, offset, plane and skip decisions are bit-identical to the serial
// code for finite inputs.
#pragma once

#include "gg_common.cuh"

namespace gg {

// Rounded arithmetic in the call's precision.
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float rsqrt_rn(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double rsqrt_rn(double a) { return __dsqrt_rn(a); }
// roundf / round: half away from zero, as C's round().
__device__ __forceinline__ float rround(float a) { return roundf(a); }
__device__ __forceinline__ double rround(double a) { return round(a); }
__device__ __forceinline__ float rabs(float a) { return fabsf(a); }
__device__ __forceinline__ double rabs(double a) { return fabs(a); }


struct Placement {
  int gu, gv, ou, ov, plane, conj_neg, skipped, support;
};

template <typename Real>
__device__ __forceinline__ Placement place_one(const PlaceParams<Real>& p,
                                               const StackView& v,
                                               unsigned long long i) {
  Placement r;
  const Real os = (Real)v.oversample;
  const Real pos_u = rmul(-p.uu[i], p.grid_scale);
  const Real pos_v = rmul(p.vv[i], p.grid_scale);
  const Real ww = p.ww[i];
  const Real rw = rround(rsqrt_rn(rabs(rmul(ww, p.w_scale))));
  // (size_t)rw < num_w_planes, else the last plane.  A NaN compares false
  // and takes the last plane.
  r.plane = (rw < (Real)v.num_planes) ? (int)rw : v.num_planes - 1;
  r.support = v.support[r.plane];
  r.conj_neg = ww > (Real)0;
  const Real ru = rround(pos_u), rv = rround(pos_v);
  // A cell index outside int range (or NaN) cannot lie on the grid: the
  // reference's conversion yields INT_MIN there and the point is skipped.
  const bool in_range = rabs(ru) < (Real)2147483648.0 &&
                        rabs(rv) < (Real)2147483648.0;
  if (in_range) {
    r.gu = (int)ru + p.grid_centre;
    r.gv = (int)rv + p.grid_centre;
    r.ou = (int)rround(rmul(rsub(ru, pos_u), os));
    r.ov = (int)rround(rmul(rsub(rv, pos_v), os));
    const long long s = r.support, G = p.grid_size;
    r.skipped = ((long long)r.gu + s >= G || (long long)r.gu - s < 0 ||
                 (long long)r.gv + s >= G || (long long)r.gv - s < 0);
  } else {
    r.gu = r.gv = r.ou = r.ov = 0;
    r.skipped = 1;
  }
  return r;
}

}  // namespace gg
