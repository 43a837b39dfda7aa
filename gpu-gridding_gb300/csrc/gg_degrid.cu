// Adjoint of the gridding map (degridding): grid -> visibilities.
//
// Forward gridding adds v_i * c~_i(cell) to every cell of visibility i's
// footprint (oskar_grid_wproj.c:190-209), with c~ the kernel tap whose
// imaginary part is negated for ww > 0.  Its exact adjoint is the gather
//   out_i = sum over the footprint of conj(c~_i(cell)) * grid(cell),
// computed here with one warp per visibility, the visibilities sorted by
// grid block and w-plane first so that neighbouring warps share grid rows
// and kernel slabs in cache: lanes take consecutive columns of each
// footprint row (coalesced grid reads) and the warp reduces by shuffles.
// There is no write conflict, so no atomics.  The reference
// has no degridder; this one is pinned by the dot-product identity
// <G x, y> = <x, G^H y> against the forward kernel and by the FP64 oracle.
#include "gg_internal.h"
#include "gg_placement.cuh"

namespace gg {

namespace {

constexpr int kDegridThreads = 256;

// Sort key of a visibility: its 32 x 32-cell block, then its w-plane
// (when the bits allow), so that consecutive warps gather from the same
// grid rows and kernel slabs; skipped visibilities sort last.
template <typename Real>
__global__ void __launch_bounds__(kDegridThreads)
k_degrid_keys(PlaceParams<Real> p, StackView v, int blocks_u, int plane_bits,
              uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const unsigned long long i =
      (unsigned long long)blockIdx.x * kDegridThreads + threadIdx.x;
  if (i >= p.num_points) return;
  const Placement r = place_one(p, v, i);
  uint32_t key = 0xFFFFFFFFu;
  if (!r.skipped) {
    const uint32_t blk = (uint32_t)(r.gv >> 5) * (uint32_t)blocks_u +
                         (uint32_t)(r.gu >> 5);
    key = (blk << plane_bits) | (plane_bits ? (uint32_t)r.plane : 0u);
  }
  keys[i] = key;
  vals[i] = (uint32_t)i;
}

// One warp per visibility, in sorted order.  Lanes are split into groups
// of G = 8, 16 or 32 consecutive footprint columns (the smallest that
// holds a row), so a warp covers 32 / G rows at a time; taps come from the
// slab stack (footprint row j at padded row kSlicePad + s +- j, quadrant
// column |ou + k*os| at residue position r*M + m), grid values from the
// footprint's rows.  The warp reduces by shuffles; no write conflicts.
template <typename Real>
__global__ void __launch_bounds__(kDegridThreads)
k_degrid(PlaceParams<Real> p, StackView v, const uint32_t* __restrict__ order,
         const Real* __restrict__ grid, Real* __restrict__ out) {
  using R2 = typename Vec2<Real>::type;
  const int lane = threadIdx.x & 31;
  const unsigned long long warps_total =
      (unsigned long long)gridDim.x * (kDegridThreads / 32);
  const R2* __restrict__ slabs = (const R2*)v.slabs;
  const R2* __restrict__ g2 = (const R2*)grid;
  const int os = v.oversample;
  for (unsigned long long w =
           (unsigned long long)blockIdx.x * (kDegridThreads / 32) +
           (threadIdx.x >> 5);
       w < p.num_points; w += warps_total) {
    const unsigned long long i = order[w];
    const Placement r = place_one(p, v, i);
    Real acc_re = 0, acc_im = 0;
    if (!r.skipped) {
      const int s = r.support;
      const int F = 2 * s + 1;
      const int G = F <= 8 ? 8 : (F <= 16 ? 16 : 32);
      const int grp = lane / G, kk = lane % G, ngrp = 32 / G;
      const int M = slab_cols_m(s, os, v.omax);
      const long long W = (long long)os * M;
      const R2* __restrict__ slab =
          slabs + v.sbase[r.plane] + abs(r.ov) * slab_taps(s, os, v.omax);
      const int ou = r.ou;
      const int ap = ((ou % os) + os) % os, an = ((-ou % os) + os) % os;
      const int bp = (ou - ap) / os, bn = (-ou - an) / os;
      const int rdir = r.ov < 0 ? -1 : 1;
      const Real sgn = r.conj_neg ? (Real)-1 : (Real)1;
      for (int j = grp - s; j <= s; j += ngrp) {
        const R2* __restrict__ trow = slab + (kSlicePad + s + rdir * j) * W;
        const R2* __restrict__ grow =
            g2 + (size_t)(r.gv + j) * p.grid_size + r.gu;
        for (int k = kk - s; k <= s; k += G) {
          const int q = ou + k * os >= 0 ? ap * M + k + bp : an * M + bn - k;
          const R2 c = __ldg(trow + q);
          const R2 gv = grow[k];
          const Real cim = sgn * c.y;
          // conj(c~) * g
          acc_re = fma(c.x, gv.x, fma(cim, gv.y, acc_re));
          acc_im = fma(c.x, gv.y, fma(-cim, gv.x, acc_im));
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc_re += __shfl_down_sync(0xffffffffu, acc_re, o);
      acc_im += __shfl_down_sync(0xffffffffu, acc_im, o);
    }
    if (lane == 0) {
      out[2 * i] = acc_re;
      out[2 * i + 1] = acc_im;
    }
  }
}

}  // namespace

template <typename Real>
cudaError_t launch_degrid_keys(PlaceParams<Real> p, StackView view,
                               int blocks_u, int plane_bits, uint32_t* keys,
                               uint32_t* vals, cudaStream_t s) {
  if (p.num_points == 0) return cudaSuccess;
  const unsigned long long blocks =
      (p.num_points + kDegridThreads - 1) / kDegridThreads;
  k_degrid_keys<Real><<<(unsigned)blocks, kDegridThreads, 0, s>>>(
      p, view, blocks_u, plane_bits, keys, vals);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_degrid(PlaceParams<Real> p, StackView view,
                          const uint32_t* order, const Real* grid,
                          Real* out_vis, cudaStream_t s) {
  if (p.num_points == 0) return cudaSuccess;
  unsigned long long warps_needed = p.num_points;
  unsigned long long blocks =
      (warps_needed + (kDegridThreads / 32) - 1) / (kDegridThreads / 32);
  if (blocks > 1u << 20) blocks = 1u << 20;
  k_degrid<Real><<<(unsigned)blocks, kDegridThreads, 0, s>>>(
      p, view, order, grid, out_vis);
  return cudaGetLastError();
}

template cudaError_t launch_degrid_keys<float>(PlaceParams<float>, StackView,
                                               int, int, uint32_t*, uint32_t*,
                                               cudaStream_t);
template cudaError_t launch_degrid_keys<double>(PlaceParams<double>,
                                                StackView, int, int,
                                                uint32_t*, uint32_t*,
                                                cudaStream_t);
template cudaError_t launch_degrid<float>(PlaceParams<float>, StackView,
                                          const uint32_t*, const float*,
                                          float*, cudaStream_t);
template cudaError_t launch_degrid<double>(PlaceParams<double>, StackView,
                                           const uint32_t*, const double*,
                                           double*, cudaStream_t);

}  // namespace gg
