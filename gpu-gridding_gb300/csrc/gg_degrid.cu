// Adjoint of the gridding map (degridding): grid -> visibilities.
//
// Forward gridding adds v_i * c~_i(cell) to every cell of visibility i's
// footprint (oskar_grid_wproj.c:190-209), with c~ the kernel tap whose
// imaginary part is negated for ww > 0.  Its exact adjoint is the gather
//   out_i = sum over the footprint of conj(c~_i(cell)) * grid(cell),
// computed here with one warp per visibility: lanes take consecutive
// columns of each footprint row (coalesced grid reads) and the warp reduces
// by shuffles.  There is no write conflict, so no atomics.  The reference
// has no degridder; this one is pinned by the dot-product identity
// <G x, y> = <x, G^H y> against the forward kernel and by the FP64 oracle.
#include "gg_internal.h"
#include "gg_placement.cuh"

namespace gg {

namespace {

constexpr int kDegridThreads = 256;

template <typename Real>
__global__ void __launch_bounds__(kDegridThreads)
k_degrid(PlaceParams<Real> p, StackView v, const Real* __restrict__ grid,
         Real* __restrict__ out) {
  using R2 = typename Vec2<Real>::type;
  const int lane = threadIdx.x & 31;
  const unsigned long long warps_total =
      (unsigned long long)gridDim.x * (kDegridThreads / 32);
  const R2* __restrict__ taps = (const R2*)v.taps;
  const R2* __restrict__ g2 = (const R2*)grid;
  for (unsigned long long i =
           (unsigned long long)blockIdx.x * (kDegridThreads / 32) +
           (threadIdx.x >> 5);
       i < p.num_points; i += warps_total) {
    const Placement r = place_one(p, v, i);
    Real acc_re = 0, acc_im = 0;
    if (!r.skipped) {
      const int s = r.support;
      const long long F = 2 * s + 1;
      const R2* __restrict__ slice =
          taps + slice_offset(v.base[r.plane], s, v.omax, abs(r.ou),
                              abs(r.ov));
      const int su = r.ou < 0 ? -1 : 1, sv = r.ov < 0 ? -1 : 1;
      const Real sgn = r.conj_neg ? (Real)-1 : (Real)1;
      for (int j = -s; j <= s; ++j) {
        const R2* __restrict__ trow = slice + (s + sv * j) * F + s;
        const R2* __restrict__ grow =
            g2 + (size_t)(r.gv + j) * p.grid_size + r.gu;
        for (int k = lane - s; k <= s; k += 32) {
          const R2 c = __ldg(trow + su * k);
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
cudaError_t launch_degrid(PlaceParams<Real> p, StackView view,
                          const Real* grid, Real* out_vis, cudaStream_t s) {
  if (p.num_points == 0) return cudaSuccess;
  unsigned long long warps_needed = p.num_points;
  unsigned long long blocks =
      (warps_needed + (kDegridThreads / 32) - 1) / (kDegridThreads / 32);
  if (blocks > 1u << 20) blocks = 1u << 20;
  k_degrid<Real><<<(unsigned)blocks, kDegridThreads, 0, s>>>(p, view, grid,
                                                              out_vis);
  return cudaGetLastError();
}

template cudaError_t launch_degrid<float>(PlaceParams<float>, StackView,
                                          const float*, float*, cudaStream_t);
template cudaError_t launch_degrid<double>(PlaceParams<double>, StackView,
                                           const double*, double*,
                                           cudaStream_t);

}  // namespace gg
