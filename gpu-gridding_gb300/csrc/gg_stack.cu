// Kernel-stack preparation: re-layout of the reference's quadrant cube into
// the residue-split layout of StackView, and the FP64 tap sums used for the
// grid normalisation.
//
// The reference re-packs its kernels on the host on every call
// (compact_wkernels, oskar_grid_wproj_gpu.cu:1461-1643).  Here the re-layout
// runs once per kernel stack on the device and the result is kept in a
// handle.
#include "gg_internal.h"

namespace gg {

namespace {


// One thread per output tap; blockIdx.y is the plane.  Output: for each
// absolute offset class (cu, cv) the (2s+1)^2 slice S[jj][kk] =
// K[|cv + (jj-s)*os|][|cu + (kk-s)*os|] (see StackView).
template <typename Real>
__global__ void k_relayout(const Real* __restrict__ conv, StackView v,
                           typename Vec2<Real>::type* __restrict__ out) {
  using R2 = typename Vec2<Real>::type;
  const int p = blockIdx.y;
  const int os = v.oversample, csh = v.conv_size_half;
  const int s = v.support[p];
  const long long F = 2 * s + 1;
  const long long rows = F + 2 * kSlicePad;   // padded slice rows
  const long long stride = slice_taps(s);     // >= rows * F, even
  const int classes = (v.omax + 1) * (v.omax + 1);
  const long long n = (long long)classes * stride;
  const long long base = v.base[p];
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const long long rem = e % stride;
    const int kk = (int)(rem % F);
    const int jj = (int)(rem / F) - kSlicePad;
    const int cls = (int)(e / stride);
    const int cu = cls / (v.omax + 1), cv = cls % (v.omax + 1);
    const int t = abs(cv + (jj - s) * os);   // row    = |off_v + j*os|
    const int c = abs(cu + (kk - s) * os);   // column = |off_u + k*os|
    R2 val;
    if (rem < rows * F && jj >= 0 && jj < F && t < csh && c < csh) {
      const size_t src = (((size_t)p * csh + t) * csh + c) * 2;
      val.x = conv[src];
      val.y = conv[src + 1];
    } else {
      // Padding rows, and taps beyond the cube (which the reference would
      // read out of bounds), are zero.
      val.x = 0; val.y = 0;
    }
    out[base + e] = val;
  }
}

// One thread per output tap of the slab stack; blockIdx.y is the plane.
// slab_{p,c}[kSlicePad + j + s][r][m] = K_p[|c + j*os|][r + m*os]; padding
// rows, and taps beyond the cube, are zero.
template <typename Real>
__global__ void k_relayout_slabs(const Real* __restrict__ conv, StackView v,
                                 typename Vec2<Real>::type* __restrict__ out) {
  using R2 = typename Vec2<Real>::type;
  const int p = blockIdx.y;
  const int os = v.oversample, csh = v.conv_size_half;
  const int s = v.support[p];
  const int F = 2 * s + 1;
  const int M = slab_cols_m(s, os, v.omax);
  const long long row_taps = (long long)os * M;
  const long long stride = slab_taps(s, os, v.omax);
  const long long n = (long long)(v.omax + 1) * stride;
  const long long base = v.sbase[p];
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(e / stride);
    const long long rem = e - c * stride;
    const int jp = (int)(rem / row_taps) - kSlicePad;
    const int in_row = (int)(rem % row_taps);
    const int col = (in_row / M) + (in_row % M) * os;   // r + m*os
    const int t = abs(c + (jp - s) * os);
    R2 val;
    if (jp >= 0 && jp < F && t < csh && col < csh) {
      const size_t src = (((size_t)p * csh + t) * csh + col) * 2;
      val.x = conv[src];
      val.y = conv[src + 1];
    } else {
      val.x = 0; val.y = 0;
    }
    out[base + e] = val;
  }
}

// Sum of the real parts of every tap a footprint uses, for one (plane,
// off_u, off_v), accumulated in FP64 in the reference's order: rows j
// outer, columns k inner (oskar_grid_wproj.c:190-208, sum += c_re).  A
// visibility's norm contribution is then tap_sum * weight, bit-identical to
// the reference's per-visibility sum.
template <typename Real>
__global__ void k_tap_sums(const Real* __restrict__ conv, StackView v,
                           double* __restrict__ tap_sum) {
  const int side = 2 * v.omax + 1;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= v.num_planes * side * side) return;
  const int p = idx / (side * side);
  const int ou = (idx / side) % side - v.omax;
  const int ov = idx % side - v.omax;
  const int s = v.support[p];
  const int os = v.oversample, csh = v.conv_size_half;
  const size_t kstart = (size_t)p * csh * csh;
  // The additions stay in the reference's order; the loads of 8 taps are
  // issued together so their latencies overlap.
  double sum = 0.0;
  for (int j = -s; j <= s; ++j) {
    const int t = abs(ov + j * os);
    const Real* row = conv + (kstart + (size_t)t * csh) * 2;
    int k = -s;
    for (; k + 7 <= s; k += 8) {
      double re[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int c = abs(ou + (k + q) * os);
        re[q] = (t < csh && c < csh) ? (double)row[(size_t)c * 2] : 0.0;
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) sum = __dadd_rn(sum, re[q]);
    }
    for (; k <= s; ++k) {
      const int c = abs(ou + k * os);
      sum = __dadd_rn(sum, (t < csh && c < csh) ? (double)row[(size_t)c * 2]
                                                : 0.0);
    }
  }
  tap_sum[idx] = sum;
}

}  // namespace

template <typename Real>
cudaError_t launch_stack_relayout(const Real* d_conv_func, StackView view,
                                  void* d_taps_out, long long total_taps,
                                  cudaStream_t s) {
  (void)total_taps;
  dim3 grid(64, view.num_planes);
  k_relayout<Real><<<grid, 256, 0, s>>>(
      d_conv_func, view, (typename Vec2<Real>::type*)d_taps_out);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_stack_relayout_slabs(const Real* d_conv_func,
                                        StackView view, void* d_out,
                                        cudaStream_t s) {
  dim3 grid(64, view.num_planes);
  k_relayout_slabs<Real><<<grid, 256, 0, s>>>(
      d_conv_func, view, (typename Vec2<Real>::type*)d_out);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_tap_sums(StackView view, double* d_tap_sum,
                            cudaStream_t s) {
  // The raw cube is needed for the reference-order sums; it is passed in
  // view.taps by the caller for this launch only.
  const int side = 2 * view.omax + 1;
  const int n = view.num_planes * side * side;
  k_tap_sums<Real><<<(n + 127) / 128, 128, 0, s>>>(
      (const Real*)view.taps, view, d_tap_sum);
  return cudaGetLastError();
}

template cudaError_t launch_stack_relayout<float>(const float*, StackView,
                                                  void*, long long,
                                                  cudaStream_t);
template cudaError_t launch_stack_relayout<double>(const double*, StackView,
                                                   void*, long long,
                                                   cudaStream_t);
template cudaError_t launch_stack_relayout_slabs<float>(const float*,
                                                        StackView, void*,
                                                        cudaStream_t);
template cudaError_t launch_stack_relayout_slabs<double>(const double*,
                                                         StackView, void*,
                                                         cudaStream_t);
template cudaError_t launch_tap_sums<float>(StackView, double*, cudaStream_t);
template cudaError_t launch_tap_sums<double>(StackView, double*,
                                             cudaStream_t);

}  // namespace gg
