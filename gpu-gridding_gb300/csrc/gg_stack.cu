// Kernel-stack preparation: re-layout of the reference's quadrant cube into
// the residue-split layout of StackView, and the FP64 tap sums used for the
// grid normalisation.
//
// The reference re-packs its kernels on the host on every call
// (compact_wkernels, oskar_grid_wproj_gpu.cu:1461-1643).  Here the re-layout
// runs once per kernel stack on the device and the result is kept in a
// handle.
#include <algorithm>
#include <type_traits>

#include "gg_internal.h"

namespace gg {

namespace {


// One thread per output tap; blockIdx.y is the plane.  Output: for each
// absolute offset class (cu, cv) the (2s+1)^2 slice S[jj][kk] =
// K[|cv + (jj-s)*os|][|cu + (kk-s)*os|] (see StackView).
template <typename Real>
__global__ void k_relayout(const Real* __restrict__ conv, StackView v,
                           typename Vec2<Real>::type* __restrict__ out,
                           const int* changed) {
  using R2 = typename Vec2<Real>::type;
  if (changed && *changed == 0) return;
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
                                 typename Vec2<Real>::type* __restrict__ out,
                                 const int* changed) {
  using R2 = typename Vec2<Real>::type;
  if (changed && *changed == 0) return;
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
                           double* __restrict__ tap_sum, const int* changed) {
  if (changed && *changed == 0) return;
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

// The same sums, one block per plane: loader warps stream the rows of
// nrows consecutive footprint rows j (for every offset class ov the row
// |ov + j*os|, real parts only) into one half of a double-buffered shared
// window while the first threads (one per offset class (ou, ov)) add the
// other half's rows in the reference's (j, k) order.  Bit-identical to
// k_tap_sums; the window is 2 * nrows * side * W values, W = omax + s*os + 1.
template <typename Real>
__global__ void k_tap_sums_rows(const Real* __restrict__ conv, StackView v,
                                double* __restrict__ tap_sum, int sum_threads,
                                int nrows, int W, const int* changed) {
  if (changed && *changed == 0) return;
  extern __shared__ __align__(16) unsigned char tap_rows_raw[];
  Real* win = (Real*)tap_rows_raw;
  // Widest planes (longest addition chains) first: supports grow with
  // the plane index in a w-projection stack.
  const int p = v.num_planes - 1 - (int)blockIdx.x;
  const int omax = v.omax, side = 2 * omax + 1;
  const int os = v.oversample, csh = v.conv_size_half;
  const int s = v.support[p];
  const int nsum = side * side;
  const size_t kstart = (size_t)p * csh * csh;
  const int tid = threadIdx.x;
  const bool summer = tid < sum_threads;
  const int lt = tid - sum_threads, nl = (int)blockDim.x - sum_threads;
  const int half = nrows * side * W;   // values per buffer half
  // Rows of footprint rows j0 .. j0 + nrows - 1 (clipped at s) into half b.
  auto load = [&](int j0, int b) {
    Real* dst = win + (size_t)b * half;
    const int n = min(nrows, s - j0 + 1) * side * W;
    for (int e0 = lt; e0 < n; e0 += 4 * nl) {
      Real x[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int e = e0 + q * nl;
        x[q] = Real(0);
        if (e < n) {
          const int rr = e / W, c = e - rr * W;
          const int jj = rr / side, r = rr - jj * side;
          const int t = abs(r - omax + (j0 + jj) * os);
          if (t < csh && c < csh)
            x[q] = conv[(kstart + (size_t)t * csh + c) * 2];
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (e0 + q * nl < n) dst[e0 + q * nl] = x[q];
    }
  };
  if (!summer) load(-s, 0);
  __syncthreads();
  double sum = 0.0;
  const int ou = tid / side - omax, r = tid % side;
  int b = 0;
  for (int j0 = -s; j0 <= s; j0 += nrows) {
    if (!summer) {
      if (j0 + nrows <= s) load(j0 + nrows, b ^ 1);
    } else if (tid < nsum) {
      const int m = min(nrows, s - j0 + 1);
      for (int jj = 0; jj < m; ++jj) {
        const Real* row = win + (size_t)b * half + ((size_t)jj * side + r) * W;
        for (int k = -s; k <= s; ++k)
          sum = __dadd_rn(sum, (double)row[abs(ou + k * os)]);
      }
    }
    __syncthreads();
    b ^= 1;
  }
  if (tid < nsum) tap_sum[(size_t)p * nsum + tid] = sum;
}

// Copies the square [0, E_p)^2 that the preparation kernels read of each
// plane p (E_p = cube_read_extent) from a cube in host memory that the
// device addresses (page-locked and mapped, or pageable on a device that
// reads pageable memory) to the same place in a device cube.  One warp per
// row at a time, rows taken grid-stride over planes x csh (rows at or past
// E_p skipped): a row's E_p complex taps are contiguous, so a warp's loads
// are coalesced whatever the row pitch, and 4 loads per lane are in flight
// before the stores.  The host link, not the SMs, bounds the copy, so a
// few blocks (about 64k loads in flight) reach its rate and leave the other
// SMs to the kernels that run beside it.
template <typename Real>
__global__ void k_cube_gather(const typename Vec2<Real>::type* __restrict__ src,
                              StackView v,
                              typename Vec2<Real>::type* __restrict__ dst) {
  using R2 = typename Vec2<Real>::type;
  const int lane = threadIdx.x & 31;
  const int csh = v.conv_size_half;
  const long long rows = (long long)v.num_planes * csh;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long f = (long long)blockIdx.x * (blockDim.x >> 5) +
                     (threadIdx.x >> 5);
       f < rows; f += warps) {
    const int p = (int)(f / csh), row = (int)(f - (long long)p * csh);
    const int e = cube_read_extent(v.support[p], v.oversample, v.omax, csh);
    if (row >= e) continue;
    const size_t off = (size_t)f * csh;
    const R2* a = src + off;
    R2* b = dst + off;
    for (int c = lane; c < e; c += 128) {
      R2 t[4];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (c + 32 * q < e) t[q] = a[c + 32 * q];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (c + 32 * q < e) b[c + 32 * q] = t[q];
    }
  }
}

// *changed = 1 if the read squares of two cubes differ in any bit (the
// squares k_cube_gather copies; same launch shape).
template <typename Real>
__global__ void k_cube_compare(const typename Vec2<Real>::type* __restrict__ a,
                               const typename Vec2<Real>::type* __restrict__ b,
                               StackView v, int* changed) {
  using W = typename std::conditional<sizeof(Real) == 4, unsigned long long,
                                      ulonglong2>::type;
  const int p = blockIdx.x;
  const int row = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const int csh = v.conv_size_half;
  const int e = cube_read_extent(v.support[p], v.oversample, v.omax, csh);
  if (row >= e) return;
  const size_t off = ((size_t)p * csh + row) * csh;
  const W* x = (const W*)(a + off);
  const W* y = (const W*)(b + off);
  bool diff = false;
  for (int c = lane; c < e; c += 32) {
    const W u = x[c], w = y[c];
    if constexpr (sizeof(Real) == 4) diff |= u != w;
    else diff |= (u.x != w.x) | (u.y != w.y);
  }
  if (__any_sync(0xffffffffu, diff) && lane == 0) *changed = 1;
}

}  // namespace

template <typename Real>
cudaError_t launch_cube_compare(const Real* a, const Real* b, StackView view,
                                int* changed, cudaStream_t s) {
  if (view.num_planes <= 0) return cudaSuccess;
  dim3 grid(view.num_planes, (view.conv_size_half + 7) / 8);
  using R2 = typename Vec2<Real>::type;
  k_cube_compare<Real><<<grid, 256, 0, s>>>((const R2*)a, (const R2*)b, view,
                                            changed);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_cube_gather(const Real* src, StackView view, Real* dst,
                               cudaStream_t s) {
  if (view.num_planes <= 0) return cudaSuccess;
  using R2 = typename Vec2<Real>::type;
  k_cube_gather<Real><<<16, 1024, 0, s>>>((const R2*)src, view, (R2*)dst);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_stack_relayout(const Real* d_conv_func, StackView view,
                                  void* d_taps_out, long long total_taps,
                                  cudaStream_t s, const int* changed) {
  (void)total_taps;
  dim3 grid(64, view.num_planes);
  k_relayout<Real><<<grid, 256, 0, s>>>(
      d_conv_func, view, (typename Vec2<Real>::type*)d_taps_out, changed);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_stack_relayout_slabs(const Real* d_conv_func,
                                        StackView view, void* d_out,
                                        cudaStream_t s, const int* changed) {
  dim3 grid(64, view.num_planes);
  k_relayout_slabs<Real><<<grid, 256, 0, s>>>(
      d_conv_func, view, (typename Vec2<Real>::type*)d_out, changed);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_tap_sums(StackView view, double* d_tap_sum,
                            int support_max, cudaStream_t s,
                            const int* changed) {
  // The raw cube is needed for the reference-order sums; it is passed in
  // view.taps by the caller for this launch only.
  const int side = 2 * view.omax + 1;
  const int nsum = side * side;
  // Row window of the block-per-plane kernel: up to 8 footprint rows per
  // half, within the default 48 KB of shared memory.
  const long long W = view.omax + (long long)support_max * view.oversample + 1;
  const long long per_row = (long long)side * W * (long long)sizeof(Real);
  const int nrows = (int)std::min<long long>(8, (48 << 10) / (2 * per_row));
  const int sum_threads = (nsum + 31) / 32 * 32;
  if (nrows >= 1 && sum_threads + 256 <= 1024) {
    const size_t smem = (size_t)2 * nrows * per_row;
    k_tap_sums_rows<Real><<<view.num_planes, sum_threads + 256, smem, s>>>(
        (const Real*)view.taps, view, d_tap_sum, sum_threads, nrows, (int)W,
        changed);
    return cudaGetLastError();
  }
  const int n = view.num_planes * nsum;
  k_tap_sums<Real><<<(n + 127) / 128, 128, 0, s>>>(
      (const Real*)view.taps, view, d_tap_sum, changed);
  return cudaGetLastError();
}

template cudaError_t launch_stack_relayout<float>(const float*, StackView,
                                                  void*, long long,
                                                  cudaStream_t, const int*);
template cudaError_t launch_stack_relayout<double>(const double*, StackView,
                                                   void*, long long,
                                                   cudaStream_t, const int*);
template cudaError_t launch_stack_relayout_slabs<float>(const float*,
                                                        StackView, void*,
                                                        cudaStream_t,
                                                        const int*);
template cudaError_t launch_stack_relayout_slabs<double>(const double*,
                                                         StackView, void*,
                                                         cudaStream_t,
                                                         const int*);
template cudaError_t launch_cube_compare<float>(const float*, const float*,
                                                StackView, int*, cudaStream_t);
template cudaError_t launch_cube_compare<double>(const double*, const double*,
                                                 StackView, int*,
                                                 cudaStream_t);
template cudaError_t launch_cube_gather<float>(const float*, StackView,
                                               float*, cudaStream_t);
template cudaError_t launch_cube_gather<double>(const double*, StackView,
                                                double*, cudaStream_t);
template cudaError_t launch_tap_sums<float>(StackView, double*, int,
                                            cudaStream_t, const int*);
template cudaError_t launch_tap_sums<double>(StackView, double*, int,
                                             cudaStream_t, const int*);

}  // namespace gg
