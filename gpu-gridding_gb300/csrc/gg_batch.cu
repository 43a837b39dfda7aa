// Kernels of the batched (multi-channel) gridding call: many grids -- e.g.
// the frequency channels or snapshots of an observation, each with its own
// number of visibilities -- gridded by one placement pass, one sort and one
// persistent tile-gridding launch.  The reference grids one channel per call
// (main.cpp:243-381 loops over blocks and calls oskar_grid_wproj_f for
// each); a batched call returns, per grid, exactly what that call returns.
//
// Per-grid norm and skip counts are reduced deterministically: every
// visibility's FP64 norm term is stored, chunks of a grid are summed by
// separate blocks in a fixed order, and each grid's chunk sums are then
// added in chunk order.
#include "gg_internal.h"
#include "gg_placement.cuh"

namespace gg {

namespace {

constexpr int kThreads = 256;

template <typename T>
__device__ __forceinline__ T warp_sum(T x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}

template <typename T>
__device__ __forceinline__ T block_sum(T x) {
  __shared__ T s[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  x = warp_sum(x);
  if (lane == 0) s[warp] = x;
  __syncthreads();
  T r = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; ++w) r += s[w];
  __syncthreads();
  return r;  // valid in thread 0
}

template <typename Real>
__global__ void __launch_bounds__(kThreads)
k_place_batched(PlaceParams<Real> p, StackView v, PlaceOut out,
                double* __restrict__ nterm) {
  using R2 = typename Vec2<Real>::type;
  const unsigned long long i =
      (unsigned long long)blockIdx.x * kThreads + threadIdx.x;
  if (i >= p.num_points) return;
  const Placement r = place_one(p, v, i);
  const Real w = p.weight[i];
  R2 vw;
  vw.x = rmul(w, p.vis[2 * i]);
  vw.y = rmul(w, p.vis[2 * i + 1]);
  ((R2*)out.vw)[i] = vw;
  out.cell[i] = pack_cell(r.gu, r.gv);
  out.meta[i] = pack_meta(r.plane, r.ou, r.ov, r.conj_neg, r.skipped);
  double t = 0.0;
  if (!r.skipped) {
    const int side = 2 * v.omax + 1;
    const double ts = v.tap_sum[((size_t)r.plane * side + (r.ou + v.omax)) *
                                    side + (r.ov + v.omax)];
    // oskar_grid_wproj.c:210: *norm += sum * weight_i (FP64).
    t = __dmul_rn(ts, (double)w);
  }
  nterm[i] = t;
}

// New amplitudes and weights on a kept geometry: weighted visibilities and
// FP64 norm terms from the stored placement (meta), no re-placement.
template <typename Real>
__global__ void __launch_bounds__(kThreads)
k_revalue(const Real* __restrict__ vis, const Real* __restrict__ weight,
          const uint32_t* __restrict__ meta, StackView v,
          unsigned long long n, typename Vec2<Real>::type* __restrict__ vw,
          double* __restrict__ nterm) {
  using R2 = typename Vec2<Real>::type;
  const unsigned long long i =
      (unsigned long long)blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const Real w = weight[i];
  R2 o;
  o.x = rmul(w, vis[2 * i]);
  o.y = rmul(w, vis[2 * i + 1]);
  vw[i] = o;
  const uint32_t m = meta[i];
  double t = 0.0;
  if (!meta_skipped(m)) {
    const int side = 2 * v.omax + 1;
    const double ts =
        v.tap_sum[((size_t)meta_plane(m) * side + (meta_ou(m) + v.omax)) *
                      side + (meta_ov(m) + v.omax)];
    t = __dmul_rn(ts, (double)w);
  }
  nterm[i] = t;
}

// One block per chunk of one grid.
__global__ void __launch_bounds__(kThreads)
k_chunk_totals(const uint32_t* __restrict__ meta,
               const double* __restrict__ nterm, StackView v,
               const unsigned long long* __restrict__ chunk_begin,
               double* __restrict__ chunk_norm,
               unsigned long long* __restrict__ chunk_skip,
               unsigned long long* __restrict__ chunk_macs) {
  const int c = blockIdx.x;
  const unsigned long long b = chunk_begin[c], e = chunk_begin[c + 1];
  double n = 0.0;
  unsigned long long skip = 0, macs = 0;
  for (unsigned long long i = b + threadIdx.x; i < e; i += kThreads) {
    const uint32_t m = meta[i];
    if (meta_skipped(m)) {
      ++skip;
    } else {
      const unsigned long long f = 2ull * v.support[meta_plane(m)] + 1;
      macs += f * f;
      n += nterm[i];
    }
  }
  n = block_sum(n);
  skip = block_sum(skip);
  macs = block_sum(macs);
  if (threadIdx.x == 0) {
    chunk_norm[c] = n;
    chunk_skip[c] = skip;
    chunk_macs[c] = macs;
  }
}

// One block: thread g adds grid g's chunks in order; the totals choose the
// tile shape of the call.
__global__ void __launch_bounds__(kThreads)
k_batch_finalize(int num_grids, const int* __restrict__ grid_chunk0,
                 const unsigned long long* __restrict__ chunk_begin,
                 const double* __restrict__ chunk_norm,
                 const unsigned long long* __restrict__ chunk_skip,
                 const unsigned long long* __restrict__ chunk_macs,
                 int forced_shape, int phases, double* d_norm,
                 unsigned long long* d_num_skipped,
                 unsigned long long* d_macs, uint32_t* d_shape) {
  unsigned long long points = 0, skips = 0, macs = 0;
  for (int g = threadIdx.x; g < num_grids; g += kThreads) {
    double n = 0.0;
    unsigned long long sk = 0;
    for (int c = grid_chunk0[g]; c < grid_chunk0[g + 1]; ++c) {
      n += chunk_norm[c];
      sk += chunk_skip[c];
      macs += chunk_macs[c];
      points += chunk_begin[c + 1] - chunk_begin[c];
    }
    d_norm[g] += n;
    d_num_skipped[g] = sk;
    skips += sk;
  }
  points = block_sum(points);
  skips = block_sum(skips);
  macs = block_sum(macs);
  if (threadIdx.x == 0) {
    *d_macs = macs;
    *d_shape = choose_shape(macs, points - skips, forced_shape, phases);
  }
}

}  // namespace

template <typename Real>
cudaError_t launch_place_batched(PlaceParams<Real> p, StackView view,
                                 PlaceOut out, double* nterm, cudaStream_t s) {
  if (p.num_points == 0) return cudaSuccess;
  const unsigned nb = (unsigned)((p.num_points + kThreads - 1) / kThreads);
  k_place_batched<Real><<<nb, kThreads, 0, s>>>(p, view, out, nterm);
  return cudaGetLastError();
}

cudaError_t launch_batch_totals(const uint32_t* meta, const double* nterm,
                                StackView view, int num_chunks,
                                const unsigned long long* chunk_begin,
                                int num_grids, const int* grid_chunk0,
                                double* chunk_norm,
                                unsigned long long* chunk_skip,
                                unsigned long long* chunk_macs,
                                int forced_shape, double* d_norm,
                                unsigned long long* d_num_skipped,
                                unsigned long long* d_macs, uint32_t* d_shape,
                                cudaStream_t s, int phases) {
  if (num_chunks > 0)
    k_chunk_totals<<<num_chunks, kThreads, 0, s>>>(
        meta, nterm, view, chunk_begin, chunk_norm, chunk_skip, chunk_macs);
  k_batch_finalize<<<1, kThreads, 0, s>>>(
      num_grids, grid_chunk0, chunk_begin, chunk_norm, chunk_skip,
      chunk_macs, forced_shape, phases, d_norm, d_num_skipped, d_macs,
      d_shape);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_revalue(const Real* vis, const Real* weight,
                           const uint32_t* meta, StackView view,
                           unsigned long long n, void* vw, double* nterm,
                           cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const unsigned nb = (unsigned)((n + kThreads - 1) / kThreads);
  k_revalue<Real><<<nb, kThreads, 0, s>>>(
      vis, weight, meta, view, n, (typename Vec2<Real>::type*)vw, nterm);
  return cudaGetLastError();
}
template cudaError_t launch_revalue<float>(const float*, const float*,
                                           const uint32_t*, StackView,
                                           unsigned long long, void*, double*,
                                           cudaStream_t);
template cudaError_t launch_revalue<double>(const double*, const double*,
                                            const uint32_t*, StackView,
                                            unsigned long long, void*,
                                            double*, cudaStream_t);

template cudaError_t launch_place_batched<float>(PlaceParams<float>,
                                                 StackView, PlaceOut, double*,
                                                 cudaStream_t);
template cudaError_t launch_place_batched<double>(PlaceParams<double>,
                                                  StackView, PlaceOut,
                                                  double*, cudaStream_t);

}  // namespace gg
