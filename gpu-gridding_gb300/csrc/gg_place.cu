// Placement of visibilities on the grid, per-visibility norm and skip
// accounting, and emission of (tile, visibility) records for binning.
//
// Placement reproduces the reference's arithmetic exactly
// (oskar_grid_wproj.c:146-187 for FP32, :57-98 for FP64): every product,
// difference, square root and rounding is an explicitly rounded IEEE
// operation (no contraction), so the cell, offset, plane and skip decisions
// are bit-identical to the serial code for finite inputs.
#include "gg_internal.h"
#include "gg_placement.cuh"

namespace gg {

namespace {

constexpr int kPlaceThreads = kPlaceBlock;

template <typename T>
__device__ __forceinline__ T warp_sum(T x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}

template <typename Real>
__global__ void __launch_bounds__(kPlaceThreads)
k_place(PlaceParams<Real> p, StackView v, TileGeom g, PlaceOut out) {
  using R2 = typename Vec2<Real>::type;
  const unsigned long long i =
      (unsigned long long)blockIdx.x * kPlaceThreads + threadIdx.x;
  double norm = 0.0;
  unsigned long long skip = 0, macs = 0;
  if (i < p.num_points) {
    const Placement r = place_one(p, v, i);
    // Degridding places coordinates only (no visibilities, weights, norm).
    const Real w = p.weight ? p.weight[i] : (Real)0;
    if (p.vis) {
      R2 vw;
      vw.x = rmul(w, p.vis[2 * i]);
      vw.y = rmul(w, p.vis[2 * i + 1]);
      ((R2*)out.vw)[i] = vw;
    }
    out.cell[i] = pack_cell(r.gu, r.gv);
    out.meta[i] = pack_meta(r.plane, r.ou, r.ov, r.conj_neg, r.skipped);
    if (r.skipped) {
      skip = 1;
    } else {
      const int s = r.support;
      const unsigned long long f = 2ull * s + 1;
      macs = f * f;
      const int side = 2 * v.omax + 1;
      const double ts =
          p.defer_norm ? 0.0
                       : v.tap_sum[((size_t)r.plane * side + (r.ou + v.omax)) *
                                       side + (r.ov + v.omax)];
      // oskar_grid_wproj.c:210: *norm += sum * weight_i (FP64).
      if (p.weight && !p.defer_norm) norm = __dmul_rn(ts, (double)w);
    }
  }
  // Block reductions by warp shuffles, then one partial per block; the
  // partials are summed in block order by k_place_finalize, so the norm is
  // the same on every run.
  __shared__ double s_norm[kPlaceThreads / 32];
  __shared__ unsigned long long s_skip[kPlaceThreads / 32];
  __shared__ unsigned long long s_macs[kPlaceThreads / 32];
  norm = warp_sum(norm);
  skip = warp_sum(skip);
  macs = warp_sum(macs);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { s_norm[warp] = norm; s_skip[warp] = skip; s_macs[warp] = macs; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double bn = 0.0;
    unsigned long long bs = 0, bm = 0;
    for (int w = 0; w < kPlaceThreads / 32; ++w) {
      bn += s_norm[w]; bs += s_skip[w]; bm += s_macs[w];
    }
    out.blk_norm[blockIdx.x] = bn;
    out.blk_skip[blockIdx.x] = bs;
    out.blk_macs[blockIdx.x] = bm;
  }
}

// The norm terms of a placement made with defer_norm: the same per-point
// products and the same block reduction as k_place, so blk_norm is
// bit-identical to what k_place would have written.
template <typename Real>
__global__ void __launch_bounds__(kPlaceThreads)
k_norm_terms(const uint32_t* __restrict__ meta, const Real* __restrict__ weight,
             unsigned long long n, StackView v, double* __restrict__ blk_norm) {
  const unsigned long long i =
      (unsigned long long)blockIdx.x * kPlaceThreads + threadIdx.x;
  double norm = 0.0;
  if (i < n) {
    const uint32_t m = meta[i];
    if (!meta_skipped(m)) {
      const int side = 2 * v.omax + 1;
      const double ts = v.tap_sum[((size_t)meta_plane(m) * side +
                                   (meta_ou(m) + v.omax)) * side +
                                  (meta_ov(m) + v.omax)];
      norm = __dmul_rn(ts, (double)weight[i]);
    }
  }
  __shared__ double s_norm[kPlaceThreads / 32];
  norm = warp_sum(norm);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) s_norm[warp] = norm;
  __syncthreads();
  if (threadIdx.x == 0) {
    double bn = 0.0;
    for (int w = 0; w < kPlaceThreads / 32; ++w) bn += s_norm[w];
    blk_norm[blockIdx.x] = bn;
  }
}

__global__ void k_place_finalize(const double* __restrict__ blk_norm,
                                 const unsigned long long* __restrict__ blk_skip,
                                 const unsigned long long* __restrict__ blk_macs,
                                 int num_blocks, unsigned long long n_points,
                                 int forced_shape, int phases,
                                 double* d_norm,
                                 unsigned long long* d_num_skipped,
                                 unsigned long long* d_macs,
                                 uint32_t* d_shape) {
  // One block; thread t sums blocks t, t+blockDim, ... in order, then a
  // fixed-shape shuffle and shared-memory tree: the same association on
  // every run, so the norm is deterministic.
  __shared__ double s_n[32];
  __shared__ unsigned long long s_s[32], s_m[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double n = 0.0;
  unsigned long long s = 0, m = 0;
  for (int b = threadIdx.x; b < num_blocks; b += blockDim.x) {
    n += blk_norm[b];
    if (blk_skip) s += blk_skip[b];
    if (blk_macs) m += blk_macs[b];
  }
  n = warp_sum(n); s = warp_sum(s); m = warp_sum(m);
  if (lane == 0) { s_n[warp] = n; s_s[warp] = s; s_m[warp] = m; }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    n = lane < nw ? s_n[lane] : 0.0;
    s = lane < nw ? s_s[lane] : 0ull;
    m = lane < nw ? s_m[lane] : 0ull;
    n = warp_sum(n); s = warp_sum(s); m = warp_sum(m);
    if (lane == 0) {
      if (d_norm) *d_norm += n;
      if (d_num_skipped) *d_num_skipped = s;
      if (d_macs) *d_macs = m;
      if (d_shape)
        *d_shape = choose_shape(m, n_points - s, forced_shape, phases);
    }
  }
}

// Records per visibility: tiles of the chosen shape its footprint touches
// (on its tile phase, see footprint_phase).
__global__ void k_count(const uint32_t* __restrict__ cell,
                        const uint32_t* __restrict__ meta,
                        unsigned long long n, StackView v,
                        const uint32_t* __restrict__ d_shape,
                        uint32_t* __restrict__ count) {
  const unsigned long long i =
      (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t m = meta[i];
  uint32_t c = 0;
  if (!meta_skipped(m)) {
    const uint32_t word = *d_shape;
    const int shape = (int)(word & 0xFFu), phases = phases_of_shape(word);
    // Tiles are 32 >> shape by 64 << shape cells, phase strips
    // (32 >> shape) / phases columns: divisions become shifts.
    const int tws = 5 - shape, ths = 6 + shape;
    const int sws = tws - (phases >= 8 ? 3 : phases >= 4 ? 2 : phases >= 2);
    const uint32_t ce = cell[i];
    const int gu = cell_u(ce), gv = cell_v(ce);
    const int s = v.support[meta_plane(m)];
    const int sh = phases > 1
                       ? footprint_phase(gu - s, gu + s, tws, sws, phases)
                             << sws
                       : 0;
    c = (uint32_t)((((gu + s + sh) >> tws) - ((gu - s + sh) >> tws) + 1) *
                   (((gv + s) >> ths) - ((gv - s) >> ths) + 1));
  }
  count[i] = c;
}

// One thread per visibility writes one record per tile its footprint
// touches.  Key = (tile, plane, |offset| class) so that after the sort each
// tile's records are contiguous and grouped by kernel slice; value = the
// visibility index.
__global__ void k_emit(const uint32_t* __restrict__ cell,
                       const uint32_t* __restrict__ meta,
                       const uint32_t* __restrict__ rec_offset,
                       unsigned long long n, StackView v, TileGeom g,
                       int grid_index, unsigned long long vis_offset,
                       uint32_t* __restrict__ keys,
                       uint32_t* __restrict__ vals,
                       const unsigned long long* __restrict__ grid_offsets,
                       int num_grids) {
  const unsigned long long i =
      (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t m = meta[i];
  if (meta_skipped(m)) return;
  if (grid_offsets) {
    // Batched call: the grid of visibility i is the channel whose range
    // [grid_offsets[g], grid_offsets[g+1]) holds it.
    int lo = 0, hi = num_grids - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (grid_offsets[mid] <= i) lo = mid; else hi = mid - 1;
    }
    grid_index = lo;
  }
  const uint32_t c = cell[i];
  const int gu = cell_u(c), gv = cell_v(c);
  const int plane = meta_plane(m);
  const int s = v.support[plane];
  // Tile sides and strips are powers of two: shifts, not divisions.
  const int tws = __ffs(g.tile_u) - 1, ths = __ffs(g.tile_v) - 1;
  const int phase = g.tile_phases > 1
                        ? footprint_phase(gu - s, gu + s, tws, g.strip_shift,
                                          g.tile_phases)
                        : 0;
  const int sh = phase << g.strip_shift;
  const int tu0 = (gu - s + sh) >> tws, tu1 = (gu + s + sh) >> tws;
  const int tv0 = (gv - s) >> ths, tv1 = (gv + s) >> ths;
  const int au = abs(meta_ou(m)), av = abs(meta_ov(m));
  uint32_t low = 0;
  if (g.phase_bits > 0) low = (uint32_t)(au * (v.omax + 1) + av);
  if (g.plane_bits > 0) low |= (uint32_t)plane << g.phase_bits;
  const int low_bits = g.plane_bits + g.phase_bits;
  const uint32_t tiles_per_grid = (uint32_t)g.tiles_u * (uint32_t)g.tiles_v;
  uint32_t pos = rec_offset[i];
  const uint32_t vid = (uint32_t)(vis_offset + i);
  for (int tv = tv0; tv <= tv1; ++tv) {
    for (int tu = tu0; tu <= tu1; ++tu) {
      uint32_t tile = (uint32_t)grid_index * tiles_per_grid +
                      (uint32_t)tv * g.tiles_u + (uint32_t)tu;
      if (g.num_groups > 1) {
        uint32_t group = g.plane_group ? (uint32_t)g.plane_group[plane] : 0u;
        if (g.split_tv > 0) {
          const uint32_t lower = tv >= g.split_tv ? 1u : 0u;
          const int base_groups =
              g.num_groups / (g.tile_phases > 1 ? g.tile_phases : 1);
          const uint32_t last = (uint32_t)(base_groups - 1 -
                                           __popc((unsigned)g.split_mask));
          uint32_t v = group;
          if (g.split_mask & 1) v = group == 0 ? lower : group + 1;
          if ((g.split_mask & 2) && group == last) v += lower;
          group = v;
        }
        if (g.tile_phases > 1)
          group = group * (uint32_t)g.tile_phases + (uint32_t)phase;
        tile += group * (uint32_t)g.tiles_total;
      }
      keys[pos] = low_bits >= 32 ? low : ((tile << low_bits) | low);
      vals[pos] = vid;
      ++pos;
    }
  }
}

// Diagnostic: per-visibility placement as the gridder computes it, as six
// int32 per visibility (cell u, cell v, off_u, off_v, plane, flags) with
// flags bit 0 = skipped, bit 1 = kernel conjugated (ww > 0).
template <typename Real>
__global__ void k_place_only(PlaceParams<Real> p, StackView v,
                             int* __restrict__ out) {
  const unsigned long long i =
      (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.num_points) return;
  const Placement r = place_one(p, v, i);
  int* o = out + 6 * i;
  o[0] = r.gu; o[1] = r.gv; o[2] = r.ou; o[3] = r.ov; o[4] = r.plane;
  o[5] = r.skipped | (r.conj_neg << 1);
}

}  // namespace

template <typename Real>
cudaError_t launch_place_only(PlaceParams<Real> p, StackView view, int* out,
                              cudaStream_t s) {
  if (p.num_points == 0) return cudaSuccess;
  const unsigned nb = (unsigned)((p.num_points + 255) / 256);
  k_place_only<Real><<<nb, 256, 0, s>>>(p, view, out);
  return cudaGetLastError();
}
template cudaError_t launch_place_only<float>(PlaceParams<float>, StackView,
                                              int*, cudaStream_t);
template cudaError_t launch_place_only<double>(PlaceParams<double>, StackView,
                                               int*, cudaStream_t);

int place_num_blocks(unsigned long long n) {
  unsigned long long nb = (n + kPlaceThreads - 1) / kPlaceThreads;
  return (int)(nb == 0 ? 1 : nb);
}

template <typename Real>
cudaError_t launch_place(PlaceParams<Real> p, StackView view, TileGeom geom,
                         int grid_index, unsigned long long vis_offset,
                         PlaceOut out, cudaStream_t s) {
  (void)grid_index; (void)vis_offset;
  const int nb = place_num_blocks(p.num_points);
  k_place<Real><<<nb, kPlaceThreads, 0, s>>>(p, view, geom, out);
  return cudaGetLastError();
}

cudaError_t launch_place_finalize(const double* blk_norm,
                                  const unsigned long long* blk_skip,
                                  const unsigned long long* blk_macs,
                                  int num_blocks, unsigned long long n,
                                  int forced_shape, double* d_norm,
                                  unsigned long long* d_num_skipped,
                                  unsigned long long* d_macs,
                                  uint32_t* d_shape, cudaStream_t s,
                                  int phases) {
  k_place_finalize<<<1, 1024, 0, s>>>(blk_norm, blk_skip, blk_macs,
                                      num_blocks, n, forced_shape, phases,
                                      d_norm, d_num_skipped, d_macs, d_shape);
  return cudaGetLastError();
}

__global__ void k_store_f64(double* p, double v) { *p = v; }

cudaError_t launch_store_f64(double* p, double v, cudaStream_t s) {
  k_store_f64<<<1, 1, 0, s>>>(p, v);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_norm_terms(const uint32_t* meta, const Real* weight,
                              unsigned long long n, StackView view,
                              double* blk_norm, double* d_norm,
                              cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int nb = place_num_blocks(n);
  k_norm_terms<Real><<<nb, kPlaceThreads, 0, s>>>(meta, weight, n, view,
                                                 blk_norm);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_place_finalize<<<1, 1024, 0, s>>>(blk_norm, nullptr, nullptr, nb, n, 0,
                                      1, d_norm, nullptr, nullptr, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_count_records(const uint32_t* cell, const uint32_t* meta,
                                 unsigned long long n, StackView view,
                                 const uint32_t* d_shape, uint32_t* count,
                                 cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_count<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(cell, meta, n, view,
                                                     d_shape, count);
  return cudaGetLastError();
}

cudaError_t launch_emit_records(const uint32_t* cell, const uint32_t* meta,
                                const uint32_t* rec_offset,
                                unsigned long long n, StackView view,
                                TileGeom geom, int grid_index,
                                unsigned long long vis_offset, uint32_t* keys,
                                uint32_t* vals, cudaStream_t s,
                                const unsigned long long* grid_offsets,
                                int num_grids) {
  if (n == 0) return cudaSuccess;
  const unsigned nb = (unsigned)((n + 255) / 256);
  k_emit<<<nb, 256, 0, s>>>(cell, meta, rec_offset, n, view, geom,
                            grid_index, vis_offset, keys, vals, grid_offsets,
                            num_grids);
  return cudaGetLastError();
}

template cudaError_t launch_norm_terms<float>(const uint32_t*, const float*,
                                              unsigned long long, StackView,
                                              double*, double*, cudaStream_t);
template cudaError_t launch_norm_terms<double>(const uint32_t*, const double*,
                                               unsigned long long, StackView,
                                               double*, double*, cudaStream_t);
template cudaError_t launch_place<float>(PlaceParams<float>, StackView,
                                         TileGeom, int, unsigned long long,
                                         PlaceOut, cudaStream_t);
template cudaError_t launch_place<double>(PlaceParams<double>, StackView,
                                          TileGeom, int, unsigned long long,
                                          PlaceOut, cudaStream_t);

}  // namespace gg
