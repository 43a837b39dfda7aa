// Tile-owning gridding.
//
// The grid is cut into tiles of 32 (u) x TV (v) cells.  After the sort each
// tile's (visibility, tile) records are contiguous; a tile's record range is
// cut into work items of at most `chunk` records.  A persistent CTA takes
// work items from a queue and keeps the item's whole tile in registers: lane
// l of warp w owns column l and rows w*WROWS .. w*WROWS+WROWS-1.  For every
// record each warp multiplies the visibility by the kernel taps of its own
// rows and columns and accumulates -- no atomics, no shared-memory
// read-modify-write.  A tile with one item is then added to the grid in
// place with one coalesced read-modify-write; a tile split over several
// items writes one partial tile per item and k_reduce_partials adds them to
// the grid in item order, so the result does not depend on scheduling.
//
// The reference's equivalent is oskar_process_tiles_dynamic
// (oskar_grid_wproj_gpu.cu:840-1309), a one-warp-per-32x16-tile kernel that
// flushes with float atomics whenever its tile changes.
//
// FP32 accumulation is compensated: each batch of records is summed in
// plain FP32 FMA, then folded into a (hi, lo) pair by Knuth's TwoSum, so
// rounding error does not grow with the number of visibilities on a cell.
#include <algorithm>
#include <type_traits>

#include "gg_internal.h"

namespace gg {

namespace {


constexpr int kTU = 32;      // tile width = warp width
constexpr int kWRows = 8;    // rows per warp
constexpr int kWarps = 8;    // warps per CTA
constexpr int kTV = kWRows * kWarps;
constexpr int kThreads = kWarps * 32;
constexpr int kBatch = kThreads;   // records staged per round

// Visibility coefficients of one record with the conjugation folded in:
// re += a*t.re + b*t.im, im += c*t.re + d*t.im.
template <typename Real>
struct alignas(4 * sizeof(Real)) Coef {
  Real a, b, c, d;
};

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

template <typename Real>
struct GridArgs {
  const WorkItem* items;
  const uint32_t* num_items;
  uint32_t* counter;
  const uint32_t* rec_vis;
  const uint32_t* cell;
  const uint32_t* meta;
  const typename Vec2<Real>::type* vw;
  StackView view;
  TileGeom geom;
  int grid_size;
  Real* grid;
  long long grid_stride;
  typename Vec2<Real>::type* partials;
};

// Per-record data staged in shared memory once per CTA (the first kBatch
// threads each prepare one record), then read by every warp with broadcast
// loads.
struct RecGeo {           // int4
  int gu_t, gv_t;         // cell of the visibility relative to the tile
  int s, F;               // support and slice side 2s+1
};
struct RecAddr {          // int4
  int slice;              // first tap of the (plane, |offset|) slice
  int su, sv;             // mirror signs of the slice (offset signs)
  int pad;
};

// Loads the kWRows taps of one record for this warp's rows into t[]; taps
// outside the footprint (rows or lanes) are zero, so the multiply-adds that
// follow need no predicates.
template <typename R2>
__device__ __forceinline__ void load_record_taps(
    const R2* __restrict__ taps, const RecGeo g, const RecAddr ad, int lane,
    int row0, R2 (&t)[kWRows]) {
  const int k = lane - g.gu_t;
  const bool act = (unsigned)(k + g.s) <= (unsigned)(2 * g.s);
  const int rlo = max(0, g.gv_t - g.s - row0);
  const int rhi = min(kWRows - 1, g.gv_t + g.s - row0);
  const int rstep = ad.sv * g.F;
  // Slice row of register row 0; columns mirrored by su.
  const R2* __restrict__ p = taps + ad.slice +
                             (g.s + ad.sv * (row0 - g.gv_t)) * g.F +
                             (g.s + ad.su * k);
#pragma unroll
  for (int r = 0; r < kWRows; ++r) {
    t[r].x = 0;
    t[r].y = 0;
    if (r >= rlo && r <= rhi && act) t[r] = __ldg(p + r * rstep);
  }
}

template <typename Real, typename R2>
__device__ __forceinline__ void mac_record(R2 (&acc)[kWRows],
                                           const R2 (&t)[kWRows],
                                           const Coef<Real> cf) {
#pragma unroll
  for (int r = 0; r < kWRows; ++r) {
    acc[r].x = fma(cf.b, t[r].y, fma(cf.a, t[r].x, acc[r].x));
    acc[r].y = fma(cf.d, t[r].y, fma(cf.c, t[r].x, acc[r].y));
  }
}

template <typename Real, bool kCompensate>
__global__ void __launch_bounds__(kThreads, sizeof(Real) == 4 ? 3 : 2)
k_grid_tiles(GridArgs<Real> a) {
  using R2 = typename Vec2<Real>::type;
  __shared__ int4 s_geo[kBatch];
  __shared__ Coef<Real> s_coef[kBatch];
  __shared__ int4 s_addr[kBatch];
  // Compensated running sums (hi, lo) of each thread's cells: the register
  // accumulators hold one batch at a time and are folded in after it.
  __shared__ R2 s_hi[kCompensate ? kWRows : 1][kThreads];
  __shared__ R2 s_lo[kCompensate ? kWRows : 1][kThreads];
  __shared__ int s_item;

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int row0 = warp * kWRows;
  const int G = a.grid_size;
  const int omax = a.view.omax;
  const R2* __restrict__ taps = (const R2*)a.view.taps;
  const int tiles_per_grid = a.geom.tiles_u * a.geom.tiles_v;

  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(a.counter, 1u);
    __syncthreads();
    const int it = s_item;
    if (it >= (int)*a.num_items) break;
    const WorkItem item = a.items[it];
    const int gi = item.tile / tiles_per_grid;
    const int tl = item.tile - gi * tiles_per_grid;
    const int u0 = (tl % a.geom.tiles_u) * kTU;
    const int v0 = (tl / a.geom.tiles_u) * kTV;

    R2 acc[kWRows];
#pragma unroll
    for (int r = 0; r < kWRows; ++r) {
      acc[r].x = acc[r].y = 0;
      if constexpr (kCompensate) {
        s_hi[r][threadIdx.x] = acc[r];
        s_lo[r][threadIdx.x] = acc[r];
      }
    }

    for (int b0 = item.rec_begin; b0 < item.rec_end; b0 += kBatch) {
      const int nb = min(kBatch, item.rec_end - b0);
      // ---- stage the batch's records ------------------------------------
      if (threadIdx.x < nb) {
        const uint32_t vid = a.rec_vis[b0 + threadIdx.x];
        const uint32_t c = a.cell[vid], m = a.meta[vid];
        const R2 v = a.vw[vid];
        const int plane = meta_plane(m);
        const int ou = meta_ou(m), ov = meta_ov(m);
        const int s = a.view.support[plane];
        int4 geo;
        geo.x = cell_u(c) - u0;
        geo.y = cell_v(c) - v0;
        geo.z = s;
        geo.w = 2 * s + 1;
        Coef<Real> cf;
        cf.a = v.x;
        cf.c = v.y;
        if (meta_conj(m)) { cf.b = v.y; cf.d = -v.x; }
        else { cf.b = -v.y; cf.d = v.x; }
        int4 ad;
        ad.x = (int)slice_offset(a.view.base[plane], s, omax, abs(ou),
                                 abs(ov));
        ad.y = ou < 0 ? -1 : 1;
        ad.z = ov < 0 ? -1 : 1;
        ad.w = 0;
        s_geo[threadIdx.x] = geo;
        s_coef[threadIdx.x] = cf;
        s_addr[threadIdx.x] = ad;
      }
      __syncthreads();
      // ---- this warp's records: those whose footprint meets its rows ----
      for (int c0 = 0; c0 < nb; c0 += 32) {
        bool touch = false;
        if (c0 + lane < nb) {
          const int4 g = s_geo[c0 + lane];
          touch = (g.y - g.z <= row0 + kWRows - 1) && (g.y + g.z >= row0);
        }
        uint32_t m = __ballot_sync(0xffffffffu, touch);
        // Two records at a time: 2*kWRows tap loads in flight per warp.
        while (m) {
          const int tA = c0 + __ffs(m) - 1;
          m &= m - 1;
          const int tB = m ? c0 + __ffs(m) - 1 : -1;
          if (m) m &= m - 1;
          R2 ta[kWRows], tb[kWRows];
          const int4 gA = s_geo[tA];
          const int4 aA = s_addr[tA];
          load_record_taps(taps, RecGeo{gA.x, gA.y, gA.z, gA.w},
                           RecAddr{aA.x, aA.y, aA.z, aA.w}, lane, row0, ta);
          if (tB >= 0) {
            const int4 gB = s_geo[tB];
            const int4 aB = s_addr[tB];
            load_record_taps(taps, RecGeo{gB.x, gB.y, gB.z, gB.w},
                             RecAddr{aB.x, aB.y, aB.z, aB.w}, lane, row0, tb);
          }
          mac_record<Real>(acc, ta, s_coef[tA]);
          if (tB >= 0) mac_record<Real>(acc, tb, s_coef[tB]);
        }
      }
      if constexpr (kCompensate) {
#pragma unroll
        for (int r = 0; r < kWRows; ++r) {
          R2 hi = s_hi[r][threadIdx.x], lo = s_lo[r][threadIdx.x];
          float s, e;
          two_sum(hi.x, acc[r].x, s, e); hi.x = s; lo.x += e;
          two_sum(hi.y, acc[r].y, s, e); hi.y = s; lo.y += e;
          s_hi[r][threadIdx.x] = hi;
          s_lo[r][threadIdx.x] = lo;
          acc[r].x = acc[r].y = 0;
        }
      }
      __syncthreads();
    }
    // ---- flush ------------------------------------------------------------
    R2 out[kWRows];
#pragma unroll
    for (int r = 0; r < kWRows; ++r) {
      if constexpr (kCompensate) {
        const R2 hi = s_hi[r][threadIdx.x], lo = s_lo[r][threadIdx.x];
        out[r].x = hi.x + lo.x;
        out[r].y = hi.y + lo.y;
      } else {
        out[r] = acc[r];
      }
    }
    const int col = u0 + lane;
    if (item.slot < 0) {
      R2* g = (R2*)(a.grid + (long long)gi * a.grid_stride);
#pragma unroll
      for (int r = 0; r < kWRows; ++r) {
        const int row = v0 + row0 + r;
        if (row < G && col < G) {
          R2* p = g + (size_t)row * G + col;
          R2 old = *p;
          old.x += out[r].x;
          old.y += out[r].y;
          *p = old;
        }
      }
    } else {
      R2* p = a.partials + (size_t)item.slot * (kTU * kTV);
#pragma unroll
      for (int r = 0; r < kWRows; ++r) p[(row0 + r) * kTU + lane] = out[r];
    }
  }
}

template <typename Real>
__global__ void k_reduce_partials(const int4* __restrict__ split_tiles,
                                  const uint32_t* __restrict__ num_split,
                                  const typename Vec2<Real>::type* __restrict__ partials,
                                  TileGeom g, int G, Real* grid,
                                  long long grid_stride) {
  using R2 = typename Vec2<Real>::type;
  const int tiles_per_grid = g.tiles_u * g.tiles_v;
  const int n = (int)*num_split;
  for (int st = blockIdx.x; st < n; st += gridDim.x) {
    const int4 d = split_tiles[st];  // tile, first slot, chunks
    const int gi = d.x / tiles_per_grid;
    const int tl = d.x - gi * tiles_per_grid;
    const int u0 = (tl % g.tiles_u) * kTU;
    const int v0 = (tl / g.tiles_u) * kTV;
    R2* gp = (R2*)(grid + (long long)gi * grid_stride);
    for (int cellix = threadIdx.x; cellix < kTU * kTV; cellix += blockDim.x) {
      const int row = v0 + cellix / kTU, col = u0 + cellix % kTU;
      if (row >= G || col >= G) continue;
      R2* p = gp + (size_t)row * G + col;
      const R2 old = *p;
      double sx = old.x, sy = old.y;
      for (int c = 0; c < d.z; ++c) {
        const R2 q = partials[(size_t)(d.y + c) * (kTU * kTV) + cellix];
        sx += q.x;
        sy += q.y;
      }
      R2 nw;
      nw.x = (Real)sx;
      nw.y = (Real)sy;
      *p = nw;
    }
  }
}

__global__ void k_tile_bounds(const uint32_t* __restrict__ keys, uint32_t n,
                              int shift, int num_tiles,
                              uint32_t* __restrict__ tile_start) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
       i <= (long long)n; i += (long long)gridDim.x * blockDim.x) {
    const long long cur = i < n ? (long long)(keys[i] >> shift) : num_tiles;
    const long long prev = i == 0 ? -1 : (long long)(keys[i - 1] >> shift);
    for (long long x = prev + 1; x <= cur; ++x) tile_start[x] = (uint32_t)i;
  }
}

// A[t] = chunks of tile t if it is split (more than one chunk), else 0;
// B[t] = 1 if tile t has exactly one chunk.
__global__ void k_item_counts(const uint32_t* __restrict__ tile_start,
                              int num_tiles, uint32_t chunk,
                              uint32_t* __restrict__ A,
                              uint32_t* __restrict__ B) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= num_tiles) return;
  const uint32_t c = tile_start[t + 1] - tile_start[t];
  const uint32_t chunks = (c + chunk - 1) / chunk;
  A[t] = chunks > 1 ? chunks : 0;
  B[t] = chunks == 1 ? 1 : 0;
}

// Split-tile chunks come first in the queue (they are the largest items),
// then the single-chunk tiles.  Partial slot = queue position of the chunk.
__global__ void k_item_emit(const uint32_t* __restrict__ tile_start,
                            int num_tiles, uint32_t chunk,
                            const uint32_t* __restrict__ sA,
                            const uint32_t* __restrict__ sB,
                            const uint32_t* __restrict__ totA,
                            const uint32_t* __restrict__ totB,
                            WorkItem* __restrict__ items,
                            int4* __restrict__ split_tiles,
                            uint32_t* __restrict__ num_split,
                            uint32_t* __restrict__ num_items) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) *num_items = *totA + *totB;
  if (t >= num_tiles) return;
  const uint32_t s0 = tile_start[t], s1 = tile_start[t + 1];
  const uint32_t c = s1 - s0;
  if (c == 0) return;
  const uint32_t chunks = (c + chunk - 1) / chunk;
  if (chunks == 1) {
    WorkItem w;
    w.tile = t; w.rec_begin = (int)s0; w.rec_end = (int)s1; w.slot = -1;
    items[*totA + sB[t]] = w;
  } else {
    const uint32_t first = sA[t];
    for (uint32_t j = 0; j < chunks; ++j) {
      WorkItem w;
      w.tile = t;
      w.rec_begin = (int)(s0 + j * chunk);
      w.rec_end = (int)min(s1, s0 + (j + 1) * chunk);
      w.slot = (int)(first + j);
      items[first + j] = w;
    }
    const uint32_t k = atomicAdd(num_split, 1u);
    split_tiles[k] = make_int4(t, (int)first, (int)chunks, 0);
  }
}

}  // namespace

cudaError_t launch_tile_bounds(const uint32_t* keys, uint32_t n, int shift,
                               int num_tiles, uint32_t* tile_start,
                               cudaStream_t s) {
  const long long work = (long long)n + 1;
  const int blocks = (int)std::min<long long>((work + 255) / 256, 65536);
  k_tile_bounds<<<blocks, 256, 0, s>>>(keys, n, shift, num_tiles, tile_start);
  return cudaGetLastError();
}

cudaError_t launch_build_items(const uint32_t* tile_start, int num_tiles,
                               uint32_t num_records, uint32_t chunk,
                               ItemBuffers b, cudaStream_t s) {
  (void)num_records;
  uint32_t* A = b.chunks;
  uint32_t* B = b.split_chunks;
  const int blocks = (num_tiles + 255) / 256;
  k_item_counts<<<blocks, 256, 0, s>>>(tile_start, num_tiles, chunk, A, B);
  cudaError_t e;
  e = exclusive_scan_u32(A, A, num_tiles, b.num_slots, b.scan_tmp, s);
  if (e != cudaSuccess) return e;
  // num_items is reused as scratch for B's total until k_item_emit.
  e = exclusive_scan_u32(B, B, num_tiles, b.counter, b.scan_tmp, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(b.num_split, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  k_item_emit<<<blocks, 256, 0, s>>>(tile_start, num_tiles, chunk, A, B,
                                     b.num_slots, b.counter, b.items,
                                     b.split_tiles, b.num_split, b.num_items);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // The persistent kernel's work counter starts at zero.
  return cudaMemsetAsync(b.counter, 0, sizeof(uint32_t), s);
}

template <typename Real>
int grid_tiles_ctas_per_sm() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &n, k_grid_tiles<Real, std::is_same<Real, float>::value>, kThreads,
          0) != cudaSuccess)
    n = 1;
  return n < 1 ? 1 : n;
}

template <typename Real>
cudaError_t launch_grid_tiles(const WorkItem* items, const uint32_t* num_items,
                              uint32_t* counter, const uint32_t* rec_vis,
                              const uint32_t* cell, const uint32_t* meta,
                              const void* vw, StackView view, TileGeom geom,
                              int grid_size, Real* grid, long long grid_stride,
                              Real* partials, int num_ctas, cudaStream_t s) {
  GridArgs<Real> a;
  a.items = items;
  a.num_items = num_items;
  a.counter = counter;
  a.rec_vis = rec_vis;
  a.cell = cell;
  a.meta = meta;
  a.vw = (const typename Vec2<Real>::type*)vw;
  a.view = view;
  a.geom = geom;
  a.grid_size = grid_size;
  a.grid = grid;
  a.grid_stride = grid_stride;
  a.partials = (typename Vec2<Real>::type*)partials;
  k_grid_tiles<Real, std::is_same<Real, float>::value>
      <<<num_ctas, kThreads, 0, s>>>(a);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_reduce_partials(const int4* split_tiles,
                                   const uint32_t* num_split, int max_split,
                                   const Real* partials, TileGeom geom,
                                   int grid_size, Real* grid,
                                   long long grid_stride, cudaStream_t s) {
  if (max_split <= 0) return cudaSuccess;
  const int blocks = std::min(max_split, 4096);
  k_reduce_partials<Real><<<blocks, 256, 0, s>>>(
      split_tiles, num_split,
      (const typename Vec2<Real>::type*)partials, geom, grid_size, grid,
      grid_stride);
  return cudaGetLastError();
}

template int grid_tiles_ctas_per_sm<float>();
template int grid_tiles_ctas_per_sm<double>();
template cudaError_t launch_grid_tiles<float>(
    const WorkItem*, const uint32_t*, uint32_t*, const uint32_t*,
    const uint32_t*, const uint32_t*, const void*, StackView, TileGeom, int,
    float*, long long, float*, int, cudaStream_t);
template cudaError_t launch_grid_tiles<double>(
    const WorkItem*, const uint32_t*, uint32_t*, const uint32_t*,
    const uint32_t*, const uint32_t*, const void*, StackView, TileGeom, int,
    double*, long long, double*, int, cudaStream_t);
template cudaError_t launch_reduce_partials<float>(const int4*,
                                                   const uint32_t*, int,
                                                   const float*, TileGeom, int,
                                                   float*, long long,
                                                   cudaStream_t);
template cudaError_t launch_reduce_partials<double>(const int4*,
                                                    const uint32_t*, int,
                                                    const double*, TileGeom,
                                                    int, double*, long long,
                                                    cudaStream_t);

}  // namespace gg
