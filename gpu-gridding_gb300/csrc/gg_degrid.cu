// Adjoint of the gridding map (degridding): grid -> visibilities.
//
// Forward gridding adds v_i * c~_i(cell) to every cell of visibility i's
// footprint (oskar_grid_wproj.c:190-209), with c~ the kernel tap whose
// imaginary part is negated for ww > 0.  Its exact adjoint is the gather
//   out_i = sum over the footprint of conj(c~_i(cell)) * grid(cell).
//
// It runs on the gridder's records: after placement, emission and the sort,
// each 32 x 64-cell tile's (visibility, tile) records are contiguous, and a
// persistent CTA takes work items (a tile and a range of its records) from
// the gridder's queue.  Its eight consumer warps hold the tile's grid
// values in registers (lane = column, kRows rows per lane, as in the
// gridder) and, for every record whose footprint meets their rows, multiply
// them by the record's taps from the slab stack and sum across the warp by
// shuffles.  The producer warp gathers and prepares the records and, once
// the consumers are done with a buffer, adds each record's warp sums in warp
// order and stores the record's partial result at its emission slot
// (rec_offset[visibility] + its tile's rank among the visibility's tiles).
// k_degrid_finish then adds each visibility's partial results in emission
// order.  Nothing is accumulated with atomics, so the result does
// not depend on scheduling.  With tile phases (see gg_grid.cu) a
// visibility's records are on its phase's tiles; the degridder only reads
// the grid, so the tiles of all phases share its one launch.
//
// The reference has no degridder; this one is pinned by the dot-product
// identity <G x, y> = <x, G^H y> against the forward kernel and by the FP64
// oracle.
#include <atomic>

#include "gg_internal.h"
#include "gg_tiles.cuh"

namespace gg {

namespace {

constexpr int kDegridTileU = 32;
using DegridShape = WarpShape<kDegridTileU>;

template <typename Real>
struct DegridArgs {
  const WorkItem* items;
  const uint32_t* num_items;  // queue length (device scalar)
  uint32_t* counter;
  uint32_t* error;            // set to 1 when a bounded wait runs out
  const uint32_t* rec_vis;    // sorted records: visibility index
  const uint32_t* cell;
  const uint32_t* meta;
  const uint32_t* rec_offset; // first emission slot of each visibility
  StackView view;
  TileGeom geom;
  int grid_size;
  const Real* grid;
  typename Vec2<Real>::type* rec_out;  // partial result per emission slot
};

// Shared-memory layout of one CTA (dynamic shared memory).
template <typename Real>
struct DegridSmem {
  using R2 = typename Vec2<Real>::type;
  R2 part[kRing][kBuf][kWarps];  // consumer warp w's sum of record t
  int4 rec[kRing][kBuf];         // slab descriptors (slab_record)
  uint32_t band[kRing][kBuf];    // bit w: the footprint meets warp w's rows
  uint32_t out[kRing][kBuf];     // emission slot | conjugated << 31
  int4 head[kRing];              // item, records (-1: no more work), flags
  uint64_t full[kRing];
  uint64_t empty[kRing];
};

__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  return __ffma2_rn(a, b, c);
}
__device__ __forceinline__ double2 fma2(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y));
}

// The producer warp: takes work items from the queue, streams their records
// through the ring and stores each finished buffer's per-record results.
// Returns false if a wait ran out.
template <typename Real>
__device__ bool degrid_produce(const DegridArgs<Real>& a,
                               DegridSmem<Real>& sm) {
  using R2 = typename Vec2<Real>::type;
  const int lane = threadIdx.x & 31;
  const int tiles_per_grid = a.geom.tiles_u * a.geom.tiles_v;
  const int end_item = (int)*a.num_items;
  // Buffer kb is done: add each record's warp sums (the warps its band bits
  // name, in warp order) and store them at the record's emission slot.
  auto flush = [&](unsigned kb) {
    const int slot = (int)(kb % kRing);
    const int nb = sm.head[slot].y;
    for (int t = lane; t < nb; t += 32) {
      const uint32_t band = sm.band[slot][t];
      R2 acc;
      acc.x = 0;
      acc.y = 0;
#pragma unroll
      for (int w = 0; w < kWarps; ++w) {
        if (band & (1u << w)) {
          acc.x += sm.part[slot][t][w].x;
          acc.y += sm.part[slot][t][w].y;
        }
      }
      a.rec_out[sm.out[slot][t] & 0x7FFFFFFFu] = acc;
    }
  };
  unsigned k = 0;
  bool done = false;
  while (!done) {
    int it = 0;
    if (lane == 0) it = (int)atomicAdd(a.counter, 1u);
    it = __shfl_sync(0xffffffffu, it, 0);
    done = it >= end_item;
    WorkItem item{0, 0, 0, -1};
    int tu = 0, tv = 0, sh = 0;
    if (!done) {
      item = a.items[it];
      const int tl = (item.tile % a.geom.tiles_total) % tiles_per_grid;
      tu = tl % a.geom.tiles_u;
      tv = tl / a.geom.tiles_u;
      sh = phase_shift(a.geom, item.tile / a.geom.tiles_total);
    }
    const int u0 = tu * DegridShape::kTileU - sh;
    const int v0 = tv * DegridShape::kTileV;
    int b0 = item.rec_begin;
    do {
      const int slot = (int)(k % kRing);
      const unsigned use = k / kRing;
      if (use > 0) {
        if (!mbar_wait(&sm.empty[slot], (use - 1) & 1)) return false;
        flush(k - kRing);
      }
      int nb = -1;
      if (!done) {
        nb = min(kBuf, item.rec_end - b0);
        uint32_t vid[kPerLane], ce[kPerLane], me[kPerLane], off[kPerLane];
#pragma unroll
        for (int q = 0; q < kPerLane; ++q) {
          const int t = q * 32 + lane;
          vid[q] = t < nb ? a.rec_vis[b0 + t] : 0u;
        }
#pragma unroll
        for (int q = 0; q < kPerLane; ++q) {
          const int t = q * 32 + lane;
          ce[q] = 0; me[q] = 0; off[q] = 0;
          if (t < nb) {
            ce[q] = a.cell[vid[q]];
            me[q] = a.meta[vid[q]];
            off[q] = a.rec_offset[vid[q]];
          }
        }
#pragma unroll
        for (int q = 0; q < kPerLane; ++q) {
          const int t = q * 32 + lane;
          if (t < nb) {
            const uint32_t m = me[q];
            const int plane = meta_plane(m);
            const int s = a.view.support[plane];
            const int gu = cell_u(ce[q]), gv = cell_v(ce[q]);
            sm.rec[slot][t] =
                a.view.oversample == 4
                    ? slab_record<kDegridTileU, 4>(a.view, plane, s,
                                                   meta_ou(m), meta_ov(m),
                                                   gu - u0, gv - v0)
                    : slab_record<kDegridTileU>(a.view, plane, s, meta_ou(m),
                                                meta_ov(m), gu - u0, gv - v0);
            uint32_t band = 0;
#pragma unroll
            for (int w = 0; w < kWarps; ++w) {
              const int r0 = v0 + w * kRows;
              if (gv - s <= r0 + kRows - 1 && gv + s >= r0) band |= 1u << w;
            }
            sm.band[slot][t] = band;
            // Rank of this tile among the visibility's tiles, in the order
            // k_emit writes them (tile rows outer, tile columns inner, on
            // the visibility's tile phase).
            const int tu0 = (gu - s + sh) / DegridShape::kTileU;
            const int tu1 = (gu + s + sh) / DegridShape::kTileU;
            const int tv0 = (gv - s) / DegridShape::kTileV;
            const uint32_t rank =
                (uint32_t)((tv - tv0) * (tu1 - tu0 + 1) + (tu - tu0));
            sm.out[slot][t] = (off[q] + rank) |
                              (meta_conj(m) ? 0x80000000u : 0u);
          }
        }
      }
      if (lane == 0) {
        const int flags = done ? 0 : ((b0 == item.rec_begin ? 1 : 0) |
                                      (b0 + kBuf >= item.rec_end ? 2 : 0));
        sm.head[slot] = make_int4(it, nb, flags, 0);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.full[slot]);
      ++k;
      b0 += kBuf;
    } while (!done && b0 < item.rec_end);
  }
  // Buffer k - 1 is the end marker; the kRing - 1 data buffers before it
  // have not been reused, so their results are still to be stored.
  for (unsigned kb = k >= kRing ? k - kRing : 0u; kb + 2 <= k; ++kb) {
    if (!mbar_wait(&sm.empty[kb % kRing], (kb / kRing) & 1)) return false;
    flush(kb);
  }
  return true;
}

// The kRows taps of one record for this lane from the slab stack; lanes
// outside the footprint's columns read zeros.  (Rows of the warp outside
// the footprint read the slab's zero padding rows.)
template <typename R2>
__device__ __forceinline__ void load_taps(const int4 ra,
                                          const R2* __restrict__ slabs,
                                          const R2* __restrict__ gzeros,
                                          int lx, int rowl, uint64_t pol,
                                          R2 (&out)[kRows]) {
  const int c0 = (ra.w >> 8) & 0xFF, cw = (int)((unsigned)ra.w >> 16);
  const bool ok = (unsigned)(lx - c0) <= (unsigned)cw;
  const int off = (lx >= (ra.w & 0xFF) ? ra.x + lx : ra.y - lx) + rowl * ra.z;
  const R2* p = ok ? slabs + off : gzeros;
  const int step = ok ? ra.z : 0;
#pragma unroll
  for (int r = 0; r < kRows; ++r) out[r] = ld_tap(p + r * step, pol);
}

// This lane's share of conj(c~) * g over its kRows cells, with
// gx[r] = (g.re, g.re) and gy[r] = (g.im, g.im): P = sum t * g.re and
// Q = sum t * g.im componentwise, so with c~ = (t.re, sgn * t.im)
//   re = P.x + sgn * Q.y,  im = Q.x - sgn * P.y.
template <typename R2, typename Real>
__device__ __forceinline__ void dot_record(const R2 (&t)[kRows],
                                           const R2 (&gx)[kRows],
                                           const R2 (&gy)[kRows], Real sgn,
                                           Real& re, Real& im) {
  R2 P, Q;
  P.x = P.y = Q.x = Q.y = 0;
#pragma unroll
  for (int r = 0; r < kRows; ++r) {
    P = fma2(t[r], gx[r], P);
    Q = fma2(t[r], gy[r], Q);
  }
  re = P.x + sgn * Q.y;
  im = Q.x - sgn * P.y;
}

template <typename Real>
__global__ void __launch_bounds__(kThreads, sizeof(Real) == 4 ? 2 : 1)
k_degrid_tiles(DegridArgs<Real> a) {
  using R2 = typename Vec2<Real>::type;
  using SM = DegridSmem<Real>;
  extern __shared__ __align__(16) unsigned char g_smem_raw[];
  SM& sm = *reinterpret_cast<SM*>(g_smem_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kRing; ++i) {
      mbar_init(&sm.full[i], 1);
      mbar_init(&sm.empty[i], kWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (warp == kWarps) {
    if (!degrid_produce<Real>(a, sm)) atomicExch(a.error, 1u);
    return;
  }

  const int rowl = warp * kRows;   // this lane's row 0 in the tile
  const int G = a.grid_size;
  const int tiles_per_grid = a.geom.tiles_u * a.geom.tiles_v;
  const R2* __restrict__ slabs = (const R2*)a.view.slabs;
  const R2* __restrict__ gzeros = (const R2*)a.view.zeros;
  const R2* __restrict__ grid = (const R2*)a.grid;
  const uint64_t pol = evict_last_policy();
  const uint32_t my_bit = 1u << warp;
  R2 gx[kRows], gy[kRows];
#pragma unroll
  for (int r = 0; r < kRows; ++r) gx[r].x = gx[r].y = gy[r].x = gy[r].y = 0;

  for (unsigned k = 0;; ++k) {
    const int slot = (int)(k % kRing);
    if (!mbar_wait(&sm.full[slot], (k / kRing) & 1)) {
      atomicExch(a.error, 1u);
      return;
    }
    const int4 head = sm.head[slot];
    const int nb = head.y;
    if (nb < 0) break;
    if (head.z & 1) {  // first buffer of a work item: load its tile
      const WorkItem item = a.items[head.x];
      const int tl = (item.tile % a.geom.tiles_total) % tiles_per_grid;
      // Tiles of later phases start left of phase 0's (and may reach past
      // either edge of the grid).
      const int col = (tl % a.geom.tiles_u) * DegridShape::kTileU + lane -
                      phase_shift(a.geom, item.tile / a.geom.tiles_total);
      const int row0 = (tl / a.geom.tiles_u) * DegridShape::kTileV + rowl;
      const bool col_in = (unsigned)col < (unsigned)G;
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        R2 g;
        g.x = g.y = 0;
        if (row0 + r < G && col_in) g = grid[(size_t)(row0 + r) * G + col];
        gx[r].x = gx[r].y = g.x;
        gy[r].x = gy[r].y = g.y;
      }
    }
    for (int c0 = 0; c0 < nb; c0 += 32) {
      const bool touch =
          c0 + lane < nb && (sm.band[slot][c0 + lane] & my_bit) != 0u;
      uint32_t m = __ballot_sync(0xffffffffu, touch);
      // Two records at a time: 2 * kRows independent tap loads per lane in
      // flight, and one shuffle tree for the pair.
      while (m) {
        const int tA = c0 + __ffs(m) - 1;
        m &= m - 1;
        R2 ta[kRows];
        load_taps(sm.rec[slot][tA], slabs, gzeros, lane, rowl, pol, ta);
        const Real sA = (sm.out[slot][tA] >> 31) ? (Real)-1 : (Real)1;
        Real reA, imA;
        if (m) {
          const int tB = c0 + __ffs(m) - 1;
          m &= m - 1;
          R2 tb[kRows];
          load_taps(sm.rec[slot][tB], slabs, gzeros, lane, rowl, pol, tb);
          const Real sB = (sm.out[slot][tB] >> 31) ? (Real)-1 : (Real)1;
          Real reB, imB;
          dot_record(ta, gx, gy, sA, reA, imA);
          dot_record(tb, gx, gy, sB, reB, imB);
          // Lanes 0-15 keep record A, lanes 16-31 record B.
          const bool upper = (lane & 16) != 0;
          Real kre = upper ? reB : reA, kim = upper ? imB : imA;
          kre += __shfl_xor_sync(0xffffffffu, upper ? reA : reB, 16);
          kim += __shfl_xor_sync(0xffffffffu, upper ? imA : imB, 16);
#pragma unroll
          for (int o = 8; o > 0; o >>= 1) {
            kre += __shfl_xor_sync(0xffffffffu, kre, o);
            kim += __shfl_xor_sync(0xffffffffu, kim, o);
          }
          if ((lane & 15) == 0) {
            R2 v;
            v.x = kre;
            v.y = kim;
            sm.part[slot][upper ? tB : tA][warp] = v;
          }
        } else {
          dot_record(ta, gx, gy, sA, reA, imA);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            reA += __shfl_xor_sync(0xffffffffu, reA, o);
            imA += __shfl_xor_sync(0xffffffffu, imA, o);
          }
          if (lane == 0) {
            R2 v;
            v.x = reA;
            v.y = imA;
            sm.part[slot][tA][warp] = v;
          }
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.empty[slot]);
  }
}

// out[i] = sum of visibility i's partial results in emission order, in the
// call's precision (a visibility has a handful of records: its footprint's
// tiles); skipped visibilities have no records and get 0.
template <typename Real>
__global__ void k_degrid_finish(const uint32_t* __restrict__ count,
                                const uint32_t* __restrict__ offset,
                                const typename Vec2<Real>::type* __restrict__
                                    rec_out,
                                unsigned long long n, Real* __restrict__ out) {
  using R2 = typename Vec2<Real>::type;
  const unsigned long long i =
      (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t c = count[i], o = offset[i];
  R2 acc;
  acc.x = acc.y = 0;
  for (uint32_t k = 0; k < c; ++k) {
    const R2 v = rec_out[o + k];
    acc.x += v.x;
    acc.y += v.y;
  }
  ((R2*)out)[i] = acc;
}

template <typename Real>
cudaError_t prepare_degrid_kernel(size_t* smem) {
  static std::atomic<unsigned long long> opted_in{0};
  *smem = sizeof(DegridSmem<Real>);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (dev < 64 && (opted_in.load() & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(k_degrid_tiles<Real>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)*smem);
  if (e == cudaSuccess && dev < 64) opted_in.fetch_or(bit);
  return e;
}

}  // namespace

template <typename Real>
int degrid_tiles_ctas_per_sm() {
  size_t smem = 0;
  int n = 0;
  if (prepare_degrid_kernel<Real>(&smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &n, k_degrid_tiles<Real>, kThreads, smem) != cudaSuccess)
    n = 1;
  return n < 1 ? 1 : n;
}

template <typename Real>
cudaError_t launch_degrid_tiles(const WorkItem* items,
                                const uint32_t* num_items, uint32_t* counter,
                                uint32_t* error, const uint32_t* rec_vis,
                                const uint32_t* cell, const uint32_t* meta,
                                const uint32_t* rec_offset, StackView view,
                                TileGeom geom, int grid_size, const Real* grid,
                                void* rec_out, int num_ctas, cudaStream_t s) {
  if (geom.tile_u != kDegridTileU || geom.tile_v != DegridShape::kTileV)
    return cudaErrorInvalidValue;
  DegridArgs<Real> a;
  a.items = items;
  a.num_items = num_items;
  a.counter = counter;
  a.error = error;
  a.rec_vis = rec_vis;
  a.cell = cell;
  a.meta = meta;
  a.rec_offset = rec_offset;
  a.view = view;
  a.geom = geom;
  a.grid_size = grid_size;
  a.grid = grid;
  a.rec_out = (typename Vec2<Real>::type*)rec_out;
  size_t smem = 0;
  cudaError_t e = prepare_degrid_kernel<Real>(&smem);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  k_degrid_tiles<Real><<<num_ctas, kThreads, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_degrid_finish(const uint32_t* count, const uint32_t* offset,
                                 const void* rec_out, unsigned long long n,
                                 Real* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const unsigned long long blocks = (n + 255) / 256;
  k_degrid_finish<Real><<<(unsigned)blocks, 256, 0, s>>>(
      count, offset, (const typename Vec2<Real>::type*)rec_out, n, out);
  return cudaGetLastError();
}

template int degrid_tiles_ctas_per_sm<float>();
template int degrid_tiles_ctas_per_sm<double>();
template cudaError_t launch_degrid_tiles<float>(
    const WorkItem*, const uint32_t*, uint32_t*, uint32_t*, const uint32_t*,
    const uint32_t*, const uint32_t*, const uint32_t*, StackView, TileGeom,
    int, const float*, void*, int, cudaStream_t);
template cudaError_t launch_degrid_tiles<double>(
    const WorkItem*, const uint32_t*, uint32_t*, uint32_t*, const uint32_t*,
    const uint32_t*, const uint32_t*, const uint32_t*, StackView, TileGeom,
    int, const double*, void*, int, cudaStream_t);
template cudaError_t launch_degrid_finish<float>(const uint32_t*,
                                                 const uint32_t*, const void*,
                                                 unsigned long long, float*,
                                                 cudaStream_t);
template cudaError_t launch_degrid_finish<double>(const uint32_t*,
                                                  const uint32_t*, const void*,
                                                  unsigned long long, double*,
                                                  cudaStream_t);

}  // namespace gg
