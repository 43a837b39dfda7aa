// Tile-owning gridding.
//
// The grid is cut into tiles of TW (u) x TV (v) cells.  After the sort each
// tile's (visibility, tile) records are contiguous and ordered by (plane,
// |offset| class); a tile's record range is cut into work items of at most
// `chunk` records.  A persistent CTA takes work items from a queue and keeps
// the item's whole tile in registers: lane (lx, ly) of consumer warp w owns
// column lx and kRows consecutive rows of the warp's band.  For every record,
// each warp whose band meets the footprint multiplies the visibility by the
// kernel taps of its own cells and accumulates -- no atomics, no
// shared-memory read-modify-write.  A tile with one item is then added to
// the grid in place with one coalesced read-modify-write; a tile split over
// several items writes one partial tile per item and k_reduce_partials (or
// k_reduce_phases) adds them to the grid in item order, so the result does
// not depend on scheduling.
//
// The CTA is warp-specialised.  One producer warp takes work items, gathers
// and prepares their records and streams them through a ring of kRing
// shared-memory buffers guarded by mbarriers; when a buffer is dominated by
// one (plane, |offset|) group that is long enough to pay for it, the producer
// also stages that group's kernel slice into one of kSlots shared-memory
// slots with a bulk asynchronous copy (cp.async.bulk, completion tracked by
// the buffer's mbarrier), and those records read their taps from shared
// memory instead of L2.  Eight consumer warps accumulate.
//
// Three warp shapes share the 2048-cell tile: TW = 32 (32 x 64 tiles, for
// large footprints), 16 (16 x 128) and 8 (8 x 256, for small footprints,
// where a 32-wide warp would leave most lanes outside the footprint).
//
// Tile phases (TileGeom::tile_phases): up to eight tile grids, each offset
// by a strip of TW / phases columns from the last; every visibility's
// records are on the grid that cuts its footprint into the fewest tile
// columns, so fewer warp steps fall on footprints cut by a tile boundary.
// One launch takes all the phases of a plane group: phase 0's single-item
// tiles add to the grid as above, every other item writes a partial tile,
// and k_reduce_phases adds those per cell in phase order after the launch
// (where the grid is the caller's host memory in place, reading and writing
// it per strip as the strip's first and last passes would).
//
// The reference's equivalent is oskar_process_tiles_dynamic
// (oskar_grid_wproj_gpu.cu:840-1309), a one-warp-per-32x16-tile kernel that
// flushes with float atomics whenever its tile changes.
//
// FP32 accumulation is compensated: each buffer of records is summed in
// plain FP32 FMA, then folded into a (hi, lo) pair by Knuth's TwoSum, so
// rounding error does not grow with the number of visibilities on a cell.
#include <algorithm>
#include <atomic>
#include <type_traits>

#include "gg_internal.h"
#include "gg_tiles.cuh"

namespace gg {

namespace {

constexpr int kSlots = 2;         // staged kernel slices
constexpr int kSliceBytes = 26624;  // per slot: (2s+15)(2s+1) taps, s <= 25 (FP32)
constexpr int kRunMin = 24;       // records of one group that pay for staging

// Visibility coefficients of one record with the conjugation folded in:
// re += a*t.re + b*t.im, im += c*t.re + d*t.im.  Stored as (a, d, c, b) so
// that the FP32 kernel can accumulate two packed pairs per cell with FP32x2
// FMAs, P += (a, d) * (t.re, t.im) and Q += (c, b) * (t.re, t.im), and
// recover re = P.x + Q.y, im = Q.x + P.y when it folds a buffer.
template <typename Real>
struct alignas(4 * sizeof(Real)) Coef {
  Real a, d, c, b;
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
  const uint32_t* group_items;  // queue start of each virtual group
  int group;                     // the launch's first virtual group
  int group_span;                // virtual groups in the launch
  uint32_t* counter;
  uint32_t* error;          // set to 1 when a bounded wait runs out
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
  // Direct mode (single grid, tile_groups non-null): the caller's grid at
  // host, addressed in place.  tile_groups[tile] = first | last << 16, the
  // first and last plane group with records in the tile: the first reads
  // the tile's cells from host, the last writes them to host, the others
  // go through grid (scratch).
  Real* host;
  const uint32_t* tile_groups;
};

// Source and destination of a grid cell's read-modify-write in virtual
// group `group`: the scratch grid g, or the caller's grid h in direct mode.
// Direct mode keeps, per strip of tile_u / tile_phases columns of a tile
// row, the first and last virtual group whose tiles hold records there
// (k_tile_groups): the first reads the cells from h, the last writes them
// to h, the others go through g.
template <typename R2>
__device__ __forceinline__ void cell_ends(const uint32_t* tile_groups,
                                          const TileGeom& geom, int tv,
                                          int col, int group, R2* g, R2* h,
                                          R2*& src, R2*& dst) {
  src = g;
  dst = g;
  if (tile_groups) {
    const uint32_t fl = tile_groups[tv * geom.strips_u + (col >> geom.strip_shift)];
    if ((int)(fl & 0xFFFFu) == group) src = h;
    if ((int)(fl >> 16) == group) dst = h;
  }
}

// Shared-memory layout of one CTA (dynamic shared memory).  Without slice
// staging the CTA needs about 50 KB, leaving the rest of the SM's unified
// L1 / shared memory to cache the taps it reads from the global stack.
template <typename Real, bool kStage>
struct Smem {
  using R2 = typename Vec2<Real>::type;
  static constexpr int kNSlots = kStage ? kSlots : 1;
  static constexpr int kSliceTaps = kStage ? kSliceBytes / (int)sizeof(R2) : 2;
  // Largest staged slice width F: (F + 2*kSlicePad) * F <= kSliceTaps.
  static constexpr int kMaxStagedF = sizeof(Real) == 4 ? 51 : 33;
  // Zero region for lanes outside a footprint: kRows rows of up to
  // kMaxStagedF taps either way from its middle.
  static constexpr int kZeroTaps = kStage ? 2 * kRows * kMaxStagedF + 2 : 2;
  static constexpr bool kComp = sizeof(Real) == 4;
  R2 slice[kNSlots][kSliceTaps];
  R2 zero[kZeroTaps];
  R2 hi[kComp ? kRows : 1][kConsumers];
  R2 lo[kComp ? kRows : 1][kConsumers];
  int4 rec[kRing][kBuf];
  Coef<Real> cf[kRing][kBuf];
  uint32_t band[kRing][kBuf];
  signed char src[kRing][kBuf];   // slice slot of the record, -1 = global
  // Half-warp record lists of the buffer being gridded (per consumer warp:
  // the records meeting its rows and columns 0..15, then 16..31).
  unsigned char half_list[kWarps][2][kBuf];
  int4 head[kRing];
  uint64_t full[kRing];
  uint64_t empty[kRing];
};
static_assert((51 + 2 * kSlicePad) * 51 <= kSliceBytes / 8, "FP32 slot size");
static_assert((33 + 2 * kSlicePad) * 33 <= kSliceBytes / 16, "FP64 slot size");

// Record data in shared memory (int4 per record).  A record whose taps are
// read from the slab stack in global memory (src < 0) holds slab_record's
// descriptor (gg_tiles.cuh).  A record whose slice is staged in a
// shared-memory slot (src >= 0) holds
//   x = org:   tap index of tile cell (0, 0) on the staged slice
//   y = rstep: +-(2s+1), slice rows per tile row (mirrored for ov < 0)
//   z = ulo:   first footprint column (tile-relative)
//   w = su * (2s+1): column mirror sign and footprint width
// so its tap for tile cell (row, col) is slice[org + row * rstep +
// col * su]; lanes whose column lies outside [ulo, ulo + 2s] read zeros.
//
// Slice-slot bookkeeping of the producer (lane-uniform).
struct SlotState {
  int group[kSlots];       // (plane, |offset| class) held, -1 = none
  unsigned last_k[kSlots]; // last ring buffer that referenced the slot
  bool used[kSlots];
};

__device__ __forceinline__ int group_of(uint32_t meta) {
  return meta_plane(meta) * 64 + abs(meta_ou(meta)) * 8 + abs(meta_ov(meta));
}

// The producer warp: takes work items from the queue and streams their
// records, staged, through the ring.  Returns false if a wait ran out.
template <typename Real, int TW, bool kStage, bool kHalves>
__device__ bool produce(const GridArgs<Real>& a, Smem<Real, kStage>& sm) {
  using R2 = typename Vec2<Real>::type;
  using WS = WarpShape<TW>;
  const int lane = threadIdx.x & 31;
  const int omax = a.view.omax;
  const int tiles_per_grid = a.geom.tiles_u * a.geom.tiles_v;
  // The launch's items: those of its virtual groups (a plane group's tile
  // phases, or one of them).
  const int first_item = (int)a.group_items[a.group];
  const int end_item = (int)a.group_items[a.group + a.group_span];
  const R2* __restrict__ taps = (const R2*)a.view.taps;
  SlotState st;
  for (int x = 0; x < kSlots; ++x) {
    st.group[x] = -1;
    st.last_k[x] = 0;
    st.used[x] = false;
  }
  unsigned k = 0;
  for (;;) {
    int it = 0;
    if (lane == 0) it = first_item + (int)atomicAdd(a.counter, 1u);
    it = __shfl_sync(0xffffffffu, it, 0);
    const bool done = it >= end_item;
    WorkItem item{0, 0, 0, -1};
    int u0 = 0, v0 = 0;
    if (!done) {
      item = a.items[it];
      const int vg = item.tile / a.geom.tiles_total;   // virtual group
      const int tl = (item.tile - vg * a.geom.tiles_total) % tiles_per_grid;
      u0 = (tl % a.geom.tiles_u) * WS::kTileU - phase_shift(a.geom, vg);
      v0 = (tl / a.geom.tiles_u) * WS::kTileV;
    }
    int b0 = item.rec_begin;
    do {
      const int slot = (int)(k % kRing);
      const unsigned use = k / kRing;
      if (use > 0 && !mbar_wait(&sm.empty[slot], (use - 1) & 1)) return false;
      int nb = -1;
      if (!done) {
        nb = min(kBuf, item.rec_end - b0);
        // Gather kPerLane records per lane; their loads are independent,
        // so they overlap.
        uint32_t vid[kPerLane], ce[kPerLane], me[kPerLane];
        R2 v[kPerLane];
        int grp[kPerLane];
#pragma unroll
        for (int q = 0; q < kPerLane; ++q) {
          const int t = q * 32 + lane;
          vid[q] = t < nb ? a.rec_vis[b0 + t] : 0u;
        }
#pragma unroll
        for (int q = 0; q < kPerLane; ++q) {
          const int t = q * 32 + lane;
          ce[q] = 0; me[q] = 0; grp[q] = -2;
          if (t < nb) {
            ce[q] = a.cell[vid[q]];
            me[q] = a.meta[vid[q]];
            v[q] = a.vw[vid[q]];
            grp[q] = group_of(me[q]);
          }
        }
        // ---- stage the slices of the buffer's dominant groups ----------
        // Candidates: the groups of the first and the last record (records
        // are sorted by group within a tile, so a long run covers one end).
        if constexpr (kStage) {
        const int last = nb - 1;
        int cand[2];
        uint32_t cand_meta[2];
        cand[0] = __shfl_sync(0xffffffffu, grp[0], 0);
        cand_meta[0] = __shfl_sync(0xffffffffu, me[0], 0);
        {
          int gl = grp[0];
          uint32_t ml = me[0];
#pragma unroll
          for (int q = 1; q < kPerLane; ++q)
            if (q == last / 32) { gl = grp[q]; ml = me[q]; }
          cand[1] = __shfl_sync(0xffffffffu, gl, last % 32);
          cand_meta[1] = __shfl_sync(0xffffffffu, ml, last % 32);
        }
#pragma unroll
        for (int ci = 0; ci < 2; ++ci) {
          const int g = cand[ci];
          if (ci == 1 && g == cand[0]) break;
          int cnt = 0;
#pragma unroll
          for (int q = 0; q < kPerLane; ++q)
            cnt += __popc(__ballot_sync(0xffffffffu, grp[q] == g));
          const int plane = meta_plane(cand_meta[ci]);
          const int s = a.view.support[plane];
          const long long bytes = slice_taps(s) * (long long)sizeof(R2);
          bool resident = false;
          for (int x = 0; x < kSlots; ++x) resident |= st.group[x] == g;
          if (resident || cnt < kRunMin || bytes > kSliceBytes) continue;
          // Take the slot used longest ago that the other candidate does
          // not hold.
          int x = 0;
          for (int y = 1; y < kSlots; ++y) {
            const bool other = st.group[x] == cand[1 - ci];
            if (other || (st.group[y] != cand[1 - ci] &&
                          st.last_k[y] < st.last_k[x]))
              x = y;
          }
          // The slot's previous contents may still be read by a buffer in
          // flight: wait for the consumers to finish it.
          if (st.used[x] && st.last_k[x] + kRing > k) {
            const unsigned kk = st.last_k[x];
            if (!mbar_wait(&sm.empty[kk % kRing], (kk / kRing) & 1))
              return false;
          }
          const long long start =
              a.view.base[plane] +
              (long long)(abs(meta_ou(cand_meta[ci])) * (omax + 1) +
                          abs(meta_ov(cand_meta[ci]))) * slice_taps(s);
          if (lane == 0) {
            mbar_expect_tx(&sm.full[slot], (uint32_t)bytes);
            bulk_copy_g2s(&sm.slice[x][0], taps + start, (uint32_t)bytes,
                          &sm.full[slot]);
          }
          st.group[x] = g;
          st.used[x] = true;
          st.last_k[x] = k;
        }
        }  // kStage
        // ---- prepare the records ---------------------------------------
#pragma unroll
        for (int q = 0; q < kPerLane; ++q) {
          const int t = q * 32 + lane;
          int src = -1;
          if constexpr (kStage) {
            for (int x = 0; x < kSlots; ++x)
              if (grp[q] == st.group[x]) src = x;
            // Slots referenced by this buffer stay reserved until it is
            // done.
            for (int x = 0; x < kSlots; ++x)
              if (__any_sync(0xffffffffu, src == x)) st.last_k[x] = k;
          }
          if (t < nb) {
            const uint32_t m = me[q];
            const int plane = meta_plane(m);
            const int ou = meta_ou(m), ov = meta_ov(m);
            const int s = a.view.support[plane];
            const int F = 2 * s + 1;
            const int gu = cell_u(ce[q]) - u0, gv = cell_v(ce[q]) - v0;
            const int su = ou < 0 ? -1 : 1, sv = ov < 0 ? -1 : 1;
            if (src < 0) {
              // Slab of (plane, |ov|); rows mirrored for ov < 0, columns by
              // residue on either side of the fold ou + k*os = 0.
              sm.rec[slot][t] =
                  a.view.oversample == 4
                      ? slab_record<TW, 4>(a.view, plane, s, ou, ov, gu, gv)
                      : slab_record<TW>(a.view, plane, s, ou, ov, gu, gv);
            } else {
              // Tap index of S[0][0] relative to the padded slice start.
              const int org = kSlicePad * F + (s - sv * gv) * F +
                              (s - su * gu);
              sm.rec[slot][t] = make_int4(org, sv * F, gu - s, su * F);
            }
            sm.src[slot][t] = (signed char)src;
            // Bit (warp * kLanesY + lane row) = that lane row's kRows rows
            // meet the footprint rows [gv - s, gv + s].
            uint32_t band = 0;
#pragma unroll
            for (int gg = 0; gg < kWarps * WS::kLanesY; ++gg) {
              const int r0 = gg * kRows;
              if (gv - s <= r0 + kRows - 1 && gv + s >= r0) band |= 1u << gg;
            }
            if constexpr (kHalves) {
              // Bits 8 and 9: the footprint meets tile columns 0..15,
              // 16..31 (the two half-warps' columns).
              if (gu - s <= 15) band |= 1u << 8;
              if (gu + s >= 16) band |= 1u << 9;
            }
            sm.band[slot][t] = band;
            Coef<Real> cf;
            cf.a = v[q].x;
            cf.c = v[q].y;
            if (meta_conj(m)) { cf.b = v[q].y; cf.d = -v[q].x; }
            else { cf.b = -v[q].y; cf.d = v[q].x; }
            sm.cf[slot][t] = cf;
          }
        }
      }
      if (lane == 0) {
        // item index, record count (-1 = no more work), first/last flags
        const int flags = done ? 0 : ((b0 == item.rec_begin ? 1 : 0) |
                                      (b0 + kBuf >= item.rec_end ? 2 : 0));
        sm.head[slot] = make_int4(it, nb, flags, 0);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.full[slot]);
      ++k;
      if (done) return true;
      b0 += kBuf;
    } while (b0 < item.rec_end);
  }
}

// The kRows taps of a record with slab descriptor ra for this lane (zeros
// outside the footprint's columns or when !inband).
template <typename R2>
__device__ __forceinline__ void load_slab_taps(const int4 ra, bool inband,
                                               const R2* __restrict__ slabs,
                                               const R2* __restrict__ gzeros,
                                               int lx, int rowl, uint64_t pol,
                                               R2 (&out)[kRows]) {
  const int c0 = (ra.w >> 8) & 0xFF, cw = (int)((unsigned)ra.w >> 16);
  const bool ok = inband && (unsigned)(lx - c0) <= (unsigned)cw;
  const int off = (lx >= (ra.w & 0xFF) ? ra.x + lx : ra.y - lx) + rowl * ra.z;
  const R2* p = ok ? slabs + off : gzeros;
  const int step = ok ? ra.z : 0;
#pragma unroll
  for (int r = 0; r < kRows; ++r) out[r] = ld_tap(p + r * step, pol);
}

// Loads the kRows taps of one record for this lane: from the record's
// slice slot in shared memory, or from the slab stack (see the record
// layout above).  Lanes outside the footprint's columns, or outside the
// warp rows the record meets, read zeros.
template <typename Real, int TW, bool kStage, typename R2>
__device__ __forceinline__ void load_record(const Smem<Real, kStage>& sm,
                                            int slot, int t,
                                            const R2* __restrict__ slabs,
                                            const R2* __restrict__ gzeros,
                                            uint32_t my_bit, int lx, int rowl,
                                            uint64_t pol, R2 (&out)[kRows]) {
  const int4 ra = sm.rec[slot][t];
  // With one lane row per warp (TW = 32) a warp only takes records that
  // meet its rows; narrower tiles check the lane's own row group.
  const bool inband = TW == 32 || (sm.band[slot][t] & my_bit) != 0u;
  if (kStage && sm.src[slot][t] >= 0) {
    const int src = sm.src[slot][t];
    const bool ok =
        inband && (unsigned)(lx - ra.z) <= (unsigned)(abs(ra.w) - 1);
    const int off = ra.x + rowl * ra.y + lx * (ra.w < 0 ? -1 : 1);
    const R2* p = ok ? &sm.slice[src][0] + off
                     : &sm.zero[Smem<Real, kStage>::kZeroTaps / 2];
#pragma unroll
    for (int r = 0; r < kRows; ++r) out[r] = p[r * ra.y];
    return;
  }
  const int c0 = (ra.w >> 8) & 0xFF, cw = (int)((unsigned)ra.w >> 16);
  const bool ok = inband && (unsigned)(lx - c0) <= (unsigned)cw;
  const int off = (lx >= (ra.w & 0xFF) ? ra.x + lx : ra.y - lx) + rowl * ra.z;
  const R2* p = ok ? slabs + off : gzeros;
  const int step = ok ? ra.z : 0;
#pragma unroll
  for (int r = 0; r < kRows; ++r) out[r] = ld_tap(p + r * step, pol);
}

// Adds one record's contribution to the lane's cells.  FP32: packed FP32x2
// FMAs into the (P, Q) pairs (see Coef); FP64: plain FMAs into (re, im).
template <typename Real, typename R2>
__device__ __forceinline__ void accumulate(const Coef<Real>& c,
                                           const R2 (&tp)[kRows],
                                           R2 (&acc)[kRows],
                                           R2 (&acq)[kRows]) {
  if constexpr (sizeof(Real) == 4) {
    const float2 cp = make_float2(c.a, c.d), cq = make_float2(c.c, c.b);
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      acc[r] = __ffma2_rn(cp, tp[r], acc[r]);
      acq[r] = __ffma2_rn(cq, tp[r], acq[r]);
    }
  } else {
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      acc[r].x = fma(c.b, tp[r].y, fma(c.a, tp[r].x, acc[r].x));
      acc[r].y = fma(c.d, tp[r].y, fma(c.c, tp[r].x, acc[r].y));
    }
  }
}

template <typename Real, bool kCompensate, int TW, bool kStage, bool kHalves>
__global__ void __launch_bounds__(kThreads, sizeof(Real) == 4 ? 2 : 1)
k_grid_tiles(GridArgs<Real> a) {
  static_assert(!kHalves || (TW == 32 && !kStage),
                "half-warp record streams: 32-wide tiles, taps from the "
                "slab stack");
  using R2 = typename Vec2<Real>::type;
  using WS = WarpShape<TW>;
  using SM = Smem<Real, kStage>;
  constexpr int G = WS::kLanesY;
  extern __shared__ __align__(16) unsigned char g_smem_raw[];
  SM& sm = *reinterpret_cast<SM*>(g_smem_raw);

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < SM::kZeroTaps; i += blockDim.x) {
    sm.zero[i].x = 0;
    sm.zero[i].y = 0;
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < kRing; ++i) {
      mbar_init(&sm.full[i], 1);
      mbar_init(&sm.empty[i], kWarps);
    }
    // Make the initialised barriers visible to the async proxy (bulk
    // copies complete transactions on them).
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  if (warp == kWarps) {
    if (!produce<Real, TW, kStage, kHalves>(a, sm)) atomicExch(a.error, 1u);
    return;
  }

  const int lx = lane % TW, ly = lane / TW;
  const int rowl = warp * WS::kBand + ly * kRows;   // this lane's row 0
  const int G_size = a.grid_size;
  const R2* __restrict__ slabs = (const R2*)a.view.slabs;
  const R2* __restrict__ gzeros = (const R2*)a.view.zeros;
  const int tiles_per_grid = a.geom.tiles_u * a.geom.tiles_v;
  const uint64_t pol = evict_last_policy();
  const uint32_t my_bit = 1u << (warp * G + ly);
  const uint32_t warp_bits = ((1u << G) - 1u) << (warp * G);

  // FP32: (P, Q) pairs of every cell (see Coef); FP64: (re, im) in acc.
  R2 acc[kRows], acq[kRows];
#pragma unroll
  for (int r = 0; r < kRows; ++r) acc[r].x = acc[r].y = acq[r].x = acq[r].y = 0;

  for (unsigned k = 0;; ++k) {
    const int slot = (int)(k % kRing);
    if (!mbar_wait(&sm.full[slot], (k / kRing) & 1)) {
      atomicExch(a.error, 1u);
      return;
    }
    const int4 head = sm.head[slot];
    const int nb = head.y;
    if (nb < 0) break;
    if (head.z & 1) {  // first buffer of a work item
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        acc[r].x = acc[r].y = acq[r].x = acq[r].y = 0;
        if constexpr (kCompensate) {
          sm.hi[r][threadIdx.x] = acc[r];
          sm.lo[r][threadIdx.x] = acc[r];
        }
      }
    }
    // ---- half-warp record streams (32-wide tiles) ------------------------
    // Each half-warp takes, in queue order, the records of the buffer that
    // meet this warp's rows and its own 16 columns (lists built from the
    // buffer's band bits), so a record that meets one half only runs beside
    // another record on the other half.  Up to three records per half at a
    // time.  Each cell still takes its records in queue order.
    if constexpr (kHalves) {
      const int hh = lane >> 4;
      unsigned char* l0 = sm.half_list[warp][0];
      unsigned char* l1 = sm.half_list[warp][1];
      const uint32_t lt = (1u << lane) - 1u;
      int n0 = 0, n1 = 0;
      for (int c0 = 0; c0 < nb; c0 += 32) {
        const uint32_t bd = c0 + lane < nb ? sm.band[slot][c0 + lane] : 0u;
        const bool mine = (bd & warp_bits) != 0u;
        const bool in0 = mine && (bd & 0x100u), in1 = mine && (bd & 0x200u);
        const uint32_t b0 = __ballot_sync(0xffffffffu, in0);
        const uint32_t b1 = __ballot_sync(0xffffffffu, in1);
        if (in0) l0[n0 + __popc(b0 & lt)] = (unsigned char)(c0 + lane);
        if (in1) l1[n1 + __popc(b1 & lt)] = (unsigned char)(c0 + lane);
        n0 += __popc(b0);
        n1 += __popc(b1);
      }
      __syncwarp();
      const unsigned char* my = hh ? l1 : l0;
      const int nmine = hh ? n1 : n0;
      const int n = max(n0, n1);
      // Entry i of this half's list; past its end the half runs the other
      // half's entry i with its taps read as zeros (so it adds nothing).
      const unsigned char* other = hh ? l0 : l1;
      auto pick = [&](int i) { return (int)(i < nmine ? my[i] : other[i]); };
      auto taps = [&](int i, int t, R2 (&out)[kRows]) {
        load_slab_taps(sm.rec[slot][t], i < nmine, slabs, gzeros, lx, rowl,
                       pol, out);
      };
      auto coef = [&](int t) -> const Coef<Real>& { return sm.cf[slot][t]; };
      for (int i = 0; i < n; i += 3) {
        const int tA = pick(i);
        R2 ta[kRows];
        taps(i, tA, ta);
        if (n - i >= 2) {
          const int tB = pick(i + 1);
          R2 tb[kRows];
          taps(i + 1, tB, tb);
          if (n - i >= 3) {
            const int tC = pick(i + 2);
            R2 tc[kRows];
            taps(i + 2, tC, tc);
            accumulate<Real>(coef(tA), ta, acc, acq);
            accumulate<Real>(coef(tB), tb, acc, acq);
            accumulate<Real>(coef(tC), tc, acc, acq);
          } else {
            accumulate<Real>(coef(tA), ta, acc, acq);
            accumulate<Real>(coef(tB), tb, acc, acq);
          }
        } else {
          accumulate<Real>(coef(tA), ta, acc, acq);
        }
      }
      __syncwarp();
    } else
    // ---- this warp's records: those whose footprint meets its band ------
    for (int c0 = 0; c0 < nb; c0 += 32) {
      const bool touch =
          c0 + lane < nb && (sm.band[slot][c0 + lane] & warp_bits) != 0u;
      uint32_t m = __ballot_sync(0xffffffffu, touch);
      // Up to three records at a time (FP32; two for FP64, whose taps take
      // twice the registers): 3 * kRows independent tap loads per lane in
      // flight.  Each cell takes the records in queue order.
      while (m) {
        const int tA = c0 + __ffs(m) - 1;
        m &= m - 1;
        R2 ta[kRows];
        load_record<Real, TW, kStage>(sm, slot, tA, slabs, gzeros, my_bit,
                                      lx, rowl, pol, ta);
        if (m) {
          const int tB = c0 + __ffs(m) - 1;
          m &= m - 1;
          R2 tb[kRows];
          load_record<Real, TW, kStage>(sm, slot, tB, slabs, gzeros, my_bit,
                                        lx, rowl, pol, tb);
          if (sizeof(Real) == 4 && m) {
            const int tC = c0 + __ffs(m) - 1;
            m &= m - 1;
            R2 tc[kRows];
            load_record<Real, TW, kStage>(sm, slot, tC, slabs, gzeros,
                                          my_bit, lx, rowl, pol, tc);
            accumulate<Real>(sm.cf[slot][tA], ta, acc, acq);
            accumulate<Real>(sm.cf[slot][tB], tb, acc, acq);
            accumulate<Real>(sm.cf[slot][tC], tc, acc, acq);
          } else {
            accumulate<Real>(sm.cf[slot][tA], ta, acc, acq);
            accumulate<Real>(sm.cf[slot][tB], tb, acc, acq);
          }
        } else {
          accumulate<Real>(sm.cf[slot][tA], ta, acc, acq);
        }
      }
    }
    if constexpr (kCompensate) {
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        R2 hi = sm.hi[r][threadIdx.x], lo = sm.lo[r][threadIdx.x];
        const float re = __fadd_rn(acc[r].x, acq[r].y);
        const float im = __fadd_rn(acq[r].x, acc[r].y);
        float s, e;
        two_sum(hi.x, re, s, e); hi.x = s; lo.x += e;
        two_sum(hi.y, im, s, e); hi.y = s; lo.y += e;
        sm.hi[r][threadIdx.x] = hi;
        sm.lo[r][threadIdx.x] = lo;
        acc[r].x = acc[r].y = acq[r].x = acq[r].y = 0;
      }
    }
    if (head.z & 2) {  // last buffer of the work item: flush its tile
      const WorkItem item = a.items[head.x];
      const int rt = item.tile % a.geom.tiles_total;   // real tile
      const int gi = rt / tiles_per_grid;
      const int tl = rt - gi * tiles_per_grid;
      const int vg = item.tile / a.geom.tiles_total;   // virtual group
      const int u0 = (tl % a.geom.tiles_u) * WS::kTileU - phase_shift(a.geom, vg);
      const int v0 = (tl / a.geom.tiles_u) * WS::kTileV;
      R2 out[kRows];
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        if constexpr (kCompensate) {
          const R2 hi = sm.hi[r][threadIdx.x], lo = sm.lo[r][threadIdx.x];
          out[r].x = hi.x + lo.x;
          out[r].y = hi.y + lo.y;
        } else {
          out[r] = acc[r];
        }
      }
      const int col = u0 + lx;
      if (item.slot < 0) {
        // Phase tiles reach past the grid's first and last columns.
        const bool col_in = (unsigned)col < (unsigned)G_size;
        R2 *src, *dst;
        cell_ends<R2>(a.tile_groups, a.geom, tl / a.geom.tiles_u,
                      col_in ? col : 0, vg,
                      (R2*)(a.grid + (long long)gi * a.grid_stride),
                      (R2*)a.host, src, dst);
#pragma unroll
        for (int r = 0; r < kRows; ++r) {
          const int row = v0 + rowl + r;
          if (row < G_size && col_in) {
            const size_t off = (size_t)row * G_size + col;
            R2 old = __ldcs(src + off);
            old.x += out[r].x;
            old.y += out[r].y;
            __stcs(dst + off, old);
          }
        }
      } else {
        // Partial tile, thread-major: entry r * kConsumers + thread.
        R2* p = a.partials + (size_t)item.slot * kCells;
#pragma unroll
        for (int r = 0; r < kRows; ++r)
          __stcs(p + r * kConsumers + threadIdx.x, out[r]);
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.empty[slot]);
  }
}

// grid(tile) += sum of the tile's partials in chunk order, accumulated in
// FP64 and rounded once, for the split tiles of one plane group (a real
// tile is split at most once per group, so the blocks of one launch never
// share a tile).  The partial layout is the kernel's thread-major one:
// entry e = r * kConsumers + consumer thread.
template <typename Real, int TW>
__global__ void k_reduce_partials(const int4* __restrict__ split_tiles,
                                  const uint32_t* __restrict__ num_split,
                                  const typename Vec2<Real>::type* __restrict__ partials,
                                  TileGeom g, int group, int G, Real* grid,
                                  long long grid_stride, Real* host,
                                  const uint32_t* __restrict__ tile_groups) {
  using R2 = typename Vec2<Real>::type;
  using WS = WarpShape<TW>;
  const int tiles_per_grid = g.tiles_u * g.tiles_v;
  const int n = (int)*num_split;
  for (int st = blockIdx.x; st < n; st += gridDim.x) {
    const int4 d = split_tiles[st];  // virtual tile, first slot, chunks
    if (d.x / g.tiles_total != group) continue;
    const int rt = d.x % g.tiles_total;
    const int gi = rt / tiles_per_grid;
    const int tl = rt - gi * tiles_per_grid;
    const int u0 = (tl % g.tiles_u) * WS::kTileU - phase_shift(g, group);
    const int v0 = (tl / g.tiles_u) * WS::kTileV;
    R2* const gg = (R2*)(grid + (long long)gi * grid_stride);
    for (int e = threadIdx.x; e < kCells; e += blockDim.x) {
      const int r = e / kConsumers, t = e % kConsumers;
      const int w = t >> 5, ln = t & 31;
      const int row = v0 + w * WS::kBand + (ln / TW) * kRows + r;
      const int col = u0 + ln % TW;
      if (row >= G || (unsigned)col >= (unsigned)G) continue;
      R2 *src, *dst;
      cell_ends<R2>(tile_groups, g, tl / g.tiles_u, col, group, gg,
                    (R2*)host, src, dst);
      const size_t off = (size_t)row * G + col;
      const R2 old = src[off];
      double sx = old.x, sy = old.y;
      for (int c = 0; c < d.z; ++c) {
        const R2 q = partials[(size_t)(d.y + c) * kCells + e];
        sx += q.x;
        sy += q.y;
      }
      R2 nw;
      nw.x = (Real)sx;
      nw.y = (Real)sy;
      dst[off] = nw;
    }
  }
}

// The partial tiles of one plane group's tile phases (virtual groups
// group0 .. group0 + P - 1, one launch of the gridding kernel), added to
// the grids in one pass: block b takes the cells of phase-0 tile position
// b and adds to each cell, phase by phase, the partial tiles of the tile of
// that phase that covers it (their chunks summed in FP64, rounded once per
// phase) -- the additions, in the same order, that one reduction launch per
// phase makes (k_reduce_partials).  A single chunk is added in the grid's
// precision: the FP64 sum of two FP32 values rounded to FP32 is their
// correctly rounded FP32 sum.  tile_slot[virtual tile] = (first partial
// slot, chunks), chunks 0 when the tile has no partial tiles.  Each thread
// keeps one column (blockDim.x a multiple of TW) and looks its phases'
// tiles up once.  kMaxPhases >= tile_phases (4 or 8: the lookups of eight
// phases take registers that four do not need).
template <typename Real, int TW, int kMaxPhases>
__global__ void __launch_bounds__(256)
k_reduce_phases(const int2* __restrict__ tile_slot,
                const typename Vec2<Real>::type* __restrict__ partials,
                TileGeom g, int group0, int G, Real* grid,
                long long grid_stride, Real* host,
                const uint32_t* __restrict__ tile_groups,
                const uint32_t* __restrict__ tile_start) {
  using R2 = typename Vec2<Real>::type;
  using WS = WarpShape<TW>;
  constexpr int kTV = WS::kTileV;
  constexpr int kRowStep = 256 / TW;    // rows between a thread's cells
  const int P = g.tile_phases;
  const int sw = 1 << g.strip_shift;
  const int real_u = g.tiles_u - 1;   // phase-0 tile columns
  const int tiles_per_grid = g.tiles_u * g.tiles_v;
  const int n = g.num_grids * real_u * g.tiles_v;
  const int C = threadIdx.x % TW, R0 = threadIdx.x / TW;
  for (int b = blockIdx.x; b < n; b += gridDim.x) {
    const int gi = b / (real_u * g.tiles_v);
    const int rem = b - gi * real_u * g.tiles_v;
    const int tv = rem / real_u, tu = rem - (rem / real_u) * real_u;
    const int col = tu * TW + C;
    // This column's tile in each phase: its slots and its column there.
    int2 sl[kMaxPhases];
    int cp[kMaxPhases];
    bool mine = false;
#pragma unroll
    for (int p = 0; p < kMaxPhases; ++p) {
      sl[p] = make_int2(0, 0);
      cp[p] = 0;
      if (p < P) {
        const int c = col + p * sw;
        const int tc = c / TW;
        cp[p] = c - tc * TW;
        sl[p] = tile_slot[(size_t)(group0 + p) * g.tiles_total +
                          (size_t)gi * tiles_per_grid +
                          (size_t)tv * g.tiles_u + tc];
        mine |= sl[p].y > 0;
      }
    }
    if (!__syncthreads_or(mine)) continue;
    if (!mine || col >= G) continue;
    R2* gg = (R2*)(grid + (long long)gi * grid_stride);
    // Direct mode (the caller's grid at host in place, one grid): the
    // column's strip was last added to at host unless phase 0's tile here
    // added itself to the scratch grid in the launch (it had records, one
    // item) or an earlier plane group touched the strip; the additions
    // here are the strip's last when its last virtual group is in this
    // launch.
    R2* src = gg;
    R2* dst = gg;
    if (tile_groups) {
      const uint32_t fl =
          tile_groups[tv * g.strips_u + (col >> g.strip_shift)];
      const int first = (int)(fl & 0xFFFFu), last = (int)(fl >> 16);
      const size_t vt0 = (size_t)group0 * g.tiles_total +
                         (size_t)gi * tiles_per_grid +
                         (size_t)tv * g.tiles_u + tu;
      const bool added0 =
          sl[0].y == 0 && tile_start[vt0 + 1] > tile_start[vt0];
      if (!added0 && first >= group0) src = (R2*)host;
      if (last < group0 + P) dst = (R2*)host;
    }
    if constexpr (sizeof(Real) == 4 && kMaxPhases <= 4) {
      bool several = false;
#pragma unroll
      for (int p = 0; p < kMaxPhases; ++p) several |= sl[p].y > 1;
      if (!several) {
        // Every phase adds at most one chunk to this column: all of the
        // thread's loads (its rows of the grid and of up to kMaxPhases
        // partial tiles) go out before the first addition, so the block
        // waits out one memory latency rather than one per row.  The
        // additions are the loop's below, in the same order.
        constexpr int kRowsPer = kTV / kRowStep;
        R2 acc[kRowsPer], pv[kMaxPhases][kRowsPer];
#pragma unroll
        for (int i = 0; i < kRowsPer; ++i) {
          const int R = R0 + i * kRowStep;
          const int row = tv * kTV + R;
          const bool in = row < G;
          const int w = R / WS::kBand, ly = (R % WS::kBand) / kRows;
          const int ent0 = (R % kRows) * kConsumers + w * 32 + ly * TW;
          acc[i] = in ? src[(size_t)row * G + col] : R2{};
#pragma unroll
          for (int p = 0; p < kMaxPhases; ++p)
            pv[p][i] = in && sl[p].y > 0
                           ? partials[(size_t)sl[p].x * kCells + ent0 + cp[p]]
                           : R2{};
        }
#pragma unroll
        for (int i = 0; i < kRowsPer; ++i) {
          const int row = tv * kTV + R0 + i * kRowStep;
          if (row >= G) break;
#pragma unroll
          for (int p = 0; p < kMaxPhases; ++p) {
            if (sl[p].y == 0) continue;
            acc[i].x += pv[p][i].x;
            acc[i].y += pv[p][i].y;
          }
          dst[(size_t)row * G + col] = acc[i];
        }
        continue;
      }
    }
#pragma unroll 4
    for (int R = R0; R < kTV; R += kRowStep) {
      const int row = tv * kTV + R;
      if (row >= G) break;
      // The cell's entry in a partial tile whose column is Cp (the
      // kernel's thread-major layout: row R is warp R / kBand, lane row
      // (R % kBand) / kRows, register row R % kRows).
      const int w = R / WS::kBand, ly = (R % WS::kBand) / kRows;
      const int ent0 = (R % kRows) * kConsumers + w * 32 + ly * TW;
      R2 acc = src[(size_t)row * G + col];
#pragma unroll
      for (int p = 0; p < kMaxPhases; ++p) {
        if (sl[p].y == 0) continue;
        const R2* q = partials + (size_t)sl[p].x * kCells + ent0 + cp[p];
        if (sl[p].y == 1) {
          const R2 v = *q;
          acc.x += v.x;
          acc.y += v.y;
        } else {
          double sx = acc.x, sy = acc.y;
          for (int k = 0; k < sl[p].y; ++k) {
            const R2 v = q[(size_t)k * kCells];
            sx += v.x;
            sy += v.y;
          }
          acc.x = (Real)sx;
          acc.y = (Real)sy;
        }
      }
      dst[(size_t)row * G + col] = acc;
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

// Per tile row of a single grid, the strips (tile_u / tile_phases columns)
// that virtual tiles with records cover: [lo, hi).
__global__ void k_touched_spans(const uint32_t* __restrict__ tile_start,
                                int num_tiles, int tiles_total, int tiles_u,
                                int phases, int strips_u,
                                uint32_t* __restrict__ lo,
                                uint32_t* __restrict__ hi) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < num_tiles;
       t += gridDim.x * blockDim.x) {
    if (tile_start[t + 1] == tile_start[t]) continue;
    const int r = t % tiles_total;
    const int p = (t / tiles_total) % phases;
    const int a = max((r % tiles_u) * phases - p, 0);
    const int b = min((r % tiles_u) * phases - p + phases, strips_u);
    if (a >= b) continue;
    atomicMin(&lo[r / tiles_u], (uint32_t)a);
    atomicMax(&hi[r / tiles_u], (uint32_t)b);
  }
}

// out[tv * strips_u + sc] = first | last << 16: the first and last virtual
// group whose tiles hold records in strip sc (tile_u / tile_phases columns)
// of tile row tv (0xFFFF | 0xFFFF << 16 when none), for a single grid.  In
// phase p the strip lies in tile column (sc + p) / tile_phases.
// *cells += the grid cells of the strips that have records (clipped to the
// grid), the cells a direct-mode call reads and writes at host.
__global__ void k_tile_groups(const uint32_t* __restrict__ tile_start,
                              TileGeom geom, int G, uint32_t* __restrict__ out,
                              unsigned long long* cells) {
  const int P = geom.tile_phases > 1 ? geom.tile_phases : 1;
  const int sw = 1 << geom.strip_shift;
  const int strips_u = geom.strips_u;
  const int n = strips_u * geom.tiles_v;
  unsigned long long mine = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const int tv = i / strips_u, sc = i % strips_u;
    uint32_t first = 0xFFFFu, last = 0xFFFFu;
    for (int g = 0; g < geom.num_groups; ++g) {
      const int tc = (sc + g % P) / P;
      const size_t v =
          (size_t)g * geom.tiles_total + (size_t)tv * geom.tiles_u + tc;
      if (tile_start[v + 1] > tile_start[v]) {
        if (first == 0xFFFFu) first = (uint32_t)g;
        last = (uint32_t)g;
      }
    }
    out[i] = first | (last << 16);
    if (first != 0xFFFFu) {
      const int u0 = sc * sw, v0 = tv * geom.tile_v;
      mine += (unsigned long long)min(sw, G - u0) * min(geom.tile_v, G - v0);
    }
  }
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, o);
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(cells, mine);
}

// Failure-path probe: every thread waits, bounded by `limit` probes, on an
// mbarrier that nothing arrives at -- the wait the gridding kernels use --
// so the wait runs out, the kernel sets the error flag and returns.
__global__ void k_wait_probe(unsigned limit, uint32_t* __restrict__ error) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  const bool ok = mbar_wait(&bar, 0, limit);
  if (!ok && threadIdx.x == 0) atomicExch(error, 1u);
}

// Virtual tile at queue rank i (see ItemBuffers::tile_order).
__device__ __forceinline__ int tile_at_rank(int i, int T,
                                            const int* __restrict__ order) {
  if (!order) return i;
  const int g = i / T;
  return g * T + order[i - g * T];
}

// Counts per queue rank i (tile t = tile_at_rank(i)):
// A[i] = chunks of t if it writes partial tiles (more than one chunk, or
// any chunk of a later tile phase), else 0;
// B[i] = 1 if t owns its tile in one chunk.
__global__ void k_item_counts(const uint32_t* __restrict__ tile_start,
                              int num_tiles, int num_groups,
                              const int* __restrict__ order, uint32_t chunk,
                              int partial_phases,
                              uint32_t* __restrict__ A,
                              uint32_t* __restrict__ B) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= num_tiles) return;
  const int T = num_tiles / num_groups;
  const int t = tile_at_rank(i, T, order);
  const uint32_t c = tile_start[t + 1] - tile_start[t];
  const uint32_t chunks = (c + chunk - 1) / chunk;
  // Later tile phases always write partial tiles (see ItemBuffers).
  const bool split = chunks > 1 || (chunks == 1 && (i / T) % partial_phases);
  A[i] = split ? chunks : 0;
  B[i] = split ? 0 : chunks;
}

// The queue is group-major (see ItemBuffers); within virtual group g the
// chunks of split tiles (every tile of a later tile phase counts as split)
// come first (they are the largest items), then the single-chunk tiles,
// each part in rank order.  With exclusive scans sA
// (split chunks) and sB (single-chunk tiles) over the ranks, group g
// starts at sA[gT] + sB[gT] (T = tiles per group), split chunk j of rank i
// sits at sA[i] + sB[gT] + j and single rank i at sA[(g+1)T] + sB[i].
// Partial slot of a split chunk = sA[i] + j.
__global__ void k_item_emit(const uint32_t* __restrict__ tile_start,
                            int num_tiles, int num_groups,
                            const int* __restrict__ order, uint32_t chunk,
                            int partial_phases,
                            const uint32_t* __restrict__ sA,
                            const uint32_t* __restrict__ sB,
                            const uint32_t* __restrict__ totA,
                            const uint32_t* __restrict__ totB,
                            WorkItem* __restrict__ items,
                            int4* __restrict__ split_tiles,
                            uint32_t* __restrict__ num_split,
                            uint32_t* __restrict__ num_items,
                            uint32_t* __restrict__ group_items,
                            int2* __restrict__ tile_slot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int T = num_tiles / num_groups;
  auto scanA = [&](int r) { return r < num_tiles ? sA[r] : *totA; };
  auto scanB = [&](int r) { return r < num_tiles ? sB[r] : *totB; };
  if (i == 0) *num_items = *totA + *totB;
  if (i <= num_groups) group_items[i] = scanA(i * T) + scanB(i * T);
  if (i >= num_tiles) return;
  const int g = i / T;
  const int t = tile_at_rank(i, T, order);
  const uint32_t s0 = tile_start[t], s1 = tile_start[t + 1];
  const uint32_t c = s1 - s0;
  const uint32_t chunks = (c + chunk - 1) / chunk;
  const bool owns = chunks == 1 && g % partial_phases == 0;
  if (tile_slot)
    tile_slot[t] = c == 0 || owns ? make_int2(0, 0)
                                  : make_int2((int)sA[i], (int)chunks);
  if (c == 0) return;
  if (owns) {
    WorkItem w;
    w.tile = t; w.rec_begin = (int)s0; w.rec_end = (int)s1; w.slot = -1;
    items[scanA((g + 1) * T) + sB[i]] = w;
  } else {
    const uint32_t first = sA[i];
    const uint32_t pos = first + scanB(g * T);
    for (uint32_t j = 0; j < chunks; ++j) {
      WorkItem w;
      w.tile = t;
      w.rec_begin = (int)(s0 + j * chunk);
      w.rec_end = (int)min(s1, s0 + (j + 1) * chunk);
      w.slot = (int)(first + j);
      items[pos + j] = w;
    }
    const uint32_t k = atomicAdd(num_split, 1u);
    split_tiles[k] = make_int4(t, (int)first, (int)chunks, 0);
  }
}

template <typename Real, int TW, bool kStage, bool kHalves = false>
void* grid_kernel_ptr() {
  return (void*)k_grid_tiles<Real, std::is_same<Real, float>::value, TW,
                             kStage, kHalves>;
}

// The kernels take more than 48 KB of dynamic shared memory: opt in before
// querying occupancy or launching.  The opt-in is made once per device, so
// later launches (replays captured in a CUDA graph among them) make no
// attribute call.
template <typename Real, int TW, bool kStage, bool kHalves = false>
cudaError_t prepare_grid_kernel(void** fn, size_t* smem) {
  static std::atomic<unsigned long long> opted_in{0};
  *fn = grid_kernel_ptr<Real, TW, kStage, kHalves>();
  *smem = sizeof(Smem<Real, kStage>);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (dev < 64 && (opted_in.load() & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(*fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)*smem);
  if (e == cudaSuccess && dev < 64) opted_in.fetch_or(bit);
  return e;
}

template <typename Real>
cudaError_t prepare_grid_kernel_for(int tile_u, bool stage, void** fn,
                                    size_t* smem, int lane_groups = 1) {
  if (lane_groups == 2 && tile_u == 32 && !stage)
    return prepare_grid_kernel<Real, 32, false, true>(fn, smem);
  if (stage)
    return tile_u == 32   ? prepare_grid_kernel<Real, 32, true>(fn, smem)
           : tile_u == 16 ? prepare_grid_kernel<Real, 16, true>(fn, smem)
                          : prepare_grid_kernel<Real, 8, true>(fn, smem);
  return tile_u == 32   ? prepare_grid_kernel<Real, 32, false>(fn, smem)
         : tile_u == 16 ? prepare_grid_kernel<Real, 16, false>(fn, smem)
                        : prepare_grid_kernel<Real, 8, false>(fn, smem);
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

cudaError_t launch_wait_probe(unsigned limit, uint32_t* error,
                              cudaStream_t s) {
  k_wait_probe<<<1, 64, 0, s>>>(limit, error);
  return cudaGetLastError();
}

cudaError_t launch_tile_groups(const uint32_t* tile_start,
                               const TileGeom& geom, int grid_size,
                               uint32_t* out, unsigned long long* cells,
                               cudaStream_t s) {
  const int n = num_strips(geom);
  const int blocks = std::min(1024, (n + 255) / 256);
  k_tile_groups<<<blocks < 1 ? 1 : blocks, 256, 0, s>>>(tile_start, geom,
                                                        grid_size, out, cells);
  return cudaGetLastError();
}

cudaError_t launch_touched_spans(const uint32_t* tile_start, int num_tiles,
                                 const TileGeom& geom, int grid_size,
                                 uint32_t* lo, uint32_t* hi, cudaStream_t s) {
  (void)grid_size;
  const int P = geom.tile_phases > 1 ? geom.tile_phases : 1;
  const int blocks = std::max(1, std::min((num_tiles + 255) / 256, 4096));
  k_touched_spans<<<blocks, 256, 0, s>>>(tile_start, num_tiles,
                                         geom.tiles_total, geom.tiles_u, P,
                                         geom.strips_u, lo, hi);
  return cudaGetLastError();
}

cudaError_t launch_build_items(const uint32_t* tile_start, int num_tiles,
                               uint32_t num_records, uint32_t chunk,
                               ItemBuffers b, cudaStream_t s) {
  (void)num_records;
  uint32_t* A = b.chunks;
  uint32_t* B = b.split_chunks;
  const int blocks = (num_tiles + 256) / 256;   // one more thread: bounds
  const int pp = b.partial_phases > 1 ? b.partial_phases : 1;
  k_item_counts<<<blocks, 256, 0, s>>>(tile_start, num_tiles, b.num_groups,
                                       b.tile_order, chunk, pp, A, B);
  cudaError_t e;
  e = exclusive_scan_u32(A, A, num_tiles, b.num_slots, b.scan_tmp, s);
  if (e != cudaSuccess) return e;
  // The work counter doubles as scratch for B's total until k_item_emit.
  e = exclusive_scan_u32(B, B, num_tiles, b.counter, b.scan_tmp, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(b.num_split, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  k_item_emit<<<blocks, 256, 0, s>>>(tile_start, num_tiles, b.num_groups,
                                     b.tile_order, chunk, pp, A, B,
                                     b.num_slots,
                                     b.counter,
                                     b.items, b.split_tiles, b.num_split,
                                     b.num_items, b.group_items,
                                     b.tile_slot);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // The persistent kernel's work counter starts at zero.
  return cudaMemsetAsync(b.counter, 0, sizeof(uint32_t), s);
}

template <typename Real>
int grid_tiles_ctas_per_sm(int tile_u, bool stage, int lane_groups) {
  void* fn = nullptr;
  size_t smem = 0;
  int n = 0;
  if (prepare_grid_kernel_for<Real>(tile_u, stage, &fn, &smem,
                                    lane_groups) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kThreads,
                                                    smem) != cudaSuccess)
    n = 1;
  return n < 1 ? 1 : n;
}

template <typename Real>
cudaError_t launch_reduce_phases(const int2* tile_slot, const Real* partials,
                                 TileGeom geom, int group0, int grid_size,
                                 Real* grid, long long grid_stride,
                                 Real* host, const uint32_t* tile_groups,
                                 const uint32_t* tile_start, cudaStream_t s) {
  const long long n =
      (long long)geom.num_grids * (geom.tiles_u - 1) * geom.tiles_v;
  if (n <= 0) return cudaSuccess;
  if (geom.tile_phases > 8) return cudaErrorInvalidValue;
  const int blocks = (int)std::min<long long>(n, 65535);
  using P2 = const typename Vec2<Real>::type*;
  const bool eight = geom.tile_phases > 4;
#define GG_REDUCE_PHASES(TW_, MP_)                                          \
  k_reduce_phases<Real, TW_, MP_><<<blocks, 256, 0, s>>>(                   \
      tile_slot, (P2)partials, geom, group0, grid_size, grid, grid_stride, \
      host, tile_groups, tile_start)
  switch (geom.tile_u) {
    case 32:
      if (eight) GG_REDUCE_PHASES(32, 8); else GG_REDUCE_PHASES(32, 4);
      break;
    case 16:
      if (eight) GG_REDUCE_PHASES(16, 8); else GG_REDUCE_PHASES(16, 4);
      break;
    case 8:
      if (eight) GG_REDUCE_PHASES(8, 8); else GG_REDUCE_PHASES(8, 4);
      break;
    default: return cudaErrorInvalidValue;
  }
#undef GG_REDUCE_PHASES
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_reduce_group(const int4* split_tiles,
                                const uint32_t* num_split, int max_split,
                                const Real* partials, TileGeom geom, int group,
                                int grid_size, Real* grid,
                                long long grid_stride, Real* host,
                                const uint32_t* tile_groups, cudaStream_t s) {
  if (max_split <= 0) return cudaSuccess;
  const int blocks = std::min(max_split, 4096);
  using P2 = const typename Vec2<Real>::type*;
  switch (geom.tile_u) {
    case 32: k_reduce_partials<Real, 32><<<blocks, 256, 0, s>>>(
        split_tiles, num_split, (P2)partials, geom, group, grid_size, grid,
        grid_stride, host, tile_groups); break;
    case 16: k_reduce_partials<Real, 16><<<blocks, 256, 0, s>>>(
        split_tiles, num_split, (P2)partials, geom, group, grid_size, grid,
        grid_stride, host, tile_groups); break;
    case 8: k_reduce_partials<Real, 8><<<blocks, 256, 0, s>>>(
        split_tiles, num_split, (P2)partials, geom, group, grid_size, grid,
        grid_stride, host, tile_groups); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_grid_tiles(const WorkItem* items,
                              const uint32_t* group_items,
                              uint32_t* counter, uint32_t* error,
                              const uint32_t* rec_vis,
                              const uint32_t* cell, const uint32_t* meta,
                              const void* vw, StackView view, TileGeom geom,
                              int grid_size, Real* grid, long long grid_stride,
                              Real* partials, const int4* split_tiles,
                              const uint32_t* num_split, int max_split,
                              int num_ctas, bool stage, cudaStream_t s,
                              const cudaEvent_t* wait_before,
                              const cudaEvent_t* record_after,
                              Real* host_grid, const uint32_t* tile_groups,
                              int group_span, const int2* tile_slot,
                              const uint32_t* tile_start) {
  GridArgs<Real> a;
  a.items = items;
  a.group_items = group_items;
  a.group = 0;
  a.counter = counter;
  a.error = error;
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
  a.host = tile_groups ? host_grid : grid;
  a.tile_groups = tile_groups;
  if (geom.tile_u != 32 && geom.tile_u != 16 && geom.tile_u != 8)
    return cudaErrorInvalidValue;
  void* fn = nullptr;
  size_t smem = 0;
  cudaError_t e = prepare_grid_kernel_for<Real>(geom.tile_u, stage, &fn,
                                                &smem, geom.lane_groups);
  if (e != cudaSuccess) return e;
  void* args[] = {&a};
  const int span = group_span > 1 ? group_span : 1;
  a.group_span = span;
  for (int g = 0; g < geom.num_groups; g += span) {
    a.group = g;
    if (wait_before && wait_before[g]) {
      e = cudaStreamWaitEvent(s, wait_before[g], 0);
      if (e != cudaSuccess) return e;
    }
    e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    e = cudaLaunchKernel(fn, dim3(num_ctas), dim3(kThreads), args, smem, s);
    if (e != cudaSuccess) return e;
    if (span > 1 && tile_slot) {
      e = launch_reduce_phases<Real>(tile_slot, partials, geom, g, grid_size,
                                     grid, grid_stride, a.host, tile_groups,
                                     tile_start, s);
      if (e != cudaSuccess) return e;
    } else {
      for (int p = 0; p < span; ++p) {
        e = launch_reduce_group<Real>(split_tiles, num_split, max_split,
                                      partials, geom, g + p, grid_size, grid,
                                      grid_stride, a.host, tile_groups, s);
        if (e != cudaSuccess) return e;
      }
    }
    if (record_after && record_after[g + span - 1]) {
      e = cudaEventRecord(record_after[g + span - 1], s);
      if (e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

template int grid_tiles_ctas_per_sm<float>(int, bool, int);
template int grid_tiles_ctas_per_sm<double>(int, bool, int);
template cudaError_t launch_grid_tiles<float>(
    const WorkItem*, const uint32_t*, uint32_t*, uint32_t*, const uint32_t*,
    const uint32_t*, const uint32_t*, const void*, StackView, TileGeom, int,
    float*, long long, float*, const int4*, const uint32_t*, int, int, bool,
    cudaStream_t, const cudaEvent_t*, const cudaEvent_t*, float*,
    const uint32_t*, int, const int2*, const uint32_t*);
template cudaError_t launch_grid_tiles<double>(
    const WorkItem*, const uint32_t*, uint32_t*, uint32_t*, const uint32_t*,
    const uint32_t*, const uint32_t*, const void*, StackView, TileGeom, int,
    double*, long long, double*, const int4*, const uint32_t*, int, int, bool,
    cudaStream_t, const cudaEvent_t*, const cudaEvent_t*, double*,
    const uint32_t*, int, const int2*, const uint32_t*);

}  // namespace gg
