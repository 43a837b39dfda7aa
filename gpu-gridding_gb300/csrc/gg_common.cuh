// Shared definitions of the GB300 gridder's CUDA sources.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

namespace gg {

// ---------------------------------------------------------------------------
// Limits of this build.
// ---------------------------------------------------------------------------
// Cell coordinates are packed as two 16-bit fields, so grid_size <= 65535.
constexpr int kMaxGridSize = 65535;
// Oversampled offsets are stored biased by 8 in 4-bit fields: |off| <= 7,
// i.e. oversample <= 14 (|off| <= (oversample + 1) / 2).
constexpr int kMaxOversample = 14;
// W-plane index is a 16-bit field.
constexpr int kMaxPlanes = 65535;

// Packed placement of one visibility (written by the placement kernel).
//   cell: u in bits 0-15, v in bits 16-31
//   meta: plane in bits 0-15, (off_u + 8) in 16-19, (off_v + 8) in 20-23,
//         conj_neg in bit 24, skipped in bit 25
__host__ __device__ inline uint32_t pack_cell(int u, int v) {
  return (uint32_t)(u & 0xFFFF) | ((uint32_t)(v & 0xFFFF) << 16);
}
__host__ __device__ inline int cell_u(uint32_t c) { return (int)(c & 0xFFFF); }
__host__ __device__ inline int cell_v(uint32_t c) { return (int)(c >> 16); }
__host__ __device__ inline uint32_t pack_meta(int plane, int ou, int ov,
                                              int conj_neg, int skipped) {
  return (uint32_t)plane | ((uint32_t)(ou + 8) << 16) |
         ((uint32_t)(ov + 8) << 20) | ((uint32_t)conj_neg << 24) |
         ((uint32_t)skipped << 25);
}
__host__ __device__ inline int meta_plane(uint32_t m) { return (int)(m & 0xFFFF); }
__host__ __device__ inline int meta_ou(uint32_t m) { return (int)((m >> 16) & 0xF) - 8; }
__host__ __device__ inline int meta_ov(uint32_t m) { return (int)((m >> 20) & 0xF) - 8; }
__host__ __device__ inline int meta_conj(uint32_t m) { return (int)((m >> 24) & 1); }
__host__ __device__ inline int meta_skipped(uint32_t m) { return (int)((m >> 25) & 1); }

// Two-component vector of the call's precision (complex value, re/im).
template <typename Real>
struct Vec2;
template <>
struct Vec2<float> { using type = float2; };
template <>
struct Vec2<double> { using type = double2; };

// ---------------------------------------------------------------------------
// Re-laid kernel stack: one dense slice per (plane, |offset| class).
// ---------------------------------------------------------------------------
// The reference stores, per plane, the first quadrant K[t][c] of an
// oversampled kernel and reads the tap of footprint cell (j, k) at
// t = |off_v + j*os|, c = |off_u + k*os| (oskar_grid_wproj.c:196-203).  For
// a given offset those taps form a (2s+1)^2 matrix; the device copy stores
// that matrix explicitly, for every plane and every absolute offset class
// (cu, cv) in [0, omax]^2:
//   S[jj][kk] = K[|cv + (jj - s)*os|][|cu + (kk - s)*os|],  jj, kk in [0, 2s]
// at slice_base(p, cu, cv) = base[p] + (cu*(omax+1) + cv) * F^2, F = 2s+1.
// A negative offset reads the mirrored slice: |-c + k*os| = |c + (-k)*os|,
// so the tap of (j, k) for offsets (ou, ov) is
//   S_{|ou|,|ov|}[s + sgn(ov)*j][s + sgn(ou)*k].
// Each slice is contiguous (one bulk copy stages it in shared memory) and a
// warp whose lanes hold consecutive k reads consecutive words.  Every slice
// carries kSlicePad zero rows above and below, so a lane whose kRows
// consecutive cells straddle the footprint's top or bottom edge reads zeros
// there instead of testing each row.
constexpr int kSlicePad = 7;

struct StackView {
  int num_planes;
  int oversample;
  int omax;                 // (oversample + 1) / 2: largest |offset|
  int conv_size_half;
  const int* support;       // [P]
  const long long* base;    // [P] first tap of plane p (complex units)
  const void* taps;         // float2 or double2
  const double* tap_sum;    // [P][2*omax+1][2*omax+1] sum of Re(tap), FP64
  const void* zeros;        // middle of a zero buffer that any lane's rows
                            // (kRows rows of any slice stride) stay inside
  const long long* sbase;   // [P] first tap of plane p in the slab stack
  const void* slabs;        // slab stack (see below)
};

// ---------------------------------------------------------------------------
// Slab stack: footprint rows in order, columns residue-major.
// ---------------------------------------------------------------------------
// For plane p and row class c = |off_v| in [0, omax] a slab holds the
// footprint's rows j = -s..s in order, each the quadrant row
// t = |c + j*os|, with kSlicePad zero rows before and after:
//   slab_{p,c}[kSlicePad + j + s][r][m] = K_p[|c + j*os|][r + m*os]
// for residues r in [0, os) and lattice indices m in [0, M), M = s + 1
// (+1 when omax >= os, i.e. os = 1).  A negative off_v reads the slab's
// rows in reverse (|-c + j*os| = |c + (-j)*os|).  Rows are stored by column
// residue: the tap of footprint column k for offset ou is
// K[.][|ou + k*os|], and on either side of the fold ou + k*os = 0 that
// column has one residue and a lattice index that moves by one per column,
// so a warp's lanes (consecutive k) read at most two contiguous runs of a
// row, and a lane's rows are evenly spaced.  Each quadrant row appears in
// the slabs of a plane about 1.5 times (against (omax + 1) times plus the
// column mirror in the per-offset slices above), which keeps the whole
// stack of a large W-projection setup in L2.
__host__ __device__ inline int slab_cols_m(int s, int os, int omax) {
  return s + 1 + (omax >= os ? 1 : 0);
}
// Taps of one slab, rounded up to an even count (16-byte aligned slabs).
__host__ __device__ inline long long slab_taps(int s, int os, int omax) {
  return ((long long)(2 * s + 1 + 2 * kSlicePad) * os *
              slab_cols_m(s, os, omax) + 1) & ~1LL;
}

// Rows and columns of a plane's quadrant cube that the stack preparation
// reads (slices and tap sums: |off| + s*os with |off| <= omax; slabs:
// columns r + m*os with r < os, m < M): the square [0, E)^2 below
// E = min(csh, 1 + max(s*os + omax, M*os - 1)).
__host__ __device__ inline int cube_read_extent(int s, int os, int omax,
                                                int csh) {
  const int a = s * os + omax, b = slab_cols_m(s, os, omax) * os - 1;
  const int e = 1 + (a > b ? a : b);
  return e < csh ? e : csh;
}

// Taps one slice occupies: padding rows included, rounded up to an even
// count so that every slice starts 16-byte aligned (bulk copies need it).
__host__ __device__ inline long long slice_taps(int s) {
  const long long F = 2 * s + 1;
  return ((F + 2 * kSlicePad) * F + 1) & ~1LL;
}

// Index of tap S[0][0] of the slice of plane p for absolute offsets
// (cu, cv) (the padding rows come before it).
__host__ __device__ inline long long slice_offset(long long plane_base,
                                                  int s, int omax, int cu,
                                                  int cv) {
  const long long F = 2 * s + 1;
  return plane_base + (long long)(cu * (omax + 1) + cv) * slice_taps(s) +
         kSlicePad * F;
}

// ---------------------------------------------------------------------------
// Call parameters.
// ---------------------------------------------------------------------------
template <typename Real>
struct PlaceParams {
  const Real* uu;
  const Real* vv;
  const Real* ww;
  const Real* vis;      // interleaved
  const Real* weight;
  Real grid_scale;      // grid_size * cell_size_rad, in the call's precision
  Real w_scale;
  int grid_size;
  int grid_centre;
  unsigned long long num_points;
  // Norm terms left to launch_norm_terms (the kernel stack's tap sums are
  // not ready yet when placement runs).
  bool defer_norm = false;
};

// Tile geometry shared by the binning and gridding kernels.
// With plane groups (num_groups > 1) the records of a call are gridded in
// one pass per group of consecutive w-planes, each group's kernel slabs
// small enough to stay in L2 during its pass; the sort key's tile field is
// then the virtual tile group * tiles_total + tile.
struct TileGeom {
  int tile_u, tile_v;        // cells per tile
  int tiles_u, tiles_v;      // tiles per grid side
  int num_grids;
  int plane_bits, phase_bits;  // low key fields below the tile index
  int phase_side;            // 2*omax+1... stored as omax+1 (|off| classes)
  int num_groups;            // plane groups (passes), >= 1
  int tiles_total;           // num_grids * tiles_u * tiles_v
  const int* plane_group;    // [P] group of each plane (num_groups > 1)
  // > 0: plane groups are gridded in two passes by tile rows (rows below
  // split_tv first) -- the first plane group when bit 0 of split_mask is
  // set, the last one when bit 1 is (single-grid calls).  Virtual groups:
  // [first upper, first lower,] middle groups..., [last upper, last lower];
  // num_groups counts them all.
  int split_tv;
  int split_mask;
  // Record streams per consumer warp of the 32-wide gridding kernel: 1 (or
  // 0) -- the whole warp takes each record that meets its rows; 2 -- each
  // half-warp (16 columns) takes the records that meet its own columns.
  int lane_groups;
  // Tile phases (1, 2, 4 or 8): the tile columns of phase p start p * tile_u /
  // tile_phases cells to the left of phase 0's, and each visibility is
  // gridded on the phase whose tiles cut its footprint into the fewest
  // columns (footprint_phase).  Tiles of different phases overlap, so each
  // phase is a pass of its own: virtual group = group * tile_phases +
  // phase.  With more than one phase tiles_u counts one more column (phase
  // p's first column starts left of the grid, its last may end past it).
  int tile_phases;
  // Strips of tile_u / tile_phases columns (a power of two, 1 << strip_shift)
  // by tile rows: the units in which a single-grid call records which
  // passes touch which cells (strips_u strips per tile row).
  int strip_shift;
  int strips_u;
};

// Columns of the tile grid of virtual group `group` left of phase 0's
// (tile_phases a power of two >= 1; a phase is one strip, 1 << strip_shift
// columns).
__host__ __device__ inline int phase_shift(const TileGeom& g, int group) {
  return (group & (g.tile_phases - 1)) << g.strip_shift;
}

// Phase of a footprint spanning cells [c0, c1] (c0 >= 0) on tiles of
// 1 << tile_shift columns: the one whose tile columns cut it into the
// fewest pieces, the lowest on ties.  Phase p's columns start p strips
// (1 << strip_shift columns) left of phase 0's.
__host__ __device__ inline int footprint_phase(int c0, int c1,
                                               int tile_shift,
                                               int strip_shift, int phases) {
  int best = 0, fewest = (c1 >> tile_shift) - (c0 >> tile_shift);
  for (int p = 1; p < phases; ++p) {
    const int sh = p << strip_shift;
    const int n = ((c1 + sh) >> tile_shift) - ((c0 + sh) >> tile_shift);
    if (n < fewest) {
      fewest = n;
      best = p;
    }
  }
  return best;
}

// Work item of the gridding kernel: a range of sorted records of one tile.
struct WorkItem {
  int tile;        // global tile index (grid * tiles_per_grid + tile)
  int rec_begin;
  int rec_end;
  int slot;        // partial-tile slot, or -1 when the item owns the tile
};

}  // namespace gg
