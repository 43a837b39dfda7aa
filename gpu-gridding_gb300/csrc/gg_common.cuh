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
// Re-laid kernel stack.
// ---------------------------------------------------------------------------
// The reference stores, per plane, the first quadrant K[t][c] of an
// oversampled kernel, t = |off_v + j*os| (row), c = |off_u + k*os| (column)
// (oskar_grid_wproj.c:196-203).  For a given offset the taps a footprint
// needs are every os-th row and column, so the device copy splits each plane
// by residue: index t = rho_v + os*m_v, c = rho_u + os*m_u is stored at
//   base[p] + ((rho_v*os + rho_u)*M[p] + m_v)*M[p] + m_u,
// M[p] = (omax + support[p]*os)/os + 1.  A warp whose lanes hold consecutive
// k then reads consecutive words, and each (rho_v, rho_u) block is a dense
// M x M square that can be staged into shared memory in one bulk copy.
struct StackView {
  int num_planes;
  int oversample;
  int omax;                 // (oversample + 1) / 2: largest |offset|
  int conv_size_half;
  const int* support;       // [P]
  const int* side;          // [P] M[p]
  const long long* base;    // [P] first element of plane p (complex units)
  const void* taps;         // float2 or double2
  const double* tap_sum;    // [P][2*omax+1][2*omax+1] sum of Re(tap), FP64
};

// Residue decomposition of x = |o + k*os| for a fixed signed offset o:
// for o + k*os >= 0, x = rp + os*(k + dp); otherwise x = rn + os*(-k + dn).
struct ResidueSplit {
  int rp, dp, rn, dn;
};
__host__ __device__ inline ResidueSplit residue_split(int o, int os) {
  // floor division and non-negative remainder of o and -o by os.
  ResidueSplit r;
  int q = o >= 0 ? o / os : -((-o + os - 1) / os);
  r.dp = q;
  r.rp = o - q * os;
  int on = -o;
  int qn = on >= 0 ? on / os : -((-on + os - 1) / os);
  r.dn = qn;
  r.rn = on - qn * os;
  return r;
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
};

// Tile geometry shared by the binning and gridding kernels.
struct TileGeom {
  int tile_u, tile_v;        // cells per tile
  int tiles_u, tiles_v;      // tiles per grid side
  int num_grids;
  int plane_bits, phase_bits;  // low key fields below the tile index
  int phase_side;            // 2*omax+1... stored as omax+1 (|off| classes)
};

// Work item of the gridding kernel: a range of sorted records of one tile.
struct WorkItem {
  int tile;        // global tile index (grid * tiles_per_grid + tile)
  int rec_begin;
  int rec_end;
  int slot;        // partial-tile slot, or -1 when the item owns the tile
};

}  // namespace gg
