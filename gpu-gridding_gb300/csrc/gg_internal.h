// Host-side declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stddef.h>

#include "gg_common.cuh"

struct gg_kernels;  // kernel-stack handle of the C ABI (gg_api.cu)

namespace gg {

// ---- device-wide exclusive scan of uint32 (gg_sort.cu) --------------------
// out[i] = in[0] + ... + in[i-1]; *d_total (if non-null) = sum of all n.
// in and out may alias.  tmp must hold scan_temp_bytes(n).
size_t scan_temp_bytes(size_t n);
cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n,
                               uint32_t* d_total, void* tmp, cudaStream_t s);
// *total (device) = sum of in[0..n) in 64 bits.
cudaError_t sum_u32(const uint32_t* in, size_t n, unsigned long long* total,
                    cudaStream_t s);

// ---- stable LSD radix sort of (key, value) pairs (gg_sort.cu) -------------
// Sorts the first n pairs by key bits [0, end_bit).  Ping-pongs between
// (keys, vals) and (keys_alt, vals_alt); on return *in_alt tells which pair
// of buffers holds the result.  tmp must hold radix_temp_bytes(n).
size_t radix_temp_bytes(size_t n);
cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals,
                             uint32_t* keys_alt, uint32_t* vals_alt, size_t n,
                             int end_bit, void* tmp, cudaStream_t s,
                             bool* in_alt);

// ---- kernel stack preparation (gg_stack.cu) -------------------------------
// Re-lays conv_func (device, [P][csh][csh] complex) into the residue-split
// layout and forms the FP64 tap sums in the reference's summation order.
// With `changed` given, each of these kernels returns at once while
// *changed == 0 (a cube equal to the one the outputs were made from).
template <typename Real>
cudaError_t launch_stack_relayout(const Real* d_conv_func, StackView view,
                                  void* d_taps_out, long long total_taps,
                                  cudaStream_t s,
                                  const int* changed = nullptr);
// Fills the slab stack (view.slabs layout, planes at view.sbase).
template <typename Real>
cudaError_t launch_stack_relayout_slabs(const Real* d_conv_func,
                                        StackView view, void* d_out,
                                        cudaStream_t s,
                                        const int* changed = nullptr);
// support_max: the largest support of the stack (sizes the row window).
template <typename Real>
cudaError_t launch_tap_sums(StackView view, double* d_tap_sum,
                            int support_max, cudaStream_t s,
                            const int* changed = nullptr);
// *changed = 1 when the read squares of cubes a and b (device) differ in
// any bit; *changed is left as it is otherwise.
template <typename Real>
cudaError_t launch_cube_compare(const Real* a, const Real* b, StackView view,
                                int* changed, cudaStream_t s);
// dst[p] = src[p] over each plane's read square [0, cube_read_extent)^2;
// src is a cube in host memory that the device addresses (view.support must
// already be on the device).
template <typename Real>
cudaError_t launch_cube_gather(const Real* src, StackView view, Real* dst,
                               cudaStream_t s);

// ---- placement and binning (gg_place.cu) ----------------------------------
// Tile shapes of the gridding kernel: every tile holds 2048 cells, tile_u
// columns by 2048 / tile_u rows.  Shape index 0, 1, 2 = tile_u 32, 16, 8.
constexpr int kNumTileShapes = 3;
__host__ __device__ inline int tile_u_of_shape(int shape) {
  return 32 >> shape;
}
__host__ __device__ inline int tile_v_of_shape(int shape) {
  return 2048 / (32 >> shape);
}

// Tile shape, slice staging and tile phases for a call, from its mean
// footprint side sqrt(macs / gridded points): narrow tiles only for tiny
// footprints (a 32-wide warp would leave most lanes outside them); kernel
// slices staged in shared memory (bit 8) when footprints are small enough
// for their slices to fit the slots, otherwise the kernel keeps its shared
// memory small so the L1 cache serves the tap loads; tile phases (bits 12
// and 13: log2 of 1, 2, 4 or 8) four when footprints are narrower than the
// tile, where offset tile grids save the most tile crossings, else one.
// forced_shape >= 0 overrides the shape, phases > 0 the phases.
__host__ __device__ inline uint32_t choose_shape(unsigned long long macs,
                                                 unsigned long long gridded,
                                                 int forced_shape,
                                                 int phases = 1) {
  const double side = gridded ? sqrt((double)macs / (double)gridded) : 0.0;
  int shape = forced_shape;
  if (shape < 0) shape = side >= 16.0 ? 0 : (side >= 8.0 ? 1 : 2);
  const uint32_t stage = side < 40.0 ? 1u : 0u;
  if (phases <= 0) phases = side < (double)tile_u_of_shape(shape) ? 4 : 1;
  const uint32_t pbits =
      phases >= 8 ? 3u : (phases >= 4 ? 2u : (phases >= 2 ? 1u : 0u));
  return (uint32_t)shape | (stage << 8) | (pbits << 12);
}
// Tile phases of a shape word made by choose_shape.
__host__ __device__ inline int phases_of_shape(uint32_t word) {
  return 1 << ((word >> 12) & 3u);
}

struct PlaceOut {
  uint32_t* cell;             // [N]
  uint32_t* meta;             // [N]
  void* vw;                   // [N] weighted visibility, Real2
  uint32_t* rec_count;        // [N] records (tiles touched) per visibility
  double* blk_norm;           // [num_blocks]
  unsigned long long* blk_skip;   // [num_blocks]
  unsigned long long* blk_macs;   // [num_blocks]
};
// Points per block of the placement kernel (its per-block partials).
constexpr int kPlaceBlock = 256;
int place_num_blocks(unsigned long long n);
template <typename Real>
cudaError_t launch_place(PlaceParams<Real> p, StackView view, TileGeom geom,
                         int grid_index, unsigned long long vis_offset,
                         PlaceOut out, cudaStream_t s);
// *p = v on stream s (device p), without a copy-engine transfer.
cudaError_t launch_store_f64(double* p, double v, cudaStream_t s);
// For a placement made with PlaceParams::defer_norm: the norm terms from
// the placed meta and the stack's tap sums, reduced in k_place's block
// order, then *d_norm += their sum exactly as launch_place_finalize would.
template <typename Real>
cudaError_t launch_norm_terms(const uint32_t* meta, const Real* weight,
                              unsigned long long n, StackView view,
                              double* blk_norm, double* d_norm,
                              cudaStream_t s);
// Sums the per-block partials: *d_norm += norm, *d_num_skipped = skips,
// *d_macs = macs (all device pointers), and picks the tile shape and tile
// phases for the call into *d_shape (choose_shape): forced_shape if >= 0,
// phases if > 0, else from the mean footprint area (macs / gridded points).
cudaError_t launch_place_finalize(const double* blk_norm,
                                  const unsigned long long* blk_skip,
                                  const unsigned long long* blk_macs,
                                  int num_blocks, unsigned long long n,
                                  int forced_shape, double* d_norm,
                                  unsigned long long* d_num_skipped,
                                  unsigned long long* d_macs,
                                  uint32_t* d_shape, cudaStream_t s,
                                  int phases = 1);
// count[i] = tiles of shape *d_shape touched by visibility i on its tile
// phase (footprint_phase; 0 if skipped).
cudaError_t launch_count_records(const uint32_t* cell, const uint32_t* meta,
                                 unsigned long long n, StackView view,
                                 const uint32_t* d_shape, uint32_t* count,
                                 cudaStream_t s);
template <typename Real>
cudaError_t launch_place_only(PlaceParams<Real> p, StackView view, int* out,
                              cudaStream_t s);
cudaError_t launch_emit_records(const uint32_t* cell, const uint32_t* meta,
                                const uint32_t* rec_offset,
                                unsigned long long n, StackView view,
                                TileGeom geom, int grid_index,
                                unsigned long long vis_offset, uint32_t* keys,
                                uint32_t* vals, cudaStream_t s,
                                const unsigned long long* grid_offsets =
                                    nullptr,
                                int num_grids = 1);
// grid_offsets (device, num_grids + 1): batched calls, where visibility i
// belongs to the grid g with grid_offsets[g] <= i < grid_offsets[g + 1].

// ---- batched calls (gg_batch.cu) ------------------------------------------
// Per-visibility placement for a batched call: like launch_place, but the
// FP64 norm term of every visibility goes to nterm[i] (0 if skipped) so the
// norm can be reduced per grid.
template <typename Real>
cudaError_t launch_place_batched(PlaceParams<Real> p, StackView view,
                                 PlaceOut out, double* nterm, cudaStream_t s);
// Weighted visibilities and norm terms for new amplitudes and weights on
// an existing placement (meta).
template <typename Real>
cudaError_t launch_revalue(const Real* vis, const Real* weight,
                           const uint32_t* meta, StackView view,
                           unsigned long long n, void* vw, double* nterm,
                           cudaStream_t s);
// Deterministic per-grid totals over a chunk table (chunk c covers
// visibilities [chunk_begin[c], chunk_begin[c+1]) of grid chunk_grid[c];
// grid g owns chunks [grid_chunk0[g], grid_chunk0[g+1])):
// d_norm[g] += sum of nterm, d_num_skipped[g] = skips, *d_macs = total
// MACs, *d_shape = choose_shape(total MACs, gridded, forced_shape).
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
                                cudaStream_t s, int phases = 1);

// ---- work decomposition and gridding (gg_grid.cu) -------------------------
cudaError_t launch_tile_bounds(const uint32_t* keys, uint32_t n, int shift,
                               int num_tiles, uint32_t* tile_start,
                               cudaStream_t s);
// One CTA whose threads wait, bounded by `limit` probes, on an mbarrier
// that nothing arrives at, then set *error (see gg_plan_probe_bounded_wait).
cudaError_t launch_wait_probe(unsigned limit, uint32_t* error,
                              cudaStream_t s);
// Touched spans of a single-grid call, in strips of tile_u / tile_phases
// columns: for every virtual tile t holding records (tile_start[t + 1] >
// tile_start[t]) of tile row r, lo[r] takes the first strip it covers and
// hi[r] the last + 1.  lo must start at 0xFFFFFFFF and hi at 0.
cudaError_t launch_touched_spans(const uint32_t* tile_start, int num_tiles,
                                 const TileGeom& geom, int grid_size,
                                 uint32_t* lo, uint32_t* hi, cudaStream_t s);
// Strips of tile_u / tile_phases columns by tile rows of a single grid: the
// units of the direct-mode group table and of the touched spans.
inline int num_strips(const TileGeom& g) { return g.strips_u * g.tiles_v; }
// Sets the strip fields of g (tile_u, tile_phases set) for a grid side.
inline void set_strips(TileGeom& g, int grid_size) {
  const int P = g.tile_phases > 1 ? g.tile_phases : 1;
  int sh = 0;
  while ((1 << (sh + 1)) <= g.tile_u / P) ++sh;
  g.strip_shift = sh;
  g.strips_u = (grid_size + (1 << sh) - 1) >> sh;
}
// Work-item queue of a call.  Tiles are virtual tiles (group * tiles_total
// + tile, see TileGeom); the queue is group-major, and within a group the
// chunks of split tiles come first.  group_items[g] .. group_items[g+1] is
// the queue range of plane group g (num_groups + 1 entries).
struct ItemBuffers {
  uint32_t* chunks;       // [num_tiles] chunks per tile (then offsets)
  uint32_t* split_chunks; // [num_tiles] chunks of split tiles (then slots)
  uint32_t* group_items;  // [num_groups + 1]
  int num_groups;
  uint32_t* num_items;    // [1]
  uint32_t* num_slots;    // [1]
  WorkItem* items;        // [capacity]
  int4* split_tiles;      // [num_tiles] (tile, first slot, chunks, -)
  uint32_t* num_split;    // [1]
  uint32_t* counter;      // [1] work counter of the persistent kernel
  void* scan_tmp;
  // Queue order of the tiles within a group: rank r of group g is virtual
  // tile g * T + tile_order[r] (T = tiles per group); null = tile order.
  const int* tile_order = nullptr;
  // > 1: the tiles of virtual groups g with g % partial_phases != 0 (tile
  // phases after the first) write partial tiles even when they have one
  // chunk, so that all the phases of a plane group share one launch.
  int partial_phases = 1;
  // [num_tiles] (first partial slot, chunks) of each virtual tile, chunks 0
  // when it writes none (filled when not null).
  int2* tile_slot = nullptr;
};
cudaError_t launch_build_items(const uint32_t* tile_start, int num_tiles,
                               uint32_t num_records, uint32_t chunk,
                               ItemBuffers b, cudaStream_t s);
// Persistent launches in virtual-group order, each over the work items of
// group_span consecutive virtual groups: with group_span = tile_phases one
// launch per plane group takes all its tile phases (the items were built
// with ItemBuffers::partial_phases = tile_phases: the first phase's
// single-chunk tiles are added to the grid by the launch, every other item
// writes a partial tile); with group_span = 1 one launch per virtual group.
// Each launch is followed by the reduction of its virtual groups' partial
// tiles in group order (grid += their partials in chunk order, FP64; all
// the phases of a launch in one pass over the grid when tile_slot, the
// item builder's map, is given): the grid takes the groups' and phases'
// contributions in order.
// wait_before[v] / record_after[v] (arrays of num_groups events, entries
// may be null): s waits for the first before the launch that starts with
// virtual group v and records the second after the launch (and its
// reductions) that ends with v.
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
                              const cudaEvent_t* wait_before = nullptr,
                              const cudaEvent_t* record_after = nullptr,
                              Real* host_grid = nullptr,
                              const uint32_t* tile_groups = nullptr,
                              int group_span = 1,
                              const int2* tile_slot = nullptr,
                              const uint32_t* tile_start = nullptr);
// Direct mode of a single-grid call: per strip (num_strips), the first and
// last virtual group (plane group and tile phase) with records there
// (first | last << 16, 0xFFFF when none), and *cells += the grid cells of
// the strips with records.  With tile_groups given, launch_grid_tiles reads
// each such strip's cells from host_grid in its first group's pass, writes
// them back there in its last group's, and keeps the sums in between in
// grid: every cell takes the same additions in the same order as when grid
// holds a copy of host_grid.
cudaError_t launch_tile_groups(const uint32_t* tile_start,
                               const TileGeom& geom, int grid_size,
                               uint32_t* out, unsigned long long* cells,
                               cudaStream_t s);
// stage: the kernel variant that stages kernel slices in shared memory;
// lane_groups: TileGeom::lane_groups.
template <typename Real>
int grid_tiles_ctas_per_sm(int tile_u, bool stage, int lane_groups = 1);

// ---- accessors defined in gg_api.cu ---------------------------------------
// Records a failure for gg_last_error() on this thread; returns code.
int record_error(int code, const char* message);
// The device view and properties of a kernel-stack handle.
bool kernels_info(const gg_kernels* k, StackView* view, int* device,
                  bool* is_double, int* num_planes);

// ---- uniform weighting (gg_weights.cu) -------------------------------------
// Keys each point by its density cell (grid_size^2 when off the grid) and
// counts the off-grid points into *d_num_skipped (which must start at 0).
template <typename Real>
cudaError_t launch_weight_keys(const Real* uu, const Real* vv,
                               unsigned long long n, Real cell_size_rad,
                               int grid_size, uint32_t* keys, uint32_t* vals,
                               unsigned long long* d_num_skipped,
                               cudaStream_t s);
// grid[cell] += the weights of the cell's points, in the order of the
// stably sorted (keys, vals).
template <typename Real>
cudaError_t launch_weight_runs(const uint32_t* keys, const uint32_t* vals,
                               unsigned long long n, const Real* weight,
                               int grid_size, Real* grid, cudaStream_t s);
template <typename Real>
cudaError_t launch_weights_read(const Real* uu, const Real* vv,
                                const Real* w_in, Real* w_out,
                                unsigned long long n, Real cell_size_rad,
                                int grid_size, const Real* grid,
                                unsigned long long* d_num_skipped,
                                cudaStream_t s);

// ---- W-kernel generation (gg_kgen.cu) -------------------------------------
// Writes the taper x chirp cube [P][csh][csh] complex into d_cube; d_total
// holds P complex FP64 normalisation sums (16 B each).
template <typename Real>
cudaError_t launch_kernel_generate(int num_planes, const int* d_support,
                                   const double* d_w_planes, int oversample,
                                   int conv_size_half, void* d_total,
                                   Real* d_cube, cudaStream_t s);

// ---- FP32 FMA throughput probe (gg_calib.cu) ------------------------------
cudaError_t measure_fp32_fma(int num_sms, double* tflops_best, float* ms_out);

// ---- adjoint (gg_degrid.cu) -----------------------------------------------
// Resident CTAs per SM of the degridding kernel.
template <typename Real>
int degrid_tiles_ctas_per_sm();
// One persistent launch over the whole work-item queue (32 x 64-cell tiles
// only): rec_out[rec_offset[v] + rank] = the record's share of
// conj(tap) * grid for every record, rank = the record's tile among
// visibility v's tiles in emission order.
template <typename Real>
cudaError_t launch_degrid_tiles(const WorkItem* items,
                                const uint32_t* num_items, uint32_t* counter,
                                uint32_t* error, const uint32_t* rec_vis,
                                const uint32_t* cell, const uint32_t* meta,
                                const uint32_t* rec_offset, StackView view,
                                TileGeom geom, int grid_size, const Real* grid,
                                void* rec_out, int num_ctas, cudaStream_t s);
// out[v] = the sum of visibility v's count[v] partial results from
// rec_out[offset[v]] on, in order.
template <typename Real>
cudaError_t launch_degrid_finish(const uint32_t* count, const uint32_t* offset,
                                 const void* rec_out, unsigned long long n,
                                 Real* out, cudaStream_t s);

}  // namespace gg
