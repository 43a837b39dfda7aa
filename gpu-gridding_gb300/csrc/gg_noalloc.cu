// Gridding without any allocation inside the call.
//
// Some callers cannot allocate device memory at the moment they grid: a
// real-time ingest loop that must not stall on cudaMalloc (which can
// synchronise the device and take milliseconds), code running inside another
// framework's memory pool or an allocator-hooked process that forbids raw
// CUDA allocations, or a caller that has to bound its device footprint up
// front.  For them gg_grid_wproj_f_device_noalloc runs the same placement,
// binning, sort, tile-gridding and partial-reduction kernels as
// gg_grid_wproj_f_device, but every byte of scratch comes from one
// file-scope device array of fixed size, g_noalloc_scratch below.  The
// caller still passes the inputs, the outputs and a kernel-stack handle made
// beforehand with gg_kernels_create_f (that set-up step does allocate).
//
// Costs of this design, stated for the caller:
// * every GPU that loads the library holds the 32 MiB array until the
//   process exits, whether or not it ever calls this entry point;
// * the array is shared by all calls on a device: calls that overlap on the
//   GPU (different streams, different host threads) race on it and must be
//   serialised by the caller;
// * a call takes at most kNoAllocMaxPoints visibilities, at most
//   kNoAllocMaxRecords (visibility, tile) records and a grid side of at most
//   kNoAllocMaxGrid; larger inputs are rejected with GG_ERR_CAPACITY and
//   leave the caller's grid, norm and num_skipped untouched (the record
//   count is known only after placement, whose norm and skip totals go to
//   the scratch array and reach the caller's outputs once the call is
//   accepted);
// * if a call's gridding kernel runs out of its bounded wait, that call has
//   already returned GG_OK; the failure is reported by the next no-alloc
//   call on the device (whoever makes it), which returns GG_ERR_CUDA
//   without touching its outputs -- the incomplete grid is the previous
//   call's;
// * the device address of the array is looked up (cudaGetSymbolAddress) by
//   the first call on each device, which must therefore be made with that
//   device current and before any stream capture begins.
// Like the allocating entry point, the call synchronises its stream once to
// read back the record count.
#include <algorithm>
#include <mutex>

#include "gg_internal.h"
#include "../../include/gpugrid.h"

namespace {

using namespace gg;

constexpr size_t kNoAllocMaxPoints = size_t(1) << 17;   // 131,072
constexpr size_t kNoAllocMaxRecords = size_t(1) << 20;  // 1,048,576
constexpr int kNoAllocMaxGrid = 8192;
constexpr int kNoAllocMaxSlots = 384;    // partial tiles of split tiles
constexpr int kNoAllocCells = 2048;      // cells per tile
constexpr size_t kNoAllocBytes = size_t(32) << 20;
constexpr int kMaxDevices = 64;

// The scratch memory of every no-alloc call on a device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once
// per device; host code must not use the symbol itself as an address).
int scratch_address(int dev, unsigned char** out) {
  if (dev < 0 || dev >= kMaxDevices)
    return record_error(GG_ERR_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return record_error(GG_ERR_CUDA,
                          "cudaGetSymbolAddress of the no-alloc scratch "
                          "array failed");
    g_scratch_addr[dev] = p;
  }
  *out = (unsigned char*)g_scratch_addr[dev];
  return GG_OK;
}

struct Carve {
  unsigned char* base;
  size_t used = 0;
  template <typename T>
  T* take(size_t count) {
    used = (used + 255) & ~size_t(255);
    T* p = (T*)(base + used);
    used += count * sizeof(T);
    return p;
  }
};

int ceil_log2_u(unsigned long long x) {
  int b = 0;
  while ((1ull << b) < x) ++b;
  return b;
}

// Commits an accepted call's placement totals to the caller's outputs:
// *d_norm += the call's norm, *d_num_skipped = its skip count.
__global__ void k_noalloc_commit(const double* __restrict__ norm,
                                 const unsigned long long* __restrict__ skip,
                                 double* d_norm,
                                 unsigned long long* d_num_skipped) {
  *d_norm += *norm;
  *d_num_skipped = *skip;
}

#define NA_CUDA(call)                                                   \
  do {                                                                  \
    if ((call) != cudaSuccess)                                          \
      return record_error(GG_ERR_CUDA, "CUDA call failed: " #call);     \
  } while (0)

}  // namespace

extern "C" GG_API int gg_grid_wproj_f_device_noalloc(
    const gg_kernels* kernels, size_t num_points, const float* d_uu,
    const float* d_vv, const float* d_ww, const float* d_vis,
    const float* d_weight, float cell_size_rad, float w_scale, int grid_size,
    unsigned long long* d_num_skipped, double* d_norm, float* d_grid,
    void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  StackView view;
  int kdev = 0, num_planes = 0;
  bool is_double = true;
  if (!kernels_info(kernels, &view, &kdev, &is_double, &num_planes))
    return record_error(GG_ERR_INVALID_ARG, "kernels is NULL");
  if (is_double)
    return record_error(GG_ERR_INVALID_ARG,
                        "the no-alloc entry point takes an FP32 kernel stack");
  if (num_points > kNoAllocMaxPoints)
    return record_error(GG_ERR_CAPACITY,
                        "num_points exceeds the no-alloc limit of 131072 "
                        "visibilities per call");
  if (grid_size < 1 || grid_size > kNoAllocMaxGrid)
    return record_error(GG_ERR_CAPACITY,
                        "grid_size exceeds the no-alloc limit of 8192");
  if (num_points > 0 && (!d_uu || !d_vv || !d_ww || !d_vis || !d_weight))
    return record_error(GG_ERR_INVALID_ARG, "an input array is NULL");
  if (!d_grid || !d_norm || !d_num_skipped)
    return record_error(GG_ERR_INVALID_ARG, "an output pointer is NULL");
  int dev = 0;
  NA_CUDA(cudaGetDevice(&dev));
  if (dev != kdev)
    return record_error(GG_ERR_INVALID_ARG,
                        "kernel stack and current device differ");
  unsigned char* scratch = nullptr;
  int r = scratch_address(dev, &scratch);
  if (r != GG_OK) return r;
  if (num_points == 0) {
    NA_CUDA(cudaMemsetAsync(d_num_skipped, 0, 8, s));
    return GG_OK;
  }

  // ---- carve the scratch array (same layout on every call) ---------------
  int max_tiles = 0;
  for (int sh = 0; sh < kNumTileShapes; ++sh) {
    const int tu = tile_u_of_shape(sh), tv = tile_v_of_shape(sh);
    max_tiles = std::max(max_tiles, ((kNoAllocMaxGrid + tu - 1) / tu) *
                                        ((kNoAllocMaxGrid + tv - 1) / tv));
  }
  const size_t maxp = kNoAllocMaxPoints, maxr = kNoAllocMaxRecords;
  const int max_blocks = place_num_blocks(maxp);
  Carve c{scratch};
  uint32_t* sc = c.take<uint32_t>(16);  // 0 total, 1 items, 2 slots,
                                        // 3 split, 4 counter, 5 shape,
                                        // 6 error
  unsigned long long* macs = c.take<unsigned long long>(1);
  // This call's norm and skip totals, committed to the caller's outputs
  // only once the call is accepted.
  double* call_norm = c.take<double>(1);
  unsigned long long* call_skip = c.take<unsigned long long>(1);
  uint32_t* cell = c.take<uint32_t>(maxp);
  uint32_t* meta = c.take<uint32_t>(maxp);
  float2* vw = c.take<float2>(maxp);
  uint32_t* count = c.take<uint32_t>(maxp);
  uint32_t* offset = c.take<uint32_t>(maxp);
  double* blk_norm = c.take<double>(max_blocks);
  unsigned long long* blk_skip = c.take<unsigned long long>(max_blocks);
  unsigned long long* blk_macs = c.take<unsigned long long>(max_blocks);
  void* scan_tmp =
      c.take<unsigned char>(scan_temp_bytes(std::max<size_t>(maxp, max_tiles)));
  uint32_t* keys0 = c.take<uint32_t>(maxr);
  uint32_t* vals0 = c.take<uint32_t>(maxr);
  uint32_t* keys1 = c.take<uint32_t>(maxr);
  uint32_t* vals1 = c.take<uint32_t>(maxr);
  void* sort_tmp = c.take<unsigned char>(radix_temp_bytes(maxr));
  uint32_t* tile_start = c.take<uint32_t>(max_tiles + 1);
  uint32_t* item_a = c.take<uint32_t>(max_tiles + 1);
  uint32_t* item_b = c.take<uint32_t>(max_tiles + 1);
  WorkItem* items = c.take<WorkItem>(max_tiles + kNoAllocMaxSlots + 16);
  int4* split_tiles = c.take<int4>(max_tiles + 1);
  float2* partials = c.take<float2>((size_t)kNoAllocMaxSlots * kNoAllocCells);
  if (c.used > kNoAllocBytes)
    return record_error(GG_ERR_UNSUPPORTED,
                        "no-alloc scratch layout exceeds the array");

  // The array keeps the previous call's contents: clear the counters this
  // call accumulates into.  Word 6, the bounded-wait error flag of the
  // tile kernel, is left for the check below.
  NA_CUDA(cudaMemsetAsync(sc, 0, 6 * sizeof(uint32_t), s));
  NA_CUDA(cudaMemsetAsync(call_norm, 0, sizeof(double), s));

  PlaceParams<float> pp;
  pp.uu = d_uu; pp.vv = d_vv; pp.ww = d_ww; pp.vis = d_vis;
  pp.weight = d_weight;
  pp.grid_scale = (float)grid_size * cell_size_rad;
  pp.w_scale = w_scale;
  pp.grid_size = grid_size;
  pp.grid_centre = grid_size / 2;
  pp.num_points = num_points;
  PlaceOut po;
  po.cell = cell;
  po.meta = meta;
  po.vw = vw;
  po.rec_count = count;
  po.blk_norm = blk_norm;
  po.blk_skip = blk_skip;
  po.blk_macs = blk_macs;
  const int nblk = place_num_blocks(num_points);
  NA_CUDA(launch_place<float>(pp, view, TileGeom{}, 0, 0, po, s));
  NA_CUDA(launch_place_finalize(blk_norm, blk_skip, blk_macs, nblk,
                                num_points, -1, call_norm, call_skip, macs,
                                sc + 5, s));
  NA_CUDA(launch_count_records(cell, meta, num_points, view, sc + 5, count,
                               s));
  NA_CUDA(exclusive_scan_u32(count, offset, num_points, sc + 0, scan_tmp, s));
  uint32_t host_sc[8] = {0};
  NA_CUDA(cudaMemcpyAsync(host_sc, sc, sizeof(host_sc),
                          cudaMemcpyDeviceToHost, s));
  NA_CUDA(cudaStreamSynchronize(s));
  if (host_sc[6]) {
    NA_CUDA(cudaMemsetAsync(sc + 6, 0, sizeof(uint32_t), s));
    return record_error(GG_ERR_CUDA,
                        "an earlier no-alloc call's tile kernel ran out of "
                        "its bounded wait; that call's grid is incomplete");
  }
  const uint32_t total = host_sc[0];
  const int shape = (int)(host_sc[5] & 0xFFu);
  const bool stage = ((host_sc[5] >> 8) & 1u) != 0;
  if (total > kNoAllocMaxRecords)
    return record_error(GG_ERR_CAPACITY,
                        "the call needs more (visibility, tile) records than "
                        "the no-alloc limit of 1048576 (grid, norm and "
                        "num_skipped untouched)");
  // Accepted: the placement totals reach the caller's outputs.
  k_noalloc_commit<<<1, 1, 0, s>>>(call_norm, call_skip, d_norm,
                                   d_num_skipped);
  NA_CUDA(cudaGetLastError());
  if (total == 0) return GG_OK;

  // ---- binning, work items, gridding, reduction ---------------------------
  TileGeom geom{};
  geom.tile_u = tile_u_of_shape(shape);
  geom.tile_v = tile_v_of_shape(shape);
  geom.tiles_u = (grid_size + geom.tile_u - 1) / geom.tile_u;
  geom.tiles_v = (grid_size + geom.tile_v - 1) / geom.tile_v;
  geom.num_grids = 1;
  geom.num_groups = 1;
  geom.tiles_total = geom.tiles_u * geom.tiles_v;
  geom.plane_group = nullptr;
  geom.tile_phases = 1;
  set_strips(geom, grid_size);
  const int num_tiles = geom.tiles_u * geom.tiles_v;
  const int tile_bits = ceil_log2_u((unsigned long long)num_tiles);
  int plane_bits = ceil_log2_u((unsigned long long)num_planes);
  int phase_bits =
      ceil_log2_u((unsigned long long)(view.omax + 1) * (view.omax + 1));
  if (tile_bits + plane_bits + phase_bits > 32) phase_bits = 0;
  if (tile_bits + plane_bits + phase_bits > 32) plane_bits = 0;
  geom.plane_bits = plane_bits;
  geom.phase_bits = phase_bits;
  geom.phase_side = view.omax + 1;
  const int low_bits = plane_bits + phase_bits;

  NA_CUDA(launch_emit_records(cell, meta, offset, num_points, view, geom, 0,
                              0, keys0, vals0, s));
  bool in_alt = false;
  NA_CUDA(radix_sort_pairs(keys0, vals0, keys1, vals1, total,
                           tile_bits + low_bits, sort_tmp, s, &in_alt));
  const uint32_t* keys = in_alt ? keys1 : keys0;
  const uint32_t* vals = in_alt ? vals1 : vals0;
  NA_CUDA(launch_tile_bounds(keys, total, low_bits, num_tiles, tile_start,
                             s));
  int sms = 0;
  NA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int num_ctas = sms * grid_tiles_ctas_per_sm<float>(geom.tile_u, stage);
  // Work items of about total / (2 * num_ctas) records, as the allocating
  // path sizes them, but never so small that the split tiles need more
  // partial-tile slots than the array holds: a tile of c > chunk records
  // splits into at most 2c / chunk chunks, so split chunks
  // <= 2 * total / chunk <= kNoAllocMaxSlots.
  const unsigned long long per_item =
      ((unsigned long long)total + 2ull * num_ctas - 1) / (2ull * num_ctas);
  const unsigned long long min_chunk =
      (2ull * total + kNoAllocMaxSlots - 1) / kNoAllocMaxSlots;
  const uint32_t chunk = (uint32_t)std::max<unsigned long long>(
      64, std::max(per_item, min_chunk));
  ItemBuffers ib;
  ib.chunks = item_a;
  ib.split_chunks = item_b;
  ib.num_items = sc + 1;
  ib.num_slots = sc + 2;
  ib.items = items;
  ib.split_tiles = split_tiles;
  ib.num_split = sc + 3;
  ib.counter = sc + 4;
  ib.group_items = sc + 8;   // two entries: one plane group
  ib.num_groups = 1;
  ib.scan_tmp = scan_tmp;
  NA_CUDA(launch_build_items(tile_start, num_tiles, total, chunk, ib, s));
  NA_CUDA(launch_grid_tiles<float>(items, sc + 8, sc + 4, sc + 6, vals, cell,
                                   meta, vw, view, geom, grid_size, d_grid, 0,
                                   (float*)partials, split_tiles, sc + 3,
                                   num_tiles, num_ctas, stage, s));
  return GG_OK;
}

extern "C" GG_API int gg_noalloc_probe_bounded_wait(unsigned iterations,
                                                    void* stream) {
  if (iterations < 1 || iterations > (1u << 20))
    return record_error(GG_ERR_INVALID_ARG, "iterations outside 1..1048576");
  int dev = 0;
  NA_CUDA(cudaGetDevice(&dev));
  unsigned char* scratch = nullptr;
  const int r = scratch_address(dev, &scratch);
  if (r != GG_OK) return r;
  // Word 6 of the first carve (the control words at offset 0).
  uint32_t* flag = (uint32_t*)scratch + 6;
  cudaStream_t s = (cudaStream_t)stream;
  NA_CUDA(launch_wait_probe(iterations, flag, s));
  NA_CUDA(cudaStreamSynchronize(s));
  return GG_OK;
}
