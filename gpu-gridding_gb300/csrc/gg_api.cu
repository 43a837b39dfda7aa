// Host orchestration and the C ABI of libgpugrid.so (declared in
// include/gpugrid.h).
//
// One gridding call runs, on one CUDA stream:
//   1. k_place         placement, skip flags, FP64 norm partials, records
//                      per visibility (tiles its footprint touches)
//   2. scan            record offsets per visibility
//   3. k_emit          (key = tile|plane|offset class, value = visibility)
//   4. radix sort      stable, so the record order is deterministic
//   5. tile bounds     record range of every tile
//   6. work items      tiles cut into chunks; split chunks get partial slots
//   7. k_grid_tiles    persistent tile-owning accumulation
//   8. reduce          split tiles: grid += partials, in chunk order
// The host synchronises once, after step 2, to size the sort buffers.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <sys/mman.h>
#include <unistd.h>

#include "gg_internal.h"
#include "../../include/gpugrid.h"

using namespace gg;

// ===========================================================================
// Errors
// ===========================================================================
namespace {

thread_local std::string t_last_error;

int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_last_error = buf;
  return code;
}

#define GG_CUDA(call)                                                      \
  do {                                                                     \
    cudaError_t e__ = (call);                                              \
    if (e__ != cudaSuccess)                                                \
      return set_error(e__ == cudaErrorMemoryAllocation ? GG_ERR_NO_MEMORY \
                                                        : GG_ERR_CUDA,     \
                       "%s failed: %s (%s:%d)", #call,                     \
                       cudaGetErrorString(e__), __FILE__, __LINE__);       \
  } while (0)

#define GG_TRY(call)              \
  do {                            \
    int r__ = (call);             \
    if (r__ != GG_OK) return r__; \
  } while (0)

// ===========================================================================
// Device buffers
// ===========================================================================
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  // Grows to at least n bytes (with 25% headroom); contents are not kept.
  int ensure(size_t n) {
    if (n <= bytes && p) return GG_OK;
    release();
    size_t want = std::max<size_t>(n + n / 4, 256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      cudaGetLastError();
      return set_error(GG_ERR_NO_MEMORY,
                       "cudaMalloc of %zu bytes failed: %s", want,
                       cudaGetErrorString(e));
    }
    bytes = want;
    return GG_OK;
  }
  template <typename T>
  T* as() const { return (T*)p; }
};

int ceil_log2(unsigned long long x) {
  int b = 0;
  while ((1ull << b) < x) ++b;
  return b;
}

// ===========================================================================
// Per-device state (mutex + stream for the drop-in entry points)
// ===========================================================================
struct DeviceState {
  std::mutex mu;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  gg_plan* plan = nullptr;  // workspace of the host-pointer entry points
  // Kernel stack of the host-pointer entry points.  Every call stages the
  // caller's cube (the caller may change it between calls) into one of two
  // buffers, the other holding the cube the stack was last made from; when
  // the geometry is the same, a device comparison of the two decides
  // whether the re-layout and tap-sum kernels run (cube_changed), so a
  // caller that passes the same cube call after call pays for its transfer
  // only.  cube_cur: buffer of the stack's cube, -1 = none.
  gg_kernels* host_kernels = nullptr;
  DevBuf host_cube[2];
  DevBuf cube_changed;
  int cube_cur = -1;
  // Side stream that uploads a host call's plane tables, visibilities and
  // (copied) grid (vis_ready, grid_ready mark the uploads), and the pinned
  // tile-row spans of the grid cells a copied call touched (spans_ready
  // marks their arrival).
  cudaStream_t copy_stream = nullptr;
  // Stream of the stack build (cube staging, comparison, re-layout, tap
  // sums), which runs beside placement and binning: tables_ready marks the
  // plane tables on the call's stream, stack_ready the finished stack.
  cudaStream_t stack_stream = nullptr;
  cudaEvent_t tables_ready = nullptr, stack_ready = nullptr;
  cudaEvent_t cube_staged = nullptr;   // the call's cube on the device
  cudaEvent_t vis_ready = nullptr;
  // The visibilities go up in kInputChunks pieces, each ready at its event.
  static constexpr int kInputChunks = 4;
  cudaEvent_t chunk_ready[kInputChunks] = {};
  cudaEvent_t grid_ready = nullptr;
  cudaEvent_t spans_ready = nullptr;
  cudaEvent_t top_done = nullptr;   // upper tile rows final (split pass)
  cudaEvent_t top_up = nullptr;     // upper grid rows uploaded
  uint32_t* h_spans = nullptr;
  static constexpr int kSpanCap = 2 * (kMaxGridSize / 64 + 2);
  // Bytes the last host-pointer gridding call moved each way.
  unsigned long long last_h2d = 0, last_d2h = 0;
  // How host-pointer gridding calls reach the caller's grid
  // (gg_host_set_grid_access), and whether kernels may address pageable
  // host memory (-1 = not asked yet).
  int grid_access = GG_GRID_ACCESS_PAGEABLE;
  int pageable_access = -1;
  // Phase timing of the host-pointer gridding calls (gg_host_set_profiling):
  // the call's start and end on its stream around the plan's phase events.
  bool profile = false;
  bool profile_valid = false;
  cudaEvent_t call_start = nullptr, call_end = nullptr, copies_done = nullptr;
  // Host clock of the last host-pointer call (ms from its entry): first
  // device work queued, final synchronisation returned, return.
  double host_ms[3] = {0.0, 0.0, 0.0};
};

std::mutex g_devices_mu;
std::vector<DeviceState*> g_devices;

int current_device(int* dev) {
  GG_CUDA(cudaGetDevice(dev));
  return GG_OK;
}

int device_state(int dev, DeviceState** out) {
  std::lock_guard<std::mutex> lk(g_devices_mu);
  if ((int)g_devices.size() <= dev) g_devices.resize(dev + 1, nullptr);
  if (!g_devices[dev]) {
    DeviceState* st = new DeviceState();
    int sms = 0;
    cudaError_t e =
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
      delete st;
      return set_error(GG_ERR_CUDA, "cudaDeviceGetAttribute: %s",
                       cudaGetErrorString(e));
    }
    st->num_sms = sms;
    // The call stream at the highest priority: the stack stream's kernels
    // (lowest) then take only the SMs the call's own kernels leave free.
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    e = cudaStreamCreateWithPriority(&st->stream, cudaStreamNonBlocking,
                                     greatest);
    if (e != cudaSuccess) {
      delete st;
      return set_error(GG_ERR_CUDA, "cudaStreamCreate: %s",
                       cudaGetErrorString(e));
    }
    g_devices[dev] = st;
  }
  *out = g_devices[dev];
  return GG_OK;
}

int num_sms_of_current(int* sms) {
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  *sms = st->num_sms;
  return GG_OK;
}

}  // namespace

// ===========================================================================
// Kernel stacks
// ===========================================================================
struct gg_kernels {
  unsigned long long id = 0;   // unique per handle (plans cache by it)
  int device = 0;
  unsigned long long h2d_bytes = 0;  // host bytes the last fill uploaded
  bool is_double = false;
  int num_planes = 0, oversample = 0, omax = 0, conv_size_half = 0;
  int support_max = 0;
  long long total_taps = 0;
  std::vector<int> h_support;
  std::vector<long long> h_base, h_sbase;
  long long total_slab_taps = 0;
  size_t zero_half_bytes = 0;
  DevBuf support, base, taps, tap_sum, zeros, sbase, slabs;

  StackView view() const {
    StackView v;
    v.num_planes = num_planes;
    v.oversample = oversample;
    v.omax = omax;
    v.conv_size_half = conv_size_half;
    v.support = support.as<int>();
    v.base = base.as<long long>();
    v.taps = taps.p;
    v.tap_sum = tap_sum.as<double>();
    v.zeros = zeros.as<char>() + zero_half_bytes;
    v.sbase = sbase.as<long long>();
    v.slabs = slabs.p;
    return v;
  }
};

namespace {

int validate_stack(size_t num_w_planes, const int* support, int oversample,
                   int conv_size_half, const void* conv_func) {
  if (num_w_planes < 1 || num_w_planes > (size_t)kMaxPlanes)
    return set_error(GG_ERR_INVALID_ARG,
                     "num_w_planes = %zu outside [1, %d]", num_w_planes,
                     kMaxPlanes);
  if (!support || !conv_func)
    return set_error(GG_ERR_INVALID_ARG, "support or conv_func is NULL");
  if (oversample < 1 || oversample > kMaxOversample)
    return set_error(GG_ERR_INVALID_ARG, "oversample = %d outside [1, %d]",
                     oversample, kMaxOversample);
  if (conv_size_half < 1)
    return set_error(GG_ERR_INVALID_ARG, "conv_size_half = %d < 1",
                     conv_size_half);
  for (size_t p = 0; p < num_w_planes; ++p) {
    const long long s = support[p];
    if (s < 0)
      return set_error(GG_ERR_INVALID_ARG, "support[%zu] = %lld < 0", p, s);
    // The reference reads taps up to |off| + s*os with |off| <= os/2; a cube
    // smaller than that is read out of bounds by the reference.
    if (s * oversample + oversample / 2 >= (long long)conv_size_half)
      return set_error(GG_ERR_INVALID_ARG,
                       "support[%zu] = %lld needs conv_size_half > %lld "
                       "(got %d)",
                       p, s, s * oversample + oversample / 2,
                       conv_size_half);
  }
  return GG_OK;
}

// (Re)builds kernel stack k from a cube: sizes, tables, the re-laid slice
// and slab stacks and the tap sums, enqueued on s.  k's device buffers are
// reused when large enough, so rebuilding one object for every call (the
// host-pointer entry points do) allocates nothing after the first call.  A
// host cube is copied through *stage (a local buffer when stage is NULL).
// With sync = false the caller must synchronise s before the host cube or
// *stage may change.
// Where kernels_fill runs its parts: the zero buffer and the plane tables
// on `light` (their copies ahead of anything the caller queues there
// next), then `between` (the caller's own work, e.g. its next uploads on
// `light`), then the heavy part (the cube's staging and the stack kernels)
// on `heavy`, after the tables (`tables`, recorded on `light`) and after
// `after` when set; `done` is recorded on `heavy` at the end.
struct StackStreams {
  cudaStream_t light, heavy;
  cudaEvent_t tables, after, done;
  std::function<int()> between;
  cudaEvent_t staged;   // recorded on `heavy` once the cube is on the device
};

template <typename Real>
int kernels_fill(gg_kernels* k, size_t num_w_planes, const int* support,
                 int oversample, int conv_size_half, const Real* conv_func,
                 int on_device, cudaStream_t s, DevBuf* stage, bool sync,
                 const Real* mapped = nullptr, const DevBuf* previous = nullptr,
                 int* changed = nullptr, const StackStreams* ss = nullptr) {
  GG_TRY(validate_stack(num_w_planes, support, oversample, conv_size_half,
                        conv_func));
  static std::atomic<unsigned long long> next_id{1};
  k->id = next_id.fetch_add(1);
  k->h2d_bytes = 0;
  k->support_max = 0;
  auto fail = [&](int code) { return code; };
  if (current_device(&k->device) != GG_OK) return fail(GG_ERR_CUDA);
  k->is_double = sizeof(Real) == 8;
  k->num_planes = (int)num_w_planes;
  k->oversample = oversample;
  k->omax = (oversample + 1) / 2;
  k->conv_size_half = conv_size_half;
  k->h_support.assign(support, support + num_w_planes);
  std::vector<long long>& base = k->h_base;
  base.resize(num_w_planes);
  long long total = 0;
  const long long classes = (long long)(k->omax + 1) * (k->omax + 1);
  for (size_t p = 0; p < num_w_planes; ++p) {
    base[p] = total;
    total += classes * slice_taps(support[p]);
    k->support_max = std::max(k->support_max, support[p]);
  }
  k->h_sbase.resize(num_w_planes);
  long long qtotal = 0;
  for (size_t p = 0; p < num_w_planes; ++p) {
    k->h_sbase[p] = qtotal;
    qtotal += (k->omax + 1) * slab_taps(support[p], oversample, k->omax);
  }
  // Slab row pitch and column bases are 16-bit fields of the gridding
  // kernel's record descriptors.
  if ((long long)oversample * (k->support_max + 2) + k->support_max + 64 >
      32767)
    return fail(set_error(GG_ERR_UNSUPPORTED,
                          "oversample * (support + 2) = %lld exceeds this "
                          "build's slab row limit",
                          (long long)oversample * (k->support_max + 2)));
  // Record descriptors hold slab offsets plus column bases in 32 bits.
  if (total > 0x7fffffffLL || qtotal > 0x7fffffffLL - (1LL << 24))
    return fail(set_error(GG_ERR_UNSUPPORTED,
                          "re-laid kernel stack has %lld taps; this build "
                          "indexes at most 2^31-1",
                          std::max(total, qtotal)));
  k->total_taps = total;
  k->total_slab_taps = qtotal;
  // Zero buffer for lanes outside a footprint: a lane reads kRows = 8 rows
  // at a stride of up to 2*s_max+1 taps either way from its middle.
  k->zero_half_bytes = (size_t)8 * (2 * k->support_max + 1) * 2 * sizeof(Real);
  int r;
  if ((r = k->support.ensure(num_w_planes * sizeof(int))) ||
      (r = k->base.ensure(num_w_planes * sizeof(long long))) ||
      (r = k->taps.ensure((size_t)total * 2 * sizeof(Real))) ||
      (r = k->zeros.ensure(2 * k->zero_half_bytes + 256)) ||
      (r = k->sbase.ensure(num_w_planes * sizeof(long long))) ||
      (r = k->slabs.ensure((size_t)qtotal * 2 * sizeof(Real) + 16)) ||
      (r = k->tap_sum.ensure(num_w_planes * (2 * k->omax + 1) *
                             (2 * k->omax + 1) * sizeof(double))))
    return fail(r);
  const cudaStream_t s_call = s;
  if (ss) s = ss->light;
  if (cudaMemsetAsync(k->zeros.p, 0, k->zeros.bytes, s) != cudaSuccess)
    return fail(set_error(GG_ERR_CUDA, "zero buffer memset failed"));
  auto cu = [&](cudaError_t e, const char* what) -> int {
    if (e == cudaSuccess) return GG_OK;
    return set_error(GG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  };
  if ((r = cu(cudaMemcpyAsync(k->support.p, support,
                              num_w_planes * sizeof(int),
                              cudaMemcpyHostToDevice, s), "support H2D")) ||
      (r = cu(cudaMemcpyAsync(k->base.p, base.data(),
                              num_w_planes * sizeof(long long),
                              cudaMemcpyHostToDevice, s), "base H2D")) ||
      (r = cu(cudaMemcpyAsync(k->sbase.p, k->h_sbase.data(),
                              num_w_planes * sizeof(long long),
                              cudaMemcpyHostToDevice, s), "sbase H2D")))
    return fail(r);
  k->h2d_bytes += num_w_planes * (sizeof(int) + 2 * sizeof(long long));
  const cudaStream_t s_tables = s;
  if (ss) {
    if ((r = cu(cudaEventRecord(ss->tables, s_tables), "tables event")))
      return fail(r);
    if (ss->between && (r = ss->between()) != GG_OK) return fail(r);
    if ((r = cu(cudaStreamWaitEvent(ss->heavy, ss->tables, 0), "wait")) ||
        (ss->after &&
         (r = cu(cudaStreamWaitEvent(ss->heavy, ss->after, 0), "wait"))))
      return fail(r);
    s = ss->heavy;
  }
  const size_t cube = num_w_planes * (size_t)conv_size_half * conv_size_half *
                      2 * sizeof(Real);
  DevBuf local;
  DevBuf& staged = stage ? *stage : local;
  const Real* d_conv = conv_func;
  if (!on_device && mapped) {
    // A host cube the device addresses: the same squares, read by a gather
    // kernel at the link's rate (3-D copies move one row of a plane per
    // DMA and run far below it).
    if ((r = staged.ensure(cube))) return fail(r);
    if ((r = cu(launch_cube_gather<Real>(mapped, k->view(), staged.as<Real>(),
                                         s),
                "cube gather")))
      return fail(r);
    for (size_t p = 0; p < num_w_planes; ++p) {
      const unsigned long long e = (unsigned long long)cube_read_extent(
          support[p], oversample, k->omax, conv_size_half);
      k->h2d_bytes += e * e * 2 * sizeof(Real);
    }
    d_conv = staged.as<Real>();
  } else if (!on_device) {
    // Only the square of each plane that the preparation kernels read goes
    // up (cube_read_extent: about a third of the cube when supports vary
    // across the stack); a run of planes with the same extent is one 3-D
    // copy.  The rest of the staging buffer is never read.
    if ((r = staged.ensure(cube))) return fail(r);
    const size_t pitch = (size_t)conv_size_half * 2 * sizeof(Real);
    const size_t plane_elems = (size_t)conv_size_half * conv_size_half * 2;
    size_t p0 = 0;
    while (p0 < num_w_planes) {
      const int e = cube_read_extent(support[p0], oversample, k->omax,
                                     conv_size_half);
      size_t p1 = p0 + 1;
      while (p1 < num_w_planes &&
             cube_read_extent(support[p1], oversample, k->omax,
                              conv_size_half) == e)
        ++p1;
      cudaMemcpy3DParms prm = {};
      prm.srcPtr = make_cudaPitchedPtr(
          (void*)(conv_func + p0 * plane_elems), pitch,
          (size_t)conv_size_half * 2 * sizeof(Real), conv_size_half);
      prm.dstPtr = make_cudaPitchedPtr(
          staged.as<Real>() + p0 * plane_elems, pitch,
          (size_t)conv_size_half * 2 * sizeof(Real), conv_size_half);
      prm.extent = make_cudaExtent((size_t)e * 2 * sizeof(Real), (size_t)e,
                                   p1 - p0);
      prm.kind = cudaMemcpyHostToDevice;
      if ((r = cu(cudaMemcpy3DAsync(&prm, s), "conv_func H2D")))
        return fail(r);
      k->h2d_bytes += (unsigned long long)e * e * 2 * sizeof(Real) * (p1 - p0);
      p0 = p1;
    }
    d_conv = staged.as<Real>();
  }
  if (ss && ss->staged &&
      (r = cu(cudaEventRecord(ss->staged, s), "staged event")))
    return fail(r);
  StackView v = k->view();
  if (changed) {
    // Re-lay only a cube that differs from previous (same geometry), whose
    // re-layout k still holds; without previous, always.
    if (previous) {
      if ((r = cu(cudaMemsetAsync(changed, 0, sizeof(int), s), "flag")) ||
          (r = cu(launch_cube_compare<Real>(d_conv, previous->as<Real>(), v,
                                            changed, s),
                  "cube compare")))
        return fail(r);
    } else {
      const int one = 1;
      if ((r = cu(cudaMemcpyAsync(changed, &one, sizeof(int),
                                  cudaMemcpyHostToDevice, s),
                  "flag")))
        return fail(r);
    }
  }
  if ((r = cu(launch_stack_relayout<Real>(d_conv, v, k->taps.p, total, s,
                                          changed),
              "relayout")))
    return fail(r);
  if ((r = cu(launch_stack_relayout_slabs<Real>(d_conv, v, k->slabs.p, s,
                                                changed),
              "slab relayout")))
    return fail(r);
  StackView raw = v;
  raw.taps = d_conv;
  if ((r = cu(launch_tap_sums<Real>(raw, k->tap_sum.as<double>(),
                                    k->support_max, s, changed),
              "tap sums")))
    return fail(r);
  if (ss && (r = cu(cudaEventRecord(ss->done, s), "stack event")))
    return fail(r);
  // The staging copy (and the caller's host array) must outlive the
  // kernels that read it.
  if (sync || !stage)
    if ((r = cu(cudaStreamSynchronize(s), "kernel stack sync")) ||
        (r = cu(cudaStreamSynchronize(s_tables), "kernel stack sync")) ||
        (r = cu(cudaStreamSynchronize(s_call), "kernel stack sync")))
      return fail(r);
  return GG_OK;
}

template <typename Real>
int kernels_create(gg_kernels** out, size_t num_w_planes, const int* support,
                   int oversample, int conv_size_half, const Real* conv_func,
                   int on_device, cudaStream_t s);

// Generates the taper x chirp cube on the device (gg_kgen.cu) and builds a
// kernel stack from it; the cube also goes to d_cube_out when given.
template <typename Real>
int kernels_generate(gg_kernels** out, size_t num_w_planes, const int* support,
                     int oversample, int conv_size_half,
                     const double* w_planes, Real* d_cube_out,
                     cudaStream_t s) {
  if (!out) return set_error(GG_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if (!w_planes) return set_error(GG_ERR_INVALID_ARG, "w_planes is NULL");
  // Same checks as a caller's cube (the cube pointer is not needed yet).
  GG_TRY(validate_stack(num_w_planes, support, oversample, conv_size_half,
                        w_planes));
  DevBuf d_support, d_w, d_total, cube;
  GG_TRY(d_support.ensure(num_w_planes * sizeof(int)));
  GG_TRY(d_w.ensure(num_w_planes * sizeof(double)));
  GG_TRY(d_total.ensure(num_w_planes * 16));
  Real* d_cube = d_cube_out;
  if (!d_cube) {
    GG_TRY(cube.ensure(num_w_planes * (size_t)conv_size_half *
                       conv_size_half * 2 * sizeof(Real)));
    d_cube = cube.as<Real>();
  }
  GG_CUDA(cudaMemcpyAsync(d_support.p, support, num_w_planes * sizeof(int),
                          cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(d_w.p, w_planes, num_w_planes * sizeof(double),
                          cudaMemcpyHostToDevice, s));
  GG_CUDA(launch_kernel_generate<Real>((int)num_w_planes, d_support.as<int>(),
                                       d_w.as<double>(), oversample,
                                       conv_size_half, d_total.p, d_cube, s));
  // kernels_create synchronises s before returning, so the temporaries
  // above outlive the kernels that read them.
  return kernels_create<Real>(out, num_w_planes, support, oversample,
                              conv_size_half, d_cube, 1, s);
}

template <typename Real>
int kernels_create(gg_kernels** out, size_t num_w_planes, const int* support,
                   int oversample, int conv_size_half, const Real* conv_func,
                   int on_device, cudaStream_t s) {
  if (!out) return set_error(GG_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  gg_kernels* k = new gg_kernels();
  const int r = kernels_fill<Real>(k, num_w_planes, support, oversample,
                                   conv_size_half, conv_func, on_device, s,
                                   nullptr, true);
  if (r != GG_OK) {
    delete k;
    return r;
  }
  *out = k;
  return GG_OK;
}

}  // namespace

// ===========================================================================
// Plans (workspace)
// ===========================================================================
struct gg_plan {
  int device = 0;
  DevBuf cell, meta, vw, rec_count, rec_offset;
  DevBuf blk_norm, blk_skip, blk_macs;
  DevBuf keys0, vals0, keys1, vals1, sort_tmp, scan_tmp;
  DevBuf tile_start, item_a, item_b, items, split_tiles, partials, tile_slot;
  DevBuf scalars;  // device scalars, see Scalar below
  uint32_t* h_scalars = nullptr;  // pinned mirror
  gg_stats stats{};
  // Phase events (recorded only when profiling is enabled).
  static constexpr int kEvents = 6;
  int forced_shape = -1;  // tile shape index, -1 = chosen per call
  int forced_stage = -1;  // slice staging 0/1, -1 = chosen per call
  int items_per_cta = 4;  // work-item granularity of heavy-tile splits
  int sort_detail = 2;    // low sort-key fields: 2 plane+class, 1 plane, 0
  int ctas_per_sm = 0;    // cap on resident gridding CTAs, 0 = none
  int plane_group_mb = 0; // slab bytes per plane group, 0 = L2 size / 2
  int queue_order = 0;    // tuning tile_order: 0 radius, 1 row by row
  int lane_groups = 0;    // tuning lane_groups: 0 automatic, 1, 2
  int tile_phases = 0;    // tuning tile_phases: 0 automatic, 1, 2, 4
  // Tile phases requested for the call being placed (0 automatic, chosen
  // with the shape; see gridding_phases).
  int call_phases = 1;
  // Batched calls larger than one sort can index (see batched_split): the
  // grids are cut into sub-batches, each gridded by its own sub-plan, which
  // keeps its geometry for replays.  A sub-plan takes the sort's transient
  // buffers (keys, the unsorted side of the values, sort and count scratch)
  // from `scratch`, its parent, so they exist once.
  gg_plan* scratch = nullptr;
  // Inputs of a host call arriving in pieces (set by the drop-in around
  // its gridding pipeline): placement of points [in_chunk_end[k-1],
  // in_chunk_end[k]) waits for in_chunk_ready[k].
  int in_chunks = 0;
  const cudaEvent_t* in_chunk_ready = nullptr;
  size_t in_chunk_end[8] = {};
  std::vector<std::unique_ptr<gg_plan>> subs;
  std::vector<int> sub_grid0;     // first grid of each sub-batch, + end
  std::vector<unsigned long long> sub_vis0;  // first visibility of each
  bool subs_valid = false;
  unsigned long long batch_limit = 0;  // visibilities per sub-batch, 0 auto
  // Event the gridding passes wait for (a grid upload on another stream),
  // or null.
  cudaEvent_t grid_wait = nullptr;
  // Kernel stack built on another stream (host calls): placement leaves
  // the norm terms out, and once stack_wait is done they are formed from
  // the placed points' weights (norm_weight, device, the call's Real) and
  // added to norm_out; the gridding and degridding kernels wait for it too.
  cudaEvent_t stack_wait = nullptr;
  const void* norm_weight = nullptr;
  double* norm_out = nullptr;
  // Touched spans (single-grid calls, when h_spans is set): per tile row
  // tv, the tile columns [lo[tv], hi[tv]) that hold records, lo at
  // h_spans[0..tiles_v) and hi after it (hi = 0: no records in the row).
  // spans_written says they were produced for the last call; spans_ready
  // (when spans_async) is recorded once they have reached h_spans.
  uint32_t* h_spans = nullptr;
  int h_spans_cap = 0;
  // Split passes (single-grid calls, when split_event is set and
  // split_row > 0): the first and the last plane group are gridded in two
  // passes by tile rows, rows [0, split_row) first (TileGeom::split_tv).
  // The first group's upper pass waits for split_wait (the upper rows'
  // upload) and its lower pass for grid_wait; split_event is recorded once
  // the upper rows are final.  split_launched says the last call recorded
  // it, split_tv is that call's split in tile rows.
  cudaEvent_t split_event = nullptr;
  cudaEvent_t split_wait = nullptr;
  int split_row = 0;
  bool split_launched = false;
  int split_tv = 0;
  cudaEvent_t spans_ready = nullptr;
  bool spans_written = false, spans_async = false;
  int spans_tiles_v = 0, spans_tile_u = 0, spans_tile_v = 0;
  DevBuf spans;
  // Plane groups of the last call (see TileGeom): table, and what it was
  // computed for.
  DevBuf plane_group, group_items;
  std::vector<int> h_plane_group;
  unsigned long long pg_kernels = 0;   // id of the kernel stack
  long long pg_budget = -1;           // requested budget (bytes)
  int pg_max_groups = 0;
  int pg_groups = 1;
  bool profile = false;
  bool events_valid = false;
  cudaEvent_t ev[kEvents] = {};
  // Batched calls: per-visibility norm terms, chunk table, chunk totals,
  // per-grid visibility offsets.
  DevBuf nterm, chunk_begin, grid_chunk0, chunk_part, grid_offsets;
  // Degridding: partial result of every record, at its emission slot.
  DevBuf rec_out;
  // Queue order of the tiles (ItemBuffers::tile_order) and the geometry it
  // was made for: grid_size, tile_u, tile_v, num_grids.
  DevBuf tile_order;
  std::vector<int> h_tile_order;
  int to_key[5] = {0, 0, 0, 0, -1};
  // Staging of the host-pointer entry points.
  DevBuf in_uu, in_vv, in_ww, in_vis, in_weight, in_grid, in_misc;
  // Direct mode of a single-grid call (see launch_tile_groups): the device
  // address of the caller's grid in host memory, or null; the per-tile
  // plane-group table; direct_launched says the last call used it.
  void* host_grid = nullptr;
  DevBuf tile_groups;
  bool direct_launched = false;
  // Geometry kept by the last batched call for replays on new amplitudes:
  // placement (cell, meta), sorted records, work items and launch shape.
  struct Kept {
    bool valid = false;
    const gg_kernels* kernels = nullptr;
    bool is_double = false;
    unsigned long long num_points = 0;
    int num_grids = 0, grid_size = 0, num_chunks = 0, num_tiles = 0;
    int num_ctas = 0, shape = 0;
    bool stage = false;
    uint32_t num_records = 0;
    TileGeom geom{};
    int group_span = 1;   // virtual groups per gridding launch
    const uint32_t* rec_vis = nullptr;
  } kept;
  ~gg_plan() {
    if (h_scalars) cudaFreeHost(h_scalars);
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
  }
  void mark(int i, cudaStream_t s) {
    if (profile) cudaEventRecord(ev[i], s);
  }
};

namespace {

enum Scalar {
  kTotalRecords = 0,
  kNumItems,
  kNumSlots,
  kNumSplit,
  kCounter,
  kShape,
  kDeviceError,   // set by a kernel whose bounded wait ran out; sticky
  kScalarCount
};
// Tile shape of the degridding kernel (32 x 64 cells).
constexpr int kDegridShape = 0;
// 64-bit device scalars live after the 32-bit ones.
constexpr size_t kScalar64Offset = 64;
enum Scalar64 {
  kMacs = 0, kSkipScratch, kDirectCells, kRecords64, kScalar64Count
};

unsigned long long* scalar64(gg_plan* p, int i) {
  return (unsigned long long*)((char*)p->scalars.p + kScalar64Offset) + i;
}

int plan_init(gg_plan* p) {
  GG_TRY(current_device(&p->device));
  GG_TRY(p->scalars.ensure(kScalar64Offset + kScalar64Count * 8));
  GG_CUDA(cudaMemset(p->scalars.p, 0, p->scalars.bytes));
  GG_CUDA(cudaMallocHost(&p->h_scalars, 64));
  return GG_OK;
}

// The device error flag of a plan (set when a kernel's bounded wait ran
// out; the call's results are then incomplete).  The stream must be idle.
int check_device_error(gg_plan* p, cudaStream_t s) {
  uint32_t flag = 0;
  GG_CUDA(cudaMemcpyAsync(&flag, p->scalars.as<uint32_t>() + kDeviceError,
                          4, cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  if (!flag && p->subs_valid)
    for (size_t k = 0; k + 1 < p->sub_grid0.size(); ++k)
      GG_TRY(check_device_error(p->subs[k].get(), s));
  if (flag)
    return set_error(GG_ERR_CUDA,
                     "a gridding kernel's bounded wait ran out; the results "
                     "of that call are incomplete");
  return GG_OK;
}

// Tile geometry and sort-key layout for one tile shape (see gg_grid.cu).
// Key = tile | plane | |offset| class in 32 bits; the low fields shrink
// (ordering within a tile gets coarser) if the grids have many tiles.
TileGeom make_geom(int shape, int grid_size, int num_grids,
                   const gg_kernels* K, int* key_bits, int sort_detail = 2,
                   int num_groups = 1, const int* plane_group = nullptr,
                   int phases = 1) {
  TileGeom g{};
  g.tile_u = tile_u_of_shape(shape);
  g.tile_v = tile_v_of_shape(shape);
  g.tile_phases = phases > 1 ? phases : 1;
  g.tiles_u = (grid_size + g.tile_u - 1) / g.tile_u + (phases > 1 ? 1 : 0);
  g.tiles_v = (grid_size + g.tile_v - 1) / g.tile_v;
  g.num_grids = num_grids;
  g.tiles_total = num_grids * g.tiles_u * g.tiles_v;
  set_strips(g, grid_size);
  g.num_groups = num_groups;
  g.plane_group = num_groups > 1 ? plane_group : nullptr;
  const int tile_bits = ceil_log2((unsigned long long)num_groups *
                                  g.tiles_total);
  int plane_bits = ceil_log2((unsigned long long)K->num_planes);
  int phase_bits =
      ceil_log2((unsigned long long)(K->omax + 1) * (K->omax + 1));
  if (sort_detail < 2) phase_bits = 0;
  if (sort_detail < 1) plane_bits = 0;
  if (tile_bits + plane_bits + phase_bits > 32) phase_bits = 0;
  if (tile_bits + plane_bits + phase_bits > 32) plane_bits = 0;
  g.plane_bits = plane_bits;
  g.phase_bits = phase_bits;
  g.phase_side = K->omax + 1;
  *key_bits = tile_bits + plane_bits + phase_bits;
  return g;
}

// Most (visibility, tile) records one visibility of support s_max can
// make with the tile shape `shape` (-1: the largest over all shapes): an
// interval of 2 s + 1 cells meets at most 2 s / w + 2 tiles of width w.
unsigned long long max_records_per_vis(int s_max, int shape) {
  unsigned long long r = 1;
  for (int sh = 0; sh < kNumTileShapes; ++sh) {
    if (shape >= 0 && sh != shape) continue;
    const unsigned long long c =
        (unsigned long long)(2 * s_max / tile_u_of_shape(sh) + 2) *
        (unsigned long long)(2 * s_max / tile_v_of_shape(sh) + 2);
    r = std::max(r, c);
  }
  return r;
}

// Record streams per consumer warp (TileGeom::lane_groups): half-warp
// streams exist for the 32-wide tiles that read taps from the slab stack;
// 0 (automatic) keeps whole warps (half-warp streams measured 4 % faster on
// the synthetic-challenge shape, 2 % slower on the SKA-LOW one).
int lane_groups_for(const gg_plan* plan, int tile_u, bool stage) {
  if (tile_u != 32 || stage) return 1;
  return plan->lane_groups == 2 ? 2 : 1;
}

// Plane groups for a call: consecutive w-planes cut into as many groups as
// the byte budget (plan->plane_group_mb, or half the L2 cache) needs, with
// even slab bytes per group, so that each gridding pass reads a stack slice
// that stays resident in L2.  At most max_groups groups (the sort key's
// spare bits).
// Uploads the plane -> group table when it changes; returns the number of
// groups in *num_groups.
int plane_groups(gg_plan* plan, const gg_kernels* K, int max_groups,
                 cudaStream_t s, int* num_groups) {
  long long budget = (long long)plan->plane_group_mb << 20;
  const long long requested = budget;
  if (budget <= 0) {
    int l2 = 0;
    GG_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, K->device));
    budget = std::max<long long>((long long)l2 / 2, 1 << 20);
  }
  max_groups = std::max(1, std::min(max_groups, 64));
  if (plan->pg_kernels == K->id && plan->pg_budget == requested &&
      plan->pg_max_groups == max_groups) {
    *num_groups = plan->pg_groups;
    return GG_OK;
  }
  const long long tap_bytes = K->is_double ? 16 : 8;
  std::vector<long long> bytes(K->num_planes);
  long long total = 0;
  for (int p = 0; p < K->num_planes; ++p) {
    bytes[p] = (K->omax + 1) *
               slab_taps(K->h_support[p], K->oversample, K->omax) * tap_bytes;
    total += bytes[p];
  }
  // More groups than allowed: widen the budget until they fit.
  budget = std::max(budget, (total + max_groups - 1) / max_groups);
  // As many groups as the budget needs, with even byte counts: plane p
  // joins the group that holds the middle of its bytes (a greedy fill to
  // the budget would leave the last group with the remainder, and the first
  // groups' slabs, at the full budget, less likely to stay in L2).
  const long long want = std::max(1LL, (total + budget - 1) / budget);
  const double target = (double)total / (double)want;
  std::vector<int>& grp = plan->h_plane_group;
  grp.assign(K->num_planes, 0);
  int g = -1;
  long long last = -1, before = 0;
  for (int p = 0; p < K->num_planes; ++p) {
    const long long q = std::min(
        want - 1, (long long)(((double)before + 0.5 * (double)bytes[p]) /
                              target));
    if (q != last) {
      ++g;
      last = q;
    }
    grp[p] = g;
    before += bytes[p];
  }
  const int groups = g + 1;
  GG_TRY(plan->plane_group.ensure((size_t)K->num_planes * sizeof(int)));
  GG_CUDA(cudaMemcpyAsync(plan->plane_group.p, grp.data(),
                          (size_t)K->num_planes * sizeof(int),
                          cudaMemcpyHostToDevice, s));
  plan->pg_kernels = K->id;
  plan->pg_budget = requested;
  plan->pg_max_groups = max_groups;
  plan->pg_groups = groups;
  *num_groups = groups;
  return GG_OK;
}

// Most tiles of a call over all shapes, with the extra tile column of
// tile phases.
int max_tiles(int grid_size, int num_grids) {
  int m = 0;
  for (int sh = 0; sh < kNumTileShapes; ++sh) {
    const int tu = tile_u_of_shape(sh), tv = tile_v_of_shape(sh);
    m = std::max(m, ((grid_size + tu - 1) / tu + 1) *
                        ((grid_size + tv - 1) / tv));
  }
  return m * num_grids;
}

// Tile phases requested for a gridding call (TileGeom::tile_phases): the
// plan's setting (0: chosen with the tile shape, see choose_shape), or 1
// where eight phases' extra sort-key bits and the split passes' would not
// fit 32-bit keys.
int gridding_phases(const gg_plan* plan, int grid_size, int num_grids) {
  if (ceil_log2((unsigned long long)max_tiles(grid_size, num_grids)) + 3 + 2 >
      32)
    return 1;
  return plan->tile_phases;
}

template <typename Real>
int place_and_count(gg_plan* plan, const gg_kernels* K,
                    const PlaceParams<Real>& pp, int forced_shape,
                    double* d_norm, unsigned long long* d_num_skipped,
                    cudaStream_t s, PlaceOut* po_out);
template <typename Real>
int bin_and_grid(gg_plan* plan, const gg_kernels* K, size_t n,
                 const PlaceOut& po, int grid_size, int num_grids,
                 const unsigned long long* d_grid_offsets, Real* d_grid,
                 long long grid_stride, cudaStream_t s);

// Per-chunk partial sums of a batched call live in one buffer: norm, skip
// and MAC count arrays of num_chunks + 1 entries each.
struct ChunkParts {
  double* norm;
  unsigned long long* skip;
  unsigned long long* macs;
};
ChunkParts chunk_parts(gg_plan* p, int num_chunks) {
  ChunkParts c;
  c.norm = p->chunk_part.as<double>();
  c.skip = (unsigned long long*)(c.norm + num_chunks + 1);
  c.macs = c.skip + num_chunks + 1;
  return c;
}

template <typename Real>
int grid_pipeline(gg_plan* plan, const gg_kernels* K, size_t num_points,
                  const Real* uu, const Real* vv, const Real* ww,
                  const Real* vis, const Real* weight, Real cell_size_rad,
                  Real w_scale, int grid_size,
                  unsigned long long* d_num_skipped, double* d_norm,
                  Real* d_grid, cudaStream_t s) {
  using R2 = typename Vec2<Real>::type;
  if (!plan || !K) return set_error(GG_ERR_INVALID_ARG, "plan or kernels is NULL");
  if (K->is_double != (sizeof(Real) == 8))
    return set_error(GG_ERR_INVALID_ARG,
                     "kernel stack precision does not match the call");
  if (grid_size < 1 || grid_size > kMaxGridSize)
    return set_error(GG_ERR_UNSUPPORTED, "grid_size = %d outside [1, %d]",
                     grid_size, kMaxGridSize);
  if (num_points > 0xFFFFFFF0ull)
    return set_error(GG_ERR_UNSUPPORTED,
                     "num_points = %zu exceeds 2^32-16 per call", num_points);
  if (num_points > 0 && (!uu || !vv || !ww || !vis || !weight))
    return set_error(GG_ERR_INVALID_ARG, "an input array is NULL");
  if (!d_grid || !d_norm || !d_num_skipped)
    return set_error(GG_ERR_INVALID_ARG, "an output pointer is NULL");
  int dev;
  GG_TRY(current_device(&dev));
  if (dev != K->device || dev != plan->device)
    return set_error(GG_ERR_INVALID_ARG,
                     "plan, kernel stack and current device differ");

  plan->stats = gg_stats{};
  plan->stats.num_points = num_points;
  plan->events_valid = false;
  plan->kept.valid = false;
  plan->subs_valid = false;

  const size_t n = num_points;
  PlaceParams<Real> pp;
  pp.uu = uu; pp.vv = vv; pp.ww = ww; pp.vis = vis; pp.weight = weight;
  // oskar_grid_wproj.c:148 (and :59): grid_scale = grid_size * cell_size
  // in the call's precision.
  pp.grid_scale = (Real)grid_size * cell_size_rad;
  pp.w_scale = w_scale;
  pp.grid_size = grid_size;
  pp.grid_centre = grid_size / 2;
  pp.num_points = n;
  pp.defer_norm = plan->stack_wait != nullptr;

  if (n == 0) {
    GG_CUDA(cudaMemsetAsync(d_num_skipped, 0, sizeof(unsigned long long), s));
    return GG_OK;
  }
  PlaceOut po;
  plan->call_phases = gridding_phases(plan, grid_size, 1);
  GG_TRY(place_and_count<Real>(plan, K, pp, plan->forced_shape, d_norm,
                               d_num_skipped, s, &po));
  return bin_and_grid<Real>(plan, K, n, po, grid_size, 1, nullptr, d_grid, 0,
                            s);
}

// The first half of a single-grid call, shared by gridding and degridding:
// placement (skip count, norm and MAC totals), records per visibility and
// their offsets, then the call's one host synchronisation (the record total
// sizes the sort buffers and the tile shape picks the kernel).  pp.vis and
// pp.weight are null for degridding, which places coordinates only.
template <typename Real>
int place_and_count(gg_plan* plan, const gg_kernels* K,
                    const PlaceParams<Real>& pp, int forced_shape,
                    double* d_norm, unsigned long long* d_num_skipped,
                    cudaStream_t s, PlaceOut* po_out) {
  using R2 = typename Vec2<Real>::type;
  const StackView view = K->view();
  const size_t n = pp.num_points;
  const int tiles_cap = max_tiles(pp.grid_size, 1);
  const int nblk = place_num_blocks(n);
  GG_TRY(plan->cell.ensure(n * 4 + 4));
  GG_TRY(plan->meta.ensure(n * 4 + 4));
  if (pp.vis) GG_TRY(plan->vw.ensure(n * sizeof(R2) + sizeof(R2)));
  GG_TRY(plan->rec_count.ensure(n * 4 + 4));
  GG_TRY(plan->rec_offset.ensure(n * 4 + 4));
  GG_TRY(plan->blk_norm.ensure(nblk * sizeof(double)));
  GG_TRY(plan->blk_skip.ensure(nblk * 8));
  GG_TRY(plan->blk_macs.ensure(nblk * 8));
  GG_TRY(plan->scan_tmp.ensure(scan_temp_bytes(std::max<size_t>(n, tiles_cap))));
  uint32_t* sc = plan->scalars.as<uint32_t>();

  plan->mark(0, s);
  PlaceOut po;
  po.cell = plan->cell.as<uint32_t>();
  po.meta = plan->meta.as<uint32_t>();
  po.vw = pp.vis ? plan->vw.p : nullptr;
  po.rec_count = plan->rec_count.as<uint32_t>();
  po.blk_norm = plan->blk_norm.as<double>();
  po.blk_skip = plan->blk_skip.as<unsigned long long>();
  po.blk_macs = plan->blk_macs.as<unsigned long long>();
  if (plan->in_chunks > 0) {
    // Each piece is placed as soon as it is on the device; the pieces
    // start on block boundaries, so the per-block partials are the ones a
    // single launch writes.
    size_t a = 0;
    for (int k = 0; k < plan->in_chunks; ++k) {
      const size_t b = plan->in_chunk_end[k];
      GG_CUDA(cudaStreamWaitEvent(s, plan->in_chunk_ready[k], 0));
      if (b <= a) continue;
      PlaceParams<Real> pk = pp;
      pk.uu = pp.uu + a; pk.vv = pp.vv + a; pk.ww = pp.ww + a;
      pk.vis = pp.vis ? pp.vis + 2 * a : nullptr;
      pk.weight = pp.weight ? pp.weight + a : nullptr;
      pk.num_points = b - a;
      PlaceOut ok = po;
      ok.cell = po.cell + a;
      ok.meta = po.meta + a;
      ok.vw = po.vw ? (void*)((R2*)po.vw + a) : nullptr;
      const size_t blk = a / kPlaceBlock;
      ok.blk_norm = po.blk_norm + blk;
      ok.blk_skip = po.blk_skip + blk;
      ok.blk_macs = po.blk_macs + blk;
      GG_CUDA(launch_place<Real>(pk, view, TileGeom{}, 0, 0, ok, s));
      a = b;
    }
  } else {
    GG_CUDA(launch_place<Real>(pp, view, TileGeom{}, 0, 0, po, s));
  }
  GG_CUDA(launch_place_finalize(po.blk_norm, po.blk_skip, po.blk_macs, nblk,
                                n, forced_shape,
                                pp.defer_norm ? nullptr : d_norm,
                                d_num_skipped, scalar64(plan, kMacs),
                                sc + kShape, s, plan->call_phases));
  GG_CUDA(launch_count_records(po.cell, po.meta, n, view, sc + kShape,
                               po.rec_count, s));
  GG_CUDA(exclusive_scan_u32(po.rec_count, plan->rec_offset.as<uint32_t>(), n,
                             sc + kTotalRecords, plan->scan_tmp.p, s));
  plan->stats.num_launches = 6;  // place, finalize, count, 3-kernel scan
  plan->mark(1, s);
  GG_CUDA(cudaMemcpyAsync(plan->h_scalars, sc, 4 * kScalarCount,
                          cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaMemcpyAsync((char*)plan->h_scalars + 32, scalar64(plan, kMacs),
                          8, cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  *po_out = po;
  return GG_OK;
}

// Records binned by tile (bin_records): the sorted (key, visibility)
// pairs, the tile geometry and each virtual tile's record range
// (plan->tile_start).
struct Bins {
  uint32_t total = 0;
  int shape = 0;
  bool stage = false;
  int num_groups = 1, num_tiles = 0, grid_size = 0;
  TileGeom geom{};
  const uint32_t* keys = nullptr;
  const uint32_t* vals = nullptr;
};

// After the host has read back the record total and the tile shape: plane
// groups, tile geometry, record emission, the sort and the tile bounds.
// Batched calls pass the device array of per-grid visibility offsets.
template <typename Real>
int bin_records(gg_plan* plan, const gg_kernels* K, size_t n,
                const PlaceOut& po, int grid_size, int num_grids,
                const unsigned long long* d_grid_offsets, cudaStream_t s,
                Bins* b) {
  const StackView view = K->view();
  if (plan->h_scalars[kDeviceError])
    return set_error(GG_ERR_CUDA,
                     "an earlier call with this plan had a gridding kernel "
                     "whose bounded wait ran out");
  const uint32_t total = plan->h_scalars[kTotalRecords];
  const int shape = (int)(plan->h_scalars[kShape] & 0xFFu);
  // The scan's 32-bit record total wraps past 2^32: where the call could
  // make that many records, count them in 64 bits and refuse the call
  // rather than size the sort from a wrapped total.
  if ((unsigned long long)n * max_records_per_vis(K->support_max, shape) >
      0xFFFFFFF0ull) {
    unsigned long long records = 0;
    GG_CUDA(sum_u32(po.rec_count, n, scalar64(plan, kRecords64), s));
    GG_CUDA(cudaMemcpyAsync(&records, scalar64(plan, kRecords64),
                            sizeof(records), cudaMemcpyDeviceToHost, s));
    GG_CUDA(cudaStreamSynchronize(s));
    if (records > 0xFFFFFFF0ull)
      return set_error(GG_ERR_UNSUPPORTED,
                       "the call makes %llu (visibility, tile) records, more "
                       "than 2^32-16; split it (batched calls do so by "
                       "grids)", records);
  }
  const bool stage = plan->forced_stage >= 0
                         ? plan->forced_stage != 0
                         : ((plan->h_scalars[kShape] >> 8) & 1u) != 0;
  plan->stats.num_records = total;
  memcpy(&plan->stats.num_macs, (char*)plan->h_scalars + 32, 8);
  int key_bits = 0;
  // Tile phases (chosen with the shape; placement counted the records with
  // them): one more tile column and a phase field in the virtual group.
  const int phases = phases_of_shape(plan->h_scalars[kShape]);
  const int phase_bits = ceil_log2((unsigned long long)phases);
  // Plane groups: as many as the key's spare bits above the tile index
  // allow (at most 64).
  const int base_bits = ceil_log2((unsigned long long)num_grids *
                                  ((grid_size + tile_u_of_shape(shape) - 1) /
                                       tile_u_of_shape(shape) +
                                   (phases > 1 ? 1 : 0)) *
                                  ((grid_size + tile_v_of_shape(shape) - 1) /
                                   tile_v_of_shape(shape)));
  // Split passes need up to two more groups, so key bits for them.  The
  // caller sets split_row (a multiple of every tile height) only on large
  // grids, where the copies they overlap outweigh the extra passes' tails.
  const int spare = 32 - base_bits - phase_bits;
  const int tile_v = tile_v_of_shape(shape);
  const bool split = plan->split_event && num_grids == 1 && spare >= 2 &&
                     plan->split_row > 0 && plan->split_row < grid_size &&
                     plan->split_row % tile_v == 0;
  int pgroups = 1;
  GG_TRY(plane_groups(plan, K,
                      spare <= 0 ? 1
                                 : (1 << std::min(6, spare)) - (split ? 2 : 0),
                      s, &pgroups));
  // One plane group: its two passes serve both the upload and the copy
  // back.  Otherwise the first group's split waits for the upload in two
  // halves and the last group's split overlaps the copy back.
  const int split_mask = !split ? 0 : (pgroups == 1 ? 1 : 3);
  const int num_groups =
      (pgroups + (split_mask & 1) + ((split_mask >> 1) & 1)) * phases;
  TileGeom geom = make_geom(shape, grid_size, num_grids, K, &key_bits,
                            plan->sort_detail, num_groups,
                            plan->plane_group.as<int>(), phases);
  geom.split_tv = split ? plan->split_row / tile_v : 0;
  geom.split_mask = split_mask;
  geom.lane_groups = lane_groups_for(plan, geom.tile_u, stage);
  const int num_tiles = num_groups * geom.tiles_total;
  plan->stats.num_plane_groups = pgroups;
  plan->split_tv = geom.split_tv;
  // The work-item scans run over every virtual tile (group, tile).
  GG_TRY(plan->scan_tmp.ensure(scan_temp_bytes((size_t)num_tiles)));
  const int low_bits = geom.plane_bits + geom.phase_bits;
  plan->stats.tile_u = geom.tile_u;
  plan->stats.tile_v = geom.tile_v;
  if ((unsigned long long)total > 0xFFFFFFF0ull)
    return set_error(GG_ERR_UNSUPPORTED, "record count overflow");
  plan->kept.num_records = total;
  plan->kept.geom = geom;
  plan->kept.shape = shape;
  plan->kept.stage = stage;
  plan->kept.num_tiles = num_tiles;
  b->total = total;
  b->shape = shape;
  b->stage = stage;
  b->num_groups = num_groups;
  b->num_tiles = num_tiles;
  b->grid_size = grid_size;
  b->geom = geom;
  if (total == 0) return GG_OK;

  // The sorted values stay with the plan (replays read them); the keys,
  // the values' other side and the sort scratch are transient and, for a
  // sub-plan, its parent's.
  gg_plan* T = plan->scratch ? plan->scratch : plan;
  const bool alt_final =
      total > 1 && key_bits > 0 && ((key_bits + 7) / 8) % 2 == 1;
  DevBuf& v0 = alt_final ? T->vals0 : plan->vals0;
  DevBuf& v1 = alt_final ? plan->vals1 : T->vals1;
  GG_TRY(T->keys0.ensure((size_t)total * 4));
  GG_TRY(v0.ensure((size_t)total * 4));
  GG_TRY(T->keys1.ensure((size_t)total * 4));
  GG_TRY(v1.ensure((size_t)total * 4));
  GG_TRY(T->sort_tmp.ensure(radix_temp_bytes(total)));
  GG_CUDA(launch_emit_records(po.cell, po.meta,
                              T->rec_offset.as<uint32_t>(), n, view, geom,
                              0, 0, T->keys0.as<uint32_t>(),
                              v0.as<uint32_t>(), s, d_grid_offsets,
                              num_grids));
  bool in_alt = false;
  GG_CUDA(radix_sort_pairs(T->keys0.as<uint32_t>(), v0.as<uint32_t>(),
                           T->keys1.as<uint32_t>(), v1.as<uint32_t>(), total,
                           key_bits, T->sort_tmp.p, s, &in_alt));
  if (in_alt != alt_final)
    return set_error(GG_ERR_CUDA, "internal: sort pass count mismatch");
  b->keys = in_alt ? T->keys1.as<uint32_t>() : T->keys0.as<uint32_t>();
  b->vals = in_alt ? v1.as<uint32_t>() : v0.as<uint32_t>();
  plan->stats.num_launches += 1 + 5 * (unsigned)((key_bits + 7) / 8);
  plan->mark(2, s);

  GG_TRY(plan->tile_start.ensure((size_t)(num_tiles + 1) * 4));
  GG_CUDA(launch_tile_bounds(b->keys, total, low_bits, num_tiles,
                             plan->tile_start.as<uint32_t>(), s));
  plan->stats.num_launches += 1;
  return GG_OK;
}

// Queue order of the tiles of one group: grid by grid, and within a grid by
// the distance of the tile's centre from the uv origin (the grid centre),
// nearest first.  On telescope data the w-plane of a visibility grows with
// its baseline, so tiles at the same distance use similar planes and the
// CTAs running at one time share more kernel slabs in L2; the heavy
// central tiles also start first.  Uploaded when the geometry changes.
int tile_queue_order(gg_plan* plan, const TileGeom& g, int grid_size,
                     cudaStream_t s, const int** out) {
  const int key[5] = {grid_size, g.tile_u, g.tile_v, g.num_grids,
                      plan->queue_order};
  if (!std::equal(key, key + 5, plan->to_key) ||
      (int)plan->h_tile_order.size() != g.tiles_total) {
    const int tpg = g.tiles_u * g.tiles_v;
    std::vector<long long> r2(g.tiles_total);
    for (int l = 0; l < g.tiles_total; ++l) {
      const int tl = l % tpg;
      const long long du =
          (long long)(tl % g.tiles_u) * g.tile_u + g.tile_u / 2 - grid_size / 2;
      const long long dv =
          (long long)(tl / g.tiles_u) * g.tile_v + g.tile_v / 2 - grid_size / 2;
      r2[l] = plan->queue_order == 1 ? l : du * du + dv * dv;
    }
    std::vector<int>& ord = plan->h_tile_order;
    ord.resize(g.tiles_total);
    for (int l = 0; l < g.tiles_total; ++l) ord[l] = l;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
      const int ga = a / tpg, gb = b / tpg;
      return ga != gb ? ga < gb : r2[a] < r2[b];
    });
    GG_TRY(plan->tile_order.ensure(ord.size() * sizeof(int)));
    GG_CUDA(cudaMemcpyAsync(plan->tile_order.p, ord.data(),
                            ord.size() * sizeof(int), cudaMemcpyHostToDevice,
                            s));
    std::copy(key, key + 5, plan->to_key);
  }
  *out = plan->tile_order.as<int>();
  return GG_OK;
}

// The work-item queue of binned records for num_ctas persistent CTAs: heavy
// tiles are split into items of `chunk` records so that each of the call's
// `passes` launches has about items_per_cta items per CTA (the gridding
// passes of the groups; the degridder's single launch asks for as many
// items as all of them).  Items: at most one
// more per tile than
// total / chunk; partial-tile slots (split tiles only): at most
// 2 * total / chunk, each a tile of partial sums when partial_tiles is set
// (gridding; the degridder's items write no tile).
template <typename Real>
int build_work_items(gg_plan* plan, const Bins& b, int num_ctas, int passes,
                     bool partial_tiles, cudaStream_t s, ItemBuffers* ib,
                     int launch_span = 1) {
  using R2 = typename Vec2<Real>::type;
  uint32_t* sc = plan->scalars.as<uint32_t>();
  const int num_tiles = b.num_tiles;
  // items_per_cta items per CTA in each of the call's passes: every pass
  // ends with a tail up to one item long.
  const unsigned long long f =
      (unsigned long long)plan->items_per_cta * (unsigned long long)passes;
  const uint32_t chunk = (uint32_t)std::max<unsigned long long>(
      64, ((unsigned long long)b.total + f * num_ctas - 1) / (f * num_ctas));
  const size_t item_cap = (size_t)num_tiles + 2 * f * (size_t)num_ctas + 16;
  const size_t slot_cap = 2 * f * (size_t)num_ctas + 16;
  plan->stats.num_ctas = num_ctas;
  plan->stats.chunk_records = chunk;
  GG_TRY(plan->item_a.ensure((size_t)num_tiles * 4 + 4));
  GG_TRY(plan->item_b.ensure((size_t)num_tiles * 4 + 4));
  GG_TRY(plan->items.ensure(item_cap * sizeof(WorkItem)));
  GG_TRY(plan->split_tiles.ensure((size_t)num_tiles * sizeof(int4) + 16));
  GG_TRY(plan->tile_slot.ensure((size_t)num_tiles * sizeof(int2) + 16));
  // Gridding launches that take all the tile phases of a plane group
  // (launch_span = tile_phases): every tile of a later phase writes partial
  // tiles, as many as the scans count (read back below).
  const int pphases = partial_tiles && launch_span > 1 ? launch_span : 1;
  if (partial_tiles && pphases == 1)
    GG_TRY(plan->partials.ensure(slot_cap * b.geom.tile_u * b.geom.tile_v *
                                 sizeof(R2)));
  GG_TRY(plan->group_items.ensure((size_t)(b.num_groups + 1) * 4));
  ib->chunks = plan->item_a.as<uint32_t>();
  ib->split_chunks = plan->item_b.as<uint32_t>();
  ib->group_items = plan->group_items.as<uint32_t>();
  ib->num_groups = b.num_groups;
  ib->num_items = sc + kNumItems;
  ib->num_slots = sc + kNumSlots;
  ib->items = plan->items.as<WorkItem>();
  ib->split_tiles = plan->split_tiles.as<int4>();
  ib->num_split = sc + kNumSplit;
  ib->counter = sc + kCounter;
  ib->scan_tmp = plan->scan_tmp.p;
  ib->partial_phases = pphases;
  ib->tile_slot = plan->tile_slot.as<int2>();
  GG_TRY(tile_queue_order(plan, b.geom, b.grid_size, s, &ib->tile_order));
  GG_CUDA(launch_build_items(plan->tile_start.as<uint32_t>(), num_tiles,
                             b.total, chunk, *ib, s));
  if (pphases > 1) {
    uint32_t slots = 0;
    GG_CUDA(cudaMemcpyAsync(&slots, ib->num_slots, sizeof(slots),
                            cudaMemcpyDeviceToHost, s));
    GG_CUDA(cudaStreamSynchronize(s));
    GG_TRY(plan->partials.ensure(((size_t)slots + 1) * b.geom.tile_u *
                                 b.geom.tile_v * sizeof(R2)));
  }
  // item counts, 2 scans, item emit
  plan->stats.num_launches += 1 + 6 + 1;
  return GG_OK;
}

// The second half of a gridding call: binning, work items, the
// tile-gridding kernel and the partial reductions.  Batched calls pass the
// device array of per-grid visibility offsets and the stride between grids.
template <typename Real>
int bin_and_grid(gg_plan* plan, const gg_kernels* K, size_t n,
                 const PlaceOut& po, int grid_size, int num_grids,
                 const unsigned long long* d_grid_offsets, Real* d_grid,
                 long long grid_stride, cudaStream_t s) {
  const StackView view = K->view();
  uint32_t* sc = plan->scalars.as<uint32_t>();
  Bins b;
  GG_TRY(bin_records<Real>(plan, K, n, po, grid_size, num_grids,
                           d_grid_offsets, s, &b));
  if (plan->stack_wait) {
    // The stack was built beside placement and binning.
    GG_CUDA(cudaStreamWaitEvent(s, plan->stack_wait, 0));
    if (plan->norm_out) {
      GG_CUDA(launch_norm_terms<Real>(po.meta, (const Real*)plan->norm_weight,
                                      n, view, plan->blk_norm.as<double>(),
                                      plan->norm_out, s));
      plan->stats.num_launches += 2;
    }
  }
  const TileGeom& geom = b.geom;
  const bool want_spans = plan->h_spans && num_grids == 1 &&
                          2 * geom.tiles_v <= plan->h_spans_cap;
  if (want_spans) {
    // Spans in strips of tile_u / tile_phases columns (launch_touched_spans).
    plan->spans_tiles_v = geom.tiles_v;
    plan->spans_tile_u = 1 << geom.strip_shift;
    plan->spans_tile_v = geom.tile_v;
    plan->spans_async = b.total > 0;
    plan->spans_written = true;
    if (b.total == 0)   // nothing is gridded: no row is touched
      memset(plan->h_spans + geom.tiles_v, 0, geom.tiles_v * sizeof(uint32_t));
  }
  if (b.total == 0) return GG_OK;

  if (want_spans) {
    const size_t half = (size_t)geom.tiles_v * sizeof(uint32_t);
    GG_TRY(plan->spans.ensure(2 * half));
    GG_CUDA(cudaMemsetAsync(plan->spans.p, 0xFF, half, s));
    GG_CUDA(cudaMemsetAsync(plan->spans.as<char>() + half, 0, half, s));
    GG_CUDA(launch_touched_spans(plan->tile_start.as<uint32_t>(), b.num_tiles,
                                 geom, grid_size, plan->spans.as<uint32_t>(),
                                 plan->spans.as<uint32_t>() + geom.tiles_v,
                                 s));
    GG_CUDA(cudaMemcpyAsync(plan->h_spans, plan->spans.p, 2 * half,
                            cudaMemcpyDeviceToHost, s));
    GG_CUDA(cudaEventRecord(plan->spans_ready, s));
    plan->stats.num_launches += 1;
  }

  int sms = 0;
  GG_TRY(num_sms_of_current(&sms));
  int per_sm = grid_tiles_ctas_per_sm<Real>(geom.tile_u, b.stage,
                                            geom.lane_groups);
  if (plan->ctas_per_sm > 0) per_sm = std::min(per_sm, plan->ctas_per_sm);
  const int num_ctas = sms * per_sm;
  plan->stats.slice_staging = b.stage ? 1 : 0;
  ItemBuffers ib;
  // The tile phases of a plane group share one launch, their later phases'
  // tiles added as partial tiles after it (where the kernels use the
  // caller's grid at host, those additions read and write it per strip).
  // Items are sized per virtual group (a phase's tiles are smaller, and
  // larger items leave longer tails).
  const int span = geom.tile_phases;
  GG_TRY(build_work_items<Real>(plan, b, num_ctas, geom.num_groups, true, s,
                                &ib, span));
  plan->kept.group_span = span;
  plan->kept.rec_vis = b.vals;
  plan->kept.num_ctas = num_ctas;
  // The upload plane group g's first launch waits for (entry g * P), and
  // the event after its last launch (entry g * P + P - 1) that marks the
  // upper rows final.
  const int P = geom.tile_phases;
  const int base_groups = geom.num_groups / P;
  std::vector<cudaEvent_t> wait_before(geom.num_groups, nullptr);
  std::vector<cudaEvent_t> record_after(geom.num_groups, nullptr);
  wait_before[0] = plan->grid_wait;
  if (geom.split_mask & 1) {
    if (plan->split_wait) wait_before[0] = plan->split_wait;
    wait_before[P] = plan->grid_wait;
  }
  const int upper_done = (geom.split_mask & 2) ? base_groups - 2
                         : geom.split_mask == 1 ? 0
                                                : -1;
  if (upper_done >= 0) record_after[upper_done * P + P - 1] = plan->split_event;
  const uint32_t* tile_groups = nullptr;
  if (plan->host_grid) {
    if (num_grids != 1 || geom.split_mask != 0 || geom.num_groups >= 0xFFFF)
      return set_error(GG_ERR_UNSUPPORTED,
                       "direct grid access needs one grid, no split passes "
                       "and fewer than 65535 plane groups");
    GG_TRY(plan->tile_groups.ensure((size_t)num_strips(geom) * 4));
    GG_CUDA(launch_tile_groups(plan->tile_start.as<uint32_t>(), geom,
                               grid_size, plan->tile_groups.as<uint32_t>(),
                               scalar64(plan, kDirectCells), s));
    tile_groups = plan->tile_groups.as<uint32_t>();
    plan->direct_launched = true;
    plan->stats.num_launches += 1;
  }
  plan->mark(3, s);
  GG_CUDA(launch_grid_tiles<Real>(
      ib.items, ib.group_items, ib.counter, sc + kDeviceError, b.vals,
      po.cell, po.meta, po.vw, view, geom, grid_size, d_grid, grid_stride,
      plan->partials.as<Real>(), ib.split_tiles, ib.num_split, b.num_tiles,
      num_ctas, b.stage, s, wait_before.data(), record_after.data(),
      (Real*)plan->host_grid, tile_groups, span, plan->tile_slot.as<int2>(),
      plan->tile_start.as<uint32_t>()));
  plan->split_launched = upper_done >= 0;
  plan->mark(4, s);
  plan->mark(5, s);
  // each gridding launch and its partial reduction (one per virtual group,
  // or one over all the phases of a launch)
  plan->stats.num_launches += 2 * (b.num_groups / span);
  plan->events_valid = plan->profile;
  return GG_OK;
}

// Many grids in one call: the visibilities of grid g are
// [h_offsets[g], h_offsets[g+1]) of the concatenated input arrays and its
// grid is d_grids + g * grid_size^2 * 2.  One placement pass, one sort and
// one persistent tile-gridding launch cover every grid.
template <typename Real>
int batched_pipeline(gg_plan* plan, const gg_kernels* K, int num_grids,
                     const unsigned long long* h_offsets, const Real* uu,
                     const Real* vv, const Real* ww, const Real* vis,
                     const Real* weight, Real cell_size_rad, Real w_scale,
                     int grid_size, unsigned long long* d_num_skipped,
                     double* d_norm, Real* d_grids, cudaStream_t s) {
  using R2 = typename Vec2<Real>::type;
  if (!plan || !K) return set_error(GG_ERR_INVALID_ARG, "plan or kernels is NULL");
  if (K->is_double != (sizeof(Real) == 8))
    return set_error(GG_ERR_INVALID_ARG,
                     "kernel stack precision does not match the call");
  if (num_grids < 1 || !h_offsets)
    return set_error(GG_ERR_INVALID_ARG, "need num_grids >= 1 and offsets");
  if (grid_size < 1 || grid_size > kMaxGridSize)
    return set_error(GG_ERR_UNSUPPORTED, "grid_size = %d outside [1, %d]",
                     grid_size, kMaxGridSize);
  if (h_offsets[0] != 0)
    return set_error(GG_ERR_INVALID_ARG, "offsets[0] must be 0");
  for (int g = 0; g < num_grids; ++g)
    if (h_offsets[g + 1] < h_offsets[g])
      return set_error(GG_ERR_INVALID_ARG,
                       "offsets must not decrease (grid %d)", g);
  const unsigned long long n = h_offsets[num_grids];
  if (n > 0xFFFFFFF0ull)
    return set_error(GG_ERR_UNSUPPORTED,
                     "%llu visibilities exceed 2^32-16 per call", n);
  if (n > 0 && (!uu || !vv || !ww || !vis || !weight))
    return set_error(GG_ERR_INVALID_ARG, "an input array is NULL");
  if (!d_grids || !d_norm || !d_num_skipped)
    return set_error(GG_ERR_INVALID_ARG, "an output pointer is NULL");
  const long long grid_stride = 2LL * grid_size * grid_size;
  int key_bits = 0;
  make_geom(0, grid_size, num_grids, K, &key_bits);
  if (ceil_log2((unsigned long long)max_tiles(grid_size, num_grids)) > 32)
    return set_error(GG_ERR_UNSUPPORTED, "too many tiles for 32-bit keys");
  int dev;
  GG_TRY(current_device(&dev));
  if (dev != K->device || dev != plan->device)
    return set_error(GG_ERR_INVALID_ARG,
                     "plan, kernel stack and current device differ");

  plan->stats = gg_stats{};
  plan->stats.num_points = n;
  plan->events_valid = false;
  plan->kept.valid = false;
  plan->subs_valid = false;
  const StackView view = K->view();
  const int tiles_cap = max_tiles(grid_size, num_grids);

  // Chunk table of the per-grid reductions (chunks never straddle grids).
  constexpr unsigned long long kChunk = 1ull << 16;
  std::vector<unsigned long long> chunk_begin;
  std::vector<int> grid_chunk0(num_grids + 1);
  for (int g = 0; g < num_grids; ++g) {
    grid_chunk0[g] = (int)chunk_begin.size();
    for (unsigned long long b = h_offsets[g]; b < h_offsets[g + 1];
         b += kChunk)
      chunk_begin.push_back(b);
  }
  grid_chunk0[num_grids] = (int)chunk_begin.size();
  const int num_chunks = (int)chunk_begin.size();
  chunk_begin.push_back(n);

  GG_TRY(plan->cell.ensure(n * 4 + 4));
  GG_TRY(plan->meta.ensure(n * 4 + 4));
  GG_TRY(plan->vw.ensure(n * sizeof(R2) + sizeof(R2)));
  // Counts and offsets of records per visibility: transient (a sub-plan
  // takes its parent's).
  gg_plan* T = plan->scratch ? plan->scratch : plan;
  GG_TRY(T->rec_count.ensure(n * 4 + 4));
  GG_TRY(T->rec_offset.ensure(n * 4 + 4));
  GG_TRY(plan->nterm.ensure(n * 8 + 8));
  GG_TRY(plan->chunk_begin.ensure(chunk_begin.size() * 8));
  GG_TRY(plan->grid_chunk0.ensure(grid_chunk0.size() * 4));
  GG_TRY(plan->chunk_part.ensure((size_t)(num_chunks + 1) * 24));
  GG_TRY(plan->grid_offsets.ensure((size_t)(num_grids + 1) * 8));
  GG_TRY(plan->scan_tmp.ensure(
      scan_temp_bytes(std::max<size_t>(n, (size_t)tiles_cap))));
  GG_CUDA(cudaMemcpyAsync(plan->chunk_begin.p, chunk_begin.data(),
                          chunk_begin.size() * 8, cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(plan->grid_chunk0.p, grid_chunk0.data(),
                          grid_chunk0.size() * 4, cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(plan->grid_offsets.p, h_offsets,
                          (size_t)(num_grids + 1) * 8, cudaMemcpyHostToDevice,
                          s));

  uint32_t* sc = plan->scalars.as<uint32_t>();
  PlaceParams<Real> pp;
  pp.uu = uu; pp.vv = vv; pp.ww = ww; pp.vis = vis; pp.weight = weight;
  pp.grid_scale = (Real)grid_size * cell_size_rad;
  pp.w_scale = w_scale;
  pp.grid_size = grid_size;
  pp.grid_centre = grid_size / 2;
  pp.num_points = n;
  PlaceOut po;
  po.cell = plan->cell.as<uint32_t>();
  po.meta = plan->meta.as<uint32_t>();
  po.vw = plan->vw.p;
  po.rec_count = T->rec_count.as<uint32_t>();
  po.blk_norm = nullptr;
  po.blk_skip = nullptr;
  po.blk_macs = nullptr;
  const ChunkParts cp = chunk_parts(plan, num_chunks);
  plan->call_phases = gridding_phases(plan, grid_size, num_grids);

  plan->mark(0, s);
  GG_CUDA(launch_place_batched<Real>(pp, view, po, plan->nterm.as<double>(),
                                     s));
  GG_CUDA(launch_batch_totals(
      po.meta, plan->nterm.as<double>(), view, num_chunks,
      plan->chunk_begin.as<unsigned long long>(), num_grids,
      plan->grid_chunk0.as<int>(), cp.norm, cp.skip, cp.macs,
      plan->forced_shape, d_norm, d_num_skipped, scalar64(plan, kMacs),
      sc + kShape, s, plan->call_phases));
  GG_CUDA(launch_count_records(po.cell, po.meta, n, view, sc + kShape,
                               po.rec_count, s));
  GG_CUDA(exclusive_scan_u32(po.rec_count, T->rec_offset.as<uint32_t>(), n,
                             sc + kTotalRecords, plan->scan_tmp.p, s));
  // place, chunk totals, finalize, count, 3-kernel scan
  plan->stats.num_launches = (num_chunks > 0 ? 7 : 6);
  plan->mark(1, s);
  GG_CUDA(cudaMemcpyAsync(plan->h_scalars, sc, 4 * kScalarCount,
                          cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaMemcpyAsync((char*)plan->h_scalars + 32, scalar64(plan, kMacs),
                          8, cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  GG_TRY(bin_and_grid<Real>(plan, K, n, po, grid_size, num_grids,
                            plan->grid_offsets.as<unsigned long long>(),
                            d_grids, grid_stride, s));
  gg_plan::Kept& kp = plan->kept;
  kp.kernels = K;
  kp.is_double = sizeof(Real) == 8;
  kp.num_points = n;
  kp.num_grids = num_grids;
  kp.grid_size = grid_size;
  kp.num_chunks = num_chunks;
  kp.valid = true;
  return GG_OK;
}

// A batched call whose records might not fit the 32-bit record indices of
// one sort (or exceed the plan's batch_limit) is cut, between grids, into
// sub-batches of consecutive grids, each of at most
// (2^32 - 16) / max_records_per_vis visibilities; each sub-batch is gridded
// by a sub-plan of its own (placement, sort and persistent gridding
// launches as in one batched call), in grid order, and keeps its geometry,
// so that a replay covers every grid.  Calls that fit go straight to
// batched_pipeline.
template <typename Real>
int batched_split(gg_plan* plan, const gg_kernels* K, int num_grids,
                  const unsigned long long* h_offsets, const Real* uu,
                  const Real* vv, const Real* ww, const Real* vis,
                  const Real* weight, Real cell_size_rad, Real w_scale,
                  int grid_size, unsigned long long* d_num_skipped,
                  double* d_norm, Real* d_grids, cudaStream_t s) {
  if (!plan || !K) return set_error(GG_ERR_INVALID_ARG, "plan or kernels is NULL");
  if (num_grids < 1 || !h_offsets)
    return set_error(GG_ERR_INVALID_ARG, "need num_grids >= 1 and offsets");
  plan->subs_valid = false;
  int s_max = 0;
  for (int p = 0; p < K->num_planes; ++p)
    s_max = std::max(s_max, K->h_support[p]);
  unsigned long long limit =
      0xFFFFFFF0ull / max_records_per_vis(s_max, plan->forced_shape);
  if (plan->batch_limit > 0) limit = std::min(limit, plan->batch_limit);
  const unsigned long long n = h_offsets[num_grids];
  if (n <= limit || num_grids == 1)
    return batched_pipeline<Real>(plan, K, num_grids, h_offsets, uu, vv, ww,
                                  vis, weight, cell_size_rad, w_scale,
                                  grid_size, d_num_skipped, d_norm, d_grids,
                                  s);
  // Sub-batches: consecutive grids while the sum stays within the limit.
  std::vector<int> g0{0};
  for (int g = 0; g < num_grids; ++g) {
    if (h_offsets[g + 1] < h_offsets[g])
      return set_error(GG_ERR_INVALID_ARG,
                       "offsets must not decrease (grid %d)", g);
    const unsigned long long cnt = h_offsets[g + 1] - h_offsets[g];
    if (cnt > limit)
      return set_error(GG_ERR_UNSUPPORTED,
                       "grid %d has %llu visibilities, more than one sort "
                       "can index with support %d (%llu); split it", g, cnt,
                       s_max, limit);
    if (h_offsets[g + 1] - h_offsets[g0.back()] > limit) g0.push_back(g);
  }
  g0.push_back(num_grids);
  const int nsub = (int)g0.size() - 1;
  while ((int)plan->subs.size() < nsub) {
    std::unique_ptr<gg_plan> c(new gg_plan());
    GG_TRY(plan_init(c.get()));
    c->scratch = plan;
    plan->subs.push_back(std::move(c));
  }
  const long long grid_stride = 2LL * grid_size * grid_size;
  gg_stats total{};
  std::vector<unsigned long long> offs;
  for (int k = 0; k < nsub; ++k) {
    gg_plan* c = plan->subs[k].get();
    c->forced_shape = plan->forced_shape;
    c->forced_stage = plan->forced_stage;
    c->items_per_cta = plan->items_per_cta;
    c->sort_detail = plan->sort_detail;
    c->ctas_per_sm = plan->ctas_per_sm;
    c->plane_group_mb = plan->plane_group_mb;
    c->queue_order = plan->queue_order;
    c->lane_groups = plan->lane_groups;
    c->tile_phases = plan->tile_phases;
    const int a = g0[k], b = g0[k + 1];
    const unsigned long long v0 = h_offsets[a];
    offs.assign(h_offsets + a, h_offsets + b + 1);
    for (auto& o : offs) o -= v0;
    GG_TRY(batched_pipeline<Real>(
        c, K, b - a, offs.data(), uu + v0, vv + v0, ww + v0, vis + 2 * v0,
        weight + v0, cell_size_rad, w_scale, grid_size, d_num_skipped + a,
        d_norm + a, d_grids + a * grid_stride, s));
    const gg_stats& st = c->stats;
    if (k == 0) total = st;
    else {
      total.num_points += st.num_points;
      total.num_records += st.num_records;
      total.num_macs += st.num_macs;
      total.num_launches += st.num_launches;
      total.num_ctas = std::max(total.num_ctas, st.num_ctas);
      total.num_plane_groups =
          std::max(total.num_plane_groups, st.num_plane_groups);
    }
  }
  plan->stats = total;
  plan->events_valid = false;
  plan->kept.valid = false;
  plan->subs_valid = false;
  plan->sub_grid0 = g0;
  plan->sub_vis0.resize(nsub);
  for (int k = 0; k < nsub; ++k) plan->sub_vis0[k] = h_offsets[g0[k]];
  plan->subs_valid = true;
  return GG_OK;
}

// Grids new amplitudes and weights on the geometry kept by the plan's last
// batched call: weighted visibilities and norm terms, per-grid totals, the
// persistent tile-gridding launch and the partial reduction.  Kernel
// launches and one memset only -- no host synchronisation, no allocation --
// so the call can be captured in a CUDA graph and replayed.
template <typename Real>
int replay_pipeline(gg_plan* plan, const gg_kernels* K, const Real* vis,
                    const Real* weight, unsigned long long* d_num_skipped,
                    double* d_norm, Real* d_grids, cudaStream_t s) {
  if (!plan || !K) return set_error(GG_ERR_INVALID_ARG, "plan or kernels is NULL");
  if (plan->subs_valid) {
    // A call cut into sub-batches: each sub-plan replays its grids.
    const int nsub = (int)plan->sub_grid0.size() - 1;
    for (int k = 0; k < nsub; ++k) {
      gg_plan* c = plan->subs[k].get();
      const int a = plan->sub_grid0[k];
      const unsigned long long v0 = plan->sub_vis0[k];
      GG_TRY(replay_pipeline<Real>(
          c, K, vis ? vis + 2 * v0 : vis, weight ? weight + v0 : weight,
          d_num_skipped ? d_num_skipped + a : d_num_skipped,
          d_norm ? d_norm + a : d_norm,
          d_grids ? d_grids + a * 2LL * c->kept.grid_size * c->kept.grid_size
                  : d_grids,
          s));
    }
    return GG_OK;
  }
  const gg_plan::Kept& kp = plan->kept;
  if (!kp.valid)
    return set_error(GG_ERR_INVALID_ARG,
                     "the plan holds no batched-call geometry to replay");
  if (kp.kernels != K || kp.is_double != (sizeof(Real) == 8))
    return set_error(GG_ERR_INVALID_ARG,
                     "replay needs the kernel stack and precision of the "
                     "batched call that made the geometry");
  if (kp.num_points > 0 && (!vis || !weight))
    return set_error(GG_ERR_INVALID_ARG, "an input array is NULL");
  if (!d_grids || !d_norm || !d_num_skipped)
    return set_error(GG_ERR_INVALID_ARG, "an output pointer is NULL");
  const StackView view = K->view();
  uint32_t* sc = plan->scalars.as<uint32_t>();
  const ChunkParts cp = chunk_parts(plan, kp.num_chunks);
  GG_CUDA(launch_revalue<Real>(vis, weight, plan->meta.as<uint32_t>(), view,
                               kp.num_points, plan->vw.p,
                               plan->nterm.as<double>(), s));
  GG_CUDA(launch_batch_totals(
      plan->meta.as<uint32_t>(), plan->nterm.as<double>(), view,
      kp.num_chunks, plan->chunk_begin.as<unsigned long long>(),
      kp.num_grids, plan->grid_chunk0.as<int>(), cp.norm, cp.skip, cp.macs,
      kp.shape, d_norm, d_num_skipped, scalar64(plan, kMacs), sc + kShape,
      s));
  if (kp.num_records == 0) return GG_OK;
  const long long grid_stride = 2LL * kp.grid_size * kp.grid_size;
  GG_CUDA(launch_grid_tiles<Real>(
      plan->items.as<WorkItem>(), plan->group_items.as<uint32_t>(),
      sc + kCounter,
      sc + kDeviceError, kp.rec_vis, plan->cell.as<uint32_t>(),
      plan->meta.as<uint32_t>(), plan->vw.p, view, kp.geom, kp.grid_size,
      d_grids, grid_stride, plan->partials.as<Real>(),
      plan->split_tiles.as<int4>(), sc + kNumSplit, kp.num_tiles, kp.num_ctas,
      kp.stage, s, nullptr, nullptr, nullptr, nullptr, kp.group_span,
      plan->tile_slot.as<int2>(), plan->tile_start.as<uint32_t>()));
  return GG_OK;
}

template <typename Real>
int degrid_pipeline(gg_plan* plan, const gg_kernels* K, size_t num_points,
                    const Real* uu, const Real* vv, const Real* ww,
                    Real cell_size_rad, Real w_scale, int grid_size,
                    const Real* d_grid, Real* d_out, cudaStream_t s) {
  if (!plan || !K) return set_error(GG_ERR_INVALID_ARG, "plan or kernels is NULL");
  if (K->is_double != (sizeof(Real) == 8))
    return set_error(GG_ERR_INVALID_ARG,
                     "kernel stack precision does not match the call");
  if (grid_size < 1 || grid_size > kMaxGridSize)
    return set_error(GG_ERR_UNSUPPORTED, "grid_size = %d outside [1, %d]",
                     grid_size, kMaxGridSize);
  if (num_points > 0 && (!uu || !vv || !ww || !d_grid || !d_out))
    return set_error(GG_ERR_INVALID_ARG, "an array is NULL");
  PlaceParams<Real> pp;
  pp.uu = uu; pp.vv = vv; pp.ww = ww; pp.vis = nullptr; pp.weight = nullptr;
  pp.grid_scale = (Real)grid_size * cell_size_rad;
  pp.w_scale = w_scale;
  pp.grid_size = grid_size;
  pp.grid_centre = grid_size / 2;
  pp.num_points = num_points;
  if (num_points == 0) return GG_OK;
  if (num_points > 0xFFFFFFF0ull)
    return set_error(GG_ERR_UNSUPPORTED,
                     "num_points = %zu exceeds 2^32-16 per call", num_points);
  int dev;
  GG_TRY(current_device(&dev));
  if (dev != K->device || dev != plan->device)
    return set_error(GG_ERR_INVALID_ARG,
                     "plan, kernel stack and current device differ");
  // The gridder's placement, records and work items (32 x 64-cell tiles;
  // geometry kept for a batched replay is discarded), then the tile
  // kernel and the per-visibility sums.
  plan->stats = gg_stats{};
  plan->stats.num_points = num_points;
  plan->events_valid = false;
  plan->kept.valid = false;
  plan->subs_valid = false;
  const size_t n = num_points;
  const StackView view = K->view();
  PlaceOut po;
  plan->call_phases = gridding_phases(plan, grid_size, 1);
  GG_TRY(place_and_count<Real>(plan, K, pp, kDegridShape, nullptr, nullptr, s,
                               &po));
  Bins b;
  GG_TRY(bin_records<Real>(plan, K, n, po, grid_size, 1, nullptr, s, &b));
  if (b.total == 0) {
    GG_CUDA(cudaMemsetAsync(d_out, 0, 2 * n * sizeof(Real), s));
    return GG_OK;
  }
  if (b.total > 0x7FFFFFFFu)
    return set_error(GG_ERR_UNSUPPORTED,
                     "%u records: degridding takes at most 2^31 - 1 per call",
                     b.total);
  int sms = 0;
  GG_TRY(num_sms_of_current(&sms));
  int per_sm = degrid_tiles_ctas_per_sm<Real>();
  if (plan->ctas_per_sm > 0) per_sm = std::min(per_sm, plan->ctas_per_sm);
  const int num_ctas = sms * per_sm;
  ItemBuffers ib;
  // One launch over the queue of all plane groups, as many items as the
  // gridding's passes together.
  GG_TRY(build_work_items<Real>(plan, b, num_ctas, b.num_groups, false, s,
                                &ib));
  GG_TRY(plan->rec_out.ensure((size_t)b.total * 2 * sizeof(Real)));
  uint32_t* sc = plan->scalars.as<uint32_t>();
  if (plan->grid_wait) GG_CUDA(cudaStreamWaitEvent(s, plan->grid_wait, 0));
  if (plan->stack_wait) GG_CUDA(cudaStreamWaitEvent(s, plan->stack_wait, 0));
  GG_CUDA(launch_degrid_tiles<Real>(
      ib.items, ib.num_items, ib.counter, sc + kDeviceError, b.vals, po.cell,
      po.meta, plan->rec_offset.as<uint32_t>(), view, b.geom, grid_size,
      d_grid, plan->rec_out.p, num_ctas, s));
  GG_CUDA(launch_degrid_finish<Real>(po.rec_count,
                                     plan->rec_offset.as<uint32_t>(),
                                     plan->rec_out.p, n, d_out, s));
  plan->stats.num_launches += 2;
  return GG_OK;
}

// True when every page of [p, p + bytes) is resident.  A page the process
// has never touched would be faulted in through the device's address
// translation on first access, at some 25 microseconds a page on a Grace
// host: such arrays (a freshly allocated zero grid, say) are copied
// instead.
bool pages_resident(const void* p, size_t bytes) {
  static const long page = sysconf(_SC_PAGESIZE);
  if (page <= 0 || bytes == 0) return false;
  const uintptr_t a = (uintptr_t)p & ~(uintptr_t)(page - 1);
  const uintptr_t e = (uintptr_t)p + bytes;
  thread_local std::vector<unsigned char> vec;
  vec.resize((e - a + page - 1) / page);
  if (mincore((void*)a, e - a, vec.data()) != 0) return false;
  for (unsigned char c : vec)
    if (!(c & 1)) return false;
  return true;
}

// The device address of a host array of a host-pointer call when kernels
// may read (and, for the grid, write) it in place under the device's access
// mode (page-locked and mapped, or pageable and resident on a device that
// reads pageable memory through the host's page tables), else null.
void* direct_host_address(DeviceState* st, int dev, const void* grid,
                          size_t bytes, size_t align) {
  if (st->grid_access == GG_GRID_ACCESS_COPY ||
      (uintptr_t)grid % align != 0)
    return nullptr;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, grid) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type == cudaMemoryTypeHost) return at.devicePointer;
  if (at.type != cudaMemoryTypeUnregistered ||
      st->grid_access != GG_GRID_ACCESS_PAGEABLE)
    return nullptr;
  if (st->pageable_access < 0) {
    // Pageable memory in place only where the device reads it through the
    // host's page tables (address translation services on a coherent link):
    // no page moves to the device, so the caller's arrays stay where they
    // are.
    int v = 0, ats = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) !=
            cudaSuccess ||
        cudaDeviceGetAttribute(
            &ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) !=
            cudaSuccess) {
      cudaGetLastError();
      v = ats = 0;
    }
    st->pageable_access = v && ats;
  }
  return st->pageable_access && pages_resident(grid, bytes)
             ? const_cast<void*>(grid)
             : nullptr;
}

// Host-pointer drop-in: inputs staged, the grid used in place or copied.
// The kernel stack of a host-pointer call in the device's reused stack
// object: the caller's cube is staged every call and re-laid only when it
// differs from the one the stack was made from (the caller holds the
// device lock and synchronises the streams before returning).
template <typename Real>
int host_kernels(DeviceState* st, size_t num_w_planes, const int* support,
                 int oversample, int conv_size_half, const Real* conv_func,
                 cudaStream_t s, std::function<int()> uploads,
                 gg_kernels** out) {
  if (!st->host_kernels) st->host_kernels = new gg_kernels();
  gg_kernels* k = st->host_kernels;
  int dev;
  GG_TRY(current_device(&dev));
  const Real* mapped = (const Real*)direct_host_address(
      st, dev, conv_func,
      num_w_planes * (size_t)conv_size_half * conv_size_half * 2 *
          sizeof(Real),
      2 * sizeof(Real));
  // The stack still holds the re-layout of host_cube[cube_cur] when the
  // geometry (precision, planes, supports, oversampling, cube size) is the
  // same as then.
  const bool same_geometry =
      st->cube_cur >= 0 && k->is_double == (sizeof(Real) == 8) &&
      k->device == dev && k->num_planes == (int)num_w_planes &&
      k->oversample == oversample && k->conv_size_half == conv_size_half &&
      std::equal(support, support + num_w_planes, k->h_support.begin());
  const int next = st->cube_cur == 0 ? 1 : 0;
  const DevBuf* previous = same_geometry ? &st->host_cube[st->cube_cur]
                                         : nullptr;
  GG_TRY(st->cube_changed.ensure(sizeof(int)));
  st->cube_cur = -1;   // until the new stack is in place
  // The plane tables go first on the side stream, then the caller's
  // uploads (`uploads`, which records vis_ready there); the heavy part runs
  // on the stack stream after them, beside placement and binning on s, and
  // stack_ready marks its end.
  const StackStreams ss{st->copy_stream, st->stack_stream, st->tables_ready,
                        st->vis_ready, st->stack_ready, std::move(uploads),
                        st->cube_staged};
  GG_TRY(kernels_fill<Real>(k, num_w_planes, support, oversample,
                            conv_size_half, conv_func, 0, s,
                            &st->host_cube[next], false, mapped, previous,
                            st->cube_changed.as<int>(), &ss));
  st->cube_cur = next;
  *out = k;
  return GG_OK;
}

int ensure_copy_stream(DeviceState* st) {
  if (!st->copy_stream)
    GG_CUDA(cudaStreamCreateWithFlags(&st->copy_stream,
                                      cudaStreamNonBlocking));
  if (!st->stack_stream) {
    int least = 0, greatest = 0;
    GG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    GG_CUDA(cudaStreamCreateWithPriority(&st->stack_stream,
                                         cudaStreamNonBlocking, least));
  }
  for (cudaEvent_t* e : {&st->vis_ready, &st->grid_ready, &st->spans_ready,
                         &st->top_done, &st->top_up, &st->tables_ready,
                         &st->stack_ready, &st->cube_staged})
    if (!*e) GG_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  for (cudaEvent_t& e : st->chunk_ready)
    if (!e) GG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  if (!st->h_spans)
    GG_CUDA(cudaMallocHost(&st->h_spans,
                           DeviceState::kSpanCap * sizeof(uint32_t)));
  return GG_OK;
}

// The workspace plan of a device's host-pointer calls (made on first use;
// the caller holds the device lock).
int ensure_device_plan(DeviceState* st) {
  if (st->plan) return GG_OK;
  gg_plan* p = new gg_plan();
  const int r = plan_init(p);
  if (r != GG_OK) {
    delete p;
    return r;
  }
  st->plan = p;
  return GG_OK;
}

template <typename Real>
int dropin(size_t num_w_planes, const int* support, int oversample,
           int conv_size_half, const Real* conv_func, size_t num_points,
           const Real* uu, const Real* vv, const Real* ww, const Real* vis,
           const Real* weight, Real cell_size_rad, Real w_scale,
           int grid_size, size_t* num_skipped, double* norm, Real* grid) {
  const auto t_entry = std::chrono::steady_clock::now();
  auto since_entry = [&]() {
    return std::chrono::duration<double, std::milli>(
               std::chrono::steady_clock::now() - t_entry)
        .count();
  };
  if (!num_skipped || !norm || !grid)
    return set_error(GG_ERR_INVALID_ARG, "num_skipped, norm or grid is NULL");
  if (grid_size < 1 || grid_size > kMaxGridSize)
    return set_error(GG_ERR_UNSUPPORTED, "grid_size = %d outside [1, %d]",
                     grid_size, kMaxGridSize);
  if (num_points > 0 && (!uu || !vv || !ww || !vis || !weight))
    return set_error(GG_ERR_INVALID_ARG, "an input array is NULL");
  GG_TRY(validate_stack(num_w_planes, support, oversample, conv_size_half,
                        conv_func));
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  std::lock_guard<std::mutex> lk(st->mu);
  cudaStream_t s = st->stream;
  GG_TRY(ensure_device_plan(st));
  gg_plan* plan = st->plan;
  const size_t n = num_points;
  const size_t grid_bytes = (size_t)grid_size * grid_size * 2 * sizeof(Real);
  const size_t row_bytes = (size_t)grid_size * 2 * sizeof(Real);
  GG_TRY(plan->in_grid.ensure(grid_bytes));
  GG_TRY(plan->in_uu.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_vv.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_ww.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_vis.ensure(2 * n * sizeof(Real) + 16));
  GG_TRY(plan->in_weight.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_misc.ensure(64));
  double* d_norm = plan->in_misc.as<double>();
  unsigned long long* d_skip = (unsigned long long*)(plan->in_misc.as<char>() + 8);
  GG_TRY(ensure_copy_stream(st));
  struct CopyGuard {   // the side streams read the caller's arrays
    cudaStream_t s, t;
    ~CopyGuard() {
      cudaStreamSynchronize(s);
      cudaStreamSynchronize(t);
    }
  } copy_guard{st->copy_stream, st->stack_stream};
  // The visibilities go over the link first, on the side stream, and
  // placement and binning start as soon as they are in.  The kernel stack
  // is built beside them on the stack stream, its cube behind the
  // visibilities on the link; placement leaves out the norm terms, which
  // are formed once the stack is ready, before the gridding passes.  In
  // copy mode the grid goes up on the side stream behind the visibilities,
  // and only the gridding passes wait for it.
  st->profile_valid = false;
  st->host_ms[0] = since_entry();
  if (st->profile) GG_CUDA(cudaEventRecord(st->call_start, s));
  cudaStream_t cs = st->copy_stream;
  // In place: the gridding kernels read and write the caller's grid over
  // the host link (no upload, no copy back, no split passes).
  void* direct = n && num_w_planes < 0xFFFF
                     ? direct_host_address(st, dev, grid, grid_bytes,
                                           2 * sizeof(Real))
                     : nullptr;
  if (st->profile) GG_CUDA(cudaStreamWaitEvent(cs, st->call_start, 0));
  // The visibilities go up in pieces of whole placement blocks, and each
  // piece is placed while the next one crosses the link.
  const int nchunks = DeviceState::kInputChunks;
  size_t chunk_end[DeviceState::kInputChunks];
  for (int k = 0; k < nchunks; ++k) {
    const size_t e = (n * (k + 1) / nchunks + kPlaceBlock - 1) /
                     kPlaceBlock * kPlaceBlock;
    chunk_end[k] = k + 1 == nchunks ? n : std::min(e, n);
  }
  auto uploads = [&]() -> int {
    size_t a = 0;
    for (int k = 0; k < nchunks; ++k) {
      const size_t b = chunk_end[k], m = b - a;
      if (m) {
        GG_CUDA(cudaMemcpyAsync(plan->in_uu.as<Real>() + a, uu + a,
                                m * sizeof(Real), cudaMemcpyHostToDevice, cs));
        GG_CUDA(cudaMemcpyAsync(plan->in_vv.as<Real>() + a, vv + a,
                                m * sizeof(Real), cudaMemcpyHostToDevice, cs));
        GG_CUDA(cudaMemcpyAsync(plan->in_ww.as<Real>() + a, ww + a,
                                m * sizeof(Real), cudaMemcpyHostToDevice, cs));
        GG_CUDA(cudaMemcpyAsync(plan->in_vis.as<Real>() + 2 * a, vis + 2 * a,
                                2 * m * sizeof(Real), cudaMemcpyHostToDevice,
                                cs));
        GG_CUDA(cudaMemcpyAsync(plan->in_weight.as<Real>() + a, weight + a,
                                m * sizeof(Real), cudaMemcpyHostToDevice, cs));
      }
      GG_CUDA(cudaEventRecord(st->chunk_ready[k], cs));
      a = b;
    }
    GG_CUDA(cudaEventRecord(st->vis_ready, cs));
    return GG_OK;
  };
  gg_kernels* K = nullptr;
  GG_TRY(host_kernels<Real>(st, num_w_planes, support, oversample,
                            conv_size_half, conv_func, s, uploads, &K));
  // On grids of 128 MiB and more the grid goes up in two halves by rows
  // (the split a multiple of 256 rows, so of every tile height): the
  // first plane group's upper pass waits for the upper half only, and the
  // upper rows go back while the last group's lower pass runs.  On smaller
  // grids the copies those passes would overlap are shorter than the extra
  // passes' tails (2048^2 FP32: 4 % slower end to end).
  const int split_row = !direct && grid_bytes >= ((size_t)128 << 20)
                            ? grid_size / 2 / 256 * 256
                            : 0;
  // Copied grids go over the link after the cube, so that the stack is
  // ready when the first pass can start.
  if (!direct && n) GG_CUDA(cudaStreamWaitEvent(cs, st->cube_staged, 0));
  if (direct) {
    // nothing to upload
  } else if (n && split_row > 0) {
    const size_t upper = (size_t)split_row * row_bytes;
    GG_CUDA(cudaMemcpyAsync(plan->in_grid.p, grid, upper,
                            cudaMemcpyHostToDevice, cs));
    GG_CUDA(cudaEventRecord(st->top_up, cs));
    GG_CUDA(cudaMemcpyAsync(plan->in_grid.as<char>() + upper,
                            (const char*)grid + upper, grid_bytes - upper,
                            cudaMemcpyHostToDevice, cs));
  } else if (n) {
    GG_CUDA(cudaMemcpyAsync(plan->in_grid.p, grid, grid_bytes,
                            cudaMemcpyHostToDevice, cs));
  }
  GG_CUDA(cudaEventRecord(st->grid_ready, cs));
  // Placement waits for each piece of the visibilities (in_chunk_ready);
  // whatever runs before it on s needs none of them.
  // The starting norm is set by a one-thread kernel rather than a copy, so
  // that it does not queue behind the uploads on the copy engines.
  GG_CUDA(launch_store_f64(d_norm, *norm, s));
  if (direct)
    GG_CUDA(cudaMemsetAsync(scalar64(plan, kDirectCells), 0,
                            sizeof(unsigned long long), s));
  plan->grid_wait = direct ? nullptr : st->grid_ready;
  plan->h_spans = direct ? nullptr : st->h_spans;
  plan->h_spans_cap = DeviceState::kSpanCap;
  plan->spans_ready = st->spans_ready;
  plan->spans_written = false;
  plan->split_event = direct ? nullptr : st->top_done;
  plan->split_wait = split_row > 0 ? st->top_up : nullptr;
  plan->split_row = split_row;
  plan->split_launched = false;
  plan->host_grid = direct;
  plan->direct_launched = false;
  plan->stack_wait = st->stack_ready;
  plan->norm_weight = plan->in_weight.p;
  plan->norm_out = d_norm;
  plan->in_chunks = nchunks;
  plan->in_chunk_ready = st->chunk_ready;
  std::copy(chunk_end, chunk_end + nchunks, plan->in_chunk_end);
  const int rc = grid_pipeline<Real>(plan, K, n, plan->in_uu.as<Real>(),
                                     plan->in_vv.as<Real>(),
                                     plan->in_ww.as<Real>(),
                                     plan->in_vis.as<Real>(),
                                     plan->in_weight.as<Real>(),
                                     cell_size_rad, w_scale, grid_size,
                                     d_skip, d_norm, plan->in_grid.as<Real>(),
                                     s);
  plan->grid_wait = nullptr;
  plan->h_spans = nullptr;
  plan->spans_ready = nullptr;
  plan->split_event = nullptr;
  plan->split_wait = nullptr;
  plan->split_row = 0;
  plan->host_grid = nullptr;
  plan->stack_wait = nullptr;
  plan->norm_weight = nullptr;
  plan->norm_out = nullptr;
  plan->in_chunks = 0;
  plan->in_chunk_ready = nullptr;
  GG_TRY(rc);
  // Copy back only what the call can have changed: cells outside every tile
  // that holds records were neither read nor written on the device, so the
  // caller's grid already holds them.  One 2-D copy per run of tile rows
  // with the same column span; the whole grid when the spans are unknown;
  // nothing when there were no visibilities.  When the last plane group was
  // gridded in two passes, the upper tile rows go back on the side stream
  // as soon as they are final, while the lower rows are still gridded.
  unsigned long long d2h_grid = 0, direct_cells = 0;
  if (direct) {
    // The kernels wrote the grid in place; only the count of the cells
    // they moved comes back (none when nothing was gridded).
    if (plan->direct_launched)
      GG_CUDA(cudaMemcpyAsync(&direct_cells, scalar64(plan, kDirectCells),
                              sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, s));
  } else if (n) {
    GG_CUDA(cudaStreamWaitEvent(s, st->grid_ready, 0));
    if (plan->spans_written) {
      if (plan->spans_async) GG_CUDA(cudaEventSynchronize(st->spans_ready));
      const int tiles_v = plan->spans_tiles_v;
      const uint32_t* lo = st->h_spans;
      const uint32_t* hi = st->h_spans + tiles_v;
      const size_t cell_bytes = 2 * sizeof(Real);
      const int split_tv = plan->split_launched ? plan->split_tv : 0;
      if (split_tv > 0) GG_CUDA(cudaStreamWaitEvent(cs, st->top_done, 0));
      for (int tv = 0; tv < tiles_v;) {
        if (hi[tv] == 0) {
          ++tv;
          continue;
        }
        int te = tv + 1;
        while (te < tiles_v && te != split_tv && lo[te] == lo[tv] &&
               hi[te] == hi[tv])
          ++te;
        const size_t r0 = (size_t)tv * plan->spans_tile_v;
        const size_t r1 =
            std::min((size_t)grid_size, (size_t)te * plan->spans_tile_v);
        const size_t c0 = (size_t)lo[tv] * plan->spans_tile_u;
        const size_t c1 =
            std::min((size_t)grid_size, (size_t)hi[tv] * plan->spans_tile_u);
        const size_t off = r0 * row_bytes + c0 * cell_bytes;
        GG_CUDA(cudaMemcpy2DAsync((char*)grid + off, row_bytes,
                                  plan->in_grid.as<char>() + off, row_bytes,
                                  (c1 - c0) * cell_bytes, r1 - r0,
                                  cudaMemcpyDeviceToHost,
                                  tv < split_tv ? cs : s));
        d2h_grid += (c1 - c0) * cell_bytes * (r1 - r0);
        tv = te;
      }
    } else {
      GG_CUDA(cudaMemcpyAsync(grid, plan->in_grid.p, grid_bytes,
                              cudaMemcpyDeviceToHost, s));
      d2h_grid = grid_bytes;
    }
  }
  double norm_out = 0.0;
  unsigned long long skip_out = 0;
  GG_CUDA(cudaMemcpyAsync(&norm_out, d_norm, sizeof(double),
                          cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaMemcpyAsync(&skip_out, d_skip, sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, s));
  if (st->profile) {
    GG_CUDA(cudaEventRecord(st->copies_done, cs));
    GG_CUDA(cudaStreamWaitEvent(s, st->copies_done, 0));
    GG_CUDA(cudaEventRecord(st->call_end, s));
  }
  GG_CUDA(cudaStreamSynchronize(s));
  GG_CUDA(cudaStreamSynchronize(cs));
  GG_CUDA(cudaStreamSynchronize(st->stack_stream));
  st->host_ms[1] = since_entry();
  GG_TRY(check_device_error(plan, s));
  st->profile_valid = st->profile && plan->events_valid;
  *norm = norm_out;
  *num_skipped = (size_t)skip_out;
  // Bytes moved: the cube and its plane tables, the inputs, the grid and
  // norm up; the grid spans, norm, skip count, the placement scalars, the
  // spans and the error flag down.
  // In place, the tiles that hold records cross the link once each way.
  const unsigned long long direct_bytes = direct_cells * 2 * sizeof(Real);
  st->last_h2d = K->h2d_bytes +
                 (n ? 6 * n * sizeof(Real) +
                          (direct ? direct_bytes : grid_bytes)
                    : 0) +
                 sizeof(double);
  st->last_d2h = d2h_grid + direct_bytes + sizeof(double) +
                 sizeof(unsigned long long) + sizeof(uint32_t) +
                 (n ? 4 * kScalarCount + 8 +
                          (plan->spans_written && plan->spans_async
                               ? 2 * (size_t)plan->spans_tiles_v * 4
                               : 0) +
                          (direct && plan->direct_launched ? 8 : 0)
                    : 0);
  st->host_ms[2] = since_entry();
  return GG_OK;
}

// ---- uniform weighting --------------------------------------------------
int weights_checks(gg_plan* plan, size_t n, int grid_size) {
  if (!plan) return set_error(GG_ERR_INVALID_ARG, "plan is NULL");
  if (grid_size < 1 || grid_size > kMaxGridSize)
    return set_error(GG_ERR_UNSUPPORTED, "grid_size = %d outside [1, %d]",
                     grid_size, kMaxGridSize);
  if (n > 0xFFFFFFF0ull)
    return set_error(GG_ERR_UNSUPPORTED,
                     "num_points = %zu exceeds 2^32-16 per call", n);
  int dev;
  GG_TRY(current_device(&dev));
  if (dev != plan->device)
    return set_error(GG_ERR_INVALID_ARG, "plan and current device differ");
  return GG_OK;
}

// Density grid: grid[cell] += weights of the cell's points, in point order
// (see gg_weights.cu).  Uses the plan's sort buffers.
template <typename Real>
int weights_write_pipeline(gg_plan* plan, size_t n, const Real* uu,
                           const Real* vv, const Real* weight,
                           Real cell_size_rad, int grid_size,
                           unsigned long long* d_num_skipped, Real* d_grid,
                           cudaStream_t s) {
  GG_TRY(weights_checks(plan, n, grid_size));
  if (n > 0 && (!uu || !vv || !weight))
    return set_error(GG_ERR_INVALID_ARG, "an input array is NULL");
  if (!d_grid || !d_num_skipped)
    return set_error(GG_ERR_INVALID_ARG, "an output pointer is NULL");
  plan->kept.valid = false;   // the sort buffers are reused below
  plan->subs_valid = false;
  GG_CUDA(cudaMemsetAsync(d_num_skipped, 0, sizeof(unsigned long long), s));
  if (n == 0) return GG_OK;
  GG_TRY(plan->keys0.ensure(n * 4));
  GG_TRY(plan->vals0.ensure(n * 4));
  GG_TRY(plan->keys1.ensure(n * 4));
  GG_TRY(plan->vals1.ensure(n * 4));
  GG_TRY(plan->sort_tmp.ensure(radix_temp_bytes(n)));
  GG_CUDA(launch_weight_keys<Real>(uu, vv, n, cell_size_rad, grid_size,
                                   plan->keys0.as<uint32_t>(),
                                   plan->vals0.as<uint32_t>(), d_num_skipped,
                                   s));
  const int key_bits =
      ceil_log2((unsigned long long)grid_size * grid_size + 1);
  bool in_alt = false;
  GG_CUDA(radix_sort_pairs(plan->keys0.as<uint32_t>(),
                           plan->vals0.as<uint32_t>(),
                           plan->keys1.as<uint32_t>(),
                           plan->vals1.as<uint32_t>(), n, key_bits,
                           plan->sort_tmp.p, s, &in_alt));
  GG_CUDA(launch_weight_runs<Real>(
      in_alt ? plan->keys1.as<uint32_t>() : plan->keys0.as<uint32_t>(),
      in_alt ? plan->vals1.as<uint32_t>() : plan->vals0.as<uint32_t>(), n,
      weight, grid_size, d_grid, s));
  return GG_OK;
}

template <typename Real>
int weights_read_pipeline(gg_plan* plan, size_t n, const Real* uu,
                          const Real* vv, const Real* w_in, Real* w_out,
                          Real cell_size_rad, int grid_size,
                          unsigned long long* d_num_skipped,
                          const Real* d_grid, cudaStream_t s) {
  GG_TRY(weights_checks(plan, n, grid_size));
  if (n > 0 && (!uu || !vv || !w_in || !w_out))
    return set_error(GG_ERR_INVALID_ARG, "an input or output array is NULL");
  if (!d_grid || !d_num_skipped)
    return set_error(GG_ERR_INVALID_ARG, "grid or num_skipped is NULL");
  GG_CUDA(cudaMemsetAsync(d_num_skipped, 0, sizeof(unsigned long long), s));
  GG_CUDA(launch_weights_read<Real>(uu, vv, w_in, w_out, n, cell_size_rad,
                                    grid_size, d_grid, d_num_skipped, s));
  return GG_OK;
}

template <typename Real>
int weights_write_host(size_t n, const Real* uu, const Real* vv,
                       const Real* weight, Real cell_size_rad, int grid_size,
                       size_t* num_skipped, Real* grid) {
  if (!num_skipped || !grid)
    return set_error(GG_ERR_INVALID_ARG, "num_skipped or grid is NULL");
  if (grid_size < 1 || grid_size > kMaxGridSize)
    return set_error(GG_ERR_UNSUPPORTED, "grid_size = %d outside [1, %d]",
                     grid_size, kMaxGridSize);
  if (n > 0 && (!uu || !vv || !weight))
    return set_error(GG_ERR_INVALID_ARG, "an input array is NULL");
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  std::lock_guard<std::mutex> lk(st->mu);
  cudaStream_t s = st->stream;
  GG_TRY(ensure_device_plan(st));
  gg_plan* plan = st->plan;
  const size_t grid_bytes = (size_t)grid_size * grid_size * sizeof(Real);
  GG_TRY(plan->in_uu.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_vv.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_weight.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_grid.ensure(grid_bytes));
  GG_TRY(plan->in_misc.ensure(64));
  unsigned long long* d_skip = plan->in_misc.as<unsigned long long>();
  if (n) {
    GG_CUDA(cudaMemcpyAsync(plan->in_uu.p, uu, n * sizeof(Real),
                            cudaMemcpyHostToDevice, s));
    GG_CUDA(cudaMemcpyAsync(plan->in_vv.p, vv, n * sizeof(Real),
                            cudaMemcpyHostToDevice, s));
    GG_CUDA(cudaMemcpyAsync(plan->in_weight.p, weight, n * sizeof(Real),
                            cudaMemcpyHostToDevice, s));
  }
  GG_CUDA(cudaMemcpyAsync(plan->in_grid.p, grid, grid_bytes,
                          cudaMemcpyHostToDevice, s));
  GG_TRY(weights_write_pipeline<Real>(
      plan, n, plan->in_uu.as<Real>(), plan->in_vv.as<Real>(),
      plan->in_weight.as<Real>(), cell_size_rad, grid_size, d_skip,
      plan->in_grid.as<Real>(), s));
  unsigned long long skip_out = 0;
  GG_CUDA(cudaMemcpyAsync(grid, plan->in_grid.p, grid_bytes,
                          cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaMemcpyAsync(&skip_out, d_skip, 8, cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  *num_skipped = (size_t)skip_out;
  return GG_OK;
}

template <typename Real>
int weights_read_host(size_t n, const Real* uu, const Real* vv,
                      const Real* w_in, Real* w_out, Real cell_size_rad,
                      int grid_size, size_t* num_skipped, const Real* grid) {
  if (!num_skipped || !grid)
    return set_error(GG_ERR_INVALID_ARG, "num_skipped or grid is NULL");
  if (grid_size < 1 || grid_size > kMaxGridSize)
    return set_error(GG_ERR_UNSUPPORTED, "grid_size = %d outside [1, %d]",
                     grid_size, kMaxGridSize);
  if (n > 0 && (!uu || !vv || !w_in || !w_out))
    return set_error(GG_ERR_INVALID_ARG, "an input or output array is NULL");
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  std::lock_guard<std::mutex> lk(st->mu);
  cudaStream_t s = st->stream;
  GG_TRY(ensure_device_plan(st));
  gg_plan* plan = st->plan;
  const size_t grid_bytes = (size_t)grid_size * grid_size * sizeof(Real);
  GG_TRY(plan->in_uu.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_vv.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_weight.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_vis.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_grid.ensure(grid_bytes));
  GG_TRY(plan->in_misc.ensure(64));
  unsigned long long* d_skip = plan->in_misc.as<unsigned long long>();
  if (n) {
    GG_CUDA(cudaMemcpyAsync(plan->in_uu.p, uu, n * sizeof(Real),
                            cudaMemcpyHostToDevice, s));
    GG_CUDA(cudaMemcpyAsync(plan->in_vv.p, vv, n * sizeof(Real),
                            cudaMemcpyHostToDevice, s));
    GG_CUDA(cudaMemcpyAsync(plan->in_weight.p, w_in, n * sizeof(Real),
                            cudaMemcpyHostToDevice, s));
    // Skipped points keep the caller's weight_out values.
    GG_CUDA(cudaMemcpyAsync(plan->in_vis.p, w_out, n * sizeof(Real),
                            cudaMemcpyHostToDevice, s));
  }
  GG_CUDA(cudaMemcpyAsync(plan->in_grid.p, grid, grid_bytes,
                          cudaMemcpyHostToDevice, s));
  GG_TRY(weights_read_pipeline<Real>(
      plan, n, plan->in_uu.as<Real>(), plan->in_vv.as<Real>(),
      plan->in_weight.as<Real>(), plan->in_vis.as<Real>(), cell_size_rad,
      grid_size, d_skip, plan->in_grid.as<Real>(), s));
  unsigned long long skip_out = 0;
  if (n)
    GG_CUDA(cudaMemcpyAsync(w_out, plan->in_vis.p, n * sizeof(Real),
                            cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaMemcpyAsync(&skip_out, d_skip, 8, cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  *num_skipped = (size_t)skip_out;
  return GG_OK;
}

// ---- degridding with host pointers ------------------------------------------
template <typename Real>
int degrid_host(size_t num_w_planes, const int* support, int oversample,
                int conv_size_half, const Real* conv_func, size_t num_points,
                const Real* uu, const Real* vv, const Real* ww,
                Real cell_size_rad, Real w_scale, int grid_size,
                const Real* grid, Real* vis) {
  if (!grid || (num_points > 0 && !vis))
    return set_error(GG_ERR_INVALID_ARG, "grid or vis is NULL");
  if (grid_size < 1 || grid_size > kMaxGridSize)
    return set_error(GG_ERR_UNSUPPORTED, "grid_size = %d outside [1, %d]",
                     grid_size, kMaxGridSize);
  if (num_points > 0 && (!uu || !vv || !ww))
    return set_error(GG_ERR_INVALID_ARG, "an input array is NULL");
  GG_TRY(validate_stack(num_w_planes, support, oversample, conv_size_half,
                        conv_func));
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  std::lock_guard<std::mutex> lk(st->mu);
  cudaStream_t s = st->stream;
  GG_TRY(ensure_device_plan(st));
  gg_plan* plan = st->plan;
  const size_t n = num_points;
  const size_t grid_bytes = (size_t)grid_size * grid_size * 2 * sizeof(Real);
  GG_TRY(plan->in_uu.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_vv.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_ww.ensure(n * sizeof(Real) + 16));
  GG_TRY(plan->in_vis.ensure(2 * n * sizeof(Real) + 16));
  GG_TRY(plan->in_grid.ensure(grid_bytes));
  // As in the gridding call: the coordinates go up first on the side
  // stream, the kernel stack is built beside placement on the stack stream
  // behind them, and the grid follows the coordinates on the side stream;
  // only the degridding kernel waits for the stack and the grid.
  GG_TRY(ensure_copy_stream(st));
  struct CopyGuard {   // the side streams read the caller's arrays
    cudaStream_t s, t;
    ~CopyGuard() {
      cudaStreamSynchronize(s);
      cudaStreamSynchronize(t);
    }
  } copy_guard{st->copy_stream, st->stack_stream};
  cudaStream_t cs = st->copy_stream;
  auto uploads = [&]() -> int {
    if (n) {
      GG_CUDA(cudaMemcpyAsync(plan->in_uu.p, uu, n * sizeof(Real),
                              cudaMemcpyHostToDevice, cs));
      GG_CUDA(cudaMemcpyAsync(plan->in_vv.p, vv, n * sizeof(Real),
                              cudaMemcpyHostToDevice, cs));
      GG_CUDA(cudaMemcpyAsync(plan->in_ww.p, ww, n * sizeof(Real),
                              cudaMemcpyHostToDevice, cs));
    }
    GG_CUDA(cudaEventRecord(st->vis_ready, cs));
    return GG_OK;
  };
  gg_kernels* K = nullptr;
  GG_TRY(host_kernels<Real>(st, num_w_planes, support, oversample,
                            conv_size_half, conv_func, s, uploads, &K));
  // A grid the device addresses is read in place by the degridding kernel
  // (each work item loads its tile once); others go up behind the cube.
  const void* direct =
      n ? direct_host_address(st, dev, grid, grid_bytes, 2 * sizeof(Real))
        : nullptr;
  if (n && !direct) {
    GG_CUDA(cudaStreamWaitEvent(cs, st->cube_staged, 0));
    GG_CUDA(cudaMemcpyAsync(plan->in_grid.p, grid, grid_bytes,
                            cudaMemcpyHostToDevice, cs));
  }
  GG_CUDA(cudaEventRecord(st->grid_ready, cs));
  GG_CUDA(cudaStreamWaitEvent(s, st->vis_ready, 0));
  plan->grid_wait = direct ? nullptr : st->grid_ready;
  plan->stack_wait = st->stack_ready;
  const int rc = degrid_pipeline<Real>(
      plan, K, n, plan->in_uu.as<Real>(), plan->in_vv.as<Real>(),
      plan->in_ww.as<Real>(), cell_size_rad, w_scale, grid_size,
      direct ? (const Real*)direct : plan->in_grid.as<Real>(),
      plan->in_vis.as<Real>(), s);
  plan->grid_wait = nullptr;
  plan->stack_wait = nullptr;
  GG_TRY(rc);
  if (n)
    GG_CUDA(cudaMemcpyAsync(vis, plan->in_vis.p, 2 * n * sizeof(Real),
                            cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  GG_CUDA(cudaStreamSynchronize(cs));
  GG_CUDA(cudaStreamSynchronize(st->stack_stream));
  return check_device_error(plan, s);
}

template <typename Real>
int place_only(const gg_kernels* K, size_t num_points, const Real* uu,
               const Real* vv, const Real* ww, Real cell_size_rad,
               Real w_scale, int grid_size, int* d_out, cudaStream_t s) {
  if (!K) return set_error(GG_ERR_INVALID_ARG, "kernels is NULL");
  if (K->is_double != (sizeof(Real) == 8))
    return set_error(GG_ERR_INVALID_ARG,
                     "kernel stack precision does not match the call");
  if (num_points > 0 && (!uu || !vv || !ww || !d_out))
    return set_error(GG_ERR_INVALID_ARG, "an array is NULL");
  PlaceParams<Real> pp;
  pp.uu = uu; pp.vv = vv; pp.ww = ww; pp.vis = nullptr; pp.weight = nullptr;
  pp.grid_scale = (Real)grid_size * cell_size_rad;
  pp.w_scale = w_scale;
  pp.grid_size = grid_size;
  pp.grid_centre = grid_size / 2;
  pp.num_points = num_points;
  GG_CUDA(launch_place_only<Real>(pp, K->view(), d_out, s));
  return GG_OK;
}

}  // namespace

// ===========================================================================
// Accessors for other translation units of the library (gg_internal.h).
// ===========================================================================
namespace gg {

int record_error(int code, const char* message) {
  return set_error(code, "%s", message);
}

bool kernels_info(const gg_kernels* k, StackView* view, int* device,
                  bool* is_double, int* num_planes) {
  if (!k) return false;
  *view = k->view();
  *device = k->device;
  *is_double = k->is_double;
  *num_planes = k->num_planes;
  return true;
}

}  // namespace gg

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

GG_API const char* gg_last_error(void) { return t_last_error.c_str(); }

GG_API const char* gg_version(void) { return "gpugrid-gb300 0.1.0"; }

GG_API int gg_grid_wproj_f(size_t num_w_planes, const int* support,
                           int oversample, int conv_size_half,
                           const float* conv_func, size_t num_points,
                           const float* uu, const float* vv, const float* ww,
                           const float* vis, const float* weight,
                           float cell_size_rad, float w_scale, int grid_size,
                           size_t* num_skipped, double* norm, float* grid) {
  t_last_error.clear();
  return dropin<float>(num_w_planes, support, oversample, conv_size_half,
                       conv_func, num_points, uu, vv, ww, vis, weight,
                       cell_size_rad, w_scale, grid_size, num_skipped, norm,
                       grid);
}

GG_API int gg_grid_wproj_d(size_t num_w_planes, const int* support,
                           int oversample, int conv_size_half,
                           const double* conv_func, size_t num_points,
                           const double* uu, const double* vv,
                           const double* ww, const double* vis,
                           const double* weight, double cell_size_rad,
                           double w_scale, int grid_size, size_t* num_skipped,
                           double* norm, double* grid) {
  t_last_error.clear();
  return dropin<double>(num_w_planes, support, oversample, conv_size_half,
                        conv_func, num_points, uu, vv, ww, vis, weight,
                        cell_size_rad, w_scale, grid_size, num_skipped, norm,
                        grid);
}

GG_API void oskar_grid_wproj_f(const size_t num_w_planes, const int* support,
                               const int oversample, const int conv_size_half,
                               const float* conv_func, const size_t num_points,
                               const float* uu, const float* vv,
                               const float* ww, const float* vis,
                               const float* weight, const float cell_size_rad,
                               const float w_scale, const int grid_size,
                               size_t* num_skipped, double* norm,
                               float* grid) {
  if (gg_grid_wproj_f(num_w_planes, support, oversample, conv_size_half,
                      conv_func, num_points, uu, vv, ww, vis, weight,
                      cell_size_rad, w_scale, grid_size, num_skipped, norm,
                      grid) != GG_OK)
    fprintf(stderr, "oskar_grid_wproj_f (gpugrid): %s\n", gg_last_error());
}

GG_API void oskar_grid_wproj_d(const size_t num_w_planes, const int* support,
                               const int oversample, const int conv_size_half,
                               const double* conv_func,
                               const size_t num_points, const double* uu,
                               const double* vv, const double* ww,
                               const double* vis, const double* weight,
                               const double cell_size_rad,
                               const double w_scale, const int grid_size,
                               size_t* num_skipped, double* norm,
                               double* grid) {
  if (gg_grid_wproj_d(num_w_planes, support, oversample, conv_size_half,
                      conv_func, num_points, uu, vv, ww, vis, weight,
                      cell_size_rad, w_scale, grid_size, num_skipped, norm,
                      grid) != GG_OK)
    fprintf(stderr, "oskar_grid_wproj_d (gpugrid): %s\n", gg_last_error());
}

GG_API int gg_kernels_create_f(gg_kernels** out, size_t num_w_planes,
                               const int* support, int oversample,
                               int conv_size_half, const float* conv_func,
                               int conv_func_on_device, void* stream) {
  t_last_error.clear();
  return kernels_create<float>(out, num_w_planes, support, oversample,
                               conv_size_half, conv_func, conv_func_on_device,
                               (cudaStream_t)stream);
}

GG_API int gg_kernels_create_d(gg_kernels** out, size_t num_w_planes,
                               const int* support, int oversample,
                               int conv_size_half, const double* conv_func,
                               int conv_func_on_device, void* stream) {
  t_last_error.clear();
  return kernels_create<double>(out, num_w_planes, support, oversample,
                                conv_size_half, conv_func,
                                conv_func_on_device, (cudaStream_t)stream);
}

GG_API int gg_kernels_generate_f(gg_kernels** out, size_t num_w_planes,
                                 const int* support, int oversample,
                                 int conv_size_half, const double* w_planes,
                                 float* d_conv_func_out, void* stream) {
  t_last_error.clear();
  return kernels_generate<float>(out, num_w_planes, support, oversample,
                                 conv_size_half, w_planes, d_conv_func_out,
                                 (cudaStream_t)stream);
}

GG_API int gg_kernels_generate_d(gg_kernels** out, size_t num_w_planes,
                                 const int* support, int oversample,
                                 int conv_size_half, const double* w_planes,
                                 double* d_conv_func_out, void* stream) {
  t_last_error.clear();
  return kernels_generate<double>(out, num_w_planes, support, oversample,
                                  conv_size_half, w_planes, d_conv_func_out,
                                  (cudaStream_t)stream);
}

GG_API int gg_kernels_destroy(gg_kernels* k) {
  delete k;
  return GG_OK;
}

GG_API int gg_plan_create(gg_plan** out) {
  t_last_error.clear();
  if (!out) return set_error(GG_ERR_INVALID_ARG, "out is NULL");
  gg_plan* p = new gg_plan();
  int r = plan_init(p);
  if (r != GG_OK) {
    delete p;
    *out = nullptr;
    return r;
  }
  *out = p;
  return GG_OK;
}

GG_API int gg_plan_destroy(gg_plan* plan) {
  delete plan;
  return GG_OK;
}

GG_API int gg_plan_set_batch_limit(gg_plan* plan,
                                   unsigned long long max_points) {
  t_last_error.clear();
  if (!plan) return set_error(GG_ERR_INVALID_ARG, "plan is NULL");
  plan->batch_limit = max_points;
  return GG_OK;
}

GG_API int gg_plan_last_stats(const gg_plan* plan, gg_stats* stats) {
  if (!plan || !stats) return set_error(GG_ERR_INVALID_ARG, "NULL argument");
  *stats = plan->stats;
  return GG_OK;
}

GG_API int gg_plan_set_tile_shape(gg_plan* plan, int tile_u) {
  t_last_error.clear();
  if (!plan) return set_error(GG_ERR_INVALID_ARG, "plan is NULL");
  if (tile_u == 0) {
    plan->forced_shape = -1;
    return GG_OK;
  }
  for (int sh = 0; sh < kNumTileShapes; ++sh)
    if (tile_u_of_shape(sh) == tile_u) {
      plan->forced_shape = sh;
      return GG_OK;
    }
  return set_error(GG_ERR_INVALID_ARG,
                   "tile_u = %d: supported tile widths are 32, 16, 8 (0 = "
                   "automatic)", tile_u);
}

GG_API int gg_plan_set_slice_staging(gg_plan* plan, int mode) {
  t_last_error.clear();
  if (!plan) return set_error(GG_ERR_INVALID_ARG, "plan is NULL");
  if (mode < -1 || mode > 1)
    return set_error(GG_ERR_INVALID_ARG,
                     "mode = %d: -1 (automatic), 0 (off) or 1 (on)", mode);
  plan->forced_stage = mode;
  return GG_OK;
}

GG_API int gg_plan_set_tuning(gg_plan* plan, const gg_tuning* t) {
  t_last_error.clear();
  if (!plan || !t) return set_error(GG_ERR_INVALID_ARG, "plan or tuning is NULL");
  if (t->items_per_cta < 1 || t->items_per_cta > 64)
    return set_error(GG_ERR_INVALID_ARG, "items_per_cta = %d outside [1, 64]",
                     t->items_per_cta);
  if (t->sort_detail < 0 || t->sort_detail > 2)
    return set_error(GG_ERR_INVALID_ARG, "sort_detail = %d: 0, 1 or 2",
                     t->sort_detail);
  if (t->ctas_per_sm < 0 || t->ctas_per_sm > 32)
    return set_error(GG_ERR_INVALID_ARG, "ctas_per_sm = %d outside [0, 32]",
                     t->ctas_per_sm);
  if (t->plane_group_mb < 0 || t->plane_group_mb > (1 << 20))
    return set_error(GG_ERR_INVALID_ARG,
                     "plane_group_mb = %d outside [0, 1048576]",
                     t->plane_group_mb);
  if (t->tile_order < 0 || t->tile_order > 1)
    return set_error(GG_ERR_INVALID_ARG, "tile_order = %d: 0 or 1",
                     t->tile_order);
  if (t->lane_groups < 0 || t->lane_groups > 2)
    return set_error(GG_ERR_INVALID_ARG, "lane_groups = %d: 0, 1 or 2",
                     t->lane_groups);
  if (t->tile_phases != 0 && t->tile_phases != 1 && t->tile_phases != 2 &&
      t->tile_phases != 4 && t->tile_phases != 8)
    return set_error(GG_ERR_INVALID_ARG, "tile_phases = %d: 0, 1, 2, 4 or 8",
                     t->tile_phases);
  const int old_shape = plan->forced_shape;
  GG_TRY(gg_plan_set_tile_shape(plan, t->tile_u));
  const int r = gg_plan_set_slice_staging(plan, t->slice_staging);
  if (r != GG_OK) {
    plan->forced_shape = old_shape;
    return r;
  }
  plan->items_per_cta = t->items_per_cta;
  plan->sort_detail = t->sort_detail;
  plan->ctas_per_sm = t->ctas_per_sm;
  plan->plane_group_mb = t->plane_group_mb;
  plan->queue_order = t->tile_order;
  plan->lane_groups = t->lane_groups;
  plan->tile_phases = t->tile_phases;
  return GG_OK;
}

GG_API int gg_plan_get_tuning(const gg_plan* plan, gg_tuning* t) {
  t_last_error.clear();
  if (!plan || !t) return set_error(GG_ERR_INVALID_ARG, "plan or tuning is NULL");
  t->tile_u = plan->forced_shape < 0 ? 0 : tile_u_of_shape(plan->forced_shape);
  t->slice_staging = plan->forced_stage;
  t->items_per_cta = plan->items_per_cta;
  t->sort_detail = plan->sort_detail;
  t->ctas_per_sm = plan->ctas_per_sm;
  t->plane_group_mb = plan->plane_group_mb;
  t->tile_order = plan->queue_order;
  t->lane_groups = plan->lane_groups;
  t->tile_phases = plan->tile_phases;
  return GG_OK;
}

GG_API int gg_host_set_tuning(const gg_tuning* t) {
  t_last_error.clear();
  const gg_tuning defaults{0, -1, 4, 2, 0, 0, 0, 0, 0};
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  std::lock_guard<std::mutex> lk(st->mu);
  GG_TRY(ensure_device_plan(st));
  return gg_plan_set_tuning(st->plan, t ? t : &defaults);
}

GG_API int gg_host_set_grid_access(int mode) {
  t_last_error.clear();
  if (mode < GG_GRID_ACCESS_COPY || mode > GG_GRID_ACCESS_PAGEABLE)
    return set_error(GG_ERR_INVALID_ARG, "grid access mode %d unknown", mode);
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  std::lock_guard<std::mutex> lk(st->mu);
  st->grid_access = mode;
  return GG_OK;
}

GG_API int gg_host_set_profiling(int enable) {
  t_last_error.clear();
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  std::lock_guard<std::mutex> lk(st->mu);
  GG_TRY(ensure_device_plan(st));
  if (enable && !st->call_start)
    for (cudaEvent_t* e : {&st->call_start, &st->call_end, &st->copies_done})
      GG_CUDA(cudaEventCreate(e));
  st->profile = enable != 0;
  st->profile_valid = false;
  return gg_plan_set_profiling(st->plan, enable);
}

GG_API int gg_host_phase_ms(float* ms, int n) {
  t_last_error.clear();
  if (!ms || n < 0) return set_error(GG_ERR_INVALID_ARG, "NULL argument");
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  std::lock_guard<std::mutex> lk(st->mu);
  if (!st->profile_valid)
    return set_error(GG_ERR_INVALID_ARG,
                     "no profiled call: enable profiling and make a "
                     "host-pointer gridding call that grids at least one "
                     "visibility");
  const gg_plan* p = st->plan;
  // staging, the plan's phases 0..3, then the rest of the call.
  cudaEvent_t marks[7] = {st->call_start, p->ev[0], p->ev[1], p->ev[2],
                          p->ev[3], p->ev[4], st->call_end};
  for (int i = 0; i < n && i < 6; ++i)
    GG_CUDA(cudaEventElapsedTime(&ms[i], marks[i], marks[i + 1]));
  for (int i = 6; i < n && i < 9; ++i) ms[i] = (float)st->host_ms[i - 6];
  return GG_OK;
}

GG_API int gg_host_get_grid_access(int* mode) {
  t_last_error.clear();
  if (!mode) return set_error(GG_ERR_INVALID_ARG, "mode is NULL");
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  std::lock_guard<std::mutex> lk(st->mu);
  *mode = st->grid_access;
  return GG_OK;
}

GG_API int gg_host_last_transfer(unsigned long long* h2d_bytes,
                                 unsigned long long* d2h_bytes) {
  t_last_error.clear();
  if (!h2d_bytes || !d2h_bytes)
    return set_error(GG_ERR_INVALID_ARG, "NULL argument");
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  std::lock_guard<std::mutex> lk(st->mu);
  *h2d_bytes = st->last_h2d;
  *d2h_bytes = st->last_d2h;
  return GG_OK;
}

GG_API int gg_host_last_call_ms(double* ms, int n) {
  t_last_error.clear();
  if (!ms || n < 0) return set_error(GG_ERR_INVALID_ARG, "NULL argument");
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  std::lock_guard<std::mutex> lk(st->mu);
  for (int i = 0; i < n && i < 3; ++i) ms[i] = st->host_ms[i];
  return GG_OK;
}

GG_API int gg_host_get_tuning(gg_tuning* t) {
  t_last_error.clear();
  if (!t) return set_error(GG_ERR_INVALID_ARG, "tuning is NULL");
  int dev;
  GG_TRY(current_device(&dev));
  DeviceState* st;
  GG_TRY(device_state(dev, &st));
  std::lock_guard<std::mutex> lk(st->mu);
  GG_TRY(ensure_device_plan(st));
  return gg_plan_get_tuning(st->plan, t);
}

GG_API int gg_plan_set_profiling(gg_plan* plan, int enable) {
  t_last_error.clear();
  if (!plan) return set_error(GG_ERR_INVALID_ARG, "plan is NULL");
  if (enable && !plan->ev[0]) {
    for (auto& e : plan->ev) GG_CUDA(cudaEventCreate(&e));
  }
  plan->profile = enable != 0;
  plan->events_valid = false;
  return GG_OK;
}

GG_API int gg_plan_phase_ms(const gg_plan* plan, float* ms, int n) {
  t_last_error.clear();
  if (!plan || !ms || n < 0)
    return set_error(GG_ERR_INVALID_ARG, "NULL argument");
  if (!plan->events_valid)
    return set_error(GG_ERR_INVALID_ARG,
                     "no profiled call: enable profiling and make a call "
                     "that grids at least one visibility");
  for (int i = 0; i < n && i < gg_plan::kEvents - 1; ++i)
    GG_CUDA(cudaEventElapsedTime(&ms[i], plan->ev[i], plan->ev[i + 1]));
  return GG_OK;
}

GG_API int gg_measure_fp32_fma_tflops(double* tflops) {
  t_last_error.clear();
  if (!tflops) return set_error(GG_ERR_INVALID_ARG, "tflops is NULL");
  int sms = 0;
  GG_TRY(num_sms_of_current(&sms));
  GG_CUDA(gg::measure_fp32_fma(sms, tflops, nullptr));
  return GG_OK;
}

GG_API int gg_grid_wproj_f_device(gg_plan* plan, const gg_kernels* kernels,
                                  size_t num_points, const float* d_uu,
                                  const float* d_vv, const float* d_ww,
                                  const float* d_vis, const float* d_weight,
                                  float cell_size_rad, float w_scale,
                                  int grid_size,
                                  unsigned long long* d_num_skipped,
                                  double* d_norm, float* d_grid,
                                  void* stream) {
  t_last_error.clear();
  return grid_pipeline<float>(plan, kernels, num_points, d_uu, d_vv, d_ww,
                              d_vis, d_weight, cell_size_rad, w_scale,
                              grid_size, d_num_skipped, d_norm, d_grid,
                              (cudaStream_t)stream);
}

GG_API int gg_grid_wproj_d_device(gg_plan* plan, const gg_kernels* kernels,
                                  size_t num_points, const double* d_uu,
                                  const double* d_vv, const double* d_ww,
                                  const double* d_vis, const double* d_weight,
                                  double cell_size_rad, double w_scale,
                                  int grid_size,
                                  unsigned long long* d_num_skipped,
                                  double* d_norm, double* d_grid,
                                  void* stream) {
  t_last_error.clear();
  return grid_pipeline<double>(plan, kernels, num_points, d_uu, d_vv, d_ww,
                               d_vis, d_weight, cell_size_rad, w_scale,
                               grid_size, d_num_skipped, d_norm, d_grid,
                               (cudaStream_t)stream);
}

GG_API int gg_grid_wproj_f_batched_device(
    gg_plan* plan, const gg_kernels* kernels, int num_grids,
    const unsigned long long* offsets, const float* d_uu, const float* d_vv,
    const float* d_ww, const float* d_vis, const float* d_weight,
    float cell_size_rad, float w_scale, int grid_size,
    unsigned long long* d_num_skipped, double* d_norm, float* d_grids,
    void* stream) {
  t_last_error.clear();
  return batched_split<float>(plan, kernels, num_grids, offsets, d_uu, d_vv,
                              d_ww, d_vis, d_weight, cell_size_rad, w_scale,
                              grid_size, d_num_skipped, d_norm, d_grids,
                              (cudaStream_t)stream);
}

GG_API int gg_grid_wproj_d_batched_device(
    gg_plan* plan, const gg_kernels* kernels, int num_grids,
    const unsigned long long* offsets, const double* d_uu,
    const double* d_vv, const double* d_ww, const double* d_vis,
    const double* d_weight, double cell_size_rad, double w_scale,
    int grid_size, unsigned long long* d_num_skipped, double* d_norm,
    double* d_grids, void* stream) {
  t_last_error.clear();
  return batched_split<double>(plan, kernels, num_grids, offsets, d_uu,
                               d_vv, d_ww, d_vis, d_weight, cell_size_rad,
                               w_scale, grid_size, d_num_skipped, d_norm,
                               d_grids, (cudaStream_t)stream);
}

GG_API int gg_grid_wproj_f_batched_replay(gg_plan* plan,
                                          const gg_kernels* kernels,
                                          const float* d_vis,
                                          const float* d_weight,
                                          unsigned long long* d_num_skipped,
                                          double* d_norm, float* d_grids,
                                          void* stream) {
  t_last_error.clear();
  return replay_pipeline<float>(plan, kernels, d_vis, d_weight,
                                d_num_skipped, d_norm, d_grids,
                                (cudaStream_t)stream);
}

GG_API int gg_grid_wproj_d_batched_replay(gg_plan* plan,
                                          const gg_kernels* kernels,
                                          const double* d_vis,
                                          const double* d_weight,
                                          unsigned long long* d_num_skipped,
                                          double* d_norm, double* d_grids,
                                          void* stream) {
  t_last_error.clear();
  return replay_pipeline<double>(plan, kernels, d_vis, d_weight,
                                 d_num_skipped, d_norm, d_grids,
                                 (cudaStream_t)stream);
}

GG_API int gg_grid_weights_write_f_device(gg_plan* plan, size_t num_points,
                                          const float* d_uu, const float* d_vv,
                                          const float* d_weight,
                                          float cell_size_rad, int grid_size,
                                          unsigned long long* d_num_skipped,
                                          float* d_grid, void* stream) {
  t_last_error.clear();
  return weights_write_pipeline<float>(plan, num_points, d_uu, d_vv, d_weight,
                                       cell_size_rad, grid_size, d_num_skipped,
                                       d_grid, (cudaStream_t)stream);
}

GG_API int gg_grid_weights_write_d_device(gg_plan* plan, size_t num_points,
                                          const double* d_uu,
                                          const double* d_vv,
                                          const double* d_weight,
                                          double cell_size_rad, int grid_size,
                                          unsigned long long* d_num_skipped,
                                          double* d_grid, void* stream) {
  t_last_error.clear();
  return weights_write_pipeline<double>(plan, num_points, d_uu, d_vv,
                                        d_weight, cell_size_rad, grid_size,
                                        d_num_skipped, d_grid,
                                        (cudaStream_t)stream);
}

GG_API int gg_grid_weights_read_f_device(gg_plan* plan, size_t num_points,
                                         const float* d_uu, const float* d_vv,
                                         const float* d_weight_in,
                                         float* d_weight_out,
                                         float cell_size_rad, int grid_size,
                                         unsigned long long* d_num_skipped,
                                         const float* d_grid, void* stream) {
  t_last_error.clear();
  return weights_read_pipeline<float>(plan, num_points, d_uu, d_vv,
                                      d_weight_in, d_weight_out, cell_size_rad,
                                      grid_size, d_num_skipped, d_grid,
                                      (cudaStream_t)stream);
}

GG_API int gg_grid_weights_read_d_device(gg_plan* plan, size_t num_points,
                                         const double* d_uu,
                                         const double* d_vv,
                                         const double* d_weight_in,
                                         double* d_weight_out,
                                         double cell_size_rad, int grid_size,
                                         unsigned long long* d_num_skipped,
                                         const double* d_grid, void* stream) {
  t_last_error.clear();
  return weights_read_pipeline<double>(plan, num_points, d_uu, d_vv,
                                       d_weight_in, d_weight_out,
                                       cell_size_rad, grid_size,
                                       d_num_skipped, d_grid,
                                       (cudaStream_t)stream);
}

GG_API int gg_grid_weights_write_f(size_t num_points, const float* uu,
                                   const float* vv, const float* weight,
                                   float cell_size_rad, int grid_size,
                                   size_t* num_skipped, float* grid) {
  t_last_error.clear();
  return weights_write_host<float>(num_points, uu, vv, weight, cell_size_rad,
                                   grid_size, num_skipped, grid);
}

GG_API int gg_grid_weights_write_d(size_t num_points, const double* uu,
                                   const double* vv, const double* weight,
                                   double cell_size_rad, int grid_size,
                                   size_t* num_skipped, double* grid) {
  t_last_error.clear();
  return weights_write_host<double>(num_points, uu, vv, weight,
                                    cell_size_rad, grid_size, num_skipped,
                                    grid);
}

GG_API int gg_grid_weights_read_f(size_t num_points, const float* uu,
                                  const float* vv, const float* weight_in,
                                  float* weight_out, float cell_size_rad,
                                  int grid_size, size_t* num_skipped,
                                  const float* grid) {
  t_last_error.clear();
  return weights_read_host<float>(num_points, uu, vv, weight_in, weight_out,
                                  cell_size_rad, grid_size, num_skipped,
                                  grid);
}

GG_API int gg_grid_weights_read_d(size_t num_points, const double* uu,
                                  const double* vv, const double* weight_in,
                                  double* weight_out, double cell_size_rad,
                                  int grid_size, size_t* num_skipped,
                                  const double* grid) {
  t_last_error.clear();
  return weights_read_host<double>(num_points, uu, vv, weight_in, weight_out,
                                   cell_size_rad, grid_size, num_skipped,
                                   grid);
}

GG_API void oskar_grid_weights_write_f(const size_t num_points,
                                       const float* uu, const float* vv,
                                       const float* weight,
                                       const float cell_size_rad,
                                       const int grid_size,
                                       size_t* num_skipped, float* grid) {
  if (gg_grid_weights_write_f(num_points, uu, vv, weight, cell_size_rad,
                              grid_size, num_skipped, grid) != GG_OK)
    fprintf(stderr, "oskar_grid_weights_write_f (gpugrid): %s\n",
            gg_last_error());
}

GG_API void oskar_grid_weights_write_d(const size_t num_points,
                                       const double* uu, const double* vv,
                                       const double* weight,
                                       const double cell_size_rad,
                                       const int grid_size,
                                       size_t* num_skipped, double* grid) {
  if (gg_grid_weights_write_d(num_points, uu, vv, weight, cell_size_rad,
                              grid_size, num_skipped, grid) != GG_OK)
    fprintf(stderr, "oskar_grid_weights_write_d (gpugrid): %s\n",
            gg_last_error());
}

GG_API void oskar_grid_weights_read_f(const size_t num_points,
                                      const float* uu, const float* vv,
                                      const float* weight_in,
                                      float* weight_out,
                                      const float cell_size_rad,
                                      const int grid_size,
                                      size_t* num_skipped, const float* grid) {
  if (gg_grid_weights_read_f(num_points, uu, vv, weight_in, weight_out,
                             cell_size_rad, grid_size, num_skipped,
                             grid) != GG_OK)
    fprintf(stderr, "oskar_grid_weights_read_f (gpugrid): %s\n",
            gg_last_error());
}

GG_API void oskar_grid_weights_read_d(const size_t num_points,
                                      const double* uu, const double* vv,
                                      const double* weight_in,
                                      double* weight_out,
                                      const double cell_size_rad,
                                      const int grid_size,
                                      size_t* num_skipped,
                                      const double* grid) {
  if (gg_grid_weights_read_d(num_points, uu, vv, weight_in, weight_out,
                             cell_size_rad, grid_size, num_skipped,
                             grid) != GG_OK)
    fprintf(stderr, "oskar_grid_weights_read_d (gpugrid): %s\n",
            gg_last_error());
}

GG_API int gg_degrid_wproj_f(size_t num_w_planes, const int* support,
                             int oversample, int conv_size_half,
                             const float* conv_func, size_t num_points,
                             const float* uu, const float* vv,
                             const float* ww, float cell_size_rad,
                             float w_scale, int grid_size, const float* grid,
                             float* vis) {
  t_last_error.clear();
  return degrid_host<float>(num_w_planes, support, oversample,
                            conv_size_half, conv_func, num_points, uu, vv, ww,
                            cell_size_rad, w_scale, grid_size, grid, vis);
}

GG_API int gg_degrid_wproj_d(size_t num_w_planes, const int* support,
                             int oversample, int conv_size_half,
                             const double* conv_func, size_t num_points,
                             const double* uu, const double* vv,
                             const double* ww, double cell_size_rad,
                             double w_scale, int grid_size,
                             const double* grid, double* vis) {
  t_last_error.clear();
  return degrid_host<double>(num_w_planes, support, oversample,
                             conv_size_half, conv_func, num_points, uu, vv,
                             ww, cell_size_rad, w_scale, grid_size, grid,
                             vis);
}

GG_API void oskar_degrid_wproj_f(const size_t num_w_planes,
                                 const int* support, const int oversample,
                                 const int conv_size_half,
                                 const float* conv_func,
                                 const size_t num_points, const float* uu,
                                 const float* vv, const float* ww,
                                 const float cell_size_rad,
                                 const float w_scale, const int grid_size,
                                 const float* grid, float* vis) {
  if (gg_degrid_wproj_f(num_w_planes, support, oversample, conv_size_half,
                        conv_func, num_points, uu, vv, ww, cell_size_rad,
                        w_scale, grid_size, grid, vis) != GG_OK)
    fprintf(stderr, "oskar_degrid_wproj_f (gpugrid): %s\n",
            gg_last_error());
}

GG_API void oskar_degrid_wproj_d(const size_t num_w_planes,
                                 const int* support, const int oversample,
                                 const int conv_size_half,
                                 const double* conv_func,
                                 const size_t num_points, const double* uu,
                                 const double* vv, const double* ww,
                                 const double cell_size_rad,
                                 const double w_scale, const int grid_size,
                                 const double* grid, double* vis) {
  if (gg_degrid_wproj_d(num_w_planes, support, oversample, conv_size_half,
                        conv_func, num_points, uu, vv, ww, cell_size_rad,
                        w_scale, grid_size, grid, vis) != GG_OK)
    fprintf(stderr, "oskar_degrid_wproj_d (gpugrid): %s\n",
            gg_last_error());
}

GG_API int gg_plan_probe_bounded_wait(gg_plan* plan, unsigned iterations,
                                      void* stream) {
  t_last_error.clear();
  if (!plan) return set_error(GG_ERR_INVALID_ARG, "plan is NULL");
  if (iterations < 1 || iterations > (1u << 20))
    return set_error(GG_ERR_INVALID_ARG,
                     "iterations = %u outside [1, 1048576]", iterations);
  int dev;
  GG_TRY(current_device(&dev));
  if (dev != plan->device)
    return set_error(GG_ERR_INVALID_ARG, "plan and current device differ");
  cudaStream_t s = (cudaStream_t)stream;
  GG_CUDA(launch_wait_probe(iterations,
                            plan->scalars.as<uint32_t>() + kDeviceError, s));
  return check_device_error(plan, s);
}

GG_API int gg_plan_check(gg_plan* plan, void* stream) {
  t_last_error.clear();
  if (!plan) return set_error(GG_ERR_INVALID_ARG, "plan is NULL");
  return check_device_error(plan, (cudaStream_t)stream);
}

GG_API int gg_place_wproj_f_device(const gg_kernels* kernels,
                                   size_t num_points, const float* d_uu,
                                   const float* d_vv, const float* d_ww,
                                   float cell_size_rad, float w_scale,
                                   int grid_size, int* d_out, void* stream) {
  t_last_error.clear();
  return place_only<float>(kernels, num_points, d_uu, d_vv, d_ww,
                           cell_size_rad, w_scale, grid_size, d_out,
                           (cudaStream_t)stream);
}

GG_API int gg_place_wproj_d_device(const gg_kernels* kernels,
                                   size_t num_points, const double* d_uu,
                                   const double* d_vv, const double* d_ww,
                                   double cell_size_rad, double w_scale,
                                   int grid_size, int* d_out, void* stream) {
  t_last_error.clear();
  return place_only<double>(kernels, num_points, d_uu, d_vv, d_ww,
                            cell_size_rad, w_scale, grid_size, d_out,
                            (cudaStream_t)stream);
}

GG_API int gg_degrid_wproj_f_device(gg_plan* plan, const gg_kernels* kernels,
                                    size_t num_points, const float* d_uu,
                                    const float* d_vv, const float* d_ww,
                                    float cell_size_rad, float w_scale,
                                    int grid_size, const float* d_grid,
                                    float* d_out_vis, void* stream) {
  t_last_error.clear();
  return degrid_pipeline<float>(plan, kernels, num_points, d_uu, d_vv, d_ww,
                                cell_size_rad, w_scale, grid_size, d_grid,
                                d_out_vis, (cudaStream_t)stream);
}

GG_API int gg_degrid_wproj_d_device(gg_plan* plan, const gg_kernels* kernels,
                                    size_t num_points, const double* d_uu,
                                    const double* d_vv, const double* d_ww,
                                    double cell_size_rad, double w_scale,
                                    int grid_size, const double* d_grid,
                                    double* d_out_vis, void* stream) {
  t_last_error.clear();
  return degrid_pipeline<double>(plan, kernels, num_points, d_uu, d_vv, d_ww,
                                 cell_size_rad, w_scale, grid_size, d_grid,
                                 d_out_vis, (cudaStream_t)stream);
}

}  // extern "C"
