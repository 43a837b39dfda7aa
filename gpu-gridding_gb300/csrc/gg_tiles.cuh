// Pieces shared by the tile-owning kernels (gridding in gg_grid.cu,
// degridding in gg_degrid.cu): the CTA shape (one producer warp, eight
// consumer warps owning a 2048-cell tile, lane = column, kRows rows per
// lane), the record ring, bounded mbarrier waits, tap loads with an L2
// keep hint, and the slab-stack descriptor of a record.
#pragma once

#include "gg_internal.h"

namespace gg {

namespace {

constexpr int kRows = 8;          // rows per lane (registers)
constexpr int kWarps = 8;         // consumer warps per CTA
constexpr int kConsumers = kWarps * 32;
constexpr int kThreads = kConsumers + 32;  // + one producer warp
constexpr int kCells = kConsumers * kRows; // 2048 cells per tile
constexpr int kRing = 4;          // record buffers in flight
constexpr int kBuf = 128;         // records per buffer
constexpr int kPerLane = kBuf / 32;
static_assert(kRows - 1 <= kSlicePad, "slices need kRows-1 padding rows");
// Bound on every mbarrier wait (each failed probe sleeps ~100 ns): a wait
// that runs out (> ~1 s) sets the error flag and the CTA returns.
constexpr unsigned kWaitLimit = 1u << 24;

template <int TW>
struct WarpShape {
  static constexpr int kLanesY = 32 / TW;          // lane rows per warp
  static constexpr int kBand = kLanesY * kRows;    // rows per warp band
  static constexpr int kTileU = TW;
  static constexpr int kTileV = kWarps * kBand;
};

// ---- mbarrier and bulk-copy helpers (shared::cta) --------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}
// Release-arrive: the caller's earlier shared-memory writes are visible to
// a thread whose wait observes the phase completion.
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
      : "memory");
}
// Adds `bytes` of expected asynchronous transactions to the current phase.
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Acquire-wait for the completion of the phase with the given parity;
// false when `limit` probes have failed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          unsigned limit = kWaitLimit) {
  for (unsigned i = 0; i < limit; ++i) {
    if (mbar_test(bar, parity)) return true;
    if (i >= 32) __nanosleep(64);
  }
  return false;
}
// Bulk copy global -> shared (16-byte aligned, size a multiple of 16),
// completing `bytes` transactions on `bar`.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src,
                                              uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Read-only tap load that asks L2 to keep the line (evict_last policy):
// the compact stack is re-read by every tile while the grid streams past.
__device__ __forceinline__ float2 ld_tap(const float2* p, uint64_t pol) {
  float2 v;
  asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
      : "=f"(v.x), "=f"(v.y)
      : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ double2 ld_tap(const double2* p, uint64_t pol) {
  double2 v;
  asm("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
      : "=d"(v.x), "=d"(v.y)
      : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ uint64_t evict_last_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;"
               : "=l"(pol));
  return pol;
}

// Slab-stack descriptor of a record (plane with support s, offsets ou,
// ov; footprint centre at tile-relative column gu, row gv; tiles TW wide):
//   x = A + Cp, y = A + Cn, z = B,
//   w = Lf | c0 << 8 | (c1 - c0) << 16
// where A is the slab tap index of tile row 0 for a column offset of 0, B
// the slab taps per tile row (+-row pitch; rows mirrored for ov < 0), Cp +
// col and Cn - col the column offsets on the non-negative and the negative
// side of the column fold (which begins at lane column Lf), and [c0, c1]
// the footprint's columns in the tile; so the tap of tile cell (row, col)
// is slabs[(col >= Lf ? x + col : y - col) + row * B] for c0 <= col <= c1.
template <int TW, int OS = 0>
__device__ __forceinline__ int4 slab_record(const StackView& v, int plane,
                                            int s, int ou, int ov, int gu,
                                            int gv) {
  // OS > 0: the oversampling known at compile time (integer divisions and
  // remainders by it become shifts and masks when it is a power of two).
  const int os = OS > 0 ? OS : v.oversample, omax = v.omax;
  const int M = slab_cols_m(s, os, omax);
  const int pitch = os * M;
  const int sb = (int)(v.sbase[plane] + abs(ov) * slab_taps(s, os, omax));
  const int A = ov >= 0 ? sb + (s + kSlicePad - gv) * pitch
                        : sb + (s + kSlicePad + gv) * pitch;
  const int B = ov >= 0 ? pitch : -pitch;
  const int ap = ((ou % os) + os) % os, an = ((-ou % os) + os) % os;
  const int bp = (ou - ap) / os, bn = (-ou - an) / os;
  const int Cp = ap * M + bp - gu, Cn = an * M + bn + gu;
  // floor(ou / os); the fold lane is gu - floor(ou / os).
  const int fl = ou >= 0 ? ou / os : -((-ou + os - 1) / os);
  const int Lf = min(max(gu - fl, 0), TW);
  const int c0 = max(gu - s, 0), c1 = min(gu + s, TW - 1);
  return make_int4(A + Cp, A + Cn, B, Lf | (c0 << 8) | ((c1 - c0) << 16));
}

}  // namespace

}  // namespace gg
