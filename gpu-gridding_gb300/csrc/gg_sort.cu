// Device-wide exclusive scan and stable LSD radix sort of (key, value)
// pairs.  These order the (visibility, tile) records by (grid, tile, plane,
// offset class) so the gridding kernel sees each tile's records contiguously
// and grouped by kernel slice.  The reference bins with an atomic bucket
// scatter whose in-bucket order changes from run to run
// (oskar_grid_wproj_gpu.cu:520-649); this sort is stable, so the record
// order -- and with it the accumulation order -- is the same on every call.
#include "gg_internal.h"

namespace gg {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // 2048

__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total to *total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x,
                                                         uint32_t* total) {
  __shared__ uint32_t warp_sums[33];  // [32] holds the block total
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  uint32_t inc = warp_inclusive_scan(x);
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < nwarps ? warp_sums[lane] : 0;
    uint32_t wi = warp_inclusive_scan(w);
    if (lane < nwarps) warp_sums[lane] = wi - w;
    if (lane == nwarps - 1) warp_sums[32] = wi;
  }
  __syncthreads();
  uint32_t result = warp_sums[warp] + inc - x;
  *total = warp_sums[32];
  __syncthreads();
  return result;
}

// Scan input loader (a functor, so other input forms can reuse the
// kernels).
struct LoadU32 {
  const uint32_t* in;
  __device__ __forceinline__ uint32_t operator()(size_t i) const {
    return in[i];
  }
};

template <typename Load>
__global__ void k_scan_reduce(Load in, size_t n,
                              uint32_t* __restrict__ block_sums) {
  const size_t base = (size_t)blockIdx.x * kScanTile;
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    size_t idx = base + (size_t)i * kScanThreads + threadIdx.x;
    if (idx < n) s += in(idx);
  }
  uint32_t total;
  block_exclusive_scan(s, &total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// Exclusive scan of the block sums in place by one block, chunk by chunk.
__global__ void k_scan_top(uint32_t* __restrict__ sums, size_t nb,
                           uint32_t* __restrict__ d_total) {
  uint32_t carry = 0;
  for (size_t base = 0; base < nb; base += blockDim.x) {
    size_t idx = base + threadIdx.x;
    uint32_t x = idx < nb ? sums[idx] : 0;
    uint32_t total;
    uint32_t ex = block_exclusive_scan(x, &total);
    if (idx < nb) sums[idx] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0 && d_total) *d_total = carry;
}

template <typename Load>
__global__ void k_scan_down(Load in, uint32_t* __restrict__ out, size_t n,
                            const uint32_t* __restrict__ block_offsets) {
  __shared__ uint32_t tile[kScanTile];
  const size_t base = (size_t)blockIdx.x * kScanTile;
  // Striped, coalesced load into shared memory.
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    int t = i * kScanThreads + threadIdx.x;
    size_t idx = base + t;
    tile[t] = idx < n ? in(idx) : 0;
  }
  __syncthreads();
  // Each thread scans its kScanItems consecutive entries.
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = tile[threadIdx.x * kScanItems + i];
    s += v[i];
  }
  uint32_t total;
  uint32_t pre = block_exclusive_scan(s, &total) + block_offsets[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    tile[threadIdx.x * kScanItems + i] = pre;
    pre += v[i];
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    int t = i * kScanThreads + threadIdx.x;
    size_t idx = base + t;
    if (idx < n) out[idx] = tile[t];
  }
}

// ---------------------------------------------------------------------------
// Radix sort: 8-bit digits, 4096 keys per block, reduce-then-scan per pass.
// ---------------------------------------------------------------------------
constexpr int kRadixThreads = 256;
constexpr int kRadixWarps = kRadixThreads / 32;
constexpr int kRadixRounds = 16;
constexpr int kRadixTile = kRadixThreads * kRadixRounds;  // 4096
constexpr int kRadixDigits = 256;

__global__ void __launch_bounds__(kRadixThreads)
k_radix_hist(const uint32_t* __restrict__ keys, size_t n, int shift,
             int num_blocks, uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[kRadixDigits];
  h[threadIdx.x] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * kRadixTile;
  // All loads first (independent, in flight together), then the counts.
  uint32_t k[kRadixRounds];
#pragma unroll
  for (int r = 0; r < kRadixRounds; ++r) {
    const size_t idx = base + (size_t)r * kRadixThreads + threadIdx.x;
    k[r] = idx < n ? keys[idx] : 0u;
  }
#pragma unroll
  for (int r = 0; r < kRadixRounds; ++r) {
    const size_t idx = base + (size_t)r * kRadixThreads + threadIdx.x;
    if (idx < n) atomicAdd(&h[(k[r] >> shift) & 0xFF], 1u);
  }
  __syncthreads();
  // Digit-major layout: the scan then yields, for each (digit, block), the
  // global position of that block's first key with that digit.
  hist[(size_t)threadIdx.x * num_blocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one 4096-key block: the keys are first ordered by digit
// in shared memory (in block order within a digit), then written out in
// that order, so keys with the same digit go to consecutive addresses and a
// warp's stores form a few contiguous runs instead of 32 scattered words.
// Warp w ranks its own 512 consecutive keys (lane l's j-th key is key
// w * 512 + j * 32 + l of the block) against warp-private digit counters,
// so the ranking needs no block barrier; one per-digit prefix over the
// warps then places every key.  hist holds the block's digit counts
// (digit-major, as k_radix_hist wrote them) and offsets their exclusive
// scan (global start of each (digit, block) run).
__global__ void __launch_bounds__(kRadixThreads, 3)
k_radix_scatter(const uint32_t* __restrict__ keys,
                const uint32_t* __restrict__ vals, size_t n, int shift,
                int num_blocks, const uint32_t* __restrict__ hist,
                const uint32_t* __restrict__ offsets,
                uint32_t* __restrict__ keys_out,
                uint32_t* __restrict__ vals_out) {
  constexpr int kPerWarp = kRadixTile / kRadixWarps;   // 512
  __shared__ uint32_t s_keys[kRadixTile];
  __shared__ uint32_t s_vals[kRadixTile];
  __shared__ uint32_t digit_base[kRadixDigits];   // global run start
  __shared__ uint32_t local_start[kRadixDigits];  // block-local run start
  // Per warp and digit: the warp's count, then the keys of the digit in
  // the warps before it.
  __shared__ uint32_t warp_count[kRadixWarps][kRadixDigits];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t cell = (size_t)threadIdx.x * num_blocks + blockIdx.x;
  digit_base[threadIdx.x] = offsets[cell];
#pragma unroll
  for (int w = 0; w < kRadixWarps; ++w) warp_count[w][threadIdx.x] = 0;
  uint32_t total;
  // (block_exclusive_scan ends with a barrier: the counters are zeroed.)
  local_start[threadIdx.x] = block_exclusive_scan(hist[cell], &total);
  const uint32_t lt_mask = (1u << lane) - 1u;
  const size_t base = (size_t)blockIdx.x * kRadixTile;
  const int valid_n = (int)min((size_t)kRadixTile, n - base);
  const int wbase = warp * kPerWarp;
  // The warp's keys and values, all loads in flight together.
  uint32_t kr[kRadixRounds], vr[kRadixRounds];
#pragma unroll
  for (int j = 0; j < kRadixRounds; ++j) {
    const int t = wbase + j * 32 + lane;
    kr[j] = t < valid_n ? keys[base + t] : 0u;
    vr[j] = t < valid_n ? vals[base + t] : 0u;
  }
  // Ranks within the warp, in key order: the digit's keys in the warp's
  // earlier rounds plus the lower lanes of this round with the same digit.
  uint32_t* cnt = warp_count[warp];
#pragma unroll
  for (int j = 0; j < kRadixRounds; ++j) {
    const bool valid = wbase + j * 32 + lane < valid_n;
    // Invalid lanes take digit 256 so they never match a valid one.
    const uint32_t digit = valid ? ((kr[j] >> shift) & 0xFF) : 256u;
    const uint32_t peers = __match_any_sync(0xffffffffu, digit);
    // The counter is read at digit & 0xFF: the load may be issued for
    // invalid lanes too, and digit 256 would lie past the warp's row (past
    // the whole array for the last warp).
    const uint32_t c_before = cnt[digit & 0xFFu];
    const uint32_t before = valid ? c_before : 0u;
    // The rank waits in s_keys at the key's own index (free until the
    // placement below, which reads it back first).
    s_keys[wbase + j * 32 + lane] = before + __popc(peers & lt_mask);
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1)
      cnt[digit & 0xFFu] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // Per digit (thread t owns digit t): the keys in the warps before each.
  {
    uint32_t running = 0;
#pragma unroll
    for (int w = 0; w < kRadixWarps; ++w) {
      const uint32_t c = warp_count[w][threadIdx.x];
      warp_count[w][threadIdx.x] = running;
      running += c;
    }
  }
  __syncthreads();   // every digit's prefix written before any is read
  uint32_t pos[kRadixRounds];
#pragma unroll
  for (int j = 0; j < kRadixRounds; ++j) {
    const uint32_t d = (kr[j] >> shift) & 0xFF;
    pos[j] = local_start[d] + warp_count[warp][d] + s_keys[wbase + j * 32 + lane];
  }
  __syncthreads();   // every rank read before any key lands in s_keys
#pragma unroll
  for (int j = 0; j < kRadixRounds; ++j) {
    // pos < valid_n for every valid key (the ranks of a digit fill its
    // block-local run); the bound also keeps a stray rank in the array.
    if (wbase + j * 32 + lane < valid_n && pos[j] < (uint32_t)kRadixTile) {
      s_keys[pos[j]] = kr[j];
      s_vals[pos[j]] = vr[j];
    }
  }
  __syncthreads();
  // Write the block out in digit order.
  for (int i = threadIdx.x; i < valid_n; i += kRadixThreads) {
    const uint32_t key = s_keys[i];
    const uint32_t d = (key >> shift) & 0xFF;
    const uint32_t pos = digit_base[d] + ((uint32_t)i - local_start[d]);
    keys_out[pos] = key;
    vals_out[pos] = s_vals[i];
  }
}

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

size_t scan_temp_bytes(size_t n) {
  size_t nb = (n + kScanTile - 1) / kScanTile;
  return align_up((nb + 1) * sizeof(uint32_t), 256);
}

template <typename Load>
static cudaError_t scan_impl(Load in, uint32_t* out, size_t n,
                             uint32_t* d_total, void* tmp, cudaStream_t s) {
  if (n == 0) {
    if (d_total) return cudaMemsetAsync(d_total, 0, sizeof(uint32_t), s);
    return cudaSuccess;
  }
  size_t nb = (n + kScanTile - 1) / kScanTile;
  uint32_t* sums = (uint32_t*)tmp;
  k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, sums);
  k_scan_top<<<1, 1024, 0, s>>>(sums, nb, d_total);
  k_scan_down<<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, sums);
  return cudaGetLastError();
}

// *total = sum of in[0..n) in 64 bits (the scan's 32-bit total wraps).
__global__ void k_sum_u32(const uint32_t* __restrict__ in, size_t n,
                          unsigned long long* __restrict__ total) {
  unsigned long long v = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    v += in[i];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __shared__ unsigned long long w[32];
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? w[threadIdx.x] : 0ull;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && v) atomicAdd(total, v);
  }
}

cudaError_t sum_u32(const uint32_t* in, size_t n, unsigned long long* total,
                    cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(total, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  if (n == 0) return cudaSuccess;
  const size_t blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  k_sum_u32<<<(unsigned)blocks, 256, 0, s>>>(in, n, total);
  return cudaGetLastError();
}

cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n,
                               uint32_t* d_total, void* tmp, cudaStream_t s) {
  return scan_impl(LoadU32{in}, out, n, d_total, tmp, s);
}

size_t radix_temp_bytes(size_t n) {
  size_t nb = (n + kRadixTile - 1) / kRadixTile;
  if (nb == 0) nb = 1;
  size_t hist = align_up(nb * kRadixDigits * sizeof(uint32_t), 256);
  return 2 * hist + scan_temp_bytes(nb * kRadixDigits);
}

cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals,
                             uint32_t* keys_alt, uint32_t* vals_alt, size_t n,
                             int end_bit, void* tmp, cudaStream_t s,
                             bool* in_alt) {
  *in_alt = false;
  if (n <= 1 || end_bit <= 0) return cudaSuccess;
  size_t nb = (n + kRadixTile - 1) / kRadixTile;
  size_t hist_bytes = align_up(nb * kRadixDigits * sizeof(uint32_t), 256);
  uint32_t* hist = (uint32_t*)tmp;
  uint32_t* offs = (uint32_t*)((char*)tmp + hist_bytes);
  void* scan_tmp = (char*)tmp + 2 * hist_bytes;
  uint32_t *k_in = keys, *v_in = vals, *k_out = keys_alt, *v_out = vals_alt;
  for (int shift = 0; shift < end_bit; shift += 8) {
    k_radix_hist<<<(unsigned)nb, kRadixThreads, 0, s>>>(k_in, n, shift,
                                                        (int)nb, hist);
    cudaError_t e = exclusive_scan_u32(hist, offs, nb * kRadixDigits, nullptr,
                                       scan_tmp, s);
    if (e != cudaSuccess) return e;
    k_radix_scatter<<<(unsigned)nb, kRadixThreads, 0, s>>>(
        k_in, v_in, n, shift, (int)nb, hist, offs, k_out, v_out);
    uint32_t* t;
    t = k_in; k_in = k_out; k_out = t;
    t = v_in; v_in = v_out; v_out = t;
    *in_alt = !*in_alt;
  }
  return cudaGetLastError();
}

}  // namespace gg
