// Uniform weighting on the GPU: the density grid of visibility weights and
// the re-weighting of visibilities by it, with the reference's arithmetic
// (utils/oskar_grid_weights.c:38-172).
//
// Cell of a visibility: (int)round(-uu * (grid_size * cell_size)) + centre
// and (int)round(vv * ...) + centre in the call's precision, the same cell
// the gridder places it in; points outside [0, grid_size) are skipped.
//
// Density: the reference adds the weights into the grid one visibility at a
// time, so each cell's sum is formed in visibility order.  Here the
// visibilities are keyed by cell and stably sorted (visibility order kept
// within a cell), and one thread adds each cell's run in that order onto
// the cell's existing value -- the same additions in the same order, so the
// density grid is bit-identical to the serial code's.
#include "gg_internal.h"
#include "gg_placement.cuh"

namespace gg {

namespace {

constexpr int kThreads = 256;

// Cell index gv * G + gu of a point, or false when it lies off the grid.
template <typename Real>
__device__ __forceinline__ bool weight_cell(Real uu, Real vv, Real scale,
                                            int grid_size, uint32_t* cell) {
  const Real ru = rround(rmul(-uu, scale)), rv = rround(rmul(vv, scale));
  // Outside int range (or NaN) the reference's conversion gives INT_MIN
  // and the point is skipped.
  if (!(rabs(ru) < (Real)2147483648.0) || !(rabs(rv) < (Real)2147483648.0))
    return false;
  const long long centre = grid_size / 2;
  const long long gu = (long long)(int)ru + centre;
  const long long gv = (long long)(int)rv + centre;
  if (gu >= grid_size || gu < 0 || gv >= grid_size || gv < 0) return false;
  *cell = (uint32_t)(gv * grid_size + gu);
  return true;
}

// key = cell (G*G for skipped points, which sort last), value = index.
template <typename Real>
__global__ void __launch_bounds__(kThreads)
k_weight_keys(const Real* __restrict__ uu, const Real* __restrict__ vv,
              unsigned long long n, Real scale, int grid_size,
              uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
              unsigned long long* __restrict__ num_skipped) {
  const unsigned long long i =
      (unsigned long long)blockIdx.x * kThreads + threadIdx.x;
  bool skip = false;
  if (i < n) {
    uint32_t c;
    skip = !weight_cell(uu[i], vv[i], scale, grid_size, &c);
    keys[i] = skip ? (uint32_t)((unsigned long long)grid_size * grid_size) : c;
    vals[i] = (uint32_t)i;
  }
  const unsigned int cnt = __popc(__ballot_sync(0xffffffffu, skip));
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(num_skipped, cnt);
}

__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }

// The first thread of each run of equal cells adds the run's weights, in
// visibility order, onto the cell.
template <typename Real>
__global__ void __launch_bounds__(kThreads)
k_weight_runs(const uint32_t* __restrict__ keys,
              const uint32_t* __restrict__ vals, unsigned long long n,
              const Real* __restrict__ weight, unsigned long long num_cells,
              Real* __restrict__ grid) {
  const unsigned long long j =
      (unsigned long long)blockIdx.x * kThreads + threadIdx.x;
  if (j >= n) return;
  const uint32_t c = keys[j];
  if (c >= num_cells || (j > 0 && keys[j - 1] == c)) return;
  Real g = grid[c];
  for (unsigned long long t = j; t < n && keys[t] == c; ++t)
    g = radd(g, weight[vals[t]]);
  grid[c] = g;
}

__device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }

// weight_out = weight_in / density, or 0 where the density is 0; skipped
// points leave weight_out untouched.
template <typename Real>
__global__ void __launch_bounds__(kThreads)
k_weights_read(const Real* __restrict__ uu, const Real* __restrict__ vv,
               const Real* __restrict__ w_in, Real* __restrict__ w_out,
               unsigned long long n, Real scale, int grid_size,
               const Real* __restrict__ grid,
               unsigned long long* __restrict__ num_skipped) {
  const unsigned long long i =
      (unsigned long long)blockIdx.x * kThreads + threadIdx.x;
  bool skip = false;
  if (i < n) {
    uint32_t c;
    skip = !weight_cell(uu[i], vv[i], scale, grid_size, &c);
    if (!skip) {
      const Real d = grid[c];
      w_out[i] = d != (Real)0 ? rdiv(w_in[i], d) : (Real)0;
    }
  }
  const unsigned int cnt = __popc(__ballot_sync(0xffffffffu, skip));
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(num_skipped, cnt);
}

unsigned blocks_for(unsigned long long n) {
  return (unsigned)((n + kThreads - 1) / kThreads);
}

}  // namespace

template <typename Real>
cudaError_t launch_weight_keys(const Real* uu, const Real* vv,
                               unsigned long long n, Real cell_size_rad,
                               int grid_size, uint32_t* keys, uint32_t* vals,
                               unsigned long long* d_num_skipped,
                               cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  // utils/oskar_grid_weights.c:46 (FP64) and :114 (FP32): grid_scale in
  // the call's precision.
  const Real scale = (Real)grid_size * cell_size_rad;
  k_weight_keys<Real><<<blocks_for(n), kThreads, 0, s>>>(
      uu, vv, n, scale, grid_size, keys, vals, d_num_skipped);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_weight_runs(const uint32_t* keys, const uint32_t* vals,
                               unsigned long long n, const Real* weight,
                               int grid_size, Real* grid, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_weight_runs<Real><<<blocks_for(n), kThreads, 0, s>>>(
      keys, vals, n, weight, (unsigned long long)grid_size * grid_size,
      grid);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_weights_read(const Real* uu, const Real* vv,
                                const Real* w_in, Real* w_out,
                                unsigned long long n, Real cell_size_rad,
                                int grid_size, const Real* grid,
                                unsigned long long* d_num_skipped,
                                cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const Real scale = (Real)grid_size * cell_size_rad;
  k_weights_read<Real><<<blocks_for(n), kThreads, 0, s>>>(
      uu, vv, w_in, w_out, n, scale, grid_size, grid, d_num_skipped);
  return cudaGetLastError();
}

template cudaError_t launch_weight_keys<float>(const float*, const float*,
                                               unsigned long long, float, int,
                                               uint32_t*, uint32_t*,
                                               unsigned long long*,
                                               cudaStream_t);
template cudaError_t launch_weight_keys<double>(const double*, const double*,
                                                unsigned long long, double,
                                                int, uint32_t*, uint32_t*,
                                                unsigned long long*,
                                                cudaStream_t);
template cudaError_t launch_weight_runs<float>(const uint32_t*,
                                               const uint32_t*,
                                               unsigned long long,
                                               const float*, int, float*,
                                               cudaStream_t);
template cudaError_t launch_weight_runs<double>(const uint32_t*,
                                                const uint32_t*,
                                                unsigned long long,
                                                const double*, int, double*,
                                                cudaStream_t);
template cudaError_t launch_weights_read<float>(const float*, const float*,
                                                const float*, float*,
                                                unsigned long long, float, int,
                                                const float*,
                                                unsigned long long*,
                                                cudaStream_t);
template cudaError_t launch_weights_read<double>(const double*,
                                                 const double*,
                                                 const double*, double*,
                                                 unsigned long long, double,
                                                 int, const double*,
                                                 unsigned long long*,
                                                 cudaStream_t);

}  // namespace gg
