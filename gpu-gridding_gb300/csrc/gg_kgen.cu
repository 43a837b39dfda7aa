// W-kernel generation on the device: the taper x chirp kernel cube the
// synthetic workloads use, built where it is consumed so that no cube
// crosses the host link (the reference reads its kernels from FITS files,
// utils/read_kernel.c:36-118, and ships them to the GPU on every call).
//
// Plane p, quadrant sample (iv, iu) in oversampled pixels,
// r2 = iv^2 + iu^2:
//   k = exp(-2 (r2 / os^2) / s_p^2) * exp(i pi w_p r2 / csh^2)
// with s_p = max(support[p], 1), normalised by the complex sum of the taps
// a visibility at zero offset uses, k[|j| os][|l| os] for j, l in
// [-s_p, s_p] with |j| os, |l| os < csh, so those taps sum to 1.  All of
// it in FP64, the result rounded once to the call's precision.
#include "gg_internal.h"

namespace gg {

namespace {

__device__ __forceinline__ double2 kernel_value(int iv, int iu, int os,
                                                int csh, double s2,
                                                double w_p) {
  const double r2 = (double)iv * iv + (double)iu * iu;
  const double taper = exp(-2.0 * (r2 / (double)(os * os)) / s2);
  const double phase = 3.141592653589793 * w_p * r2 / ((double)csh * csh);
  double sn, cs;
  sincos(phase, &sn, &cs);
  return make_double2(taper * cs, taper * sn);
}

// One block per plane: the complex sum of the zero-offset footprint taps.
__global__ void k_kgen_norm(const int* __restrict__ support,
                            const double* __restrict__ w_planes, int os,
                            int csh, double2* __restrict__ total) {
  const int p = blockIdx.x;
  const int s = max(support[p], 1);
  const double s2 = (double)(s * s);
  const int F = 2 * s + 1;
  double re = 0.0, im = 0.0;
  for (int e = threadIdx.x; e < F * F; e += blockDim.x) {
    const int iv = abs(e / F - s) * os, iu = abs(e % F - s) * os;
    if (iv < csh && iu < csh) {
      const double2 k = kernel_value(iv, iu, os, csh, s2, w_planes[p]);
      re += k.x;
      im += k.y;
    }
  }
  __shared__ double sre[256], sim[256];
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      sre[threadIdx.x] += sre[threadIdx.x + h];
      sim[threadIdx.x] += sim[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) total[p] = make_double2(sre[0], sim[0]);
}

// cube[p][iv][iu] = k / total[p], rounded once to Real.
template <typename Real>
__global__ void k_kgen_cube(const int* __restrict__ support,
                            const double* __restrict__ w_planes, int os,
                            int csh, const double2* __restrict__ total,
                            Real* __restrict__ cube) {
  const int p = blockIdx.y;
  const int s = max(support[p], 1);
  const double s2 = (double)(s * s);
  const double2 t = total[p];
  const double den = t.x * t.x + t.y * t.y;
  const long long n = (long long)csh * csh;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const int iv = (int)(e / csh), iu = (int)(e % csh);
    const double2 k = kernel_value(iv, iu, os, csh, s2, w_planes[p]);
    const size_t o = ((size_t)p * n + e) * 2;
    cube[o] = (Real)((k.x * t.x + k.y * t.y) / den);
    cube[o + 1] = (Real)((k.y * t.x - k.x * t.y) / den);
  }
}

}  // namespace

template <typename Real>
cudaError_t launch_kernel_generate(int num_planes, const int* d_support,
                                   const double* d_w_planes, int oversample,
                                   int conv_size_half, void* d_total,
                                   Real* d_cube, cudaStream_t s) {
  k_kgen_norm<<<num_planes, 256, 0, s>>>(d_support, d_w_planes, oversample,
                                         conv_size_half, (double2*)d_total);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  dim3 grid(64, num_planes);
  k_kgen_cube<Real><<<grid, 256, 0, s>>>(d_support, d_w_planes, oversample,
                                         conv_size_half,
                                         (const double2*)d_total, d_cube);
  return cudaGetLastError();
}

template cudaError_t launch_kernel_generate<float>(int, const int*,
                                                   const double*, int, int,
                                                   void*, float*,
                                                   cudaStream_t);
template cudaError_t launch_kernel_generate<double>(int, const int*,
                                                    const double*, int, int,
                                                    void*, double*,
                                                    cudaStream_t);

}  // namespace gg
