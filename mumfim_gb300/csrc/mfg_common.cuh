// Device helpers shared by the relaxation kernels.
#ifndef MFG_COMMON_CUH
#define MFG_COMMON_CUH

#include <cfloat>
#include <cstdint>

#include "mfg_internal.h"

namespace mfg {

// Block-wide reductions over NT threads; the result is returned to every
// thread. The combination order is fixed (warp butterfly, then warp 0 over
// the warp partials), so a given block size always produces the same bits.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* red) {
  constexpr int NW = NT / 32;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = (l < NW) ? red[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (l == 0) red[NW] = t;
  }
  __syncthreads();
  return red[NW];
}

template <int NT>
__device__ __forceinline__ double block_min(double v, double* red) {
  constexpr int NW = NT / 32;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = (l < NW) ? red[l] : DBL_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t = fmin(t, __shfl_xor_sync(0xffffffffu, t, o));
    if (l == 0) red[NW] = t;
  }
  __syncthreads();
  return red[NW];
}

// B:127-154 updateVolume determinant, row-major F.
__device__ __forceinline__ double jacobian(const double* dg) {
  return dg[0] * (dg[4] * dg[8] - dg[5] * dg[7]) - dg[1] * (dg[3] * dg[8] - dg[5] * dg[6]) +
         dg[2] * (dg[3] * dg[7] - dg[4] * dg[6]);
}

}  // namespace mfg

#endif
