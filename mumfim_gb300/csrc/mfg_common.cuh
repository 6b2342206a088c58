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

#ifndef MFG_SERVER_LOOP_CUH
#define MFG_SERVER_LOOP_CUH
namespace mfg {

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Persistent serving loop of one CTA: claim the next request from the ring,
// solve its RVE with `solve`, publish the completion record, repeat. Every
// wait is bounded: a CTA that finds no work for `idle_ns` (or after
// kServerMaxPolls polls) leaves; the host relaunches the kernel while work is
// pending. Requests and completions live in host-mapped memory; the claim
// counter lives in device memory.
constexpr long long kServerMaxPolls = 1LL << 26;

template <typename Solve>
__device__ void server_loop(const ServerArgs& sa, Solve solve) {
  __shared__ long long s_idx;
  __shared__ double s_F[9];
  __shared__ int s_req[2];
  for (;;) {
    if (threadIdx.x == 0) {
      long long idx = -1;
      const unsigned long long t0 = global_ns();
      for (long long polls = 0; polls < kServerMaxPolls; ++polls) {
        if (*sa.stop) break;
        const unsigned long long h = *reinterpret_cast<volatile unsigned long long*>(sa.head);
        const long long t = *sa.tail;
        if (static_cast<long long>(h) < t) {
          if (atomicCAS(sa.head, h, h + 1) == h) {
            idx = static_cast<long long>(h);
            break;
          }
          continue;
        }
        if (global_ns() - t0 > sa.idle_ns) break;
        __nanosleep(1000);
      }
      __threadfence_system();  // order the ring entry after the tail we saw
      if (idx >= 0) {
        // The host may reuse this ring slot after `cap` requests: read it with
        // volatile loads (no stale L1 line) into shared memory.
        const volatile ServerReq* q = sa.ring + (idx % sa.cap);
        s_req[0] = q->rve;
        s_req[1] = q->update_coords;
        for (int k = 0; k < 9; ++k) s_F[k] = q->F[k];
      }
      s_idx = idx;
    }
    __syncthreads();
    const long long idx = s_idx;
    const int rve = s_req[0];
    const int update = s_req[1];
    __syncthreads();
    if (idx < 0) return;
    const unsigned long long t_claim = global_ns();
    RunArgs a;
    a.F = s_F;
    a.n_F = 1;
    a.update_coords = update;
    a.sigma = sa.sigma;
    a.st_status = sa.st_status;
    a.st_steps = sa.st_steps;
    a.st_residual = sa.st_residual;
    solve(a, rve);  // ends with __syncthreads()
    if (threadIdx.x == 0) {
      __threadfence();
      ServerDone* d = sa.done + (idx % sa.cap);
      d->rve = rve;
      d->status = sa.st_status[rve];
      d->steps = sa.st_steps[rve];
      d->residual = sa.st_residual[rve];
      for (int k = 0; k < 6; ++k) d->sigma[k] = sa.sigma[6 * rve + k];
      d->t_claim_ns = static_cast<long long>(t_claim);
      d->t_done_ns = static_cast<long long>(global_ns());
      __threadfence_system();
      *reinterpret_cast<volatile long long*>(&d->ticket_plus1) = idx + 1;
      __threadfence_system();
    }
    __syncthreads();
  }
}

}  // namespace mfg
#endif
