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

// System-scope accesses to host-mapped memory: the host writes the request
// ring, tail and stop flag and reads the completion records while the kernel
// runs, so these go around the GPU caches (relaxed / release at .sys scope).
__device__ __forceinline__ long long ld_sys(const volatile long long* p) {
  long long v;
  asm volatile("ld.relaxed.sys.global.s64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_sys(const volatile int* p) {
  int v;
  asm volatile("ld.relaxed.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ double ld_sys(const volatile double* p) {
  double v;
  asm volatile("ld.relaxed.sys.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ long long ld_acquire_sys(const volatile long long* p) {
  long long v;
  asm volatile("ld.acquire.sys.global.s64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_sys(volatile long long* p, long long v) {
  asm volatile("st.relaxed.sys.global.s64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_sys(volatile int* p, int v) {
  asm volatile("st.relaxed.sys.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_sys(volatile double* p, double v) {
  asm volatile("st.relaxed.sys.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ void st_release_sys(volatile long long* p, long long v) {
  asm volatile("st.release.sys.global.s64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ long long ld_gpu(const volatile long long* p) {
  long long v;
  asm volatile("ld.relaxed.gpu.global.s64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_gpu(const volatile int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Persistent serving loop of one CTA: claim the next request from the ring,
// solve its RVE with `solve`, publish the completion record, repeat.
// Shutdown is collective, so the kernel never thins out to a few CTAs: a CTA
// may start closing only when every CTA of the grid is waiting and no
// request has been claimed anywhere for `idle_ns`; closing sets a flag that
// makes every CTA leave at its next poll, and the host relaunches the kernel
// whenever work is pending after it ended. Every wait is bounded: by the
// idle timeout, by `max_wait_ns` of device time per wait (a host that stops
// publishing, or never sets the stop flag, frees the SMs within that time),
// and by kServerMaxPolls polls. Requests and completions live in host-mapped
// memory; the counters the CTAs poll (published, claimed, stop) live in
// device memory, so idle CTAs never hammer a host cache line the host is
// writing.
constexpr long long kServerMaxPolls = 1LL << 26;

// True once a wait that started at t0 has lasted longer than the server's
// bound on one wait.
__device__ __forceinline__ bool server_wait_expired(const ServerArgs& sa, unsigned long long t0,
                                                    unsigned long long now) {
  return now > t0 && now - t0 > sa.max_wait_ns;
}

// One attempt to claim the next published request of a ring (a few CAS
// retries under contention): its ring index, or -1 when none is waiting.
__device__ __forceinline__ long long server_try_claim(const ServerArgs& sa) {
  for (int tries = 0; tries < 64; ++tries) {
    const unsigned long long h = *reinterpret_cast<volatile unsigned long long*>(sa.head);
    const long long t = ld_gpu(sa.tail);
    if (static_cast<long long>(h) >= t) return -1;
    if (atomicCAS(sa.head, h, h + 1) == h) {
      atomicMax(sa.last_claim, global_ns());
      return static_cast<long long>(h);
    }
  }
  return -1;
}

// True when a ring holds published requests nobody has claimed yet.
__device__ __forceinline__ bool server_pending(const ServerArgs& sa) {
  const unsigned long long h = *reinterpret_cast<volatile unsigned long long*>(sa.head);
  return static_cast<long long>(h) < ld_gpu(sa.tail);
}

// Copies request `idx` into shared memory. The host may reuse the ring slot
// after `cap` requests: read it with system-scope loads (no stale L1 line).
__device__ __forceinline__ void server_read_request(const ServerArgs& sa, long long idx,
                                                    int* s_req, double* s_F) {
  __threadfence_system();  // order the ring entry after the tail we saw
  const volatile ServerReq* q = sa.ring + (idx % sa.cap);
  s_req[0] = ld_sys(&q->rve);
  s_req[1] = ld_sys(&q->flags);
  for (int k = 0; k < 9; ++k) s_F[k] = ld_sys(&q->F[k]);
}

// Publishes the completion record of request `idx` (one thread); with
// `stiffness`, also the RVE's material stiffness and the worst status of its
// perturbed solves.
__device__ __forceinline__ void server_publish_done(const ServerArgs& sa, long long idx, int rve,
                                                    unsigned long long t_claim,
                                                    bool stiffness = false) {
  __threadfence();
  volatile ServerDone* d = sa.done + (idx % sa.cap);
  st_sys(&d->rve, rve);
  st_sys(&d->status, sa.st_status[rve]);
  st_sys(&d->steps, sa.st_steps[rve]);
  st_sys(&d->residual, sa.st_residual[rve]);
  for (int k = 0; k < 6; ++k) st_sys(&d->sigma[k], sa.sigma[6 * rve + k]);
  st_sys(&d->stiff_status, stiffness ? sa.stiff_status[rve] : -1);
  if (stiffness)
    for (int k = 0; k < 36; ++k) st_sys(&d->C[k], sa.C[36 * rve + k]);
  st_sys(&d->t_claim_ns, static_cast<long long>(t_claim));
  st_sys(&d->t_done_ns, static_cast<long long>(global_ns()));
  __threadfence_system();
  st_release_sys(&d->ticket_plus1, idx + 1);
}

// Arguments of perturbed solve i of a request's material stiffness: the
// i-th perturbation gradient, no update, results into the stiffness scratch.
__device__ __forceinline__ RunArgs stiffness_args(const ServerArgs& sa, int i) {
  RunArgs a;
  a.F = sa.stiff_F + 9 * i;
  a.n_F = 1;
  a.update_coords = 0;
  a.sigma = sa.sigma1;
  a.st_status = sa.st1_status;
  a.st_steps = sa.st1_steps;
  a.st_residual = sa.st1_residual;
  return a;
}

// Column i of the RVE's stiffness from perturbed solve i, C[j][i] =
// (sigma_i[j] - sigma[j]) / h around the stress of the last updating run
// (BatchedFiberRVEAnalysisExplicit.h:396-403), and the worst perturbed
// status; threads 0-5 of the CTA that holds the stress. The caller
// separates successive calls with a barrier.
__device__ __forceinline__ void stiffness_column(const ServerArgs& sa, int rve, int i) {
  const int j = threadIdx.x;
  if (j < 6)
    sa.C[36 * rve + 6 * j + i] = (sa.sigma1[6 * rve + j] - sa.cur_stress[6 * rve + j]) / kStiffStep;
  if (j == 0) {
    const int st = sa.st1_status[rve];
    sa.stiff_status[rve] = i == 0 ? st : max(sa.stiff_status[rve], st);
  }
}

template <typename Solve>
__device__ void server_loop(const ServerArgs& sa, Solve solve) {
  __shared__ long long s_idx;
  __shared__ double s_F[9];
  __shared__ int s_req[2];
  for (;;) {
    if (threadIdx.x == 0) {
      long long idx = -1;
      const unsigned long long t0 = global_ns();
      atomicAdd(sa.idle_ctas, 1);
      for (long long polls = 0; polls < kServerMaxPolls; ++polls) {
        if (ld_gpu(sa.stop) || ld_gpu(sa.closing)) break;
        const unsigned long long h = *reinterpret_cast<volatile unsigned long long*>(sa.head);
        const long long t = ld_gpu(sa.tail);
        if (static_cast<long long>(h) < t) {
          if (atomicCAS(sa.head, h, h + 1) == h) {
            idx = static_cast<long long>(h);
            atomicMax(sa.last_claim, global_ns());
            break;
          }
          continue;
        }
        const unsigned long long now = global_ns();
        const unsigned long long last =
            *reinterpret_cast<volatile unsigned long long*>(sa.last_claim);
        const unsigned long long since = last > t0 ? last : t0;
        if (now > since && now - since > sa.idle_ns &&
            ld_gpu(sa.idle_ctas) == static_cast<int>(gridDim.x)) {
          atomicExch(sa.closing, 1);
          break;
        }
        if (server_wait_expired(sa, t0, now)) break;
        __nanosleep(2000);
      }
      atomicSub(sa.idle_ctas, 1);
      if (idx >= 0) server_read_request(sa, idx, s_req, s_F);
      s_idx = idx;
    }
    __syncthreads();
    const long long idx = s_idx;
    const int rve = s_req[0];
    const int flags = s_req[1];
    __syncthreads();
    if (idx < 0) return;
    const unsigned long long t_claim = global_ns();
    RunArgs a;
    a.F = s_F;
    a.n_F = 1;
    a.update_coords = flags & kReqUpdate;
    a.sigma = sa.sigma;
    a.st_status = sa.st_status;
    a.st_steps = sa.st_steps;
    a.st_residual = sa.st_residual;
    // the request's solve, then with kReqStiffness the six perturbed solves
    // of mfg_batch_material_stiffness(), in its order, on this CTA (one call
    // site, so the solve is inlined once)
    const bool stiff = (flags & kReqStiffness) != 0;
    for (int k = 0; k <= (stiff ? 6 : 0); ++k) {
      solve(k == 0 ? a : stiffness_args(sa, k - 1), rve);  // ends with __syncthreads()
      if (k > 0) {
        stiffness_column(sa, rve, k - 1);
        __syncthreads();
      }
    }
    if (threadIdx.x == 0) server_publish_done(sa, idx, rve, t_claim, stiff);
    __syncthreads();
  }
}

}  // namespace mfg
#endif
