// Mixed-precision relaxation: FP32 forces and integrator, FP64 where it
// matters.
//
// Same algorithm and step structure as the plain FP64 kernel
// (mfg_relax_f64.cu; reference: BatchedFiberRVEAnalysisExplicitTeamOuterLoop.h:180-437),
// with these precision choices:
//  - positions are the FP64 reference X plus an FP32 displacement u_hi with
//    an FP32 compensation u_lo (TwoSum / Kahan), so increments far below an
//    FP32 ulp of u still accumulate: u = u_hi + u_lo to ~1e-14;
//  - fiber forces use the Green strain formed from the displacement
//    difference, g = (dX.du + du.du/2) / l0^2, which keeps its relative
//    precision at small strain (the length-ratio form 0.5(l^2/l0^2 - 1)
//    cancels catastrophically in FP32). For the linear law
//    T/l = lambda E A g / l = E A g / l0 needs neither sqrt nor division;
//  - velocities, the damping force and both kicks are FP32;
//  - FP64 is kept for the critical time step (FP64 lengths every 100 steps),
//    the residual norm, and the stress homogenisation, exactly where the
//    reference reduces over the whole RVE.
// The persistent FP64 state of the batch (x, u, volume) is read at the
// start and written at the end of every run, so both precisions share it.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "mfg_common.cuh"
#include "mfg_internal.h"
#include "mfg_mixed.h"

namespace mfg {

struct MixedState {
  float* u_hi = nullptr;  // 3 * nt
  float* u_lo = nullptr;  // 3 * nt
  float* v = nullptr;     // 3 * nt
  float* minv = nullptr;  // nt, 1 / m
  float* m32 = nullptr;   // nt
  float* dX = nullptr;    // 3 * et reference fiber vectors X[n2] - X[n1]
  float* rl0 = nullptr;   // et, 1 / l0
  float* nrm = nullptr;   // 3 * et per-fiber force vectors (scratch)
  int sms = 1;
  int occ = 1;
};

namespace {

constexpr int kThreadsMixed = 512;

__global__ void mixed_prepare_kernel(const DevBatch b, MixedState ms) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i < b.nt) {
    const double m = b.m[i];
    ms.m32[i] = static_cast<float>(m);
    ms.minv[i] = static_cast<float>(1.0 / m);
  }
}

__global__ void mixed_prepare_fibers_kernel(const DevBatch b, MixedState ms) {
  for (int rve = blockIdx.y; rve < b.n_rve; rve += gridDim.y) {
    const RveDesc d = b.desc[rve];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.n_fibers) continue;
    const int64_t fo = d.fiber_off + e, no = d.node_off;
    const int2 c = b.conn[fo];
    for (int k = 0; k < 3; ++k) {
      const double* X = b.X + k * b.nt + no;
      ms.dX[k * b.et + fo] = static_cast<float>(X[c.y] - X[c.x]);
    }
    ms.rl0[fo] = static_cast<float>(1.0 / b.l0[fo]);
  }
}

struct MixedView {
  const double *X0, *X1, *X2;
  double *x0, *x1, *x2, *u0, *u1, *u2;
  float *h0, *h1, *h2, *lo0, *lo1, *lo2, *v0, *v1, *v2;
  const float *minv, *m32;
  const int2* conn;
  const float *dX0, *dX1, *dX2, *rl0;
  float *n0, *n1, *n2;
  double *fi0, *fi1, *fi2;
  const int32_t* rowptr;
  const int32_t* inc;
  double* ramp;
};

__device__ __forceinline__ MixedView make_view(const DevBatch& b, const MixedState& ms,
                                               const RveDesc& d) {
  MixedView r;
  const int64_t nt = b.nt, et = b.et, no = d.node_off, fo = d.fiber_off;
  r.X0 = b.X + no; r.X1 = b.X + nt + no; r.X2 = b.X + 2 * nt + no;
  r.x0 = b.x + no; r.x1 = b.x + nt + no; r.x2 = b.x + 2 * nt + no;
  r.u0 = b.u + no; r.u1 = b.u + nt + no; r.u2 = b.u + 2 * nt + no;
  r.h0 = ms.u_hi + no; r.h1 = ms.u_hi + nt + no; r.h2 = ms.u_hi + 2 * nt + no;
  r.lo0 = ms.u_lo + no; r.lo1 = ms.u_lo + nt + no; r.lo2 = ms.u_lo + 2 * nt + no;
  r.v0 = ms.v + no; r.v1 = ms.v + nt + no; r.v2 = ms.v + 2 * nt + no;
  r.minv = ms.minv + no;
  r.m32 = ms.m32 + no;
  r.conn = b.conn + fo;
  r.dX0 = ms.dX + fo; r.dX1 = ms.dX + et + fo; r.dX2 = ms.dX + 2 * et + fo;
  r.rl0 = ms.rl0 + fo;
  r.n0 = ms.nrm + fo; r.n1 = ms.nrm + et + fo; r.n2 = ms.nrm + 2 * et + fo;
  r.fi0 = b.fint + no; r.fi1 = b.fint + nt + no; r.fi2 = b.fint + 2 * nt + no;
  r.rowptr = b.rowptr + d.row_off;
  r.inc = b.inc + d.inc_off;
  r.ramp = b.ramp + 6 * d.bnd_off;
  return r;
}

// Per-RVE constants of the fiber law in the T/l form used here.
struct Law {
  int nonlinear;
  float ea;      // E A
  float ea_b;    // E A / B            (toe:  T/l = (E A / B / l0) expm1(B g))
  float B;
  float lt;      // transition stretch
  float Mt, bt;  // linear continuation T = Mt (lambda - lt) + bt above lt
};

__device__ __forceinline__ Law make_law(const RveDesc& d) {
  Law L;
  L.nonlinear = d.law == 1;
  L.ea = static_cast<float>(d.E * d.A);
  L.B = static_cast<float>(d.B);
  L.lt = static_cast<float>(d.lt);
  L.ea_b = 0.f;
  L.Mt = 0.f;
  L.bt = 0.f;
  if (L.nonlinear) {
    // FiberReactions.cc:16-71 with alpha = E A / B, g_t = (lt^2 - 1)/2:
    //   m l0 = alpha ((1 + lt^2 B) e^{B g_t} - 1),  b = alpha lt (e^{B g_t} - 1)
    const double alpha = d.E * d.A / d.B;
    const double gt = 0.5 * (d.lt * d.lt - 1.0);
    const double eg = exp(d.B * gt);
    L.ea_b = static_cast<float>(alpha);
    L.Mt = static_cast<float>(alpha * ((1.0 + d.lt * d.lt * d.B) * eg - 1.0));
    L.bt = static_cast<float>(alpha * d.lt * (eg - 1.0));
  }
  return L;
}

// T / l of one fiber from its Green strain g and 1/l0.
__device__ __forceinline__ float tension_over_length(const Law& L, float g, float rl0) {
  if (!L.nonlinear) return L.ea * g * rl0;
  const float lam2 = fmaf(2.f, g, 1.f);
  if (g < 0.f) {
    // below the compressive transition (ratio 1): T = E A (lambda - 1)
    const float lam = sqrtf(fmaxf(lam2, 0.f));
    const float lm1 = 2.f * g / (lam + 1.f);
    return L.ea * lm1 * rl0 / lam;
  }
  const float lam = sqrtf(lam2);
  if (lam > L.lt) {
    const float T = fmaf(L.Mt, lam - L.lt, L.bt);
    return T * rl0 / lam;
  }
  // toe: T = alpha lambda (e^{B g} - 1), so T / l = alpha (e^{B g} - 1) / l0
  return L.ea_b * expm1f(L.B * g) * rl0;
}

// TwoSum accumulation of an increment into (hi, lo).
__device__ __forceinline__ void comp_add(float& hi, float& lo, float inc) {
  const float y = inc + lo;
  const float s = hi + y;
  const float bp = s - hi;
  const float ap = s - bp;
  lo = (hi - ap) + (y - bp);
  hi = s;
}

__device__ __forceinline__ void split(double u, float& hi, float& lo) {
  hi = static_cast<float>(u);
  lo = static_cast<float>(u - static_cast<double>(hi));
}

__device__ __forceinline__ void gather_f32(const MixedView& r, int i, float& a0, float& a1,
                                           float& a2) {
  a0 = 0.f; a1 = 0.f; a2 = 0.f;
  const int pb = r.rowptr[i], pe = r.rowptr[i + 1];
  for (int p = pb; p < pe; ++p) {
    const int code = __ldg(r.inc + p);
    const int e = code >> 1;
    const float s = (code & 1) ? 1.f : -1.f;
    a0 = fmaf(s, r.n0[e], a0);
    a1 = fmaf(s, r.n1[e], a1);
    a2 = fmaf(s, r.n2[e], a2);
  }
}

// Fiber pass in FP32; every UPDATE_FREQ steps also the FP64 lengths for
// dt_crit. Returns the thread's minimum FP64 length (DBL_MAX otherwise).
__device__ __forceinline__ double fiber_pass_mixed(const MixedView& r, const RveDesc& d,
                                                   const Law& L, bool want_lmin) {
  double lmin = DBL_MAX;
  for (int e = threadIdx.x; e < d.n_fibers; e += kThreadsMixed) {
    const int2 c = __ldg(r.conn + e);
    const float du0 = (r.h0[c.y] - r.h0[c.x]) + (r.lo0[c.y] - r.lo0[c.x]);
    const float du1 = (r.h1[c.y] - r.h1[c.x]) + (r.lo1[c.y] - r.lo1[c.x]);
    const float du2 = (r.h2[c.y] - r.h2[c.x]) + (r.lo2[c.y] - r.lo2[c.x]);
    const float X0 = __ldg(r.dX0 + e), X1 = __ldg(r.dX1 + e), X2 = __ldg(r.dX2 + e);
    const float rl0 = __ldg(r.rl0 + e);
    const float dxdu = fmaf(X0, du0, fmaf(X1, du1, X2 * du2));
    const float dudu = fmaf(du0, du0, fmaf(du1, du1, du2 * du2));
    const float g = fmaf(0.5f, dudu, dxdu) * (rl0 * rl0);
    const float t = tension_over_length(L, g, rl0);
    r.n0[e] = (X0 + du0) * t;
    r.n1[e] = (X1 + du1) * t;
    r.n2[e] = (X2 + du2) * t;
    if (want_lmin) {
      const double a0 = (r.X0[c.y] + (static_cast<double>(r.h0[c.y]) + r.lo0[c.y])) -
                        (r.X0[c.x] + (static_cast<double>(r.h0[c.x]) + r.lo0[c.x]));
      const double a1 = (r.X1[c.y] + (static_cast<double>(r.h1[c.y]) + r.lo1[c.y])) -
                        (r.X1[c.x] + (static_cast<double>(r.h1[c.x]) + r.lo1[c.x]));
      const double a2 = (r.X2[c.y] + (static_cast<double>(r.h2[c.y]) + r.lo2[c.y])) -
                        (r.X2[c.x] + (static_cast<double>(r.h2[c.x]) + r.lo2[c.x]));
      lmin = fmin(lmin, sqrt(a0 * a0 + a1 * a1 + a2 * a2));
    }
  }
  return lmin;
}

__device__ void solve_rve_mixed(const DevBatch& b, const MixedState& ms, const RunArgs& a, int rve,
                                double* red) {
  const RveDesc d = b.desc[rve];
  const MixedView r = make_view(b, ms, d);
  const Law L = make_law(d);
  const int N = d.n_nodes, NF = d.n_free;
  const int tid = threadIdx.x;
  const double* F = a.F + 9 * (a.n_F > 1 ? rve : 0);
  const bool ramp = d.mode == 1;
  double Fm[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Fm[k] = F[k];
  if (a.update_coords && tid == 0) b.vol[rve] = jacobian(Fm) * b.vol[rve];

  // ---- prologue in FP64: predictor, split into (hi, lo), v = 0 -------------
  for (int i = tid; i < N; i += kThreadsMixed) {
    const double xo0 = r.x0[i], xo1 = r.x1[i], xo2 = r.x2[i];
    double up0 = r.u0[i], up1 = r.u1[i], up2 = r.u2[i];
    if (!ramp) {
      up0 = (Fm[0] - 1) * xo0 + Fm[1] * xo1 + Fm[2] * xo2 + up0;
      up1 = Fm[3] * xo0 + (Fm[4] - 1) * xo1 + Fm[5] * xo2 + up1;
      up2 = Fm[6] * xo0 + Fm[7] * xo1 + (Fm[8] - 1) * xo2 + up2;
    }
    const double X0 = r.X0[i], X1 = r.X1[i], X2 = r.X2[i];
    const double xn0 = X0 + up0, xn1 = X1 + up1, xn2 = X2 + up2;
    float hi, lo;
    split(xn0 - X0, hi, lo); r.h0[i] = hi; r.lo0[i] = lo;
    split(xn1 - X1, hi, lo); r.h1[i] = hi; r.lo1[i] = lo;
    split(xn2 - X2, hi, lo); r.h2[i] = hi; r.lo2[i] = lo;
    r.v0[i] = 0.f; r.v1[i] = 0.f; r.v2[i] = 0.f;
    if (ramp && i >= NF) {
      double* rb = r.ramp + 6 * (i - NF);
      rb[0] = xn0; rb[1] = xn1; rb[2] = xn2;
      rb[3] = (Fm[0] - 1) * xn0 + Fm[1] * xn1 + Fm[2] * xn2;
      rb[4] = Fm[3] * xn0 + (Fm[4] - 1) * xn1 + Fm[5] * xn2;
      rb[5] = Fm[6] * xn0 + Fm[7] * xn1 + (Fm[8] - 1) * xn2;
    }
  }
  __syncthreads();
  double dt_crit = block_min<kThreadsMixed>(fiber_pass_mixed(r, d, L, true), red) / d.sound_speed;

  const int cap = d.max_steps;
  const float c = static_cast<float>(d.c);
  int step = 0;
  double residual = 10.0;
  float h_prev = 0.f;
  int status = 0;
  for (;;) {
    const bool res_step = step > 0 && ((step - 1) % kUpdateFreq) == 0;
    if (res_step) {
      double part = 0.0;
      for (int i = tid; i < NF; i += kThreadsMixed) {
        float a0, a1, a2;
        gather_f32(r, i, a0, a1, a2);
        part += static_cast<double>(a0) * a0 + static_cast<double>(a1) * a1 +
                static_cast<double>(a2) * a2;
      }
      residual = sqrt(block_sum<kThreadsMixed>(part, red));
      if (!isfinite(residual)) {
        status = 4;
        break;
      }
    }
    if (!ramp && res_step && !(residual > d.tol)) break;
    if (step >= cap) break;
    const double hd = d.crit * dt_crit * 0.5;
    const float h = static_cast<float>(hd);
    const float hk = h_prev + h;  // trailing kick of step-1 + leading kick of step
    const float h2 = static_cast<float>(2.0 * hd);
    for (int i = tid; i < NF; i += kThreadsMixed) {
      float a0, a1, a2;
      gather_f32(r, i, a0, a1, a2);
      const float mi = r.minv[i];
      const float mc = r.m32[i] * c;
      float w0 = r.v0[i], w1 = r.v1[i], w2 = r.v2[i];
      const float f0 = -a0 - mc * w0;
      const float f1 = -a1 - mc * w1;
      const float f2 = -a2 - mc * w2;
      w0 = fmaf(hk * mi, f0, w0);
      w1 = fmaf(hk * mi, f1, w1);
      w2 = fmaf(hk * mi, f2, w2);
      r.v0[i] = w0; r.v1[i] = w1; r.v2[i] = w2;
      float hi, lo;
      hi = r.h0[i]; lo = r.lo0[i]; comp_add(hi, lo, h2 * w0); r.h0[i] = hi; r.lo0[i] = lo;
      hi = r.h1[i]; lo = r.lo1[i]; comp_add(hi, lo, h2 * w1); r.h1[i] = hi; r.lo1[i] = lo;
      hi = r.h2[i]; lo = r.lo2[i]; comp_add(hi, lo, h2 * w2); r.h2[i] = hi; r.lo2[i] = lo;
    }
    if (ramp) {
      const double alpha = static_cast<double>(step + 1) / static_cast<double>(d.max_steps);
      for (int i = NF + tid; i < N; i += kThreadsMixed) {
        const double* rb = r.ramp + 6 * (i - NF);
        float hi, lo;
        split((rb[0] + alpha * rb[3]) - r.X0[i], hi, lo); r.h0[i] = hi; r.lo0[i] = lo;
        split((rb[1] + alpha * rb[4]) - r.X1[i], hi, lo); r.h1[i] = hi; r.lo1[i] = lo;
        split((rb[2] + alpha * rb[5]) - r.X2[i], hi, lo); r.h2[i] = hi; r.lo2[i] = lo;
      }
    }
    __syncthreads();
    const bool dt_step = (step % kUpdateFreq) == 0;
    const double lmin = fiber_pass_mixed(r, d, L, dt_step);
    if (dt_step) {
      dt_crit = block_min<kThreadsMixed>(lmin, red) / d.sound_speed;
    } else {
      __syncthreads();
    }
    h_prev = h;
    ++step;
  }
  if (status == 0 && !ramp && residual > d.tol) status = 3;

  // ---- finalize: FP64 positions, boundary f_int, stress ---------------------
  for (int i = tid; i < N; i += kThreadsMixed) {
    const double X0 = r.X0[i], X1 = r.X1[i], X2 = r.X2[i];
    const double x0 = X0 + (static_cast<double>(r.h0[i]) + r.lo0[i]);
    const double x1 = X1 + (static_cast<double>(r.h1[i]) + r.lo1[i]);
    const double x2 = X2 + (static_cast<double>(r.h2[i]) + r.lo2[i]);
    r.x0[i] = x0; r.x1[i] = x1; r.x2[i] = x2;
    if (a.update_coords) {
      r.u0[i] = x0 - X0; r.u1[i] = x1 - X1; r.u2[i] = x2 - X2;
    }
    if (i >= NF) {
      float a0, a1, a2;
      gather_f32(r, i, a0, a1, a2);
      r.fi0[i] = a0; r.fi1[i] = a1; r.fi2[i] = a2;
    }
  }
  __syncthreads();
  if (tid < 6) {
    double s = 0.0;
    const int k = tid;
    for (int i = NF; i < N; ++i) {
      const double f1 = r.fi0[i], f2 = r.fi1[i], f3 = r.fi2[i];
      const double crd1 = r.x0[i], crd2 = r.x1[i], crd3 = r.x2[i];
      double t;
      switch (k) {
        case 0: t = crd1 * f1; break;
        case 1: t = crd2 * f2; break;
        case 2: t = crd3 * f3; break;
        case 3: t = 0.5 * (crd2 * f3 + crd3 * f2); break;
        case 4: t = 0.5 * (crd1 * f3 + crd3 * f1); break;
        default: t = 0.5 * (crd1 * f2 + crd2 * f1); break;
      }
      s += t;
    }
    s *= d.scale / b.vol[rve];
    a.sigma[6 * rve + k] = s;
    if (a.update_coords) b.cur_stress[6 * rve + k] = s;
    if (!isfinite(s)) status = 4;
  }
  const unsigned bad = __ballot_sync(0xffffffffu, tid < 32 && status == 4);
  if (tid == 0) {
    a.st_status[rve] = bad ? 4 : status;
    a.st_steps[rve] = step;
    a.st_residual[rve] = residual;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kThreadsMixed) relax_mixed_kernel(const DevBatch b,
                                                                    const MixedState ms,
                                                                    const RunArgs a) {
  __shared__ double red[kThreadsMixed / 32 + 1];
  __shared__ int s_rve;
  for (;;) {
    if (threadIdx.x == 0) {
      const int w = atomicAdd(b.queue, 1);
      s_rve = w < b.n_rve ? b.order[w] : -1;
    }
    __syncthreads();
    const int rve = s_rve;
    __syncthreads();
    if (rve < 0) break;
    solve_rve_mixed(b, ms, a, rve, red);
  }
}

template <typename T>
cudaError_t alloc(T** p, size_t n) {
  return cudaMalloc(reinterpret_cast<void**>(p), (n > 0 ? n : 1) * sizeof(T));
}

}  // namespace

MixedState* mixed_new() { return new MixedState(); }

void mixed_destroy(MixedState* ms) {
  if (!ms) return;
  for (float* p : {ms->u_hi, ms->u_lo, ms->v, ms->minv, ms->m32, ms->dX, ms->rl0, ms->nrm})
    if (p) cudaFree(p);
  delete ms;
}

cudaError_t mixed_create(MixedState& ms, const DevBatch& b, const std::vector<RveDesc>& desc,
                         int sms, cudaStream_t s) {
  cudaError_t e;
  const size_t nt = static_cast<size_t>(b.nt), et = static_cast<size_t>(b.et);
  if ((e = alloc(&ms.u_hi, 3 * nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.u_lo, 3 * nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.v, 3 * nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.minv, nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.m32, nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.dX, 3 * et)) != cudaSuccess) return e;
  if ((e = alloc(&ms.rl0, et)) != cudaSuccess) return e;
  if ((e = alloc(&ms.nrm, 3 * et)) != cudaSuccess) return e;
  ms.sms = sms;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, relax_mixed_kernel, kThreadsMixed, 0) !=
          cudaSuccess ||
      occ < 1)
    occ = 1;
  ms.occ = occ;
  const int64_t n = std::max<int64_t>(b.nt, 1);
  mixed_prepare_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(b, ms);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  int max_e = 1;
  for (const RveDesc& d : desc) max_e = std::max(max_e, d.n_fibers);
  dim3 grid(static_cast<unsigned>((max_e + 255) / 256),
            static_cast<unsigned>(std::min(b.n_rve, 65535)));
  mixed_prepare_fibers_kernel<<<grid, 256, 0, s>>>(b, ms);
  return cudaGetLastError();
}

cudaError_t run_mixed(MixedState& ms, const DevBatch& b, const RunArgs& a, cudaStream_t s,
                      int* launches) {
  const int grid = std::min(b.n_rve, ms.sms * ms.occ);
  relax_mixed_kernel<<<grid, kThreadsMixed, 0, s>>>(b, ms, a);
  *launches = 1;
  return cudaGetLastError();
}

}  // namespace mfg
