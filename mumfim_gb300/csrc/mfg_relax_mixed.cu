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
//  - the RAMP boundary moves by an exact FP32 (hi, lo) per-step increment,
//    accumulated with TwoSum: recomputing u0 + alpha d in FP32 every step
//    jitters boundary nodes by ~ulp(d), which the very short fibers kNN
//    networks attach to the boundary turn into large strain noise;
//  - velocities, the damping force and both kicks are FP32;
//  - FP64 is kept for the critical time step (FP64 lengths every 100 steps),
//    the residual norm, and the stress homogenisation, exactly where the
//    reference reduces over the whole RVE.
// The persistent FP64 state of the batch (x, u, volume) is read at the
// start and written at the end of every run, so both precisions share it.
//
// Memory placement, chosen per RVE inside one persistent launch (one CTA of
// 512 threads per SM, up to 220 KB of dynamic shared memory):
//   RESIDENT_ALL  u_hi, u_lo (24 B/node) and the per-fiber force vectors
//                 (16 B/fiber) live in shared memory for the whole solve;
//   RESIDENT_NODE only u_hi, u_lo in shared memory, force vectors in global;
//   STREAM        everything in global memory (L2 / HBM).
// Per-fiber constants (end nodes, reference vector dX, 1/l0) and per-node
// constants / velocities always stream from global with coalesced loads.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "mfg_common.cuh"
#include "mfg_internal.h"
#include "mfg_mixed.h"

namespace mfg {

struct MixedState {
  float* u_hi = nullptr;   // 3 * nt (STREAM placement)
  float* u_lo = nullptr;   // 3 * nt
  float4* v = nullptr;     // nt, velocity (w unused)
  float2* mass = nullptr;  // nt, (1 / m, m)
  float4* fcon = nullptr;  // et, (X[n2] - X[n1], 1 / l0) rounded to FP32
  float4* nrm = nullptr;   // et, per-fiber force vectors (scratch; w unused)
  int sms = 1;
  int smem_bytes = 0;
};

namespace {

constexpr int kThreadsMixed = 1024;
constexpr int kSmemBytesMixed = 220 * 1024;

__global__ void mixed_prepare_kernel(const DevBatch b, MixedState ms) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i < b.nt) {
    const double m = b.m[i];
    ms.mass[i] = make_float2(static_cast<float>(1.0 / m), static_cast<float>(m));
  }
}

__global__ void mixed_prepare_fibers_kernel(const DevBatch b, MixedState ms) {
  for (int rve = blockIdx.y; rve < b.n_rve; rve += gridDim.y) {
    const RveDesc d = b.desc[rve];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.n_fibers) continue;
    const int64_t fo = d.fiber_off + e, no = d.node_off;
    const int2 c = b.conn[fo];
    float dx[3];
    for (int k = 0; k < 3; ++k) {
      const double* X = b.X + k * b.nt + no;
      dx[k] = static_cast<float>(X[c.y] - X[c.x]);
    }
    ms.fcon[fo] = make_float4(dx[0], dx[1], dx[2], static_cast<float>(1.0 / b.l0[fo]));
  }
}

// Per-RVE constants of the fiber law in the T/l form used here.
struct Law {
  int nonlinear;
  float ea;      // E A
  float ea_b;    // alpha = E A / B (toe: T/l = alpha expm1(B g) / l0)
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

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bp = s - a;
  const float ap = s - bp;
  e = (a - ap) + (b - bp);
}

__device__ __forceinline__ void split(double u, float& hi, float& lo) {
  hi = static_cast<float>(u);
  lo = static_cast<float>(u - static_cast<double>(hi));
}

// A three-component float field: component k of node i at c[k][i].
struct Field3 {
  float* c[3];
  __device__ __forceinline__ void set(float* base, int64_t stride) {
    c[0] = base;
    c[1] = base + stride;
    c[2] = base + 2 * stride;
  }
  __device__ __forceinline__ float& operator()(int k, int i) const { return c[k][i]; }
};

struct Rve {
  RveDesc d;
  Law L;
  Field3 hi, lo;        // node displacement (hi, lo)
  float4* n;            // fiber force vectors
  float4* v;            // node velocity (global)
  const float2* mass;   // (1 / m, m)
  const float4* fcon;   // (dX, 1 / l0)
  const int2* conn;
  const int32_t* rowptr;
  const int32_t* inc;
  float* ramp;          // per boundary node: step increment d/n as (hi[3], lo[3])
  int64_t node_off, nt;
};

// Nodal internal force: incident fiber vectors in the node's CSR order,
// subtracted at a fiber's first end and added at its second.
__device__ __forceinline__ void gather(const Rve& r, int i, float& a0, float& a1, float& a2) {
  a0 = 0.f; a1 = 0.f; a2 = 0.f;
  const int pb = __ldg(r.rowptr + i), pe = __ldg(r.rowptr + i + 1);
  for (int p = pb; p < pe; ++p) {
    const int code = __ldg(r.inc + p);
    const float4 t = r.n[code >> 1];
    const float sg = (code & 1) ? 1.f : -1.f;
    a0 = fmaf(sg, t.x, a0);
    a1 = fmaf(sg, t.y, a1);
    a2 = fmaf(sg, t.z, a2);
  }
}

// Force vector of one fiber. The displacement difference du is formed with a
// TwoSum of the hi parts plus the lo parts, so it is accurate to FP32 of du
// itself; the Green strain follows from du (g l0^2 = du.(dX + du/2)), which
// keeps its relative precision at small strain where 0.5(l^2/l0^2 - 1)
// would cancel.
__device__ __forceinline__ void fiber_force(const Rve& r, int e) {
  const int2 c = __ldg(r.conn + e);
  float du[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float d, ed;
    two_sum(r.hi(k, c.y), -r.hi(k, c.x), d, ed);
    du[k] = d + (ed + (r.lo(k, c.y) - r.lo(k, c.x)));
  }
  const float4 fc = __ldg(r.fcon + e);
  const float gn = fmaf(du[0], fmaf(0.5f, du[0], fc.x),
                        fmaf(du[1], fmaf(0.5f, du[1], fc.y), du[2] * fmaf(0.5f, du[2], fc.z)));
  const float g = gn * (fc.w * fc.w);
  const float t = tension_over_length(r.L, g, fc.w);
  r.n[e] = make_float4((fc.x + du[0]) * t, (fc.y + du[1]) * t, (fc.z + du[2]) * t, 0.f);
}

// FP64 length of one fiber in the current configuration.
__device__ __forceinline__ double length64(const Rve& r, const double* X, int e) {
  const int2 c = __ldg(r.conn + e);
  double s2 = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double* Xk = X + k * r.nt + r.node_off;
    const double a = Xk[c.x] + (static_cast<double>(r.hi(k, c.x)) + r.lo(k, c.x));
    const double bq = Xk[c.y] + (static_cast<double>(r.hi(k, c.y)) + r.lo(k, c.y));
    s2 += (bq - a) * (bq - a);
  }
  return sqrt(s2);
}

__device__ void solve_rve_mixed(const DevBatch& b, const MixedState& ms, const RunArgs& a, int rve,
                                double* red, float* smem, int smem_floats) {
  Rve r;
  r.d = b.desc[rve];
  const RveDesc& d = r.d;
  r.L = make_law(d);
  const int N = d.n_nodes, NF = d.n_free, E = d.n_fibers;
  const int tid = threadIdx.x;
  const int64_t no = d.node_off, fo = d.fiber_off, nt = b.nt, et = b.et;
  r.node_off = no;
  r.nt = nt;
  // placement
  // force vectors first (16-byte aligned), then the node fields
  const int64_t node_floats = 6LL * N, all_floats = 6LL * N + 4LL * E;
  if (all_floats <= smem_floats) {
    r.n = reinterpret_cast<float4*>(smem);
    r.hi.set(smem + 4 * E, N);
    r.lo.set(smem + 4 * E + 3 * N, N);
  } else if (node_floats <= smem_floats) {
    r.n = ms.nrm + fo;
    r.hi.set(smem, N);
    r.lo.set(smem + 3 * N, N);
  } else {
    r.n = ms.nrm + fo;
    r.hi.set(ms.u_hi + no, nt);
    r.lo.set(ms.u_lo + no, nt);
  }
  (void)et;
  r.v = ms.v + no;
  r.mass = ms.mass + no;
  r.fcon = ms.fcon + fo;
  r.conn = b.conn + fo;
  r.rowptr = b.rowptr + d.row_off;
  r.inc = b.inc + d.inc_off;
  r.ramp = reinterpret_cast<float*>(b.ramp + 6 * d.bnd_off);  // 12 floats per boundary node
  const double* F = a.F + 9 * (a.n_F > 1 ? rve : 0);
  const bool ramp = d.mode == 1;
  double Fm[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Fm[k] = F[k];
  if (a.update_coords && tid == 0) b.vol[rve] = jacobian(Fm) * b.vol[rve];

  // ---- prologue in FP64: predictor, split into (hi, lo), v = 0 -------------
  for (int i = tid; i < N; i += kThreadsMixed) {
    double xo[3], up[3], X[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      xo[k] = b.x[k * nt + no + i];
      up[k] = b.u[k * nt + no + i];
      X[k] = b.X[k * nt + no + i];
    }
    if (!ramp) {
      const double u0 = (Fm[0] - 1) * xo[0] + Fm[1] * xo[1] + Fm[2] * xo[2] + up[0];
      const double u1 = Fm[3] * xo[0] + (Fm[4] - 1) * xo[1] + Fm[5] * xo[2] + up[1];
      const double u2 = Fm[6] * xo[0] + Fm[7] * xo[1] + (Fm[8] - 1) * xo[2] + up[2];
      up[0] = u0; up[1] = u1; up[2] = u2;
    }
    double xn[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      xn[k] = X[k] + up[k];
      float hi, lo;
      split(xn[k] - X[k], hi, lo);
      r.hi(k, i) = hi;
      r.lo(k, i) = lo;
    }
    r.v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ramp && i >= NF) {
      // The boundary moves by d/n per step, d = (F - I) x0. The increment is
      // kept as an exact FP32 pair and accumulated without rounding into
      // (hi, lo): recomputing u0 + alpha d in FP32 every step would jitter
      // the boundary by ~ulp(d) per step, i.e. a large strain noise on the
      // very short fibers that kNN networks attach to the boundary.
      float* rb = r.ramp + 12 * (i - NF);
      const double inv_n = 1.0 / static_cast<double>(d.max_steps);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double inc = ((Fm[3 * k + 0] - (k == 0)) * xn[0] + (Fm[3 * k + 1] - (k == 1)) * xn[1] +
                            (Fm[3 * k + 2] - (k == 2)) * xn[2]) * inv_n;
        const float ih = static_cast<float>(inc);
        rb[k] = ih;
        rb[3 + k] = static_cast<float>(inc - static_cast<double>(ih));
      }
    }
  }
  __syncthreads();
  double lmin = DBL_MAX;
  for (int e = tid; e < E; e += kThreadsMixed) {
    fiber_force(r, e);
    lmin = fmin(lmin, length64(r, b.X, e));
  }
  double dt_crit = block_min<kThreadsMixed>(lmin, red) / d.sound_speed;

  const int cap = d.max_steps;
  const float c = static_cast<float>(d.c);
  float h_cur = static_cast<float>(d.crit * dt_crit * 0.5);
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
        gather(r, i, a0, a1, a2);
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
    // per-step scalars in FP32 (h changes only when dt_crit does)
    const float h = h_cur;
    const float hk = h_prev + h;  // trailing kick of step-1 + leading kick of step
    const float h2 = h + h;
    for (int i = tid; i < NF; i += kThreadsMixed) {
      float f[3];
      gather(r, i, f[0], f[1], f[2]);
      const float2 mm = __ldg(r.mass + i);
      const float mc = mm.y * c;
      const float km = hk * mm.x;
      float4 w = r.v[i];
      w.x = fmaf(km, -f[0] - mc * w.x, w.x);
      w.y = fmaf(km, -f[1] - mc * w.y, w.y);
      w.z = fmaf(km, -f[2] - mc * w.z, w.z);
      r.v[i] = w;
      const float wk[3] = {w.x, w.y, w.z};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        float hi = r.hi(k, i), lo = r.lo(k, i);
        comp_add(hi, lo, h2 * wk[k]);
        r.hi(k, i) = hi;
        r.lo(k, i) = lo;
      }
    }
    if (ramp) {
      for (int i = NF + tid; i < N; i += kThreadsMixed) {
        const float* rb = r.ramp + 12 * (i - NF);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          float s, e;
          two_sum(r.hi(k, i), rb[k], s, e);
          r.hi(k, i) = s;
          r.lo(k, i) = r.lo(k, i) + (e + rb[3 + k]);
        }
      }
    }
    __syncthreads();
    const bool dt_step = (step % kUpdateFreq) == 0;
    if (dt_step) {
      double lm = DBL_MAX;
      for (int e = tid; e < E; e += kThreadsMixed) {
        fiber_force(r, e);
        lm = fmin(lm, length64(r, b.X, e));
      }
      dt_crit = block_min<kThreadsMixed>(lm, red) / d.sound_speed;
      h_cur = static_cast<float>(d.crit * dt_crit * 0.5);
    } else {
      int e = tid;
      for (; e + kThreadsMixed < E; e += 2 * kThreadsMixed) {
        fiber_force(r, e);
        fiber_force(r, e + kThreadsMixed);
      }
      if (e < E) fiber_force(r, e);
      __syncthreads();
    }
    h_prev = h;
    ++step;
  }
  if (status == 0 && !ramp && residual > d.tol) status = 3;

  // ---- finalize: FP64 positions, boundary f_int, stress ---------------------
  for (int i = tid; i < N; i += kThreadsMixed) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double Xk = b.X[k * nt + no + i];
      const double xk = Xk + (static_cast<double>(r.hi(k, i)) + r.lo(k, i));
      b.x[k * nt + no + i] = xk;
      if (a.update_coords) b.u[k * nt + no + i] = xk - Xk;
    }
    if (i >= NF) {
      float a0, a1, a2;
      gather(r, i, a0, a1, a2);
      b.fint[no + i] = a0;
      b.fint[nt + no + i] = a1;
      b.fint[2 * nt + no + i] = a2;
    }
  }
  __syncthreads();
  if (tid < 6) {
    double s = 0.0;
    const int k = tid;
    const int32_t* bo = b.bnd + d.bnd_off;
    const double* x0 = b.x + no;
    const double* x1 = b.x + nt + no;
    const double* x2 = b.x + 2 * nt + no;
    for (int q = 0; q < N - NF; ++q) {
      const int i = bo[q];
      const double f1 = b.fint[no + i], f2 = b.fint[nt + no + i], f3 = b.fint[2 * nt + no + i];
      const double crd1 = x0[i], crd2 = x1[i], crd3 = x2[i];
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

__global__ void __launch_bounds__(kThreadsMixed, 1)
relax_mixed_kernel(const DevBatch b, const MixedState ms, const RunArgs a, int smem_floats) {
  extern __shared__ float smem[];
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
    solve_rve_mixed(b, ms, a, rve, red, smem, smem_floats);
  }
}

__global__ void __launch_bounds__(kThreadsMixed, 1)
server_mixed_kernel(const DevBatch b, const MixedState ms, const ServerArgs sa, int smem_floats) {
  extern __shared__ float smem[];
  __shared__ double red[kThreadsMixed / 32 + 1];
  server_loop(sa, [&](const RunArgs& a, int rve) {
    solve_rve_mixed(b, ms, a, rve, red, smem, smem_floats);
  });
}

template <typename T>
cudaError_t alloc(T** p, size_t n) {
  return cudaMalloc(reinterpret_cast<void**>(p), (n > 0 ? n : 1) * sizeof(T));
}

}  // namespace

MixedState* mixed_new() { return new MixedState(); }

void mixed_destroy(MixedState* ms) {
  if (!ms) return;
  for (void* p : {static_cast<void*>(ms->u_hi), static_cast<void*>(ms->u_lo),
                  static_cast<void*>(ms->v), static_cast<void*>(ms->mass),
                  static_cast<void*>(ms->fcon), static_cast<void*>(ms->nrm)})
    if (p) cudaFree(p);
  delete ms;
}

cudaError_t mixed_create(MixedState& ms, const DevBatch& b, const std::vector<RveDesc>& desc,
                         int sms, cudaStream_t s) {
  cudaError_t e;
  const size_t nt = static_cast<size_t>(b.nt), et = static_cast<size_t>(b.et);
  if ((e = alloc(&ms.u_hi, 3 * nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.u_lo, 3 * nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.v, nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.mass, nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.fcon, et)) != cudaSuccess) return e;
  if ((e = alloc(&ms.nrm, et)) != cudaSuccess) return e;
  ms.sms = sms;
  ms.smem_bytes = kSmemBytesMixed;
  if ((e = cudaFuncSetAttribute(relax_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                kSmemBytesMixed)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(server_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                kSmemBytesMixed)) != cudaSuccess)
    return e;
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

cudaError_t launch_server_mixed(MixedState& ms, const DevBatch& b, const ServerArgs& sa,
                                cudaStream_t s) {
  server_mixed_kernel<<<ms.sms, kThreadsMixed, ms.smem_bytes, s>>>(b, ms, sa,
                                                                   ms.smem_bytes / sizeof(float));
  return cudaGetLastError();
}

cudaError_t run_mixed(MixedState& ms, const DevBatch& b, const RunArgs& a, cudaStream_t s,
                      int* launches) {
  const int grid = std::min(b.n_rve, ms.sms);
  relax_mixed_kernel<<<grid, kThreadsMixed, ms.smem_bytes, s>>>(b, ms, a,
                                                               ms.smem_bytes / sizeof(float));
  *launches = 1;
  return cudaGetLastError();
}

}  // namespace mfg
