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
#include <type_traits>
#include <vector>

#include <cooperative_groups.h>

#include "mfg_common.cuh"
#include "mfg_internal.h"
#include "mfg_mixed.h"

namespace cg = cooperative_groups;

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
  // Size buckets of the batch run: bucket q is solved by clusters of
  // kClusterSizes[q] CTAs; its RVEs, most fibers first, are
  // order[bucket_off[q] .. bucket_off[q + 1]).
  int32_t* order = nullptr;
  int32_t* queues = nullptr;  // one claim counter per bucket
  int bucket_off[5] = {0, 0, 0, 0, 0};
  int bucket_grid[4] = {0, 0, 0, 0};
  cudaStream_t side[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[4] = {nullptr, nullptr, nullptr, nullptr};
};

namespace {

constexpr int kThreadsMixed = 1024;
constexpr int kSmemBytesMixed = 220 * 1024;
constexpr int kClusterSizes[4] = {8, 4, 2, 1};

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

// Node displacement (hi, lo) of an RVE solved by one CTA: in its shared
// memory (resident placements) or in global memory (streaming placement).
// Also the view a CTA of a cluster has of the nodes it owns, by local index.
struct LocalNodes {
  Field3 h, l;
  __device__ __forceinline__ float& hi(int k, int j) const { return h(k, j); }
  __device__ __forceinline__ float& lo(int k, int j) const { return l(k, j); }
  __device__ __forceinline__ void load(int j, float (&uh)[3], float (&ul)[3]) const {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      uh[k] = h(k, j);
      ul[k] = l(k, j);
    }
  }
};

// Node displacement of an RVE split over the CL CTAs of a thread-block
// cluster, read through distributed shared memory: CTA o holds nodes
// [o*chunk, (o+1)*chunk) as six blocks of `chunk` floats (hi x, y, z, lo x,
// y, z) at the same shared-memory offset `base` in every CTA.
template <int CL>
struct ClusterNodes {
  uint32_t base;  // shared-window address of this CTA's block
  int chunk;
  __device__ __forceinline__ void load(int j, float (&uh)[3], float (&ul)[3]) const {
    int o = 0;
#pragma unroll
    for (int q = 1; q < CL; ++q) o += (j >= q * chunk) ? 1 : 0;
    const uint32_t local = base + 4u * static_cast<uint32_t>(j - o * chunk);
    uint32_t remote;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(o));
    const uint32_t stride = 4u * static_cast<uint32_t>(chunk);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(uh[k]) : "r"(remote + k * stride));
      asm volatile("ld.shared::cluster.f32 %0, [%1];"
                   : "=f"(ul[k])
                   : "r"(remote + (3 + k) * stride));
    }
  }
};

template <int CL>
struct ClusterOps {
  __device__ static int rank() {
    if constexpr (CL > 1) return static_cast<int>(cg::this_cluster().block_rank());
    return 0;
  }
  // Block barrier, or cluster barrier (release / acquire at cluster scope,
  // which also orders the global-memory force vectors between CTAs).
  __device__ static void sync() {
    if constexpr (CL > 1)
      cg::this_cluster().sync();
    else
      __syncthreads();
  }
  // Combines a block-reduced value over the cluster in fixed rank order, so
  // every CTA gets the same bits.
  template <bool kMin>
  __device__ static double combine(double part, double* slot) {
    if constexpr (CL == 1) {
      return part;
    } else {
      cg::cluster_group cl = cg::this_cluster();
      if (threadIdx.x == 0) *slot = part;
      cl.sync();
      double t = kMin ? DBL_MAX : 0.0;
#pragma unroll
      for (int o = 0; o < CL; ++o) {
        const double v = *cl.map_shared_rank(slot, o);
        t = kMin ? fmin(t, v) : t + v;
      }
      cl.sync();
      return t;
    }
  }
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
template <class Nodes>
__device__ __forceinline__ void fiber_force(const Rve& r, const Nodes& u, int e) {
  const int2 c = __ldg(r.conn + e);
  float ah[3], al[3], bh[3], bl[3];
  u.load(c.x, ah, al);
  u.load(c.y, bh, bl);
  float du[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float d, ed;
    two_sum(bh[k], -ah[k], d, ed);
    du[k] = d + (ed + (bl[k] - al[k]));
  }
  const float4 fc = __ldg(r.fcon + e);
  const float gn = fmaf(du[0], fmaf(0.5f, du[0], fc.x),
                        fmaf(du[1], fmaf(0.5f, du[1], fc.y), du[2] * fmaf(0.5f, du[2], fc.z)));
  const float g = gn * (fc.w * fc.w);
  const float t = tension_over_length(r.L, g, fc.w);
  r.n[e] = make_float4((fc.x + du[0]) * t, (fc.y + du[1]) * t, (fc.z + du[2]) * t, 0.f);
}

// FP64 length of one fiber in the current configuration.
template <class Nodes>
__device__ __forceinline__ double length64(const Rve& r, const Nodes& u, const double* X, int e) {
  const int2 c = __ldg(r.conn + e);
  float ah[3], al[3], bh[3], bl[3];
  u.load(c.x, ah, al);
  u.load(c.y, bh, bl);
  double s2 = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double* Xk = X + k * r.nt + r.node_off;
    const double a = Xk[c.x] + (static_cast<double>(ah[k]) + al[k]);
    const double bq = Xk[c.y] + (static_cast<double>(bh[k]) + bl[k]);
    s2 += (bq - a) * (bq - a);
  }
  return sqrt(s2);
}

// One RVE solved by one CTA (CL = 1) or by the CL CTAs of a cluster, each
// owning a contiguous range of nodes (storage order is Morton-sorted, so a
// range is a compact region of the RVE) and a range of fiber slots.
template <int CL>
__device__ void solve_rve_mixed(const DevBatch& b, const MixedState& ms, const RunArgs& a, int rve,
                                double* red, double* cred, float* smem, int smem_floats) {
  using Ops = ClusterOps<CL>;
  Rve r;
  r.d = b.desc[rve];
  const RveDesc& d = r.d;
  r.L = make_law(d);
  const int N = d.n_nodes, NF = d.n_free, E = d.n_fibers;
  const int tid = threadIdx.x;
  const int64_t no = d.node_off, fo = d.fiber_off, nt = b.nt;
  r.node_off = no;
  r.nt = nt;
  const int rank = Ops::rank();
  const int chunk = (N + CL - 1) / CL;
  const int n_lo = CL > 1 ? min(N, rank * chunk) : 0;
  const int n_hi = CL > 1 ? min(N, n_lo + chunk) : N;
  const int e_lo = static_cast<int>(static_cast<int64_t>(E) * rank / CL);
  const int e_hi = static_cast<int>(static_cast<int64_t>(E) * (rank + 1) / CL);
  using Nodes = std::conditional_t<(CL > 1), ClusterNodes<CL>, LocalNodes>;
  Nodes u;        // every node of the RVE (fiber pass)
  LocalNodes own;  // the nodes this CTA updates, by index - n_lo
  if constexpr (CL > 1) {
    r.n = ms.nrm + fo;
    u.chunk = chunk;
    u.base = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
    own.h.set(smem, chunk);
    own.l.set(smem + 3 * chunk, chunk);
  } else {
    // placement: force vectors first (16-byte aligned), then the node fields
    const int64_t node_floats = 6LL * N, all_floats = 6LL * N + 4LL * E;
    if (all_floats <= smem_floats) {
      r.n = reinterpret_cast<float4*>(smem);
      own.h.set(smem + 4 * E, N);
      own.l.set(smem + 4 * E + 3 * N, N);
    } else if (node_floats <= smem_floats) {
      r.n = ms.nrm + fo;
      own.h.set(smem, N);
      own.l.set(smem + 3 * N, N);
    } else {
      r.n = ms.nrm + fo;
      own.h.set(ms.u_hi + no, nt);
      own.l.set(ms.u_lo + no, nt);
    }
    u = own;
  }
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
  if (a.update_coords && rank == 0 && tid == 0) b.vol[rve] = jacobian(Fm) * b.vol[rve];

  // ---- prologue in FP64: predictor, split into (hi, lo), v = 0 -------------
  for (int i = n_lo + tid; i < n_hi; i += kThreadsMixed) {
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
      own.hi(k, i - n_lo) = hi;
      own.lo(k, i - n_lo) = lo;
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
  Ops::sync();
  double lmin = DBL_MAX;
  for (int e = e_lo + tid; e < e_hi; e += kThreadsMixed) {
    fiber_force(r, u, e);
    lmin = fmin(lmin, length64(r, u, b.X, e));
  }
  double dt_crit =
      Ops::template combine<true>(block_min<kThreadsMixed>(lmin, red), cred) / d.sound_speed;

  const int cap = d.max_steps;
  const float c = static_cast<float>(d.c);
  float h_cur = static_cast<float>(d.crit * dt_crit * 0.5);
  const int f_hi = min(n_hi, NF);  // own free nodes [n_lo, f_hi)
  const int b_lo = max(n_lo, NF);  // own boundary nodes [b_lo, n_hi)
  int step = 0;
  double residual = 10.0;
  float h_prev = 0.f;
  int status = 0;
  for (;;) {
    const bool res_step = step > 0 && ((step - 1) % kUpdateFreq) == 0;
    if (res_step) {
      double part = 0.0;
      for (int i = n_lo + tid; i < f_hi; i += kThreadsMixed) {
        float a0, a1, a2;
        gather(r, i, a0, a1, a2);
        part += static_cast<double>(a0) * a0 + static_cast<double>(a1) * a1 +
                static_cast<double>(a2) * a2;
      }
      residual = sqrt(Ops::template combine<false>(block_sum<kThreadsMixed>(part, red), cred));
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
    for (int i = n_lo + tid; i < f_hi; i += kThreadsMixed) {
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
        float hi = own.hi(k, i - n_lo), lo = own.lo(k, i - n_lo);
        comp_add(hi, lo, h2 * wk[k]);
        own.hi(k, i - n_lo) = hi;
        own.lo(k, i - n_lo) = lo;
      }
    }
    if (ramp) {
      for (int i = b_lo + tid; i < n_hi; i += kThreadsMixed) {
        const float* rb = r.ramp + 12 * (i - NF);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          float s, e;
          two_sum(own.hi(k, i - n_lo), rb[k], s, e);
          own.hi(k, i - n_lo) = s;
          own.lo(k, i - n_lo) = own.lo(k, i - n_lo) + (e + rb[3 + k]);
        }
      }
    }
    Ops::sync();
    const bool dt_step = (step % kUpdateFreq) == 0;
    if (dt_step) {
      double lm = DBL_MAX;
      for (int e = e_lo + tid; e < e_hi; e += kThreadsMixed) {
        fiber_force(r, u, e);
        lm = fmin(lm, length64(r, u, b.X, e));
      }
      dt_crit =
          Ops::template combine<true>(block_min<kThreadsMixed>(lm, red), cred) / d.sound_speed;
      h_cur = static_cast<float>(d.crit * dt_crit * 0.5);
    } else {
      int e = e_lo + tid;
      for (; e + kThreadsMixed < e_hi; e += 2 * kThreadsMixed) {
        fiber_force(r, u, e);
        fiber_force(r, u, e + kThreadsMixed);
      }
      if (e < e_hi) fiber_force(r, u, e);
      Ops::sync();
    }
    h_prev = h;
    ++step;
  }
  if (status == 0 && !ramp && residual > d.tol) status = 3;

  // ---- finalize: FP64 positions, boundary f_int, stress ---------------------
  for (int i = n_lo + tid; i < n_hi; i += kThreadsMixed) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double Xk = b.X[k * nt + no + i];
      const double xk = Xk + (static_cast<double>(own.hi(k, i - n_lo)) + own.lo(k, i - n_lo));
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
  Ops::sync();
  if (rank == 0 && tid < 6) {
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
  if (rank == 0 && tid == 0) {
    a.st_status[rve] = bad ? 4 : status;
    a.st_steps[rve] = step;
    a.st_residual[rve] = residual;
  }
  Ops::sync();
}

// Persistent relaxation over one size bucket: CTA (or cluster) after cluster
// takes the next RVE of `order` (largest first) until the bucket is empty.
template <int CL>
__global__ void __launch_bounds__(kThreadsMixed, 1)
relax_mixed_kernel(const DevBatch b, const MixedState ms, const RunArgs a, int smem_floats,
                   const int32_t* order, int n_order, int32_t* queue) {
  extern __shared__ float smem[];
  __shared__ double red[kThreadsMixed / 32 + 1];
  __shared__ double cred[1];
  __shared__ int s_rve;
  for (;;) {
    if (ClusterOps<CL>::rank() == 0 && threadIdx.x == 0) {
      const int w = atomicAdd(queue, 1);
      s_rve = w < n_order ? order[w] : -1;
    }
    int rve;
    if constexpr (CL > 1) {
      cg::cluster_group cl = cg::this_cluster();
      cl.sync();
      rve = *cl.map_shared_rank(&s_rve, 0);
      cl.sync();
    } else {
      __syncthreads();
      rve = s_rve;
      __syncthreads();
    }
    if (rve < 0) break;
    solve_rve_mixed<CL>(b, ms, a, rve, red, cred, smem, smem_floats);
  }
}

__global__ void __launch_bounds__(kThreadsMixed, 1)
server_mixed_kernel(const DevBatch b, const MixedState ms, const ServerArgs sa, int smem_floats) {
  extern __shared__ float smem[];
  __shared__ double red[kThreadsMixed / 32 + 1];
  __shared__ double cred[1];
  server_loop(sa, [&](const RunArgs& a, int rve) {
    solve_rve_mixed<1>(b, ms, a, rve, red, cred, smem, smem_floats);
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
                  static_cast<void*>(ms->fcon), static_cast<void*>(ms->nrm),
                  static_cast<void*>(ms->order), static_cast<void*>(ms->queues)})
    if (p) cudaFree(p);
  for (int q = 0; q < 4; ++q) {
    if (ms->side[q]) cudaStreamDestroy(ms->side[q]);
    if (ms->join[q]) cudaEventDestroy(ms->join[q]);
  }
  if (ms->fork) cudaEventDestroy(ms->fork);
  delete ms;
}

namespace {

// Bucket of an RVE: the smallest cluster whose CTAs hold its node
// displacements (24 B per node) in shared memory; RVEs too large even for
// the largest cluster are solved by one CTA from global memory.
int bucket_of(const RveDesc& d, int smem_floats) {
  for (int q = 3; q >= 0; --q) {
    const int cl = kClusterSizes[q];
    const int64_t chunk = (static_cast<int64_t>(d.n_nodes) + cl - 1) / cl;
    if (6 * chunk <= smem_floats) return q;
  }
  return 3;
}

template <int CL>
cudaError_t launch_bucket(const MixedState& ms, const DevBatch& b, const RunArgs& a, int q,
                          cudaStream_t s) {
  const int n = ms.bucket_off[q + 1] - ms.bucket_off[q];
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(ms.bucket_grid[q]), 1, 1);
  cfg.blockDim = dim3(kThreadsMixed, 1, 1);
  cfg.dynamicSmemBytes = static_cast<size_t>(ms.smem_bytes);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = CL > 1 ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, relax_mixed_kernel<CL>, b, ms, a,
                            static_cast<int>(ms.smem_bytes / sizeof(float)),
                            static_cast<const int32_t*>(ms.order + ms.bucket_off[q]), n,
                            ms.queues + q);
}

template <int CL>
cudaError_t max_clusters(const MixedState& ms, int* out) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(CL * ms.sms), 1, 1);
  cfg.blockDim = dim3(kThreadsMixed, 1, 1);
  cfg.dynamicSmemBytes = static_cast<size_t>(ms.smem_bytes);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaOccupancyMaxActiveClusters(out, relax_mixed_kernel<CL>, &cfg);
}

}  // namespace

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
  if ((e = alloc(&ms.order, desc.size())) != cudaSuccess) return e;
  if ((e = alloc(&ms.queues, 4)) != cudaSuccess) return e;
  ms.sms = sms;
  ms.smem_bytes = kSmemBytesMixed;
  const int smem_floats = kSmemBytesMixed / static_cast<int>(sizeof(float));
  if ((e = cudaFuncSetAttribute(relax_mixed_kernel<1>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytesMixed)) !=
          cudaSuccess ||
      (e = cudaFuncSetAttribute(relax_mixed_kernel<2>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytesMixed)) !=
          cudaSuccess ||
      (e = cudaFuncSetAttribute(relax_mixed_kernel<4>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytesMixed)) !=
          cudaSuccess ||
      (e = cudaFuncSetAttribute(relax_mixed_kernel<8>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytesMixed)) !=
          cudaSuccess ||
      (e = cudaFuncSetAttribute(server_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                kSmemBytesMixed)) != cudaSuccess)
    return e;

  // size buckets, each in longest-processing-time order
  std::vector<std::vector<int32_t>> bucket(4);
  for (size_t r = 0; r < desc.size(); ++r)
    bucket[bucket_of(desc[r], smem_floats)].push_back(static_cast<int32_t>(r));
  std::vector<int32_t> order;
  order.reserve(desc.size());
  for (int q = 0; q < 4; ++q) {
    std::stable_sort(bucket[q].begin(), bucket[q].end(),
                     [&](int32_t x, int32_t y) { return desc[x].n_fibers > desc[y].n_fibers; });
    ms.bucket_off[q] = static_cast<int>(order.size());
    order.insert(order.end(), bucket[q].begin(), bucket[q].end());
  }
  ms.bucket_off[4] = static_cast<int>(order.size());
  if (!order.empty() &&
      (e = cudaMemcpyAsync(ms.order, order.data(), order.size() * sizeof(int32_t),
                           cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return e;
  for (int q = 0; q < 4; ++q) {
    const int n = ms.bucket_off[q + 1] - ms.bucket_off[q];
    const int cl = kClusterSizes[q];
    int clusters = sms / cl;
    if (n > 0 && cl > 1) {
      clusters = 0;
      switch (cl) {
        case 8: e = max_clusters<8>(ms, &clusters); break;
        case 4: e = max_clusters<4>(ms, &clusters); break;
        default: e = max_clusters<2>(ms, &clusters); break;
      }
      if (e != cudaSuccess) return e;
      if (clusters < 1) return cudaErrorInvalidConfiguration;
    }
    ms.bucket_grid[q] = cl * std::min(n, std::max(clusters, 1));
    if ((e = cudaStreamCreateWithFlags(&ms.side[q], cudaStreamNonBlocking)) != cudaSuccess)
      return e;
    if ((e = cudaEventCreateWithFlags(&ms.join[q], cudaEventDisableTiming)) != cudaSuccess)
      return e;
  }
  if ((e = cudaEventCreateWithFlags(&ms.fork, cudaEventDisableTiming)) != cudaSuccess) return e;

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

// One launch per non-empty size bucket, each on its own stream so that the
// buckets run concurrently: the largest clusters are launched first, and the
// CTAs of the later buckets take over SMs as the earlier buckets drain.
cudaError_t run_mixed(MixedState& ms, const DevBatch& b, const RunArgs& a, cudaStream_t s,
                      int* launches) {
  cudaError_t e;
  *launches = 0;
  if ((e = cudaMemsetAsync(ms.queues, 0, 4 * sizeof(int32_t), s)) != cudaSuccess) return e;
  if ((e = cudaEventRecord(ms.fork, s)) != cudaSuccess) return e;
  for (int q = 0; q < 4; ++q) {
    if (ms.bucket_off[q + 1] == ms.bucket_off[q]) continue;
    cudaStream_t sq = ms.side[q];
    if ((e = cudaStreamWaitEvent(sq, ms.fork, 0)) != cudaSuccess) return e;
    switch (kClusterSizes[q]) {
      case 8: e = launch_bucket<8>(ms, b, a, q, sq); break;
      case 4: e = launch_bucket<4>(ms, b, a, q, sq); break;
      case 2: e = launch_bucket<2>(ms, b, a, q, sq); break;
      default: e = launch_bucket<1>(ms, b, a, q, sq); break;
    }
    if (e != cudaSuccess) return e;
    ++*launches;
    if ((e = cudaEventRecord(ms.join[q], sq)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(s, ms.join[q], 0)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace mfg
