// Mixed-precision relaxation: FP32 forces and integrator, FP64 where it
// matters.
//
// Same algorithm and step structure as the plain FP64 kernel
// (mfg_relax_f64.cu; reference: BatchedFiberRVEAnalysisExplicitTeamOuterLoop.h:180-437),
// with these precision choices:
//  - positions are the FP64 reference X plus an FP32 displacement hi with an
//    FP32 compensation lo (TwoSum), so increments far below an FP32 ulp of u
//    still accumulate: u = hi + lo to ~1e-14;
//  - fiber forces use the Green strain formed from the displacement
//    difference, g = (dX.du + du.du/2) / l0^2, which keeps its relative
//    precision at small strain (the length-ratio form 0.5(l^2/l0^2 - 1)
//    cancels catastrophically in FP32). For the linear law
//    T/l = lambda E A g / l = E A g / l0 needs neither sqrt nor division;
//  - the RAMP boundary moves by an exact FP32 (hi, lo) per-step increment,
//    accumulated with TwoSum: recomputing u0 + alpha d in FP32 every step
//    jitters boundary nodes by ~ulp(d), which the very short fibers kNN
//    networks attach to the boundary turn into large strain noise;
//  - velocities, the damping force, both kicks and the critical time step's
//    lengths (l0 sqrt(1 + 2g)) are FP32;
//  - FP64 is kept for the residual norm and the stress homogenisation, where
//    the reference reduces over the whole RVE, and for the persistent state
//    of the batch (x, u, volume), read at the start and written at the end
//    of every run, so both precisions share it.
//
// Two solves give the same bits: a fiber-centric one (a fiber pass stores
// each fiber's force vector, a node pass gathers them) and a node-centric
// one (each node forms its incident fibers' vectors from the end records;
// nothing but the node state in shared memory).
//
// Placement: one CTA of 1024 threads per SM with 220 KB of dynamic shared
// memory, in size buckets launched concurrently. RVEs run node-centric on
// one CTA or on the 2, 4 or 8 CTAs of a thread-block cluster, each CTA
// keeping its nodes' records (hi, lo) and velocities in shared memory and
// reading other CTAs' through distributed shared memory; where a second copy
// of the records fits at that size, the drift fuses into the kick and a
// step has one barrier instead of two. On the nonlinear law, or on request,
// RVEs whose whole state fits one CTA's shared memory (or half of it, two
// per CTA) run fiber-centric instead.
// Those RVEs get their own fiber and node order (cluster_order) that keeps
// most loads local and the warps' work even. RVEs too large for a cluster of
// 8 run fiber-centric on one CTA, placed by size at run time down to global
// memory.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <thread>
#include <type_traits>
#include <vector>

#include <cooperative_groups.h>

#include "mfg_common.cuh"
#include "mfg_internal.h"
#include "mumfim_gpu.h"
#include "mfg_mixed.h"
#include "mfg_mixed_order.h"

namespace cg = cooperative_groups;

namespace mfg {

// One run context of a mixed batch: the per-bucket claim counters, the
// streams and events a run forks over, the captured graph of its last
// arguments, and the run-time placement's global scratch. Context 0 serves
// the batch's runs; contexts 1-6 the concurrent perturbed solves of the
// material stiffness, which run at the same time on the same batch.
constexpr int kMixedBuckets = 10;
struct MixedRunCtx {
  int32_t* queues = nullptr;  // one claim counter per bucket (device)
  float* u_hl = nullptr;      // run-time placement scratch; null: the batch's own
  float* v = nullptr;
  float4* nrm = nullptr;
  cudaStream_t side[kMixedBuckets] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[kMixedBuckets] = {};
  cudaStream_t capture = nullptr;
  cudaGraphExec_t graph = nullptr;
  RunArgs graph_args{};
  const double* graph_x = nullptr;  // the batch view's coordinates the graph was captured for
  int graph_launches = 0;
  bool ready = false;
};

struct MixedState {
  float* u_hl = nullptr;   // 6 * nt, node records (hi x, y, z, lo x, y, z); run-time placement
  float* v = nullptr;      // 3 * nt, velocity (x, y, z per node); run-time placement
  float2* mass = nullptr;  // nt, (1 / m, m)
  float4* fcon = nullptr;  // et, (X[n2] - X[n1], 1 / l0) rounded to FP32
  float4* nrm = nullptr;   // et, per-fiber force vectors of the run-time placement (w unused)
  // RVEs with an order of their own (cluster_order: all but the run-time
  // placement): per fiber position the two end nodes as (owner CTA << 24 |
  // local record) and the read-only data, per CSR incidence (fiber position
  // << 1 | end). The run-time placement uses the batch's own order, node ids
  // and incidence codes.
  int2* econn = nullptr;      // et
  float4* fconc = nullptr;    // et
  int32_t* icode = nullptr;   // 2 * et
  int32_t* mslot = nullptr;   // et, position of each fiber slot in that order
  // Their nodes: each CTA's free nodes whose neighbours are all its own come
  // first, each group ordered by degree; gnode maps a node position to the
  // batch node index, and the CSR rows and masses follow the positions.
  int32_t* gnode = nullptr;    // nt
  int32_t* mrowptr = nullptr;  // nt + n_rve
  float2* mmass = nullptr;     // nt
  // Node-centric RVEs: per node position its (first incidence, degree) in
  // the RVE's SELL-32 incidence block, which starts at sell_off[rve]; per
  // incidence the other end's code and the fiber's data (solve_rve_nodal).
  int2* nsell = nullptr;         // nt
  int64_t* sell_off = nullptr;   // n_rve
  int32_t* ncode = nullptr;      // set-up only: SELL element codes, packed into nfc
  float4* nfc = nullptr;         // SELL elements
  int64_t n_sell = 0;
  int64_t* nfib_tmp = nullptr;   // set-up only: fiber of each SELL element
  int32_t* h_cl = nullptr;     // host, per RVE: cluster size of its batch bucket
  int32_t* rve_bucket = nullptr;  // device, per RVE: its batch bucket (serving kernels)
  int server_grid = 0;         // CTAs of the cluster serving kernel
  int sms = 1;
  int smem_bytes = 0;
  // Size buckets of the batch run (kBucket[q]: cluster size and solve); the
  // RVEs of bucket q, most fibers first, are order[bucket_off[q] ..
  // bucket_off[q + 1]).
  int32_t* order = nullptr;
  int bucket_off[kMixedBuckets + 1] = {};
  int bucket_grid[kMixedBuckets] = {};
  // Run contexts (host memory; kernels never touch this pointer). A run is a
  // CUDA graph (queue reset, fork, one launch per bucket, join), captured
  // per context for the last run arguments and replayed while they stay
  // the same.
  MixedRunCtx* ctx = nullptr;
};

namespace {

constexpr int kThreadsMixed = 1024;
constexpr int kSmemBytesMixed = 220 * 1024;
// Size buckets, launched in this order (largest clusters first).
struct BucketKind {
  int cl;      // CTAs per cluster
  bool all;    // fiber-centric: force vectors in shared memory too
  bool nodal;  // node-centric solve (node state in shared memory)
  int ng;      // RVEs solved side by side by one CTA (fiber-centric, all on chip)
  bool db;     // node-centric on one CTA with two copies of the node records
};
constexpr int kBuckets = kMixedBuckets;
constexpr BucketKind kBucket[kBuckets] = {
    {8, false, true, 1, false}, {4, false, true, 1, true},   {4, false, true, 1, false},
    {2, false, true, 1, true},  {2, false, true, 1, false},  {1, false, true, 1, false},
    {1, false, true, 1, true},  {1, true, false, 1, false},  {1, true, false, 2, false},
    {1, false, false, 1, false}};
// Placement preference (bucket_of): the first bucket whose shared memory
// holds the RVE, else the last bucket. At each cluster size two copies of
// the node records come first where they fit.
constexpr int kPref[] = {8, 7, 6, 5, 3, 4, 1, 2, 0};
// The single-CTA buckets with an RVE order of their own, by kind.
constexpr int kQNodal1 = 5, kQNodalDB = 6, kQFiberAll = 7, kQFiberPair = 8;
static_assert(kBucket[kQNodal1].cl == 1 && kBucket[kQNodal1].nodal, "bucket table");
static_assert(kBucket[kQNodalDB].cl == 1 && kBucket[kQNodalDB].db, "bucket table");
static_assert(kBucket[kQFiberAll].cl == 1 && kBucket[kQFiberAll].all, "bucket table");
static_assert(kBucket[kQFiberPair].all && kBucket[kQFiberPair].ng == 2, "bucket table");

__global__ void mixed_prepare_kernel(const DevBatch b, MixedState ms) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i < b.nt) {
    const double m = b.m[i];
    ms.mass[i] = make_float2(static_cast<float>(1.0 / m), static_cast<float>(m));
  }
}

__global__ void mixed_prepare_order_kernel(const DevBatch b, MixedState ms) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i < b.nt) ms.mmass[i] = ms.mass[ms.gnode[i]];
}

// 1 / l0 of a fiber from its FP32 reference difference. Every solve takes
// 1 / l0 from this one expression -- the fiber-centric ones from the value
// the set-up stores, the node-centric one by recomputing it from the dX it
// loads -- so a fiber's force vector is the same bits in every solve.
__device__ __forceinline__ float inv_length(float dx, float dy, float dz) {
  const float s = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float r = rsqrtf(s);
  // one Newton step, r (1 + (1 - s r^2) / 2): the approximate reciprocal
  // square root to about half an ulp
  return fmaf(r * 0.5f, fmaf(-s * r, r, 1.f), r);
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
    ms.fcon[fo] = make_float4(dx[0], dx[1], dx[2], inv_length(dx[0], dx[1], dx[2]));
    ms.fconc[d.fiber_off + ms.mslot[fo]] = ms.fcon[fo];
  }
}

// Node-centric incidence records (fiber -1: padding): the fiber's reference
// difference oriented from the other end to the incidence's node (X[n2] -
// X[n1] at the fiber's second end, its negation at the first) and, in the
// fourth word, the other end's node code (the set-up codes carry the end in
// bit 0, which is shifted out). One 16-byte load per incidence; 1 / l0 is
// recomputed from dX (inv_length).
__global__ void mixed_prepare_sell_kernel(const MixedState ms, const int32_t* ncode,
                                          const int64_t* nfib, int64_t n) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i < n) {
    const int64_t e = nfib[i];
    const int code = ncode[i];
    float4 fc = e >= 0 ? ms.fcon[e] : make_float4(0.f, 0.f, 0.f, 0.f);
    if (!(code & 1)) {
      fc.x = -fc.x;
      fc.y = -fc.y;
      fc.z = -fc.z;
    }
    reinterpret_cast<int4*>(ms.nfc)[i] =
        make_int4(__float_as_int(fc.x), __float_as_int(fc.y), __float_as_int(fc.z), code >> 1);
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

struct Rve {
  RveDesc d;
  Law L;
  float4* n;            // fiber force vectors (fiber-centric solve)
  const float2* mass;   // (1 / m, m)
  const float4* fcon;   // (dX, 1 / l0)
  const int2* conn;     // end nodes (node ids, or cluster codes)
  const int32_t* rowptr;
  const int32_t* inc;   // incidences (slot << 1 | end)
  float* ramp;          // per boundary node: step increment d/n as (hi[3], lo[3])
  int64_t node_off, nt;
};

// Shared-window address of `local` in CTA `o` of this cluster.
__device__ __forceinline__ uint32_t cluster_addr(uint32_t local, uint32_t o) {
  uint32_t remote;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(o));
  return remote;
}

// A node record: displacement hi x, y, z and lo x, y, z.
struct NodeRec {
  float hi[3], lo[3];
};

// Node records of an RVE solved by one CTA (shared or global memory), by
// node id; also a cluster CTA's view of its own nodes, by local record.
// Two arrays over the same n slots: (hi x, hi y, hi z, lo x) as one 16-byte
// word, then (lo y, lo z) as one 8-byte word, so a record is one 128-bit
// and one 64-bit access. A warp's gather of 32 scattered records then meets
// fewer bank conflicts than with three 64-bit accesses to a 24-byte record
// (a 128-bit access is served a quarter-warp at a time).
struct LocalNodes {
  float4* a;
  float2* b;
  // the two arrays over n slots from p (16-byte aligned)
  __device__ __forceinline__ static LocalNodes at(float* p, int64_t n) {
    return {reinterpret_cast<float4*>(p), reinterpret_cast<float2*>(p + 4 * n)};
  }
  __device__ __forceinline__ NodeRec load(int j) const {
    const float4 p = a[j];
    const float2 q = b[j];
    return {{p.x, p.y, p.z}, {p.w, q.x, q.y}};
  }
  __device__ __forceinline__ void put(int j, const NodeRec& r) const {
    a[j] = make_float4(r.hi[0], r.hi[1], r.hi[2], r.lo[0]);
    b[j] = make_float2(r.lo[1], r.lo[2]);
  }
};

// Node records of an RVE split over the CTAs of a cluster, read through
// distributed shared memory. CTA o owns a contiguous block of the free nodes
// and one of the boundary nodes (both segments are Morton-sorted, so the two
// blocks cover the same region of the RVE) and keeps their records at the
// same shared-memory offsets in every CTA (the two arrays of LocalNodes, at
// base_a and base_b); an end node is given by its code (owner << 24 |
// record).
template <int CL>
struct ClusterNodes {
  uint32_t base_a, base_b;
  __device__ __forceinline__ void point_at(const LocalNodes& own) {
    base_a = static_cast<uint32_t>(__cvta_generic_to_shared(own.a));
    base_b = static_cast<uint32_t>(__cvta_generic_to_shared(own.b));
  }
  __device__ __forceinline__ NodeRec load(int code) const {
    const uint32_t o = static_cast<uint32_t>(code) >> 24;
    const uint32_t j = static_cast<uint32_t>(code) & 0xFFFFFFu;
    const uint32_t pa = cluster_addr(base_a + 16u * j, o);
    const uint32_t pb = cluster_addr(base_b + 8u * j, o);
    float4 p;
    float2 q;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(p.x), "=f"(p.y), "=f"(p.z), "=f"(p.w)
                 : "r"(pa));
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(q.x), "=f"(q.y) : "r"(pb));
    return {{p.x, p.y, p.z}, {p.w, q.x, q.y}};
  }
};

// Fiber force vectors in the CTA's shared memory or in global memory, by
// incidence code (slot << 1 | end).
struct LocalForces {
  const float4* p;
  __device__ __forceinline__ float4 load(int code) const { return p[code >> 1]; }
};

template <int CL>
struct ClusterOps {
  __device__ static int rank() {
    if constexpr (CL > 1) return static_cast<int>(cg::this_cluster().block_rank());
    return 0;
  }
  // Block barrier, or cluster barrier (release / acquire at cluster scope,
  // which also orders the CTAs' shared-memory writes for their peers).
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

// The threads that solve one RVE: the whole CTA (NG = 1) or one of NG equal
// groups of it, each synchronised by its own named barrier (barrier 0 is
// the CTA's), so that small RVEs can share a CTA without waiting for each
// other.
template <int NG>
struct Group {
  static_assert(NG == 1 || NG == 2, "one or two RVEs per CTA");
  static constexpr int kSize = kThreadsMixed / NG;
  __device__ static int index() { return NG == 1 ? 0 : static_cast<int>(threadIdx.x) / kSize; }
  __device__ static int tid() {
    return NG == 1 ? static_cast<int>(threadIdx.x) : static_cast<int>(threadIdx.x) % kSize;
  }
  __device__ static void sync() {
    if constexpr (NG == 1)
      __syncthreads();
    else
      asm volatile("bar.sync %0, %1;" ::"r"(1 + index()), "r"(kSize) : "memory");
  }
};

// Minimum over a group (min is exact, so the order does not matter).
template <int NG>
__device__ __forceinline__ double group_min(double v, double* red) {
  if constexpr (NG == 1) {
    return block_min<kThreadsMixed>(v, red);
  } else {
    constexpr int NW = Group<NG>::kSize / 32;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = Group<NG>::tid() >> 5, l = threadIdx.x & 31;
    Group<NG>::sync();
    if (l == 0) red[w] = v;
    Group<NG>::sync();
    if (w == 0) {
      double t = (l < NW) ? red[l] : DBL_MAX;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t = fmin(t, __shfl_xor_sync(0xffffffffu, t, o));
      if (l == 0) red[NW] = t;
    }
    Group<NG>::sync();
    return red[NW];
  }
}

// Sum over kThreadsMixed "virtual threads" in the fixed order of
// block_sum<kThreadsMixed>: thread t of a group of kSize threads holds the
// partial sums acc[j] of virtual threads t + j kSize. Each virtual warp is
// reduced by the same butterfly over the same lanes, and its partial lands
// in the same slot, so a group of any size gives the bits of a whole CTA.
template <int NG>
__device__ __forceinline__ double group_sum(const double (&acc)[NG], double* red) {
  if constexpr (NG == 1) {
    return block_sum<kThreadsMixed>(acc[0], red);
  } else {
    constexpr int NWV = kThreadsMixed / 32;       // virtual warps
    constexpr int NWG = Group<NG>::kSize / 32;    // warps of the group
    double v[NG];
#pragma unroll
    for (int j = 0; j < NG; ++j) {
      v[j] = acc[j];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
    }
    const int w = Group<NG>::tid() >> 5, l = threadIdx.x & 31;
    Group<NG>::sync();
    if (l == 0) {
#pragma unroll
      for (int j = 0; j < NG; ++j) red[w + j * NWG] = v[j];
    }
    Group<NG>::sync();
    if (w == 0) {
      double t = (l < NWV) ? red[l] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if (l == 0) red[NWV] = t;
    }
    Group<NG>::sync();
    return red[NWV];
  }
}

// Nodal internal force: incident fiber vectors in the node's CSR order,
// subtracted at a fiber's first end and added at its second.
template <class Forces>
__device__ __forceinline__ void gather_row(const Rve& r, const Forces& fv, int pb, int pe, float& a0,
                                           float& a1, float& a2) {
  a0 = 0.f; a1 = 0.f; a2 = 0.f;
  int p = pb;
  // four incidences in flight, summed in CSR order
  for (; p + 4 <= pe; p += 4) {
    int code[4];
    float4 t[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) code[q] = __ldg(r.inc + p + q);
#pragma unroll
    for (int q = 0; q < 4; ++q) t[q] = fv.load(code[q]);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float sg = (code[q] & 1) ? 1.f : -1.f;
      a0 = fmaf(sg, t[q].x, a0);
      a1 = fmaf(sg, t[q].y, a1);
      a2 = fmaf(sg, t[q].z, a2);
    }
  }
  for (; p < pe; ++p) {
    const int code = __ldg(r.inc + p);
    const float4 t = fv.load(code);
    const float sg = (code & 1) ? 1.f : -1.f;
    a0 = fmaf(sg, t.x, a0);
    a1 = fmaf(sg, t.y, a1);
    a2 = fmaf(sg, t.z, a2);
  }
}

template <class Forces>
__device__ __forceinline__ void gather(const Rve& r, const Forces& fv, int i, float& a0, float& a1,
                                       float& a2) {
  gather_row(r, fv, __ldg(r.rowptr + i), __ldg(r.rowptr + i + 1), a0, a1, a2);
}

// Read-only data of one fiber (end nodes; dX and 1/l0) and of one node (CSR
// row bounds; 1/m and m), loaded one item ahead of its use in the passes.
struct FiberConst {
  int2 c;
  float4 fc;
};
struct NodeConst {
  int pb, pe;
  float2 mm;
};
__device__ __forceinline__ FiberConst load_fiber(const Rve& r, int e) {
  return {__ldg(r.conn + e), __ldg(r.fcon + e)};
}
__device__ __forceinline__ NodeConst load_node(const Rve& r, int i) {
  return {__ldg(r.rowptr + i), __ldg(r.rowptr + i + 1), __ldg(r.mass + i)};
}

// Force vector of one fiber. The displacement difference du is the
// difference of the hi parts plus the difference of the lo parts. Where the
// two hi parts are within a factor of two of each other -- every short
// fiber, whose end displacements nearly agree -- their FP32 difference is
// exact (Sterbenz); elsewhere its rounding is within one ulp of du itself.
// So du is accurate to FP32 of du, not of u, and the Green strain formed
// from it (g l0^2 = du.(dX + du/2)) keeps its relative precision at small
// strain, where 0.5(l^2/l0^2 - 1) would cancel.
// Returns the current length l0 sqrt(1 + 2g), which the critical time step
// needs every 100 steps (unused, and so not computed, on the other steps).
//
// The steps are split so that the node-centric pass (which forms the same
// vector from either end) runs exactly the same arithmetic.
__device__ __forceinline__ void disp_diff(const NodeRec& na, const NodeRec& nb, float du[3]) {
#pragma unroll
  for (int q = 0; q < 3; ++q)
    du[q] = __fadd_rn(__fsub_rn(nb.hi[q], na.hi[q]), __fsub_rn(nb.lo[q], na.lo[q]));
}
__device__ __forceinline__ float green(const float du[3], const float4& fc) {
  const float gn = fmaf(du[0], fmaf(0.5f, du[0], fc.x),
                        fmaf(du[1], fmaf(0.5f, du[1], fc.y), du[2] * fmaf(0.5f, du[2], fc.z)));
  return gn * (fc.w * fc.w);
}
__device__ __forceinline__ float4 force_vec(const Law& L, const float du[3], const float4& fc,
                                            float g) {
  const float t = tension_over_length(L, g, fc.w);
  return make_float4((fc.x + du[0]) * t, (fc.y + du[1]) * t, (fc.z + du[2]) * t, 0.f);
}
__device__ __forceinline__ float fiber_length(float g, float rl0) {
  return sqrtf(fmaxf(fmaf(2.f, g, 1.f), 0.f)) / rl0;
}

template <class Nodes>
__device__ __forceinline__ float fiber_force(const Rve& r, const Nodes& u, int e,
                                             const FiberConst& k) {
  float du[3];
  disp_diff(u.load(k.c.x), u.load(k.c.y), du);
  const float g = green(du, k.fc);
  r.n[e] = force_vec(r.L, du, k.fc, g);
  return fiber_length(g, k.fc.w);
}

// Force vectors of fiber slots e_lo + tid, + group size, ... < e_hi, the
// next slot's read-only data loaded while the current one is computed.
// Returns the shortest current length among them when kLen.
template <bool kLen, int NG = 1, class Nodes>
__device__ __forceinline__ float fiber_pass(const Rve& r, const Nodes& u, int e_lo, int e_hi) {
  float lmin = FLT_MAX;
  int e = e_lo + Group<NG>::tid();
  if (e >= e_hi) return lmin;
  FiberConst cur = load_fiber(r, e);
  for (;;) {
    const int en = e + Group<NG>::kSize;
    const bool more = en < e_hi;
    FiberConst nxt = cur;
    if (more) nxt = load_fiber(r, en);
    const float l = fiber_force(r, u, e, cur);
    if (kLen) lmin = fminf(lmin, l);
    if (!more) break;
    cur = nxt;
    e = en;
  }
  return lmin;
}

// Stress of one RVE (BatchedFiberRVEAnalysisExplicitBase.h:58-126) in FP64
// by one CTA, and its status record. Each Voigt component is a pass over the
// boundary nodes: each thread sums a strided share in the reference's
// boundary order, then a fixed-order block reduction. The FP64 kernel keeps
// the reference's serial sum; here any fixed order will do, and it keeps the
// result independent of what else runs (and of the group size: group_sum
// keeps the order of a whole CTA). One component at a time keeps NG
// accumulators live.
template <int NG = 1>
__device__ __forceinline__ void mixed_stress(const DevBatch& b, const RunArgs& a, int rve,
                                             int status, int step, double residual, double* red,
                                             bool leader) {
  const RveDesc& d = b.desc[rve];
  const int tid = Group<NG>::tid();
  const int64_t no = d.node_off, nt = b.nt;
  const int32_t* bo = b.bnd + d.bnd_off;
  const int nb = leader ? d.n_nodes - d.n_free : 0;  // every CTA reduces, one sums
  const double sc = d.scale / b.vol[rve];
  bool bad = false;
#pragma unroll 1
  for (int k = 0; k < 6; ++k) {
    // component k: (i, j) index pair of the symmetric part x_i f_j
    const int ci = k < 3 ? k : (k == 3 ? 1 : 0);
    const int cj = k < 3 ? k : (k == 5 ? 1 : 2);
    const double* xi = b.x + ci * nt + no;
    const double* xj = b.x + cj * nt + no;
    const double* fi = b.fint + ci * nt + no;
    const double* fj = b.fint + cj * nt + no;
    // virtual thread t + j kSize sums q = t + j kSize + m kThreadsMixed
    double acc[NG];
#pragma unroll
    for (int j = 0; j < NG; ++j) acc[j] = 0.0;
    for (int q = tid, j = 0; q < nb; q += Group<NG>::kSize, j = (j + 1 == NG ? 0 : j + 1)) {
      const int i = bo[q];
      const double t = k < 3 ? xi[i] * fi[i] : 0.5 * (xi[i] * fj[i] + xj[i] * fi[i]);
#pragma unroll
      for (int jj = 0; jj < NG; ++jj)
        if (jj == j) acc[jj] += t;
    }
    const double sk = group_sum<NG>(acc, red) * sc;
    bad = bad || !isfinite(sk);
    if (leader && tid == 0) {
      a.sigma[6 * rve + k] = sk;
      if (a.update_coords) b.cur_stress[6 * rve + k] = sk;
    }
  }
  if (leader && tid == 0) {
    a.st_status[rve] = bad ? 4 : status;
    a.st_steps[rve] = step;
    a.st_residual[rve] = residual;
  }
}

// Node slots rounded up to an even count, so that an array of records after
// another starts on a 16-byte boundary.
__host__ __device__ inline int64_t even_slots(int64_t n) { return (n + 1) & ~static_cast<int64_t>(1); }

// Shared-memory floats per CTA of an RVE solved by CL CTAs: 9 per node slot
// (displacement hi, lo and velocity; ceil(NF/CL) free plus ceil(NB/CL)
// boundary slots), 15 with two copies of the node records, plus 4 per fiber
// slot (ceil(E/CL)) when the force vectors are kept in shared memory too
// (all: the fiber-centric single CTA).
__host__ __device__ inline int64_t cluster_floats(int n_nodes, int n_free, int n_fibers, int cl,
                                                  bool all, bool two_copies = false) {
  const int64_t nb = n_nodes - n_free;
  const int64_t cap = even_slots((static_cast<int64_t>(n_free) + cl - 1) / cl + (nb + cl - 1) / cl);
  const int64_t echunk = (static_cast<int64_t>(n_fibers) + cl - 1) / cl;
  return (two_copies ? 15 : 9) * cap + (all ? 4 * echunk : 0);
}

// Prologue of a solve in FP64 for the CTA's own nodes: the affine predictor
// (BatchedFiberRVEAnalysisExplicitBase.h:16-57) or, in RAMP mode, the
// boundary's per-step increment; displacements split into (hi, lo); v = 0.
// kOrder: the RVE has its own node order (gnode maps positions to nodes).
template <bool kOrder, int NG = 1>
__device__ __forceinline__ void mixed_prologue(const DevBatch& b, const MixedState& ms,
                                               const Rve& r, const double Fm[9], bool ramp,
                                               int f_lo, int g_lo, int nfo, int n_own, int fchunk,
                                               const LocalNodes& own, float* vel) {
  const RveDesc& d = r.d;
  const int NF = d.n_free, tid = Group<NG>::tid();
  const int64_t no = d.node_off, nt = b.nt;
  for (int t = tid; t < n_own; t += Group<NG>::kSize) {
    const int i = t < nfo ? f_lo + t : g_lo + (t - nfo);
    const int li = t < nfo ? t : fchunk + (t - nfo);
    const int64_t gi = kOrder ? __ldg(ms.gnode + no + i) : no + i;  // batch node index
    double xo[3], up[3], X[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      xo[k] = b.x[k * nt + gi];
      up[k] = b.u[k * nt + gi];
      X[k] = b.X[k * nt + gi];
    }
    if (!ramp) {
      const double u0 = (Fm[0] - 1) * xo[0] + Fm[1] * xo[1] + Fm[2] * xo[2] + up[0];
      const double u1 = Fm[3] * xo[0] + (Fm[4] - 1) * xo[1] + Fm[5] * xo[2] + up[1];
      const double u2 = Fm[6] * xo[0] + Fm[7] * xo[1] + (Fm[8] - 1) * xo[2] + up[2];
      up[0] = u0; up[1] = u1; up[2] = u2;
    }
    double xn[3];
    NodeRec nr;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      xn[k] = X[k] + up[k];
      split(xn[k] - X[k], nr.hi[k], nr.lo[k]);
      vel[3 * li + k] = 0.f;
    }
    own.put(li, nr);
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
}

// RAMP mode: the own boundary nodes move by their exact (hi, lo) increment.
template <int NG = 1>
__device__ __forceinline__ void ramp_boundary(const Rve& r, const LocalNodes& own, int g_lo,
                                              int g_hi, int fchunk, const LocalNodes* dst = nullptr) {
  const int NF = r.d.n_free;
  for (int i = g_lo + Group<NG>::tid(); i < g_hi; i += Group<NG>::kSize) {
    const float* rb = r.ramp + 12 * (i - NF);
    const int li = fchunk + (i - g_lo);
    NodeRec nr = own.load(li);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float s, e;
      two_sum(nr.hi[k], rb[k], s, e);
      nr.hi[k] = s;
      nr.lo[k] = nr.lo[k] + (e + rb[3 + k]);
    }
    (dst ? *dst : own).put(li, nr);  // in place, or into the other copy
  }
}

// One RVE solved by one CTA, fiber-centric: a fiber pass forms every
// fiber's force vector once, a node pass gathers them per node. With kAll
// the CTA keeps everything in shared memory (the caller guarantees it fits,
// so every shared access compiles as one) and the RVE has its own node
// order (cluster_order); without kAll it places the RVE by its size at run
// time, in the batch's order: everything in shared memory, the node state
// only, the displacements only, or everything in global memory.
template <bool kAll, int NG = 1>
__device__ void solve_rve_mixed(const DevBatch& b, const MixedState& ms, const RunArgs& a, int rve,
                                double* red, float* smem, int smem_floats) {
  static_assert(NG == 1 || kAll, "RVEs share a CTA only when their state fits its shared memory");
  using G = Group<NG>;  // the threads solving this RVE
  Rve r;
  r.d = b.desc[rve];
  const RveDesc& d = r.d;
  r.L = make_law(d);
  const int N = d.n_nodes, NF = d.n_free, E = d.n_fibers;
  const int tid = G::tid();
  const int64_t no = d.node_off, fo = d.fiber_off, nt = b.nt;
  r.node_off = no;
  r.nt = nt;
  // the group owns every node (free [0, NF), boundary [NF, N), local index =
  // node position) and every fiber slot
  const int rank = 0;
  const int f_lo = 0, f_hi = NF, g_lo = NF, g_hi = N, nfo = NF, n_own = N, fchunk = NF;
  const int e_lo = 0, e_hi = E;
  LocalNodes own;  // the node records, by local index
  float* vel;      // their velocities (x, y, z), by local index
  LocalForces fv;  // every fiber force vector of the RVE (node pass)
  r.conn = b.conn + fo;
  r.fcon = ms.fcon + fo;
  r.inc = b.inc + d.inc_off;
  r.rowptr = b.rowptr + d.row_off;
  r.mass = ms.mass + no;
  if constexpr (kAll) {
    // this RVE's own fiber and node order (cluster_order)
    r.conn = ms.econn + fo;
    r.fcon = ms.fconc + fo;
    r.inc = ms.icode + d.inc_off;
    r.rowptr = ms.mrowptr + d.row_off;
    r.mass = ms.mmass + no;
  }
  // force vectors first (16-byte aligned), then the node records, then the
  // velocities
  if (kAll || cluster_floats(N, NF, E, 1, true) <= smem_floats) {
    r.n = reinterpret_cast<float4*>(smem);
    own = LocalNodes::at(smem + 4 * E, N);
    vel = smem + 4 * E + 6 * N;
  } else if (cluster_floats(N, NF, E, 1, false) <= smem_floats) {
    r.n = ms.nrm + fo;
    own = LocalNodes::at(smem, N);
    vel = smem + 6 * N;
  } else if (6LL * N <= smem_floats) {
    r.n = ms.nrm + fo;
    own = LocalNodes::at(smem, N);
    vel = ms.v + 3 * no;
  } else {
    r.n = ms.nrm + fo;
    own = {reinterpret_cast<float4*>(ms.u_hl) + no, reinterpret_cast<float2*>(ms.u_hl + 4 * nt) + no};
    vel = ms.v + 3 * no;
  }
  fv.p = r.n;
  const LocalNodes& u = own;  // every node of the RVE (fiber pass)
  r.ramp = reinterpret_cast<float*>(b.ramp + 6 * d.bnd_off);  // 12 floats per boundary node
  const double* F = a.F + 9 * (a.n_F > 1 ? rve : 0);
  const bool ramp = d.mode == 1;
  double Fm[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Fm[k] = F[k];
  if (a.update_coords && rank == 0 && tid == 0) b.vol[rve] = jacobian(Fm) * b.vol[rve];

  // ---- prologue in FP64: predictor, split into (hi, lo), v = 0 -------------
  mixed_prologue<kAll, NG>(b, ms, r, Fm, ramp, f_lo, g_lo, nfo, n_own, fchunk, own, vel);
  G::sync();
  // critical step from the shortest current fiber (FP32 length from the
  // Green strain, ~1e-7 relative; h itself is an FP32 number)
  const float lmin = fiber_pass<true, NG>(r, u, e_lo, e_hi);
  double dt_crit = group_min<NG>(lmin, red) / d.sound_speed;

  const int step_cap = d.max_steps;
  const float c = static_cast<float>(d.c);
  float h_cur = static_cast<float>(d.crit * dt_crit * 0.5);
  int step = 0;
  double residual = 10.0;
  float h_prev = 0.f;
  int status = 0;
  for (;;) {
    const bool res_step = step > 0 && ((step - 1) % kUpdateFreq) == 0;
    if (res_step) {
      // virtual thread tid + j kSize sums the nodes tid + j kSize + m kThreadsMixed
      double part[NG];
#pragma unroll
      for (int j = 0; j < NG; ++j) part[j] = 0.0;
      for (int i = f_lo + tid, j = 0; i < f_hi; i += G::kSize, j = (j + 1 == NG ? 0 : j + 1)) {
        float a0, a1, a2;
        gather(r, fv, i, a0, a1, a2);
        const double q2 = static_cast<double>(a0) * a0 + static_cast<double>(a1) * a1 +
                          static_cast<double>(a2) * a2;
#pragma unroll
        for (int jj = 0; jj < NG; ++jj)
          if (jj == j) part[jj] += q2;
      }
      residual = sqrt(group_sum<NG>(part, red));
      if (!isfinite(residual)) {
        status = 4;
        break;
      }
    }
    if (!ramp && res_step && !(residual > d.tol)) break;
    if (step >= step_cap) break;
    // per-step scalars in FP32 (h changes only when dt_crit does)
    const float h = h_cur;
    const float hk = h_prev + h;  // trailing kick of step-1 + leading kick of step
    const float h2 = h + h;
    // node pass over the own free nodes, the next node's row bounds and mass
    // loaded while the current one is gathered
    if (f_lo + tid < f_hi) {
      int i = f_lo + tid;
      NodeConst cur = load_node(r, i);
      for (;;) {
        const int in = i + G::kSize;
        const bool more = in < f_hi;
        NodeConst nxt = cur;
        if (more) nxt = load_node(r, in);
        float f[3];
        gather_row(r, fv, cur.pb, cur.pe, f[0], f[1], f[2]);
        const float mc = cur.mm.y * c;
        const float km = hk * cur.mm.x;
        const int li = i - f_lo;
        NodeRec nr = own.load(li);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          float w = vel[3 * li + k];
          w = fmaf(km, -f[k] - mc * w, w);
          vel[3 * li + k] = w;
          comp_add(nr.hi[k], nr.lo[k], h2 * w);
        }
        own.put(li, nr);
        if (!more) break;
        cur = nxt;
        i = in;
      }
    }
    if (ramp) ramp_boundary<NG>(r, own, g_lo, g_hi, fchunk);
    G::sync();
    const bool dt_step = (step % kUpdateFreq) == 0;
    if (dt_step) {
      const float lm = fiber_pass<true, NG>(r, u, e_lo, e_hi);
      dt_crit = group_min<NG>(lm, red) / d.sound_speed;
      h_cur = static_cast<float>(d.crit * dt_crit * 0.5);
    } else {
      fiber_pass<false, NG>(r, u, e_lo, e_hi);
      G::sync();
    }
    h_prev = h;
    ++step;
  }
  if (status == 0 && !ramp && residual > d.tol) status = 3;

  // ---- finalize: FP64 positions, boundary f_int, stress ---------------------
  for (int t = tid; t < n_own; t += G::kSize) {
    const int i = t < nfo ? f_lo + t : g_lo + (t - nfo);
    const int li = t < nfo ? t : fchunk + (t - nfo);
    const int64_t gi = kAll ? __ldg(ms.gnode + no + i) : no + i;  // batch node index
    const NodeRec nr = own.load(li);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double Xk = b.X[k * nt + gi];
      const double xk = Xk + (static_cast<double>(nr.hi[k]) + nr.lo[k]);
      b.x[k * nt + gi] = xk;
      if (a.update_coords) b.u[k * nt + gi] = xk - Xk;
    }
    if (i >= NF) {
      float a0, a1, a2;
      gather(r, fv, i, a0, a1, a2);
      b.fint[no + i] = a0;
      b.fint[nt + no + i] = a1;
      b.fint[2 * nt + no + i] = a2;
    }
  }
  G::sync();
  mixed_stress<NG>(b, a, rve, status, step, residual, red, rank == 0);
  G::sync();
}

// ---- node-centric solve -----------------------------------------------------
//
// Each thread owns nodes and forms the force vector of every fiber incident
// to them from the fiber's two end records, in the node's CSR order: every
// fiber is evaluated at both of its ends (twice the fiber arithmetic) and no
// force vector is stored. Shared memory then holds only the node state
// (records and velocities, 9 floats per node), and a step's shared-memory
// traffic is the end records plus the own state, against records, force
// vector stores and force vector gathers in the fiber-centric solve above.
// The vector of a fiber is the same bits at either end and as the fiber
// pass forms it (below), so both solves give the same results.
//
// Incidences are stored sliced by warp (SELL-32): the own nodes of a CTA, in
// the order its threads visit them (free nodes, then boundary nodes), form
// slices of 32, a slice as wide as its largest degree, and the k-th
// incidence of the node at lane l of a slice is at slice base + 32 k + l. A
// warp's loads of incidence records are then contiguous. An incidence is
// one 16-byte record: the fiber's reference difference oriented from the
// other end to this node, X_me - X_o, and the other end's node code
// (mixed_prepare_sell_kernel); 1 / l0 is recomputed from the difference
// with the expression the fiber-centric solves' stored value comes from
// (inv_length), which a negation leaves unchanged.
//
// With both differences taken from the other end to this node, the vector
// (dX + du) T / l is the fiber's force vector at its second end and exactly
// its negation at the first: the rounded difference of the negated operands
// is the negated difference (rounding to nearest is symmetric), the Green
// strain is unchanged under (dX, du) -> (-dX, -du), and so is T / l. Adding
// it is the same rounding as subtracting the second-end vector, so the sums
// are the bits the fiber-centric solve gathers.

// Internal force of one node with record `me` from its deg incidences
// starting at p.
template <class Nodes>
__device__ __forceinline__ void nodal_force(const Law& L, const Nodes& u, const float4* nfc, int p,
                                            int deg, const NodeRec& me, float& a0, float& a1,
                                            float& a2) {
  a0 = 0.f; a1 = 0.f; a2 = 0.f;
  if (deg <= 0) return;
  const int4* rec = reinterpret_cast<const int4*>(nfc);
  int4 q = __ldg(rec + p);
  for (int k = 1;; ++k) {
    const bool more = k < deg;
    int4 qn = q;
    if (more) {
      p += 32;
      qn = __ldg(rec + p);
    }
    const float dx = __int_as_float(q.x), dy = __int_as_float(q.y), dz = __int_as_float(q.z);
    const float4 fc = make_float4(dx, dy, dz, inv_length(dx, dy, dz));
    const NodeRec o = u.load(q.w);
    float du[3];
    disp_diff(o, me, du);  // x_me - x_o
    const float g = green(du, fc);
    const float4 f = force_vec(L, du, fc, g);
    // an add that is never fused with the product forming f: the vector is
    // rounded before it is summed, as when the fiber-centric solve gathers it
    a0 = __fadd_rn(a0, f.x);
    a1 = __fadd_rn(a1, f.y);
    a2 = __fadd_rn(a2, f.z);
    if (!more) break;
    q = qn;
  }
}

// Pass A of the node-centric step: force and kick (v += hk f / m - damping)
// of the CTA's own free nodes t = tid, tid + kThreadsMixed, ... < nfo, the
// next node's row and mass loaded while the current one is summed. With
// kRes also returns this thread's share of the squared residual norm.
// With kFuse (two copies of the node records) the same thread then drifts
// the node at once, x += 2 h v with the new v, into the other copy `nxt`:
// the arithmetic of pass B, without its barrier.
template <bool kRes, bool kFuse = false, class Nodes>
__device__ __forceinline__ double nodal_kick(const Law& L, const Nodes& u, const LocalNodes& own,
                                             float* vel, const float4* nfc,
                                             const int2* srow, const float2* mass, int nfo,
                                             float hk, float c, const LocalNodes* nxt = nullptr,
                                             float h2 = 0.f) {
  double part = 0.0;
  int t = threadIdx.x;
  if (t >= nfo) return part;
  int2 sr = __ldg(srow + t);
  float2 mm = __ldg(mass + t);
  for (;;) {
    const int tn = t + kThreadsMixed;
    const bool more = tn < nfo;
    int2 srn = sr;
    float2 mmn = mm;
    if (more) {
      srn = __ldg(srow + tn);
      mmn = __ldg(mass + tn);
    }
    float f[3];
    const NodeRec me = own.load(t);
    nodal_force(L, u, nfc, sr.x, sr.y, me, f[0], f[1], f[2]);
    if constexpr (kRes)
      part += static_cast<double>(f[0]) * f[0] + static_cast<double>(f[1]) * f[1] +
              static_cast<double>(f[2]) * f[2];
    const float mc = mm.y * c;
    const float km = hk * mm.x;
    float wn[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float w = vel[3 * t + k];
      w = fmaf(km, -f[k] - mc * w, w);
      vel[3 * t + k] = w;
      wn[k] = w;
    }
    if constexpr (kFuse) {
      NodeRec nr = me;
#pragma unroll
      for (int k = 0; k < 3; ++k) comp_add(nr.hi[k], nr.lo[k], h2 * wn[k]);
      nxt->put(t, nr);
    }
    if (!more) break;
    t = tn;
    sr = srn;
    mm = mmn;
  }
  return part;
}

// Shortest current length among fiber slots e_lo + tid, + kThreadsMixed, ...
// < e_hi (the critical time step's input, every 100 steps).
template <class Nodes>
__device__ __forceinline__ float length_pass(const Rve& r, const Nodes& u, int e_lo, int e_hi) {
  float lmin = FLT_MAX;
  for (int e = e_lo + static_cast<int>(threadIdx.x); e < e_hi; e += kThreadsMixed) {
    const FiberConst k = load_fiber(r, e);
    float du[3];
    disp_diff(u.load(k.c.x), u.load(k.c.y), du);
    lmin = fminf(lmin, fiber_length(green(du, k.fc), k.fc.w));
  }
  return lmin;
}

// One RVE by one CTA or the CL CTAs of a cluster, node-centric; every CTA
// keeps its own nodes' records and velocities in shared memory (the caller
// guarantees 9 floats per node slot fit). Node ranges per CTA, the node
// order and the fiber-slot ranges (used by the length pass) are those of
// the fiber-centric cluster solve.
//
// Step structure (same arithmetic and order as the fiber-centric solve):
// on every 100th step the length pass refreshes the time step; pass A forms
// each own free node's force, sums the residual on those steps and applies
// the kick (v += h f / m, both half kicks in one); pass B, after a barrier,
// drifts the own free nodes (x += 2h v) and moves the RAMP boundary.
template <int CL, bool kDB = false>
__device__ void solve_rve_nodal(const DevBatch& b, const MixedState& ms, const RunArgs& a, int rve,
                                double* red, double* cred, float* smem) {
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
  const int NB = N - NF;
  const int fchunk = (NF + CL - 1) / CL, bchunk = (NB + CL - 1) / CL, cap = fchunk + bchunk;
  const int f_lo = min(NF, rank * fchunk), f_hi = min(NF, f_lo + fchunk);
  const int g_lo = NF + min(NB, rank * bchunk), g_hi = NF + min(NB, rank * bchunk + bchunk);
  const int nfo = f_hi - f_lo, n_own = nfo + (g_hi - g_lo);
  const int echunk = (E + CL - 1) / CL;
  const int e_lo = min(E, rank * echunk);
  const int e_hi = min(E, e_lo + echunk);
  using Nodes = std::conditional_t<(CL > 1), ClusterNodes<CL>, LocalNodes>;
  Nodes u;         // every node of the RVE
  // the node records this CTA updates, by local index (an even slot count,
  // so the next array starts on a 16-byte boundary)
  const int64_t slots = even_slots(cap);
  LocalNodes own = LocalNodes::at(smem, slots);
  // kDB: a second copy of the records, which each step drifts into; the two
  // copies swap roles every step
  LocalNodes nxt = LocalNodes::at(smem + 6 * slots, slots);
  float* vel = smem + (kDB ? 12 : 6) * slots;
  if constexpr (CL > 1)
    u.point_at(own);
  else
    u = own;
  r.conn = ms.econn + fo;
  r.fcon = ms.fconc + fo;
  r.ramp = reinterpret_cast<float*>(b.ramp + 6 * d.bnd_off);
  const int2* srow = ms.nsell + no;  // by node position: (first incidence, degree)
  const int64_t so = ms.sell_off[rve];
  const float4* nfc = ms.nfc + so;
  const float2* mass = ms.mmass + no;
  const double* F = a.F + 9 * (a.n_F > 1 ? rve : 0);
  const bool ramp = d.mode == 1;
  double Fm[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Fm[k] = F[k];
  if (a.update_coords && rank == 0 && tid == 0) b.vol[rve] = jacobian(Fm) * b.vol[rve];
  mixed_prologue<true>(b, ms, r, Fm, ramp, f_lo, g_lo, nfo, n_own, fchunk, own, vel);
  Ops::sync();
  if constexpr (kDB) {
    // boundary records in the second copy too (RAMP moves them into it every
    // step; RELAX never moves them); read there only after a step's barrier
    for (int t = tid; t < g_hi - g_lo; t += kThreadsMixed)
      nxt.put(fchunk + t, own.load(fchunk + t));
  }
  double dt_crit = Ops::template combine<true>(
                       block_min<kThreadsMixed>(length_pass(r, u, e_lo, e_hi), red), cred) /
                   d.sound_speed;

  const int step_cap = d.max_steps;
  const float c = static_cast<float>(d.c);
  float h_cur = static_cast<float>(d.crit * dt_crit * 0.5);
  int step = 0;
  double residual = 10.0;
  float h_prev = 0.f;
  int status = 0;
  for (;;) {
    const bool res_step = step > 0 && ((step - 1) % kUpdateFreq) == 0;
    if (!res_step && step >= step_cap) break;
    if (res_step) {
      // the time step from the positions after the last drift
      dt_crit = Ops::template combine<true>(
                    block_min<kThreadsMixed>(length_pass(r, u, e_lo, e_hi), red), cred) /
                d.sound_speed;
      h_cur = static_cast<float>(d.crit * dt_crit * 0.5);
    }
    const float h = h_cur;
    const float hk = h_prev + h;  // trailing kick of step-1 + leading kick of step
    const float h2 = h + h;
    // pass A (compiled apart for the residual steps, so that the FP64
    // residual sum costs nothing on the others); with two record copies
    // pass B is fused into it and writes the other copy
    const double part =
        res_step ? nodal_kick<true, kDB>(r.L, u, own, vel, nfc, srow + f_lo, mass + f_lo, nfo, hk,
                                         c, &nxt, h2)
                 : nodal_kick<false, kDB>(r.L, u, own, vel, nfc, srow + f_lo, mass + f_lo, nfo,
                                          hk, c, &nxt, h2);
    if (res_step) {
      residual = sqrt(Ops::template combine<false>(block_sum<kThreadsMixed>(part, red), cred));
      // a break keeps the copy of the step's start: the drift is dropped
      if (!isfinite(residual)) {
        status = 4;
        break;
      }
      if (!ramp && !(residual > d.tol)) break;
      if (step >= step_cap) break;
    } else if constexpr (!kDB) {
      Ops::sync();
    }
    if constexpr (!kDB) {
      // pass B: drift
      for (int t = tid; t < nfo; t += kThreadsMixed) {
        NodeRec nr = own.load(t);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float w = vel[3 * t + k];
          comp_add(nr.hi[k], nr.lo[k], h2 * w);
        }
        own.put(t, nr);
      }
    }
    if (ramp) ramp_boundary(r, own, g_lo, g_hi, fchunk, kDB ? &nxt : nullptr);
    Ops::sync();
    if constexpr (kDB) {
      const LocalNodes t = own;
      own = nxt;
      nxt = t;
      if constexpr (CL > 1)
        u.point_at(own);
      else
        u = own;
    }
    h_prev = h;
    ++step;
  }
  if (status == 0 && !ramp && residual > d.tol) status = 3;

  // ---- finalize: FP64 positions, boundary f_int, stress ---------------------
  for (int t = tid; t < n_own; t += kThreadsMixed) {
    const int i = t < nfo ? f_lo + t : g_lo + (t - nfo);
    const int li = t < nfo ? t : fchunk + (t - nfo);
    const int64_t gi = __ldg(ms.gnode + no + i);  // batch node index
    const NodeRec nr = own.load(li);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double Xk = b.X[k * nt + gi];
      const double xk = Xk + (static_cast<double>(nr.hi[k]) + nr.lo[k]);
      b.x[k * nt + gi] = xk;
      if (a.update_coords) b.u[k * nt + gi] = xk - Xk;
    }
    if (i >= NF) {
      const int2 sr = __ldg(srow + i);
      float a0, a1, a2;
      nodal_force(r.L, u, nfc, sr.x, sr.y, nr, a0, a1, a2);
      b.fint[no + i] = a0;
      b.fint[nt + no + i] = a1;
      b.fint[2 * nt + no + i] = a2;
    }
  }
  Ops::sync();
  mixed_stress(b, a, rve, status, step, residual, red, rank == 0);
  Ops::sync();
}

// Persistent relaxation over one size bucket: CTA (or cluster) after cluster
// takes the next RVE of `order` (largest first) until the bucket is empty.
// With NG = 2 each half of the CTA is a group that takes RVEs on its own,
// in half of the shared memory, synchronised by its own named barrier.
template <int CL, bool kAll, bool kNodal, int NG, bool kDB>
__global__ void __launch_bounds__(kThreadsMixed, 1)
relax_mixed_kernel(const DevBatch b, const MixedState ms, const RunArgs a, int smem_floats,
                   const int32_t* order, int n_order, int32_t* queue) {
  static_assert(kNodal || CL == 1, "the fiber-centric solve runs on one CTA");
  static_assert(NG == 1 || (CL == 1 && kAll && !kNodal), "only small fiber-centric RVEs pair up");
  static_assert(!kDB || kNodal, "two record copies: node-centric solve");
  constexpr int kRed = kThreadsMixed / 32 + 1;
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  __shared__ double red[NG * kRed];
  __shared__ double cred[1];
  __shared__ int s_rve[NG];
  const int g = Group<NG>::index();
  for (;;) {
    if (ClusterOps<CL>::rank() == 0 && Group<NG>::tid() == 0) {
      const int w = atomicAdd(queue, 1);
      s_rve[g] = w < n_order ? order[w] : -1;
    }
    int rve;
    if constexpr (CL > 1) {
      cg::cluster_group cl = cg::this_cluster();
      cl.sync();
      rve = *cl.map_shared_rank(&s_rve[0], 0);
      cl.sync();
    } else {
      Group<NG>::sync();
      rve = s_rve[g];
      Group<NG>::sync();
    }
    if (rve < 0) break;
    if constexpr (kNodal)
      solve_rve_nodal<CL, kDB>(b, ms, a, rve, red, cred, smem);
    else
      solve_rve_mixed<kAll, NG>(b, ms, a, rve, red + g * kRed, smem + g * (smem_floats / NG),
                                smem_floats / NG);
  }
}

// One RVE solved by one CTA of a serving kernel: with the solve of its batch
// bucket where that is a single CTA with an order of its own, else with the
// run-time placement. Every solve gives the same bits.
__device__ __forceinline__ void serve_one_cta(const DevBatch& b, const MixedState& ms,
                                              const RunArgs& a, int rve, double* red, double* cred,
                                              float* smem, int smem_floats) {
  const int q = __ldg(ms.rve_bucket + rve);
  if (q == kQNodal1)
    solve_rve_nodal<1>(b, ms, a, rve, red, cred, smem);
  else if (q == kQNodalDB)
    solve_rve_nodal<1, true>(b, ms, a, rve, red, cred, smem);
  else if (q == kQFiberAll || q == kQFiberPair)
    solve_rve_mixed<true>(b, ms, a, rve, red, smem, smem_floats);
  else
    solve_rve_mixed<false>(b, ms, a, rve, red, smem, smem_floats);
}

__global__ void __launch_bounds__(kThreadsMixed, 1)
server_mixed_kernel(const DevBatch b, const MixedState ms, const ServerArgs sa, int smem_floats) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  __shared__ double red[kThreadsMixed / 32 + 1];
  __shared__ double cred[1];
  server_loop(sa, [&](const RunArgs& a, int rve) {
    serve_one_cta(b, ms, a, rve, red, cred, smem, smem_floats);
  });
}

// Serving kernel for batches with cluster-solved RVEs: persistent 4-CTA
// clusters. A cluster's leader (rank 0, thread 0) takes the next request of
// the large-RVE ring and the cluster solves it together; when that ring is
// empty and the small-RVE ring is not, the cluster's CTAs take small
// requests one by one, each solving on its own, until the small ring runs
// dry, a large request is waiting, or kSmallPerRound are done, and then meet
// at one cluster barrier. Every cluster barrier is reached by all CTAs the
// same number of times: every loop is bounded, and the decision to leave is
// taken by the leader and broadcast before anyone acts on it. Shutdown is
// collective as in server_loop, with clusters as the units.
constexpr int kClusterServe = 4;
constexpr int kSmallPerRound = 16;
enum : int { kServeExit = 0, kServeBig = 1, kServeSmall = 2 };

__global__ void __launch_bounds__(kThreadsMixed, 1)
server_cluster_kernel(const DevBatch b, const MixedState ms, const ServerArgs big,
                      const ServerArgs small, int smem_floats) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  __shared__ double red[kThreadsMixed / 32 + 1];
  __shared__ double cred[1];
  __shared__ long long s_idx;
  __shared__ double s_F[9];
  __shared__ int s_req[2];
  __shared__ int s_mode;
  __shared__ RunArgs s_args;  // read by the solves where needed, not held in registers
  __shared__ RunArgs s_args1;  // the perturbed solves of a request's stiffness
  cg::cluster_group cl = cg::this_cluster();
  const int rank = static_cast<int>(cl.block_rank());
  const int tid = threadIdx.x;
  const int units = static_cast<int>(gridDim.x) / kClusterServe;
  // Both rings share the per-RVE result arrays, so one RunArgs serves both;
  // only update_coords changes per request.
  if (tid == 0) {
    s_args.F = s_F;
    s_args.n_F = 1;
    s_args.update_coords = 0;
    s_args.sigma = big.sigma;
    s_args.st_status = big.st_status;
    s_args.st_steps = big.st_steps;
    s_args.st_residual = big.st_residual;
  }
  __syncthreads();
  for (;;) {
    // ---- the leader picks the cluster's next job --------------------------
    if (rank == 0 && tid == 0) {
      int mode = kServeExit;
      long long idx = -1;
      const unsigned long long t0 = global_ns();
      atomicAdd(big.idle_ctas, 1);
      for (long long polls = 0; polls < kServerMaxPolls; ++polls) {
        if (ld_gpu(big.stop) || ld_gpu(big.closing)) break;
        idx = server_try_claim(big);
        if (idx >= 0) {
          mode = kServeBig;
          break;
        }
        if (server_pending(small)) {
          mode = kServeSmall;
          break;
        }
        const unsigned long long now = global_ns();
        const unsigned long long last =
            *reinterpret_cast<volatile unsigned long long*>(big.last_claim);
        const unsigned long long since = last > t0 ? last : t0;
        if (now > since && now - since > big.idle_ns && ld_gpu(big.idle_ctas) == units) {
          atomicExch(big.closing, 1);
          break;
        }
        if (server_wait_expired(big, t0, now)) break;
        __nanosleep(2000);
      }
      atomicSub(big.idle_ctas, 1);
      if (mode == kServeBig) server_read_request(big, idx, s_req, s_F);
      s_mode = mode;
      s_idx = idx;
    }
    cl.sync();
    if (rank != 0) {
      // copy the leader's decision and request into this CTA
      if (tid == 0) s_mode = *cl.map_shared_rank(&s_mode, 0);
      if (tid == 1) s_idx = *cl.map_shared_rank(&s_idx, 0);
      if (tid >= 2 && tid < 4) s_req[tid - 2] = *cl.map_shared_rank(&s_req[tid - 2], 0);
      if (tid >= 4 && tid < 13) s_F[tid - 4] = *cl.map_shared_rank(&s_F[tid - 4], 0);
    }
    cl.sync();
    const int mode = s_mode;
    if (mode == kServeExit) return;
    if (mode == kServeBig) {
      const long long idx = s_idx;
      const int rve = s_req[0];
      const int flags = s_req[1];
      const unsigned long long t_claim = global_ns();
      if (tid == 0) s_args.update_coords = flags & kReqUpdate;
      __syncthreads();
      // the request's solve, then with kReqStiffness the six perturbed
      // solves of its stiffness, by the cluster
      const bool stiff = (flags & kReqStiffness) != 0;
      for (int k = 0; k <= (stiff ? 6 : 0); ++k) {
        if (k > 0) {
          if (tid == 0) s_args1 = stiffness_args(big, k - 1);
          __syncthreads();
        }
        solve_rve_nodal<kClusterServe>(b, ms, k == 0 ? s_args : s_args1, rve, red, cred,
                                       smem);  // ends with a cluster barrier
        if (k > 0) {
          if (rank == 0) stiffness_column(big, rve, k - 1);
          __syncthreads();
        }
      }
      if (rank == 0 && tid == 0) server_publish_done(big, idx, rve, t_claim, stiff);
      cl.sync();
      continue;
    }
    // ---- small requests, CTA by CTA ---------------------------------------
    for (int k = 0; k < kSmallPerRound; ++k) {
      if (tid == 0) {
        long long idx = -1;
        if (!ld_gpu(small.stop) && !ld_gpu(small.closing) && !server_pending(big))
          idx = server_try_claim(small);
        if (idx >= 0) {
          server_read_request(small, idx, s_req, s_F);
          s_args.update_coords = s_req[1] & kReqUpdate;
        }
        s_idx = idx;
      }
      __syncthreads();
      const long long idx = s_idx;
      const int rve = s_req[0];
      const int flags = s_req[1];
      __syncthreads();
      if (idx < 0) break;
      const unsigned long long t_claim = global_ns();
      const bool stiff = (flags & kReqStiffness) != 0;
      for (int j = 0; j <= (stiff ? 6 : 0); ++j) {
        if (j > 0) {
          if (tid == 0) s_args1 = stiffness_args(small, j - 1);
          __syncthreads();
        }
        serve_one_cta(b, ms, j == 0 ? s_args : s_args1, rve, red, cred, smem,
                      smem_floats);  // ends with __syncthreads()
        if (j > 0) {
          stiffness_column(small, rve, j - 1);
          __syncthreads();
        }
      }
      if (tid == 0) server_publish_done(small, idx, rve, t_claim, stiff);
      __syncthreads();
    }
    cl.sync();
  }
}

template <typename T>
cudaError_t alloc(T** p, size_t n) {
  return cudaMalloc(reinterpret_cast<void**>(p), (n > 0 ? n : 1) * sizeof(T));
}

}  // namespace

MixedState* mixed_new() { return new MixedState(); }

namespace {

void ctx_release(MixedRunCtx& c) {
  for (void* p : {static_cast<void*>(c.queues), static_cast<void*>(c.u_hl),
                  static_cast<void*>(c.v), static_cast<void*>(c.nrm)})
    if (p) cudaFree(p);
  if (c.graph) cudaGraphExecDestroy(c.graph);
  if (c.capture) cudaStreamDestroy(c.capture);
  for (int q = 0; q < kBuckets; ++q) {
    if (c.side[q]) cudaStreamDestroy(c.side[q]);
    if (c.join[q]) cudaEventDestroy(c.join[q]);
  }
  if (c.fork) cudaEventDestroy(c.fork);
  c = MixedRunCtx{};
}

// Creates run context `c` (claim counters, streams, events); with
// own_scratch, also its own run-time placement scratch, sized like the
// batch's.
cudaError_t ctx_init(MixedRunCtx& c, size_t nt, size_t et, bool own_scratch) {
  cudaError_t e;
  if ((e = cudaMalloc(reinterpret_cast<void**>(&c.queues), kBuckets * sizeof(int32_t))) !=
      cudaSuccess)
    return e;
  if (own_scratch) {
    if ((e = cudaMalloc(reinterpret_cast<void**>(&c.u_hl), 6 * std::max<size_t>(nt, 1) *
                                                              sizeof(float))) != cudaSuccess ||
        (e = cudaMalloc(reinterpret_cast<void**>(&c.v), 3 * std::max<size_t>(nt, 1) *
                                                           sizeof(float))) != cudaSuccess ||
        (e = cudaMalloc(reinterpret_cast<void**>(&c.nrm), std::max<size_t>(et, 1) *
                                                             sizeof(float4))) != cudaSuccess)
      return e;
  }
  for (int q = 0; q < kBuckets; ++q) {
    if ((e = cudaStreamCreateWithFlags(&c.side[q], cudaStreamNonBlocking)) != cudaSuccess)
      return e;
    if ((e = cudaEventCreateWithFlags(&c.join[q], cudaEventDisableTiming)) != cudaSuccess)
      return e;
  }
  if ((e = cudaEventCreateWithFlags(&c.fork, cudaEventDisableTiming)) != cudaSuccess) return e;
  if ((e = cudaStreamCreateWithFlags(&c.capture, cudaStreamNonBlocking)) != cudaSuccess) return e;
  c.ready = true;
  return cudaSuccess;
}

}  // namespace

void mixed_destroy(MixedState* ms) {
  if (!ms) return;
  if (ms->ctx) {
    for (int k = 0; k < kMixedContexts; ++k) ctx_release(ms->ctx[k]);
    delete[] ms->ctx;
  }
  for (void* p : {static_cast<void*>(ms->u_hl), static_cast<void*>(ms->econn),
                  static_cast<void*>(ms->icode), static_cast<void*>(ms->mslot),
                  static_cast<void*>(ms->gnode), static_cast<void*>(ms->mrowptr),
                  static_cast<void*>(ms->mmass), static_cast<void*>(ms->nsell),
                  static_cast<void*>(ms->sell_off), static_cast<void*>(ms->ncode),
                  static_cast<void*>(ms->nfc), static_cast<void*>(ms->nfib_tmp),
                  static_cast<void*>(ms->fconc),
                  static_cast<void*>(ms->v), static_cast<void*>(ms->mass),
                  static_cast<void*>(ms->fcon), static_cast<void*>(ms->nrm),
                  static_cast<void*>(ms->order), static_cast<void*>(ms->rve_bucket)})
    if (p) cudaFree(p);
  delete[] ms->h_cl;
  delete ms;
}

namespace {

// Bucket of an RVE: the smallest of one CTA or a cluster of 2, 4 or 8 CTAs
// whose shared memory holds its node state (node-centric solve; at that
// size with two copies of the node records where they fit), else one
// CTA that keeps what fits in shared memory and streams the rest from global
// memory (fiber-centric solve). Clusters of 8 are the last resort: with
// 220 KB per CTA only 15 of them (120 SMs) are resident at once, against 36
// clusters of 4 (144 SMs). Clusters above max_cluster CTAs are not used,
// nor clusters of 2 in the serving layout (the serving kernel solves in
// clusters of 4 only).
// With the fiber-centric small solve, RVEs whose whole state fits half a
// CTA's shared memory come first (two of them share a CTA, at most
// rves_per_cta), then those whose whole state fits one CTA; otherwise those
// buckets are skipped and every RVE whose node state fits takes the
// node-centric solve. small_solve (mfg_small_rve_solve) picks the solve;
// AUTO takes the fiber-centric one for RVEs on the nonlinear law, whose
// exponential the node-centric solve would evaluate at both ends of every
// fiber, and the node-centric one for the linear law, where it runs 2 %
// (500 - 1,300 nodes) to 37 % (1,300 - 3,300 nodes) faster.
int bucket_of(const RveDesc& d, int smem_floats, int max_cluster, bool serving_layout,
              int small_solve, int rves_per_cta) {
  const bool fiber_small =
      small_solve == MFG_SMALL_FIBER_CENTRIC ||
      (small_solve == MFG_SMALL_AUTO && d.law == MFG_LAW_NONLINEAR);
  for (int q : kPref)
    if ((fiber_small || !kBucket[q].all) && kBucket[q].cl <= max_cluster &&
        !(serving_layout && kBucket[q].cl == 2) && kBucket[q].ng <= rves_per_cta &&
        cluster_floats(d.n_nodes, d.n_free, d.n_fibers, kBucket[q].cl,
                       kBucket[q].all && !kBucket[q].nodal, kBucket[q].db) <=
            smem_floats / kBucket[q].ng)
      return q;
  return kBuckets - 1;
}

// Calls fn(std::integral_constant<int, q>{}) for the run-time bucket index q.
template <class Fn>
cudaError_t with_bucket(int q, Fn&& fn) {
  switch (q) {
    case 0: return fn(std::integral_constant<int, 0>{});
    case 1: return fn(std::integral_constant<int, 1>{});
    case 2: return fn(std::integral_constant<int, 2>{});
    case 3: return fn(std::integral_constant<int, 3>{});
    case 4: return fn(std::integral_constant<int, 4>{});
    case 5: return fn(std::integral_constant<int, 5>{});
    case 6: return fn(std::integral_constant<int, 6>{});
    case 7: return fn(std::integral_constant<int, 7>{});
    case 8: return fn(std::integral_constant<int, 8>{});
    case 9: return fn(std::integral_constant<int, 9>{});
    default: return cudaErrorInvalidValue;
  }
}
static_assert(kBuckets == 10, "with_bucket covers every bucket");

template <int CL, bool kAll>
cudaLaunchConfig_t launch_config(const MixedState& ms, unsigned grid, cudaStream_t s,
                                 cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid, 1, 1);
  cfg.blockDim = dim3(kThreadsMixed, 1, 1);
  cfg.dynamicSmemBytes = static_cast<size_t>(ms.smem_bytes);
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = CL > 1 ? 1 : 0;
  return cfg;
}

template <int Q>
cudaError_t launch_bucket(const MixedState& ms, const DevBatch& b, const RunArgs& a,
                          int32_t* queue, cudaStream_t s) {
  constexpr BucketKind k = kBucket[Q];
  const int n = ms.bucket_off[Q + 1] - ms.bucket_off[Q];
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg =
      launch_config<k.cl, k.all>(ms, static_cast<unsigned>(ms.bucket_grid[Q]), s, attr);
  return cudaLaunchKernelEx(&cfg, relax_mixed_kernel<k.cl, k.all, k.nodal, k.ng, k.db>, b, ms, a,
                            static_cast<int>(ms.smem_bytes / sizeof(float)),
                            static_cast<const int32_t*>(ms.order + ms.bucket_off[Q]), n, queue);
}

template <int Q>
cudaError_t setup_bucket(MixedState& ms, int n) {
  constexpr BucketKind k = kBucket[Q];
  cudaError_t e = cudaFuncSetAttribute(relax_mixed_kernel<k.cl, k.all, k.nodal, k.ng, k.db>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       ms.smem_bytes);
  if (e != cudaSuccess) return e;
  int clusters = ms.sms;
  if (k.cl > 1 && n > 0) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg =
        launch_config<k.cl, k.all>(ms, static_cast<unsigned>(k.cl * ms.sms), nullptr, attr);
    clusters = 0;
    if ((e = cudaOccupancyMaxActiveClusters(&clusters,
                                            relax_mixed_kernel<k.cl, k.all, k.nodal, k.ng, k.db>,
                                            &cfg)) != cudaSuccess)
      return e;
    if (clusters < 1) return cudaErrorInvalidConfiguration;
  }
  // CTAs (or clusters) for n RVEs at k.ng RVEs each, at most one per SM
  ms.bucket_grid[Q] = k.cl * std::min((n + k.ng - 1) / k.ng, clusters);
  return cudaSuccess;
}

}  // namespace

cudaError_t mixed_create(MixedState& ms, const DevBatch& b, const std::vector<RveDesc>& desc,
                         const std::vector<int2>& conn, const std::vector<int32_t>& rowptr,
                         const std::vector<int32_t>& inc, int sms, int max_cluster,
                         bool serving_layout, int small_solve, int rves_per_cta,
                         cudaStream_t s) {
  cudaError_t e;
  const size_t nt = static_cast<size_t>(b.nt), et = static_cast<size_t>(b.et);
  if ((e = alloc(&ms.u_hl, 6 * nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.v, 3 * nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.mass, nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.fcon, et)) != cudaSuccess) return e;
  if ((e = alloc(&ms.nrm, et)) != cudaSuccess) return e;
  if ((e = alloc(&ms.econn, et)) != cudaSuccess) return e;
  if ((e = alloc(&ms.fconc, et)) != cudaSuccess) return e;
  if ((e = alloc(&ms.icode, 2 * et)) != cudaSuccess) return e;
  if ((e = alloc(&ms.mslot, et)) != cudaSuccess) return e;
  if ((e = alloc(&ms.gnode, nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.mrowptr, rowptr.size())) != cudaSuccess) return e;
  if ((e = alloc(&ms.mmass, nt)) != cudaSuccess) return e;
  if ((e = alloc(&ms.order, desc.size())) != cudaSuccess) return e;
  ms.ctx = new MixedRunCtx[kMixedContexts];
  if ((e = ctx_init(ms.ctx[0], nt, et, false)) != cudaSuccess) return e;
  ms.sms = sms;
  ms.smem_bytes = kSmemBytesMixed;
  const int smem_floats = kSmemBytesMixed / static_cast<int>(sizeof(float));
  if ((e = cudaFuncSetAttribute(server_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                kSmemBytesMixed)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(server_cluster_kernel,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytesMixed)) !=
          cudaSuccess)
    return e;
  {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = launch_config<kClusterServe, false>(
        ms, static_cast<unsigned>(kClusterServe * sms), nullptr, attr);
    int clusters = 0;
    if ((e = cudaOccupancyMaxActiveClusters(&clusters, server_cluster_kernel, &cfg)) !=
        cudaSuccess)
      return e;
    ms.server_grid = kClusterServe * clusters;
  }

  // size buckets, each in longest-processing-time order
  std::vector<std::vector<int32_t>> bucket(kBuckets);
  std::vector<int> rve_q(desc.size());
  ms.h_cl = new int32_t[std::max<size_t>(desc.size(), 1)];
  for (size_t r = 0; r < desc.size(); ++r) {
    rve_q[r] = bucket_of(desc[r], smem_floats, max_cluster, serving_layout, small_solve,
                         rves_per_cta);
    bucket[rve_q[r]].push_back(static_cast<int32_t>(r));
    ms.h_cl[r] = kBucket[rve_q[r]].cl;
  }
  if ((e = alloc(&ms.rve_bucket, desc.size())) != cudaSuccess ||
      (!desc.empty() &&
       (e = cudaMemcpy(ms.rve_bucket, rve_q.data(), desc.size() * sizeof(int32_t),
                       cudaMemcpyHostToDevice)) != cudaSuccess))
    return e;
  {
    // fiber order and codes of the cluster-solved RVEs
    std::vector<int2> econn(et);
    std::vector<int32_t> icode(2 * et), mslot(et), gnode(nt), mrowptr(rowptr.size());
    std::vector<std::thread> pool;
    const int nthr = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    for (int t = 0; t < nthr; ++t)
      pool.emplace_back([&, t] {
        for (size_t r = t; r < desc.size(); r += nthr)
          cluster_order(desc[r], kBucket[rve_q[r]].cl,
                        kBucket[rve_q[r]].all || kBucket[rve_q[r]].nodal,
                        kBucket[rve_q[r]].nodal, conn, rowptr, inc, econn, icode, mslot, gnode,
                        mrowptr);
      });
    for (auto& th : pool) th.join();
    if ((e = cudaMemcpy(ms.econn, econn.data(), et * sizeof(int2), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (e = cudaMemcpy(ms.icode, icode.data(), 2 * et * sizeof(int32_t),
                        cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(ms.mslot, mslot.data(), et * sizeof(int32_t), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (e = cudaMemcpy(ms.gnode, gnode.data(), nt * sizeof(int32_t), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (e = cudaMemcpy(ms.mrowptr, mrowptr.data(), mrowptr.size() * sizeof(int32_t),
                        cudaMemcpyHostToDevice)) != cudaSuccess)
      return e;

    // SELL incidence blocks of the node-centric RVEs
    std::vector<int64_t> sell_off(desc.size() + 1, 0);
    {
      std::vector<std::thread> sp;
      for (int t = 0; t < nthr; ++t)
        sp.emplace_back([&, t] {
          for (size_t r = t; r < desc.size(); r += nthr)
            if (kBucket[rve_q[r]].nodal)
              sell_off[r + 1] = sell_layout(desc[r], kBucket[rve_q[r]].cl, conn, rowptr, inc,
                                            gnode, 0, nullptr, nullptr, nullptr);
        });
      for (auto& th : sp) th.join();
    }
    for (size_t r = 0; r < desc.size(); ++r) sell_off[r + 1] += sell_off[r];
    const int64_t n_sell = sell_off[desc.size()];
    ms.n_sell = n_sell;
    std::vector<int2> nsell(nt, make_int2(0, 0));
    std::vector<int32_t> ncode(static_cast<size_t>(n_sell), 0);
    std::vector<int64_t> nfib(static_cast<size_t>(n_sell), -1);
    {
      std::vector<std::thread> sp;
      for (int t = 0; t < nthr; ++t)
        sp.emplace_back([&, t] {
          for (size_t r = t; r < desc.size(); r += nthr)
            if (kBucket[rve_q[r]].nodal)
              sell_layout(desc[r], kBucket[rve_q[r]].cl, conn, rowptr, inc, gnode, sell_off[r],
                          nsell.data(), ncode.data(), nfib.data());
        });
      for (auto& th : sp) th.join();
    }
    if ((e = alloc(&ms.nsell, nt)) != cudaSuccess ||
        (e = alloc(&ms.sell_off, desc.size())) != cudaSuccess ||
        (e = alloc(&ms.ncode, static_cast<size_t>(n_sell))) != cudaSuccess ||
        (e = alloc(&ms.nfc, static_cast<size_t>(n_sell))) != cudaSuccess ||
        (e = alloc(&ms.nfib_tmp, static_cast<size_t>(n_sell))) != cudaSuccess)
      return e;
    if ((e = cudaMemcpy(ms.nsell, nsell.data(), nt * sizeof(int2), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (!desc.empty() &&
         (e = cudaMemcpy(ms.sell_off, sell_off.data(), desc.size() * sizeof(int64_t),
                         cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (n_sell > 0 &&
         ((e = cudaMemcpy(ms.ncode, ncode.data(), n_sell * sizeof(int32_t),
                          cudaMemcpyHostToDevice)) != cudaSuccess ||
          (e = cudaMemcpy(ms.nfib_tmp, nfib.data(), n_sell * sizeof(int64_t),
                          cudaMemcpyHostToDevice)) != cudaSuccess)))
      return e;
  }
  std::vector<int32_t> order;
  order.reserve(desc.size());
  for (int q = 0; q < kBuckets; ++q) {
    std::stable_sort(bucket[q].begin(), bucket[q].end(),
                     [&](int32_t x, int32_t y) { return desc[x].n_fibers > desc[y].n_fibers; });
    ms.bucket_off[q] = static_cast<int>(order.size());
    order.insert(order.end(), bucket[q].begin(), bucket[q].end());
  }
  ms.bucket_off[kBuckets] = static_cast<int>(order.size());
  if (!order.empty() &&
      (e = cudaMemcpy(ms.order, order.data(), order.size() * sizeof(int32_t),
                      cudaMemcpyHostToDevice)) != cudaSuccess)
    return e;
  for (int q = 0; q < kBuckets; ++q) {
    const int n = ms.bucket_off[q + 1] - ms.bucket_off[q];
    e = with_bucket(q, [&](auto Q) { return setup_bucket<decltype(Q)::value>(ms, n); });
    if (e != cudaSuccess) return e;
  }

  const int64_t n = std::max<int64_t>(b.nt, 1);
  mixed_prepare_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(b, ms);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  mixed_prepare_order_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(b, ms);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  int max_e = 1;
  for (const RveDesc& d : desc) max_e = std::max(max_e, d.n_fibers);
  dim3 grid(static_cast<unsigned>((max_e + 255) / 256),
            static_cast<unsigned>(std::min(b.n_rve, 65535)));
  mixed_prepare_fibers_kernel<<<grid, 256, 0, s>>>(b, ms);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (ms.n_sell > 0) {
    mixed_prepare_sell_kernel<<<static_cast<unsigned>((ms.n_sell + 255) / 256), 256, 0, s>>>(
        ms, ms.ncode, ms.nfib_tmp, ms.n_sell);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  // the fiber ids were only needed to fill the incidences' fiber data
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  cudaFree(ms.nfib_tmp);
  ms.nfib_tmp = nullptr;
  cudaFree(ms.ncode);
  ms.ncode = nullptr;
  return cudaSuccess;
}

int mixed_rve_cluster(const MixedState& ms, int rve) { return ms.h_cl ? ms.h_cl[rve] : 1; }

bool mixed_serves_in_clusters(const MixedState& ms, int rve) {
  return mixed_rve_cluster(ms, rve) == kClusterServe;
}

cudaError_t launch_server_mixed(MixedState& ms, const DevBatch& b, const ServerArgs& small,
                                const ServerArgs* big, cudaStream_t s) {
  const int smem_floats = static_cast<int>(ms.smem_bytes / sizeof(float));
  if (!big) {
    server_mixed_kernel<<<ms.sms, kThreadsMixed, ms.smem_bytes, s>>>(b, ms, small, smem_floats);
    return cudaGetLastError();
  }
  if (ms.server_grid < kClusterServe) return cudaErrorInvalidConfiguration;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg =
      launch_config<kClusterServe, false>(ms, static_cast<unsigned>(ms.server_grid), s, attr);
  return cudaLaunchKernelEx(&cfg, server_cluster_kernel, b, ms, *big, small, smem_floats);
}

namespace {

// One launch per non-empty size bucket, each on its own stream of context
// `c` so that the buckets run concurrently: the largest clusters are
// launched first, and the CTAs of the later buckets take over SMs as the
// earlier buckets drain.
cudaError_t enqueue_buckets(const MixedState& ms, MixedRunCtx& c, const DevBatch& b,
                            const RunArgs& a, cudaStream_t s, int* launches) {
  cudaError_t e;
  *launches = 0;
  if ((e = cudaMemsetAsync(c.queues, 0, kBuckets * sizeof(int32_t), s)) != cudaSuccess) return e;
  if ((e = cudaEventRecord(c.fork, s)) != cudaSuccess) return e;
  for (int q = 0; q < kBuckets; ++q) {
    if (ms.bucket_off[q + 1] == ms.bucket_off[q]) continue;
    cudaStream_t sq = c.side[q];
    if ((e = cudaStreamWaitEvent(sq, c.fork, 0)) != cudaSuccess) return e;
    int32_t* queue = c.queues + q;
    e = with_bucket(q, [&](auto Q) {
      return launch_bucket<decltype(Q)::value>(ms, b, a, queue, sq);
    });
    if (e != cudaSuccess) return e;
    ++*launches;
    if ((e = cudaEventRecord(c.join[q], sq)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(s, c.join[q], 0)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

bool same_args(const RunArgs& x, const RunArgs& y) {
  return x.F == y.F && x.n_F == y.n_F && x.update_coords == y.update_coords &&
         x.sigma == y.sigma && x.st_status == y.st_status && x.st_steps == y.st_steps &&
         x.st_residual == y.st_residual;
}

}  // namespace

cudaError_t mixed_prepare_contexts(MixedState& ms, const DevBatch& b, int n) {
  if (n >= kMixedContexts) return cudaErrorInvalidValue;
  // the run-time placement keeps node records, velocities and force vectors
  // in global memory: concurrent runs need their own
  const bool runtime_bucket = ms.bucket_off[kBuckets] > ms.bucket_off[kBuckets - 1];
  for (int k = 1; k <= n; ++k) {
    if (ms.ctx[k].ready) continue;
    cudaError_t e = ctx_init(ms.ctx[k], static_cast<size_t>(b.nt), static_cast<size_t>(b.et),
                             runtime_bucket);
    if (e != cudaSuccess) {
      ctx_release(ms.ctx[k]);
      return e;
    }
  }
  return cudaSuccess;
}

// A run replays context k's captured graph when the arguments (the batch
// view's coordinates, device pointers and flags) are those it was captured
// with; otherwise the bucket launches are captured on the context's private
// stream into a new graph first.
cudaError_t run_mixed(MixedState& ms, const DevBatch& b, const RunArgs& a, cudaStream_t s,
                      int* launches, int k) {
  if (k < 0 || k >= kMixedContexts || !ms.ctx[k].ready) return cudaErrorInvalidValue;
  MixedRunCtx& c = ms.ctx[k];
  cudaError_t e;
  if (!c.graph || !same_args(c.graph_args, a) || c.graph_x != b.x) {
    MixedState msc = ms;  // the kernels' view: this context's run-time scratch
    if (c.u_hl) {
      msc.u_hl = c.u_hl;
      msc.v = c.v;
      msc.nrm = c.nrm;
    }
    if ((e = cudaStreamBeginCapture(c.capture, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
      return e;
    int n = 0;
    const cudaError_t ec = enqueue_buckets(msc, c, b, a, c.capture, &n);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(c.capture, &g);
    if (ec != cudaSuccess || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return ec != cudaSuccess ? ec : e;
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return e;
    if (c.graph) cudaGraphExecDestroy(c.graph);
    c.graph = exec;
    c.graph_args = a;
    c.graph_x = b.x;
    c.graph_launches = n;
  }
  *launches = c.graph_launches;
  return cudaGraphLaunch(c.graph, s);
}

}  // namespace mfg
