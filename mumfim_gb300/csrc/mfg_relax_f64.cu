// Plain FP64 relaxation kernel: one persistent CTA solves one RVE at a time.
//
// Restates, in one launch, the reference's affine predictor
// (src/mumfim/microscale/batched_analysis/BatchedFiberRVEAnalysisExplicitBase.h:16-57),
// volume update (same file :127-154), the three TeamOuterLoop kernels
// (src/mumfim/microscale/batched_analysis/BatchedFiberRVEAnalysisExplicitTeamOuterLoop.h:215-434)
// and the Cauchy stress (BatchedFiberRVEAnalysisExplicitBase.h:58-126).
//
// Bit-exactness with a serial run of the same algorithm:
//  - this file is compiled with --fmad=false and every expression keeps the
//    reference's operation order; division and sqrt are IEEE (nvcc default);
//  - nodal forces are gathered node by node over a CSR list of incident
//    fibers in ascending fiber id, which adds the per-fiber force vectors in
//    exactly the order the serial scatter f_int[n1] -= t; f_int[n2] += t
//    does, instead of the reference's nondeterministic global atomics;
//  - the stress is summed by six threads, one per Voigt component, in
//    boundary-list order.
// Only the residual norm uses a tree reduction; it decides when to stop and
// is compared against the tolerance, never written into the state.
//
// Step structure. The reference's step s is
//   kick(h_s) + drift | lengths | forces | kick(h_s)
// with a barrier between each. The trailing kick of step s and the leading
// kick + drift of step s+1 touch only node-local data, so they are fused into
// one node pass that starts by gathering the forces of step s:
//   node pass  : f = gather(nrm); v += h_s f/m; v += h_{s+1} f/m; x += 2h_{s+1} v
//   fiber pass : l = |x2 - x1|; T = law(l0, l); nrm = (x2 - x1) * (T / l)
// giving two block barriers per step.
#include <cfloat>
#include <climits>

#include "mumfim_gpu.h"

#include "mfg_common.cuh"
#include "mfg_internal.h"

namespace mfg {
namespace {

constexpr int kThreadsF64 = 256;

// BatchedFiberRVEAnalysisExplicitBase.h:155-172
__device__ __forceinline__ double linear_force(double orig_length, double length, double E,
                                               double A) {
  double length_ratio = length / orig_length;
  double green_strain = 1.0 / 2.0 * (length_ratio * length_ratio - 1);
  return length_ratio * E * A * green_strain;
}

// NonlinearReaction::forceReaction().first (src/mumfim/microscale/FiberReactions.cc:16-71),
// compressive transition ratio 1.0 (FiberNetworkIO_impl.h:35).
__device__ __forceinline__ double nl_force(double alpha, double B, double lr, double gs) {
  return alpha * lr * (exp(B * gs) - 1);
}
__device__ __forceinline__ double nl_deriv(double alpha, double B, double lr, double l0,
                                           double gs) {
  return alpha / l0 * ((1 + lr * lr * B) * exp(B * gs) - 1);
}
__device__ __forceinline__ double nonlinear_force(double orig_length, double length, double E,
                                                  double A, double B, double lt) {
  const double cmp = 1.0;
  double length_ratio = length / orig_length;
  double alpha = E * A / B;
  if (length_ratio > lt) {
    double gt = 1.0 / 2.0 * (lt * lt - 1);
    double m = nl_deriv(alpha, B, lt, orig_length, gt);
    double b = nl_force(alpha, B, lt, gt);
    return m * (length_ratio - lt) * orig_length + b;
  } else if (length_ratio < cmp) {
    double gc = 1.0 / 2.0 * (cmp * cmp - 1);
    double m = nl_deriv(alpha, B, cmp, orig_length, gc);
    double b = nl_force(alpha, B, cmp, gc);
    return m * (length_ratio - cmp) * orig_length + b;
  }
  double gs = 1.0 / 2.0 * (length_ratio * length_ratio - 1);
  return nl_force(alpha, B, length_ratio, gs);
}

struct RveView {
  const double *X0, *X1, *X2;
  double *x0, *x1, *x2, *u0, *u1, *u2, *v0, *v1, *v2;
  const double* m;
  const int2* conn;
  const double* l0;
  double *n0, *n1, *n2;
  double *fi0, *fi1, *fi2;
  const int32_t* rowptr;
  const int32_t* inc;
  double* ramp;
};

__device__ __forceinline__ RveView make_view(const DevBatch& b, const RveDesc& d) {
  RveView r;
  const int64_t nt = b.nt, et = b.et, no = d.node_off, fo = d.fiber_off;
  r.X0 = b.X + no; r.X1 = b.X + nt + no; r.X2 = b.X + 2 * nt + no;
  r.x0 = b.x + no; r.x1 = b.x + nt + no; r.x2 = b.x + 2 * nt + no;
  r.u0 = b.u + no; r.u1 = b.u + nt + no; r.u2 = b.u + 2 * nt + no;
  r.v0 = b.v + no; r.v1 = b.v + nt + no; r.v2 = b.v + 2 * nt + no;
  r.fi0 = b.fint + no; r.fi1 = b.fint + nt + no; r.fi2 = b.fint + 2 * nt + no;
  r.m = b.m + no;
  r.conn = b.conn + fo;
  r.l0 = b.l0 + fo;
  r.n0 = b.nrm + fo; r.n1 = b.nrm + et + fo; r.n2 = b.nrm + 2 * et + fo;
  r.rowptr = b.rowptr + d.row_off;
  r.inc = b.inc + d.inc_off;
  r.ramp = b.ramp + 6 * d.bnd_off;
  return r;
}

// f_int of node i: incident fiber vectors in ascending fiber id, subtracted at
// the fiber's first node and added at its second
// (BatchedFiberRVEAnalysisExplicitBase.h:246-251 in serial order).
__device__ __forceinline__ void gather_fint(const RveView& r, int i, double& a0, double& a1,
                                            double& a2) {
  a0 = 0.0; a1 = 0.0; a2 = 0.0;
  const int pb = r.rowptr[i], pe = r.rowptr[i + 1];
  for (int p = pb; p < pe; ++p) {
    const int code = __ldg(r.inc + p);
    const int e = code >> 1;
    const double t0 = r.n0[e], t1 = r.n1[e], t2 = r.n2[e];
    if (code & 1) {
      a0 = a0 + t0; a1 = a1 + t1; a2 = a2 + t2;
    } else {
      a0 = a0 - t0; a1 = a1 - t1; a2 = a2 - t2;
    }
  }
}

// Fiber pass: lengths, reaction force and per-fiber force vector
// (TeamOuterLoop.h:53-82 and BatchedFiberRVEAnalysisExplicitBase.h:203-252).
// Returns this thread's minimum length.
__device__ __forceinline__ double fiber_pass(const RveView& r, const RveDesc& d) {
  double lmin = DBL_MAX;
  for (int e = threadIdx.x; e < d.n_fibers; e += kThreadsF64) {
    const int2 c = __ldg(r.conn + e);
    const double d0 = r.x0[c.y] - r.x0[c.x];
    const double d1 = r.x1[c.y] - r.x1[c.x];
    const double d2 = r.x2[c.y] - r.x2[c.x];
    const double l = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    lmin = fmin(lmin, l);
    const double l0 = __ldg(r.l0 + e);
    const double frc = d.law == 1 ? nonlinear_force(l0, l, d.E, d.A, d.B, d.lt)
                                  : linear_force(l0, l, d.E, d.A);
    const double frc_ovr_l = frc / l;
    r.n0[e] = d0 * frc_ovr_l;
    r.n1[e] = d1 * frc_ovr_l;
    r.n2[e] = d2 * frc_ovr_l;
  }
  return lmin;
}

__device__ void solve_rve(const DevBatch& b, const RunArgs& a, int rve, double* red) {
  const RveDesc d = b.desc[rve];
  const RveView r = make_view(b, d);
  const int N = d.n_nodes, NF = d.n_free;
  const int tid = threadIdx.x;
  const double* F = a.F + 9 * (a.n_F > 1 ? rve : 0);
  const bool ramp = d.mode == 1;
  double Fm[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Fm[k] = F[k];
  // updateVolume (BatchedFiberRVEAnalysisExplicit.h:271)
  if (a.update_coords && tid == 0) b.vol[rve] = jacobian(Fm) * b.vol[rve];

  // ---- prologue: predictor (RELAX), x = X + u, v = 0, RAMP increments ----
  for (int i = tid; i < N; i += kThreadsF64) {
    const double xo0 = r.x0[i], xo1 = r.x1[i], xo2 = r.x2[i];
    double up0 = r.u0[i], up1 = r.u1[i], up2 = r.u2[i];
    if (!ramp) {
      up0 = (Fm[0] - 1) * xo0 + (Fm[1] - 0) * xo1 + (Fm[2] - 0) * xo2 + up0;
      up1 = (Fm[3] - 0) * xo0 + (Fm[4] - 1) * xo1 + (Fm[5] - 0) * xo2 + up1;
      up2 = (Fm[6] - 0) * xo0 + (Fm[7] - 0) * xo1 + (Fm[8] - 1) * xo2 + up2;
    }
    const double xn0 = r.X0[i] + up0, xn1 = r.X1[i] + up1, xn2 = r.X2[i] + up2;
    r.x0[i] = xn0; r.x1[i] = xn1; r.x2[i] = xn2;
    r.v0[i] = 0.0; r.v1[i] = 0.0; r.v2[i] = 0.0;
    if (ramp && i >= NF) {
      double* rb = r.ramp + 6 * (i - NF);
      rb[0] = xn0; rb[1] = xn1; rb[2] = xn2;
      rb[3] = (Fm[0] - 1) * xn0 + (Fm[1] - 0) * xn1 + (Fm[2] - 0) * xn2;
      rb[4] = (Fm[3] - 0) * xn0 + (Fm[4] - 1) * xn1 + (Fm[5] - 0) * xn2;
      rb[5] = (Fm[6] - 0) * xn0 + (Fm[7] - 0) * xn1 + (Fm[8] - 1) * xn2;
    }
  }
  __syncthreads();

  // ---- RunInitialization: lengths, dt_crit, first forces -----------------
  double dt_crit = block_min<kThreadsF64>(fiber_pass(r, d), red) / d.sound_speed;

  // ---- main loop ---------------------------------------------------------
  const int cap = d.max_steps;  // host resolves the default cap for RELAX
  int step = 0;
  double residual = 10.0;
  double h_prev = 0.0;
  int status = 0;
  for (;;) {
    // `step` steps are complete. Every UPDATE_FREQ steps the residual of the
    // last step's forces is refreshed (TeamOuterLoop.h:119-133); the loop
    // condition is the reference's (TeamOuterLoop.h:371) plus the step cap.
    const bool res_step = step > 0 && ((step - 1) % kUpdateFreq) == 0;
    if (res_step) {
      double part = 0.0;
      for (int i = tid; i < NF; i += kThreadsF64) {
        double a0, a1, a2;
        gather_fint(r, i, a0, a1, a2);
        const double l0r = -a0, l1r = -a1, l2r = -a2;
        part += l0r * l0r + l1r * l1r + l2r * l2r;
      }
      residual = sqrt(block_sum<kThreadsF64>(part, red));
      if (!isfinite(residual)) {
        status = 4;  // MFG_E_NONFINITE
        break;
      }
    }
    if (!ramp && res_step && !(residual > d.tol)) break;
    if (step >= cap) break;  // RAMP: exactly max_steps steps; RELAX: cap reached
    const double h = d.crit * dt_crit * 0.5;  // TeamOuterLoop.h:345
    // node pass: trailing kick of step-1, leading kick + drift of step
    for (int i = tid; i < NF; i += kThreadsF64) {
      double a0, a1, a2;
      gather_fint(r, i, a0, a1, a2);
      const double mass = r.m[i];
      const double mc = mass * d.c;
      double w0 = r.v0[i], w1 = r.v1[i], w2 = r.v2[i];
      // f = -f_int - c m v (BatchedFiberRVEAnalysisExplicitBase.h:253-274)
      const double f0 = -a0 - mc * w0;
      const double f1 = -a1 - mc * w1;
      const double f2 = -a2 - mc * w2;
      if (step > 0) {  // updateAccelVel (BatchedFiberRVEAnalysisExplicitBase.h:275-287)
        w0 += h_prev * f0 / mass;
        w1 += h_prev * f1 / mass;
        w2 += h_prev * f2 / mass;
      }
      // updates (TeamOuterLoop.h:157-175)
      w0 = w0 + h * f0 / mass;
      w1 = w1 + h * f1 / mass;
      w2 = w2 + h * f2 / mass;
      r.v0[i] = w0; r.v1[i] = w1; r.v2[i] = w2;
      r.x0[i] = r.x0[i] + 2 * h * w0;
      r.x1[i] = r.x1[i] + 2 * h * w1;
      r.x2[i] = r.x2[i] + 2 * h * w2;
    }
    if (ramp) {
      const double alpha = static_cast<double>(step + 1) / static_cast<double>(d.max_steps);
      for (int i = NF + tid; i < N; i += kThreadsF64) {
        const double* rb = r.ramp + 6 * (i - NF);
        r.x0[i] = rb[0] + alpha * rb[3];
        r.x1[i] = rb[1] + alpha * rb[4];
        r.x2[i] = rb[2] + alpha * rb[5];
      }
    }
    __syncthreads();
    const double lmin = fiber_pass(r, d);
    if (step % kUpdateFreq == 0) {
      dt_crit = block_min<kThreadsF64>(lmin, red) / d.sound_speed;
    } else {
      __syncthreads();
    }
    h_prev = h;
    ++step;
  }
  if (status == 0 && !ramp && residual > d.tol) status = 3;  // MFG_E_NOT_CONVERGED

  // ---- FinalizeData: boundary f_int, u = x - X -----------------------------
  for (int i = NF + tid; i < N; i += kThreadsF64) {
    double a0, a1, a2;
    gather_fint(r, i, a0, a1, a2);
    r.fi0[i] = a0; r.fi1[i] = a1; r.fi2[i] = a2;
  }
  if (a.update_coords) {
    for (int i = tid; i < N; i += kThreadsF64) {
      r.u0[i] = r.x0[i] - r.X0[i];
      r.u1[i] = r.x1[i] - r.X1[i];
      r.u2[i] = r.x2[i] - r.X2[i];
    }
  }
  __syncthreads();
  // ---- computeCauchyStress: one thread per Voigt component, serial order --
  if (tid < 6) {
    double s = 0.0;
    const int k = tid;
    const int32_t* bo = b.bnd + d.bnd_off;
    for (int q = 0; q < N - NF; ++q) {
      const int i = bo[q];
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
  // status word: any thread of the first warp that saw a non-finite stress
  const unsigned bad = __ballot_sync(0xffffffffu, tid < 32 && status == 4);
  if (tid == 0) {
    a.st_status[rve] = bad ? 4 : status;
    a.st_steps[rve] = step;
    a.st_residual[rve] = residual;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kThreadsF64) relax_f64_kernel(const DevBatch b, const RunArgs a) {
  __shared__ double red[kThreadsF64 / 32 + 1];
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
    solve_rve(b, a, rve, red);
  }
}

__global__ void __launch_bounds__(kThreadsF64) server_f64_kernel(const DevBatch b,
                                                                 const ServerArgs sa) {
  __shared__ double red[kThreadsF64 / 32 + 1];
  server_loop(sa, [&](const RunArgs& a, int rve) { solve_rve(b, a, rve, red); });
}

}  // namespace

cudaError_t launch_server_f64(const DevBatch& b, const ServerArgs& sa, int grid, cudaStream_t s) {
  server_f64_kernel<<<grid, kThreadsF64, 0, s>>>(b, sa);
  return cudaGetLastError();
}

cudaError_t launch_relax_f64(const DevBatch& b, const RunArgs& a, int threads, int grid,
                             cudaStream_t s) {
  (void)threads;
  relax_f64_kernel<<<grid, kThreadsF64, 0, s>>>(b, a);
  return cudaGetLastError();
}

int relax_f64_max_blocks_per_sm(int threads) {
  (void)threads;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, relax_f64_kernel, kThreadsF64, 0) !=
      cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

// ---- fixed-scratch variant ---------------------------------------------------
// The same relaxation kernel, with every scratch buffer it writes (per-fiber
// force vectors, internal forces, RAMP boundary data, the work counter and the
// per-RVE status words) carved out of one file-scope device array instead of
// buffers allocated with the batch. Every GPU that loads this library holds
// the array until the process exits; all calls on a device share it.
static __device__ __align__(256) unsigned char g_relax_scratch[MFG_NOALLOC_SCRATCH_BYTES];

namespace {

inline size_t align256(size_t n) { return (n + 255) & ~static_cast<size_t>(255); }

}  // namespace

// Device address of the scratch array on the current device. The host-side
// symbol is only a stand-in for it. Looking the address up also loads this
// file's device code on the device if it is not loaded yet (CUDA loads
// modules lazily), and loading it is what reserves the array, so batch
// creation calls this once ahead of any solve. The lookup is repeated on
// every solve rather than cached, so an address never outlives the context
// it belongs to; once the module is loaded the lookup allocates nothing.
cudaError_t relax_f64_static_scratch_address(void** addr) {
  *addr = nullptr;
  return cudaGetSymbolAddress(addr, g_relax_scratch);
}

size_t relax_f64_static_scratch_bytes(const DevBatch& b, int64_t n_boundary_total) {
  const size_t R = static_cast<size_t>(b.n_rve);
  return align256(sizeof(int32_t)) + align256(R * sizeof(int32_t)) * 2 +
         align256(R * sizeof(double)) + align256(3 * static_cast<size_t>(b.et) * sizeof(double)) +
         align256(3 * static_cast<size_t>(b.nt) * sizeof(double)) +
         align256(6 * static_cast<size_t>(n_boundary_total > 0 ? n_boundary_total : 1) *
                  sizeof(double));
}

cudaError_t launch_relax_f64_static(const DevBatch& batch, const RunArgs& args, int grid,
                                    int64_t n_boundary_total, cudaStream_t s,
                                    StaticStatus* status) {
  if (relax_f64_static_scratch_bytes(batch, n_boundary_total) > MFG_NOALLOC_SCRATCH_BYTES)
    return cudaErrorInvalidValue;
  void* addr = nullptr;
  cudaError_t e = relax_f64_static_scratch_address(&addr);
  if (e != cudaSuccess) return e;
  unsigned char* base = static_cast<unsigned char*>(addr);
  const size_t R = static_cast<size_t>(batch.n_rve);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char* p = base + off;
    off += align256(bytes);
    return p;
  };
  DevBatch b = batch;
  RunArgs a = args;
  b.queue = reinterpret_cast<int32_t*>(take(sizeof(int32_t)));
  a.st_status = reinterpret_cast<int32_t*>(take(R * sizeof(int32_t)));
  a.st_steps = reinterpret_cast<int32_t*>(take(R * sizeof(int32_t)));
  a.st_residual = reinterpret_cast<double*>(take(R * sizeof(double)));
  b.nrm = reinterpret_cast<double*>(take(3 * static_cast<size_t>(b.et) * sizeof(double)));
  b.fint = reinterpret_cast<double*>(take(3 * static_cast<size_t>(b.nt) * sizeof(double)));
  b.ramp = reinterpret_cast<double*>(
      take(6 * static_cast<size_t>(n_boundary_total > 0 ? n_boundary_total : 1) * sizeof(double)));
  // The work counter is the only scratch read before it is written.
  e = cudaMemsetAsync(b.queue, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return e;
  relax_f64_kernel<<<grid, kThreadsF64, 0, s>>>(b, a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  status->status = a.st_status;
  status->steps = a.st_steps;
  status->residual = a.st_residual;
  return cudaSuccess;
}

}  // namespace mfg
