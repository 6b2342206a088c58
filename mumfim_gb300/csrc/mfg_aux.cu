// Orientation tensors and status packing.
#include "mfg_common.cuh"
#include "mfg_internal.h"
#include "mumfim_gpu.h"

namespace mfg {
namespace {

constexpr int kThreadsOrient = 256;

// Mean n (x) n over the fibers of one RVE in the current configuration
// (src/mumfim/microscale/batched_analysis/BatchedComputeOrientationTensor.h:145-186);
// with a normal, fiber directions are first projected onto the plane it
// defines (same file :55-144), after the reference's division of the normal
// by its squared length. Partial sums use a fixed-order block reduction
// instead of the reference's shared-memory atomics.
__global__ void __launch_bounds__(kThreadsOrient)
orientation_kernel(const DevBatch b, const double* normal, double* omega) {
  __shared__ double red[kThreadsOrient / 32 + 1];
  const int rve = blockIdx.x;
  const RveDesc d = b.desc[rve];
  const double* x0 = b.x + d.node_off;
  const double* x1 = b.x + b.nt + d.node_off;
  const double* x2 = b.x + 2 * b.nt + d.node_off;
  double nv0 = 0, nv1 = 0, nv2 = 0;
  if (normal) {
    nv0 = normal[3 * rve];
    nv1 = normal[3 * rve + 1];
    nv2 = normal[3 * rve + 2];
    const double n = nv0 * nv0 + nv1 * nv1 + nv2 * nv2;
    nv0 = nv0 / n;
    nv1 = nv1 / n;
    nv2 = nv2 / n;
  }
  double s[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) s[k] = 0.0;
  for (int e = threadIdx.x; e < d.n_fibers; e += kThreadsOrient) {
    const int2 c = b.conn[d.fiber_off + e];
    double lx = x0[c.y] - x0[c.x];
    double ly = x1[c.y] - x1[c.x];
    double lz = x2[c.y] - x2[c.x];
    double l = sqrt(lx * lx + ly * ly + lz * lz);
    lx = lx / l;
    ly = ly / l;
    lz = lz / l;
    if (normal) {
      const double dotn = lx * nv0 + ly * nv1 + lz * nv2;
      lx = lx - nv0 * dotn;
      ly = ly - nv1 * dotn;
      lz = lz - nv2 * dotn;
      l = sqrt(lx * lx + ly * ly + lz * lz);
      lx = lx / l;
      ly = ly / l;
      lz = lz / l;
    }
    const double dv[3] = {lx, ly, lz};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) s[3 * i + j] += dv[i] * dv[j];
  }
  for (int k = 0; k < 9; ++k) {
    const double t = block_sum<kThreadsOrient>(s[k], red);
    if (threadIdx.x == 0) omega[9 * rve + k] = t / d.n_fibers;
  }
}

__global__ void pack_status_kernel(const int32_t* status, const int32_t* steps,
                                   const double* residual, int n, mfg_rve_status* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    mfg_rve_status r;
    r.status = status[i];
    r.steps = steps[i];
    r.residual = residual[i];
    out[i] = r;
  }
}

}  // namespace

cudaError_t launch_orientation(const DevBatch& b, const double* normal, double* omega,
                               cudaStream_t s) {
  orientation_kernel<<<b.n_rve, kThreadsOrient, 0, s>>>(b, normal, omega);
  return cudaGetLastError();
}

cudaError_t launch_pack_status(const int32_t* status, const int32_t* steps,
                               const double* residual, int n, void* out, cudaStream_t s) {
  pack_status_kernel<<<(n + 255) / 256, 256, 0, s>>>(status, steps, residual, n,
                                                    static_cast<mfg_rve_status*>(out));
  return cudaGetLastError();
}

}  // namespace mfg
