// Macro/micro coupling front-end of the batched solve: the scale conversion
// the multiscale service applies to every network, and the per-iteration and
// per-step record exchange (src/mumfim/microscale/MultiscaleRVEAnalysis.cc:
// 197-305, MultiscaleCoupling.{h,cc}). Host code over the public C ABI.
#include <cmath>
#include <cstring>
#include <vector>

#include "mfg_internal.h"
#include "mumfim_gpu.h"

namespace mfg {
mfg_status set_error(mfg_status s, const char* msg);  // mfg_host.cpp
}
using mfg::set_error;

extern "C" {

mfg_status mfg_scale_conversion(int32_t n_nodes, const double* coords, int32_t n_fibers,
                                const int32_t* connectivity, double fiber_radius,
                                double volume_fraction, double* factor) {
  if (!coords || !connectivity || !factor || n_nodes < 1 || n_fibers < 1)
    return set_error(MFG_E_INVALID, "scale conversion: NULL argument or empty network");
  if (!(fiber_radius > 0) || !(volume_fraction > 0) || !std::isfinite(fiber_radius) ||
      !std::isfinite(volume_fraction))
    return set_error(MFG_E_INVALID,
                     "scale conversion: fiber radius and volume fraction must be positive");
  // total fiber length in the reference configuration, fibers in mesh order
  // (calcDimMeasures over the edges, summed front to back)
  double total = 0.0;
  for (int32_t e = 0; e < n_fibers; ++e) {
    const int32_t a = connectivity[2 * e], b = connectivity[2 * e + 1];
    if (a < 0 || b < 0 || a >= n_nodes || b >= n_nodes)
      return set_error(MFG_E_INVALID, "scale conversion: fiber end node out of range");
    const double dx = coords[3 * b] - coords[3 * a];
    const double dy = coords[3 * b + 1] - coords[3 * a + 1];
    const double dz = coords[3 * b + 2] - coords[3 * a + 2];
    total += std::sqrt(dx * dx + dy * dy + dz * dz);
  }
  const double pi = 4 * std::atan(1.0);
  const double area = pi * fiber_radius * fiber_radius;
  const double dim = std::sqrt(total * area / volume_fraction);
  *factor = 1 / (dim * dim);
  if (!std::isfinite(*factor))
    return set_error(MFG_E_NONFINITE, "scale conversion: non-finite factor (zero total length?)");
  set_error(MFG_OK, "");
  return MFG_OK;
}

mfg_status mfg_batch_micro_fo_iterate(mfg_batch* batch, const double* data, double* results,
                                      mfg_rve_status* status) {
  mfg::Trace trace("mfg_batch_micro_fo_iterate");
  if (!batch || !data || !results) return set_error(MFG_E_INVALID, "NULL argument");
  const int32_t R = mfg_batch_size(batch);
  if (R < 1) return set_error(MFG_E_INVALID, "empty batch");
  std::vector<double> sigma(6 * static_cast<size_t>(R)), C(36 * static_cast<size_t>(R));
  const mfg_status run = mfg_batch_run(batch, data, R, sigma.data(), 1, status);
  if (run == MFG_E_INVALID || run == MFG_E_CUDA || run == MFG_E_OOM || run == MFG_E_NO_DEVICE)
    return run;
  const mfg_status stiff = mfg_batch_material_stiffness(batch, C.data());
  if (stiff == MFG_E_INVALID || stiff == MFG_E_CUDA || stiff == MFG_E_OOM) return stiff;
  for (int32_t r = 0; r < R; ++r) {
    double* out = results + static_cast<size_t>(MFG_MICRO_FO_RESULT) * r;
    std::memcpy(out, &sigma[6 * static_cast<size_t>(r)], 6 * sizeof(double));
    out[6] = out[7] = out[8] = 0.0;  // averaged volume stress, unused by the reference
    std::memcpy(out + 9, &C[36 * static_cast<size_t>(r)], 36 * sizeof(double));
  }
  return run != MFG_OK ? run : stiff;
}

mfg_status mfg_batch_micro_fo_step(mfg_batch* batch, const double* params, double* step_results) {
  mfg::Trace trace("mfg_batch_micro_fo_step");
  if (!batch || !params || !step_results) return set_error(MFG_E_INVALID, "NULL argument");
  const int32_t R = mfg_batch_size(batch);
  if (R < 1) return set_error(MFG_E_INVALID, "empty batch");
  std::vector<double> o3(9 * static_cast<size_t>(R)), o2(9 * static_cast<size_t>(R)),
      normal(3 * static_cast<size_t>(R));
  for (int32_t r = 0; r < R; ++r)
    for (int k = 0; k < 3; ++k)
      normal[3 * r + k] = params[static_cast<size_t>(MFG_MICRO_FO_PARAMS) * r +
                                 MFG_PRM_ORIENTATION_AXIS_X + k];
  mfg_status st = mfg_batch_orientation_3d(batch, o3.data());
  if (st != MFG_OK) return st;
  if ((st = mfg_batch_orientation_2d(batch, normal.data(), o2.data())) != MFG_OK) return st;
  for (int32_t r = 0; r < R; ++r) {
    double* out = step_results + static_cast<size_t>(MFG_MICRO_FO_STEP_RESULT) * r;
    std::memcpy(out, &o3[9 * static_cast<size_t>(r)], 9 * sizeof(double));
    std::memcpy(out + 9, &o2[9 * static_cast<size_t>(r)], 9 * sizeof(double));
  }
  return MFG_OK;
}

}  // extern "C"
