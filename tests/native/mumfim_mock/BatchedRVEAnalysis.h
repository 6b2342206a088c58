// Stand-in for mumfim's abstract batched analysis (the interface the shim
// derives from): the same constructor argument and virtual method set, on the
// Kokkos stand-in. Test infrastructure only.
#ifndef MFG_TEST_BATCHED_RVE_ANALYSIS_H
#define MFG_TEST_BATCHED_RVE_ANALYSIS_H
#include "Kokkos_mock.h"
#include "MicroFOParams.h"

namespace mumfim {
template <typename Scalar, typename Ordinal, typename ExeSpace>
class BatchedRVEAnalysis {
 protected:
  Ordinal num_rves_;

 public:
  explicit BatchedRVEAnalysis(Ordinal num_rves) : num_rves_(num_rves) {}
  virtual ~BatchedRVEAnalysis() = default;
  virtual bool run(Kokkos::DualView<Scalar* [3][3], ExeSpace> dfmGrds,
                   Kokkos::DualView<Scalar* [6], ExeSpace> sigma, bool update_coords = true) = 0;
  virtual void computeMaterialStiffness(Kokkos::DualView<Scalar* [6][6], ExeSpace> C) = 0;
  virtual void compute3DOrientationTensor(Kokkos::DualView<Scalar* [3][3], ExeSpace>) {}
  virtual void compute2DOrientationTensor(Kokkos::DualView<Scalar* [3], ExeSpace>,
                                          Kokkos::DualView<Scalar* [3][3], ExeSpace>) {}
};
}  // namespace mumfim
#endif
