// Mixed-precision relaxation (placeholder until the kernel lands).
#include "mfg_mixed.h"

namespace mfg {

struct MixedState {
  int dummy = 0;
};

MixedState* mixed_new() { return new MixedState(); }
void mixed_destroy(MixedState* ms) { delete ms; }

cudaError_t mixed_create(MixedState&, const DevBatch&, const std::vector<RveDesc>&, int,
                         cudaStream_t) {
  return cudaErrorNotSupported;
}

cudaError_t run_mixed(MixedState&, const DevBatch&, const RunArgs&, cudaStream_t, int* launches) {
  *launches = 0;
  return cudaErrorNotSupported;
}

}  // namespace mfg
