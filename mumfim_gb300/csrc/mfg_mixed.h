// Mixed-precision relaxation (FP32 forces and integrator on FP64 reference
// coordinates plus Kahan-compensated FP32 displacements).
#ifndef MFG_MIXED_H
#define MFG_MIXED_H

#include <vector>

#include <cuda_runtime.h>

#include "mfg_internal.h"

namespace mfg {

struct MixedState;
MixedState* mixed_new();

// Run contexts of a mixed batch: 0 for its runs, 1..kMixedContexts-1 for
// runs in flight at the same time on the same batch (the concurrent
// perturbed solves of the material stiffness).
constexpr int kMixedContexts = 7;

// Allocates the mixed-precision working set of a batch and places its RVEs
// in size buckets. conn, rowptr and inc are the batch's packed fiber ends
// and CSR rows on the host (RVEs with an order of their own, and the
// node-centric incidence blocks, are built from them). max_cluster bounds
// the cluster size; serving_layout takes clusters of 4 where the batch
// layout would take 2. small_solve (mfg_small_rve_solve) picks the solve of
// the RVEs whose node state fits one CTA; with the fiber-centric one, up to
// rves_per_cta (1 or 2) small RVEs share a CTA.
cudaError_t mixed_create(MixedState& ms, const DevBatch& b, const std::vector<RveDesc>& desc,
                         const std::vector<int2>& conn, const std::vector<int32_t>& rowptr,
                         const std::vector<int32_t>& inc, int sms, int max_cluster,
                         bool serving_layout, int small_solve, int rves_per_cta,
                         cudaStream_t s);
// One run: reads the persistent FP64 state (x, u, vol), relaxes in mixed
// precision and writes the FP64 state, stress and status back. `ctx` picks
// the run context (0 for the batch's runs); runs on different contexts may
// be in flight together when their batch views write disjoint state.
cudaError_t run_mixed(MixedState& ms, const DevBatch& b, const RunArgs& a, cudaStream_t s,
                      int* launches, int ctx = 0);
// Creates run contexts 1..n (n < kMixedContexts) if they do not exist yet.
cudaError_t mixed_prepare_contexts(MixedState& ms, const DevBatch& b, int n);
void mixed_destroy(MixedState* ms);
// Persistent serving kernel on the mixed-precision solve. Without `big`, one
// CTA per SM serves the `small` ring; with it, 4-CTA clusters serve the
// `big` ring (RVEs for which mixed_serves_in_clusters) as clusters and the
// `small` ring CTA by CTA.
cudaError_t launch_server_mixed(MixedState& ms, const DevBatch& b, const ServerArgs& small,
                                const ServerArgs* big, cudaStream_t s);
// Cluster size of an RVE's batch bucket, and whether the serving kernel
// solves it as a cluster.
int mixed_rve_cluster(const MixedState& ms, int rve);
bool mixed_serves_in_clusters(const MixedState& ms, int rve);

struct MixedStateDeleter {
  void operator()(MixedState* p) const { mixed_destroy(p); }
};

}  // namespace mfg

#endif
