// Host-side order of the mixed-precision RVEs with an order of their own
// (mfg_relax_mixed.cu): the fiber and node order of cluster-solved and
// all-on-chip RVEs, and the node-centric solve's incidence blocks. Built
// once per batch at set-up; the kernels read the arrays these fill.
#ifndef MFG_MIXED_ORDER_H
#define MFG_MIXED_ORDER_H

#include <cstdint>
#include <vector>

#include "mfg_internal.h"

namespace mfg {

// Fiber and node order of an RVE with its own order: one solved by a
// cluster of cl CTAs, or by one CTA with all its state in shared memory.
//
// Fibers: each goes to the CTA that owns its lower-numbered end (a free node
// whenever the fiber has one); within a CTA, fibers with both ends owned by
// that CTA come first, then the fibers that cross to another CTA, each group
// in slot order. CTA o takes fiber positions [o*echunk, (o+1)*echunk) in the
// length pass, so most warps see only local end nodes: a load of about 37
// cycles through the cluster window against about 200 for a peer CTA's
// shared memory.
//
// Nodes: within each CTA's block of free nodes, those whose neighbours are
// all owned by that CTA come first, and within each group the nodes by
// degree, so the lanes of a warp run loops of nearly the same length (+6 %
// for the fiber-centric single CTA) and the warps that wait on other CTAs
// are few. heavy_first (node-centric solve) orders by falling degree, so the
// threads' last, partial round over the nodes gets the lightest ones (+13 %
// on config 2 against rising degree); the fiber-centric solve keeps rising
// degree. Boundary nodes keep their places.
//
// Writes the fiber positions (mslot), the end-node codes by position
// (econn), the node index by node position (gnode, batch-wide), and the CSR
// rows by node position (mrowptr) with their incidences as (fiber position
// << 1 | end) (icode), which the single-CTA fiber-centric solve reads. RVEs
// without their own order (own_order false) keep the batch's order.
void cluster_order(const RveDesc& d, int cl, bool own_order, bool heavy_first,
                   const std::vector<int2>& conn,
                   const std::vector<int32_t>& rowptr, const std::vector<int32_t>& inc,
                   std::vector<int2>& econn, std::vector<int32_t>& icode,
                   std::vector<int32_t>& mslot, std::vector<int32_t>& gnode,
                   std::vector<int32_t>& mrowptr);

// SELL-32 incidence block of a node-centric RVE (see solve_rve_nodal), from
// its node order (gnode): for each CTA of the cluster its own nodes in the
// order its threads visit them (free, then boundary) form slices of 32, each
// as wide as its largest degree. Returns the block's element count; when
// ncode is given, also fills the block (at base) and the nodes' rows.
int64_t sell_layout(const RveDesc& d, int cl, const std::vector<int2>& conn,
                    const std::vector<int32_t>& rowptr, const std::vector<int32_t>& inc,
                    const std::vector<int32_t>& gnode, int64_t base, int2* nsell, int32_t* ncode,
                    int64_t* nfib);

}  // namespace mfg

#endif
