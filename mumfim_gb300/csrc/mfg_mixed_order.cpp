// Host-side order of the mixed-precision RVEs (declared, with what each
// function writes, in mfg_mixed_order.h).
#include "mfg_mixed_order.h"

#include <algorithm>
#include <utility>

namespace mfg {

void cluster_order(const RveDesc& d, int cl, bool own_order, bool heavy_first,
                   const std::vector<int2>& conn,
                   const std::vector<int32_t>& rowptr, const std::vector<int32_t>& inc,
                   std::vector<int2>& econn, std::vector<int32_t>& icode,
                   std::vector<int32_t>& mslot, std::vector<int32_t>& gnode,
                   std::vector<int32_t>& mrowptr) {
  const int N = d.n_nodes, E = d.n_fibers, NF = d.n_free, NB = d.n_nodes - d.n_free;
  const int64_t fo = d.fiber_off, io = d.inc_off, no = d.node_off, ro = d.row_off;
  if (!own_order) {
    for (int e = 0; e < E; ++e) {
      mslot[fo + e] = e;
      econn[fo + e] = conn[fo + e];
    }
    for (int64_t p = 0; p < 2LL * E; ++p) icode[io + p] = inc[io + p];
    for (int j = 0; j < N; ++j) gnode[no + j] = static_cast<int32_t>(no + j);
    for (int j = 0; j <= N; ++j) mrowptr[ro + j] = rowptr[ro + j];
    return;
  }
  const int fchunk = (NF + cl - 1) / cl, bchunk = (NB + cl - 1) / cl;
  auto owner = [&](int j) { return j < NF ? j / fchunk : (j - NF) / bchunk; };
  // fibers: stable counting sort by (owner of the lower end, crossing)
  std::vector<int> key(E), start(2 * cl + 1, 0);
  for (int e = 0; e < E; ++e) {
    const int2 c = conn[fo + e];
    const int o = owner(std::min(c.x, c.y));
    key[e] = 2 * o + ((owner(c.x) == o && owner(c.y) == o) ? 0 : 1);
    ++start[key[e] + 1];
  }
  for (int k = 0; k < 2 * cl; ++k) start[k + 1] += start[k];
  for (int e = 0; e < E; ++e) mslot[fo + e] = start[key[e]]++;
  // nodes: position of each node (identity but for the free blocks)
  std::vector<int> pos(N);
  for (int j = 0; j < N; ++j) pos[j] = j;
  for (int o = 0; o < cl; ++o) {
    const int f_lo = std::min(NF, o * fchunk), f_hi = std::min(NF, f_lo + fchunk);
    std::vector<std::pair<int, int>> order;  // (group * 1024 + degree rank, node)
    order.reserve(f_hi - f_lo);
    for (int j = f_lo; j < f_hi; ++j) {
      bool local = true;
      for (int p = rowptr[ro + j]; p < rowptr[ro + j + 1] && local; ++p) {
        const int ic = inc[io + p];
        const int2 c = conn[fo + (ic >> 1)];
        local = owner((ic & 1) ? c.x : c.y) == o;
      }
      const int deg = std::min(rowptr[ro + j + 1] - rowptr[ro + j], 1023);
      order.emplace_back((local ? 0 : 1024) + (heavy_first ? 1023 - deg : deg), j);
    }
    std::stable_sort(order.begin(), order.end(),
                     [](const std::pair<int, int>& x, const std::pair<int, int>& y) {
                       return x.first < y.first;
                     });
    int q = f_lo;
    for (const auto& kv : order) pos[kv.second] = q++;
  }
  auto code = [&](int j) {
    const int o = owner(j);
    const int local = j < NF ? pos[j] - o * fchunk : fchunk + (j - NF) - o * bchunk;
    return (o << 24) | local;
  };
  for (int e = 0; e < E; ++e) {
    const int2 c = conn[fo + e];
    econn[fo + mslot[fo + e]] = make_int2(code(c.x), code(c.y));
  }
  std::vector<int> at(N);
  for (int j = 0; j < N; ++j) at[pos[j]] = j;
  int64_t q = 0;
  mrowptr[ro] = 0;
  for (int P = 0; P < N; ++P) {
    const int j = at[P];
    gnode[no + P] = static_cast<int32_t>(no + j);
    for (int p = rowptr[ro + j]; p < rowptr[ro + j + 1]; ++p, ++q) {
      const int ic = inc[io + p];
      icode[io + q] = (mslot[fo + (ic >> 1)] << 1) | (ic & 1);
    }
    mrowptr[ro + P + 1] = static_cast<int32_t>(q);
  }
}

int64_t sell_layout(const RveDesc& d, int cl, const std::vector<int2>& conn,
                    const std::vector<int32_t>& rowptr, const std::vector<int32_t>& inc,
                    const std::vector<int32_t>& gnode, int64_t base, int2* nsell, int32_t* ncode,
                    int64_t* nfib) {
  const int N = d.n_nodes, NF = d.n_free, NB = N - NF;
  const int64_t no = d.node_off, ro = d.row_off, io = d.inc_off, fo = d.fiber_off;
  const int fchunk = (NF + cl - 1) / cl, bchunk = (NB + cl - 1) / cl;
  std::vector<int> pos;
  if (ncode) {
    pos.resize(N);
    for (int P = 0; P < N; ++P) pos[gnode[no + P] - no] = P;
  }
  // code of the node at position P: (owner CTA << 24) | local record
  auto code_of = [&](int P) {
    if (P < NF) {
      const int o = P / fchunk;
      return (o << 24) | (P - o * fchunk);
    }
    const int o = (P - NF) / bchunk;
    return (o << 24) | (fchunk + (P - NF) - o * bchunk);
  };
  int64_t q = 0;
  for (int o = 0; o < cl; ++o) {
    const int f_lo = std::min(NF, o * fchunk), f_hi = std::min(NF, f_lo + fchunk);
    const int g_lo = NF + std::min(NB, o * bchunk), g_hi = NF + std::min(NB, o * bchunk + bchunk);
    const int nfo = f_hi - f_lo, n_own = nfo + (g_hi - g_lo);
    for (int s0 = 0; s0 < n_own; s0 += 32) {
      int w = 0;
      for (int t = s0; t < std::min(n_own, s0 + 32); ++t) {
        const int P = t < nfo ? f_lo + t : g_lo + (t - nfo);
        const int j = gnode[no + P] - static_cast<int32_t>(no);
        const int deg = rowptr[ro + j + 1] - rowptr[ro + j];
        w = std::max(w, deg);
        if (!ncode) continue;
        const int64_t at = q + (t - s0);
        nsell[no + P] = make_int2(static_cast<int>(at), deg);
        for (int k = 0; k < deg; ++k) {
          const int ic = inc[io + rowptr[ro + j] + k];
          const int2 c = conn[fo + (ic >> 1)];
          const int other = (ic & 1) ? c.x : c.y;
          ncode[base + at + 32LL * k] = (code_of(pos[other]) << 1) | (ic & 1);
          nfib[base + at + 32LL * k] = fo + (ic >> 1);
        }
      }
      q += 32LL * w;
    }
  }
  return q;
}

}  // namespace mfg
