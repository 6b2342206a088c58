// Checks the host-side order of the mixed-precision RVEs (mfg_mixed_order.h)
// on random networks, for every cluster size and both degree orders:
//  - gnode is a permutation that keeps boundary nodes in place and free
//    nodes among the free ones;
//  - every fiber's end codes (econn) decode to its end nodes, in order;
//  - every node-centric incidence (SELL-32 block) lies inside the block, sits
//    at its node's lane, decodes to the other end of the node's k-th CSR
//    incidence with the right end bit and fiber, and names a record inside
//    the owner CTA's node slots.
// Prints "bad=0" and exits 0 when every check holds.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "mfg_mixed_order.h"

using namespace mfg;

int main() {
  std::mt19937 rng(3);
  int bad = 0;
  auto fail = [&](const char* what) {
    if (++bad <= 10) std::printf("fail: %s\n", what);
  };
  for (int trial = 0; trial < 40; ++trial) {
    const int N = 50 + static_cast<int>(rng() % 9000);
    const int NB = static_cast<int>(rng() % (N / 5 + 1)), NF = N - NB;
    std::vector<int2> conn;
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < 2; ++k) {
        const int o = (j + 1 + static_cast<int>(rng() % 40)) % N;
        conn.push_back(make_int2(j, o));
      }
    const int E = static_cast<int>(conn.size());
    // CSR rows in ascending fiber order: (fiber << 1) | end, end 1 = second end
    std::vector<int32_t> rowptr(N + 1, 0), inc(2 * E);
    for (int e = 0; e < E; ++e) {
      rowptr[conn[e].x + 1]++;
      rowptr[conn[e].y + 1]++;
    }
    for (int j = 0; j < N; ++j) rowptr[j + 1] += rowptr[j];
    std::vector<int> fill(rowptr.begin(), rowptr.end() - 1);
    for (int e = 0; e < E; ++e) {
      inc[fill[conn[e].x]++] = (e << 1) | 0;
      inc[fill[conn[e].y]++] = (e << 1) | 1;
    }
    RveDesc d{};
    d.n_nodes = N;
    d.n_free = NF;
    d.n_fibers = E;
    for (int cl : {1, 2, 4, 8}) {
      const bool heavy = (trial & 1) != 0;
      std::vector<int2> econn(E);
      std::vector<int32_t> icode(2 * E), mslot(E), gnode(N), mrowptr(N + 1);
      cluster_order(d, cl, true, heavy, conn, rowptr, inc, econn, icode, mslot, gnode, mrowptr);
      const int64_t n = sell_layout(d, cl, conn, rowptr, inc, gnode, 0, nullptr, nullptr, nullptr);
      std::vector<int2> nsell(N, make_int2(-1, -1));
      std::vector<int32_t> ncode(n, 0);
      std::vector<int64_t> nfib(n, -1);
      if (sell_layout(d, cl, conn, rowptr, inc, gnode, 0, nsell.data(), ncode.data(),
                      nfib.data()) != n)
        fail("block size differs between the two calls");
      const int fchunk = (NF + cl - 1) / cl, bchunk = (NB + cl - 1) / cl, cap = fchunk + bchunk;
      std::vector<int> seen(N, 0);
      for (int P = 0; P < N; ++P) seen[gnode[P]]++;
      for (int j = 0; j < N; ++j)
        if (seen[j] != 1) {
          fail("gnode is not a permutation");
          break;
        }
      auto decode = [&](int code) {
        const int o = code >> 24, local = code & 0xFFFFFF;
        return local < fchunk ? o * fchunk + local : NF + o * bchunk + (local - fchunk);
      };
      for (int o = 0; o < cl; ++o) {
        const int f_lo = std::min(NF, o * fchunk), f_hi = std::min(NF, f_lo + fchunk);
        const int g_lo = NF + std::min(NB, o * bchunk);
        const int g_hi = NF + std::min(NB, o * bchunk + bchunk);
        const int nfo = f_hi - f_lo, n_own = nfo + (g_hi - g_lo);
        for (int t = 0; t < n_own; ++t) {
          const int P = t < nfo ? f_lo + t : g_lo + (t - nfo);
          const int j = gnode[P];
          if (P >= NF && j != P) fail("boundary node moved");
          if (P < NF && j >= NF) fail("boundary node among the free ones");
          const int2 sr = nsell[P];
          const int deg = rowptr[j + 1] - rowptr[j];
          if (sr.y != deg || sr.x % 32 != t % 32) fail("row start or degree");
          for (int k = 0; k < deg; ++k) {
            const int64_t p = sr.x + 32LL * k;
            if (p < 0 || p >= n) {
              fail("incidence outside the block");
              continue;
            }
            const int code = ncode[p] >> 1, end = ncode[p] & 1;
            if ((code >> 24) >= cl || (code & 0xFFFFFF) >= cap) {
              fail("record outside the owner's slots");
              continue;
            }
            const int ic = inc[rowptr[j] + k];
            const int2 c = conn[ic >> 1];
            const int other = (ic & 1) ? c.x : c.y;
            if (gnode[decode(code)] != other || end != (ic & 1) || nfib[p] != (ic >> 1))
              fail("incidence decodes to the wrong neighbour");
          }
        }
      }
      for (int e = 0; e < E; ++e) {
        const int2 c = econn[mslot[e]];
        if (gnode[decode(c.x)] != conn[e].x || gnode[decode(c.y)] != conn[e].y) {
          fail("fiber end codes");
          break;
        }
      }
    }
  }
  std::printf("bad=%d\n", bad);
  return bad != 0;
}
