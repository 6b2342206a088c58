// Seeded k-nearest-neighbour fiber networks (see include/mumfim_netgen.h).
//
// Built with -ffp-contract=off so that no multiply-add is fused on any
// platform: the generated coordinates are bit-identical on x86-64 and
// aarch64.
#include "mumfim_netgen.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <utility>
#include <vector>

namespace {

inline double uniform01(std::mt19937_64& rng) {
  // 53 random mantissa bits -> [0,1), exact.
  return static_cast<double>(rng() >> 11) * 0x1.0p-53;
}

// Cody-Waite split of ln 2 (the fdlibm constants).
constexpr double kLn2Hi = 6.93147180369123816490e-01;
constexpr double kLn2Lo = 1.90821492927058770002e-10;
constexpr double kInvLn2 = 1.44269504088896338700e+00;

double exp_portable(double x) {
  if (x != x) return x;
  if (x > 709.0) return HUGE_VAL;
  if (x < -745.0) return 0.0;
  double kd = std::floor(x * kInvLn2 + 0.5);
  double r = (x - kd * kLn2Hi) - kd * kLn2Lo;  // |r| <= ~0.35
  // Taylor series of e^r to degree 16, Horner form.
  double p = 1.0;
  for (int n = 16; n >= 1; --n) p = 1.0 + p * r / static_cast<double>(n);
  return std::ldexp(p, static_cast<int>(kd));
}

double log_portable(double x) {
  if (x != x || x < 0.0) return NAN;
  if (x == 0.0) return -HUGE_VAL;
  if (std::isinf(x)) return x;
  int e = 0;
  double m = std::frexp(x, &e);  // x = m * 2^e, m in [0.5, 1)
  if (m < 0.70710678118654752440) {
    m *= 2.0;
    e -= 1;
  }
  // log(m) = 2 atanh(s), s = (m-1)/(m+1), |s| <= 0.1716
  double s = (m - 1.0) / (m + 1.0);
  double s2 = s * s;
  double sum = 0.0;
  for (int n = 29; n >= 1; n -= 2) sum = 1.0 / static_cast<double>(n) + s2 * sum;
  double lm = 2.0 * s * sum;
  double ed = static_cast<double>(e);
  return (ed * kLn2Hi + lm) + ed * kLn2Lo;
}

struct Grid {
  int g;
  double h;
  std::vector<int> start;  // g^3 + 1
  std::vector<int> items;
  int cell_of(double c) const {
    int i = static_cast<int>((c + 0.5) / h);
    return i < 0 ? 0 : (i >= g ? g - 1 : i);
  }
};

}  // namespace

extern "C" double mfg_portable_exp(double x) { return exp_portable(x); }
extern "C" double mfg_portable_log(double x) { return log_portable(x); }

extern "C" void mfg_generate_uniform(uint64_t seed, int32_t n, double* out) {
  std::mt19937_64 rng(seed);
  for (int32_t i = 0; i < n; ++i) out[i] = uniform01(rng);
}

extern "C" void mfg_generate_normal(uint64_t seed, int32_t n, double* out) {
  std::mt19937_64 rng(seed);
  int32_t i = 0;
  while (i < n) {
    double a = 2.0 * uniform01(rng) - 1.0;
    double b = 2.0 * uniform01(rng) - 1.0;
    double q = a * a + b * b;
    if (q >= 1.0 || q == 0.0) continue;
    double f = std::sqrt(-2.0 * log_portable(q) / q);
    out[i++] = a * f;
    if (i < n) out[i++] = b * f;
  }
}

extern "C" int32_t mfg_generate_knn_network(int32_t n_nodes, int32_t k, uint64_t seed,
                                            double snap, double min_sep, double* coords,
                                            int32_t* conn, int32_t max_fibers) {
  if (n_nodes < 2 || k < 1 || k >= n_nodes || !coords || !conn || max_fibers < 1) return -1;
  const int n = n_nodes;
  std::mt19937_64 rng(seed);

  // ---- node placement with face snapping and a minimum separation -------
  // A coarse placement grid (cells >= min_sep) finds near neighbours of a
  // candidate among the nodes placed so far.
  int gp = std::max(1, static_cast<int>(std::cbrt(static_cast<double>(n) / 2.0)));
  double hp = 1.0 / gp;
  std::vector<std::vector<int>> pcells(static_cast<size_t>(gp) * gp * gp);
  auto pcell = [&](double c) {
    int i = static_cast<int>((c + 0.5) / hp);
    return i < 0 ? 0 : (i >= gp ? gp - 1 : i);
  };
  const double sep2 = min_sep * min_sep;
  for (int i = 0; i < n; ++i) {
    int attempts = 0;
    for (;;) {
      if (++attempts > 1000000) return -1;
      double p[3];
      for (int d = 0; d < 3; ++d) {
        double c = uniform01(rng) - 0.5;
        if (std::fabs(c - 0.5) < snap) c = 0.5;
        if (std::fabs(c + 0.5) < snap) c = -0.5;
        p[d] = c;
      }
      int cx = pcell(p[0]), cy = pcell(p[1]), cz = pcell(p[2]);
      bool ok = true;
      for (int dx = -1; dx <= 1 && ok; ++dx)
        for (int dy = -1; dy <= 1 && ok; ++dy)
          for (int dz = -1; dz <= 1 && ok; ++dz) {
            int ax = cx + dx, ay = cy + dy, az = cz + dz;
            if (ax < 0 || ay < 0 || az < 0 || ax >= gp || ay >= gp || az >= gp) continue;
            for (int j : pcells[(static_cast<size_t>(ax) * gp + ay) * gp + az]) {
              double ex = coords[3 * j] - p[0], ey = coords[3 * j + 1] - p[1],
                     ez = coords[3 * j + 2] - p[2];
              if (ex * ex + ey * ey + ez * ez < sep2) {
                ok = false;
                break;
              }
            }
          }
      if (!ok) continue;
      coords[3 * i] = p[0];
      coords[3 * i + 1] = p[1];
      coords[3 * i + 2] = p[2];
      pcells[(static_cast<size_t>(cx) * gp + cy) * gp + cz].push_back(i);
      break;
    }
  }

  // ---- k nearest neighbours on a uniform bucket grid ---------------------
  Grid grid;
  grid.g = std::max(1, static_cast<int>(std::cbrt(static_cast<double>(n) / 2.0)));
  grid.h = 1.0 / grid.g;
  const int g = grid.g;
  const size_t ncell = static_cast<size_t>(g) * g * g;
  std::vector<int> cell_of_node(n);
  std::vector<int> count(ncell + 1, 0);
  for (int i = 0; i < n; ++i) {
    int c = (grid.cell_of(coords[3 * i]) * g + grid.cell_of(coords[3 * i + 1])) * g +
            grid.cell_of(coords[3 * i + 2]);
    cell_of_node[i] = c;
    count[c + 1]++;
  }
  grid.start.assign(ncell + 1, 0);
  for (size_t c = 0; c < ncell; ++c) grid.start[c + 1] = grid.start[c] + count[c + 1];
  grid.items.resize(n);
  {
    std::vector<int> fill(grid.start.begin(), grid.start.end() - 1);
    for (int i = 0; i < n; ++i) grid.items[fill[cell_of_node[i]]++] = i;
  }

  std::vector<std::pair<int32_t, int32_t>> edges;
  edges.reserve(static_cast<size_t>(n) * k);
  std::vector<std::pair<double, int>> best;  // (dist^2, id), sorted, size <= k
  for (int i = 0; i < n; ++i) {
    const double px = coords[3 * i], py = coords[3 * i + 1], pz = coords[3 * i + 2];
    const int cx = grid.cell_of(px), cy = grid.cell_of(py), cz = grid.cell_of(pz);
    best.clear();
    for (int r = 0; r <= g; ++r) {
      for (int ax = cx - r; ax <= cx + r; ++ax) {
        if (ax < 0 || ax >= g) continue;
        for (int ay = cy - r; ay <= cy + r; ++ay) {
          if (ay < 0 || ay >= g) continue;
          for (int az = cz - r; az <= cz + r; ++az) {
            if (az < 0 || az >= g) continue;
            int cheb = std::max(std::abs(ax - cx), std::max(std::abs(ay - cy), std::abs(az - cz)));
            if (cheb != r) continue;  // only the shell at distance r
            size_t c = (static_cast<size_t>(ax) * g + ay) * g + az;
            for (int t = grid.start[c]; t < grid.start[c + 1]; ++t) {
              int j = grid.items[t];
              if (j == i) continue;
              double ex = coords[3 * j] - px, ey = coords[3 * j + 1] - py,
                     ez = coords[3 * j + 2] - pz;
              std::pair<double, int> cand(ex * ex + ey * ey + ez * ez, j);
              if (static_cast<int>(best.size()) < k) {
                best.insert(std::upper_bound(best.begin(), best.end(), cand), cand);
              } else if (cand < best.back()) {
                best.pop_back();
                best.insert(std::upper_bound(best.begin(), best.end(), cand), cand);
              }
            }
          }
        }
      }
      // Every node in a shell beyond r is at least r*h away.
      if (static_cast<int>(best.size()) == k) {
        double reach = static_cast<double>(r) * grid.h;
        if (best.back().first <= reach * reach) break;
      }
    }
    for (auto& b : best) {
      int j = b.second;
      edges.emplace_back(std::min(i, j), std::max(i, j));
    }
  }
  std::sort(edges.begin(), edges.end());
  edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
  if (static_cast<int64_t>(edges.size()) > max_fibers) return -1;
  for (size_t e = 0; e < edges.size(); ++e) {
    conn[2 * e] = edges[e].first;
    conn[2 * e + 1] = edges[e].second;
  }
  return static_cast<int32_t>(edges.size());
}
