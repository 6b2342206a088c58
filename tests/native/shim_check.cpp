// Drives the integration shim (the C++ class a mumfim maintainer adds, read
// out of INTEGRATION.md into BatchedFiberRVEAnalysisGB300.h by the test) on
// stand-in mumfim types, through libmumfim_gpu.
//
//   shim_check create <policy> <input>   construct the shim; prints "created"
//                                        or the mumfim_error it threw
//   shim_check solve <policy> <input>    construct, run (updating), stiffness,
//                                        3-D orientation; prints sigma, C and
//                                        omega as one JSON object
// policy: reference | network. The input is whitespace-separated text:
// n_rve, then per RVE "law E radius density B lt cmp scale damping n_nodes
// n_fibers",
// the coordinates, the connectivity and the 9 entries of F.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "BatchedFiberRVEAnalysisGB300.h"

using namespace mumfim;
using Exe = Kokkos::DefaultExecutionSpace;

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: shim_check create|solve reference|network input\n");
    return 2;
  }
  const std::string mode = argv[1];
  const LawPolicy policy = std::string(argv[2]) == "network" ? LawPolicy::NetworkLaw
                                                             : LawPolicy::Reference;
  std::ifstream in(argv[3]);
  int n_rve = 0;
  in >> n_rve;
  std::vector<std::shared_ptr<const FiberNetwork>> nets;
  std::vector<std::shared_ptr<const MicroSolutionStrategy>> strategies;
  Kokkos::DualView<double* [3][3], Exe> F("F", n_rve);
  for (int r = 0; r < n_rve; ++r) {
    int law = 0, nn = 0, ne = 0;
    double E, radius, rho, B, lt, cmp, scale, damping;
    in >> law >> E >> radius >> rho >> B >> lt >> cmp >> scale >> damping >> nn >> ne;
    auto mesh = std::make_shared<apf::Mesh>();
    mesh->points.resize(nn);
    for (auto& p : mesh->points) in >> p[0] >> p[1] >> p[2];
    mesh->edges.resize(ne);
    for (auto& e : mesh->edges) in >> e[0] >> e[1];
    mesh->finalize();
    std::shared_ptr<FiberReaction> rc;
    if (law == 1) {
      auto nl = std::make_shared<NonlinearReaction>();
      nl->B = B;
      nl->length_ratio_trns = lt;
      nl->cmp_ratio_trns = cmp;
      rc = nl;
    } else {
      rc = std::make_shared<LinearReaction>();
    }
    rc->E = E;
    rc->fiber_area = radius * radius * M_PI;
    rc->fiber_density = rho;
    nets.push_back(std::make_shared<FiberNetwork>(mesh, std::vector<std::shared_ptr<FiberReaction>>{rc},
                                                  scale));
    auto ex = std::make_shared<MicroSolutionStrategyExplicit>();
    ex->visc_damp_coeff = damping;
    strategies.push_back(ex);
    for (int k = 0; k < 9; ++k) in >> F.h_view.data()[9 * r + k];
  }
  if (!in) {
    std::fprintf(stderr, "bad input\n");
    return 2;
  }
  try {
    BatchedFiberRVEAnalysisGB300<Exe> shim(nets, strategies, policy);
    if (mode == "create") {
      std::printf("created\n");
      return 0;
    }
    Kokkos::DualView<double* [6], Exe> sigma("sigma", n_rve);
    Kokkos::DualView<double* [6][6], Exe> C("C", n_rve);
    Kokkos::DualView<double* [3][3], Exe> omega("omega", n_rve);
    const bool converged = shim.run(F, sigma, true);
    shim.computeMaterialStiffness(C);
    shim.compute3DOrientationTensor(omega);
    auto dump = [](const char* name, const double* p, size_t n, bool last) {
      std::printf("\"%s\": [", name);
      for (size_t i = 0; i < n; ++i) std::printf("%s%.17g", i ? ", " : "", p[i]);
      std::printf("]%s", last ? "" : ", ");
    };
    std::printf("{\"converged\": %s, ", converged ? "true" : "false");
    dump("sigma", sigma.h_view.data(), 6 * static_cast<size_t>(n_rve), false);
    dump("C", C.h_view.data(), 36 * static_cast<size_t>(n_rve), false);
    dump("omega", omega.h_view.data(), 9 * static_cast<size_t>(n_rve), true);
    std::printf("}\n");
  } catch (const mumfim_error& e) {
    std::printf("mumfim_error: %s\n", e.what());
  }
  return 0;
}
