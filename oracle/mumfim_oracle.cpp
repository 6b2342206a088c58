// mumfim_oracle.cpp -- CPU restatement of the reference's batched explicit
// fiber-network RVE solve. TEST INFRASTRUCTURE ONLY (see mumfim_oracle.h).
//
// Reference files (paths inside the mumfim source tree):
//   B   = src/mumfim/microscale/batched_analysis/BatchedFiberRVEAnalysisExplicitBase.h
//   T   = src/mumfim/microscale/batched_analysis/BatchedFiberRVEAnalysisExplicitTeamOuterLoop.h
//   A   = src/mumfim/microscale/BatchedFiberRVEAnalysisExplicit.h
//   R   = src/mumfim/microscale/batched_analysis/BatchedReorderMesh.h
//   O   = src/mumfim/microscale/batched_analysis/BatchedComputeOrientationTensor.h
//   FR  = src/mumfim/microscale/FiberReactions.cc
//
// Order of floating-point operations is the reference's, with the serial
// (TEAM_SIZE = 1) order for every team loop and atomic scatter.
#include "mumfim_oracle.h"

#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <vector>

namespace {

constexpr int kUpdateFreq = 100;  // T:4

struct Rve {
  int N = 0, E = 0, nb = 0, nfree = 0;
  std::vector<int> perm;  // original id -> solver id
  std::vector<int> conn;  // [2e + j], solver ids
  // node arrays, row-major [3i + k], solver order
  std::vector<double> X, x, u, v, ftot, fint, m;
  std::vector<double> l0, l;
  std::vector<double> ramp0, rampd;  // RAMP mode: boundary start and increment
  // reaction 0 and strategy
  int law = 0;
  double Emod = 0, area = 0, rho = 0, B = 0, lt = 0;
  double c = 0, crit = 0.8, tol = 1e-6;
  int max_steps = 0, mode = MFG_MODE_RELAX;
  double scale = 1.0, V = 1.0, sound_speed = 1.0;
  double current_stress[6] = {0, 0, 0, 0, 0, 0};
};

// ---- fiber laws ---------------------------------------------------------
// B:155-172 (identical to LinearReaction::forceReaction().first, FR:5-15)
inline double linear_force(double orig_length, double length, double E, double A) {
  double length_ratio = length / orig_length;
  double green_strain = 1.0 / 2.0 * (length_ratio * length_ratio - 1);
  return length_ratio * E * A * green_strain;
}
// NonlinearReaction::forceReaction().first, FR:16-71, with cmp_ratio_trns = 1
// (FiberNetworkIO_impl.h:35).
inline double nl_force(double alpha, double B, double lr, double gs) {
  return alpha * lr * (std::exp(B * gs) - 1);  // FR:65-71 computeNLForce
}
inline double nl_deriv(double alpha, double B, double lr, double l0, double gs) {
  return alpha / l0 * ((1 + lr * lr * B) * std::exp(B * gs) - 1);  // FR:72-80
}
inline double nonlinear_force(double orig_length, double length, double E, double A,
                              double B, double lt) {
  const double cmp = 1.0;
  double length_ratio = length / orig_length;
  double alpha = E * A / B;
  if (length_ratio > lt) {
    double gt = 1.0 / 2.0 * (lt * lt - 1);
    double m = nl_deriv(alpha, B, lt, orig_length, gt);
    double b = nl_force(alpha, B, lt, gt);
    return m * (length_ratio - lt) * orig_length + b;
  } else if (length_ratio < cmp) {
    double gc = 1.0 / 2.0 * (cmp * cmp - 1);
    double m = nl_deriv(alpha, B, cmp, orig_length, gc);
    double b = nl_force(alpha, B, cmp, gc);
    return m * (length_ratio - cmp) * orig_length + b;
  }
  double gs = 1.0 / 2.0 * (length_ratio * length_ratio - 1);
  return nl_force(alpha, B, length_ratio, gs);
}
inline double fiber_force(const Rve& r, double l0, double l) {
  return r.law == MFG_LAW_NONLINEAR ? nonlinear_force(l0, l, r.Emod, r.area, r.B, r.lt)
                                    : linear_force(l0, l, r.Emod, r.area);
}

// ---- step pieces ----------------------------------------------------------
// B:203-215 getElementLength
inline double element_length(const std::vector<double>& c, int n1, int n2) {
  double x1 = c[3 * n2] - c[3 * n1];
  double x2 = c[3 * n2 + 1] - c[3 * n1 + 1];
  double x3 = c[3 * n2 + 2] - c[3 * n1 + 2];
  return std::sqrt(x1 * x1 + x2 * x2 + x3 * x3);
}

// T:53-82 getElementLengths; returns the min when requested.
double element_lengths(const Rve& r, const std::vector<double>& c, std::vector<double>& out) {
  double lmin = std::numeric_limits<double>::max();
  for (int e = 0; e < r.E; ++e) {
    out[e] = element_length(c, r.conn[2 * e], r.conn[2 * e + 1]);
    if (out[e] < lmin) lmin = out[e];
  }
  return lmin;
}

// T:83-143 getForces over nodes [0, nvert): zero f_int (B:216-224), serial
// scatter over every fiber (B:225-252), then f = -f_int - c m v (B:253-274).
// Returns sqrt(sum of squared residuals) (T:119-133).
double get_forces(Rve& r, int nvert) {
  for (int i = 0; i < nvert; ++i)
    for (int j = 0; j < 3; ++j) r.fint[3 * i + j] = 0;
  for (int e = 0; e < r.E; ++e) {
    double local_l = r.l[e];
    double frc = fiber_force(r, r.l0[e], local_l);
    double frc_ovr_l = frc / local_l;
    int n1 = r.conn[2 * e], n2 = r.conn[2 * e + 1];
    double nrm1 = (r.x[3 * n2] - r.x[3 * n1]) * frc_ovr_l;
    double nrm2 = (r.x[3 * n2 + 1] - r.x[3 * n1 + 1]) * frc_ovr_l;
    double nrm3 = (r.x[3 * n2 + 2] - r.x[3 * n1 + 2]) * frc_ovr_l;
    r.fint[3 * n1] -= nrm1;
    r.fint[3 * n2] += nrm1;
    r.fint[3 * n1 + 1] -= nrm2;
    r.fint[3 * n2 + 1] += nrm2;
    r.fint[3 * n1 + 2] -= nrm3;
    r.fint[3 * n2 + 2] += nrm3;
  }
  double residual = 0;
  for (int i = 0; i < nvert; ++i) {
    double mass = r.m[i] * r.c;
    double res_i = 0;
    for (int j = 0; j < 3; ++j) {
      double f_damp = mass * r.v[3 * i + j];
      double local_residual = -r.fint[3 * i + j];
      r.ftot[3 * i + j] = local_residual - f_damp;
      res_i += local_residual * local_residual;
    }
    residual += res_i;
  }
  return std::sqrt(residual);
}

// B:16-57 applyIncrementalDeformationToDisplacement, one node.
inline void affine_increment(const double* F, const double* xc, double* out_du_plus_u) {
  for (int k = 0; k < 3; ++k) {
    out_du_plus_u[k] = (F[3 * k + 0] - (k == 0 ? 1 : 0)) * xc[0] +
                       (F[3 * k + 1] - (k == 1 ? 1 : 0)) * xc[1] +
                       (F[3 * k + 2] - (k == 2 ? 1 : 0)) * xc[2] + out_du_plus_u[k];
  }
}

// RAMP protocol: total boundary increment d = (F - I) x0 of one node, with the
// predictor's operation order minus its "+ u" term.
inline void ramp_increment(const double* F, const double* xc, double* d) {
  for (int k = 0; k < 3; ++k) {
    d[k] = (F[3 * k + 0] - (k == 0 ? 1 : 0)) * xc[0] + (F[3 * k + 1] - (k == 1 ? 1 : 0)) * xc[1] +
           (F[3 * k + 2] - (k == 2 ? 1 : 0)) * xc[2];
  }
}

// T:180-437 TeamOuterLoop::run for one RVE, plus the RAMP protocol.
void relax(Rve& r, const double* F, mfg_rve_status* st) {
  const int N = r.N, nfree = r.nfree;
  // RunInitialization (T:215-289)
  double dt_crit = element_lengths(r, r.X, r.l0) / r.sound_speed;  // T:267-269
  for (int i = 0; i < N; ++i)                                      // T:272-274
    for (int j = 0; j < 3; ++j) r.x[3 * i + j] = r.X[3 * i + j] + r.u[3 * i + j];
  dt_crit = element_lengths(r, r.x, r.l) / r.sound_speed;  // T:276-278
  (void)dt_crit;
  double dt_crit_run = dt_crit;
  get_forces(r, nfree);  // T:281-286 (free nodes)
  if (r.mode == MFG_MODE_RAMP) {
    for (int b = 0; b < r.nb; ++b) {
      int i = nfree + b;
      double d[3];
      ramp_increment(F, &r.x[3 * i], d);
      for (int j = 0; j < 3; ++j) {
        r.ramp0[3 * b + j] = r.x[3 * i + j];
        r.rampd[3 * b + j] = d[j];
      }
    }
  }
  // main loop (T:291-372)
  int step = 0;
  double residual = 10.0;
  bool nonfinite = false;
  const double crit = r.crit;
  for (;;) {
    double dt_nphalf = crit * dt_crit_run * 0.5;  // T:345
    // updates (T:157-175)
    for (int i = 0; i < nfree; ++i) {
      double mass = r.m[i];
      for (int j = 0; j < 3; ++j) {
        double v_local = r.v[3 * i + j] + dt_nphalf * r.ftot[3 * i + j] / mass;
        r.v[3 * i + j] = v_local;
        r.x[3 * i + j] = r.x[3 * i + j] + 2 * dt_nphalf * v_local;
      }
    }
    if (r.mode == MFG_MODE_RAMP) {
      double alpha = static_cast<double>(step + 1) / static_cast<double>(r.max_steps);
      for (int b = 0; b < r.nb; ++b)
        for (int j = 0; j < 3; ++j)
          r.x[3 * (nfree + b) + j] = r.ramp0[3 * b + j] + alpha * r.rampd[3 * b + j];
    }
    // getElementLengths (T:352-354; dt_crit refresh every UPDATE_FREQ, T:61-75)
    double lmin = element_lengths(r, r.x, r.l);
    if (step % kUpdateFreq == 0) dt_crit_run = lmin / r.sound_speed;
    // getForces (T:356-361)
    double res = get_forces(r, nfree);
    if (step % kUpdateFreq == 0) residual = res;
    // updateAccelVels (T:363-365; B:275-287)
    for (int i = 0; i < nfree; ++i) {
      double mass = r.m[i];
      for (int j = 0; j < 3; ++j) r.v[3 * i + j] += dt_nphalf * r.ftot[3 * i + j] / mass;
    }
    ++step;
    if (!std::isfinite(residual)) {
      nonfinite = true;
      break;
    }
    if (r.mode == MFG_MODE_RAMP) {
      if (step >= r.max_steps) break;
    } else {
      if (!(residual > r.tol)) break;  // T:371
      if (step >= (r.max_steps > 0 ? r.max_steps : MFG_DEFAULT_STEP_CAP)) break;
    }
  }
  // FinalizeData (T:374-434): forces on every node, then u = x - X.
  get_forces(r, N);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < 3; ++j) r.u[3 * i + j] = r.x[3 * i + j] - r.X[3 * i + j];
  st->steps = step;
  st->residual = residual;
  if (nonfinite)
    st->status = MFG_E_NONFINITE;
  else if (r.mode == MFG_MODE_RELAX && residual > r.tol)
    st->status = MFG_E_NOT_CONVERGED;
  else
    st->status = MFG_OK;
}

// B:58-126 computeCauchyStress, serial order over the boundary list.
void cauchy_stress(const Rve& r, double* s) {
  for (int k = 0; k < 6; ++k) s[k] = 0;
  for (int b = 0; b < r.nb; ++b) {
    int vert = r.nfree + b;
    double f1 = r.fint[3 * vert], f2 = r.fint[3 * vert + 1], f3 = r.fint[3 * vert + 2];
    double crd1 = r.x[3 * vert], crd2 = r.x[3 * vert + 1], crd3 = r.x[3 * vert + 2];
    s[0] += crd1 * f1;
    s[1] += crd2 * f2;
    s[2] += crd3 * f3;
    s[3] += 0.5 * (crd2 * f3 + crd3 * f2);
    s[4] += 0.5 * (crd1 * f3 + crd3 * f1);
    s[5] += 0.5 * (crd1 * f2 + crd2 * f1);
  }
  for (int k = 0; k < 6; ++k) s[k] *= r.scale / r.V;
}

// B:127-154 updateVolume, one RVE.
inline double jacobian(const double* dg) {
  return dg[0] * (dg[4] * dg[8] - dg[5] * dg[7]) - dg[1] * (dg[3] * dg[8] - dg[5] * dg[6]) +
         dg[2] * (dg[3] * dg[7] - dg[4] * dg[6]);
}

// A:257-320 run(), one RVE.
void run_one(Rve& r, const double* F, double* sigma, bool update_coords, mfg_rve_status* st) {
  std::vector<double> u_copy;
  if (!update_coords)
    u_copy = r.u;  // A:264-267
  else
    r.V = jacobian(F) * r.V;  // A:271
  if (r.mode == MFG_MODE_RELAX) {
    for (int i = 0; i < r.N; ++i) affine_increment(F, &r.x[3 * i], &r.u[3 * i]);  // A:275
  }
  for (auto& vv : r.v) vv = 0;  // A:296
  relax(r, F, st);              // A:298
  cauchy_stress(r, sigma);      // A:306
  if (!update_coords)
    r.u = u_copy;  // A:309-313
  else
    for (int k = 0; k < 6; ++k) r.current_stress[k] = sigma[k];  // A:314-317
  if (!std::isfinite(sigma[0] + sigma[1] + sigma[2] + sigma[3] + sigma[4] + sigma[5]) &&
      st->status == MFG_OK)
    st->status = MFG_E_NONFINITE;
}

// Solves RVEs on n_threads host threads, one RVE per thread at a time, each
// thread taking the next unsolved RVE (balances RVEs of uneven size).
template <typename Fn>
void parallel_over(int n, int n_threads, Fn fn) {
  if (n_threads <= 1 || n <= 1) {
    for (int i = 0; i < n; ++i) fn(i);
    return;
  }
  if (n_threads > n) n_threads = n;
  std::atomic<int> next{0};
  std::vector<std::thread> th;
  for (int t = 0; t < n_threads; ++t) {
    th.emplace_back([&]() {
      for (int i = next++; i < n; i = next++) fn(i);
    });
  }
  for (auto& x : th) x.join();
}

// RVE.h:86-103 onBoundary(crd, side::all) with RVE(0.5) and eps = 1e-8.
inline bool on_boundary(const double* crd) {
  const double cr = 0.5, eps = 1e-8;
  return std::fabs(cr * 1.0 - crd[0]) < eps || std::fabs(cr * -1.0 - crd[0]) < eps ||
         std::fabs(cr * -1.0 - crd[1]) < eps || std::fabs(cr * 1.0 - crd[1]) < eps ||
         std::fabs(cr * -1.0 - crd[2]) < eps || std::fabs(cr * 1.0 - crd[2]) < eps;
}

}  // namespace

struct orc_batch {
  std::vector<Rve> rves;
};

extern "C" {

void orc_reorder_permutation(int32_t n_vert, const int32_t* fixed, int32_t n_fixed,
                             int32_t* perm) {
  // R:54-73: mark fixed vertices with their list position + 1, then a scan
  // gives free vertices i - (#fixed before i) and fixed ones nfree + position.
  for (int i = 0; i < n_vert; ++i) perm[i] = 0;
  for (int i = 0; i < n_fixed; ++i) perm[fixed[i]] = i + 1;
  int update = 0;
  for (int i = 0; i < n_vert; ++i) {
    int val = perm[i];
    bool is_fixed = val > 0;
    update += is_fixed ? 1 : 0;
    perm[i] = is_fixed ? (n_vert - n_fixed) + (val - 1) : i - update;
  }
}

int32_t orc_boundary_nodes(int32_t n_nodes, const double* coords, int32_t* out) {
  int32_t nb = 0;
  for (int i = 0; i < n_nodes; ++i)
    if (on_boundary(&coords[3 * i])) out[nb++] = i;
  return nb;
}

void orc_nodal_mass(int32_t n_nodes, const double* coords, int32_t n_fibers,
                    const int32_t* conn, double density, double area, double* mass) {
  // MassIntegrator.cc:16-56 with row-sum lumping: each fiber end receives
  // rho*A*L0/2, accumulated in fiber order (BatchedMesh.h:113-130).
  std::vector<double> X(coords, coords + 3 * n_nodes);
  for (int i = 0; i < n_nodes; ++i) mass[i] = 0;
  for (int e = 0; e < n_fibers; ++e) {
    int n1 = conn[2 * e], n2 = conn[2 * e + 1];
    double l0 = element_length(X, n1, n2);
    double me = density * area * l0 * 0.5;
    mass[n1] = mass[n1] + me;
    mass[n2] = mass[n2] + me;
  }
}

double orc_scale_conversion(int32_t n_nodes, const double* coords, int32_t n_fibers,
                            const int32_t* conn, double fiber_radius, double volume_fraction) {
  // MultiscaleCoupling.cc:7-23: the RVE edge d = sqrt(L A / vf) from the
  // summed edge lengths L (calcDimMeasures, Utility_impl.h:6-17, summed with
  // std::accumulate) and A = pi r^2 (MultiscaleRVEAnalysis.cc:162-163);
  // the conversion factor is 1 / d^2.
  std::vector<double> X(coords, coords + 3 * n_nodes);
  double total = 0.0;
  for (int e = 0; e < n_fibers; ++e) total += element_length(X, conn[2 * e], conn[2 * e + 1]);
  const double pi = 4 * std::atan(1.0);
  const double fbr_area = pi * fiber_radius * fiber_radius;
  const double rve_dim = std::sqrt(total * fbr_area / volume_fraction);
  return 1 / (rve_dim * rve_dim);
}

orc_batch* orc_batch_create(const mfg_network* nets, const mfg_strategy* ss, int32_t n_rve) {
  if (!nets || !ss || n_rve < 1) return nullptr;
  auto b = std::make_unique<orc_batch>();
  b->rves.resize(n_rve);
  for (int r = 0; r < n_rve; ++r) {
    const mfg_network& net = nets[r];
    Rve& rv = b->rves[r];
    const int N = net.n_nodes, E = net.n_fibers;
    if (N < 2 || E < 1) return nullptr;
    rv.N = N;
    rv.E = E;
    // reaction 0 and strategy (A:202-218)
    rv.law = net.reaction.law;
    rv.area = net.reaction.radius * net.reaction.radius * M_PI;  // FiberNetworkIO_impl.h:26
    rv.Emod = net.reaction.youngs_modulus;
    rv.rho = net.reaction.density;
    rv.B = net.reaction.B;
    rv.lt = net.reaction.length_ratio_trns;
    rv.c = ss[r].visc_damp_coeff;
    rv.crit = ss[r].crit_time_scale_factor;
    rv.tol = ss[r].residual_tol;
    rv.max_steps = ss[r].max_steps;
    rv.mode = ss[r].mode;
    rv.scale = net.scale_factor;
    rv.sound_speed = std::sqrt(rv.Emod / rv.rho);  // T:72
    // boundary (A:190-202), mass (A:280-283), reorder (A:284-291)
    std::vector<int32_t> fixed(N);
    int nb = orc_boundary_nodes(N, net.coords, fixed.data());
    fixed.resize(nb);
    rv.nb = nb;
    rv.nfree = N - nb;
    std::vector<double> mass(N);
    orc_nodal_mass(N, net.coords, E, net.connectivity, rv.rho, rv.area, mass.data());
    rv.perm.resize(N);
    orc_reorder_permutation(N, fixed.data(), nb, rv.perm.data());
    rv.X.assign(3 * N, 0.0);
    rv.m.assign(N, 0.0);
    for (int i = 0; i < N; ++i) {
      int p = rv.perm[i];
      for (int j = 0; j < 3; ++j) rv.X[3 * p + j] = net.coords[3 * i + j];
      rv.m[p] = mass[i];
    }
    rv.conn.resize(2 * E);
    for (int e = 0; e < 2 * E; ++e) rv.conn[e] = rv.perm[net.connectivity[e]];
    rv.x = rv.X;  // A:305-308
    rv.u.assign(3 * N, 0.0);
    rv.v.assign(3 * N, 0.0);
    rv.ftot.assign(3 * N, 0.0);
    rv.fint.assign(3 * N, 0.0);
    rv.l0.assign(E, 0.0);
    rv.l.assign(E, 0.0);
    rv.ramp0.assign(3 * nb, 0.0);
    rv.rampd.assign(3 * nb, 0.0);
    rv.V = 1.0;  // A:115-118
  }
  return b.release();
}

void orc_batch_destroy(orc_batch* b) { delete b; }

int32_t orc_batch_run(orc_batch* b, const double* F, int32_t n_F, double* sigma,
                      int32_t update_coords, mfg_rve_status* status, int32_t n_threads) {
  const int R = static_cast<int>(b->rves.size());
  if (!F || !sigma || (n_F != 1 && n_F != R)) return MFG_E_INVALID;
  if (update_coords && n_F != R) return MFG_E_INVALID;  // B:136-142
  std::vector<mfg_rve_status> st(R);
  parallel_over(R, n_threads, [&](int r) {
    const double* Fr = F + 9 * (n_F > 1 ? r : 0);
    run_one(b->rves[r], Fr, sigma + 6 * r, update_coords != 0, &st[r]);
  });
  int32_t worst = MFG_OK;
  for (int r = 0; r < R; ++r) {
    if (status) status[r] = st[r];
    if (st[r].status > worst) worst = st[r].status;
  }
  return worst;
}

int32_t orc_batch_material_stiffness(orc_batch* b, double* C, int32_t n_threads) {
  // A:321-405
  const int R = static_cast<int>(b->rves.size());
  constexpr double h = 1E-5;
  double D1 = std::sqrt(1.0 / (1 - 2 * h));
  constexpr double l1 = 1;
  constexpr double l2 = (1 + h) / (1 - h * h);
  constexpr double l3 = (1 - h) / (1 - h * h);
  double l2pl3 = 0.5 * (std::sqrt(l2) + std::sqrt(l3));
  double l2ml3 = 0.5 * (std::sqrt(l2) - std::sqrt(l3));
  std::vector<double> sigma1(6 * R);
  int32_t worst = MFG_OK;
  for (int i = 0; i < 6; ++i) {
    double Fa[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    switch (i) {
      case 0: Fa[0] = D1; Fa[4] = 1; Fa[8] = 1; break;
      case 1: Fa[0] = 1; Fa[4] = D1; Fa[8] = 1; break;
      case 2: Fa[0] = 1; Fa[4] = 1; Fa[8] = D1; break;
      case 3: Fa[0] = l1; Fa[4] = l2pl3; Fa[8] = l2pl3; Fa[5] = l2ml3; Fa[7] = l2ml3; break;
      case 4: Fa[0] = l2pl3; Fa[4] = l1; Fa[8] = l2pl3; Fa[2] = l2ml3; Fa[6] = l2ml3; break;
      case 5: Fa[0] = l2pl3; Fa[4] = l2pl3; Fa[8] = l1; Fa[1] = l2ml3; Fa[3] = l2ml3; break;
    }
    int32_t s = orc_batch_run(b, Fa, 1, sigma1.data(), 0, nullptr, n_threads);
    if (s > worst) worst = s;
    for (int r = 0; r < R; ++r)
      for (int j = 0; j < 6; ++j)
        C[36 * r + 6 * j + i] = (sigma1[6 * r + j] - b->rves[r].current_stress[j]) / h;
  }
  return worst;
}

int32_t orc_batch_orientation_3d(orc_batch* b, double* omega) {
  // O:145-186 on the current coordinates, serial fiber order.
  for (size_t r = 0; r < b->rves.size(); ++r) {
    const Rve& rv = b->rves[r];
    double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int e = 0; e < rv.E; ++e) {
      int n1 = rv.conn[2 * e], n2 = rv.conn[2 * e + 1];
      double lx = rv.x[3 * n2] - rv.x[3 * n1];
      double ly = rv.x[3 * n2 + 1] - rv.x[3 * n1 + 1];
      double lz = rv.x[3 * n2 + 2] - rv.x[3 * n1 + 2];
      double l = std::sqrt(lx * lx + ly * ly + lz * lz);
      lx = lx / l;
      ly = ly / l;
      lz = lz / l;
      double d[3] = {lx, ly, lz};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) s[3 * i + j] += d[i] * d[j];
    }
    for (int k = 0; k < 9; ++k) omega[9 * r + k] = s[k] / rv.E;
  }
  return MFG_OK;
}

int32_t orc_batch_orientation_2d(orc_batch* b, const double* normal, double* omega) {
  // O:55-144. The reference "normalises" the normal by its squared length.
  for (size_t r = 0; r < b->rves.size(); ++r) {
    const Rve& rv = b->rves[r];
    double nv[3] = {normal[3 * r], normal[3 * r + 1], normal[3 * r + 2]};
    double n = nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2];
    nv[0] = nv[0] / n;
    nv[1] = nv[1] / n;
    nv[2] = nv[2] / n;
    double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int e = 0; e < rv.E; ++e) {
      int n1 = rv.conn[2 * e], n2 = rv.conn[2 * e + 1];
      double lx = rv.x[3 * n2] - rv.x[3 * n1];
      double ly = rv.x[3 * n2 + 1] - rv.x[3 * n1 + 1];
      double lz = rv.x[3 * n2 + 2] - rv.x[3 * n1 + 2];
      double l = std::sqrt(lx * lx + ly * ly + lz * lz);
      lx = lx / l;
      ly = ly / l;
      lz = lz / l;
      double dotn = lx * nv[0] + ly * nv[1] + lz * nv[2];
      lx = lx - nv[0] * dotn;
      ly = ly - nv[1] * dotn;
      lz = lz - nv[2] * dotn;
      l = std::sqrt(lx * lx + ly * ly + lz * lz);
      lx = lx / l;
      ly = ly / l;
      lz = lz / l;
      double d[3] = {lx, ly, lz};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) s[3 * i + j] += d[i] * d[j];
    }
    for (int k = 0; k < 9; ++k) omega[9 * r + k] = s[k] / rv.E;
  }
  return MFG_OK;
}

int32_t orc_batch_get_displacements(orc_batch* b, int32_t rve, double* u) {
  if (rve < 0 || rve >= static_cast<int32_t>(b->rves.size())) return MFG_E_INVALID;
  const Rve& rv = b->rves[rve];
  for (int i = 0; i < rv.N; ++i)
    for (int j = 0; j < 3; ++j) u[3 * i + j] = rv.u[3 * rv.perm[i] + j];
  return MFG_OK;
}

int32_t orc_batch_get_coordinates(orc_batch* b, int32_t rve, double* x) {
  if (rve < 0 || rve >= static_cast<int32_t>(b->rves.size())) return MFG_E_INVALID;
  const Rve& rv = b->rves[rve];
  for (int i = 0; i < rv.N; ++i)
    for (int j = 0; j < 3; ++j) x[3 * i + j] = rv.x[3 * rv.perm[i] + j];
  return MFG_OK;
}

int32_t orc_batch_get_current_stress(orc_batch* b, double* sigma) {
  for (size_t r = 0; r < b->rves.size(); ++r)
    for (int k = 0; k < 6; ++k) sigma[6 * r + k] = b->rves[r].current_stress[k];
  return MFG_OK;
}

}  // extern "C"
