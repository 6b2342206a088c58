// Host side of the C ABI in include/mumfim_gpu.h.
//
// Set-up restates the constructor of the reference's batched analysis
// (src/mumfim/microscale/BatchedFiberRVEAnalysisExplicit.h:80-256) on plain
// arrays: boundary nodes (RVE.h:86-103, RVE_impl.h:5-20), row-sum lumped mass
// (MassIntegrator.cc:16-56 via BatchedMesh.h:113-130), boundary-last
// permutation (BatchedReorderMesh.h:54-73), plus the CSR fiber incidence the
// GPU kernels gather forces over. Compiled with -ffp-contract=off: the mass
// and reference lengths computed here feed the bit-exact FP64 kernel.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "mfg_internal.h"
#include "mfg_metrics.h"
#include "mfg_mixed.h"
#include "mumfim_gpu.h"

namespace {

thread_local std::string g_last_error;

mfg_status fail(mfg_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return s;
}

}  // namespace

namespace mfg {
// Error message for mfg_last_error() from the library's other host files.
mfg_status set_error(mfg_status s, const char* msg) { return fail(s, "%s", msg); }
}  // namespace mfg

namespace {

#define MFG_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(e_ == cudaErrorMemoryAllocation ? MFG_E_OOM : MFG_E_CUDA, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                    \
  } while (0)

// RVE(0.5).onBoundary(crd, side::all) with eps = 1e-8 (RVE.h:86-103).
inline bool on_boundary(const double* crd) {
  const double cr = 0.5, eps = 1e-8;
  return std::fabs(cr * 1.0 - crd[0]) < eps || std::fabs(cr * -1.0 - crd[0]) < eps ||
         std::fabs(cr * -1.0 - crd[1]) < eps || std::fabs(cr * 1.0 - crd[1]) < eps ||
         std::fabs(cr * -1.0 - crd[2]) < eps || std::fabs(cr * 1.0 - crd[2]) < eps;
}

// getElementLength (BatchedFiberRVEAnalysisExplicitBase.h:203-215).
inline double seg_length(const double* a, const double* b) {
  double x1 = b[0] - a[0];
  double x2 = b[1] - a[1];
  double x3 = b[2] - a[2];
  return std::sqrt(x1 * x1 + x2 * x2 + x3 * x3);
}

// Host-side product of the set-up of one RVE, solver (boundary-last) order.
struct RveSetup {
  int n_nodes = 0, n_free = 0, n_fibers = 0;
  std::vector<int32_t> perm;  // original id -> storage id
  std::vector<double> X;      // 3 x n_nodes, component blocks
  std::vector<double> m;
  std::vector<int32_t> conn;  // 2 x n_fibers interleaved (n1, n2)
  std::vector<double> l0;
  std::vector<int32_t> rowptr;  // n_nodes + 1
  std::vector<int32_t> inc;     // 2 * n_fibers
  std::vector<int32_t> bnd_order;  // boundary nodes in the reference's order
  std::string error;
};

void setup_rve(const mfg_network& net, RveSetup& s) {
  const int N = net.n_nodes, E = net.n_fibers;
  if (N < 2 || E < 1 || !net.coords || !net.connectivity) {
    s.error = "network needs at least 2 nodes, 1 fiber and non-null arrays";
    return;
  }
  for (int64_t k = 0; k < 3LL * N; ++k)
    if (!std::isfinite(net.coords[k])) {
      s.error = "non-finite node coordinate";
      return;
    }
  for (int e = 0; e < E; ++e) {
    int a = net.connectivity[2 * e], b = net.connectivity[2 * e + 1];
    if (a < 0 || b < 0 || a >= N || b >= N) {
      s.error = "fiber " + std::to_string(e) + " references a node outside [0, n_nodes)";
      return;
    }
    if (a == b) {
      s.error = "fiber " + std::to_string(e) + " is a self-loop";
      return;
    }
  }
  const mfg_reaction& rc = net.reaction;
  const double area = rc.radius * rc.radius * M_PI;  // FiberNetworkIO_impl.h:26
  // boundary list in mesh order (BatchedFiberRVEAnalysisExplicit.h:190-202)
  std::vector<int32_t> fixed;
  for (int i = 0; i < N; ++i)
    if (on_boundary(&net.coords[3 * i])) fixed.push_back(i);
  const int nb = static_cast<int>(fixed.size());
  // row-sum lumped mass, original order, fiber order
  std::vector<double> mass(N, 0.0);
  std::vector<int> degree(N, 0);
  for (int e = 0; e < E; ++e) {
    int n1 = net.connectivity[2 * e], n2 = net.connectivity[2 * e + 1];
    double l0 = seg_length(&net.coords[3 * n1], &net.coords[3 * n2]);
    if (!(l0 > 0.0)) {
      s.error = "fiber " + std::to_string(e) + " has zero length";
      return;
    }
    double me = rc.density * area * l0 * 0.5;
    mass[n1] = mass[n1] + me;
    mass[n2] = mass[n2] + me;
    degree[n1]++;
    degree[n2]++;
  }
  // boundary-last permutation (BatchedReorderMesh.h:54-73)
  std::vector<int32_t> ref(N, 0);
  for (int i = 0; i < nb; ++i) ref[fixed[i]] = i + 1;
  int update = 0;
  for (int i = 0; i < N; ++i) {
    int val = ref[i];
    bool is_fixed = val > 0;
    update += is_fixed ? 1 : 0;
    ref[i] = is_fixed ? (N - nb) + (val - 1) : i - update;
  }
  for (int i = 0; i < N; ++i)
    if (degree[i] == 0 && ref[i] < N - nb) {
      s.error = "free node " + std::to_string(i) + " has no fibers (zero lumped mass)";
      return;
    }
  // Storage order: still boundary-last, but each segment sorted along a
  // Morton curve of the reference coordinates, so that a fiber's two end
  // nodes sit close together in memory. Nothing numerical depends on it:
  // each node's CSR row keeps the original fiber order and the stress visits
  // the boundary in the reference's order (bnd_order).
  auto morton = [&](int i) {
    uint64_t code = 0;
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
      double t = (net.coords[3 * i + k] + 0.5) * 1024.0;
      q[k] = static_cast<uint32_t>(t < 0 ? 0 : (t > 1023 ? 1023 : t));
    }
    for (int bit = 9; bit >= 0; --bit)
      for (int k = 0; k < 3; ++k) code = (code << 1) | ((q[k] >> bit) & 1u);
    return code;
  };
  std::vector<int32_t> by_ref(N);
  for (int i = 0; i < N; ++i) by_ref[ref[i]] = i;  // reference order -> original id
  std::vector<uint64_t> key(N);
  for (int i = 0; i < N; ++i) key[i] = morton(i);
  std::vector<int32_t> store(by_ref);
  std::stable_sort(store.begin(), store.begin() + (N - nb),
                   [&](int a, int b) { return key[a] < key[b]; });
  std::stable_sort(store.begin() + (N - nb), store.end(),
                   [&](int a, int b) { return key[a] < key[b]; });
  s.perm.assign(N, 0);
  for (int j = 0; j < N; ++j) s.perm[store[j]] = j;
  s.bnd_order.resize(nb);
  for (int k = 0; k < nb; ++k) s.bnd_order[k] = s.perm[by_ref[N - nb + k]];
  s.n_nodes = N;
  s.n_free = N - nb;
  s.n_fibers = E;
  s.X.assign(3 * static_cast<size_t>(N), 0.0);
  s.m.assign(N, 0.0);
  for (int i = 0; i < N; ++i) {
    int p = s.perm[i];
    for (int k = 0; k < 3; ++k) s.X[static_cast<size_t>(k) * N + p] = net.coords[3 * i + k];
    s.m[p] = mass[i];
  }
  // fiber slots ordered by their lower end node, then the other end
  std::vector<int32_t> slot_fiber(E);
  std::iota(slot_fiber.begin(), slot_fiber.end(), 0);
  auto ends = [&](int e) {
    int a = s.perm[net.connectivity[2 * e]], b = s.perm[net.connectivity[2 * e + 1]];
    return std::make_pair(std::min(a, b), std::max(a, b));
  };
  std::stable_sort(slot_fiber.begin(), slot_fiber.end(),
                   [&](int x, int y) { return ends(x) < ends(y); });
  std::vector<int32_t> fiber_slot(E);
  for (int j = 0; j < E; ++j) fiber_slot[slot_fiber[j]] = j;
  s.conn.resize(2 * static_cast<size_t>(E));
  s.l0.resize(E);
  std::vector<int32_t> cnt(N + 1, 0);
  for (int j = 0; j < E; ++j) {
    const int e = slot_fiber[j];
    int a = s.perm[net.connectivity[2 * e]], b = s.perm[net.connectivity[2 * e + 1]];
    s.conn[2 * j] = a;
    s.conn[2 * j + 1] = b;
    double pa[3] = {s.X[a], s.X[N + a], s.X[2 * static_cast<size_t>(N) + a]};
    double pb[3] = {s.X[b], s.X[N + b], s.X[2 * static_cast<size_t>(N) + b]};
    s.l0[j] = seg_length(pa, pb);
    cnt[a + 1]++;
    cnt[b + 1]++;
  }
  // CSR incidence: per node, fibers in ascending ORIGINAL id (the serial
  // scatter order), stored as (slot << 1) | end with end 0 = first node.
  s.rowptr.assign(N + 1, 0);
  for (int i = 0; i < N; ++i) s.rowptr[i + 1] = s.rowptr[i] + cnt[i + 1];
  s.inc.resize(2 * static_cast<size_t>(E));
  std::vector<int32_t> fill(s.rowptr.begin(), s.rowptr.end() - 1);
  for (int e = 0; e < E; ++e)
    for (int j = 0; j < 2; ++j) {
      const int node = s.perm[net.connectivity[2 * e + j]];
      s.inc[fill[node]++] = (fiber_slot[e] << 1) | j;
    }
}

template <typename Fn>
void parallel_for(int n, Fn fn) {
  int nt = static_cast<int>(std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), 32u));
  if (n < 4 || nt <= 1) {
    for (int i = 0; i < n; ++i) fn(i);
    return;
  }
  nt = std::min(nt, n);
  std::atomic<int> next{0};
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&]() {
      for (int i = next++; i < n; i = next++) fn(i);
    });
  for (auto& x : th) x.join();
}

template <typename T>
struct DevArray {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    n = std::max<size_t>(count, 1);
    return cudaMalloc(&p, n * sizeof(T));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
  }
};

// Scratch of the concurrent perturbed solves of the material stiffness: six
// sets of every array a non-updating run writes (coordinates, velocities,
// internal forces, force vectors, RAMP data, stresses, status words, work
// counter), allocated on first use and kept with the batch.
constexpr int kStiffSlots = 6;
struct StiffSlots {
  bool ready = false;
  DevArray<double> x, v, fint, nrm, ramp, sigma, res, F;
  DevArray<int32_t> status, steps, queue;
  cudaStream_t st[kStiffSlots] = {};
  cudaEvent_t fork = nullptr, join[kStiffSlots] = {};
  void release() {
    for (auto* a : {&x, &v, &fint, &nrm, &ramp, &sigma, &res, &F}) a->release();
    for (auto* a : {&status, &steps, &queue}) a->release();
    for (int k = 0; k < kStiffSlots; ++k) {
      if (st[k]) cudaStreamDestroy(st[k]);
      if (join[k]) cudaEventDestroy(join[k]);
      st[k] = nullptr;
      join[k] = nullptr;
    }
    if (fork) cudaEventDestroy(fork);
    fork = nullptr;
    ready = false;
  }
};

// The six perturbation gradients of the FD stiffness, row-major, h = 1e-5
// (BatchedFiberRVEAnalysisExplicit.h:331-395).
constexpr double kStiffH = 1E-5;
void perturbation_gradients(double Fa[kStiffSlots][9]) {
  constexpr double h = kStiffH;
  double D1 = std::sqrt(1.0 / (1 - 2 * h));
  constexpr double l1 = 1;
  constexpr double l2 = (1 + h) / (1 - h * h);
  constexpr double l3 = (1 - h) / (1 - h * h);
  double l2pl3 = 0.5 * (std::sqrt(l2) + std::sqrt(l3));
  double l2ml3 = 0.5 * (std::sqrt(l2) - std::sqrt(l3));
  for (int i = 0; i < kStiffSlots; ++i) {
    double* F = Fa[i];
    for (int k = 0; k < 9; ++k) F[k] = 0;
    switch (i) {
      case 0: F[0] = D1; F[4] = 1; F[8] = 1; break;
      case 1: F[0] = 1; F[4] = D1; F[8] = 1; break;
      case 2: F[0] = 1; F[4] = 1; F[8] = D1; break;
      case 3: F[0] = l1; F[4] = l2pl3; F[8] = l2pl3; F[5] = l2ml3; F[7] = l2ml3; break;
      case 4: F[0] = l2pl3; F[4] = l1; F[8] = l2pl3; F[2] = l2ml3; F[6] = l2ml3; break;
      default: F[0] = l2pl3; F[4] = l2pl3; F[8] = l1; F[1] = l2ml3; F[3] = l2ml3; break;
    }
  }
}

}  // namespace

struct mfg_batch {
  int device = 0;
  int precision = MFG_PREC_F64;
  int R = 0;
  int64_t nt = 0, et = 0, nbt = 0;
  std::vector<int> n_nodes, n_free, n_fibers;
  std::vector<std::vector<int32_t>> perm;
  std::vector<mfg::RveDesc> desc;
  int sms = 1;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_run0 = nullptr, ev_relax0 = nullptr, ev_relax1 = nullptr, ev_run1 = nullptr;
  int last_launches = 0;
  bool timing_valid = false;
  // device buffers
  DevArray<mfg::RveDesc> d_desc;
  DevArray<double> d_X, d_x, d_u, d_v, d_m, d_l0, d_nrm, d_fint, d_ramp, d_vol, d_cur;
  DevArray<int2> d_conn;
  DevArray<int32_t> d_rowptr, d_inc, d_bnd, d_order, d_queue;
  // per-run scratch
  DevArray<double> d_F, d_sigma, d_res, d_omega;
  DevArray<int32_t> d_status, d_steps;
  DevArray<mfg_rve_status> d_st;
  mfg::DevBatch dev{};
  std::unique_ptr<mfg::MixedState, mfg::MixedStateDeleter> mixed;
  int stiffness = MFG_STIFFNESS_AUTO;
  bool all_ramp = false;
  StiffSlots stiff;

  ~mfg_batch() {
    if (device >= 0) cudaSetDevice(device);
    stiff.release();
    mixed.reset();
    for (auto* a : {&d_X, &d_x, &d_u, &d_v, &d_m, &d_l0, &d_nrm, &d_fint, &d_ramp, &d_vol, &d_cur,
                    &d_F, &d_sigma, &d_res, &d_omega})
      a->release();
    d_desc.release();
    d_conn.release();
    for (auto* a : {&d_rowptr, &d_inc, &d_bnd, &d_order, &d_queue, &d_status, &d_steps})
      a->release();
    d_st.release();
    for (auto* e : {&ev_run0, &ev_relax0, &ev_relax1, &ev_run1})
      if (*e) cudaEventDestroy(*e);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

mfg_status check_strategy(const mfg_strategy& s, int r) {
  if (!(s.visc_damp_coeff >= 0.0) || !std::isfinite(s.visc_damp_coeff))
    return fail(MFG_E_INVALID, "rve %d: damping must be finite and >= 0", r);
  if (!(s.crit_time_scale_factor > 0.0) || !std::isfinite(s.crit_time_scale_factor))
    return fail(MFG_E_INVALID, "rve %d: critical time scale factor must be > 0", r);
  if (!(s.residual_tol >= 0.0) || !std::isfinite(s.residual_tol))
    return fail(MFG_E_INVALID, "rve %d: residual tolerance must be finite and >= 0", r);
  if (s.mode != MFG_MODE_RELAX && s.mode != MFG_MODE_RAMP)
    return fail(MFG_E_INVALID, "rve %d: unknown mode %d", r, s.mode);
  if (s.mode == MFG_MODE_RAMP && s.max_steps < 1)
    return fail(MFG_E_INVALID, "rve %d: RAMP mode needs max_steps >= 1", r);
  return MFG_OK;
}

mfg_status check_reaction(const mfg_reaction& rc, int r) {
  if (rc.law != MFG_LAW_LINEAR && rc.law != MFG_LAW_NONLINEAR)
    return fail(MFG_E_INVALID, "rve %d: unknown fiber law %d", r, rc.law);
  if (!(rc.radius > 0) || !(rc.youngs_modulus > 0) || !(rc.density > 0) ||
      !std::isfinite(rc.radius) || !std::isfinite(rc.youngs_modulus) || !std::isfinite(rc.density))
    return fail(MFG_E_INVALID, "rve %d: radius, modulus and density must be finite and > 0", r);
  if (rc.law == MFG_LAW_NONLINEAR &&
      (!(rc.B > 0) || !std::isfinite(rc.B) || !(rc.length_ratio_trns >= 1.0) ||
       !std::isfinite(rc.length_ratio_trns)))
    return fail(MFG_E_INVALID, "rve %d: nonlinear law needs B > 0 and length_ratio_trns >= 1", r);
  return MFG_OK;
}

template <typename T>
mfg_status upload(DevArray<T>& d, const std::vector<T>& h, cudaStream_t s) {
  MFG_CUDA(d.alloc(h.size()));
  if (!h.empty()) MFG_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return MFG_OK;
}

mfg_status enqueue_run(mfg_batch* b, const double* F_dev, int32_t n_F, double* sigma_dev,
                       int32_t update_coords, cudaStream_t s) {
  MFG_CUDA(cudaMemsetAsync(b->d_queue.p, 0, sizeof(int32_t), s));
  mfg::RunArgs a{};
  a.F = F_dev;
  a.n_F = n_F;
  a.update_coords = update_coords;
  a.sigma = sigma_dev;
  a.st_status = b->d_status.p;
  a.st_steps = b->d_steps.p;
  a.st_residual = b->d_res.p;
  MFG_CUDA(cudaEventRecord(b->ev_relax0, s));
  cudaError_t e;
  if (b->precision == MFG_PREC_MIXED) {
    e = mfg::run_mixed(*b->mixed, b->dev, a, s, &b->last_launches);
  } else {
    int occ = mfg::relax_f64_max_blocks_per_sm(0);
    int grid = std::min(b->R, b->sms * occ);
    e = mfg::launch_relax_f64(b->dev, a, 0, grid, s);
    b->last_launches = 1;
  }
  if (e != cudaSuccess)
    return fail(MFG_E_CUDA, "relaxation launch failed: %s", cudaGetErrorString(e));
  MFG_CUDA(cudaEventRecord(b->ev_relax1, s));
  return MFG_OK;
}

mfg_status check_run_args(mfg_batch* b, int32_t n_F, int32_t update_coords) {
  if (n_F != 1 && n_F != b->R)
    return fail(MFG_E_INVALID, "F must hold 1 or n_rve (%d) matrices, got %d", b->R, n_F);
  if (update_coords && n_F != b->R)
    // BatchedFiberRVEAnalysisExplicitBase.h:136-142
    return fail(MFG_E_INVALID,
                "The volume and deformation gradients must have the same extent corresponding "
                "to the number of RVEs.");
  return MFG_OK;
}

}  // namespace

extern "C" {

int32_t mfg_abi_version(void) { return MFG_ABI_VERSION; }

const char* mfg_status_string(mfg_status s) {
  switch (s) {
    case MFG_OK: return "MFG_OK";
    case MFG_E_INVALID: return "MFG_E_INVALID";
    case MFG_E_OOM: return "MFG_E_OOM";
    case MFG_E_NOT_CONVERGED: return "MFG_E_NOT_CONVERGED";
    case MFG_E_NONFINITE: return "MFG_E_NONFINITE";
    case MFG_E_TIMEOUT: return "MFG_E_TIMEOUT";
    case MFG_E_CUDA: return "MFG_E_CUDA";
    case MFG_E_NO_DEVICE: return "MFG_E_NO_DEVICE";
    case MFG_E_BUSY: return "MFG_E_BUSY";
  }
  return "MFG_E_UNKNOWN";
}

const char* mfg_last_error(void) { return g_last_error.c_str(); }

void mfg_default_strategy(mfg_strategy* out) {
  if (!out) return;
  out->visc_damp_coeff = 0.5;
  out->crit_time_scale_factor = 0.8;
  out->residual_tol = 1e-6;
  out->max_steps = 0;
  out->mode = MFG_MODE_RELAX;
}

void mfg_default_options(mfg_options* out) {
  if (!out) return;
  std::memset(out, 0, sizeof(*out));
  out->precision = MFG_PREC_F64;
}

static mfg_status batch_create_impl(const mfg_network* nets, const mfg_strategy* strategies,
                                    int32_t n_rve, const mfg_options* options, mfg_batch** out) {
  mfg::Trace trace("mfg_batch_create");
  g_last_error.clear();
  if (!out) return fail(MFG_E_INVALID, "out is NULL");
  *out = nullptr;
  if (!nets || !strategies || n_rve < 1)
    return fail(MFG_E_INVALID, "There must be a solution strategy for each fiber network!");
  mfg_options opt;
  mfg_default_options(&opt);
  if (options) opt = *options;
  if (opt.precision != MFG_PREC_F64 && opt.precision != MFG_PREC_MIXED)
    return fail(MFG_E_INVALID, "unknown precision %d", opt.precision);
  if (opt.max_cluster_ctas != 0 && opt.max_cluster_ctas != 1 && opt.max_cluster_ctas != 2 &&
      opt.max_cluster_ctas != 4 && opt.max_cluster_ctas != 8)
    return fail(MFG_E_INVALID, "max_cluster_ctas must be 0, 1, 2, 4 or 8 (got %d)",
                opt.max_cluster_ctas);
  if (opt.cluster_layout != MFG_LAYOUT_BATCH && opt.cluster_layout != MFG_LAYOUT_SERVING)
    return fail(MFG_E_INVALID, "cluster_layout must be MFG_LAYOUT_BATCH or MFG_LAYOUT_SERVING "
                "(got %d)", opt.cluster_layout);
  if (opt.small_rves_per_cta < 0 || opt.small_rves_per_cta > 2)
    return fail(MFG_E_INVALID, "small_rves_per_cta must be 0, 1 or 2 (got %d)",
                opt.small_rves_per_cta);
  if (opt.small_rve_solve != MFG_SMALL_AUTO && opt.small_rve_solve != MFG_SMALL_NODE_CENTRIC &&
      opt.small_rve_solve != MFG_SMALL_FIBER_CENTRIC)
    return fail(MFG_E_INVALID, "small_rve_solve must be MFG_SMALL_AUTO, _NODE_CENTRIC or "
                "_FIBER_CENTRIC (got %d)", opt.small_rve_solve);
  if (opt.stiffness != MFG_STIFFNESS_AUTO && opt.stiffness != MFG_STIFFNESS_SEQUENTIAL &&
      opt.stiffness != MFG_STIFFNESS_CONCURRENT)
    return fail(MFG_E_INVALID, "stiffness must be MFG_STIFFNESS_AUTO, _SEQUENTIAL or _CONCURRENT "
                "(got %d)", opt.stiffness);
  for (int r = 0; r < n_rve; ++r) {
    mfg_status st = check_strategy(strategies[r], r);
    if (st != MFG_OK) return st;
    st = check_reaction(nets[r].reaction, r);
    if (st != MFG_OK) return st;
    if (!(nets[r].scale_factor > 0) || !std::isfinite(nets[r].scale_factor))
      return fail(MFG_E_INVALID, "rve %d: scale factor must be finite and > 0", r);
  }
  // ---- host set-up, in parallel over RVEs ------------------------------
  std::vector<RveSetup> su(n_rve);
  parallel_for(n_rve, [&](int r) { setup_rve(nets[r], su[r]); });
  for (int r = 0; r < n_rve; ++r)
    if (!su[r].error.empty()) return fail(MFG_E_INVALID, "rve %d: %s", r, su[r].error.c_str());

  // ---- device ------------------------------------------------------------
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
    return fail(MFG_E_NO_DEVICE, "no CUDA device available");
  if (opt.device < 0 || opt.device >= ndev)
    return fail(MFG_E_NO_DEVICE, "device %d out of range (%d devices)", opt.device, ndev);
  MFG_CUDA(cudaSetDevice(opt.device));
  cudaDeviceProp prop;
  MFG_CUDA(cudaGetDeviceProperties(&prop, opt.device));
  if (prop.major < 10)
    return fail(MFG_E_NO_DEVICE, "device %d (%s, sm_%d%d) is not a Blackwell GPU", opt.device,
                prop.name, prop.major, prop.minor);

  std::unique_ptr<mfg_batch> b(new mfg_batch());
  b->device = opt.device;
  b->precision = opt.precision;
  b->stiffness = opt.stiffness;
  b->all_ramp = true;
  for (int r = 0; r < n_rve; ++r) b->all_ramp = b->all_ramp && strategies[r].mode == MFG_MODE_RAMP;
  b->R = n_rve;
  b->sms = prop.multiProcessorCount;
  b->n_nodes.resize(n_rve);
  b->n_free.resize(n_rve);
  b->n_fibers.resize(n_rve);
  b->perm.resize(n_rve);
  b->desc.resize(n_rve);
  int64_t no = 0, fo = 0, io = 0, ro = 0, bo = 0;
  for (int r = 0; r < n_rve; ++r) {
    const RveSetup& s = su[r];
    mfg::RveDesc& d = b->desc[r];
    std::memset(&d, 0, sizeof(d));
    d.node_off = no;
    d.fiber_off = fo;
    d.inc_off = io;
    d.row_off = ro;
    d.bnd_off = bo;
    d.n_nodes = s.n_nodes;
    d.n_free = s.n_free;
    d.n_fibers = s.n_fibers;
    const mfg_reaction& rc = nets[r].reaction;
    const mfg_strategy& st = strategies[r];
    d.law = rc.law;
    d.E = rc.youngs_modulus;
    d.A = rc.radius * rc.radius * M_PI;
    d.B = rc.B;
    d.lt = rc.length_ratio_trns;
    d.c = st.visc_damp_coeff;
    d.crit = st.crit_time_scale_factor;
    d.tol = st.residual_tol;
    d.mode = st.mode;
    d.max_steps = st.mode == MFG_MODE_RAMP ? st.max_steps
                                           : (st.max_steps > 0 ? st.max_steps : MFG_DEFAULT_STEP_CAP);
    d.sound_speed = std::sqrt(rc.youngs_modulus / rc.density);  // TeamOuterLoop.h:72
    d.scale = nets[r].scale_factor;
    no += s.n_nodes;
    fo += s.n_fibers;
    io += 2LL * s.n_fibers;
    ro += s.n_nodes + 1;
    bo += s.n_nodes - s.n_free;
    b->n_nodes[r] = s.n_nodes;
    b->n_free[r] = s.n_free;
    b->n_fibers[r] = s.n_fibers;
    b->perm[r] = s.perm;
  }
  b->nt = no;
  b->et = fo;
  b->nbt = bo;
  const int64_t nt = no, et = fo;

  // ---- pack ------------------------------------------------------------
  std::vector<double> X(3 * nt), m(nt), l0(et);
  std::vector<int2> conn(et);
  std::vector<int32_t> rowptr(ro), inc(io), bnd(std::max<int64_t>(bo, 1));
  parallel_for(n_rve, [&](int r) {
    const RveSetup& s = su[r];
    const mfg::RveDesc& d = b->desc[r];
    const int N = s.n_nodes;
    for (int k = 0; k < 3; ++k)
      std::memcpy(&X[k * nt + d.node_off], &s.X[static_cast<size_t>(k) * N], N * sizeof(double));
    std::memcpy(&m[d.node_off], s.m.data(), N * sizeof(double));
    for (int e = 0; e < s.n_fibers; ++e) conn[d.fiber_off + e] = make_int2(s.conn[2 * e], s.conn[2 * e + 1]);
    std::memcpy(&l0[d.fiber_off], s.l0.data(), s.n_fibers * sizeof(double));
    std::memcpy(&rowptr[d.row_off], s.rowptr.data(), (N + 1) * sizeof(int32_t));
    std::memcpy(&inc[d.inc_off], s.inc.data(), 2 * s.n_fibers * sizeof(int32_t));
    if (!s.bnd_order.empty())
      std::memcpy(&bnd[d.bnd_off], s.bnd_order.data(), s.bnd_order.size() * sizeof(int32_t));
  });
  // persistent-queue order: most fibers first (longest-processing-time first)
  std::vector<int32_t> order(n_rve);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    return b->n_fibers[a] > b->n_fibers[c];
  });

  // ---- device ------------------------------------------------------------
  MFG_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  for (auto* e : {&b->ev_run0, &b->ev_relax0, &b->ev_relax1, &b->ev_run1})
    MFG_CUDA(cudaEventCreate(e));
  cudaStream_t s = b->stream;
  mfg_status st;
  if ((st = upload(b->d_desc, b->desc, s)) != MFG_OK) return st;
  if ((st = upload(b->d_X, X, s)) != MFG_OK) return st;
  MFG_CUDA(b->d_x.alloc(3 * nt));
  MFG_CUDA(cudaMemcpyAsync(b->d_x.p, b->d_X.p, 3 * nt * sizeof(double), cudaMemcpyDeviceToDevice, s));
  MFG_CUDA(b->d_u.alloc(3 * nt));
  MFG_CUDA(cudaMemsetAsync(b->d_u.p, 0, 3 * nt * sizeof(double), s));
  MFG_CUDA(b->d_v.alloc(3 * nt));
  MFG_CUDA(cudaMemsetAsync(b->d_v.p, 0, 3 * nt * sizeof(double), s));
  MFG_CUDA(b->d_fint.alloc(3 * nt));
  MFG_CUDA(cudaMemsetAsync(b->d_fint.p, 0, 3 * nt * sizeof(double), s));
  if ((st = upload(b->d_m, m, s)) != MFG_OK) return st;
  if ((st = upload(b->d_conn, conn, s)) != MFG_OK) return st;
  if ((st = upload(b->d_l0, l0, s)) != MFG_OK) return st;
  MFG_CUDA(b->d_nrm.alloc(3 * et));
  if ((st = upload(b->d_rowptr, rowptr, s)) != MFG_OK) return st;
  if ((st = upload(b->d_inc, inc, s)) != MFG_OK) return st;
  if ((st = upload(b->d_bnd, bnd, s)) != MFG_OK) return st;
  MFG_CUDA(b->d_ramp.alloc(6 * std::max<int64_t>(b->nbt, 1)));
  std::vector<double> ones(n_rve, 1.0);  // BatchedFiberRVEAnalysisExplicit.h:115-118
  if ((st = upload(b->d_vol, ones, s)) != MFG_OK) return st;
  MFG_CUDA(b->d_cur.alloc(6 * n_rve));
  MFG_CUDA(cudaMemsetAsync(b->d_cur.p, 0, 6 * n_rve * sizeof(double), s));
  if ((st = upload(b->d_order, order, s)) != MFG_OK) return st;
  MFG_CUDA(b->d_queue.alloc(1));
  MFG_CUDA(b->d_F.alloc(9 * n_rve));
  MFG_CUDA(b->d_sigma.alloc(6 * n_rve));
  MFG_CUDA(b->d_omega.alloc(9 * n_rve));
  MFG_CUDA(b->d_res.alloc(n_rve));
  MFG_CUDA(b->d_status.alloc(n_rve));
  MFG_CUDA(b->d_steps.alloc(n_rve));
  MFG_CUDA(b->d_st.alloc(n_rve));

  mfg::DevBatch& dv = b->dev;
  dv.n_rve = n_rve;
  dv.nt = nt;
  dv.et = et;
  dv.desc = b->d_desc.p;
  dv.X = b->d_X.p;
  dv.x = b->d_x.p;
  dv.u = b->d_u.p;
  dv.v = b->d_v.p;
  dv.m = b->d_m.p;
  dv.conn = b->d_conn.p;
  dv.l0 = b->d_l0.p;
  dv.nrm = b->d_nrm.p;
  dv.fint = b->d_fint.p;
  dv.rowptr = b->d_rowptr.p;
  dv.inc = b->d_inc.p;
  dv.bnd = b->d_bnd.p;
  dv.ramp = b->d_ramp.p;
  dv.vol = b->d_vol.p;
  dv.cur_stress = b->d_cur.p;
  dv.order = b->d_order.p;
  dv.queue = b->d_queue.p;
  if (b->precision == MFG_PREC_F64) {
    // Load the module that holds the no-allocation solve's scratch array now,
    // so that mfg_batch_run_device_noalloc() never reserves it mid-solve.
    void* scratch = nullptr;
    MFG_CUDA(mfg::relax_f64_static_scratch_address(&scratch));
  }
  if (b->precision == MFG_PREC_MIXED) {
    b->mixed.reset(mfg::mixed_new());
    cudaError_t e =
        b->mixed ? mfg::mixed_create(*b->mixed, dv, b->desc, conn, rowptr, inc, b->sms,
                                     opt.max_cluster_ctas > 0 ? opt.max_cluster_ctas : 8,
                                     opt.cluster_layout == MFG_LAYOUT_SERVING,
                                     opt.small_rve_solve,
                                     opt.small_rves_per_cta > 0 ? opt.small_rves_per_cta : 2, s)
                 : cudaErrorMemoryAllocation;
    if (e != cudaSuccess)
      return fail(e == cudaErrorMemoryAllocation ? MFG_E_OOM : MFG_E_CUDA,
                  "mixed-precision set-up failed: %s", cudaGetErrorString(e));
  }
  MFG_CUDA(cudaStreamSynchronize(s));
  *out = b.release();
  return MFG_OK;
}

mfg_status mfg_batch_destroy(mfg_batch* batch) {
  delete batch;
  return MFG_OK;
}

int32_t mfg_batch_size(const mfg_batch* b) { return b ? b->R : 0; }
int32_t mfg_batch_n_nodes(const mfg_batch* b, int32_t r) {
  return (b && r >= 0 && r < b->R) ? b->n_nodes[r] : -1;
}
int32_t mfg_batch_n_fibers(const mfg_batch* b, int32_t r) {
  return (b && r >= 0 && r < b->R) ? b->n_fibers[r] : -1;
}

static mfg_status batch_run_device_impl(mfg_batch* b, const double* F_dev, int32_t n_F,
                                        double* sigma_dev, int32_t update_coords,
                                        mfg_rve_status* status_dev, void* stream) {
  mfg::Trace trace("mfg_batch_run_device");
  g_last_error.clear();
  if (!b || !F_dev || !sigma_dev) return fail(MFG_E_INVALID, "NULL argument");
  mfg_status st = check_run_args(b, n_F, update_coords);
  if (st != MFG_OK) return st;
  MFG_CUDA(cudaSetDevice(b->device));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : b->stream;
  b->timing_valid = false;
  MFG_CUDA(cudaEventRecord(b->ev_run0, s));
  if ((st = enqueue_run(b, F_dev, n_F, sigma_dev, update_coords, s)) != MFG_OK) return st;
  if (status_dev) {
    cudaError_t e = mfg::launch_pack_status(b->d_status.p, b->d_steps.p, b->d_res.p, b->R,
                                            status_dev, s);
    if (e != cudaSuccess) return fail(MFG_E_CUDA, "status pack failed: %s", cudaGetErrorString(e));
    b->last_launches += 1;
  }
  MFG_CUDA(cudaEventRecord(b->ev_run1, s));
  b->timing_valid = true;
  return MFG_OK;
}

mfg_status mfg_batch_run_device_noalloc(mfg_batch* b, const double* F_dev, int32_t n_F,
                                        double* sigma_dev, int32_t update_coords,
                                        mfg_rve_status* status_dev, void* stream) {
  mfg::Trace trace("mfg_batch_run_device_noalloc");
  g_last_error.clear();
  if (!b || !F_dev || !sigma_dev) return fail(MFG_E_INVALID, "NULL argument");
  if (b->precision != MFG_PREC_F64)
    return fail(MFG_E_INVALID, "the no-allocation solve runs FP64 batches only");
  mfg_status st = check_run_args(b, n_F, update_coords);
  if (st != MFG_OK) return st;
  const size_t need = mfg::relax_f64_static_scratch_bytes(b->dev, b->nbt);
  if (need > MFG_NOALLOC_SCRATCH_BYTES)
    return fail(MFG_E_INVALID, "batch needs %zu bytes of scratch, the fixed array holds %u",
                need, static_cast<unsigned>(MFG_NOALLOC_SCRATCH_BYTES));
  MFG_CUDA(cudaSetDevice(b->device));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : b->stream;
  b->timing_valid = false;
  MFG_CUDA(cudaEventRecord(b->ev_run0, s));
  mfg::RunArgs a{};
  a.F = F_dev;
  a.n_F = n_F;
  a.update_coords = update_coords;
  a.sigma = sigma_dev;
  MFG_CUDA(cudaEventRecord(b->ev_relax0, s));
  const int grid = std::min(b->R, b->sms * mfg::relax_f64_max_blocks_per_sm(0));
  mfg::StaticStatus ss{};
  cudaError_t e = mfg::launch_relax_f64_static(b->dev, a, grid, b->nbt, s, &ss);
  if (e != cudaSuccess)
    return fail(MFG_E_CUDA, "fixed-scratch relaxation launch failed: %s", cudaGetErrorString(e));
  b->last_launches = 1;
  MFG_CUDA(cudaEventRecord(b->ev_relax1, s));
  if (status_dev) {
    e = mfg::launch_pack_status(ss.status, ss.steps, ss.residual, b->R, status_dev, s);
    if (e != cudaSuccess) return fail(MFG_E_CUDA, "status pack failed: %s", cudaGetErrorString(e));
    b->last_launches += 1;
  }
  MFG_CUDA(cudaEventRecord(b->ev_run1, s));
  b->timing_valid = true;
  return MFG_OK;
}

static mfg_status batch_run_impl(mfg_batch* b, const double* F, int32_t n_F, double* sigma,
                                 int32_t update_coords, mfg_rve_status* status) {
  mfg::Trace trace("mfg_batch_run");
  g_last_error.clear();
  if (!b || !F || !sigma) return fail(MFG_E_INVALID, "NULL argument");
  mfg_status st = check_run_args(b, n_F, update_coords);
  if (st != MFG_OK) return st;
  MFG_CUDA(cudaSetDevice(b->device));
  cudaStream_t s = b->stream;
  b->timing_valid = false;
  MFG_CUDA(cudaEventRecord(b->ev_run0, s));
  MFG_CUDA(cudaMemcpyAsync(b->d_F.p, F, 9 * sizeof(double) * n_F, cudaMemcpyHostToDevice, s));
  if ((st = enqueue_run(b, b->d_F.p, n_F, b->d_sigma.p, update_coords, s)) != MFG_OK) return st;
  cudaError_t e = mfg::launch_pack_status(b->d_status.p, b->d_steps.p, b->d_res.p, b->R,
                                          b->d_st.p, s);
  if (e != cudaSuccess) return fail(MFG_E_CUDA, "status pack failed: %s", cudaGetErrorString(e));
  b->last_launches += 1;
  std::vector<mfg_rve_status> hst(b->R);
  MFG_CUDA(cudaMemcpyAsync(sigma, b->d_sigma.p, 6 * sizeof(double) * b->R, cudaMemcpyDeviceToHost, s));
  MFG_CUDA(cudaMemcpyAsync(hst.data(), b->d_st.p, sizeof(mfg_rve_status) * b->R,
                           cudaMemcpyDeviceToHost, s));
  MFG_CUDA(cudaEventRecord(b->ev_run1, s));
  MFG_CUDA(cudaStreamSynchronize(s));
  b->timing_valid = true;
  int worst = MFG_OK;
  for (int r = 0; r < b->R; ++r) {
    if (status) status[r] = hst[r];
    if (hst[r].status > worst) worst = hst[r].status;
  }
  if (worst != MFG_OK)
    fail(static_cast<mfg_status>(worst), "%s in at least one RVE",
         mfg_status_string(static_cast<mfg_status>(worst)));
  return static_cast<mfg_status>(worst);
}

}  // extern "C"

namespace {

// Allocates the concurrent stiffness solves' scratch on first use.
mfg_status stiff_slots_ready(mfg_batch* b) {
  StiffSlots& sl = b->stiff;
  if (sl.ready) return MFG_OK;
  const size_t K = kStiffSlots, nt = b->nt, et = b->et, R = b->R;
  const size_t nbt = std::max<int64_t>(b->nbt, 1);
  cudaError_t e = cudaSuccess;
  for (auto [a, n] : {std::pair{&sl.x, K * 3 * nt}, std::pair{&sl.v, K * 3 * nt},
                      std::pair{&sl.fint, K * 3 * nt}, std::pair{&sl.nrm, K * 3 * et},
                      std::pair{&sl.ramp, K * 6 * nbt}, std::pair{&sl.sigma, K * 6 * R},
                      std::pair{&sl.res, K * R}, std::pair{&sl.F, K * 9}})
    if (e == cudaSuccess) e = a->alloc(n);
  for (auto [a, n] : {std::pair{&sl.status, K * R}, std::pair{&sl.steps, K * R},
                      std::pair{&sl.queue, K}})
    if (e == cudaSuccess) e = a->alloc(n);
  for (size_t k = 0; k < K && e == cudaSuccess; ++k) {
    e = cudaStreamCreateWithFlags(&sl.st[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.join[k], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.fork, cudaEventDisableTiming);
  if (e == cudaSuccess && b->precision == MFG_PREC_MIXED)
    e = mfg::mixed_prepare_contexts(*b->mixed, b->dev, kStiffSlots);
  if (e != cudaSuccess) {
    sl.release();
    return fail(e == cudaErrorMemoryAllocation ? MFG_E_OOM : MFG_E_CUDA,
                "concurrent stiffness scratch: %s", cudaGetErrorString(e));
  }
  sl.ready = true;
  return MFG_OK;
}

// The six perturbed, non-updating solves in flight at once, one slot of
// scratch each, all starting from the state of the last updating run; the
// batch's current coordinates end as the sixth solve leaves them, as after
// the reference's six sequential runs. sigma1 receives 6 x n_rve x 6.
mfg_status stiffness_concurrent(mfg_batch* b, const double Fa[kStiffSlots][9], double* sigma1,
                                mfg_status* worst) {
  mfg_status st = stiff_slots_ready(b);
  if (st != MFG_OK) return st;
  StiffSlots& sl = b->stiff;
  cudaStream_t s = b->stream;
  const int64_t nt = b->nt, et = b->et, R = b->R, nbt = std::max<int64_t>(b->nbt, 1);
  b->timing_valid = false;
  MFG_CUDA(cudaEventRecord(b->ev_run0, s));
  MFG_CUDA(cudaMemcpyAsync(sl.F.p, Fa, sizeof(double) * 9 * kStiffSlots, cudaMemcpyHostToDevice, s));
  for (int k = 0; k < kStiffSlots; ++k)
    MFG_CUDA(cudaMemcpyAsync(sl.x.p + 3 * nt * k, b->d_x.p, 3 * nt * sizeof(double),
                             cudaMemcpyDeviceToDevice, s));
  MFG_CUDA(cudaEventRecord(b->ev_relax0, s));
  MFG_CUDA(cudaEventRecord(sl.fork, s));
  int launches = 0;
  const int grid = std::min(b->R, b->sms * mfg::relax_f64_max_blocks_per_sm(0));
  for (int k = 0; k < kStiffSlots; ++k) {
    cudaStream_t sk = sl.st[k];
    MFG_CUDA(cudaStreamWaitEvent(sk, sl.fork, 0));
    mfg::DevBatch bk = b->dev;
    bk.x = sl.x.p + 3 * nt * k;
    bk.v = sl.v.p + 3 * nt * k;
    bk.fint = sl.fint.p + 3 * nt * k;
    bk.nrm = sl.nrm.p + 3 * et * k;
    bk.ramp = sl.ramp.p + 6 * nbt * k;
    bk.queue = sl.queue.p + k;
    mfg::RunArgs ak{};
    ak.F = sl.F.p + 9 * k;
    ak.n_F = 1;
    ak.update_coords = 0;
    ak.sigma = sl.sigma.p + 6 * R * k;
    ak.st_status = sl.status.p + R * k;
    ak.st_steps = sl.steps.p + R * k;
    ak.st_residual = sl.res.p + R * k;
    cudaError_t e;
    if (b->precision == MFG_PREC_MIXED) {
      int n = 0;
      e = mfg::run_mixed(*b->mixed, bk, ak, sk, &n, k + 1);
      launches += n;
    } else {
      e = cudaMemsetAsync(bk.queue, 0, sizeof(int32_t), sk);
      if (e == cudaSuccess) e = mfg::launch_relax_f64(bk, ak, 0, grid, sk);
      launches += 1;
    }
    if (e != cudaSuccess)
      return fail(MFG_E_CUDA, "stiffness solve %d failed to launch: %s", k, cudaGetErrorString(e));
    MFG_CUDA(cudaEventRecord(sl.join[k], sk));
    MFG_CUDA(cudaStreamWaitEvent(s, sl.join[k], 0));
  }
  MFG_CUDA(cudaEventRecord(b->ev_relax1, s));
  b->last_launches = launches;
  MFG_CUDA(cudaMemcpyAsync(b->d_x.p, sl.x.p + 3 * nt * (kStiffSlots - 1), 3 * nt * sizeof(double),
                           cudaMemcpyDeviceToDevice, s));
  std::vector<int32_t> hst(static_cast<size_t>(kStiffSlots) * R);
  MFG_CUDA(cudaMemcpyAsync(sigma1, sl.sigma.p, sizeof(double) * 6 * R * kStiffSlots,
                           cudaMemcpyDeviceToHost, s));
  MFG_CUDA(cudaMemcpyAsync(hst.data(), sl.status.p, sizeof(int32_t) * R * kStiffSlots,
                           cudaMemcpyDeviceToHost, s));
  MFG_CUDA(cudaEventRecord(b->ev_run1, s));
  MFG_CUDA(cudaStreamSynchronize(s));
  b->timing_valid = true;
  *worst = MFG_OK;
  for (int32_t v : hst)
    if (v > *worst) *worst = static_cast<mfg_status>(v);
  return MFG_OK;
}

}  // namespace

extern "C" {

static mfg_status material_stiffness_impl(mfg_batch* b, double* C) {
  mfg::Trace trace("mfg_batch_material_stiffness");
  g_last_error.clear();
  if (!b || !C) return fail(MFG_E_INVALID, "NULL argument");
  MFG_CUDA(cudaSetDevice(b->device));
  // BatchedFiberRVEAnalysisExplicit.h:321-405
  constexpr double h = kStiffH;
  double Fa[kStiffSlots][9];
  perturbation_gradients(Fa);
  std::vector<double> cur(6 * b->R), sigma1(6 * b->R * static_cast<size_t>(kStiffSlots));
  MFG_CUDA(cudaMemcpy(cur.data(), b->d_cur.p, 6 * sizeof(double) * b->R, cudaMemcpyDeviceToHost));
  mfg_status worst = MFG_OK;
  const bool concurrent = b->stiffness == MFG_STIFFNESS_CONCURRENT ||
                          (b->stiffness == MFG_STIFFNESS_AUTO && b->all_ramp);
  if (concurrent) {
    mfg_status st = stiffness_concurrent(b, Fa, sigma1.data(), &worst);
    if (st != MFG_OK) return st;
  } else {
    for (int i = 0; i < kStiffSlots; ++i) {
      mfg_status st = mfg_batch_run(b, Fa[i], 1, sigma1.data() + 6 * b->R * i, 0, nullptr);
      if (st == MFG_E_INVALID || st == MFG_E_CUDA || st == MFG_E_OOM) return st;
      if (st > worst) worst = st;
    }
  }
  for (int i = 0; i < kStiffSlots; ++i)
    for (int r = 0; r < b->R; ++r)
      for (int j = 0; j < 6; ++j)
        C[36 * r + 6 * j + i] = (sigma1[6 * b->R * i + 6 * r + j] - cur[6 * r + j]) / h;
  if (worst != MFG_OK)
    fail(worst, "%s in at least one perturbed solve", mfg_status_string(worst));
  return worst;
}

mfg_status mfg_batch_orientation_3d(mfg_batch* b, double* omega) {
  return mfg_batch_orientation_2d(b, nullptr, omega);
}

mfg_status mfg_batch_orientation_2d(mfg_batch* b, const double* normal, double* omega) {
  mfg::Trace trace("mfg_batch_orientation");
  g_last_error.clear();
  if (!b || !omega) return fail(MFG_E_INVALID, "NULL argument");
  MFG_CUDA(cudaSetDevice(b->device));
  cudaStream_t s = b->stream;
  const double* nd = nullptr;
  if (normal) {
    MFG_CUDA(cudaMemcpyAsync(b->d_F.p, normal, 3 * sizeof(double) * b->R, cudaMemcpyHostToDevice, s));
    nd = b->d_F.p;
  }
  cudaError_t e = mfg::launch_orientation(b->dev, nd, b->d_omega.p, s);
  if (e != cudaSuccess) return fail(MFG_E_CUDA, "orientation launch failed: %s", cudaGetErrorString(e));
  MFG_CUDA(cudaMemcpyAsync(omega, b->d_omega.p, 9 * sizeof(double) * b->R, cudaMemcpyDeviceToHost, s));
  MFG_CUDA(cudaStreamSynchronize(s));
  return MFG_OK;
}

static mfg_status get_node_field(mfg_batch* b, int32_t rve, const double* field, double* out) {
  if (!b || !out || rve < 0 || rve >= b->R) return fail(MFG_E_INVALID, "bad rve or NULL output");
  MFG_CUDA(cudaSetDevice(b->device));
  const mfg::RveDesc& d = b->desc[rve];
  const int N = d.n_nodes;
  std::vector<double> tmp(3 * static_cast<size_t>(N));
  for (int k = 0; k < 3; ++k)
    MFG_CUDA(cudaMemcpyAsync(&tmp[static_cast<size_t>(k) * N], field + k * b->nt + d.node_off,
                             N * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  MFG_CUDA(cudaStreamSynchronize(b->stream));
  const auto& perm = b->perm[rve];
  for (int i = 0; i < N; ++i)
    for (int k = 0; k < 3; ++k) out[3 * i + k] = tmp[static_cast<size_t>(k) * N + perm[i]];
  return MFG_OK;
}

mfg_status mfg_batch_get_displacements(mfg_batch* b, int32_t rve, double* u) {
  g_last_error.clear();
  return get_node_field(b, rve, b ? b->d_u.p : nullptr, u);
}

mfg_status mfg_batch_get_coordinates(mfg_batch* b, int32_t rve, double* x) {
  g_last_error.clear();
  return get_node_field(b, rve, b ? b->d_x.p : nullptr, x);
}

mfg_status mfg_batch_get_current_stress(mfg_batch* b, double* sigma) {
  g_last_error.clear();
  if (!b || !sigma) return fail(MFG_E_INVALID, "NULL argument");
  MFG_CUDA(cudaSetDevice(b->device));
  MFG_CUDA(cudaMemcpy(sigma, b->d_cur.p, 6 * sizeof(double) * b->R, cudaMemcpyDeviceToHost));
  return MFG_OK;
}

size_t mfg_batch_state_bytes(const mfg_batch* b, int32_t rve) {
  if (!b || rve < 0 || rve >= b->R) return 0;
  return (6 * static_cast<size_t>(b->n_nodes[rve]) + 7) * sizeof(double);
}

mfg_status mfg_batch_export_state(mfg_batch* b, int32_t rve, void* buf, size_t bytes) {
  mfg::Trace trace("mfg_batch_export_state");
  g_last_error.clear();
  if (!b || !buf || rve < 0 || rve >= b->R) return fail(MFG_E_INVALID, "bad rve or NULL buffer");
  if (bytes < mfg_batch_state_bytes(b, rve)) return fail(MFG_E_INVALID, "buffer too small");
  MFG_CUDA(cudaSetDevice(b->device));
  const mfg::RveDesc& d = b->desc[rve];
  const size_t N = d.n_nodes;
  double* o = static_cast<double*>(buf);
  for (int k = 0; k < 3; ++k) {
    MFG_CUDA(cudaMemcpyAsync(o + k * N, b->d_u.p + k * b->nt + d.node_off, N * sizeof(double),
                             cudaMemcpyDeviceToHost, b->stream));
    MFG_CUDA(cudaMemcpyAsync(o + (3 + k) * N, b->d_x.p + k * b->nt + d.node_off, N * sizeof(double),
                             cudaMemcpyDeviceToHost, b->stream));
  }
  MFG_CUDA(cudaMemcpyAsync(o + 6 * N, b->d_vol.p + rve, sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  MFG_CUDA(cudaMemcpyAsync(o + 6 * N + 1, b->d_cur.p + 6 * rve, 6 * sizeof(double),
                           cudaMemcpyDeviceToHost, b->stream));
  MFG_CUDA(cudaStreamSynchronize(b->stream));
  return MFG_OK;
}

mfg_status mfg_batch_import_state(mfg_batch* b, int32_t rve, const void* buf, size_t bytes) {
  mfg::Trace trace("mfg_batch_import_state");
  g_last_error.clear();
  if (!b || !buf || rve < 0 || rve >= b->R) return fail(MFG_E_INVALID, "bad rve or NULL buffer");
  if (bytes < mfg_batch_state_bytes(b, rve)) return fail(MFG_E_INVALID, "buffer too small");
  MFG_CUDA(cudaSetDevice(b->device));
  const mfg::RveDesc& d = b->desc[rve];
  const size_t N = d.n_nodes;
  const double* o = static_cast<const double*>(buf);
  for (size_t k = 0; k < 6 * N + 7; ++k)
    if (!std::isfinite(o[k])) return fail(MFG_E_INVALID, "state holds a non-finite value");
  for (int k = 0; k < 3; ++k) {
    MFG_CUDA(cudaMemcpyAsync(b->d_u.p + k * b->nt + d.node_off, o + k * N, N * sizeof(double),
                             cudaMemcpyHostToDevice, b->stream));
    MFG_CUDA(cudaMemcpyAsync(b->d_x.p + k * b->nt + d.node_off, o + (3 + k) * N, N * sizeof(double),
                             cudaMemcpyHostToDevice, b->stream));
  }
  MFG_CUDA(cudaMemcpyAsync(b->d_vol.p + rve, o + 6 * N, sizeof(double), cudaMemcpyHostToDevice, b->stream));
  MFG_CUDA(cudaMemcpyAsync(b->d_cur.p + 6 * rve, o + 6 * N + 1, 6 * sizeof(double),
                           cudaMemcpyHostToDevice, b->stream));
  MFG_CUDA(cudaStreamSynchronize(b->stream));
  return MFG_OK;
}

mfg_status mfg_batch_last_timing(mfg_batch* b, float* relax_ms, float* run_ms) {
  g_last_error.clear();
  if (!b) return fail(MFG_E_INVALID, "NULL batch");
  if (!b->timing_valid) return fail(MFG_E_INVALID, "no completed run to time");
  MFG_CUDA(cudaSetDevice(b->device));
  MFG_CUDA(cudaEventSynchronize(b->ev_run1));
  if (relax_ms) MFG_CUDA(cudaEventElapsedTime(relax_ms, b->ev_relax0, b->ev_relax1));
  if (run_ms) MFG_CUDA(cudaEventElapsedTime(run_ms, b->ev_run0, b->ev_run1));
  return MFG_OK;
}

int32_t mfg_batch_last_launches(const mfg_batch* b) { return b ? b->last_launches : 0; }

}  // extern "C"

// ============================================================================
// Serving: continuous batching over a persistent kernel.
// ============================================================================
#include <chrono>
#include <deque>

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct PendingReq {
  int64_t ticket;
  int32_t flags;  // mfg::kReqUpdate | mfg::kReqStiffness
  double F[9];
  double t_submit;
};

// Device footprint of a batch's state (FP64 arrays, CSR, and the mixed
// working set when used), for admission against the HBM budget.
double batch_bytes(int64_t nt, int64_t et, int64_t nbt, int64_t R, bool mixed) {
  double b = nt * (5 * 3 * 8.0 + 8 + 4) + et * (8.0 + 8 + 24 + 8) + nbt * (48.0 + 4) + R * 200.0;
  if (mixed)  // + node-centric incidences (about 2.3 per fiber, with the set-up fiber ids)
    b += nt * (24.0 + 12 + 8 + 4 + 4 + 8 + 8) + et * (16.0 + 16 + 16 + 8 + 8 + 4 + 64) + R * 20.0;
  return b;
}

}  // namespace

// One request ring of a server: requests in host-mapped memory, the
// published count in device memory, completion records in host-mapped
// memory, and the host's bookkeeping per ring slot.
struct ServerLane {
  mfg::ServerReq* ring_h = nullptr;
  long long* tail_stage = nullptr;  // pinned, one published count per ring slot
  long long* tail_d = nullptr;
  mfg::ServerDone* done_h = nullptr;
  unsigned long long* head_d = nullptr;
  mfg::ServerArgs args{};
  int64_t tail = 0;    // ring entries published
  int64_t oldest = 0;  // oldest ring entry not yet returned
  std::vector<int64_t> slot_ticket;
  std::vector<double> slot_submit;
  std::vector<uint8_t> slot_returned;

  void release() {
    if (ring_h) cudaFreeHost(ring_h);
    if (tail_stage) cudaFreeHost(tail_stage);
    if (done_h) cudaFreeHost(done_h);
    if (tail_d) cudaFree(tail_d);
    if (head_d) cudaFree(head_d);
    ring_h = nullptr;
    tail_stage = nullptr;
    done_h = nullptr;
    tail_d = nullptr;
    head_d = nullptr;
  }
};

struct mfg_server {
  mfg_batch* batch = nullptr;
  cudaStream_t stream = nullptr;   // the persistent kernel
  cudaStream_t ctrl = nullptr;     // small copies of the published counts and stop flag
  int64_t cap = 0;
  unsigned long long idle_ns = 0;
  unsigned long long max_wait_ns = 0;
  // lane 0 serves RVEs solved by one CTA; lane 1, when present, the RVEs the
  // mixed serving kernel solves with 4-CTA clusters
  std::vector<ServerLane> lanes;
  std::vector<uint8_t> lane_of;     // per RVE
  int32_t* stop_stage = nullptr;    // pinned
  int32_t* stop_d = nullptr;
  unsigned long long* last_d = nullptr;
  int* ctl_d = nullptr;  // [0] idle CTAs (or clusters), [1] closing
  DevArray<double> sigma, res;
  DevArray<int32_t> st, steps;
  // stiffness of a request: perturbation gradients, perturbed-solve scratch, result
  DevArray<double> stiff_F, sigma1, res1, C;
  DevArray<int32_t> st1, steps1, stiff_status;
  int64_t next_ticket = 0;
  int64_t launches = 0;
  std::vector<uint8_t> busy;
  std::vector<std::deque<PendingReq>> held;
  int64_t n_held = 0;
  bool launched = false;

  int64_t in_flight() const {
    int64_t n = n_held;
    for (const ServerLane& l : lanes) n += l.tail - l.oldest;
    return n;
  }

  ~mfg_server() {
    if (batch) cudaSetDevice(batch->device);
    if (stop_d && stop_stage && ctrl) {
      *stop_stage = 1;
      cudaMemcpyAsync(stop_d, stop_stage, sizeof(int32_t), cudaMemcpyHostToDevice, ctrl);
      cudaStreamSynchronize(ctrl);
    }
    if (stream) {
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
    }
    if (ctrl) cudaStreamDestroy(ctrl);
    for (ServerLane& l : lanes) l.release();
    if (stop_stage) cudaFreeHost(stop_stage);
    if (stop_d) cudaFree(stop_d);
    if (last_d) cudaFree(last_d);
    if (ctl_d) cudaFree(ctl_d);
    for (auto* a : {&sigma, &res, &stiff_F, &sigma1, &res1, &C}) a->release();
    for (auto* a : {&st, &steps, &st1, &steps1, &stiff_status}) a->release();
    mfg_batch_destroy(batch);
  }
};

namespace {

mfg_status server_ensure_running(mfg_server* sv) {
  if (sv->launched) {
    cudaError_t q = cudaStreamQuery(sv->stream);
    if (q == cudaErrorNotReady) return MFG_OK;
    if (q != cudaSuccess)
      return fail(MFG_E_CUDA, "serving kernel failed: %s", cudaGetErrorString(q));
  }
  // a fresh kernel starts with no CTA waiting and the closing flag down
  MFG_CUDA(cudaMemsetAsync(sv->ctl_d, 0, 2 * sizeof(int), sv->stream));
  const mfg::ServerArgs* big = sv->lanes.size() > 1 ? &sv->lanes[1].args : nullptr;
  cudaError_t e = sv->batch->precision == MFG_PREC_MIXED
                      ? mfg::launch_server_mixed(*sv->batch->mixed, sv->batch->dev,
                                                 sv->lanes[0].args, big, sv->stream)
                      : mfg::launch_server_f64(sv->batch->dev, sv->lanes[0].args,
                                               sv->batch->sms * mfg::relax_f64_max_blocks_per_sm(0),
                                               sv->stream);
  if (e != cudaSuccess) return fail(MFG_E_CUDA, "serving launch failed: %s", cudaGetErrorString(e));
  sv->launched = true;
  sv->launches++;
  return MFG_OK;
}

// Writes one request into its RVE's ring and publishes it: the entry is
// stored first, then the new published count is copied into device memory
// on the control stream, where the kernel polls it.
mfg_status server_publish(mfg_server* sv, int32_t rve, const PendingReq& p) {
  ServerLane& l = sv->lanes[sv->lane_of[rve]];
  const int64_t idx = l.tail;
  mfg::ServerReq& q = l.ring_h[idx % sv->cap];
  q.rve = rve;
  q.flags = p.flags;
  q.ticket = p.ticket;
  for (int k = 0; k < 9; ++k) q.F[k] = p.F[k];
  l.slot_ticket[idx % sv->cap] = p.ticket;
  l.slot_submit[idx % sv->cap] = p.t_submit;
  l.slot_returned[idx % sv->cap] = 0;
  std::atomic_thread_fence(std::memory_order_seq_cst);
  l.tail = idx + 1;
  l.tail_stage[idx % sv->cap] = l.tail;
  sv->busy[rve] = 1;
  MFG_CUDA(cudaMemcpyAsync(l.tail_d, &l.tail_stage[idx % sv->cap], sizeof(long long),
                           cudaMemcpyHostToDevice, sv->ctrl));
  return MFG_OK;
}

mfg_status server_lane_create(mfg_server* sv, ServerLane& l) {
  MFG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&l.ring_h), sv->cap * sizeof(mfg::ServerReq),
                         cudaHostAllocMapped));
  MFG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&l.done_h), sv->cap * sizeof(mfg::ServerDone),
                         cudaHostAllocMapped));
  MFG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&l.tail_stage), sv->cap * sizeof(long long),
                         cudaHostAllocDefault));
  MFG_CUDA(cudaMalloc(reinterpret_cast<void**>(&l.tail_d), sizeof(long long)));
  MFG_CUDA(cudaMemset(l.tail_d, 0, sizeof(long long)));
  std::memset(l.done_h, 0, sv->cap * sizeof(mfg::ServerDone));
  MFG_CUDA(cudaMalloc(reinterpret_cast<void**>(&l.head_d), sizeof(unsigned long long)));
  MFG_CUDA(cudaMemset(l.head_d, 0, sizeof(unsigned long long)));
  mfg::ServerArgs& a = l.args;
  MFG_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(const_cast<mfg::ServerReq**>(&a.ring)),
                                    l.ring_h, 0));
  a.tail = l.tail_d;
  a.stop = sv->stop_d;
  MFG_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&a.done), l.done_h, 0));
  a.head = l.head_d;
  a.last_claim = sv->last_d;
  a.idle_ctas = sv->ctl_d;
  a.closing = sv->ctl_d + 1;
  a.cap = sv->cap;
  a.idle_ns = sv->idle_ns;
  a.max_wait_ns = sv->max_wait_ns;
  a.sigma = sv->sigma.p;
  a.st_status = sv->st.p;
  a.st_steps = sv->steps.p;
  a.st_residual = sv->res.p;
  a.stiff_F = sv->stiff_F.p;
  a.cur_stress = sv->batch->d_cur.p;
  a.sigma1 = sv->sigma1.p;
  a.st1_status = sv->st1.p;
  a.st1_steps = sv->steps1.p;
  a.st1_residual = sv->res1.p;
  a.C = sv->C.p;
  a.stiff_status = sv->stiff_status.p;
  l.slot_ticket.assign(sv->cap, -1);
  l.slot_submit.assign(sv->cap, 0.0);
  l.slot_returned.assign(sv->cap, 1);
  return MFG_OK;
}

}  // namespace

extern "C" {

void mfg_default_server_options(mfg_server_options* out) {
  if (!out) return;
  std::memset(out, 0, sizeof(*out));
  out->precision = MFG_PREC_MIXED;
}

mfg_status mfg_server_create(const mfg_network* nets, const mfg_strategy* strategies,
                             int32_t n_rve, const mfg_server_options* options, mfg_server** out) {
  mfg::Trace trace("mfg_server_create");
  g_last_error.clear();
  if (!out) return fail(MFG_E_INVALID, "out is NULL");
  *out = nullptr;
  mfg_server_options opt;
  mfg_default_server_options(&opt);
  if (options) opt = *options;
  if (opt.capacity < 0 || opt.idle_timeout_us < 0 || !(opt.hbm_budget_bytes >= 0) ||
      opt.max_wait_ms < 0)
    return fail(MFG_E_INVALID, "negative server option");
  mfg_options bo;
  mfg_default_options(&bo);
  bo.precision = opt.precision;
  bo.device = opt.device;
  bo.cluster_layout = MFG_LAYOUT_SERVING;
  // admission: the device state of every registered RVE must fit the budget
  if (nets && n_rve > 0) {
    int64_t nt = 0, et = 0;
    for (int r = 0; r < n_rve; ++r) {
      nt += std::max(nets[r].n_nodes, 0);
      et += std::max(nets[r].n_fibers, 0);
    }
    const double need = batch_bytes(nt, et, nt / 8, n_rve, opt.precision == MFG_PREC_MIXED);
    double budget = opt.hbm_budget_bytes;
    if (budget <= 0) {
      size_t fr = 0, tot = 0;
      if (cudaSetDevice(opt.device) == cudaSuccess && cudaMemGetInfo(&fr, &tot) == cudaSuccess)
        budget = 0.9 * static_cast<double>(fr);
    }
    if (budget > 0 && need > budget)
      return fail(MFG_E_BUSY, "admission refused: %.3g bytes of RVE state exceed the %.3g-byte "
                  "HBM budget", need, budget);
  }
  mfg_batch* b = nullptr;
  mfg_status st = mfg_batch_create(nets, strategies, n_rve, &bo, &b);
  if (st != MFG_OK) return st;
  std::unique_ptr<mfg_server> sv(new mfg_server());
  sv->batch = b;
  sv->cap = opt.capacity > 0 ? opt.capacity : 65536;
  sv->idle_ns = 1000ULL * static_cast<unsigned long long>(opt.idle_timeout_us > 0 ? opt.idle_timeout_us
                                                                                   : 20000);
  sv->max_wait_ns =
      1000000ULL * static_cast<unsigned long long>(opt.max_wait_ms > 0 ? opt.max_wait_ms : 5000);
  MFG_CUDA(cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking));
  MFG_CUDA(cudaStreamCreateWithFlags(&sv->ctrl, cudaStreamNonBlocking));
  MFG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&sv->stop_stage), 64, cudaHostAllocDefault));
  MFG_CUDA(cudaMalloc(reinterpret_cast<void**>(&sv->stop_d), sizeof(int32_t)));
  MFG_CUDA(cudaMemset(sv->stop_d, 0, sizeof(int32_t)));
  *sv->stop_stage = 0;
  MFG_CUDA(cudaMalloc(reinterpret_cast<void**>(&sv->last_d), sizeof(unsigned long long)));
  MFG_CUDA(cudaMemset(sv->last_d, 0, sizeof(unsigned long long)));
  MFG_CUDA(cudaMalloc(reinterpret_cast<void**>(&sv->ctl_d), 2 * sizeof(int)));
  MFG_CUDA(cudaMemset(sv->ctl_d, 0, 2 * sizeof(int)));
  MFG_CUDA(sv->sigma.alloc(6 * static_cast<size_t>(n_rve)));
  MFG_CUDA(sv->res.alloc(n_rve));
  MFG_CUDA(sv->st.alloc(n_rve));
  MFG_CUDA(sv->steps.alloc(n_rve));
  {
    double Fa[kStiffSlots][9];
    perturbation_gradients(Fa);
    MFG_CUDA(sv->stiff_F.alloc(9 * kStiffSlots));
    MFG_CUDA(cudaMemcpy(sv->stiff_F.p, Fa, sizeof(Fa), cudaMemcpyHostToDevice));
  }
  MFG_CUDA(sv->sigma1.alloc(6 * static_cast<size_t>(n_rve)));
  MFG_CUDA(sv->res1.alloc(n_rve));
  MFG_CUDA(sv->C.alloc(36 * static_cast<size_t>(n_rve)));
  MFG_CUDA(sv->st1.alloc(n_rve));
  MFG_CUDA(sv->steps1.alloc(n_rve));
  MFG_CUDA(sv->stiff_status.alloc(n_rve));
  // RVEs the mixed serving kernel solves with clusters get their own ring
  sv->lane_of.assign(n_rve, 0);
  bool clusters = false;
  if (b->precision == MFG_PREC_MIXED)
    for (int r = 0; r < n_rve; ++r)
      if (mfg::mixed_serves_in_clusters(*b->mixed, r)) {
        sv->lane_of[r] = 1;
        clusters = true;
      }
  sv->lanes.resize(clusters ? 2 : 1);
  for (ServerLane& l : sv->lanes)
    if ((st = server_lane_create(sv.get(), l)) != MFG_OK) return st;
  sv->busy.assign(n_rve, 0);
  sv->held.resize(n_rve);
  MFG_CUDA(cudaDeviceSynchronize());
  *out = sv.release();
  return MFG_OK;
}

double mfg_device_bytes_estimate(const mfg_network* nets, int32_t n_rve, int32_t precision) {
  if (!nets || n_rve < 1) return 0.0;
  int64_t nt = 0, et = 0;
  for (int r = 0; r < n_rve; ++r) {
    nt += std::max(nets[r].n_nodes, 0);
    et += std::max(nets[r].n_fibers, 0);
  }
  return batch_bytes(nt, et, nt / 8, n_rve, precision == MFG_PREC_MIXED);
}

mfg_status mfg_server_submit(mfg_server* sv, int32_t rve, const double* F, int32_t update_coords,
                             int64_t* ticket) {
  return mfg_server_submit_ex(sv, rve, F, update_coords, 0, ticket);
}

mfg_status mfg_server_submit_ex(mfg_server* sv, int32_t rve, const double* F,
                                int32_t update_coords, int32_t stiffness, int64_t* ticket) {
  g_last_error.clear();
  if (!sv || !F) return fail(MFG_E_INVALID, "NULL argument");
  if (rve < 0 || rve >= sv->batch->R) return fail(MFG_E_INVALID, "rve %d out of range", rve);
  for (int k = 0; k < 9; ++k)
    if (!std::isfinite(F[k])) return fail(MFG_E_INVALID, "non-finite deformation gradient");
  if (sv->in_flight() >= sv->cap)
    return fail(MFG_E_BUSY, "request ring full (%lld entries)", static_cast<long long>(sv->cap));
  MFG_CUDA(cudaSetDevice(sv->batch->device));
  PendingReq p;
  p.ticket = sv->next_ticket++;
  p.flags = (update_coords ? mfg::kReqUpdate : 0) | (stiffness ? mfg::kReqStiffness : 0);
  for (int k = 0; k < 9; ++k) p.F[k] = F[k];
  p.t_submit = now_s();
  if (ticket) *ticket = p.ticket;
  if (sv->busy[rve]) {
    sv->held[rve].push_back(p);
    sv->n_held++;
    return MFG_OK;
  }
  mfg_status st = server_publish(sv, rve, p);
  if (st != MFG_OK) return st;
  return server_ensure_running(sv);
}

static mfg_status server_poll_impl(mfg_server* sv, mfg_server_result* out, int32_t capacity,
                                   int32_t* n_out, int32_t timeout_ms) {
  g_last_error.clear();
  if (!sv || !n_out || (capacity > 0 && !out)) return fail(MFG_E_INVALID, "NULL argument");
  *n_out = 0;
  MFG_CUDA(cudaSetDevice(sv->batch->device));
  const double t_end = now_s() + 1e-3 * std::max(timeout_ms, 0);
  for (;;) {
    int32_t n = 0;
    for (ServerLane& l : sv->lanes) {
      for (int64_t idx = l.oldest; idx < l.tail && n < capacity; ++idx) {
        const int64_t slot = idx % sv->cap;
        if (l.slot_returned[slot]) continue;
        const mfg::ServerDone& d = l.done_h[slot];
        const long long flag = *reinterpret_cast<const volatile long long*>(&d.ticket_plus1);
        if (flag != idx + 1) continue;
        std::atomic_thread_fence(std::memory_order_acquire);
        mfg_server_result& r = out[n++];
        r.ticket = l.slot_ticket[slot];
        r.rve = d.rve;
        r.status = d.status;
        r.steps = d.steps;
        r.stiffness_status = d.stiff_status;
        r.residual = d.residual;
        for (int k = 0; k < 6; ++k) r.sigma[k] = d.sigma[k];
        for (int k = 0; k < 36; ++k) r.C[k] = d.stiff_status >= 0 ? d.C[k] : 0.0;
        r.latency_s = now_s() - l.slot_submit[slot];
        r.device_s = 1e-9 * static_cast<double>(d.t_done_ns - d.t_claim_ns);
        r.t_claim_ns = d.t_claim_ns;
        r.t_done_ns = d.t_done_ns;
        l.slot_returned[slot] = 1;
        sv->busy[d.rve] = 0;
        if (!sv->held[d.rve].empty()) {
          PendingReq p = sv->held[d.rve].front();
          sv->held[d.rve].pop_front();
          sv->n_held--;
          mfg_status st = server_publish(sv, d.rve, p);
          if (st != MFG_OK) return st;
        }
      }
      while (l.oldest < l.tail && l.slot_returned[l.oldest % sv->cap]) l.oldest++;
    }
    const bool outstanding = sv->in_flight() > 0;
    if (outstanding) {
      mfg_status st = server_ensure_running(sv);
      if (st != MFG_OK) return st;
    }
    if (n > 0) {
      *n_out = n;
      return MFG_OK;
    }
    if (!outstanding) return MFG_OK;
    if (now_s() >= t_end)
      return fail(MFG_E_TIMEOUT, "no request completed within %d ms", timeout_ms);
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

int64_t mfg_server_outstanding(const mfg_server* sv) { return sv ? sv->in_flight() : 0; }

int64_t mfg_server_launches(const mfg_server* sv) { return sv ? sv->launches : 0; }

mfg_batch* mfg_server_batch(mfg_server* sv) { return sv ? sv->batch : nullptr; }

mfg_status mfg_server_destroy(mfg_server* sv) {
  mfg::Trace trace("mfg_server_destroy");
  delete sv;
  return MFG_OK;
}

}  // extern "C"

// ============================================================================
// Metrics records (mfg_metrics.cpp): one JSON line per outermost call.
// ============================================================================
namespace {

thread_local int g_metrics_depth = 0;

struct MetricsScope {
  bool top;
  MetricsScope() : top(g_metrics_depth++ == 0) {}
  ~MetricsScope() { --g_metrics_depth; }
  bool log() const { return top && mfg::metrics_enabled(); }
};

const char* precision_name(int p) { return p == MFG_PREC_MIXED ? "mixed" : "f64"; }

std::string status_fields(const char* call, mfg_status st) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), "\"call\": \"%s\", \"status\": \"%s\"", call,
                mfg_status_string(st));
  std::string o = buf;
  if (st != MFG_OK && !g_last_error.empty())
    o += ", \"message\": \"" + mfg::json_escape(g_last_error.c_str()) + "\"";
  return o;
}

// Device times of the last run from the batch's events (completed runs only).
void event_times(mfg_batch* b, float* relax_ms, float* run_ms) {
  *relax_ms = -1.f;
  *run_ms = -1.f;
  if (!b || !b->timing_valid) return;
  if (cudaEventSynchronize(b->ev_run1) != cudaSuccess) return;
  if (cudaEventElapsedTime(relax_ms, b->ev_relax0, b->ev_relax1) != cudaSuccess) *relax_ms = -1.f;
  if (cudaEventElapsedTime(run_ms, b->ev_run0, b->ev_run1) != cudaSuccess) *run_ms = -1.f;
}

}  // namespace

extern "C" {

mfg_status mfg_batch_create(const mfg_network* nets, const mfg_strategy* strategies,
                            int32_t n_rve, const mfg_options* options, mfg_batch** out) {
  MetricsScope ms;
  const double t0 = mfg::wall_seconds();
  const mfg_status st = batch_create_impl(nets, strategies, n_rve, options, out);
  if (ms.log()) {
    std::string f = status_fields("mfg_batch_create", st);
    char buf[256];
    std::snprintf(buf, sizeof(buf), ", \"n_rve\": %d, \"precision\": \"%s\", \"setup_ms\": %.3f",
                  n_rve, precision_name(options ? options->precision : MFG_PREC_F64),
                  1e3 * (mfg::wall_seconds() - t0));
    f += buf;
    if (st == MFG_OK && out && *out) {
      std::snprintf(buf, sizeof(buf), ", \"nodes\": %lld, \"fibers\": %lld, \"device\": %d",
                    static_cast<long long>((*out)->nt), static_cast<long long>((*out)->et),
                    (*out)->device);
      f += buf;
    }
    mfg::metrics_write(f);
  }
  return st;
}

mfg_status mfg_batch_run(mfg_batch* b, const double* F, int32_t n_F, double* sigma,
                         int32_t update_coords, mfg_rve_status* status) {
  MetricsScope ms;
  if (!ms.log()) return batch_run_impl(b, F, n_F, sigma, update_coords, status);
  const double t0 = mfg::wall_seconds();
  std::vector<mfg_rve_status> tmp;
  mfg_rve_status* st_out = status;
  if (!st_out && b && b->R > 0) {
    tmp.resize(b->R);
    st_out = tmp.data();
  }
  const mfg_status st = batch_run_impl(b, F, n_F, sigma, update_coords, st_out);
  const double wall_ms = 1e3 * (mfg::wall_seconds() - t0);
  std::string f = status_fields("mfg_batch_run", st);
  char buf[512];
  if (b && st_out && st != MFG_E_INVALID && st != MFG_E_CUDA && st != MFG_E_OOM) {
    int counts[9] = {};
    long long smin = -1, smax = 0;
    double ssum = 0, rmax = 0, fs = 0;
    for (int r = 0; r < b->R; ++r) {
      const mfg_rve_status& x = st_out[r];
      if (x.status >= 0 && x.status < 9) counts[x.status]++;
      smin = smin < 0 ? x.steps : std::min<long long>(smin, x.steps);
      smax = std::max<long long>(smax, x.steps);
      ssum += x.steps;
      if (std::isfinite(x.residual)) rmax = std::max(rmax, x.residual);
      fs += static_cast<double>(b->n_fibers[r]) * x.steps;
    }
    float relax_ms, run_ms;
    event_times(b, &relax_ms, &run_ms);
    std::snprintf(buf, sizeof(buf),
                  ", \"n_rve\": %d, \"precision\": \"%s\", \"update_coords\": %d, \"n_F\": %d, "
                  "\"ok\": %d, \"not_converged\": %d, \"nonfinite\": %d, \"steps_min\": %lld, "
                  "\"steps_max\": %lld, \"steps_mean\": %.1f, \"residual_max\": %.6e, "
                  "\"fiber_steps\": %.6e, \"relax_ms\": %.3f, \"run_ms\": %.3f, "
                  "\"wall_ms\": %.3f, \"launches\": %d",
                  b->R, precision_name(b->precision), update_coords ? 1 : 0, n_F, counts[MFG_OK],
                  counts[MFG_E_NOT_CONVERGED], counts[MFG_E_NONFINITE], smin, smax,
                  ssum / std::max(1, b->R), rmax, fs, relax_ms, run_ms, wall_ms, b->last_launches);
    f += buf;
  }
  mfg::metrics_write(f);
  return st;
}

mfg_status mfg_batch_run_device(mfg_batch* b, const double* F_dev, int32_t n_F, double* sigma_dev,
                                int32_t update_coords, mfg_rve_status* status_dev, void* stream) {
  MetricsScope ms;
  const mfg_status st =
      batch_run_device_impl(b, F_dev, n_F, sigma_dev, update_coords, status_dev, stream);
  if (ms.log()) {
    // enqueued, not completed: no per-RVE figures (they are on the device)
    std::string f = status_fields("mfg_batch_run_device", st);
    char buf[160];
    std::snprintf(buf, sizeof(buf), ", \"n_rve\": %d, \"update_coords\": %d, \"launches\": %d",
                  b ? b->R : 0, update_coords ? 1 : 0, b ? b->last_launches : 0);
    f += buf;
    mfg::metrics_write(f);
  }
  return st;
}

mfg_status mfg_batch_material_stiffness(mfg_batch* b, double* C) {
  MetricsScope ms;
  const double t0 = mfg::wall_seconds();
  const mfg_status st = material_stiffness_impl(b, C);
  if (ms.log()) {
    std::string f = status_fields("mfg_batch_material_stiffness", st);
    if (b) {
      const bool conc = b->stiffness == MFG_STIFFNESS_CONCURRENT ||
                        (b->stiffness == MFG_STIFFNESS_AUTO && b->all_ramp);
      char buf[200];
      std::snprintf(buf, sizeof(buf),
                    ", \"n_rve\": %d, \"precision\": \"%s\", \"solves\": \"%s\", \"wall_ms\": %.3f",
                    b->R, precision_name(b->precision), conc ? "concurrent" : "sequential",
                    1e3 * (mfg::wall_seconds() - t0));
      f += buf;
    }
    mfg::metrics_write(f);
  }
  return st;
}

mfg_status mfg_server_poll(mfg_server* sv, mfg_server_result* out, int32_t capacity,
                           int32_t* n_out, int32_t timeout_ms) {
  MetricsScope ms;
  const mfg_status st = server_poll_impl(sv, out, capacity, n_out, timeout_ms);
  const int n = n_out ? *n_out : 0;
  if (ms.log() && (n > 0 || st != MFG_OK)) {
    std::string f = status_fields("mfg_server_poll", st);
    double lmax = 0, lsum = 0, dmax = 0;
    int bad = 0;
    for (int i = 0; i < n; ++i) {
      lmax = std::max(lmax, out[i].latency_s);
      lsum += out[i].latency_s;
      dmax = std::max(dmax, out[i].device_s);
      bad += out[i].status != MFG_OK;
    }
    char buf[256];
    std::snprintf(buf, sizeof(buf),
                  ", \"results\": %d, \"not_ok\": %d, \"latency_ms_mean\": %.3f, "
                  "\"latency_ms_max\": %.3f, \"device_ms_max\": %.3f, \"outstanding\": %lld",
                  n, bad, n ? 1e3 * lsum / n : 0.0, 1e3 * lmax, 1e3 * dmax,
                  static_cast<long long>(sv ? sv->in_flight() : 0));
    f += buf;
    mfg::metrics_write(f);
  }
  return st;
}

}  // extern "C"
