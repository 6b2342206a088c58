// Internal layout shared by the host library and the CUDA kernels.
//
// A batch is packed like the reference's PackedData (PackedData.h:78-175):
// every per-node array holds all RVEs back to back, and each quantity with
// three components is stored as three contiguous component blocks of
// `n_nodes_total` entries (structure of arrays), so a warp reading 32
// consecutive nodes of one component issues one coalesced transaction.
// Node ids inside an RVE are boundary-last: free nodes [0, n_free), boundary
// nodes [n_free, n_nodes); each segment is sorted along a Morton curve of the
// reference coordinates for locality. `bnd` lists the boundary nodes in the
// reference's boundary order, which the stress sum follows.
#ifndef MFG_INTERNAL_H
#define MFG_INTERNAL_H

#include <cstdint>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

namespace mfg {

// A named NVTX range for the duration of a scope: the phases of each call
// as a profiler shows them (Nsight Systems, ncu --nvtx), the counterpart of
// the reference's Kokkos kernel labels for Kokkos Tools. Without a tool
// attached a push or pop is a branch.
struct Trace {
  explicit Trace(const char* name) { nvtxRangePushA(name); }
  ~Trace() { nvtxRangePop(); }
  Trace(const Trace&) = delete;
  Trace& operator=(const Trace&) = delete;
};

constexpr int kUpdateFreq = 100;  // dt and residual refresh period (TeamOuterLoop.h:4)

struct RveDesc {
  int64_t node_off;   // first node in the packed node arrays
  int64_t fiber_off;  // first fiber in the packed fiber arrays
  int64_t inc_off;    // first entry in the packed CSR incidence array
  int64_t row_off;    // first entry in the packed CSR row pointer array
  int64_t bnd_off;    // first boundary node in the packed boundary scratch
  int32_t n_nodes, n_free, n_fibers, law;
  int32_t max_steps, mode, pad0, pad1;
  double E, A, B, lt;  // reaction 0: modulus, area, nonlinear B and transition ratio
  double c, crit, tol; // strategy
  double sound_speed;  // sqrt(E / rho)
  double scale;        // stress scale factor
};

// Device pointers of one batch, FP64 state.
struct DevBatch {
  int32_t n_rve;
  int64_t nt;  // total nodes
  int64_t et;  // total fibers
  const RveDesc* desc;
  const double* X;   // 3 * nt reference coordinates
  double* x;         // 3 * nt current coordinates
  double* u;         // 3 * nt displacement
  double* v;         // 3 * nt velocity
  const double* m;   // nt lumped mass
  const int2* conn;  // et fiber end nodes (RVE-local ids)
  const double* l0;  // et reference lengths
  double* nrm;       // 3 * et per-fiber force vectors (scratch)
  double* fint;      // 3 * nt internal force (boundary rows used by the stress)
  const int32_t* rowptr;  // per RVE n_nodes + 1 offsets into that RVE's incidences
  const int32_t* inc;     // 2 * et incidences: (local fiber slot << 1) | end
  const int32_t* bnd;     // total boundary nodes: local ids in the reference's boundary order
  double* ramp;      // 6 * total boundary nodes: RAMP start and increment
  double* vol;       // n_rve current volume
  double* cur_stress;  // n_rve * 6 stress of the last updating run
  const int32_t* order;  // n_rve RVE ids, most work first
  int32_t* queue;        // work counter for the persistent launch
};

struct RunArgs {
  const double* F;  // device, n_F * 9
  int32_t n_F;
  int32_t update_coords;
  double* sigma;        // device, n_rve * 6
  int32_t* st_status;   // device, n_rve
  int32_t* st_steps;    // device, n_rve
  double* st_residual;  // device, n_rve
};

// Serving: request ring and completion records in host-mapped memory.
constexpr int kReqUpdate = 1;     // ServerReq.flags: update the RVE's state
constexpr int kReqStiffness = 2;  // ServerReq.flags: also return the material stiffness
constexpr double kStiffStep = 1E-5;  // FD step of the stiffness (BatchedFiberRVEAnalysisExplicit.h:334)
struct ServerReq {
  int rve;
  int flags;  // kReqUpdate | kReqStiffness
  long long ticket;
  double F[9];
  double pad[1];
};
struct ServerDone {
  long long ticket_plus1;  // written last: ticket + 1 once the record is valid
  int rve, status, steps;
  int stiff_status;  // worst status of the six perturbed solves; -1: no stiffness requested
  double residual;
  double sigma[6];
  long long t_claim_ns, t_done_ns;  // device %globaltimer
  double C[36];  // material stiffness C[6 j + i], when requested
};
struct ServerArgs {
  const ServerReq* ring;            // host-mapped, cap entries
  const volatile long long* tail;   // device: requests published so far (copied in by the host)
  const volatile int32_t* stop;     // device: set by the host to end the kernel
  unsigned long long* head;         // device, requests claimed so far
  unsigned long long* last_claim;   // device, %globaltimer of the latest claim by any CTA
  int* idle_ctas;                   // device, CTAs currently waiting for work
  int* closing;                     // device, set once the kernel is shutting down
  ServerDone* done;                 // host-mapped, cap entries
  long long cap;
  unsigned long long idle_ns;
  unsigned long long max_wait_ns;   // longest a CTA waits for work before it leaves
  double* sigma;                    // device per-RVE scratch, n_rve * 6
  int32_t* st_status;
  int32_t* st_steps;
  double* st_residual;
  // material stiffness of a request (kReqStiffness): the six perturbation
  // gradients, per-RVE scratch of the perturbed solves and the result
  const double* stiff_F;            // device, 6 x 9
  const double* cur_stress;         // the batch's stress of the last updating run, n_rve * 6
  double* sigma1;                   // n_rve * 6
  int32_t* st1_status;              // n_rve
  int32_t* st1_steps;
  double* st1_residual;
  double* C;                        // n_rve * 36
  int32_t* stiff_status;            // n_rve
};
cudaError_t launch_server_f64(const DevBatch& b, const ServerArgs& sa, int grid, cudaStream_t s);

// Launchers (mfg_relax_f64.cu). Return cudaGetLastError() of the launch.
cudaError_t launch_relax_f64(const DevBatch& b, const RunArgs& a, int threads, int grid,
                             cudaStream_t s);
int relax_f64_max_blocks_per_sm(int threads);

// Fixed-scratch variant of the FP64 launch (mfg_relax_f64.cu): scratch comes
// from a file-scope device array of MFG_NOALLOC_SCRATCH_BYTES bytes; no
// allocation. Returns cudaErrorInvalidValue when the batch needs more scratch.
struct StaticStatus {
  int32_t* status;
  int32_t* steps;
  double* residual;
};
size_t relax_f64_static_scratch_bytes(const DevBatch& b, int64_t n_boundary_total);
// Device address of that array on the current device; the first lookup on a
// device loads the module that holds it (and so reserves it).
cudaError_t relax_f64_static_scratch_address(void** addr);
cudaError_t launch_relax_f64_static(const DevBatch& b, const RunArgs& a, int grid,
                                    int64_t n_boundary_total, cudaStream_t s, StaticStatus* status);

// Orientation tensors (mfg_aux.cu), omega device n_rve * 9, normal device n_rve * 3
cudaError_t launch_orientation(const DevBatch& b, const double* normal, double* omega,
                               cudaStream_t s);
// Gathers status arrays into mfg_rve_status-shaped records (device).
cudaError_t launch_pack_status(const int32_t* status, const int32_t* steps,
                               const double* residual, int n, void* out, cudaStream_t s);

}  // namespace mfg

#endif
