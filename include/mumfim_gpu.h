/*
 * mumfim_gpu.h -- C ABI of the GB300 batched explicit fiber-network RVE solver.
 *
 * This is the drop-in boundary for MuMFiM's batched microscale analysis. Every
 * entry point below names the reference interface it replaces (paths are
 * relative to the mumfim source tree).
 *
 * Conventions
 *  - Plain C types only: host pointers + sizes in, integer status codes out.
 *    No function calls exit() or abort(); failures return an mfg_status and
 *    leave a message readable with mfg_last_error() (thread local).
 *  - Deformation gradients are row-major 3x3 (F[r*9 + 3*i + j] = F_ij), the
 *    same order the reference's DualView<Scalar*[3][3]> holds on the host.
 *  - Stress is Cauchy stress in Voigt order [xx, yy, zz, yz, xz, xy]
 *    (src/mumfim/microscale/batched_analysis/BatchedFiberRVEAnalysisExplicitBase.h:102-116).
 *  - Material stiffness C[r*36 + 6*j + i] = d sigma_j / d (perturbation i),
 *    i.e. C(rve, row j, column i) as in BatchedFiberRVEAnalysisExplicit.h:449-457.
 *  - Node-indexed outputs are always in the caller's ORIGINAL node order; the
 *    boundary-last reordering the solver uses internally is never visible.
 *  - One mfg_batch must be used by one host thread at a time.
 */
#ifndef MUMFIM_GPU_H
#define MUMFIM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MFG_ABI_VERSION 1

/* Step cap applied in MFG_MODE_RELAX when mfg_strategy.max_steps <= 0. The
 * reference loops without a cap (TeamOuterLoop.h:340-371); a cap turns a
 * network that never relaxes into MFG_E_NOT_CONVERGED instead of a hang. */
#define MFG_DEFAULT_STEP_CAP 1000000

/* Status codes. The reference prints to cerr and calls std::exit on bad sizes
 * (BatchedFiberRVEAnalysisExplicitBase.h:136-142,
 * BatchedFiberRVEAnalysisExplicit.h:85-90,324-330) and reports nothing on
 * non-convergence; these codes replace both behaviours. */
typedef enum mfg_status {
  MFG_OK = 0,
  MFG_E_INVALID = 1,       /* bad argument, size mismatch, malformed network */
  MFG_E_OOM = 2,           /* device or host allocation failed */
  MFG_E_NOT_CONVERGED = 3, /* step cap reached before residual <= tol */
  MFG_E_NONFINITE = 4,     /* NaN/Inf met in the residual or the stress */
  MFG_E_TIMEOUT = 5,       /* a bounded wait gave up (serving queue) */
  MFG_E_CUDA = 6,          /* a CUDA runtime call failed */
  MFG_E_NO_DEVICE = 7,     /* no usable sm_103 device */
  MFG_E_BUSY = 8           /* serving: no free slot / HBM for admission */
} mfg_status;

/* Fiber constitutive law ids, as in the .params format and the enum order of
 * src/mumfim/microscale/FiberReactions.h:9-13 (linear = 0, nonlinear = 1). */
typedef enum mfg_law { MFG_LAW_LINEAR = 0, MFG_LAW_NONLINEAR = 1 } mfg_law;

/* One fiber reaction (FiberReactions.h:15-43). The fiber area is
 * radius * radius * pi exactly as the .params reader forms it
 * (FiberNetworkIO_impl.h:23-27). `B` and `length_ratio_trns` are used by the
 * nonlinear law only; its compressive transition ratio is fixed at 1.0
 * (FiberNetworkIO_impl.h:35). */
typedef struct mfg_reaction {
  int32_t law;
  int32_t pad_;
  double radius;
  double youngs_modulus;
  double density;
  double B;
  double length_ratio_trns;
} mfg_reaction;

/* One RVE's fiber network in the reference frame: the data the reference pulls
 * out of the APF mesh in BatchedMesh.h:23-150. Nodes inside 1e-8 of a face of
 * the cube [-0.5,0.5]^3 are the fixed boundary (RVE.h:86-103). As in the
 * reference, only reaction 0 drives the batched solve
 * (BatchedFiberRVEAnalysisExplicit.h:202-212). */
typedef struct mfg_network {
  int32_t n_nodes;
  int32_t n_fibers;
  const double* coords;        /* n_nodes x 3, row-major */
  const int32_t* connectivity; /* n_fibers x 2, 0-based node ids */
  mfg_reaction reaction;
  double scale_factor; /* FiberNetwork::getScaleConversion(), default 1 */
} mfg_network;

/* Solve mode. RELAX is the reference's algorithm: affine predictor on every
 * node, then damped explicit relaxation until the free-node residual is
 * <= residual_tol, checked every 100 steps
 * (BatchedFiberRVEAnalysisExplicitTeamOuterLoop.h:291-372). RAMP is the
 * fixed-step protocol: no predictor, the boundary moves linearly from its
 * start position to F * start over exactly max_steps steps. Both share the
 * same step. */
typedef enum mfg_mode { MFG_MODE_RELAX = 0, MFG_MODE_RAMP = 1 } mfg_mode;

/* Per-RVE solution strategy (MicroSolutionStrategyExplicit, MicroFOParams.h:82-95).
 * The reference's batched kernel ignores the configured critical time-scale
 * factor and uses 0.8 (TeamOuterLoop.h:312); pass 0.8 for reference behaviour. */
typedef struct mfg_strategy {
  double visc_damp_coeff;        /* mass-proportional damping c */
  double crit_time_scale_factor; /* dt = factor * l_min / sqrt(E/rho) */
  double residual_tol;           /* reference: 1e-6 */
  int32_t max_steps;             /* RELAX: step cap (<= 0: MFG_DEFAULT_STEP_CAP); RAMP: steps */
  int32_t mode;                  /* mfg_mode */
} mfg_strategy;

/* Arithmetic of the solve. F64 is the plain kernel: IEEE FP64 with the
 * reference's operation order and no contraction, bit-identical to a serial
 * CPU run of the same algorithm. MIXED runs fiber forces and the integrator in
 * FP32 on top of FP64 reference coordinates plus Kahan-compensated FP32
 * displacements, and keeps FP64 for the stress, the residual and dt. */
typedef enum mfg_precision { MFG_PREC_F64 = 0, MFG_PREC_MIXED = 1 } mfg_precision;

typedef struct mfg_options {
  int32_t precision;        /* mfg_precision */
  int32_t device;           /* CUDA device ordinal */
  int32_t threads_per_rve;  /* ignored: the CTA size is fixed per precision */
  int32_t max_cluster_ctas; /* mixed precision: largest thread-block cluster an RVE
                               may be split over (1, 2, 4 or 8; 0 = 8). 1 solves
                               every RVE on one CTA, with the same results. */
  int32_t cluster_layout;   /* mixed precision: mfg_cluster_layout. MFG_LAYOUT_SERVING
                               places RVEs that need a cluster on clusters of 4
                               (never 2), the size the serving kernel solves in
                               clusters; the results are the same either way. */
  int32_t stiffness;        /* mfg_stiffness_solves: how mfg_batch_material_stiffness()
                               runs its six perturbed solves */
  int32_t small_rves_per_cta; /* mixed precision, MFG_SMALL_FIBER_CENTRIC only: how many
                               small RVEs (whole state within half a CTA's shared
                               memory) one CTA solves side by side, 1 or 2 (0 = 2);
                               the results are the same either way */
  int32_t small_rve_solve;  /* mixed precision: mfg_small_rve_solve */
} mfg_options;

/* Mixed precision: the solve of an RVE whose node state fits one CTA. Both
 * give the same bits; only the speed differs.
 *  NODE_CENTRIC   every incident fiber evaluated at each free node, node
 *                 state in shared memory (the solve of the larger RVEs too).
 *  FIBER_CENTRIC  a fiber pass stores each fiber's force vector, a node pass
 *                 gathers them; the whole state in shared memory where it
 *                 fits, two small RVEs per CTA by small_rves_per_cta.
 *  AUTO           per RVE: NODE_CENTRIC on the linear law (faster on every
 *                 size measured), FIBER_CENTRIC on the nonlinear law (whose
 *                 exponential NODE_CENTRIC evaluates at both fiber ends). */
typedef enum mfg_small_rve_solve {
  MFG_SMALL_AUTO = 0,
  MFG_SMALL_NODE_CENTRIC = 1,
  MFG_SMALL_FIBER_CENTRIC = 2
} mfg_small_rve_solve;

/* The six perturbed solves of mfg_batch_material_stiffness(). The reference
 * runs them as six whole-batch runs one after the other
 * (BatchedFiberRVEAnalysisExplicit.h:321-405), and each non-updating run
 * leaves its relaxed current coordinates behind (it restores only the
 * displacement), which the next run's affine predictor starts from. In RAMP
 * mode nothing reads those coordinates, so the six solves are independent.
 *  CONCURRENT   all six solves of every RVE in flight at once (six sets of
 *               per-solve scratch, 6 x the FP64 node and fiber work arrays),
 *               each starting from the state of the last updating run; the
 *               current coordinates end as the sixth solve leaves them. In
 *               RAMP mode this gives the sequential results bit for bit; in
 *               RELAX mode each predictor starts from the last updating
 *               run's coordinates instead of the previous perturbation's, so
 *               results differ within the relaxation tolerance.
 *  SEQUENTIAL   the reference's order, in every mode.
 *  AUTO         CONCURRENT when every RVE of the batch is in RAMP mode (where
 *               it is exact), else SEQUENTIAL. */
typedef enum mfg_stiffness_solves {
  MFG_STIFFNESS_AUTO = 0,
  MFG_STIFFNESS_SEQUENTIAL = 1,
  MFG_STIFFNESS_CONCURRENT = 2
} mfg_stiffness_solves;

typedef enum mfg_cluster_layout {
  MFG_LAYOUT_BATCH = 0,   /* smallest of 1, 2, 4, 8 CTAs that holds the RVE */
  MFG_LAYOUT_SERVING = 1  /* 1, 4 or 8 CTAs (mfg_server_create uses this) */
} mfg_cluster_layout;

/* Per-RVE outcome of one solve. */
typedef struct mfg_rve_status {
  int32_t status;  /* MFG_OK, MFG_E_NOT_CONVERGED or MFG_E_NONFINITE */
  int32_t steps;   /* explicit steps taken */
  double residual; /* last residual norm evaluated */
} mfg_rve_status;

typedef struct mfg_batch mfg_batch;

/* ---- library ---------------------------------------------------------- */
int32_t mfg_abi_version(void);
const char* mfg_status_string(mfg_status s);
/* Message of the last failure on the calling thread ("" when none). */
const char* mfg_last_error(void);
void mfg_default_strategy(mfg_strategy* out);
void mfg_default_options(mfg_options* out);

/* ---- batch lifecycle -------------------------------------------------- */
/* Replaces BatchedFiberRVEAnalysisExplicit(fiber_networks, solution_strategies)
 * (src/mumfim/microscale/BatchedFiberRVEAnalysisExplicit.h:80-256): finds the
 * boundary, lumps the nodal mass (row-sum, rho*A*L0/2 per fiber end), builds
 * the boundary-last permutation and the CSR fiber incidence, and uploads the
 * batch to the device. `nets` and `strategies` hold n_rve entries each. */
mfg_status mfg_batch_create(const mfg_network* nets, const mfg_strategy* strategies,
                            int32_t n_rve, const mfg_options* options, mfg_batch** out);
/* Frees every device and host resource of the batch. NULL is a no-op. */
mfg_status mfg_batch_destroy(mfg_batch* batch);
int32_t mfg_batch_size(const mfg_batch* batch);
int32_t mfg_batch_n_nodes(const mfg_batch* batch, int32_t rve);
int32_t mfg_batch_n_fibers(const mfg_batch* batch, int32_t rve);

/* ---- the hot path ----------------------------------------------------- */
/* Replaces BatchedRVEAnalysis::run(F, sigma, update_coords)
 * (src/mumfim/microscale/BatchedRVEAnalysis.h:29-31; implementation
 * BatchedFiberRVEAnalysisExplicit.h:257-320). F holds n_F row-major 3x3
 * incremental deformation gradients; n_F == 1 broadcasts to every RVE
 * (BatchedFiberRVEAnalysisExplicitBase.h:36) and is only valid with
 * update_coords == 0, as in the reference. sigma receives n_rve x 6 Voigt
 * Cauchy stresses. update_coords == 0 restores the displacement afterwards
 * (the reference's transactional run). status (n_rve entries) may be NULL.
 * Returns MFG_OK, or the worst per-RVE status, or an error. Blocking. */
mfg_status mfg_batch_run(mfg_batch* batch, const double* F, int32_t n_F, double* sigma,
                         int32_t update_coords, mfg_rve_status* status);
/* Same solve with device-resident F (n_F x 9) and sigma (n_rve x 6) pointers,
 * enqueued on `stream` (a cudaStream_t; NULL = the batch's own stream).
 * Returns after enqueueing; status_dev (device, n_rve entries) may be NULL. */
mfg_status mfg_batch_run_device(mfg_batch* batch, const double* F_dev, int32_t n_F,
                                double* sigma_dev, int32_t update_coords,
                                mfg_rve_status* status_dev, void* stream);
/* Replaces BatchedRVEAnalysis::computeMaterialStiffness(C)
 * (BatchedRVEAnalysis.h:36-37; BatchedFiberRVEAnalysisExplicit.h:321-405):
 * six perturbed, non-updating solves at h = 1e-5 around the stress of the last
 * updating run. C receives n_rve x 36 values, C[r*36 + 6*j + i]. */
mfg_status mfg_batch_material_stiffness(mfg_batch* batch, double* C);
/* Replaces compute3DOrientationTensor(omega) (BatchedRVEAnalysis.h:38-43;
 * BatchedComputeOrientationTensor.h:145-186): mean n (x) n over fibers in the
 * current configuration. omega: n_rve x 9, row-major. */
mfg_status mfg_batch_orientation_3d(mfg_batch* batch, double* omega);
/* Replaces compute2DOrientationTensor(normal, omega) (BatchedRVEAnalysis.h:44-50;
 * BatchedComputeOrientationTensor.h:55-144): fiber directions projected onto
 * the plane with the given normal (n_rve x 3) before averaging. */
mfg_status mfg_batch_orientation_2d(mfg_batch* batch, const double* normal, double* omega);

/* ---- state access ----------------------------------------------------- */
/* Node displacement u = x - X of one RVE (n_nodes x 3, original order). */
mfg_status mfg_batch_get_displacements(mfg_batch* batch, int32_t rve, double* u);
/* Current coordinates x of one RVE (n_nodes x 3, original order). */
mfg_status mfg_batch_get_coordinates(mfg_batch* batch, int32_t rve, double* x);
/* Stress of the last updating run (the reference's current_stress_),
 * n_rve x 6. */
mfg_status mfg_batch_get_current_stress(mfg_batch* batch, double* sigma);
/* Size in bytes of one RVE's exported state. */
size_t mfg_batch_state_bytes(const mfg_batch* batch, int32_t rve);
/* Copy one RVE's persistent state (u, x, volume, last stress) to / from a host
 * buffer of mfg_batch_state_bytes() bytes. The reference keeps this state only
 * in device memory between runs; export/import lets a caller evict and
 * restore an RVE. */
mfg_status mfg_batch_export_state(mfg_batch* batch, int32_t rve, void* buf, size_t bytes);
mfg_status mfg_batch_import_state(mfg_batch* batch, int32_t rve, const void* buf, size_t bytes);

/* ---- multiscale coupling ---------------------------------------------- */
/* Record sizes of the macro/micro exchange (MultiscaleMicroFOParams.h:79-104):
 * micro_fo_data = F (9), micro_fo_result = sigma (6) + averaged volume stress
 * (3, zero as in the reference) + stiffness (36), micro_fo_step_result = 3-D
 * orientation tensor (9) + 2-D orientation tensor (9), micro_fo_params = the
 * fiber_param_fields below. */
#define MFG_MICRO_FO_DATA 9
#define MFG_MICRO_FO_RESULT 45
#define MFG_MICRO_FO_STEP_RESULT 18
enum {
  MFG_PRM_FIBER_RADIUS = 0,
  MFG_PRM_VOLUME_FRACTION = 1,
  MFG_PRM_YOUNGS_MODULUS = 2,
  MFG_PRM_NONLINEAR_PARAM = 3,
  MFG_PRM_LINEAR_TRANSITION = 4,
  MFG_PRM_ORIENTATION_AXIS_X = 5,
  MFG_PRM_ORIENTATION_AXIS_Y = 6,
  MFG_PRM_ORIENTATION_AXIS_Z = 7,
  MFG_MICRO_FO_PARAMS = 8
};
/* Replaces calcScaleConversion(mesh, fbr_area, fbr_vol_frc)
 * (src/mumfim/microscale/MultiscaleCoupling.cc:7-23, called at
 * MultiscaleRVEAnalysis.cc:159-167): with L the summed reference length of
 * the fibers and A = pi r^2, the RVE edge is d = sqrt(L A / volume_fraction)
 * and the factor 1 / d^2 goes into mfg_network.scale_factor. Host only. */
mfg_status mfg_scale_conversion(int32_t n_nodes, const double* coords, int32_t n_fibers,
                                const int32_t* connectivity, double fiber_radius,
                                double volume_fraction, double* factor);
/* One macro iteration of the batched microscale service
 * (MultiscaleRVEAnalysis.cc:232-289): data holds n_rve micro_fo_data records
 * (row-major F), the batch runs with update_coords = 1, the stiffness follows,
 * and results receives n_rve micro_fo_result records. status may be NULL.
 * Returns what mfg_batch_run() returns (results are filled either way), or
 * the stiffness's error. Blocking. */
mfg_status mfg_batch_micro_fo_iterate(mfg_batch* batch, const double* data, double* results,
                                      mfg_rve_status* status);
/* Step results of the service (recoverMultiscaleStepResults,
 * MultiscaleCoupling.h:46-66): params holds n_rve micro_fo_params records;
 * step_results receives n_rve micro_fo_step_result records, the 2-D tensor
 * taken about each record's orientation axis. */
mfg_status mfg_batch_micro_fo_step(mfg_batch* batch, const double* params, double* step_results);

/* ---- solve without allocating ------------------------------------------ */
/* Size of the device array that mfg_batch_run_device_noalloc() takes its
 * scratch from (16 MiB). mfg_batch_create() of an FP64 batch reserves it on
 * the batch's device (CUDA loads the code that holds it lazily, and the
 * create call forces that load), and the device holds it until the process
 * exits. */
#define MFG_NOALLOC_SCRATCH_BYTES (16u << 20)

/* No counterpart in the reference. Same solve as mfg_batch_run_device() on
 * an FP64 batch, for callers that must not allocate device memory while they
 * solve: for instance a macroscale code whose device memory is owned by its
 * own pool allocator (every byte it has not handed out is spoken for), or a
 * time-stepping loop that forbids allocation after start-up. The call makes no
 * cudaMalloc/cudaFree and calls no allocating library routine: the kernel's
 * scratch (per-fiber force vectors, internal forces, RAMP boundary data, the
 * work counter and the per-RVE status words) comes from one file-scope device
 * array of MFG_NOALLOC_SCRATCH_BYTES bytes. The caller still passes the
 * inputs and outputs (device F and sigma, optional device status, as in
 * mfg_batch_run_device()); the batch keeps the RVE state.
 *  - Scratch need: 8 * (3 * fibers + 3 * nodes + 6 * boundary nodes) bytes
 *    over the whole batch plus 16 bytes per RVE (each piece rounded up to 256
 *    bytes). Larger batches get MFG_E_INVALID with the need in the message.
 *  - Every call looks up the array's device address with the batch's device
 *    current (a lookup, no allocation: the batch's creation already loaded
 *    the array). Do not use a batch across a cudaDeviceReset() of its
 *    device: the reset frees the batch's memory and the array with it.
 *  - Every call shares the one array: calls whose work overlaps on the GPU
 *    (other streams, other batches, other host threads) race on it and must
 *    be serialised by the caller. The array keeps the last call's contents;
 *    the call clears what must start at zero.
 *  - MIXED-precision batches are rejected (MFG_E_INVALID).
 * Returns after enqueueing on `stream` (NULL = the batch's own stream). */
mfg_status mfg_batch_run_device_noalloc(mfg_batch* batch, const double* F_dev, int32_t n_F,
                                        double* sigma_dev, int32_t update_coords,
                                        mfg_rve_status* status_dev, void* stream);

/* ---- serving --------------------------------------------------------- */
/* Replaces the microscale service loop of the multiscale coupling
 * (MultiscaleRVEAnalysis::run, src/mumfim/microscale/MultiscaleRVEAnalysis.cc:197-305):
 * instead of one blocking batch per macro iteration, integration points
 * submit deformation-gradient increments as they arrive and collect stresses
 * as they complete. Every registered RVE keeps its state on the device
 * between requests. A persistent kernel (one CTA per SM) claims requests from
 * a ring in host-mapped memory and solves each RVE as soon as a CTA frees up,
 * so requests that arrive while others are on the GPU join the running work
 * (continuous batching). Each solve is the same deterministic per-RVE
 * computation as mfg_batch_run(), so a result does not depend on what else is
 * in flight. Requests for an RVE that is already in flight wait on the host
 * and go out in submission order. */
typedef struct mfg_server mfg_server;

typedef struct mfg_server_options {
  int32_t precision;        /* mfg_precision (MFG_PREC_MIXED is the served path) */
  int32_t device;
  int32_t capacity;         /* request ring entries; 0 = 65536 */
  int32_t idle_timeout_us;  /* persistent kernel exits after this long without work; 0 = 20000 */
  double hbm_budget_bytes;  /* admission cap on the device state of all RVEs; 0 = free HBM */
  int32_t max_wait_ms;      /* longest a persistent-kernel CTA waits for work before it
                               leaves (device time; a host that stalls or is abandoned
                               frees the SMs within this); 0 = 5000 */
  int32_t reserved[3];
} mfg_server_options;

/* One completed request. sigma maps onto micro_fo_result.data[0..5] and C
 * onto micro_fo_result.data[9..44] (MultiscaleMicroFOParams.h:93-98). */
typedef struct mfg_server_result {
  int64_t ticket;
  int32_t rve;
  int32_t status;  /* MFG_OK, MFG_E_NOT_CONVERGED or MFG_E_NONFINITE */
  int32_t steps;
  int32_t stiffness_status;  /* worst status of the six perturbed solves; -1 when the
                                request did not ask for the stiffness */
  double residual;
  double sigma[6];
  double latency_s;  /* submit -> result seen by mfg_server_poll, host clock */
  double device_s;   /* claim -> completion on the device (stiffness solves included) */
  int64_t t_claim_ns;  /* device %globaltimer when a CTA claimed the request */
  int64_t t_done_ns;   /* device %globaltimer when its result was published */
  double C[36];        /* material stiffness C[6 j + i] as mfg_batch_material_stiffness()
                          returns it (zeros unless requested) */
} mfg_server_result;

void mfg_default_server_options(mfg_server_options* out);
/* No counterpart in the reference (which keeps every RVE on the device).
 * Estimated device memory, in bytes, of a batch or server of these n_rve
 * networks in the given precision: the figure mfg_server_create() admits
 * against its HBM budget, for a caller that pages RVEs in and out of the
 * device (export/import) under a budget of its own. Host only. */
double mfg_device_bytes_estimate(const mfg_network* nets, int32_t n_rve, int32_t precision);
/* Registers n_rve RVEs (as mfg_batch_create) and starts serving. Returns
 * MFG_E_BUSY when the RVEs' device state would exceed the HBM budget. */
mfg_status mfg_server_create(const mfg_network* nets, const mfg_strategy* strategies,
                             int32_t n_rve, const mfg_server_options* options, mfg_server** out);
/* Queues one solve of `rve` with the row-major increment F (9 doubles,
 * micro_fo_data.data). Non-blocking. MFG_E_BUSY when the ring is full. */
mfg_status mfg_server_submit(mfg_server* server, int32_t rve, const double* F,
                             int32_t update_coords, int64_t* ticket);
/* As mfg_server_submit(); with `stiffness` nonzero the request also returns
 * the RVE's material stiffness, the one computeMaterialStiffness(C) gives
 * after run() in the reference's service loop (MultiscaleRVEAnalysis.cc:257-258;
 * BatchedFiberRVEAnalysisExplicit.h:321-405): right after the request's own
 * solve the CTA (or cluster) that ran it runs the six perturbed,
 * non-updating solves in the reference's order, around the stress of the
 * RVE's last updating run. Stress and stiffness together make a full
 * micro_fo_result, bit-identical to mfg_batch_run() followed by a
 * sequential mfg_batch_material_stiffness() on the same RVE. */
mfg_status mfg_server_submit_ex(mfg_server* server, int32_t rve, const double* F,
                                int32_t update_coords, int32_t stiffness, int64_t* ticket);
/* Returns up to `capacity` completed requests, waiting up to timeout_ms for
 * the first one. MFG_E_TIMEOUT when work is outstanding and none completed. */
mfg_status mfg_server_poll(mfg_server* server, mfg_server_result* out, int32_t capacity,
                           int32_t* n_out, int32_t timeout_ms);
/* Requests submitted and not yet returned by mfg_server_poll. */
int64_t mfg_server_outstanding(const mfg_server* server);
/* Number of persistent-kernel launches so far. */
int64_t mfg_server_launches(const mfg_server* server);
/* The batch holding the RVE state, for state access while no request is
 * outstanding (displacements, export/import, orientation tensors). */
mfg_batch* mfg_server_batch(mfg_server* server);
/* Stops the kernel (after the solves in flight), frees everything. */
mfg_status mfg_server_destroy(mfg_server* server);

/* ---- metrics ---------------------------------------------------------- */
/* Structured log for a service loop (the reference has only its timing
 * prints, MultiscaleRVEAnalysis.cc:241,283-286): with a file set, every
 * mfg_batch_create, mfg_batch_run, mfg_batch_run_device,
 * mfg_batch_material_stiffness and every mfg_server_poll that returned
 * results or timed out appends one JSON object per line -- the call, its
 * status and message, sizes, per-RVE status counts, step counts, the
 * largest residual, fiber-steps and device / wall times. NULL or "" turns
 * it off. The MFG_METRICS_LOG environment variable sets it at the first
 * call when this function was never called. Process-wide, thread-safe. */
mfg_status mfg_set_metrics_log(const char* path);

/* ---- timing ----------------------------------------------------------- */
/* Device time of the last run's relaxation kernel and of the whole run, in
 * milliseconds, from CUDA events recorded on the launching stream. Valid
 * after the run has completed on the device. */
mfg_status mfg_batch_last_timing(mfg_batch* batch, float* relax_ms, float* run_ms);
/* Number of kernels the last run launched. */
int32_t mfg_batch_last_launches(const mfg_batch* batch);

#ifdef __cplusplus
}
#endif
#endif /* MUMFIM_GPU_H */
