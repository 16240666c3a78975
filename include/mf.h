/*
 * mf.h -- C ABI of the GB300 magnetization-and-force library (libmfgb.so).
 *
 * Drop-in boundary for the reference's solver class
 *   Libo::cuda_magnet_cgOptimizer   magnetic_solver/magnetic_force.cuh:36-174
 *                                   magnetic_solver/magnetic_force.cu:608-1410
 * and for the FMMTL direct evaluation of its two pair kernels
 *   fmmtl::direct                   fmmtl_minimum/fmmtl/Direct.hpp:62-74
 *   DipoleBKernel                   fmmtl_minimum/kernel/Dipole_B.kern:13-134
 *   DipoleHessianKernel             fmmtl_minimum/kernel/Dipole_hessian.kern:19-278
 *
 * Plain C: pointers, sizes and status codes only.  Every call returns an
 * mf_status; mf_last_error() gives a message for the calling thread's last
 * failure.  A handle is used by one host thread at a time.  All device work
 * of a handle runs on the handle's stream (mf_set_stream; default: the
 * legacy default stream).  Calls that hand results to host memory return
 * after the copy has completed.
 *
 * Layouts.  Host arrays passed to the solver are AoS float [n][3] (the
 * reference's std::vector<float3>) unless MF_LAYOUT_SOA is given, in which
 * case x[n], y[n], z[n] follow one another.  Published results (MF_Q_*) live
 * on the device as SoA float arrays, like the reference's
 * cuda_abstract_vector members (dev_x, dev_y, dev_z).
 */
#ifndef MF_GB300_H
#define MF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MF_ABI_VERSION 4

typedef enum mf_status {
  MF_OK = 0,
  MF_ERR_INVALID_ARG = 1,   /* bad pointer, size, NaN/Inf input, unknown key */
  MF_ERR_OOM = 2,           /* device allocation failed */
  MF_ERR_NOT_CONVERGED = 3, /* solver hit its iteration cap above tolerance */
  MF_ERR_CUDA = 4,          /* a CUDA runtime call failed */
  MF_ERR_TIMEOUT = 5,       /* a kernel's bounded wait ran out (device error word set) */
  MF_ERR_BUDGET = 6,        /* admission refused: over the HBM budget */
  MF_ERR_UNSUPPORTED = 7,   /* no CUDA device / feature not available */
  MF_ERR_BUSY = 8           /* serving queue full */
} mf_status;

typedef enum mf_layout { MF_LAYOUT_AOS = 0, MF_LAYOUT_SOA = 1 } mf_layout;
typedef enum mf_where { MF_HOST = 0, MF_DEVICE = 1 } mf_where;
typedef enum mf_precision { MF_FP32 = 0, MF_FP64 = 1 } mf_precision;

/* Quantities a solver publishes (the reference's public members). */
typedef enum mf_quantity {
  MF_Q_POSITIONS = 0, /* xyz                 magnetic_force.cuh:136 */
  MF_Q_M = 1,         /* M = V chi/(1+chi) b magnetic_force.cuh:140 */
  MF_Q_B_OVER_MU0 = 2,/* total_B_over_mu0   magnetic_force.cuh:141 */
  MF_Q_HEXT = 3,      /* Hext               magnetic_force.cuh:138 */
  MF_Q_FORCE = 4,     /* magnetic_bodyforce magnetic_force.cuh:152 */
  MF_Q_DHEXTDX = 5,   /* dHextdx            magnetic_force.cuh:148 */
  MF_Q_DHEXTDY = 6,   /* dHextdy            magnetic_force.cuh:149 */
  MF_Q_DHEXTDZ = 7,   /* dHextdz            magnetic_force.cuh:150 */
  MF_Q_VELOCITY = 8   /* harness state of mf_advance (not in the reference) */
} mf_quantity;

/* Solver algorithms. */
typedef enum mf_solver_kind {
  /* The reference's least-squares nonlinear CG: 3 field products per
   * iteration, absolute RMS tolerance, stop on error increase, restart every
   * 10 iterations (magnetic_force.cu:874-1095, :1275-1315).  Default. */
  MF_SOLVER_NLCG = 0,
  /* Conjugate gradients on (I - c G) b = Hext (symmetric positive definite),
   * one field product per iteration, FP64 inner products, stop on relative
   * residual |r|/|Hext| < rel_tol. */
  MF_SOLVER_CG = 1
} mf_solver_kind;

/* Option keys for mf_set_option / mf_get_option. */
typedef enum mf_option {
  MF_OPT_TOLERANCE = 0,     /* NLCG absolute RMS tolerance (reference default 0.1) */
  MF_OPT_MAX_ITERATION = 1, /* NLCG iteration cap (reference default 80) */
  MF_OPT_NAIVE = 2,         /* 1: reproduce the reference's naive CUDA path:
                               external sources use h (not ext_mag_h) and the
                               external force term gets an extra mu0
                               (magnetic_force.cu:1118, :589-600) */
  MF_OPT_SOLVER = 3,        /* mf_solver_kind */
  MF_OPT_REL_TOL = 4,       /* CG relative residual tolerance (default 1e-6 FP32, 1e-8 FP64) */
  MF_OPT_CG_MAX_ITER = 5,   /* CG iteration cap (default 500) */
  MF_OPT_CRIT_SIZE = 6,     /* accepted for compatibility (crit_size, :647); the FMM's leaf
                               size is MF_OPT_FMM_LEAF */
  MF_OPT_CHECK_INTERVAL = 7,/* CG: iterations launched between host convergence checks
                               (default 1 for N >= 16384, else 4) */
  MF_OPT_KERNEL_TIMING = 8, /* 1: time every all-pairs launch (and every FMM product as a
                               whole) with CUDA events (mf_get_kernel_stats) */
  MF_OPT_FMM = 9,           /* field and force products of FP32 handles: 0 auto (field
                               products through the FMM above 65,536 particles, the Kelvin
                               force above 90,000; all-pairs below), 1 always the FMM,
                               2 always all-pairs.  FP64 handles are all-pairs. */
  MF_OPT_FMM_ORDER = 10,    /* expansion order P counted as the reference counts it
                               (terms of degree n < P): 4..9, default 8.  The reference's
                               default is 6 (magnetic_force.cu:661); at 6 the field here is
                               3e-5 from FP64 direct sums, at 8 2-3e-6. */
  MF_OPT_FMM_THETA = 11,    /* multipole acceptance aperture of the field products, default 0.5
                               (FMMOptions.hpp:118) */
  MF_OPT_FMM_LEAF = 12,     /* FMM leaf level: the deepest whose boxes hold at least this many
                               particles on average (default 12) */
  MF_OPT_AUTOTUNE = 13,     /* block shapes of the FP32 all-pairs launches: 0 fixed default,
                               1 tuned (default; each new body and size class is timed once
                               per process on the scene's own data), 2 tuned choices only when
                               already cached.  MF_AUTOTUNE=0 in the environment makes 0 the
                               default for handles and batches. */
  MF_OPT_PAIR_SYMMETRIC = 14,/* FP32 packed field and force products of the handle's scene,
                               each unordered pair evaluated once for both particles (a pair
                               kernel and a per-particle finish) instead of every ordered
                               pair: 0 never, 1 where tuning measured it faster (default;
                               without tuning, the force only), 2 always.  On the FMM path
                               the force's near field is evaluated once per unordered box
                               pair with 2, and with 1 from 1,048,576 particles on.  Not in
                               the reference. */
  MF_OPT_FMM_FORCE_THETA = 15,/* aperture of the Kelvin force (and the external gradient tensor)
                               products on the FMM path, default 0.44; they use the smaller of
                               this and MF_OPT_FMM_THETA.  The force takes the Hessian of the
                               local expansion, whose error relative to the small net force
                               of a magnetised body is ~40x the field's: 1.3e-4 at 0.5 and
                               P = 8, 6.6e-6 at 0.44 and P = 10 (1,048,576 particles).  Not in
                               the reference. */
  MF_OPT_FMM_FORCE_ORDER = 16,/* expansion order P of those products (4..10), default 10: two
                               degrees more than the field's default let the wider aperture
                               meet 1e-5 with fewer near pairs.  Not in the reference. */
  MF_OPT_FUSED_PRODUCTS = 17 /* FP32 handles whose field and force both run once per unordered
                               pair: the solve's first residual product also forms the
                               Kelvin force of the same magnetization in the same launch,
                               used by mf_eval_force if the solve then needs no iteration
                               (the warm start stands, so M is unchanged) and discarded
                               otherwise.  0 never, 1 after a solve whose warm start stood
                               (default), 2 every solve.  Results equal the separate
                               products' to FP32 rounding.  Not in the reference. */
} mf_option;

/* Construction parameters: the reference's CtorParam (magnetic_force.cuh:39-76). */
typedef struct mf_params {
  int64_t num_particles;
  float h;
  float ext_mag_h;
  float volume;
  float chi;
  float const_ext_field[3];
  const float* target_pos;     /* host AoS [num_particles][3] */
  const float* ext_source_pos; /* host AoS [n_ext][3], may be NULL if n_ext == 0 */
  const float* ext_source_M;   /* host AoS [n_ext][3] */
  int64_t n_ext;
  int32_t precision;           /* mf_precision */
  int32_t device;              /* CUDA device ordinal */
} mf_params;

typedef struct mf_solver mf_solver;

/* Status text and the calling thread's last error message. */
const char* mf_status_string(mf_status s);
const char* mf_last_error(void);
int mf_abi_version(void);

/* Constructor / destructor.
 * Replaces cuda_magnet_cgOptimizer::cuda_magnet_cgOptimizer(CtorParam)
 * (magnetic_force.cu:608-703) and ~cuda_magnet_cgOptimizer. */
mf_status mf_create(const mf_params* p, mf_solver** out);
mf_status mf_destroy(mf_solver* s);

/* Stream all of the handle's work is issued on (cudaStream_t as void*). */
mf_status mf_set_stream(mf_solver* s, void* stream);

/* setTargetpos(const std::vector<float3>&) (magnetic_force.cu:806-871), with
 * Resize (magnetic_force.cu:706-743): a new particle count keeps the first
 * min(old, new) entries of total_B_over_mu0 as the warm start (new entries
 * start at zero).  `where` says whether xyz is host or device memory. */
mf_status mf_set_positions(mf_solver* s, const float* xyz, int64_t n, int32_t layout, int32_t where);

/* setHext(const setHextParams&) (magnetic_force.cu:746-803). */
mf_status mf_set_external(mf_solver* s, const float H0[3], const float* src_pos, const float* src_M,
                          int64_t n_src, float ext_mag_h);

/* solve(size_t niter) (magnetic_force.cu:874-888).  Runs the configured
 * solver; *iters (may be NULL) gets the iterations run and *final_err the
 * last error (NLCG: 0.5|r|^2 as in total_error; CG: |r|/|Hext|).
 * NLCG returns MF_OK whenever it stops as the reference would; CG returns
 * MF_ERR_NOT_CONVERGED if it reached its cap above tolerance. */
mf_status mf_solve(mf_solver* s, int64_t niter, int64_t* iters, double* final_err);

/* The NLCG error history of the last solve (total_error, magnetic_force.cuh:116).
 * Copies min(cap, len) doubles into dst and returns the length in *len. */
mf_status mf_get_error_history(mf_solver* s, double* dst, int64_t cap, int64_t* len);

/* evaluate_fitted_near_foece() (magnetic_force.cu:890-997): M = c b, then the
 * Kelvin force F_i = (Rext_i + sum_j T_ij) m_i into MF_Q_FORCE. */
mf_status mf_eval_force(mf_solver* s);

/* Copy a published quantity (n x 3 floats) to dst in the given layout.
 * where == MF_DEVICE copies device-to-device. */
mf_status mf_get(mf_solver* s, int32_t quantity, float* dst, int32_t layout, int32_t where);
/* Same for FP64 solvers' full-precision values (FP32 solvers convert). */
mf_status mf_get_f64(mf_solver* s, int32_t quantity, double* dst, int32_t layout, int32_t where);

/* Device SoA pointers of a published quantity (the reference's public
 * members' dev_x / dev_y / dev_z).  Valid until the next call that changes
 * the particle count. */
mf_status mf_device_soa(mf_solver* s, int32_t quantity, float** x, float** y, float** z);

mf_status mf_num_particles(mf_solver* s, int64_t* n);

mf_status mf_set_option(mf_solver* s, int32_t key, double value);
mf_status mf_get_option(mf_solver* s, int32_t key, double* value);

/* export_data / export_force (magnetic_force.cu:1318-1410): one line per
 * particle, "i x y z v0 v1 v2 H0 H1 H2", v = total_B_over_mu0 / force. */
mf_status mf_export_data(mf_solver* s, const char* path);
mf_status mf_export_force(mf_solver* s, const char* path);

/* One timestep of the benchmark harness, all on the device: solve (warm
 * start), force, then symplectic Euler v += dt F / (rho V), x += dt v with
 * unit density.  Not part of the reference (its caller moves the particles). */
mf_status mf_advance(mf_solver* s, double dt, int64_t niter, int64_t* iters);

/* Counters: field products, force passes and pair interactions issued by
 * this handle since creation (or the last reset). */
typedef struct mf_counters {
  int64_t field_products;
  int64_t force_passes;
  double field_pairs;
  double force_pairs;
  int64_t kernel_launches;
} mf_counters;
mf_status mf_get_counters(mf_solver* s, mf_counters* c);
mf_status mf_reset_counters(mf_solver* s);

/* Per-kernel device time of a handle's all-pairs launches, measured with
 * CUDA events on the handle's stream while MF_OPT_KERNEL_TIMING is on.
 * Launches that found their solve already stopped are not counted.
 * Reset by mf_reset_counters.  Synchronises the handle's stream. */
typedef enum mf_kernel_kind {
  MF_K_FIELD = 0,           /* field products (an FMM product timed as a whole) */
  MF_K_FORCE = 1,           /* force products (likewise) */
  MF_K_TENSOR = 2,          /* external gradient tensor */
  MF_K_FMM_NEAR_FIELD = 3,  /* the FMM near-field kernel of field products; pairs = executed near pairs */
  MF_K_FMM_NEAR_FORCE = 4,  /* the FMM near-field kernel of force products */
  MF_K_FMM_FAR = 5,         /* the FMM far-field stages (gather, P2M, M2M, M2L, L2L); pairs = M2L translations */
  MF_K_FIELD_FORCE = 6      /* field and force in one launch (MF_OPT_FUSED_PRODUCTS); pairs = both
                               products' pairs, evals = unordered pairs */
} mf_kernel_kind;
typedef struct mf_kernel_stats {
  int64_t launches;
  double total_ms;
  double pairs;  /* ordered target-source pairs the launches covered */
  double evals;  /* pair evaluations the algorithm needs for them: equal to
                    pairs, except for the force product of one scene, where
                    one evaluation serves both particles of an unordered pair
                    (n (n - 1) / 2 per scene) */
} mf_kernel_stats;
mf_status mf_get_kernel_stats(mf_solver* s, int32_t kind, mf_kernel_stats* out);

/* The autotuner's choices so far in this process, one line per (device,
 * body, size class): the chosen block shape (threads x targets per thread /
 * sources per tile) and the measured ms of every shape.  Writes at most cap
 * bytes (NUL-terminated); *len gets the full length.  Not in the reference. */
mf_status mf_autotune_report(char* buf, int64_t cap, int64_t* len);

/* Shape and work of the handle's FMM (uniform octree over the current
 * positions; built on the first product after the positions change).
 * Replaces the tree and interaction-list state of the reference's
 * fmmtl::kernel_matrix plans (KernelMatrixPlan.hpp:75-113). */
typedef struct mf_fmm_stats {
  int32_t active;            /* 1 if the handle's field products use the FMM */
  int32_t levels;            /* box grid levels, root included */
  int32_t leaf_level;
  int32_t degree;            /* expansion degree (order - 1) */
  int64_t leaf_boxes;        /* boxes of the leaf grid */
  int64_t occupied_leaves;
  int32_t max_leaf;          /* particles in the fullest leaf box */
  int32_t near_rows;         /* rows of near leaf boxes per target box */
  double p2p_pairs;          /* near-field pairs executed per product */
  double m2l_per_product;    /* multipole-to-local translations per product */
  int32_t launches_per_product;
  int32_t force_active;      /* 1 if the handle's Kelvin force uses the FMM */
  int64_t field_products;    /* FMM products since the last mf_reset_counters */
  int64_t force_products;
  double theta;              /* aperture of the field products */
  double force_theta;        /* aperture of the force products */
  double force_p2p_pairs;    /* near-field pairs per force product (0 unless force_active) */
  double force_m2l_per_product;
} mf_fmm_stats;
mf_status mf_get_fmm_stats(mf_solver* s, mf_fmm_stats* out);

/* out = G(moments): B/mu0_i = sum_j K_B(x_i - x_j; h) m_j over the handle's
 * particles, through the path its products take (FMM or all-pairs).  moments
 * and out are float [n][3] (AOS) or [3][n] (SOA) in host or device memory.
 * Replaces cuda_magnet_cgOptimizer::G (magnetic_force.cu:1196-1271). */
mf_status mf_apply_field(mf_solver* s, const float* moments, int32_t layout, int32_t where, float* out);

/* Measured dense FP32 FMA throughput of the current device in TFLOP/s
 * (independent FFMA chains on every SM, timed with CUDA events): the
 * denominator of the all-pairs kernels' roofline.  Not in the reference. */
mf_status mf_probe_fp32_peak(double* tflops);

/* ---------------------------------------------------------------------- */
/* Direct all-pairs evaluation of the reference's pair kernels on device    */
/* buffers (AoS float [n][3] device arrays; results overwritten).           */
/* ---------------------------------------------------------------------- */

/* results_i = sum_j DipoleBKernel{h}(targets_i, sources_j) * charges_j
 * Replaces fmmtl::direct(DipoleBKernel, ...) (Direct.hpp:62-74 ->
 * S2T.hpp:57-79) and the naive cuda_Apply_G / cuda_ext_field_kernel bodies
 * (magnetic_force.cu:8-237).  Allocates its scratch on first use. */
mf_status mf_direct_field(const float* targets, int64_t nt, const float* sources, const float* charges,
                          int64_t ns, float h, float* results, void* stream);

/* results9_i = sum_j DipoleHessianKernel{h}(targets_i, sources_j) * charges_j,
 * 3x3 per target in glm column-major order (results9[i*9 + c*3 + r]).
 * Replaces fmmtl::direct(DipoleHessianKernel, ...) and
 * cuda_ext_fitted_force_tensor_kernel (magnetic_force.cu:432-512). */
mf_status mf_direct_force_tensor(const float* targets, int64_t nt, const float* sources,
                                 const float* charges, int64_t ns, float h, float* results9, void* stream);

/* F_i = (sum_j T(x_i - x_j; h) m_j) m_i over one particle set, plus
 * Rext_i m_i when rext9 (device [n][9], may be NULL) is given: the force
 * assembly of fitted_force_ofM_kernel / evaluate_fitted_near_foece
 * (magnetic_force.cu:516-605, :968-980). */
mf_status mf_direct_force(const float* pos, const float* mom, int64_t n, float h, const float* rext9,
                          int32_t naive_quirks, float* force, void* stream);

/* Frees the scratch the mf_direct_* calls keep per device. */
mf_status mf_release_scratch(void);

/* Debug (off by default; not in the reference, whose kernels check nothing,
 * cuda_abstract_vector.cuh:169-175): the staging waits of the all-pairs and
 * once-per-pair kernels launched from now on give up after `limit` try-waits
 * (0: at once), so the bounded-wait error path can be exercised: the launch
 * reports MF_ERR_TIMEOUT, its copies in flight are drained with the default
 * bound before each CTA leaves, and the scratch is reset for the next call.
 * limit < 0 restores the default bound.  Process-wide. */
mf_status mf_debug_stage_wait_limit(int64_t limit);

/* ---------------------------------------------------------------------- */
/* FMM matrix over a source set and a target set: the replacement of       */
/* fmmtl::kernel_matrix<DipoleBSpherical>(kernel, sources, targets) and    */
/* its operator* (fmmtl/KernelMatrix.hpp:26-164, :127-131).  The octree,   */
/* lists and near-field cell list are built once at creation; each product */
/* takes new charges.  Host AoS float arrays.                              */
/* ---------------------------------------------------------------------- */
typedef struct mf_fmm mf_fmm;
/* targets may be NULL (nt ignored): the targets are the sources.  order is
 * P as the reference counts it (4..9), theta the acceptance aperture of the
 * field product, leaf_min the mean particles per leaf box.  The Hessian
 * product uses the aperture min(theta, 0.44) and the order 10, as the
 * handles' force does (MF_OPT_FMM_FORCE_THETA, MF_OPT_FMM_FORCE_ORDER): its
 * lists are built on its first call. */
mf_status mf_fmm_create(const float* sources, int64_t ns, const float* targets, int64_t nt, float h, int32_t order,
                        double theta, int32_t leaf_min, int32_t device, mf_fmm** out);
mf_status mf_fmm_destroy(mf_fmm* f);
/* results[nt][3] = sum_j DipoleBKernel{h}(targets_i, sources_j) * charges_j */
mf_status mf_fmm_field(mf_fmm* f, const float* charges, float* results);
/* results9[nt][9] = sum_j DipoleHessianKernel{h}(targets_i, sources_j) * charges_j, the 3x3 force
 * tensor per target in glm column-major order (results9[i*9 + c*3 + r]), as mf_direct_force_tensor:
 * the kernel_matrix<DipoleHessianSpherical> product. */
mf_status mf_fmm_hessian(mf_fmm* f, const float* charges, float* results9);
mf_status mf_fmm_get_stats(mf_fmm* f, mf_fmm_stats* out);

/* ---------------------------------------------------------------------- */
/* Batched scenes.  Not in the reference, which solves one object per       */
/* cuda_magnet_cgOptimizer instance: here many independent objects (each   */
/* the reference's problem with its own particles, h, V, chi and uniform    */
/* external field) advance together, every stage one launch for all of     */
/* them, FP32 pair arithmetic and FP64 solver sums.                         */
/* ---------------------------------------------------------------------- */
typedef struct mf_scene_desc {
  int64_t n;          /* particles */
  const float* pos;   /* host AoS [n][3] */
  float h;            /* smoothing length */
  float volume;       /* particle volume V */
  float chi;          /* susceptibility */
  float H0[3];        /* uniform external field */
} mf_scene_desc;

typedef struct mf_batch mf_batch;

mf_status mf_batch_create(const mf_scene_desc* scenes, int32_t n_scenes, int32_t device, mf_batch** out);
mf_status mf_batch_destroy(mf_batch* b);
mf_status mf_batch_set_stream(mf_batch* b, void* stream);
mf_status mf_batch_num_scenes(mf_batch* b, int32_t* n);

/* CG solve of every scene's magnetization (warm start), each scene stopping
 * at relative residual rel_tol or after max_iter iterations.  *max_iters
 * (may be NULL) gets the most iterations any scene ran, *worst_res the
 * largest final relative residual. */
mf_status mf_batch_solve(mf_batch* b, int64_t max_iter, double rel_tol, int64_t* max_iters, double* worst_res);

/* Kelvin force of every scene (after a solve). */
mf_status mf_batch_eval_force(mf_batch* b);

/* `steps` timesteps: solve (at most iters_per_step CG iterations, rel_tol),
 * force, symplectic Euler with unit density.  With use_graph != 0 one
 * timestep is captured in a CUDA graph on first use (for these dt,
 * iters_per_step, rel_tol) and replayed. */
mf_status mf_batch_advance(mf_batch* b, double dt, int32_t steps, int32_t iters_per_step, double rel_tol,
                           int32_t use_graph);

/* A scene's quantity (MF_Q_POSITIONS, MF_Q_M, MF_Q_B_OVER_MU0, MF_Q_HEXT,
 * MF_Q_FORCE, MF_Q_VELOCITY) into host AoS dst [n][3]. */
mf_status mf_batch_get(mf_batch* b, int32_t scene, int32_t quantity, float* dst);

/* Per-scene relative residuals and iterations of the last solve. */
mf_status mf_batch_solver_state(mf_batch* b, double* rel_res, double* iters);

mf_status mf_batch_get_counters(mf_batch* b, mf_counters* c);
mf_status mf_batch_reset_counters(mf_batch* b);

/* ---------------------------------------------------------------------- */
/* Serving: a request queue with continuous batching (not in the reference).*/
/* A request is a scene to advance by steps_per_request timesteps.  Each    */
/* mf_server_step admits queued requests while the HBM budget and the slot  */
/* limit allow, advances every running request by one timestep in shared   */
/* batched launches, and retires finished requests (their final state is   */
/* kept for mf_server_result).  Particle state stays on the device while a  */
/* request runs.  Requests above 65,536 particles run as their own solver */
/* handle (field products through the FMM at P = 8, the Kelvin force as    */
/* MF_OPT_FMM's automatic choice picks it), on a host thread and a stream of their own */
/* started at admission: their timesteps overlap the batch on the device   */
/* and do not wait for ticks; a tick retires them once finished.  A server */
/* is used by one host thread at a time.  While a server exists, device    */
/* memory the library frees is parked (cudaFree would wait for the FMM     */
/* requests' kernels) and released at a tick with no FMM request running, */
/* past 8 GB parked, on an allocation failure, or by mf_server_destroy.    */
/* ---------------------------------------------------------------------- */
typedef struct mf_server_config {
  double hbm_budget_bytes;   /* admission budget for request state (e.g. 120e9) */
  int32_t max_active;        /* running requests at most */
  int32_t steps_per_request; /* timesteps each request runs */
  int32_t iters_per_step;    /* CG iterations per timestep at most (warm start) */
  int32_t device;
  double rel_tol;            /* CG relative tolerance */
  double dt;                 /* timestep */
} mf_server_config;

typedef struct mf_server_stats {
  int64_t submitted, running, queued, completed;
  int64_t ticks, rebatches;
  double bytes_in_use;
  double field_pairs, force_pairs;
  double busy_ms;            /* wall time spent in mf_server_step */
} mf_server_stats;

typedef struct mf_server mf_server;

mf_status mf_server_create(const mf_server_config* cfg, mf_server** out);
mf_status mf_server_destroy(mf_server* s);
/* Queues a copy of the scene.  MF_ERR_BUDGET if it alone exceeds the budget. */
mf_status mf_server_submit(mf_server* s, const mf_scene_desc* scene, int64_t* request_id);
/* One tick; *active gets the requests that ran, *completed those retired.
 * *tick_ms (may be NULL) gets the tick's wall time.  mf_server_stats.ticks
 * counts the ticks in which the batch took a timestep.  With only FMM
 * requests running and none finished, a tick waits about 0.5 ms. */
mf_status mf_server_step(mf_server* s, int32_t* active, int32_t* completed, double* tick_ms);
/* state: 0 queued, 1 running, 2 done, 3 failed (its error was returned by
 * the mf_server_step that found it).  *latency_ms: submit to done (done only). */
mf_status mf_server_poll(mf_server* s, int64_t request_id, int32_t* state, int32_t* steps_done,
                         double* latency_ms);
/* Final MF_Q_POSITIONS, MF_Q_VELOCITY, MF_Q_M, MF_Q_B_OVER_MU0 or MF_Q_FORCE of a
 * done request, host AoS [n][3]. */
mf_status mf_server_result(mf_server* s, int64_t request_id, int32_t quantity, float* dst);
mf_status mf_server_get_stats(mf_server* s, mf_server_stats* out);
/* Wall time (ms) of each timestep a request has taken so far, oldest first:
 * for a batch member, its tick from the start until its step was done on the
 * device (a rebatch in that tick included); for a request above 65,536
 * particles (run by the FMM on a host thread and stream of its own), each
 * timestep until its stream was idle.  Copies min(count, capacity) values;
 * *count gets the number of steps taken. */
mf_status mf_server_step_times(mf_server* s, int64_t request_id, double* ms, int32_t capacity, int32_t* count);

/* mf_direct_field without any device allocation.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc -- hosts that
 * have handed the device's whole memory budget to their own pool allocator,
 * or loops that cannot take cudaMalloc's device-wide synchronisation.  All
 * scratch (about 11.5 MiB: packed copies of the inputs, FP64 partial sums,
 * tickets, an error word) lives in one static device array that every GPU
 * loading the library holds until the process exits.  Same arguments and
 * results as mf_direct_field; nt and ns must each be at most 65,536
 * (MF_ERR_INVALID_ARG otherwise).  The first call on a device, with that
 * device current, looks up the array's device address; make it before any
 * stream capture.  Calls share the array: calls that overlap on the GPU race
 * and must be serialised by the caller.  Returns after the results are
 * written (synchronises `stream`). */
mf_status mf_direct_field_noalloc(const float* targets, int64_t nt, const float* sources,
                                  const float* charges, int64_t ns, float h, float* results, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MF_GB300_H */
