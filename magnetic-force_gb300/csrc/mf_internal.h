// mf_internal.h -- shared declarations of the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mf.h"
#include "mf_allpairs.cuh"

namespace mfgb {

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------
void set_last_error(const std::string& msg);
mf_status fail(mf_status s, const std::string& msg);
mf_status cuda_fail(cudaError_t e, const char* what);

#define MF_CUDA_TRY(expr)                                       \
  do {                                                          \
    cudaError_t _e = (expr);                                    \
    if (_e != cudaSuccess) return ::mfgb::cuda_fail(_e, #expr); \
  } while (0)

#define MF_TRY(expr)            \
  do {                          \
    mf_status _s = (expr);      \
    if (_s != MF_OK) return _s; \
  } while (0)

// ---------------------------------------------------------------------------
// Device buffer (owning, growable)
// ---------------------------------------------------------------------------
// Device and pinned-host frees.  cudaFree and cudaFreeHost wait for every
// stream of the device.  While deferral is on (a serving loop whose FMM
// requests keep other streams busy for tens of milliseconds at a time), frees
// are parked and done by flush_deferred_frees() at a point where that wait is
// short; a failed device allocation flushes them and retries.  Nests.
void device_free(void* p, size_t bytes);
void pinned_free(void* p);
void defer_frees(bool on);
size_t deferred_bytes();
void flush_deferred_frees();

struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : ptr(o.ptr), bytes(o.bytes) {
    o.ptr = nullptr;
    o.bytes = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      ptr = o.ptr;
      bytes = o.bytes;
      o.ptr = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (ptr) device_free(ptr, bytes);
    ptr = nullptr;
    bytes = 0;
  }
  // Ensure at least `want` bytes.  keep: preserve the old contents on growth;
  // zero: clear bytes beyond the preserved prefix.
  mf_status reserve(size_t want, bool keep = false, bool zero = false);
  // Same, with a quarter of headroom when it has to grow: for buffers sized
  // by the particles' current extent (cell and box grids), which change a
  // little every timestep and would otherwise reallocate often.
  mf_status reserve_slack(size_t want) { return want <= bytes ? MF_OK : reserve(want + want / 4 + 256); }
  // Same, at least doubling when it has to grow: for buffers whose size
  // follows a changing set of scenes (batch layouts, launch plans, scratch),
  // so that growth -- whose cudaFree waits for every stream of the device --
  // happens a logarithmic number of times.
  mf_status reserve_grow(size_t want, bool keep = false, bool zero = false) {
    return want <= bytes ? MF_OK : reserve(std::max(want, 2 * bytes), keep, zero);
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(ptr);
  }
};

// ---------------------------------------------------------------------------
// All-pairs launch configurations.
// ---------------------------------------------------------------------------
// Field / Force / Tensor: one packed record per source, exact pair branches
// (both precisions).  FieldF2 / ForceF2: FP32 pair-layout sources, two
// sources per instruction, clamped far form plus a near-field correction
// array (mf_cells.cu) added in the epilogue.
enum class Body { Field = 0, Force = 1, Tensor = 2, FieldF2 = 3, ForceF2 = 4 };

// Scene sizes from which the packed path (clamped far form + near-field
// correction) beats the exact-branch kernels.  Near pairs per particle are
// fixed by the density (~270 inside 2h, ~2100 inside 4h at h = 2 spacings)
// while far pairs grow with N, and a corrected near pair costs several far
// pairs, so small scenes stay on the exact-branch kernels.
// Force, one scene alone: 0.43 ms exact against 0.51 ms packed at 12,288
// particles, 0.70 against 0.66 at 16,384.
constexpr int64_t kPackedFieldMin = 2048;
constexpr int64_t kPackedForceMin = 14336;
// Force inside a batch: one packed launch and one correction launch serve all
// large scenes, so the packed path wins from smaller scenes on (256 scenes of
// 512..32,768 particles: 92.2 ms per step at 12,288, 89.7 ms at 4,096, flat
// below).
constexpr int64_t kBatchPackedForceMin = 4096;
// Direct entries (no tuning): the packed products once per unordered pair
// from this size on.  Measured against the best all-pairs shape at 32,768
// particles: force 0.82 against 1.04 ms; at 16,384 the all-pairs field wins
// (0.206 against 0.213 ms).
constexpr int64_t kSymDirectMin = 32768;
// FMM handles: the force's near field once per unordered box pair from this
// size on.  Measured when the force's aperture was 0.3 (its half stencil ~4x
// the partial-sum planes of 0.5): force products on the r = 0.3 cylinder
// took 84.0 against 90.2 ms for every ordered pair at 1,048,576 particles,
// but 188.6 against 128.8 at 524,288 (leaf boxes of ~330 particles there)
// and 49.3 against 35.3 at 262,144.
constexpr int64_t kSymNearMin = 1048576;

template <class Real, Body B>
struct KCfg;
// FP32: 256 threads x 2 targets, 256-source tiles, 3 stages (24 KB of smem).
template <>
struct KCfg<float, Body::Field> {
  static constexpr int TPB = 256, TPT = 2, TILE = 256, STAGES = 3, kOut = 3;
};
template <>
struct KCfg<float, Body::Force> {
  static constexpr int TPB = 256, TPT = 2, TILE = 256, STAGES = 3, kOut = 3;
};
template <>
struct KCfg<float, Body::Tensor> {
  static constexpr int TPB = 128, TPT = 1, TILE = 256, STAGES = 3, kOut = 6;
};
template <>
struct KCfg<float, Body::FieldF2> {
  static constexpr int TPB = 256, TPT = 2, TILE = 256, STAGES = 3, kOut = 3;
};
template <>
struct KCfg<float, Body::ForceF2> {
  static constexpr int TPB = 256, TPT = 2, TILE = 256, STAGES = 3, kOut = 4;
};
// FP64: 128 threads x 1 target, 128-source tiles of 32-byte records.
template <>
struct KCfg<double, Body::Field> {
  static constexpr int TPB = 128, TPT = 1, TILE = 128, STAGES = 3, kOut = 3;
};
template <>
struct KCfg<double, Body::Force> {
  static constexpr int TPB = 128, TPT = 1, TILE = 128, STAGES = 3, kOut = 3;
};
template <>
struct KCfg<double, Body::Tensor> {
  static constexpr int TPB = 128, TPT = 1, TILE = 128, STAGES = 3, kOut = 6;
};

// Block shapes of the FP32 all-pairs launches (the exact-branch Field / Force
// bodies and the packed FieldF2 / ForceF2 ones): threads per CTA, targets per
// thread, sources per staged tile.  Shape 0 is the default (the KCfg above);
// the autotuner picks among all of them per body and size class.
struct Shape {
  int tpb, tpt, tile;
};
constexpr int kShapes = 5;
constexpr Shape kShapeTable[kShapes] = {{256, 2, 256}, {128, 2, 256}, {256, 1, 256}, {128, 4, 128}, {128, 4, 256}};
inline bool shaped(Body b) { return b != Body::Tensor; }
// Shape index of the packed field / force evaluated once per unordered pair
// (mf_sympair.cu), for scenes whose targets are their sources.
constexpr int kShapeSym = kShapes;

// One scene of a launch before it is laid out in step space.  nt > 0, ns > 0.
struct SceneSpec {
  int64_t t_off, nt, s_off, ns;
  double h;
  double scale = 1.0;
  double coef_add = 0.0;   // field: coefficient of add4
  double coef_add2 = 0.0;  // field: coefficient of add4b
  double cvec[3] = {0.0, 0.0, 0.0};
  int32_t flag_index = -1; // row in done_flags (default: the scene's position in the plan)
};

// A laid-out launch: device scene table plus its step-space totals.
template <class Real>
struct Plan {
  Body body = Body::Field;
  int shape = 0;  // FP32 shaped bodies: index into kShapeTable, or kShapeSym
  int64_t total_steps = 0;
  int64_t total_tb = 0;
  int32_t n_scenes = 0;
  double pairs = 0.0;  // sum over scenes of nt * ns
  double evals = 0.0;  // pair evaluations needed: pairs, or n (n - 1) / 2 per scene when one serves both particles
  DevBuf d_scenes;
  std::vector<SceneDesc<Real>> host;  // the table as uploaded
};

// Build (and synchronously upload) a plan.  Empty scenes are rejected.
// `shape` applies to FP32 shaped bodies (0 otherwise).
template <class Real>
mf_status build_plan(Body body, const std::vector<SceneSpec>& specs, Plan<Real>& plan, int shape = 0);
// Re-upload a plan whose per-scene coefficients (scale, coef_add*, cvec) changed.
template <class Real>
mf_status refresh_plan_coefs(const std::vector<SceneSpec>& specs, Plan<Real>& plan);

// Scratch of all-pairs launches: FP64 partials, tickets, error word.
struct Scratch {
  DevBuf partials;
  DevBuf counters;
  DevBuf err;
  mf_status ensure(size_t partial_doubles, size_t n_counters);
  // Read and clear the device error word (synchronises `st`).
  mf_status check(cudaStream_t st);
};

// Pointers of one launch.
template <class Real>
struct LaunchIO {
  using R4 = typename Vec4T<Real>::type;
  const R4* tpos = nullptr;
  const R4* tmom = nullptr;
  const R4* spos = nullptr;
  const R4* smom = nullptr;
  Real* out[9] = {};
  R4* out4 = nullptr;
  const R4* add4 = nullptr;
  const R4* add4b = nullptr;
  const Real* rext[9] = {};
  int naive_quirks = 0;
  const double* done_flags = nullptr;
  int done_stride = 0;
  const R4* corr4 = nullptr;
  const int32_t* done_count = nullptr;
  int32_t done_total = 0;
};

// A scene's epilogue coefficients in its launch table.
template <class Real>
void fill_scene_coefs(const SceneSpec& s, SceneDesc<Real>& d);

// The packed field / force products evaluated once per unordered pair
// (mf_sympair.cu; plans of shape kShapeSym, built and run through build_plan
// and run_plan): packed FP32 bodies on scenes whose targets are their
// sources, each starting at an even index.  A launch is the pair kernel plus
// the per-particle finish with the body's epilogue; the scratch holds FP32
// block sums, 3 floats per particle of a block per ordered block pair.
bool sym_eligible(Body body, const std::vector<SceneSpec>& specs);
mf_status build_sym_plan(Body body, const std::vector<SceneSpec>& specs, Plan<float>& plan);
void sym_needs(const Plan<float>& plan, size_t* partial_doubles);
mf_status run_sym(const Plan<float>& plan, const LaunchIO<float>& io, double* partials, int32_t* err,
                  cudaStream_t st);

// The field and the Kelvin force of the same dipoles once per unordered pair
// in one launch (mf_sympair.cu).  The plan is a packed field plan (its
// epilogue coefficients) cut into the fused kernel's own blocks; io is the
// field's (pair-layout sources and targets, correction, addends).  The
// field's epilogue is applied; the force's pair sums, for those dipoles and
// not yet corrected or scaled, go to gsum[3 n] (FP64).
// run_sym_force_from_sums then applies the force's epilogue (a force plan's
// scenes, io with the force's dipoles M, correction and outputs) to gsum
// scaled by c^2, for dipoles M = c times those of the fused launch: c^2 = c2
// for every scene, or, where rows is given, c = float(rows[flag_index *
// row_stride + c_index]) per scene; where kept is given, only the scenes
// whose kept[flag_index] is non-zero are written.
mf_status build_symff_plan(const std::vector<SceneSpec>& specs, Plan<float>& plan);
void symff_needs(const Plan<float>& plan, size_t* partial_doubles);
mf_status run_symff(const Plan<float>& plan, const LaunchIO<float>& io, double* partials, double* gsum,
                    int32_t* err, cudaStream_t st);
mf_status run_sym_force_from_sums(const Plan<float>& plan, const LaunchIO<float>& io, const double* gsum, double c2,
                                  const double* kept, const double* rows, int row_stride, int c_index, int32_t* err,
                                  cudaStream_t st);
// Default of MF_OPT_FUSED_PRODUCTS for new handles, and whether batches fuse
// (MF_FUSED_PRODUCTS=0|1|2 in the environment; 1 when unset).
int default_fused_mode();

// Scratch sizes a plan needs.
template <class Real>
void plan_scratch_needs(const Plan<Real>& plan, size_t* partial_doubles, size_t* n_counters);

// Launch a plan on `st`.  Grows `scratch` if needed (allocation happens only
// outside stream capture; a captured launch must have been sized before).
template <class Real>
mf_status run_plan(const Plan<Real>& plan, const LaunchIO<Real>& io, Scratch& scratch, cudaStream_t st);

// Same, with caller-provided scratch pointers (no allocation at all).
template <class Real>
mf_status run_plan_raw(const Plan<Real>& plan, const LaunchIO<Real>& io, double* partials,
                       int32_t* counters, int32_t* err, cudaStream_t st);

// Builds an FP32 plan with the autotuned block shape.  On the first launch of
// a (device, body, size class) every shape is timed on this plan's own data
// (`io`, whose outputs are overwritten): one warm-up and two timed launches
// each, CUDA events on `st`; the fastest is cached.  Off, or a body without
// shapes, builds shape 0; CachedOnly uses a cached choice and never times.
enum class Tune { Off = 0, OnMiss = 1, CachedOnly = 2 };
//
// allow_sym: where the scenes are eligible (sym_eligible), the launch once per
// unordered pair (kShapeSym) is one more candidate; without tuning it is the
// default for the packed force.
mf_status tuned_plan(Body body, const std::vector<SceneSpec>& specs, Plan<float>& plan, const LaunchIO<float>& io,
                     Scratch& scratch, cudaStream_t st, Tune mode, bool allow_sym = false);
// The shape a plan gets without tuning.
int default_shape(Body body, const std::vector<SceneSpec>& specs, bool allow_sym);
// Default tuning mode of new handles and batches: OnMiss unless the
// environment sets MF_AUTOTUNE=0.
Tune default_tune_mode();
// Handles and batches created on the calling thread from now on start in
// this tune mode (a Tune value; -1 restores the process default).  The
// process default MF_AUTOTUNE=0 still wins.
void set_thread_tune_mode(int mode);
// Debug setting carried by every all-pairs and once-per-pair launch
// (AllPairsArgs::stage_wait_debug): 0 the default staging-wait bound, k > 0
// staging waits give up after k - 1 try-waits.  Process-wide.
uint32_t stage_wait_debug();
void set_stage_wait_debug(uint32_t v);
// Default pair-symmetric mode of new handles and batches (MF_OPT_PAIR_SYMMETRIC:
// 0 never, 1 tuned, 2 always): 1 unless the environment sets MF_PAIR_SYMMETRIC.
int default_sym_mode();

int device_sms(int device);
int current_device();

// ---------------------------------------------------------------------------
// Autotuner of the block shapes (mf_allpairs.cu)
// ---------------------------------------------------------------------------
// Size class of a launch: log2 of its pairs and of its scene count.
uint32_t tune_class(const std::vector<SceneSpec>& specs);
// Shape for (device, body, class): the cached choice, or -1 when not tuned yet.
int tuned_shape(Body body, uint32_t cls, bool sym_offered);  // kShapeSym when the pair-symmetric launch won
// Text table of the tuned choices (device, body, class, ms per shape).
std::string autotune_report();

// ---------------------------------------------------------------------------
// Uniform-grid cell lists and the near-field correction pass (mf_cells.cu)
// ---------------------------------------------------------------------------
struct CellGrid {
  float ox, oy, oz, inv_cs;  // grid origin and 1 / cell size
  int32_t nx, ny, nz;
  int32_t reach_field;       // cells to scan each way for r < 2h
  int32_t reach_force;       // cells to scan each way for r <= 4h
  int32_t pad;
  int64_t cell_off;          // first cell of this scene in the global arrays
  int64_t p_off, n;          // particle range of the scene
  int64_t k_off;             // particles of the scenes before this one
  PairConsts<float> pc;
};

struct CellSceneSpec {
  int64_t p_off, n;
  double h;
};

class CellList {
 public:
  // Bins the particles of every scene into cells of edge >= 2h; particles of
  // a cell are listed in increasing index order (deterministic sums).
  // Synchronises `st` once (the bounding boxes are read on the host).
  mf_status build(const float4* pos4, const std::vector<CellSceneSpec>& scenes, cudaStream_t st,
                  double margin_h = 0.0);
  // Re-bins moved particles on the grids of the last build (no host
  // synchronisation, so it can be captured in a CUDA graph).  Particles that
  // left a grid are binned into its border cells, which keeps every
  // neighbour within reach; build() with a margin (in units of h) leaves room.
  mf_status rebin(const float4* pos4, cudaStream_t st);
  // corr_i = sum over j within 2h (resp. 4h) of [exact pair term - the
  // clamped far term the packed all-pairs loop gave that pair], in the
  // all-pairs kernels' output units.  Targets = sources = the binned set.
  // done_flags (per-scene solver rows) skip stopped scenes; done_count /
  // done_total make the launch a no-op once every scene has stopped.
  mf_status field_correction(const float4* pos4, const float4* mom4, float4* corr, cudaStream_t st,
                             const double* done_flags = nullptr, int done_stride = 0,
                             const int32_t* done_count = nullptr, int done_total = 0) const;
  mf_status force_correction(const float4* pos4, const float4* mom4, float4* corr, cudaStream_t st) const;
  // Scenes (by build order) whose field / force use the exact-branch kernels
  // and so need no correction.
  mf_status set_skips(const std::vector<int32_t>& field, const std::vector<int32_t>& force);
  // Field correction at separate targets tpos4[0..nt) (single-scene lists).
  mf_status field_correction_at(const float4* tpos4, int64_t nt, const float4* pos4, const float4* mom4,
                                float4* corr, cudaStream_t st) const;
  // Force-tensor correction at separate targets: corr2[2i] = (xx, yy, zz, 0),
  // corr2[2i + 1] = (xy, xz, yz, 0).
  mf_status tensor_correction_at(const float4* tpos4, int64_t nt, const float4* pos4, const float4* mom4,
                                 float4* corr2, cudaStream_t st) const;
  int64_t particles() const { return n_total_; }
  int64_t cells() const { return n_cells_; }
  const std::vector<CellGrid>& grids() const { return host_grids_; }
  // Bounding box of scene s at the last build (lo xyz, hi xyz; no margin).
  const double* bbox(int s) const { return host_bbox_.data() + 6 * size_t(s); }

 private:
  DevBuf grids_, bbox_, cell_start_, cursor_, perm_, perm_tmp_, cell_of_;
  DevBuf scan_tiles_;  // tile sums / offsets of the cell-count scan
  DevBuf skip_field_, skip_force_;  // per scene: 1 = not on the packed path
  bool skip_field_on_ = false, skip_force_on_ = false;  // a list is in use
  DevBuf spos_, smom_;              // positions and dipoles in cell order (per correction)
  std::vector<CellGrid> host_grids_;
  std::vector<double> host_bbox_;
  int64_t n_total_ = 0, n_cells_ = 0;
  int32_t n_scenes_ = 0;
};

// ---------------------------------------------------------------------------
// Uniform-octree FMM for one scene (mf_fmm.cu)
// ---------------------------------------------------------------------------
struct FmmConfig {
  int order = 8;         // expansion terms per degree as the reference counts them (n < P); degree P-1
  double theta = 0.5;    // multipole acceptance aperture (FMMOptions.hpp:56-78)
  // Leaf level: the deepest with at least this many particles per box on
  // average over the grid's boxes.  Levels differ by 8x in occupancy, and
  // boxes of ~15 at the deeper level measured faster than ~120 at the coarser
  // one (196,608-particle cylinder, force / field ms: 17.0 / 5.9 against
  // 26.1 / 6.2), boxes of ~10 slower than ~80 (1,048,576: 122 / 36 against
  // 90 / 18), so 12 keeps the mean occupancy in [12, 96).  Scenes that fill
  // their bounding box sparsely (spheres) gained most: 196,608 particles in a
  // sphere, 17 / 4 ms against 65 / 24 at the former default of 64.
  int leaf_min = 12;
  // Aperture of the Kelvin force and force-tensor products, which take the
  // Hessian of the local expansion: it converges one degree later than the
  // field, and inside a magnetised body the far boxes' Hessians cancel to a
  // small net force, so the same truncation error is ~40x larger relative to
  // the result.  Measured against FP64 direct sums on a cylinder of 1,048,576
  // particles: at P = 8, 1.3e-4 at 0.5, 9.3e-6 at 0.36, 4.7e-6 at 0.32 (field
  // at 0.5: 3.3e-6); at P = 9, 4.8e-6 at 0.36; at P = 10, 2.2e-5 at 0.48,
  // 6.6e-6 at 0.44, 3.6e-6 at 0.4.  On the same cylinder's shape at 262,144
  // particles P = 10 gives 1.2e-5 at 0.48 and 6.4e-6 at 0.44, on spheres of
  // 150,000-262,144 particles 2.9-3.6e-6 at 0.44.  0.44 holds every one of
  // these within 1e-5 with a margin of 1.5x.  The force uses min(theta, this).
  double theta_force = 0.44;
  double force_theta() const { return theta_force < theta ? theta_force : theta; }
  // Expansion order of the Kelvin force and force-tensor products (0: the
  // field's).  Orders above the field's let the force take a wider aperture
  // for the same error, so fewer near pairs: at the 1,048,576-particle
  // cylinder the force product takes 66 ms at P = 8 and 0.32, 51 at P = 9 and
  // 0.36, 34 at P = 10 and 0.44, all within 7e-6 of the oracle.
  int order_force = 10;
  int force_order() const { return order_force > 0 ? order_force : order; }
  // Whether the force products need lists or expansions of their own.
  bool force_tree() const { return force_theta() < theta || force_order() != order; }
};

// One level of the uniform box grid (level 0 is one box holding the scene).
struct FmmLevel {
  int32_t nx, ny, nz, pad;
  int64_t nbox;      // nx * ny * nz
  int64_t box_off;   // first box of this level in the per-box arrays of all levels
  float side;        // box edge
  float ox, oy, oz;  // grid origin (shared by all levels)
};

struct FmmStats {
  int32_t levels = 0, leaf_level = 0, degree = 0, pad = 0;
  int64_t leaf_boxes = 0, occupied_leaves = 0;
  double p2p_pairs = 0;   // executed near-field pairs per product (real sources)
  double p2p_self_pairs = 0;  // of those, pairs within one leaf box (sum of n^2)
  double m2l_per_product = 0;
  int32_t max_leaf = 0, near_rows = 0;
};

class Fmm {
 public:
  // Builds the box grids, bins the particles of pos4[0..n) into leaf boxes
  // and lays out the interaction lists.  Synchronises `st` (the bounding box
  // and the leaf occupancy are read on the host).
  // tpos4[0..nt): separate targets (null: the targets are the sources).
  // bbox (lo xyz, hi xyz) must hold the sources and the targets.
  mf_status build(const float4* pos4, int64_t n, const float4* tpos4, int64_t nt, double h, const double* bbox,
                  const FmmConfig& cfg, cudaStream_t st);
  // out = epilogue(far field + near field + corr4) of the field (kForce false)
  // or Kelvin force (kForce true) of the dipoles smom at every target (every
  // particle when the targets are the sources; `a.tpos` holds the targets).  `a`
  // carries the epilogue's pointers (tpos, tmom, out, out4, add4, add4b, rext,
  // corr4, err) exactly as for an all-pairs launch; `sc` its coefficients.
  // `done`: a solver stop flag; every launch is a no-op once it is non-zero.
  // marks (optional, 4 events): recorded before and after the far-field
  // stages (gather .. L2L), then before and after the near-field kernel.
  // kind: 0 field, 1 Kelvin force, 2 force tensor (6 entries through the
  // tensor epilogue; a.corr4 then holds two records per target).
  // sym_near (Kelvin force, targets = sources): the near field once per
  // unordered box pair (k_fmm_near_sym, partial sums per source and writer
  // box offset, ~1 KB per particle), read back by the near-field kernel.
  mf_status product(int kind, const float4* pos4, const float4* smom, const AllPairsArgs<float>& a,
                    const SceneDesc<float>& sc, cudaStream_t st, const double* done,
                    cudaEvent_t* marks = nullptr, bool sym_near = false);
  // Near-field pair evaluations of one force product with sym_near.
  double sym_near_evals() { return 0.5 * (stats().p2p_pairs + stats().p2p_self_pairs); }
  // Shape and work of the last build (waits for its device counts).
  const FmmStats& stats();
  int launches_per_product() const { return launches_; }
  Fmm() = default;
  Fmm(const Fmm&) = delete;
  Fmm& operator=(const Fmm&) = delete;
  ~Fmm();

 private:
  template <int Q>
  mf_status product_q(int kind, const float4* pos4, const float4* smom, const AllPairsArgs<float>& a,
                      const SceneDesc<float>& sc, cudaStream_t st, const double* done, cudaEvent_t* marks,
                      bool sym_near);
  FmmConfig cfg_;
  FmmStats stats_;
  int degree_ = 5;
  int64_t n_ = 0, n_slots_ = 0;
  std::vector<FmmLevel> lv_;
  std::vector<int64_t> list_off_, list_cnt_;  // per (level, class)
  std::vector<int32_t> chunks_;               // M2L splits per level
  int n_rows_ = 0;
  int n_hrows_ = 0, n_off_ = 0;  // half-stencil rows and their box offsets (sym_near)
  int launches_ = 0;
  DevBuf cell_of_, cnt_, start_, cursor_, perm_tmp_, perm_, pos2s_, mom2s_;
  DevBuf occ_, mcoef_, lcoef_, lpart_, lists_, rows_, dtab_, stat_, lofs_;
  DevBuf hrows_, npart_;  // half-stencil rows; near-field partial sums (sym_near)
  // Separate targets: occupancy per level and leaf binning.
  DevBuf tocc_, tcell_of_, tstart_, tcursor_, tperm_tmp_, tperm_;
  bool separate_ = false;
  int64_t nt_ = 0;
  std::vector<int4> host_list_, host_rows_, host_hrows_;  // as last uploaded
  std::vector<int32_t> host_dkey_;           // degree and offsets of the uploaded derivative table
  unsigned long long* hstat_ = nullptr;      // pinned: near pairs, largest leaf, M2L count, occupied leaves, in-box pairs
  cudaEvent_t stat_ev_ = nullptr;
  bool stat_pending_ = false;
  std::vector<float> host_dt_;
  std::vector<int64_t> host_lofs_;
};

// Packed records -> pair layout (sources 2p, 2p+1 as (x_a, x_b, y_a, y_b),
// (z_a, z_b, 0, 0)); a missing partner (odd n) is written as zeros.
void to_pairs(const float4* src, float4* dst, int64_t n, cudaStream_t st, const int32_t* done_count = nullptr,
              int done_total = 0);

}  // namespace mfgb

// Element-wise equality of CUDA's int4 (host-side comparison of uploaded tables).
inline bool operator==(const int4& a, const int4& b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }
inline bool operator!=(const int4& a, const int4& b) { return !(a == b); }

