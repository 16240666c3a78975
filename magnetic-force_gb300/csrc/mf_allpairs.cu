// mf_allpairs.cu -- plans, scratch and launches of the all-pairs kernel.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>

#include <atomic>
#include <vector>
#include "mf_internal.h"

namespace mfgb {

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }
const char* last_error_cstr() { return g_last_error.c_str(); }

mf_status fail(mf_status s, const std::string& msg) {
  g_last_error = msg;
  return s;
}

mf_status cuda_fail(cudaError_t e, const char* what) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s failed: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
  g_last_error = buf;
  if (e == cudaErrorMemoryAllocation) return MF_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return MF_ERR_UNSUPPORTED;
  return MF_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// DevBuf / Scratch
// ---------------------------------------------------------------------------
namespace {
// Parked frees.  Never destroyed: device buffers owned by static objects of
// other files may be released at process exit, after this file's statics.
struct Parked {
  std::mutex mu;
  std::vector<std::pair<void*, size_t>> dev;
  std::vector<void*> host;
};
Parked& parked() {
  static Parked* p = new Parked();
  return *p;
}
std::atomic<int> g_defer{0};
std::atomic<size_t> g_deferred_bytes{0};
}  // namespace

void device_free(void* p, size_t bytes) {
  if (!p) return;
  if (g_defer.load() > 0) {
    Parked& k = parked();
    std::lock_guard<std::mutex> lk(k.mu);
    k.dev.emplace_back(p, bytes);
    g_deferred_bytes += bytes;
    return;
  }
  cudaFree(p);
}

void pinned_free(void* p) {
  if (!p) return;
  if (g_defer.load() > 0) {
    Parked& k = parked();
    std::lock_guard<std::mutex> lk(k.mu);
    k.host.push_back(p);
    return;
  }
  cudaFreeHost(p);
}

void defer_frees(bool on) { g_defer += on ? 1 : -1; }
size_t deferred_bytes() { return g_deferred_bytes.load(); }

void flush_deferred_frees() {
  std::vector<std::pair<void*, size_t>> dev;
  std::vector<void*> host;
  {
    Parked& k = parked();
    std::lock_guard<std::mutex> lk(k.mu);
    dev.swap(k.dev);
    host.swap(k.host);
    g_deferred_bytes = 0;
  }
  for (auto& d : dev) cudaFree(d.first);
  for (void* h : host) cudaFreeHost(h);
}

mf_status DevBuf::reserve(size_t want, bool keep, bool zero) {
  if (want == 0) want = 16;
  if (want <= bytes) return MF_OK;
  void* p = nullptr;
  cudaError_t ea = cudaMalloc(&p, want);
  if (ea == cudaErrorMemoryAllocation && deferred_bytes() > 0) {
    cudaGetLastError();  // clear the allocation error, then retry with the parked frees done
    flush_deferred_frees();
    ea = cudaMalloc(&p, want);
  }
  if (ea != cudaSuccess) return cuda_fail(ea, "cudaMalloc");
  size_t kept = 0;
  if (keep && ptr && bytes) {
    cudaError_t e = cudaMemcpy(p, ptr, bytes, cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) {
      cudaFree(p);
      return cuda_fail(e, "cudaMemcpy(grow)");
    }
    kept = bytes;
  }
  if (zero) {
    cudaError_t e = cudaMemset(static_cast<char*>(p) + kept, 0, want - kept);
    if (e != cudaSuccess) {
      cudaFree(p);
      return cuda_fail(e, "cudaMemset(grow)");
    }
  }
  release();
  ptr = p;
  bytes = want;
  return MF_OK;
}

mf_status Scratch::ensure(size_t partial_doubles, size_t n_counters) {
  MF_TRY(partials.reserve_grow(partial_doubles * sizeof(double)));
  MF_TRY(counters.reserve_grow(n_counters * sizeof(int32_t), /*keep=*/true, /*zero=*/true));
  MF_TRY(err.reserve(16, true, true));
  return MF_OK;
}

mf_status Scratch::check(cudaStream_t st) {
  if (!err.ptr) return MF_OK;
  int32_t host = 0;
  MF_CUDA_TRY(cudaMemcpyAsync(&host, err.ptr, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  MF_CUDA_TRY(cudaStreamSynchronize(st));
  if (host != 0) {
    // Leave the scratch in its between-launches state again.
    MF_CUDA_TRY(cudaMemsetAsync(err.ptr, 0, err.bytes, st));
    if (counters.ptr) MF_CUDA_TRY(cudaMemsetAsync(counters.ptr, 0, counters.bytes, st));
    MF_CUDA_TRY(cudaStreamSynchronize(st));
    char buf[128];
    snprintf(buf, sizeof(buf), "kernel wait ran out (device error %d); results of that launch are invalid",
             int(host));
    return fail(MF_ERR_TIMEOUT, buf);
  }
  return MF_OK;
}

// ---------------------------------------------------------------------------
// Device facts
// ---------------------------------------------------------------------------
int current_device() {
  int d = 0;
  cudaGetDevice(&d);
  return d;
}

int device_sms(int device) {
  static std::mutex mu;
  static int cache[64] = {};
  std::lock_guard<std::mutex> lk(mu);
  if (device < 0 || device >= 64) return 1;
  if (!cache[device]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    cache[device] = v > 0 ? v : 1;
  }
  return cache[device];
}

// ---------------------------------------------------------------------------
// Kernel selection
// ---------------------------------------------------------------------------
template <class Real, Body B>
struct BodyOf;
template <class Real>
struct BodyOf<Real, Body::Field> {
  using type = FieldBody<Real>;
};
template <class Real>
struct BodyOf<Real, Body::Force> {
  using type = ForceBody<Real>;
};
template <class Real>
struct BodyOf<Real, Body::Tensor> {
  using type = TensorBody<Real>;
};
template <>
struct BodyOf<float, Body::FieldF2> {
  using type = FieldF2Body;
};
template <>
struct BodyOf<float, Body::ForceF2> {
  using type = ForceF2Body;
};

// Packed two-source bodies exist in FP32 only.
template <class Real>
constexpr bool has_f2() {
  return std::is_same<Real, float>::value;
}

// Launch configuration: FP32 shaped bodies take shape S of kShapeTable;
// the tensor body and FP64 keep KCfg (shape 0 only).
template <class Real, Body B, int S, bool kShaped = std::is_same<Real, float>::value && B != Body::Tensor>
struct LCfg : KCfg<Real, B> {};
template <class Real, Body B, int S>
struct LCfg<Real, B, S, true> {
  static constexpr int TPB = kShapeTable[S].tpb, TPT = kShapeTable[S].tpt, TILE = kShapeTable[S].tile;
  static constexpr int STAGES = 3, kOut = KCfg<Real, B>::kOut;
};

template <class Real, Body B, int S = 0>
struct Launcher {
  using C = LCfg<Real, B, S>;
  using BT = typename BodyOf<Real, B>::type;
  static_assert(BT::kOut == C::kOut, "partial-sum slots must match the body's outputs");
  static constexpr int TBT = C::TPB * C::TPT;
  static constexpr size_t kSmem = size_t(C::STAGES) * StageLayout<Real, C::TILE>::kBytes;

  static auto kernel() { return allpairs_kernel<Real, BT, C::TPB, C::TPT, C::TILE, C::STAGES>; }

  // Resident CTAs per device (occupancy x SMs); sets the smem attribute once per device.
  static int max_grid(int device) {
    static std::mutex mu;
    static int cache[64] = {};
    std::lock_guard<std::mutex> lk(mu);
    if (device < 0 || device >= 64) device = 0;
    if (!cache[device]) {
      auto k = kernel();
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmem));
      int per_sm = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, C::TPB, kSmem);
      if (per_sm < 1) per_sm = 1;
      cache[device] = per_sm * device_sms(device);
    }
    return cache[device];
  }

  static mf_status launch(const Plan<Real>& plan, const LaunchIO<Real>& io, double* partials,
                          int32_t* counters, int32_t* err, cudaStream_t st) {
    if (plan.total_steps <= 0) return MF_OK;
    const int dev = current_device();
    const int64_t g = std::min<int64_t>(plan.total_steps, max_grid(dev));
    AllPairsArgs<Real> a;
    memset(&a, 0, sizeof(a));
    a.scenes = plan.d_scenes.template as<SceneDesc<Real>>();
    a.n_scenes = plan.n_scenes;
    a.total_steps = plan.total_steps;
    a.tpos = io.tpos;
    a.tmom = io.tmom;
    a.spos = io.spos;
    a.smom = io.smom;
    for (int k = 0; k < 9; ++k) {
      a.out[k] = io.out[k];
      a.rext[k] = io.rext[k];
    }
    a.out4 = io.out4;
    a.add4 = io.add4;
    a.add4b = io.add4b;
    a.naive_quirks = io.naive_quirks;
    a.done_flags = io.done_flags;
    a.done_stride = io.done_stride;
    a.corr4 = io.corr4;
    a.done_count = io.done_count;
    a.done_total = io.done_total;
    a.partials = partials;
    a.counters = counters;
    a.err = err;
    a.stage_wait_debug = stage_wait_debug();
    kernel()<<<unsigned(g), C::TPB, kSmem, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "allpairs_kernel launch");
    return MF_OK;
  }

  static void needs(const Plan<Real>& plan, size_t* pd, size_t* nc) {
    const int64_t g = std::min<int64_t>(plan.total_steps, max_grid(current_device()));
    *pd = size_t(g) * 2 * TBT * C::kOut;
    *nc = size_t(plan.total_tb);
  }
};

template <class Real>
static void cfg_of(Body b, int* tile, int* tbt, int shape) {
  if (std::is_same<Real, float>::value && shaped(b)) {
    const Shape& sh = kShapeTable[shape];
    *tile = sh.tile;
    *tbt = sh.tpb * sh.tpt;
    return;
  }
  switch (b) {
    case Body::Field:
      *tile = KCfg<Real, Body::Field>::TILE;
      *tbt = KCfg<Real, Body::Field>::TPB * KCfg<Real, Body::Field>::TPT;
      break;
    case Body::Force:
      *tile = KCfg<Real, Body::Force>::TILE;
      *tbt = KCfg<Real, Body::Force>::TPB * KCfg<Real, Body::Force>::TPT;
      break;
    case Body::Tensor:
      *tile = KCfg<Real, Body::Tensor>::TILE;
      *tbt = KCfg<Real, Body::Tensor>::TPB * KCfg<Real, Body::Tensor>::TPT;
      break;
    case Body::FieldF2:
      *tile = KCfg<float, Body::FieldF2>::TILE;
      *tbt = KCfg<float, Body::FieldF2>::TPB * KCfg<float, Body::FieldF2>::TPT;
      break;
    case Body::ForceF2:
      *tile = KCfg<float, Body::ForceF2>::TILE;
      *tbt = KCfg<float, Body::ForceF2>::TPB * KCfg<float, Body::ForceF2>::TPT;
      break;
  }
}

template <class Real>
void fill_scene_coefs(const SceneSpec& s, SceneDesc<Real>& d) {
  d.pc = make_pair_consts<Real>(s.h);
  d.scale = Real(s.scale);
  d.coef_add = Real(s.coef_add);
  d.coef_add2 = Real(s.coef_add2);
  for (int k = 0; k < 3; ++k) d.cvec[k] = Real(s.cvec[k]);
}

template <class Real>
mf_status build_plan(Body body, const std::vector<SceneSpec>& specs, Plan<Real>& plan, int shape) {
  if constexpr (std::is_same<Real, float>::value)
    if (shape == kShapeSym) return build_sym_plan(body, specs, plan);
  if (shape < 0 || shape >= kShapes || (shape != 0 && !(std::is_same<Real, float>::value && shaped(body))))
    return fail(MF_ERR_INVALID_ARG, "build_plan: bad block shape");
  int tile = 0, tbt = 0;
  cfg_of<Real>(body, &tile, &tbt, shape);
  plan.body = body;
  plan.shape = shape;
  plan.host.clear();
  plan.host.reserve(specs.size());
  int64_t step = 0, tbo = 0;
  double pairs = 0;
  for (const SceneSpec& s : specs) {
    if (s.nt <= 0 || s.ns <= 0) return fail(MF_ERR_INVALID_ARG, "build_plan: empty scene");
    if (!(s.h > 0.0)) return fail(MF_ERR_INVALID_ARG, "build_plan: smoothing length must be > 0");
    SceneDesc<Real> d;
    memset(&d, 0, sizeof(d));
    d.t_off = s.t_off;
    d.nt = s.nt;
    d.s_off = s.s_off;
    d.ns = s.ns;
    d.n_tiles = int32_t((s.ns + tile - 1) / tile);
    d.n_tb = int32_t((s.nt + tbt - 1) / tbt);
    d.step_off = step;
    d.tb_off = tbo;
    d.flag_index = s.flag_index >= 0 ? s.flag_index : int32_t(plan.host.size());
    fill_scene_coefs(s, d);
    step += int64_t(d.n_tiles) * d.n_tb;
    tbo += d.n_tb;
    pairs += double(s.nt) * double(s.ns);
    plan.host.push_back(d);
  }
  plan.total_steps = step;
  plan.total_tb = tbo;
  plan.n_scenes = int32_t(plan.host.size());
  plan.pairs = pairs;
  plan.evals = pairs;
  const size_t bytes = plan.host.size() * sizeof(SceneDesc<Real>);
  MF_TRY(plan.d_scenes.reserve_grow(bytes));
  if (bytes) MF_CUDA_TRY(cudaMemcpy(plan.d_scenes.ptr, plan.host.data(), bytes, cudaMemcpyHostToDevice));
  return MF_OK;
}

template <class Real>
mf_status refresh_plan_coefs(const std::vector<SceneSpec>& specs, Plan<Real>& plan) {
  if (specs.size() != plan.host.size()) return fail(MF_ERR_INVALID_ARG, "refresh_plan_coefs: size");
  for (size_t i = 0; i < specs.size(); ++i) fill_scene_coefs(specs[i], plan.host[i]);
  const size_t bytes = plan.host.size() * sizeof(SceneDesc<Real>);
  if (bytes) MF_CUDA_TRY(cudaMemcpy(plan.d_scenes.ptr, plan.host.data(), bytes, cudaMemcpyHostToDevice));
  return MF_OK;
}

// Shape dispatch: FP32 shaped bodies on plan.shape, everything else shape 0.
template <class Real, Body B>
struct Shaped {
  static void needs(const Plan<Real>& plan, size_t* pd, size_t* nc) {
    if constexpr (std::is_same<Real, float>::value && B != Body::Tensor) {
      switch (plan.shape) {
        case 1: return Launcher<Real, B, 1>::needs(plan, pd, nc);
        case 2: return Launcher<Real, B, 2>::needs(plan, pd, nc);
        case 3: return Launcher<Real, B, 3>::needs(plan, pd, nc);
        case 4: return Launcher<Real, B, 4>::needs(plan, pd, nc);
        default: break;
      }
    }
    Launcher<Real, B, 0>::needs(plan, pd, nc);
  }
  static mf_status launch(const Plan<Real>& plan, const LaunchIO<Real>& io, double* partials, int32_t* counters,
                          int32_t* err, cudaStream_t st) {
    if constexpr (std::is_same<Real, float>::value && B != Body::Tensor) {
      switch (plan.shape) {
        case 1: return Launcher<Real, B, 1>::launch(plan, io, partials, counters, err, st);
        case 2: return Launcher<Real, B, 2>::launch(plan, io, partials, counters, err, st);
        case 3: return Launcher<Real, B, 3>::launch(plan, io, partials, counters, err, st);
        case 4: return Launcher<Real, B, 4>::launch(plan, io, partials, counters, err, st);
        default: break;
      }
    }
    return Launcher<Real, B, 0>::launch(plan, io, partials, counters, err, st);
  }
};

template <class Real>
void plan_scratch_needs(const Plan<Real>& plan, size_t* pd, size_t* nc) {
  if constexpr (std::is_same<Real, float>::value)
    if (plan.shape == kShapeSym) {
      sym_needs(plan, pd);
      *nc = 0;
      return;
    }
  switch (plan.body) {
    case Body::Field: Shaped<Real, Body::Field>::needs(plan, pd, nc); break;
    case Body::Force: Shaped<Real, Body::Force>::needs(plan, pd, nc); break;
    case Body::Tensor: Shaped<Real, Body::Tensor>::needs(plan, pd, nc); break;
    case Body::FieldF2:
      if constexpr (has_f2<Real>()) Shaped<float, Body::FieldF2>::needs(plan, pd, nc);
      break;
    case Body::ForceF2:
      if constexpr (has_f2<Real>()) Shaped<float, Body::ForceF2>::needs(plan, pd, nc);
      break;
  }
}

template <class Real>
mf_status run_plan_raw(const Plan<Real>& plan, const LaunchIO<Real>& io, double* partials, int32_t* counters,
                       int32_t* err, cudaStream_t st) {
  if constexpr (std::is_same<Real, float>::value)
    if (plan.shape == kShapeSym) return run_sym(plan, io, partials, err, st);
  switch (plan.body) {
    case Body::Field: return Shaped<Real, Body::Field>::launch(plan, io, partials, counters, err, st);
    case Body::Force: return Shaped<Real, Body::Force>::launch(plan, io, partials, counters, err, st);
    case Body::Tensor: return Shaped<Real, Body::Tensor>::launch(plan, io, partials, counters, err, st);
    case Body::FieldF2:
      if constexpr (has_f2<Real>()) return Shaped<float, Body::FieldF2>::launch(plan, io, partials, counters, err, st);
      break;
    case Body::ForceF2:
      if constexpr (has_f2<Real>()) return Shaped<float, Body::ForceF2>::launch(plan, io, partials, counters, err, st);
      break;
  }
  return fail(MF_ERR_UNSUPPORTED, "packed two-source kernels exist in FP32 only");
}

template <class Real>
mf_status run_plan(const Plan<Real>& plan, const LaunchIO<Real>& io, Scratch& scratch, cudaStream_t st) {
  size_t pd = 0, nc = 0;
  plan_scratch_needs(plan, &pd, &nc);
  MF_TRY(scratch.ensure(pd, nc));
  return run_plan_raw(plan, io, scratch.partials.as<double>(), scratch.counters.as<int32_t>(),
                      scratch.err.as<int32_t>(), st);
}

// ---------------------------------------------------------------------------
// Autotuner
// ---------------------------------------------------------------------------
namespace {
// shape kShapeSym: the launch once per unordered pair, a candidate only
// where the caller offered it (its entries are keyed apart).
struct TuneEntry {
  int shape = 0;
  int n = kShapes;  // candidates timed
  float ms[kShapes + 1] = {};
};
constexpr int kSymKey = 16;  // added to the body in the cache key when the symmetric launch was offered
std::mutex g_tune_mu;
std::map<std::tuple<int, int, uint32_t>, TuneEntry> g_tune;

int ilog2(double v) {
  int k = 0;
  while (v >= 2.0 && k < 255) {
    v *= 0.5;
    ++k;
  }
  return k;
}
const char* body_name(Body b) {
  switch (b) {
    case Body::Field: return "field";
    case Body::Force: return "force";
    case Body::Tensor: return "tensor";
    case Body::FieldF2: return "field_packed";
    case Body::ForceF2: return "force_packed";
  }
  return "?";
}
}  // namespace

uint32_t tune_class(const std::vector<SceneSpec>& specs) {
  double pairs = 0;
  for (const SceneSpec& s : specs) pairs += double(s.nt) * double(s.ns);
  return (uint32_t(ilog2(pairs)) << 8) | uint32_t(std::min(ilog2(double(specs.size())), 255));
}

int tuned_shape(Body body, uint32_t cls, bool sym_offered) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(std::make_tuple(current_device(), int(body) + (sym_offered ? kSymKey : 0), cls));
  return it == g_tune.end() ? -1 : it->second.shape;
}

int default_sym_mode() {
  static const int mode = [] {
    const char* e = getenv("MF_PAIR_SYMMETRIC");
    return (e && (e[0] == '0' || e[0] == '2') && e[1] == 0) ? e[0] - '0' : 1;
  }();
  return mode;
}

namespace {
thread_local int t_tune_override = -1;  // -1: none; else a Tune value for handles made on this thread
}

Tune default_tune_mode() {
  static const Tune mode = [] {
    const char* e = getenv("MF_AUTOTUNE");
    return (e && e[0] == '0') ? Tune::Off : Tune::OnMiss;
  }();
  if (t_tune_override >= 0 && mode != Tune::Off) return Tune(t_tune_override);
  return mode;
}

void set_thread_tune_mode(int mode) { t_tune_override = mode; }

namespace {
std::atomic<uint32_t> g_stage_wait_debug{0};
}
uint32_t stage_wait_debug() { return g_stage_wait_debug.load(std::memory_order_relaxed); }
void set_stage_wait_debug(uint32_t v) { g_stage_wait_debug.store(v, std::memory_order_relaxed); }

int default_shape(Body body, const std::vector<SceneSpec>& specs, bool allow_sym) {
  return allow_sym && body == Body::ForceF2 && sym_eligible(body, specs) ? kShapeSym : 0;
}

mf_status tuned_plan(Body body, const std::vector<SceneSpec>& specs, Plan<float>& plan, const LaunchIO<float>& io,
                     Scratch& scratch, cudaStream_t st, Tune mode, bool allow_sym) {
  const bool offer = allow_sym && sym_eligible(body, specs);
  if (mode == Tune::Off || !shaped(body)) return build_plan<float>(body, specs, plan, default_shape(body, specs, offer));
  const uint32_t cls = tune_class(specs);
  const int known = tuned_shape(body, cls, offer);
  if (known >= 0) return build_plan<float>(body, specs, plan, known);
  if (mode == Tune::CachedOnly) return build_plan<float>(body, specs, plan, default_shape(body, specs, offer));
  TuneEntry te;
  te.n = kShapes + (offer ? 1 : 0);
  float best = 1e30f;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  MF_CUDA_TRY(cudaEventCreate(&e0));
  MF_CUDA_TRY(cudaEventCreate(&e1));
  mf_status status = MF_OK;
  for (int s = 0; s < te.n && status == MF_OK; ++s) {
    Plan<float> p;
    status = build_plan<float>(body, specs, p, s);
    if (status != MF_OK) break;
    status = run_plan<float>(p, io, scratch, st);  // warm-up (grows the scratch outside the timing)
    if (status != MF_OK) break;
    cudaEventRecord(e0, st);
    for (int r = 0; r < 2 && status == MF_OK; ++r) status = run_plan<float>(p, io, scratch, st);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) status = cuda_fail(cudaGetLastError(), "autotune timing");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    te.ms[s] = ms * 0.5f;
    if (te.ms[s] < best) {
      best = te.ms[s];
      te.shape = s;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  MF_TRY(status);
  MF_TRY(scratch.check(st));
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[std::make_tuple(current_device(), int(body) + (offer ? kSymKey : 0), cls)] = te;
  }
  return build_plan<float>(body, specs, plan, te.shape);
}

std::string autotune_report() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  std::string out;
  char line[256];
  for (const auto& kv : g_tune) {
    const TuneEntry& e = kv.second;
    const int kb = std::get<1>(kv.first);
    const char* extra = kb >= kSymKey ? "+sym" : "";
    if (e.shape == kShapeSym)
      snprintf(line, sizeof(line), "device %d %s%s pairs~2^%u scenes~2^%u: shape %d (once per unordered pair) ms",
               std::get<0>(kv.first), body_name(Body(kb % kSymKey)), extra, std::get<2>(kv.first) >> 8,
               std::get<2>(kv.first) & 255u, e.shape);
    else
      snprintf(line, sizeof(line), "device %d %s%s pairs~2^%u scenes~2^%u: shape %d (%dx%d/%d) ms",
               std::get<0>(kv.first), body_name(Body(kb % kSymKey)), extra, std::get<2>(kv.first) >> 8,
               std::get<2>(kv.first) & 255u, e.shape, kShapeTable[e.shape].tpb, kShapeTable[e.shape].tpt,
               kShapeTable[e.shape].tile);
    out += line;
    for (int s = 0; s < e.n; ++s) {
      snprintf(line, sizeof(line), " %.4f", double(e.ms[s]));
      out += line;
    }
    out += "\n";
  }
  return out;
}

#define MF_INSTANTIATE(R)                                                                                  \
  template mf_status build_plan<R>(Body, const std::vector<SceneSpec>&, Plan<R>&, int);                   \
  template void fill_scene_coefs<R>(const SceneSpec&, SceneDesc<R>&);                                     \
  template mf_status refresh_plan_coefs<R>(const std::vector<SceneSpec>&, Plan<R>&);                      \
  template void plan_scratch_needs<R>(const Plan<R>&, size_t*, size_t*);                                  \
  template mf_status run_plan<R>(const Plan<R>&, const LaunchIO<R>&, Scratch&, cudaStream_t);             \
  template mf_status run_plan_raw<R>(const Plan<R>&, const LaunchIO<R>&, double*, int32_t*, int32_t*,     \
                                     cudaStream_t);
MF_INSTANTIATE(float)
MF_INSTANTIATE(double)
#undef MF_INSTANTIATE

}  // namespace mfgb
