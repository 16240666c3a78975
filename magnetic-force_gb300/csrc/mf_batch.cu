// mf_batch.cu -- many independent scenes advanced together (mf_batch_* in mf.h).
//
// Every scene is the reference's problem (its own particles, h, V, chi and
// uniform external field).  Scenes are laid out back to back (each starting
// at an even index, so the pair-layout source tiles never straddle two
// scenes) and every stage of the step is one launch for all of them:
//   * the all-pairs field / force kernels take all scenes in one flat step
//     space (mf_allpairs.cuh), so small and large scenes share the SMs evenly;
//   * the near-field correction runs over one cell list holding every scene;
//   * the CG vector updates and FP64 inner products reduce per scene
//     (blockIdx.y = scene) with the scalar steps applied on the device;
//   * a scene whose solve has stopped is skipped by every later launch, and
//     a launch does nothing once all scenes have stopped, so a fixed number of
//     iterations can be captured in a CUDA graph.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "mf_internal.h"
#include "mf_vec.cuh"

namespace mfgb {
namespace {

__global__ void k_batch_init_rows(double* scal, int n, double tol, double maxit, int32_t* done_count) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    double* row = scal + int64_t(s) * kScal;
    for (int k = 0; k < S_CONST_C; ++k) row[k] = 0.0;
    row[S_TOL] = tol;
    row[S_MAXIT] = maxit;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *done_count = 0;
}

// After a solve: a packed-force scene whose solve made no CG update kept its
// b, so its force comes from the sums the fused residual launch kept
// (kept[s] = 1); the others take their own force product (kept[s] = 0).
// kept_count counts the first kind: the force product does nothing when
// every scene kept its b.
__global__ void k_batch_mark_kept(const double* __restrict__ scal, const int32_t* __restrict__ ids, int n_ids,
                                  double* __restrict__ kept, int32_t* __restrict__ kept_count) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n_ids; j += gridDim.x * blockDim.x) {
    const int s = ids[j];
    const bool k = scal[int64_t(s) * kScal + S_ITERS] == 0.0;
    kept[s] = k ? 1.0 : 0.0;
    if (k) atomicAdd(kept_count, 1);
  }
}

// M = c b per scene (the dipoles of the force pass).
struct BPublish {
  static constexpr int kN = 0;
  const float4* b;
  float4* mom;
  __device__ bool skip(const double*) const { return false; }
  __device__ void elem(int64_t i, double*, const double* row) const {
    const float c = float(row[S_CONST_C]);
    const float4 v = b[i];
    mom[i] = make_float4(c * v.x, c * v.y, c * v.z, 0.f);
  }
  __device__ void finish(const double*, double*) const {}
};

// Symplectic Euler with the scene's 1 / mass.
struct BIntegrate {
  static constexpr int kN = 0;
  const float* fx;
  const float* fy;
  const float* fz;
  float4* vel;
  float4* pos;
  float dt;
  __device__ bool skip(const double*) const { return false; }
  __device__ void elem(int64_t i, double*, const double* row) const {
    const float im = float(row[S_CONST_INVM]);
    float4 v = vel[i], p = pos[i];
    v.x += dt * fx[i] * im;
    v.y += dt * fy[i] * im;
    v.z += dt * fz[i] * im;
    p.x += dt * v.x;
    p.y += dt * v.y;
    p.z += dt * v.z;
    vel[i] = v;
    pos[i] = p;
  }
  __device__ void finish(const double*, double*) const {}
};

}  // namespace

class Batch {
 public:
  ~Batch() {
    if (gexec_) cudaGraphExecDestroy(gexec_);
    if (own_stream_) cudaStreamDestroy(own_stream_);
    if (pinned_) pinned_free(pinned_);
  }

  // Device-resident state of one scene: n positions, velocities and warm
  // starts (packed float4 records).
  struct SceneState {
    float4* pos;
    float4* vel;
    float4* b;
  };

  // Scenes from host positions (dev == nullptr), or from device-resident
  // state (dev[s] for scene s; the descriptors' pos pointers are unused).
  mf_status init(const mf_scene_desc* d, int n, int device, const SceneState* dev = nullptr,
               Tune tune = default_tune_mode()) {
    tune_ = tune;
    if (n <= 0 || !d) return fail(MF_ERR_INVALID_ARG, "no scenes");
    device_ = device;
    sms_ = device_sms(device);
    int64_t off = 0, max_n = 0;
    for (int s = 0; s < n; ++s) {
      const mf_scene_desc& x = d[s];
      if (x.n <= 0 || (!dev && !x.pos)) return fail(MF_ERR_INVALID_ARG, "scene without particles");
      if (!(x.h > 0.f) || !(x.volume > 0.f) || !std::isfinite(x.h) || !std::isfinite(x.volume))
        return fail(MF_ERR_INVALID_ARG, "scene h and volume must be finite and > 0");
      if (!std::isfinite(x.chi) || x.chi <= -1.f) return fail(MF_ERR_INVALID_ARG, "scene chi must be > -1");
      if (!dev)
        for (int64_t i = 0; i < 3 * x.n; ++i)
          if (!std::isfinite(x.pos[i])) return fail(MF_ERR_INVALID_ARG, "non-finite particle position");
      SI si;
      si.off = off;
      si.n = x.n;
      si.h = x.h;
      si.V = x.volume;
      si.chi = x.chi;
      for (int k = 0; k < 3; ++k) si.H0[k] = x.H0[k];
      sc_.push_back(si);
      off += x.n + (x.n & 1);  // next scene starts at an even index
      max_n = std::max(max_n, x.n);
    }
    n_alloc_ = off;
    if (!own_stream_) {
      int lo = 0, hi = 0;  // numerically lower is the higher priority
      MF_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
      MF_CUDA_TRY(cudaStreamCreateWithPriority(&own_stream_, cudaStreamNonBlocking, priority_ ? hi : lo));
    }
    st_ = own_stream_;
    if (!pinned_) MF_CUDA_TRY(cudaMallocHost(&pinned_, 64));

    // Buffers may come from an earlier layout (adopt_buffers): clear them.
    const size_t v4 = size_t(n_alloc_ + 2) * sizeof(float4);
    for (DevBuf* b : {&pos4_, &pos2_, &vel4_, &b4_, &r4_, &p4_, &q4_, &hext4_, &mom4_, &mom2_, &corr_}) {
      MF_TRY(b->reserve_grow(v4));
      MF_CUDA_TRY(cudaMemsetAsync(b->ptr, 0, v4, st_));
    }
    MF_TRY(fs_.reserve_grow(size_t(3 * n_alloc_) * sizeof(float)));
    MF_CUDA_TRY(cudaMemsetAsync(fs_.ptr, 0, size_t(3 * n_alloc_) * sizeof(float), st_));
    MF_CUDA_TRY(cudaStreamSynchronize(st_));

    // Positions, external field, solver constants.
    std::vector<float4> hp(size_t(n_alloc_ + 2), make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<float4> hh(size_t(n_alloc_ + 2), make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<double> rows(size_t(n) * kScal, 0.0);
    std::vector<VecRange> rg(static_cast<size_t>(n));
    for (int s = 0; s < n; ++s) {
      const SI& si = sc_[size_t(s)];
      for (int64_t i = 0; i < si.n; ++i) {
        if (!dev) hp[size_t(si.off + i)] = make_float4(d[s].pos[3 * i], d[s].pos[3 * i + 1], d[s].pos[3 * i + 2], 0.f);
        hh[size_t(si.off + i)] = make_float4(si.H0[0], si.H0[1], si.H0[2], 0.f);
      }
      // A scene with an odd count borrows its dummy partner's slot at its end:
      // park it on the scene's first particle (zero dipole, contributes nothing).
      if ((si.n & 1) && !dev) hp[size_t(si.off + si.n)] = hp[size_t(si.off)];
      double* row = &rows[size_t(s) * kScal];
      row[S_CONST_C] = si.V * si.chi / (1.0 + si.chi);
      row[S_CONST_INVM] = 1.0 / si.V;
      for (int k = 0; k < 3; ++k) row[S_CONST_H0 + k] = si.H0[k];
      rg[size_t(s)] = VecRange{si.off, si.n};
    }
    MF_CUDA_TRY(cudaMemcpy(pos4_.ptr, hp.data(), v4, cudaMemcpyHostToDevice));
    if (dev) {
      for (int s = 0; s < n; ++s) {
        const SI& si = sc_[size_t(s)];
        const size_t bytes = size_t(si.n) * sizeof(float4);
        MF_CUDA_TRY(cudaMemcpyAsync(pos4_.as<float4>() + si.off, dev[s].pos, bytes, cudaMemcpyDeviceToDevice, st_));
        MF_CUDA_TRY(cudaMemcpyAsync(vel4_.as<float4>() + si.off, dev[s].vel, bytes, cudaMemcpyDeviceToDevice, st_));
        MF_CUDA_TRY(cudaMemcpyAsync(b4_.as<float4>() + si.off, dev[s].b, bytes, cudaMemcpyDeviceToDevice, st_));
        if (si.n & 1)
          MF_CUDA_TRY(cudaMemcpyAsync(pos4_.as<float4>() + si.off + si.n, dev[s].pos, sizeof(float4),
                                      cudaMemcpyDeviceToDevice, st_));
      }
      MF_CUDA_TRY(cudaStreamSynchronize(st_));
    }
    MF_CUDA_TRY(cudaMemcpy(hext4_.ptr, hh.data(), v4, cudaMemcpyHostToDevice));
    MF_TRY(scal_.reserve_grow(rows.size() * sizeof(double)));
    MF_CUDA_TRY(cudaMemcpy(scal_.ptr, rows.data(), rows.size() * sizeof(double), cudaMemcpyHostToDevice));
    MF_TRY(ranges_.reserve_grow(rg.size() * sizeof(VecRange)));
    MF_CUDA_TRY(cudaMemcpy(ranges_.ptr, rg.data(), rg.size() * sizeof(VecRange), cudaMemcpyHostToDevice));
    red_gx_ = int(std::min<int64_t>((max_n + 255) / 256, 16));
    MF_TRY(red_part_.reserve_grow(size_t(n) * red_gx_ * 2 * sizeof(double)));
    MF_TRY(red_tickets_.reserve_grow(size_t(n) * sizeof(int32_t)));
    MF_CUDA_TRY(cudaMemsetAsync(red_tickets_.ptr, 0, size_t(n) * sizeof(int32_t), st_));
    MF_TRY(done_count_.reserve(16));
    MF_CUDA_TRY(cudaMemsetAsync(done_count_.ptr, 0, 16, st_));

    // Launch plans, one scene table per kind of product and path: [0] the
    // exact-branch kernels for scenes below kPacked*Min, [1] the packed
    // kernels plus near-field correction for the larger ones.
    std::vector<SceneSpec> resid[2], cgq[2], force[2];
    std::vector<int32_t> skip_field, skip_force;
    for (size_t k = 0; k < sc_.size(); ++k) {
      const SI& si = sc_[k];
      SceneSpec b;
      b.t_off = si.off;
      b.nt = si.n;
      b.s_off = si.off;
      b.ns = si.n;
      b.h = si.h;
      b.flag_index = int32_t(k);
      const int pf = si.n >= kPackedFieldMin ? 1 : 0;
      const int pg = si.n >= kBatchPackedForceMin ? 1 : 0;
      const double c = si.V * si.chi / (1.0 + si.chi);
      SceneSpec r = b;  // r = c G b + Hext - b
      r.scale = c;
      r.coef_add = 1.0;
      r.coef_add2 = -1.0;
      resid[pf].push_back(r);
      SceneSpec q = b;  // q = p - c G p
      q.scale = -c;
      q.coef_add = 1.0;
      cgq[pf].push_back(q);
      force[pg].push_back(b);
      skip_field.push_back(pf ? 0 : 1);
      skip_force.push_back(pg ? 0 : 1);
      pairs_ += double(si.n) * double(si.n);
    }
    for (int p = 0; p < 2; ++p) {
      const Body fb = p ? Body::FieldF2 : Body::Field;
      const Body gb = p ? Body::ForceF2 : Body::Force;
      // Block shapes from the autotuner, timed on these scenes (the tuning
      // launches write the q and force scratch only).
      LaunchIO<float> io;
      io.tpos = pos4_.as<float4>();
      io.spos = p ? pos2_.as<float4>() : pos4_.as<float4>();
      io.smom = p ? mom2_.as<float4>() : mom4_.as<float4>();
      io.corr4 = p ? corr_.as<float4>() : nullptr;
      io.out4 = q4_.as<float4>();
      LaunchIO<float> ig = io;
      ig.out4 = nullptr;
      ig.tmom = mom4_.as<float4>();
      for (int k = 0; k < 3; ++k) ig.out[k] = fs_.as<float>() + int64_t(k) * n_alloc_;
      // The packed products may run once per unordered pair (kShapeSym):
      // the tuner's candidate, and without tuning the force's default.
      // (MF_PAIR_SYMMETRIC=0 never, 2 always).
      auto pick = [&](Body body, const std::vector<SceneSpec>& specs, Plan<float>& plan,
                      const LaunchIO<float>& lio) -> mf_status {
        if (sym_mode_ == 2 && sym_eligible(body, specs)) return build_plan<float>(body, specs, plan, kShapeSym);
        return tuned_plan(body, specs, plan, lio, scr_, st_, tune_, sym_mode_ == 1);
      };
      if (!resid[p].empty()) {
        MF_TRY(pick(fb, cgq[p], plan_cgq_[p], io));
        MF_TRY(build_plan<float>(fb, resid[p], plan_resid_[p], plan_cgq_[p].shape));
      }
      if (!force[p].empty()) MF_TRY(pick(gb, force[p], plan_force_[p], ig));
      for (const Plan<float>* pl : {&plan_resid_[p], &plan_cgq_[p], &plan_force_[p]}) {
        if (pl->n_scenes == 0) continue;
        size_t pd = 0, nc = 0;
        plan_scratch_needs(*pl, &pd, &nc);
        MF_TRY(scr_.ensure(pd, nc));
      }
    }

    // The packed scenes' residual and force in one launch where both run once
    // per unordered pair (MF_FUSED_PRODUCTS=0 never): plan_ff_ covers the
    // packed field scenes; the force sums of those below the packed force
    // threshold are not used.
    ff_ = ff_valid_ = false;
    n_ff_ids_ = 0;
    if (default_fused_mode() != 0 && plan_resid_[1].n_scenes && plan_force_[1].n_scenes &&
        plan_resid_[1].shape == kShapeSym && plan_force_[1].shape == kShapeSym) {
      MF_TRY(build_symff_plan(resid[1], plan_ff_));
      size_t pd = 0;
      symff_needs(plan_ff_, &pd);
      MF_TRY(scr_.ensure(pd, 0));
      MF_TRY(ff_sum_.reserve_grow(size_t(3 * n_alloc_) * sizeof(double)));
      std::vector<int32_t> ids;
      for (const SceneDesc<float>& x : plan_force_[1].host) ids.push_back(x.flag_index);
      MF_TRY(ff_ids_.reserve_grow(ids.size() * sizeof(int32_t)));
      MF_CUDA_TRY(cudaMemcpy(ff_ids_.ptr, ids.data(), ids.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
      MF_TRY(kept_.reserve_grow(size_t(n) * sizeof(double)));
      MF_CUDA_TRY(cudaMemsetAsync(kept_.ptr, 0, size_t(n) * sizeof(double), st_));
      MF_TRY(kept_count_.reserve_grow(16));
      n_ff_ids_ = int(ids.size());
      ff_ = true;
    }

    std::vector<CellSceneSpec> cs;
    for (const SI& si : sc_) cs.push_back(CellSceneSpec{si.off, si.n, si.h});
    MF_TRY(cells_.build(pos4_.as<float4>(), cs, st_, /*margin_h=*/2.0));
    MF_TRY(cells_.set_skips(skip_field, skip_force));
    to_pairs(pos4_.as<float4>(), pos2_.as<float4>(), n_alloc_, st_);
    MF_CUDA_TRY(cudaGetLastError());
    MF_CUDA_TRY(cudaStreamSynchronize(st_));
    iters_base_.assign(size_t(n), 0.0);
    return MF_OK;
  }

  void set_stream(cudaStream_t s) {
    st_ = s ? s : own_stream_;
    drop_graph();
  }
  // Before init: create the batch's own stream at the device's highest
  // priority (the served loop's shared batch, ahead of its FMM requests).
  void set_high_priority() { priority_ = true; }

  // Takes over another batch's device buffers, stream and pinned word (a
  // serving rebatch, with `o` idle): init() then grows only what is too
  // small, so a membership change usually frees and allocates nothing --
  // cudaFree would wait for every stream of the device, the FMM requests'
  // included.
  void adopt_buffers(Batch& o) {
    std::swap(own_stream_, o.own_stream_);
    st_ = own_stream_;
    std::swap(pinned_, o.pinned_);
    for (auto pr : {std::make_pair(&pos4_, &o.pos4_), std::make_pair(&pos2_, &o.pos2_),
                    std::make_pair(&vel4_, &o.vel4_), std::make_pair(&b4_, &o.b4_), std::make_pair(&r4_, &o.r4_),
                    std::make_pair(&p4_, &o.p4_), std::make_pair(&q4_, &o.q4_), std::make_pair(&hext4_, &o.hext4_),
                    std::make_pair(&mom4_, &o.mom4_), std::make_pair(&mom2_, &o.mom2_),
                    std::make_pair(&corr_, &o.corr_), std::make_pair(&fs_, &o.fs_),
                    std::make_pair(&scal_, &o.scal_), std::make_pair(&ranges_, &o.ranges_),
                    std::make_pair(&red_part_, &o.red_part_), std::make_pair(&red_tickets_, &o.red_tickets_),
                    std::make_pair(&done_count_, &o.done_count_), std::make_pair(&ff_sum_, &o.ff_sum_),
                    std::make_pair(&ff_ids_, &o.ff_ids_), std::make_pair(&kept_, &o.kept_),
                    std::make_pair(&kept_count_, &o.kept_count_)})
      *pr.first = std::move(*pr.second);
    scr_ = std::move(o.scr_);
    cells_ = std::move(o.cells_);
    for (int p = 0; p < 2; ++p) {  // launch plans: their device tables
      for (auto pr : {std::make_pair(&plan_resid_[p], &o.plan_resid_[p]), std::make_pair(&plan_cgq_[p], &o.plan_cgq_[p]),
                      std::make_pair(&plan_force_[p], &o.plan_force_[p])}) {
        *pr.first = std::move(*pr.second);
        pr.first->n_scenes = 0;
        pr.first->host.clear();
      }
    }
    plan_ff_ = std::move(o.plan_ff_);
    plan_ff_.n_scenes = 0;
    plan_ff_.host.clear();

  }
  int scenes() const { return int(sc_.size()); }

  // ---- solve -----------------------------------------------------------------
  mf_status solve(int64_t max_iter, double tol, bool host_checks) {
    const int n = scenes();
    ff_valid_ = false;
    k_batch_init_rows<<<(n + 127) / 128, 128, 0, st_>>>(scal_.as<double>(), n, tol, double(max_iter),
                                                        done_count_.as<int32_t>());
    MF_CUDA_TRY(cudaGetLastError());
    ++ctr_.kernel_launches;
    // r = c G b + Hext - b (with the packed scenes' force of b, where fused)
    MF_TRY(field(plan_resid_, b4_.as<float4>(), r4_.as<float4>(), hext4_.as<float4>(), b4_.as<float4>(), false, ff_));
    MF_TRY(reduce(CgStart<float4>{r4_.as<float4>(), p4_.as<float4>(), hext4_.as<float4>(), done_count_.as<int32_t>()}));
    ++solves_;
    for (int64_t it = 0; it < max_iter; ++it) {
      MF_TRY(field(plan_cgq_, p4_.as<float4>(), q4_.as<float4>(), p4_.as<float4>(), nullptr, true));
      MF_TRY(reduce(CgPq<float4>{p4_.as<float4>(), q4_.as<float4>(), done_count_.as<int32_t>()}));
      MF_TRY(reduce(CgUpdate<float, float4>{b4_.as<float4>(), r4_.as<float4>(), p4_.as<float4>(), q4_.as<float4>(),
                                            done_count_.as<int32_t>()}));
      MF_TRY(reduce(CgDirection<float, float4>{r4_.as<float4>(), p4_.as<float4>()}));
      if (host_checks && (it % 4 == 3 || it + 1 == max_iter)) {
        MF_CUDA_TRY(cudaMemcpyAsync(pinned_, done_count_.ptr, sizeof(int32_t), cudaMemcpyDeviceToHost, st_));
        MF_CUDA_TRY(cudaStreamSynchronize(st_));
        if (*static_cast<int32_t*>(pinned_) >= n) break;
      }
    }
    MF_TRY(reduce(BPublish{b4_.as<float4>(), mom4_.as<float4>()}));
    ff_valid_ = ff_;
    return MF_OK;
  }

  mf_status eval_force() {
    LaunchIO<float> io;
    io.tpos = pos4_.as<float4>();
    io.tmom = mom4_.as<float4>();
    float* F = fs_.as<float>();
    for (int k = 0; k < 3; ++k) io.out[k] = F + int64_t(k) * n_alloc_;
    if (plan_force_[0].n_scenes) {  // small scenes: exact branches, records as sources
      LaunchIO<float> s = io;
      s.spos = pos4_.as<float4>();
      s.smom = mom4_.as<float4>();
      MF_TRY(run_plan<float>(plan_force_[0], s, scr_, st_));
      ctr_.kernel_launches += 1;
    }
    if (plan_force_[1].n_scenes) {  // large scenes: packed pairs + correction
      to_pairs(mom4_.as<float4>(), mom2_.as<float4>(), n_alloc_, st_);
      MF_TRY(cells_.force_correction(pos4_.as<float4>(), mom4_.as<float4>(), corr_.as<float4>(), st_));
      io.spos = pos2_.as<float4>();
      io.smom = mom2_.as<float4>();
      io.corr4 = corr_.as<float4>();
      if (ff_ && ff_valid_) {
        // Scenes whose solve kept b: the force from the fused launch's sums;
        // the others (skipped by the first) through their force product.
        MF_CUDA_TRY(cudaMemsetAsync(kept_count_.ptr, 0, sizeof(int32_t), st_));
        k_batch_mark_kept<<<(n_ff_ids_ + 127) / 128, 128, 0, st_>>>(scal_.as<double>(), ff_ids_.as<int32_t>(),
                                                                     n_ff_ids_, kept_.as<double>(),
                                                                     kept_count_.as<int32_t>());
        MF_CUDA_TRY(cudaGetLastError());
        LaunchIO<float> g = io;
        g.done_flags = kept_.as<double>();
        g.done_stride = 1;
        g.done_count = kept_count_.as<int32_t>();
        g.done_total = n_ff_ids_;
        MF_TRY(run_plan<float>(plan_force_[1], g, scr_, st_));
        MF_TRY(run_sym_force_from_sums(plan_force_[1], io, ff_sum_.as<double>(), 0.0, kept_.as<double>(),
                                       scal_.as<double>(), kScal, S_CONST_C, scr_.err.as<int32_t>(), st_));
        ctr_.kernel_launches += 6;
      } else {
        MF_TRY(run_plan<float>(plan_force_[1], io, scr_, st_));
        ctr_.kernel_launches += plan_force_[1].shape == kShapeSym ? 4 : 3;
      }
    }
    ctr_.force_passes += 1;
    ctr_.force_pairs += pairs_;
    return MF_OK;
  }

  mf_status step(double dt, int iters, double tol) {
    MF_TRY(solve(iters, tol, false));
    MF_TRY(eval_force());
    const float* F = fs_.as<float>();
    MF_TRY(reduce(BIntegrate{F, F + n_alloc_, F + 2 * n_alloc_, vel4_.as<float4>(), pos4_.as<float4>(), float(dt)}));
    ff_valid_ = false;  // the kept sums belong to the old positions
    MF_TRY(cells_.rebin(pos4_.as<float4>(), st_));
    to_pairs(pos4_.as<float4>(), pos2_.as<float4>(), n_alloc_, st_);
    MF_CUDA_TRY(cudaGetLastError());
    ctr_.kernel_launches += 8;
    return MF_OK;
  }

  mf_status advance(double dt, int steps, int iters, double tol, bool graph) {
    if (steps < 0 || iters < 0) return fail(MF_ERR_INVALID_ARG, "negative steps or iterations");
    if (!graph) {
      for (int k = 0; k < steps; ++k) MF_TRY(step(dt, iters, tol));
      MF_CUDA_TRY(cudaStreamSynchronize(st_));
      MF_TRY(scr_.check(st_));
      return MF_OK;
    }
    if (!gexec_ || g_dt_ != dt || g_iters_ != iters || g_tol_ != tol) {
      drop_graph();
      cudaGraph_t gr = nullptr;
      MF_CUDA_TRY(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
      const mf_counters saved = ctr_;
      mf_status s = step(dt, iters, tol);
      cudaError_t e = cudaStreamEndCapture(st_, &gr);
      launches_per_step_ = ctr_.kernel_launches - saved.kernel_launches;
      force_per_step_ = ctr_.force_passes - saved.force_passes;
      ctr_ = saved;  // capture records the launches; the replays count them
      if (s != MF_OK) {
        if (gr) cudaGraphDestroy(gr);
        return s;
      }
      if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
      e = cudaGraphInstantiate(&gexec_, gr, 0);
      cudaGraphDestroy(gr);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
      g_dt_ = dt;
      g_iters_ = iters;
      g_tol_ = tol;
    }
    for (int k = 0; k < steps; ++k) {
      MF_CUDA_TRY(cudaGraphLaunch(gexec_, st_));
      ++solves_;
      ctr_.kernel_launches += launches_per_step_;
      ctr_.force_passes += force_per_step_;
      ctr_.force_pairs += double(force_per_step_) * pairs_;
    }
    MF_CUDA_TRY(cudaStreamSynchronize(st_));
    MF_TRY(scr_.check(st_));
    return MF_OK;
  }

  // ---- results ---------------------------------------------------------------
  mf_status get(int scene, int q, float* dst) {
    if (scene < 0 || scene >= scenes()) return fail(MF_ERR_INVALID_ARG, "scene index out of range");
    if (!dst) return fail(MF_ERR_INVALID_ARG, "dst is NULL");
    const SI& si = sc_[size_t(scene)];
    MF_CUDA_TRY(cudaStreamSynchronize(st_));
    if (q == MF_Q_FORCE) {
      std::vector<float> t(size_t(si.n));
      for (int k = 0; k < 3; ++k) {
        MF_CUDA_TRY(cudaMemcpy(t.data(), fs_.as<float>() + int64_t(k) * n_alloc_ + si.off,
                               size_t(si.n) * sizeof(float), cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < si.n; ++i) dst[3 * i + k] = t[size_t(i)];
      }
      return MF_OK;
    }
    const DevBuf* src = nullptr;
    switch (q) {
      case MF_Q_POSITIONS: src = &pos4_; break;
      case MF_Q_M: src = &mom4_; break;
      case MF_Q_B_OVER_MU0: src = &b4_; break;
      case MF_Q_HEXT: src = &hext4_; break;
      case MF_Q_VELOCITY: src = &vel4_; break;
      default: return fail(MF_ERR_INVALID_ARG, "quantity not kept for batched scenes");
    }
    std::vector<float4> t(size_t(si.n));
    MF_CUDA_TRY(cudaMemcpy(t.data(), src->as<float4>() + si.off, size_t(si.n) * sizeof(float4),
                           cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < si.n; ++i) {
      dst[3 * i] = t[size_t(i)].x;
      dst[3 * i + 1] = t[size_t(i)].y;
      dst[3 * i + 2] = t[size_t(i)].z;
    }
    return MF_OK;
  }

  mf_status solver_state(double* relres, double* iters) {
    const int n = scenes();
    std::vector<double> rows(size_t(n) * kScal);
    MF_CUDA_TRY(cudaStreamSynchronize(st_));
    MF_CUDA_TRY(cudaMemcpy(rows.data(), scal_.ptr, rows.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int s = 0; s < n; ++s) {
      if (relres) relres[s] = rows[size_t(s) * kScal + S_RELRES];
      if (iters) iters[s] = rows[size_t(s) * kScal + S_ITERS];
    }
    return MF_OK;
  }

  // Field pairs actually evaluated: every solve runs one residual product for
  // every scene, and each CG iteration a product for the scenes still going.
  mf_status counters(mf_counters* c) {
    const int n = scenes();
    std::vector<double> rows(size_t(n) * kScal);
    MF_CUDA_TRY(cudaStreamSynchronize(st_));
    MF_CUDA_TRY(cudaMemcpy(rows.data(), scal_.ptr, rows.size() * sizeof(double), cudaMemcpyDeviceToHost));
    double fp = 0;
    int64_t products = 0;
    for (int s = 0; s < n; ++s) {
      const double nn = double(sc_[size_t(s)].n) * double(sc_[size_t(s)].n);
      const double it = rows[size_t(s) * kScal + S_ITERS_TOTAL] - iters_base_[s];
      fp += nn * (double(solves_ - solves_base_) + it);
      products = std::max<int64_t>(products, int64_t(it));
    }
    *c = ctr_;
    c->field_pairs = fp;
    c->field_products = products + (solves_ - solves_base_);
    return MF_OK;
  }

  mf_status reset_counters() {
    const int n = scenes();
    std::vector<double> rows(size_t(n) * kScal);
    MF_CUDA_TRY(cudaStreamSynchronize(st_));
    MF_CUDA_TRY(cudaMemcpy(rows.data(), scal_.ptr, rows.size() * sizeof(double), cudaMemcpyDeviceToHost));
    iters_base_.assign(size_t(n), 0.0);
    for (int s = 0; s < n; ++s) iters_base_[size_t(s)] = rows[size_t(s) * kScal + S_ITERS_TOTAL];
    solves_base_ = solves_;
    ctr_ = mf_counters{};
    return MF_OK;
  }

  // Copies scene s's positions, velocities and warm start out (device to device).
  mf_status export_state(int s, const SceneState& dst) {
    const SI& si = sc_[size_t(s)];
    const size_t bytes = size_t(si.n) * sizeof(float4);
    MF_CUDA_TRY(cudaMemcpyAsync(dst.pos, pos4_.as<float4>() + si.off, bytes, cudaMemcpyDeviceToDevice, st_));
    MF_CUDA_TRY(cudaMemcpyAsync(dst.vel, vel4_.as<float4>() + si.off, bytes, cudaMemcpyDeviceToDevice, st_));
    MF_CUDA_TRY(cudaMemcpyAsync(dst.b, b4_.as<float4>() + si.off, bytes, cudaMemcpyDeviceToDevice, st_));
    return MF_OK;
  }

  cudaStream_t stream() const { return st_; }
  int device_ = 0;

 private:
  struct SI {
    int64_t off, n;
    double h, V, chi;
    float H0[3];
  };

  mf_status field(const Plan<float>* plans, const float4* src_mom, float4* out4, const float4* add4,
                  const float4* add4b, bool skip_done, bool fused = false) {
    const int n = scenes();
    const int32_t* dc = skip_done ? done_count_.as<int32_t>() : nullptr;
    LaunchIO<float> io;
    io.tpos = pos4_.as<float4>();
    io.out4 = out4;
    io.add4 = add4;
    io.add4b = add4b;
    if (skip_done) {
      io.done_flags = scal_.as<double>();
      io.done_stride = kScal;
      io.done_count = dc;
      io.done_total = n;
    }
    if (plans[0].n_scenes) {  // small scenes: exact branches, records as sources
      LaunchIO<float> s = io;
      s.spos = pos4_.as<float4>();
      s.smom = src_mom;
      MF_TRY(run_plan<float>(plans[0], s, scr_, st_));
      ctr_.kernel_launches += 1;
    }
    if (plans[1].n_scenes) {  // large scenes: packed pairs + correction
      to_pairs(src_mom, mom2_.as<float4>(), n_alloc_, st_, dc, n);
      MF_TRY(cells_.field_correction(pos4_.as<float4>(), src_mom, corr_.as<float4>(), st_,
                                     skip_done ? scal_.as<double>() : nullptr, kScal, dc, n));
      io.spos = pos2_.as<float4>();
      io.smom = mom2_.as<float4>();
      io.corr4 = corr_.as<float4>();
      if (fused) {
        MF_TRY(run_symff(plan_ff_, io, scr_.partials.as<double>(), ff_sum_.as<double>(), scr_.err.as<int32_t>(), st_));
        ctr_.kernel_launches += 4;
      } else {
        MF_TRY(run_plan<float>(plans[1], io, scr_, st_));
        ctr_.kernel_launches += plans[1].shape == kShapeSym ? 4 : 3;
      }
    }
    return MF_OK;
  }

  template <class Op>
  mf_status reduce(const Op& op) {
    const dim3 grid{static_cast<unsigned>(red_gx_), static_cast<unsigned>(scenes())};
    reduce_kernel<Op><<<grid, 256, 0, st_>>>(op, ranges_.as<VecRange>(), scal_.as<double>(),
                                             red_part_.as<double>(), red_tickets_.as<int32_t>());
    MF_CUDA_TRY(cudaGetLastError());
    ++ctr_.kernel_launches;
    return MF_OK;
  }

  void drop_graph() {
    if (gexec_) cudaGraphExecDestroy(gexec_);
    gexec_ = nullptr;
  }

  std::vector<SI> sc_;
  int64_t n_alloc_ = 0;
  double pairs_ = 0;
  int sms_ = 1;
  int red_gx_ = 1;
  cudaStream_t st_ = nullptr, own_stream_ = nullptr;
  bool priority_ = false;
  void* pinned_ = nullptr;
  DevBuf pos4_, pos2_, vel4_, b4_, r4_, p4_, q4_, hext4_, mom4_, mom2_, corr_, fs_;
  DevBuf scal_, ranges_, red_part_, red_tickets_, done_count_;
  Plan<float> plan_resid_[2], plan_cgq_[2], plan_force_[2];  // [0] exact branches, [1] packed
  // The packed scenes' residual and force in one launch (run_symff): its
  // plan, the force sums it keeps (for b), the packed force scenes and their
  // kept flags (k_batch_mark_kept).  ff_valid_: the kept sums are those of
  // the current b and positions.
  Plan<float> plan_ff_;
  DevBuf ff_sum_, ff_ids_, kept_, kept_count_;
  int n_ff_ids_ = 0;
  bool ff_ = false, ff_valid_ = false;
  Tune tune_ = Tune::OnMiss;
  int sym_mode_ = default_sym_mode();  // pair-symmetric products: 0 never, 1 tuned, 2 always
  Scratch scr_;
  CellList cells_;
  mf_counters ctr_ = {};
  int64_t solves_ = 0, solves_base_ = 0;
  std::vector<double> iters_base_;
  cudaGraphExec_t gexec_ = nullptr;
  double g_dt_ = 0, g_tol_ = 0;
  int g_iters_ = -1;
  int64_t launches_per_step_ = 0, force_per_step_ = 0;
};

// ---------------------------------------------------------------------------
// Serving with continuous batching.
// ---------------------------------------------------------------------------
// Requests above this many particles run as their own solver handle (field
// products through the FMM at P = 8, the Kelvin force as the handle's
// automatic choice picks it), each on a host thread and a stream of its own, so their
// kernels overlap the batch's on the device and their host-side waits never
// hold up the serving loop; smaller ones join the all-pairs batch.
constexpr int64_t kServeFmmMin = 65536;

class Server {
  using Clock = std::chrono::steady_clock;

 public:
  // Frees are deferred while the server lives (device_free): a rebatch or a
  // finished FMM request would otherwise wait in cudaFree for the other FMM
  // requests' kernels (measured: rebatch ticks of 125-800 ms against under
  // 1 ms with no FMM request running).  They are done at the end of a tick
  // with no FMM request in flight, or past kDeferredMax bytes.
  static constexpr size_t kDeferredMax = size_t(8) << 30;
  Server() { defer_frees(true); }
  ~Server() {
    for (auto& kv : reqs_)
      if (kv.second.job) kv.second.job->cancel.store(true);
    for (auto& kv : reqs_)
      if (kv.second.job && kv.second.job->th.joinable()) kv.second.job->th.join();
    batch_.reset();
    pool_.clear();
    for (auto& kv : reqs_) kv.second.state.release();
    defer_frees(false);
    flush_deferred_frees();
  }

  mf_status init(const mf_server_config& c) {
    if (!(c.hbm_budget_bytes > 0) || c.max_active <= 0 || c.steps_per_request <= 0 || c.iters_per_step < 0 ||
        !(c.rel_tol > 0) || !std::isfinite(c.dt))
      return fail(MF_ERR_INVALID_ARG, "bad server configuration");
    cfg_ = c;
    return MF_OK;
  }

  // Device bytes a running request holds.  Batch member: its own state (3
  // records per particle) plus its share of the batch buffers, cell list and
  // scratch.  FMM request: a solver handle's vectors, published arrays, cell
  // list and octree.
  static double need_bytes(int64_t n) {
    // FMM requests: the handle's state and trees, 1.5 KB per particle of
    // near-field partial sums where the force's near field runs once per box
    // pair ((1 + 125 half-stencil offsets) x 3 floats at the force's aperture
    // 0.44), and, where the force is the all-pairs product once per unordered
    // pair, its block sums (12 KB per ordered pair of 1,024-particle blocks).
    if (n > kServeFmmMin) {
      const double nb = std::ceil(double(n) / 1024.0);
      return double(n) * (720.0 + 1536.0) + 12288.0 * nb * nb + 64.0 * 1024 * 1024;
    }
    return double(n) * 320.0 + 4.0 * 1024 * 1024;
  }

  mf_status submit(const mf_scene_desc& d, int64_t* id) {
    if (d.n <= 0 || !d.pos) return fail(MF_ERR_INVALID_ARG, "scene without particles");
    // The same checks as a batch layout or a solver handle makes, here so a
    // bad request is refused alone instead of failing a rebuild or its thread.
    if (!(d.h > 0.f) || !(d.volume > 0.f) || !std::isfinite(d.h) || !std::isfinite(d.volume))
      return fail(MF_ERR_INVALID_ARG, "scene h and volume must be finite and > 0");
    if (!std::isfinite(d.chi) || d.chi <= -1.f) return fail(MF_ERR_INVALID_ARG, "scene chi must be > -1");
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(d.H0[k])) return fail(MF_ERR_INVALID_ARG, "scene H0 must be finite");
    if (need_bytes(d.n) > cfg_.hbm_budget_bytes) return fail(MF_ERR_BUDGET, "scene exceeds the HBM budget");
    for (int64_t i = 0; i < 3 * d.n; ++i)
      if (!std::isfinite(d.pos[i])) return fail(MF_ERR_INVALID_ARG, "non-finite particle position");
    Req r;
    r.id = next_id_++;
    r.d = d;
    r.pos.assign(d.pos, d.pos + 3 * d.n);
    r.d.pos = nullptr;
    r.t_submit = Clock::now();
    queue_.push_back(r.id);
    reqs_.emplace(r.id, std::move(r));
    ++stats_.submitted;
    if (id) *id = reqs_.rbegin()->first;
    return MF_OK;
  }

  mf_status step(int32_t* n_active, int32_t* n_completed, double* tick_ms) {
    const auto t0 = Clock::now();
    int completed = 0;
    // Admit in arrival order while the budget and the slots allow.
    while (!queue_.empty() && int(active_.size()) < cfg_.max_active) {
      Req& r = reqs_.at(queue_.front());
      const double need = need_bytes(r.d.n);
      if (used_ + need > cfg_.hbm_budget_bytes) break;
      if (r.d.n > kServeFmmMin) {
        r.job.reset(new FmmJob());
        FmmJob* j = r.job.get();
        j->th = std::thread(fmm_worker, j, r.d, r.pos.data(), cfg_);
        used_ += need;
        r.phase = 1;
        fmm_active_.push_back(r.id);
        queue_.pop_front();
        continue;
      }
      const size_t bytes = size_t(r.d.n) * sizeof(float4);
      MF_TRY(take_state(r.state, 3 * bytes));
      std::vector<float4> p(size_t(r.d.n));
      for (int64_t i = 0; i < r.d.n; ++i) p[size_t(i)] = make_float4(r.pos[3 * i], r.pos[3 * i + 1], r.pos[3 * i + 2], 0.f);
      MF_CUDA_TRY(cudaMemcpy(r.state.ptr, p.data(), bytes, cudaMemcpyHostToDevice));
      used_ += need;
      r.phase = 1;
      active_.push_back(r.id);
      queue_.pop_front();
      dirty_ = true;
    }
    if (!active_.empty()) {
      ++stats_.ticks;
      if (dirty_) MF_TRY(rebatch());
      MF_TRY(batch_->step(cfg_.dt, cfg_.iters_per_step, cfg_.rel_tol));  // enqueued, not waited for
    }
    // FMM requests run on their own threads: retire the finished ones.
    {
      std::vector<int64_t> keep;
      for (int64_t id : fmm_active_) {
        Req& r = reqs_.at(id);
        FmmJob* j = r.job.get();
        if (!j->done.load(std::memory_order_acquire)) {
          keep.push_back(id);
          continue;
        }
        j->th.join();
        if (j->status != MF_OK) {
          const mf_status st = j->status;
          const std::string msg = "served FMM request: " + j->err;
          r.job.reset();
          r.phase = 3;
          r.t_done = Clock::now();
          used_ -= need_bytes(r.d.n);
          fmm_active_.erase(std::find(fmm_active_.begin(), fmm_active_.end(), id));
          return fail(st, msg);  // returns at once: the loop's iterator is not used again
        }
        r.out = std::move(j->out);
        r.step_ms = std::move(j->step_ms);
        r.steps = j->steps.load();
        r.t_done = j->t_done;
        stats_.field_pairs += j->ctr.field_pairs;
        stats_.force_pairs += j->ctr.force_pairs;
        r.job.reset();
        r.phase = 2;
        used_ -= need_bytes(r.d.n);
        ++completed;
        ++stats_.completed;
      }
      fmm_active_ = keep;
    }
    if (!active_.empty()) {
      MF_CUDA_TRY(cudaStreamSynchronize(batch_->stream()));
      // each member's step latency: from the tick's start to its step done
      const double step_ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
      for (int64_t id : active_) {
        Req& r = reqs_.at(id);
        ++r.steps;
        r.step_ms.push_back(step_ms);
      }
      // Retire finished requests: keep their final state on the host.
      std::vector<int64_t> keep;
      for (size_t k = 0; k < members_.size(); ++k) {
        Req& r = reqs_.at(members_[k]);
        if (r.steps >= cfg_.steps_per_request) {
          const int s = int(k);
          r.out.resize(5);
          const int qs[5] = {MF_Q_POSITIONS, MF_Q_VELOCITY, MF_Q_M, MF_Q_B_OVER_MU0, MF_Q_FORCE};
          for (int j = 0; j < 5; ++j) {
            r.out[size_t(j)].resize(size_t(3 * r.d.n));
            MF_TRY(batch_->get(s, qs[j], r.out[size_t(j)].data()));
          }
          give_state(std::move(r.state));
          used_ -= need_bytes(r.d.n);
          r.phase = 2;
          r.t_done = Clock::now();
          ++completed;
          ++stats_.completed;
          dirty_ = true;
        } else {
          keep.push_back(r.id);
        }
      }
      active_ = keep;
    } else if (!fmm_active_.empty() && completed == 0) {
      // Only FMM requests running and none finished: give their threads the
      // host for a moment instead of returning to a caller that polls.
      std::this_thread::sleep_for(std::chrono::microseconds(500));
    }
    // Parked frees: now, if no FMM request is in flight (the batch stream was
    // synchronised above), or past the cap.
    if ((fmm_active_.empty() && deferred_bytes() > 0) || deferred_bytes() > kDeferredMax) flush_deferred_frees();
    const double ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
    stats_.busy_ms += ms;
    if (n_active) *n_active = int32_t(active_.size() + fmm_active_.size() + size_t(completed));
    if (n_completed) *n_completed = completed;
    if (tick_ms) *tick_ms = ms;
    return MF_OK;
  }

  mf_status poll(int64_t id, int32_t* phase, int32_t* steps, double* latency_ms) {
    auto it = reqs_.find(id);
    if (it == reqs_.end()) return fail(MF_ERR_INVALID_ARG, "unknown request");
    const Req& r = it->second;
    if (phase) *phase = r.phase;
    if (steps) *steps = r.job ? r.job->steps.load() : r.steps;
    if (latency_ms)
      *latency_ms = r.phase == 2 ? std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count() : -1.0;
    return MF_OK;
  }

  mf_status result(int64_t id, int q, float* dst) {
    auto it = reqs_.find(id);
    if (it == reqs_.end()) return fail(MF_ERR_INVALID_ARG, "unknown request");
    const Req& r = it->second;
    if (r.phase == 3) return fail(MF_ERR_INVALID_ARG, "request failed");
    if (r.phase != 2) return fail(MF_ERR_INVALID_ARG, "request not done");
    if (!dst) return fail(MF_ERR_INVALID_ARG, "dst is NULL");
    int j = -1;
    switch (q) {
      case MF_Q_POSITIONS: j = 0; break;
      case MF_Q_VELOCITY: j = 1; break;
      case MF_Q_M: j = 2; break;
      case MF_Q_B_OVER_MU0: j = 3; break;
      case MF_Q_FORCE: j = 4; break;
      default: return fail(MF_ERR_INVALID_ARG, "quantity not kept for served requests");
    }
    std::copy(r.out[size_t(j)].begin(), r.out[size_t(j)].end(), dst);
    return MF_OK;
  }

  mf_status get_stats(mf_server_stats* out) {
    mf_server_stats s = stats_;
    s.running = int64_t(active_.size() + fmm_active_.size());
    s.queued = int64_t(queue_.size());
    s.bytes_in_use = used_;
    if (batch_) {
      mf_counters c{};
      MF_TRY(batch_->counters(&c));
      s.field_pairs += c.field_pairs;
      s.force_pairs += c.force_pairs;
    }
    *out = s;
    return MF_OK;
  }

  // Wall time of each timestep a request has taken so far: for a batch
  // member, the tick from its start until the member's step was done on the
  // device (a rebatch in that tick included); for an FMM request, each
  // mf_advance on its thread until its stream was idle.
  mf_status step_times(int64_t id, double* ms, int32_t cap, int32_t* count) {
    auto it = reqs_.find(id);
    if (it == reqs_.end()) return fail(MF_ERR_INVALID_ARG, "unknown request");
    if (cap < 0 || (cap > 0 && !ms)) return fail(MF_ERR_INVALID_ARG, "bad output buffer");
    Req& r = it->second;
    std::vector<double> v;
    if (r.job) {
      std::lock_guard<std::mutex> lk(r.job->mu);
      v = r.job->step_ms;
    } else {
      v = r.step_ms;
    }
    if (count) *count = int32_t(v.size());
    std::copy(v.begin(), v.begin() + std::min<size_t>(v.size(), size_t(cap)), ms);
    return MF_OK;
  }

 private:
  // An FMM request's thread and what it hands back.  Until `done` is set the
  // serving loop reads only `steps` and, under `mu`, `step_ms`.
  struct FmmJob {
    std::thread th;
    std::atomic<bool> done{false}, cancel{false};
    std::atomic<int32_t> steps{0};
    std::mutex mu;
    std::vector<double> step_ms;
    std::vector<std::vector<float>> out;
    mf_counters ctr{};
    mf_status status = MF_OK;
    std::string err;
    Clock::time_point t_done;
  };

  struct Req {
    int64_t id = 0;
    mf_scene_desc d{};
    std::vector<float> pos;
    DevBuf state;  // [3][n] float4: positions, velocities, warm start
    int32_t phase = 0;
    int32_t steps = 0;
    Clock::time_point t_submit, t_done;
    std::vector<std::vector<float>> out;
    std::vector<double> step_ms;  // wall time of each timestep taken
    std::unique_ptr<FmmJob> job;  // FMM requests while they run
  };

  // The thread of an FMM request: a solver handle on its own non-blocking
  // stream (CG to the server's tolerance, the handle's automatic choice of
  // FMM or all-pairs per product, tuned block shapes only where already
  // cached, so no timing lands on the request), a converged cold
  // solve, the request's timesteps, then the read-back of its final state.
  static void fmm_worker(FmmJob* j, mf_scene_desc d, const float* pos, mf_server_config cfg) {
    mf_solver* sv = nullptr;
    cudaStream_t stream = nullptr;
    auto run = [&]() -> mf_status {
      MF_CUDA_TRY(cudaSetDevice(cfg.device));
      set_thread_tune_mode(int(Tune::CachedOnly));
      mf_params p{};
      p.num_particles = d.n;
      p.h = d.h;
      p.ext_mag_h = d.h;
      p.volume = d.volume;
      p.chi = d.chi;
      for (int k = 0; k < 3; ++k) p.const_ext_field[k] = d.H0[k];
      p.target_pos = pos;
      p.precision = MF_FP32;
      p.device = cfg.device;
      MF_TRY(mf_create(&p, &sv));
      {
        int lo = 0, hi = 0;  // the lowest priority: the shared batch goes first
        MF_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        MF_CUDA_TRY(cudaStreamCreateWithPriority(&stream, cudaStreamNonBlocking, lo));
      }
      MF_TRY(mf_set_stream(sv, stream));
      MF_TRY(mf_set_option(sv, MF_OPT_SOLVER, MF_SOLVER_CG));
      MF_TRY(mf_set_option(sv, MF_OPT_REL_TOL, cfg.rel_tol));
      MF_TRY(mf_set_option(sv, MF_OPT_FMM, 0));
      int64_t it = 0;
      double rr = 0;
      mf_status s = mf_solve(sv, 500, &it, &rr);
      if (s != MF_OK && s != MF_ERR_NOT_CONVERGED) return s;
      for (int k = 0; k < cfg.steps_per_request; ++k) {
        if (j->cancel.load()) return MF_OK;
        const auto t0 = Clock::now();
        s = mf_advance(sv, cfg.dt, cfg.iters_per_step, &it);
        if (s != MF_OK && s != MF_ERR_NOT_CONVERGED) return s;
        MF_CUDA_TRY(cudaStreamSynchronize(stream));
        const double ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
        {
          std::lock_guard<std::mutex> lk(j->mu);
          j->step_ms.push_back(ms);
        }
        j->steps.fetch_add(1);
      }
      j->out.resize(5);
      const int qs[5] = {MF_Q_POSITIONS, MF_Q_VELOCITY, MF_Q_M, MF_Q_B_OVER_MU0, MF_Q_FORCE};
      for (int q = 0; q < 5; ++q) {
        j->out[size_t(q)].resize(size_t(3 * d.n));
        MF_TRY(mf_get(sv, qs[q], j->out[size_t(q)].data(), MF_LAYOUT_AOS, MF_HOST));
      }
      MF_TRY(mf_get_counters(sv, &j->ctr));
      return MF_OK;
    };
    mf_status s = MF_OK;
    try {
      s = run();
    } catch (const std::bad_alloc&) {
      s = fail(MF_ERR_OOM, "host allocation failed");
    } catch (const std::exception& e) {
      s = fail(MF_ERR_CUDA, e.what());
    }
    if (s != MF_OK) j->err = mf_last_error();
    if (sv) mf_destroy(sv);
    if (stream) cudaStreamDestroy(stream);
    j->status = s;
    j->t_done = Clock::now();
    j->done.store(true, std::memory_order_release);
  }

  // Device state of retired batch members is kept for later admissions:
  // cudaFree would wait for every stream of the device, the FMM requests'
  // included.  At most kPoolMax buffers are kept; they are not counted in
  // the admission budget (the requests that used them were).
  static constexpr size_t kPoolMax = 16;
  mf_status take_state(DevBuf& dst, size_t bytes) {
    size_t best = pool_.size();
    for (size_t k = 0; k < pool_.size(); ++k)
      if (pool_[k].bytes >= bytes && (best == pool_.size() || pool_[k].bytes < pool_[best].bytes)) best = k;
    if (best < pool_.size()) {
      dst = std::move(pool_[best]);
      pool_.erase(pool_.begin() + std::ptrdiff_t(best));
    } else {
      MF_TRY(dst.reserve(bytes));
    }
    MF_CUDA_TRY(cudaMemset(dst.ptr, 0, bytes));
    return MF_OK;
  }
  void give_state(DevBuf&& b) {
    pool_.push_back(std::move(b));
    if (pool_.size() > kPoolMax) {  // drop the smallest
      size_t k = 0;
      for (size_t j = 1; j < pool_.size(); ++j)
        if (pool_[j].bytes < pool_[k].bytes) k = j;
      pool_.erase(pool_.begin() + std::ptrdiff_t(k));
    }
  }

  Batch::SceneState state_of(Req& r) {
    float4* base = r.state.as<float4>();
    return Batch::SceneState{base, base + r.d.n, base + 2 * r.d.n};
  }

  // Membership changed: save the continuing requests' state out of the old
  // batch, lay out a new one over all running requests, bring new ones to a
  // converged magnetization.
  mf_status rebatch() {
    if (batch_) {
      for (size_t k = 0; k < members_.size(); ++k) {
        Req& r = reqs_.at(members_[k]);
        if (r.phase == 1) MF_TRY(batch_->export_state(int(k), state_of(r)));
      }
      MF_CUDA_TRY(cudaStreamSynchronize(batch_->stream()));
      mf_counters c{};
      MF_TRY(batch_->counters(&c));
      stats_.field_pairs += c.field_pairs;
      stats_.force_pairs += c.force_pairs;
    }
    members_ = active_;
    std::vector<mf_scene_desc> descs;
    std::vector<Batch::SceneState> st;
    for (int64_t id : members_) {
      Req& r = reqs_.at(id);
      descs.push_back(r.d);
      st.push_back(state_of(r));
    }
    std::unique_ptr<Batch> nb(new Batch());
    nb->set_high_priority();
    if (batch_) {
      nb->adopt_buffers(*batch_);
      batch_.reset();
    }
    batch_ = std::move(nb);
    batch_->device_ = cfg_.device;
    // Rebatching happens between timesteps: use tuned shapes already cached,
    // never time new ones on the request path.
    MF_TRY(batch_->init(descs.data(), int(descs.size()), cfg_.device, st.data(),
                        default_tune_mode() == Tune::Off ? Tune::Off : Tune::CachedOnly));
    MF_TRY(batch_->solve(500, cfg_.rel_tol, true));
    ++stats_.rebatches;
    dirty_ = false;
    return MF_OK;
  }

  mf_server_config cfg_{};
  std::map<int64_t, Req> reqs_;
  std::deque<int64_t> queue_;
  std::vector<int64_t> active_, members_, fmm_active_;
  std::unique_ptr<Batch> batch_;
  std::vector<DevBuf> pool_;  // device state of retired batch members, for reuse
  bool dirty_ = false;
  double used_ = 0;
  int64_t next_id_ = 1;
  mf_server_stats stats_{};
};

}  // namespace mfgb

using namespace mfgb;

struct mf_server {
  std::unique_ptr<Server> s;
  int device = 0;
};

namespace {
template <class F>
mf_status sguard(mf_server* s, F&& fn) {
  if (!s || !s->s) return fail(MF_ERR_INVALID_ARG, "NULL server handle");
  try {
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return fn(*s->s);
  } catch (const std::bad_alloc&) {
    return fail(MF_ERR_OOM, "host allocation failed");
  } catch (const std::out_of_range&) {
    return fail(MF_ERR_INVALID_ARG, "unknown request");
  } catch (...) {
    return fail(MF_ERR_CUDA, "unexpected exception");
  }
}
}  // namespace

extern "C" {

mf_status mf_server_create(const mf_server_config* cfg, mf_server** out) {
  if (!cfg || !out) return fail(MF_ERR_INVALID_ARG, "NULL argument");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(MF_ERR_UNSUPPORTED, "no CUDA device available");
  if (cfg->device < 0 || cfg->device >= ndev) return fail(MF_ERR_INVALID_ARG, "bad device ordinal");
  try {
    MF_CUDA_TRY(cudaSetDevice(cfg->device));
    std::unique_ptr<mf_server> h(new mf_server);
    h->device = cfg->device;
    h->s.reset(new Server());
    MF_TRY(h->s->init(*cfg));
    *out = h.release();
    return MF_OK;
  } catch (const std::bad_alloc&) {
    return fail(MF_ERR_OOM, "host allocation failed");
  }
}

mf_status mf_server_destroy(mf_server* s) {
  if (!s) return MF_OK;
  cudaSetDevice(s->device);
  delete s;
  return MF_OK;
}

mf_status mf_server_submit(mf_server* s, const mf_scene_desc* scene, int64_t* request_id) {
  return sguard(s, [&](Server& x) {
    if (!scene) return fail(MF_ERR_INVALID_ARG, "NULL scene");
    return x.submit(*scene, request_id);
  });
}

mf_status mf_server_step(mf_server* s, int32_t* active, int32_t* completed, double* tick_ms) {
  return sguard(s, [&](Server& x) { return x.step(active, completed, tick_ms); });
}

mf_status mf_server_poll(mf_server* s, int64_t request_id, int32_t* state, int32_t* steps_done, double* latency_ms) {
  return sguard(s, [&](Server& x) { return x.poll(request_id, state, steps_done, latency_ms); });
}

mf_status mf_server_result(mf_server* s, int64_t request_id, int32_t quantity, float* dst) {
  return sguard(s, [&](Server& x) { return x.result(request_id, quantity, dst); });
}

mf_status mf_server_get_stats(mf_server* s, mf_server_stats* out) {
  return sguard(s, [&](Server& x) {
    if (!out) return fail(MF_ERR_INVALID_ARG, "NULL");
    return x.get_stats(out);
  });
}

mf_status mf_server_step_times(mf_server* s, int64_t request_id, double* ms, int32_t capacity, int32_t* count) {
  return sguard(s, [&](Server& x) { return x.step_times(request_id, ms, capacity, count); });
}

}  // extern "C"

struct mf_batch {
  std::unique_ptr<Batch> b;
  int device = 0;
};

namespace {
template <class F>
mf_status bguard(mf_batch* b, F&& fn) {
  if (!b || !b->b) return fail(MF_ERR_INVALID_ARG, "NULL batch handle");
  try {
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return fn(*b->b);
  } catch (const std::bad_alloc&) {
    return fail(MF_ERR_OOM, "host allocation failed");
  } catch (...) {
    return fail(MF_ERR_CUDA, "unexpected exception");
  }
}
}  // namespace

extern "C" {

mf_status mf_batch_create(const mf_scene_desc* scenes, int32_t n_scenes, int32_t device, mf_batch** out) {
  if (!out) return fail(MF_ERR_INVALID_ARG, "NULL out");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(MF_ERR_UNSUPPORTED, "no CUDA device available");
  if (device < 0 || device >= ndev) return fail(MF_ERR_INVALID_ARG, "bad device ordinal");
  try {
    MF_CUDA_TRY(cudaSetDevice(device));
    std::unique_ptr<mf_batch> h(new mf_batch);
    h->device = device;
    h->b.reset(new Batch());
    h->b->device_ = device;
    MF_TRY(h->b->init(scenes, n_scenes, device));
    *out = h.release();
    return MF_OK;
  } catch (const std::bad_alloc&) {
    return fail(MF_ERR_OOM, "host allocation failed");
  }
}

mf_status mf_batch_destroy(mf_batch* b) {
  if (!b) return MF_OK;
  cudaSetDevice(b->device);
  if (b->b) cudaStreamSynchronize(b->b->stream());
  delete b;
  return MF_OK;
}

mf_status mf_batch_set_stream(mf_batch* b, void* stream) {
  return bguard(b, [&](Batch& x) {
    x.set_stream(static_cast<cudaStream_t>(stream));
    return MF_OK;
  });
}

mf_status mf_batch_num_scenes(mf_batch* b, int32_t* n) {
  return bguard(b, [&](Batch& x) {
    if (!n) return fail(MF_ERR_INVALID_ARG, "NULL");
    *n = x.scenes();
    return MF_OK;
  });
}

mf_status mf_batch_solve(mf_batch* b, int64_t max_iter, double rel_tol, int64_t* max_iters, double* worst_res) {
  return bguard(b, [&](Batch& x) {
    if (max_iter < 0 || !(rel_tol > 0)) return fail(MF_ERR_INVALID_ARG, "bad iteration cap or tolerance");
    MF_TRY(x.solve(max_iter, rel_tol, true));
    std::vector<double> rr(size_t(x.scenes())), it(size_t(x.scenes()));
    MF_TRY(x.solver_state(rr.data(), it.data()));
    if (max_iters) *max_iters = int64_t(*std::max_element(it.begin(), it.end()));
    const double worst = *std::max_element(rr.begin(), rr.end());
    if (worst_res) *worst_res = worst;
    return worst < rel_tol ? MF_OK : fail(MF_ERR_NOT_CONVERGED, "some scenes stopped above tolerance");
  });
}

mf_status mf_batch_eval_force(mf_batch* b) {
  return bguard(b, [&](Batch& x) { return x.eval_force(); });
}

mf_status mf_batch_advance(mf_batch* b, double dt, int32_t steps, int32_t iters_per_step, double rel_tol,
                           int32_t use_graph) {
  return bguard(b, [&](Batch& x) {
    if (!std::isfinite(dt) || !(rel_tol > 0)) return fail(MF_ERR_INVALID_ARG, "bad dt or tolerance");
    return x.advance(dt, steps, iters_per_step, rel_tol, use_graph != 0);
  });
}

mf_status mf_batch_get(mf_batch* b, int32_t scene, int32_t quantity, float* dst) {
  return bguard(b, [&](Batch& x) { return x.get(scene, quantity, dst); });
}

mf_status mf_batch_solver_state(mf_batch* b, double* rel_res, double* iters) {
  return bguard(b, [&](Batch& x) { return x.solver_state(rel_res, iters); });
}

mf_status mf_batch_get_counters(mf_batch* b, mf_counters* c) {
  return bguard(b, [&](Batch& x) {
    if (!c) return fail(MF_ERR_INVALID_ARG, "NULL");
    return x.counters(c);
  });
}

mf_status mf_batch_reset_counters(mf_batch* b) {
  return bguard(b, [&](Batch& x) { return x.reset_counters(); });
}

}  // extern "C"
