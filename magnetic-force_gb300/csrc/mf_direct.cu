// mf_direct.cu -- direct all-pairs evaluation of the reference's pair kernels
// on caller-owned device buffers (the fmmtl::direct replacement of mf.h).
//
// The caller's AoS [n][3] arrays are packed into 16-byte records so source
// tiles can be staged by bulk copies; that packing space, the plan table and
// the kernel scratch live in one context per device, created on first use
// and kept until mf_release_scratch() or process exit.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "mf_internal.h"

namespace mfgb {
namespace {

__global__ void k_pack_aos(int64_t n, const float* __restrict__ src, float4* __restrict__ dst) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    dst[i] = make_float4(src[3 * i], src[3 * i + 1], src[3 * i + 2], 0.f);
}

// SoA (k arrays of n) -> AoS [n][k]
__global__ void k_soa_to_aos_k(int64_t n, int k, const float* __restrict__ soa, float* __restrict__ aos) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    for (int c = 0; c < k; ++c) aos[i * k + c] = soa[int64_t(c) * n + i];
}

// AoS [n][k] -> SoA
__global__ void k_aos_to_soa_k(int64_t n, int k, const float* __restrict__ aos, float* __restrict__ soa) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    for (int c = 0; c < k; ++c) soa[int64_t(c) * n + i] = aos[i * k + c];
}

unsigned grid_for(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  return unsigned(g);
}

constexpr int kBodies = 5;

struct DirectCtx {
  std::mutex mu;
  DevBuf t4, s4, m4, tm4, soa, aux, s2, m2, corr;
  Scratch scr;
  CellList cells;
  Plan<float> plan[kBodies];
  bool plan_ok[kBodies] = {};
  int64_t plan_nt[kBodies] = {}, plan_ns[kBodies] = {};
  double plan_h[kBodies] = {};
  void release() {
    for (DevBuf* b : {&t4, &s4, &m4, &tm4, &soa, &aux, &s2, &m2, &corr}) b->release();
    scr.partials.release();
    scr.counters.release();
    scr.err.release();
    cells = CellList();
    for (int b = 0; b < kBodies; ++b) {
      plan[b].d_scenes.release();
      plan_ok[b] = false;
    }
  }
};

DirectCtx g_ctx[64];

mf_status get_plan(DirectCtx& c, Body body, int64_t nt, int64_t ns, double h, int shape, const Plan<float>** out) {
  const int b = int(body);
  if (!c.plan_ok[b] || c.plan_nt[b] != nt || c.plan_ns[b] != ns || c.plan_h[b] != h || c.plan[b].shape != shape) {
    SceneSpec s;
    s.t_off = 0;
    s.nt = nt;
    s.s_off = 0;
    s.ns = ns;
    s.h = h;
    s.scale = 1.0;
    MF_TRY(build_plan<float>(body, {s}, c.plan[b], shape));
    c.plan_ok[b] = true;
    c.plan_nt[b] = nt;
    c.plan_ns[b] = ns;
    c.plan_h[b] = h;
  }
  *out = &c.plan[b];
  return MF_OK;
}

mf_status check_common(const void* a, int64_t na, const void* b, const void* c, int64_t nb, float h) {
  if (na < 0 || nb < 0) return fail(MF_ERR_INVALID_ARG, "negative count");
  if (na > 0 && !a) return fail(MF_ERR_INVALID_ARG, "NULL target array");
  if (nb > 0 && (!b || !c)) return fail(MF_ERR_INVALID_ARG, "NULL source array");
  if (!(h > 0.f) || !std::isfinite(h)) return fail(MF_ERR_INVALID_ARG, "h must be finite and > 0");
  return MF_OK;
}

mf_status direct_impl(Body body, const float* targets, int64_t nt, const float* sources, const float* charges,
                      int64_t ns, float h, const float* rext9, int naive, float* results, cudaStream_t st) {
  const int dev = current_device();
  if (dev < 0 || dev >= 64) return fail(MF_ERR_UNSUPPORTED, "device ordinal out of range");
  DirectCtx& c = g_ctx[dev];
  std::lock_guard<std::mutex> lk(c.mu);
  const int kOut = body == Body::Tensor ? 9 : 3;
  if (nt == 0) return MF_OK;
  if (ns == 0) {
    MF_CUDA_TRY(cudaMemsetAsync(results, 0, size_t(nt) * kOut * sizeof(float), st));
    MF_CUDA_TRY(cudaStreamSynchronize(st));
    return MF_OK;
  }
  MF_TRY(c.t4.reserve(size_t(nt) * sizeof(float4)));
  MF_TRY(c.s4.reserve(size_t(ns) * sizeof(float4)));
  MF_TRY(c.m4.reserve(size_t(ns) * sizeof(float4)));
  MF_TRY(c.soa.reserve(size_t(nt) * kOut * sizeof(float)));
  k_pack_aos<<<grid_for(nt), 256, 0, st>>>(nt, targets, c.t4.as<float4>());
  k_pack_aos<<<grid_for(ns), 256, 0, st>>>(ns, sources, c.s4.as<float4>());
  k_pack_aos<<<grid_for(ns), 256, 0, st>>>(ns, charges, c.m4.as<float4>());
  MF_CUDA_TRY(cudaGetLastError());
  LaunchIO<float> io;
  io.tpos = c.t4.as<float4>();
  io.spos = c.s4.as<float4>();
  io.smom = c.m4.as<float4>();
  // Field and force go through the packed two-source kernels: sources in pair
  // layout, a cell list over the sources, and the near-field correction.
  Body launch_body = body;
  if (body == Body::Field || body == Body::Force) {
    const size_t pair_bytes = size_t(ns + 1) * sizeof(float4);
    MF_TRY(c.s2.reserve(pair_bytes));
    MF_TRY(c.m2.reserve(pair_bytes));
    MF_TRY(c.corr.reserve(size_t(nt) * sizeof(float4)));
    to_pairs(c.s4.as<float4>(), c.s2.as<float4>(), ns, st);
    to_pairs(c.m4.as<float4>(), c.m2.as<float4>(), ns, st);
    MF_CUDA_TRY(cudaGetLastError());
    MF_TRY(c.cells.build(c.s4.as<float4>(), {CellSceneSpec{0, ns, double(h)}}, st));
    if (body == Body::Field) {
      if (targets == sources && nt == ns)
        MF_TRY(c.cells.field_correction(c.s4.as<float4>(), c.m4.as<float4>(), c.corr.as<float4>(), st));
      else
        MF_TRY(c.cells.field_correction_at(c.t4.as<float4>(), nt, c.s4.as<float4>(), c.m4.as<float4>(),
                                           c.corr.as<float4>(), st));
      launch_body = Body::FieldF2;
    } else {
      MF_TRY(c.cells.force_correction(c.s4.as<float4>(), c.m4.as<float4>(), c.corr.as<float4>(), st));
      launch_body = Body::ForceF2;
    }
    io.spos = c.s2.as<float4>();
    io.smom = c.m2.as<float4>();
    io.corr4 = c.corr.as<float4>();
  }
  // One particle set (the force always; the field when the caller passes
  // the sources as the targets): each unordered pair once for both
  // particles from kSymDirectMin particles on (no tuning on this path: a
  // call can be seconds long), per MF_PAIR_SYMMETRIC.
  int shape = 0;
  if ((launch_body == Body::FieldF2 || launch_body == Body::ForceF2) &&
      (body == Body::Force || (targets == sources && nt == ns))) {
    const int mode = default_sym_mode();
    if (mode == 2 || (mode == 1 && nt >= kSymDirectMin)) shape = kShapeSym;
  }
  if (shape == kShapeSym) io.tpos = c.s4.as<float4>();  // the same records as the sources
  const Plan<float>* plan = nullptr;
  MF_TRY(get_plan(c, launch_body, nt, ns, h, shape, &plan));
  float* soa = c.soa.as<float>();
  for (int k = 0; k < kOut; ++k) io.out[k] = soa + int64_t(k) * nt;
  if (body == Body::Force) {
    io.tmom = c.m4.as<float4>();  // one particle set: target dipoles = sources' dipoles
    io.naive_quirks = naive;
    if (rext9) {
      MF_TRY(c.aux.reserve(size_t(nt) * 9 * sizeof(float)));
      k_aos_to_soa_k<<<grid_for(nt), 256, 0, st>>>(nt, 9, rext9, c.aux.as<float>());
      MF_CUDA_TRY(cudaGetLastError());
      for (int k = 0; k < 9; ++k) io.rext[k] = c.aux.as<float>() + int64_t(k) * nt;
    }
  }
  MF_TRY(run_plan<float>(*plan, io, c.scr, st));
  k_soa_to_aos_k<<<grid_for(nt), 256, 0, st>>>(nt, kOut, soa, results);
  MF_CUDA_TRY(cudaGetLastError());
  MF_TRY(c.scr.check(st));  // synchronises the stream
  return MF_OK;
}

}  // namespace
}  // namespace mfgb

using namespace mfgb;

extern "C" {

mf_status mf_direct_field(const float* targets, int64_t nt, const float* sources, const float* charges,
                          int64_t ns, float h, float* results, void* stream) {
  MF_TRY(check_common(targets, nt, sources, charges, ns, h));
  if (nt > 0 && !results) return fail(MF_ERR_INVALID_ARG, "NULL results");
  return direct_impl(Body::Field, targets, nt, sources, charges, ns, h, nullptr, 0, results,
                     static_cast<cudaStream_t>(stream));
}

mf_status mf_direct_force_tensor(const float* targets, int64_t nt, const float* sources, const float* charges,
                                 int64_t ns, float h, float* results9, void* stream) {
  MF_TRY(check_common(targets, nt, sources, charges, ns, h));
  if (nt > 0 && !results9) return fail(MF_ERR_INVALID_ARG, "NULL results");
  return direct_impl(Body::Tensor, targets, nt, sources, charges, ns, h, nullptr, 0, results9,
                     static_cast<cudaStream_t>(stream));
}

mf_status mf_direct_force(const float* pos, const float* mom, int64_t n, float h, const float* rext9,
                          int32_t naive_quirks, float* force, void* stream) {
  MF_TRY(check_common(pos, n, pos, mom, n, h));
  if (n > 0 && !force) return fail(MF_ERR_INVALID_ARG, "NULL force");
  return direct_impl(Body::Force, pos, n, pos, mom, n, h, rext9, naive_quirks ? 1 : 0, force,
                     static_cast<cudaStream_t>(stream));
}

mf_status mf_debug_stage_wait_limit(int64_t limit) {
  if (limit < 0) set_stage_wait_debug(0);
  else set_stage_wait_debug(uint32_t(std::min<int64_t>(limit, int64_t(kWaitLimit)) + 1));
  return MF_OK;
}

mf_status mf_release_scratch(void) {
  const int dev = current_device();
  if (dev < 0 || dev >= 64) return MF_OK;
  std::lock_guard<std::mutex> lk(g_ctx[dev].mu);
  g_ctx[dev].release();
  return MF_OK;
}

}  // extern "C"
