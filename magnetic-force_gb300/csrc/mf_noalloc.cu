// mf_noalloc.cu -- mf_direct_field_noalloc: the direct B/mu0 field evaluation
// of mf_direct_field with every byte of its scratch in one file-scope device
// array, for callers that must not allocate device memory.
//
// Scratch held in g_noalloc_scratch (one copy per device that loads the
// library, resident until the process exits):
//   packed targets, sources and dipoles    3 x 65,536 x 16 B
//   SoA result staging                     65,536 x 12 B
//   FP64 partials of split target blocks   320 CTAs x 2 x 512 x 3 x 8 B
//   tickets, scene record, error word
// about 11.5 MiB in all.  Sizes beyond 65,536 targets or sources are refused.
//
// Host code never touches g_noalloc_scratch by name: its host-side symbol is a
// stand-in, not a device address.  The first call on a device (with that
// device current) looks the device address up once with cudaGetSymbolAddress
// and caches it; make that first call before any stream capture.
// Every call reuses the same array and leaves its contents behind; the call
// clears what must start at zero (tickets, error word).  Two calls whose
// kernels overlap on the GPU (different streams, or different host threads)
// race on the array: serialise them.
#include <cmath>
#include <cstring>
#include <mutex>

#include "mf_internal.h"

namespace mfgb {
namespace {

using Cfg = KCfg<float, Body::Field>;
constexpr int64_t kMaxN = 65536;
constexpr int kMaxGrid = 320;
constexpr int kTBT = Cfg::TPB * Cfg::TPT;
constexpr int64_t kMaxTB = (kMaxN + kTBT - 1) / kTBT;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffT4 = 0;
constexpr size_t kOffS4 = align256(kOffT4 + kMaxN * sizeof(float4));
constexpr size_t kOffM4 = align256(kOffS4 + kMaxN * sizeof(float4));
constexpr size_t kOffSoa = align256(kOffM4 + kMaxN * sizeof(float4));
constexpr size_t kOffPart = align256(kOffSoa + kMaxN * 3 * sizeof(float));
constexpr size_t kOffCnt = align256(kOffPart + size_t(kMaxGrid) * 2 * kTBT * 3 * sizeof(double));
constexpr size_t kOffScene = align256(kOffCnt + kMaxTB * sizeof(int32_t));
constexpr size_t kOffErr = align256(kOffScene + sizeof(SceneDesc<float>));
constexpr size_t kBytes = align256(kOffErr + 16);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

using Kern = void (*)(const AllPairsArgs<float>);
Kern field_kernel() { return allpairs_kernel<float, FieldBody<float>, Cfg::TPB, Cfg::TPT, Cfg::TILE, Cfg::STAGES>; }
constexpr size_t kSmem = size_t(Cfg::STAGES) * StageLayout<float, Cfg::TILE>::kBytes;

// Per-device set-up: the array's device address and the launch shape.
struct DevState {
  unsigned char* base = nullptr;
  int grid_cap = 0;
};
std::mutex g_mu;
DevState g_dev[64];

__global__ void k_pack(int64_t n, const float* __restrict__ src, float4* __restrict__ dst) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    dst[i] = make_float4(src[3 * i], src[3 * i + 1], src[3 * i + 2], 0.f);
}

__global__ void k_unpack(int64_t n, const float* __restrict__ soa, float* __restrict__ aos) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    aos[3 * i] = soa[i];
    aos[3 * i + 1] = soa[n + i];
    aos[3 * i + 2] = soa[2 * n + i];
  }
}

// Writes this call's scene record and clears the tickets and the error word.
__global__ void k_prepare(SceneDesc<float> sc, SceneDesc<float>* scene, int32_t* counters, int n_counters,
                          int32_t* err) {
  for (int i = threadIdx.x; i < n_counters; i += blockDim.x) counters[i] = 0;
  if (threadIdx.x == 0) {
    *scene = sc;
    *err = 0;
  }
}

unsigned grid_for(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 1024) g = 1024;
  return unsigned(g < 1 ? 1 : g);
}

mf_status setup(int dev, DevState** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  DevState& d = g_dev[dev];
  if (!d.base) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    e = cudaFuncSetAttribute(field_kernel(), cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmem));
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, field_kernel(), Cfg::TPB, kSmem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
    const int g = (per_sm < 1 ? 1 : per_sm) * sms;
    d.grid_cap = g < kMaxGrid ? g : kMaxGrid;
    d.base = static_cast<unsigned char*>(p);
  }
  *out = &d;
  return MF_OK;
}

}  // namespace
}  // namespace mfgb

using namespace mfgb;

extern "C" mf_status mf_direct_field_noalloc(const float* targets, int64_t nt, const float* sources,
                                             const float* charges, int64_t ns, float h, float* results,
                                             void* stream) {
  if (nt < 0 || ns < 0) return fail(MF_ERR_INVALID_ARG, "negative count");
  if (nt > kMaxN || ns > kMaxN)
    return fail(MF_ERR_INVALID_ARG, "mf_direct_field_noalloc: at most 65536 targets and 65536 sources");
  if ((nt > 0 && (!targets || !results)) || (ns > 0 && (!sources || !charges)))
    return fail(MF_ERR_INVALID_ARG, "NULL array");
  if (!(h > 0.f) || !std::isfinite(h)) return fail(MF_ERR_INVALID_ARG, "h must be finite and > 0");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (nt == 0) return MF_OK;
  if (ns == 0) {
    MF_CUDA_TRY(cudaMemsetAsync(results, 0, size_t(nt) * 3 * sizeof(float), st));
    MF_CUDA_TRY(cudaStreamSynchronize(st));
    return MF_OK;
  }
  int dev = 0;
  MF_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(MF_ERR_UNSUPPORTED, "device ordinal out of range");
  DevState* d = nullptr;
  MF_TRY(setup(dev, &d));

  float4* t4 = reinterpret_cast<float4*>(d->base + kOffT4);
  float4* s4 = reinterpret_cast<float4*>(d->base + kOffS4);
  float4* m4 = reinterpret_cast<float4*>(d->base + kOffM4);
  float* soa = reinterpret_cast<float*>(d->base + kOffSoa);
  double* partials = reinterpret_cast<double*>(d->base + kOffPart);
  int32_t* counters = reinterpret_cast<int32_t*>(d->base + kOffCnt);
  SceneDesc<float>* scene = reinterpret_cast<SceneDesc<float>*>(d->base + kOffScene);
  int32_t* err = reinterpret_cast<int32_t*>(d->base + kOffErr);

  // The one scene of this call, laid out in step space as build_plan does.
  SceneDesc<float> sc;
  memset(&sc, 0, sizeof(sc));
  sc.t_off = 0;
  sc.nt = nt;
  sc.s_off = 0;
  sc.ns = ns;
  sc.n_tiles = int32_t((ns + Cfg::TILE - 1) / Cfg::TILE);
  sc.n_tb = int32_t((nt + kTBT - 1) / kTBT);
  sc.step_off = 0;
  sc.tb_off = 0;
  sc.pc = make_pair_consts<float>(double(h));
  sc.scale = 1.f;
  const int64_t total_steps = int64_t(sc.n_tiles) * sc.n_tb;

  k_prepare<<<1, 128, 0, st>>>(sc, scene, counters, int(kMaxTB), err);
  k_pack<<<grid_for(nt), 256, 0, st>>>(nt, targets, t4);
  k_pack<<<grid_for(ns), 256, 0, st>>>(ns, sources, s4);
  k_pack<<<grid_for(ns), 256, 0, st>>>(ns, charges, m4);
  MF_CUDA_TRY(cudaGetLastError());

  AllPairsArgs<float> a;
  memset(&a, 0, sizeof(a));
  a.scenes = scene;
  a.n_scenes = 1;
  a.total_steps = total_steps;
  a.tpos = t4;
  a.spos = s4;
  a.smom = m4;
  for (int k = 0; k < 3; ++k) a.out[k] = soa + int64_t(k) * nt;
  a.partials = partials;
  a.counters = counters;
  a.err = err;
  const int64_t g = total_steps < d->grid_cap ? total_steps : d->grid_cap;
  field_kernel()<<<unsigned(g), Cfg::TPB, kSmem, st>>>(a);
  MF_CUDA_TRY(cudaGetLastError());
  k_unpack<<<grid_for(nt), 256, 0, st>>>(nt, soa, results);
  MF_CUDA_TRY(cudaGetLastError());

  int32_t host_err = 0;
  MF_CUDA_TRY(cudaMemcpyAsync(&host_err, err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  MF_CUDA_TRY(cudaStreamSynchronize(st));
  if (host_err != 0) return fail(MF_ERR_TIMEOUT, "kernel wait ran out; results are invalid");
  return MF_OK;
}
