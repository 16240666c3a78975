// mf_sympair.cu -- the packed field and force products evaluated once per
// unordered pair of particles.
//
// Both clamped far-form pair terms are symmetric in the pair:
//   * the dipole field tensor T(d) = 3 d d^T r^-5 - I r^-3 is even in d, so
//     the field at i from j is T m_j and the field at j from i is T m_i;
//   * the Kelvin force f_ij = P (d (s.m) + s (d.m) + m (d.s)) + Q (d.s)(d.m) d
//     is antisymmetric, f_ji = -f_ij (the dipoles swap places, d changes sign).
// So one evaluation of the pair's scalars serves both particles.
//
// Work layout.  A scene's particles are cut into blocks of TB = TPB * TPT
// (targets strided by TPB, as in the all-pairs kernel); a source tile is one
// block.  The steps are the (I, J) block pairs with I <= J, row by row, split
// evenly over persistent CTAs.
//   * I < J: each thread holds TPT targets of block I in registers and sweeps
//     tile J (bulk-copied to shared memory on an mbarrier pipeline, 2 sources
//     per packed f32x2 instruction).  Each pair adds into the target's sum
//     and into the tile's source sums; those are reduced over the warp by a
//     fixed shuffle tree and over the warps in a fixed order.
//   * I == J: the block against itself, every ordered pair, target side only.
// Every step writes its FP32 block sums (scaled to the all-pairs kernels'
// output units) into part[K][X] -- the sums for block K from partner block
// X, SoA per block pair -- so each entry is written exactly once.
// k_sym_finish then adds, per particle, the nb entries of its block's row
// (compensated FP32, in a fixed order) and applies the body's epilogue
// (correction, scale and addends for the field; correction, external
// gradient and scale for the force).  Results do not depend on scheduling.
// Force targets are read from the AoS records, field targets from the same
// pair-layout records as the sources.
#include <mutex>

#include "mf_internal.h"
#include "mf_sym.cuh"

namespace mfgb {
namespace {

constexpr int kSymTPB = 128, kSymTPT = 8, kSymStages = 2;
constexpr int kSymTB = kSymTPB * kSymTPT;  // particles per block = sources per tile
constexpr int kSymWarps = kSymTPB / 32;
constexpr size_t kSymSmem = size_t(kSymStages) * 2 * kSymTB * sizeof(float4);
// A tile's source sums are reduced over the warps in kSymSplit phases (the
// per-warp buffer holds one phase: less shared memory per CTA), and over the
// lanes kSymPair items at a time (one shuffle tree for 6 * kSymPair values).
// Measured at N = 65,536 / 131,072 (ms per product; TPB x TPT, stages,
// split, pair): 128x4 3,1,1 3.41 / 13.02; 128x4 2,2,2 3.23 / 12.66;
// 128x4 2,2,4 3.14 / 12.31; 128x8 2,2,1 3.01 / 12.00; 128x8 2,4,2 2.94 /
// 11.68; 64x8 2,2,2 2.95 / 11.56; 128x8 2,2,2 2.88 / 11.47 (254 registers,
// 2 CTAs per SM).
// (The field body sets its own split and pair counts below.)
constexpr int kSymSplit = 2, kSymPair = 2;

// Step l of a scene with nb blocks -> (I, J), row I holding nb - I steps.
__device__ __forceinline__ void sym_block_pair(int64_t l, int nb, int& I, int& J) {
  // start(I) = I nb - I (I - 1) / 2; solve for the largest I with start(I) <= l.
  const double b = 2.0 * nb + 1.0;
  int i = int((b - sqrt(b * b - 8.0 * double(l))) * 0.5);
  if (i < 0) i = 0;
  if (i > nb - 1) i = nb - 1;
  auto start = [&](int r) { return int64_t(r) * nb - int64_t(r) * (r - 1) / 2; };
  while (i > 0 && start(i) > l) --i;
  while (i < nb - 1 && start(i + 1) <= l) ++i;
  I = i;
  J = i + int(l - start(i));
}

// What one pair item adds on both sides, and the scaling of the sums.
template <bool kForce>
struct SymBody;

// Kelvin force: f_ij into the target, -f_ij into the source.
template <>
struct SymBody<true> {
  static constexpr float kSrcSign = -1.f;
  // Targets from the AoS records (a force product always has them; reading
  // them from the pair records cost 3 % in the force kernel at N = 65,536).
  static constexpr bool kAosTargets = true;
  static constexpr int kSplit = kSymSplit, kPair = kSymPair;
  __device__ static float near2(const PairConsts<float>& pc) { return pc.near2_force; }
  __device__ static float scale() { return float(kForceK); }
  __device__ static void pair(float2 tx, float2 ty, float2 tz, float2 tmx, float2 tmy, float2 tmz,
                              const PairItems::Item& it, float near2, float2* acc, float2* src) {
    sym_force_pair2(tx, ty, tz, tmx, tmy, tmz, it, near2, acc, src);
  }
};

// Dipole field: the target gets T m_s, the source T m_t, each accumulated as
// -(3 d (d.m) r^-5 - m r^-3) = d (d.m) (-3 r^-5) + m r^-3 with FMAs straight
// into the sums (30 packed operations per target and item); the scale
// -1/(4 pi) gives the all-pairs field kernels' output units.
template <>
struct SymBody<false> {
  static constexpr float kSrcSign = 1.f;
  static constexpr bool kAosTargets = false;  // a field product carries the pair records only
  static constexpr int kSplit = 2, kPair = 2;
  __device__ static float near2(const PairConsts<float>& pc) { return pc.near2_field; }
  __device__ static float scale() { return -float(kInv4Pi); }
  __device__ static void pair(float2 tx, float2 ty, float2 tz, float2 tmx, float2 tmy, float2 tmz,
                              const PairItems::Item& it, float near2, float2* acc, float2* src) {
    sym_field_pair2(tx, ty, tz, tmx, tmy, tmz, it, near2, acc, src);
  }
};

// Particle g of the pair-layout records (two particles per 32-byte item):
// component k of lane g & 1.
__device__ __forceinline__ float3 pair_rec(const float4* __restrict__ p4, int64_t g) {
  const int64_t b = g & ~int64_t(1);
  const float4 p0 = p4[b], p1 = p4[b + 1];
  return (g & 1) ? make_float3(p0.y, p0.w, p1.y) : make_float3(p0.x, p0.z, p1.x);
}

__device__ __forceinline__ bool scene_done(const AllPairsArgs<float>& a, const SceneDesc<float>& sc) {
  return a.done_flags && a.done_flags[int64_t(sc.flag_index) * a.done_stride] != 0.0;
}

template <bool kForce>
__global__ void __launch_bounds__(kSymTPB) k_sym(const AllPairsArgs<float> a, float* __restrict__ part) {
  using BodyT = SymBody<kForce>;
  constexpr int TPB = kSymTPB, TPT = kSymTPT, TB = kSymTB, STAGES = kSymStages;
  constexpr int SPLIT = BodyT::kSplit, NH = TB / 2 / SPLIT, P = BodyT::kPair;
  constexpr int NV = P * 6 <= 8 ? 8 : (P * 6 <= 16 ? 16 : 32);
  static_assert(NH % P == 0, "phase items");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  // per warp: the source sums of the phase's pair items, [item][component * 2 + source of the pair]
  // (row stride 6: the lanes' writes of one item, and 32 threads' reads of
  // consecutive sources, fall in distinct banks)
  __shared__ float s_srcf[kSymWarps][NH * 6];

  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int64_t T = a.total_steps, G = gridDim.x, b = blockIdx.x;
  const int64_t k_begin = step_start(T, G, b), k_end = step_start(T, G, b + 1);
  if (k_begin >= k_end) return;
  // A launch whose solves have all stopped does nothing.
  if (a.n_scenes == 1 && scene_done(a, a.scenes[0])) return;
  if (a.done_count && *a.done_count >= a.done_total) return;
  auto stage_pos = [&](int s) { return reinterpret_cast<float4*>(smem_raw) + size_t(s) * 2 * TB; };
  auto stage_mom = [&](int s) { return stage_pos(s) + TB; };
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) mbar_init(&full_bar[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // Producer (thread 0): stage source block J of step k into stage s.
  auto issue = [&](int64_t k, int s) {
    const int si = find_scene(a.scenes, a.n_scenes, k);
    const SceneDesc<float>& sc = a.scenes[si];
    int I, J;
    sym_block_pair(k - sc.step_off, sc.n_tb, I, J);
    const int64_t first = sc.s_off + int64_t(J) * TB;
    const int64_t rem = sc.ns - int64_t(J) * TB;
    const int cnt = int(rem < TB ? rem : TB);
    const uint32_t bytes = PairItems::tile_bytes(cnt);
    mbar_arrive_expect_tx(&full_bar[s], 2 * bytes);
    bulk_g2s(stage_pos(s), a.spos + first, bytes, &full_bar[s]);
    bulk_g2s(stage_mom(s), a.smom + first, bytes, &full_bar[s]);
  };
  if (tid == 0)
    for (int s = 0; s < STAGES && k_begin + s < k_end; ++s) issue(k_begin + s, s);

  float2 tx[TPT], ty[TPT], tz[TPT], tmx[TPT], tmy[TPT], tmz[TPT];
  int cur_si = -1, cur_I = -1;
  int64_t k_fail = -1;
  for (int64_t k = k_begin; k < k_end; ++k) {
    const int64_t u = k - k_begin;
    const int s = int(u % STAGES);
    const int si = find_scene(a.scenes, a.n_scenes, k);
    const SceneDesc<float>& sc = a.scenes[si];
    const int nb = sc.n_tb;
    int I, J;
    sym_block_pair(k - sc.step_off, nb, I, J);
    if (si != cur_si || I != cur_I) {  // the targets of block I
      // Slots past the scene's end hold a zero dipole: their terms vanish
      // on the source side of every pair, and their own sums are not read.
#pragma unroll
      for (int t = 0; t < TPT; ++t) {
        const int64_t li = int64_t(I) * TB + t * TPB + tid;
        const bool live = li < sc.nt;
        float3 p, m;
        if constexpr (BodyT::kAosTargets) {
          const float4 q = a.tpos[sc.t_off + (live ? li : 0)];
          const float4 w = live ? a.tmom[sc.t_off + li] : make_float4(0.f, 0.f, 0.f, 0.f);
          p = make_float3(q.x, q.y, q.z);
          m = make_float3(w.x, w.y, w.z);
        } else {
          p = pair_rec(a.spos, sc.t_off + (live ? li : 0));
          m = live ? pair_rec(a.smom, sc.t_off + li) : make_float3(0.f, 0.f, 0.f);
        }
        tx[t] = f2_dup(p.x);
        ty[t] = f2_dup(p.y);
        tz[t] = f2_dup(p.z);
        tmx[t] = f2_dup(m.x);
        tmy[t] = f2_dup(m.y);
        tmz[t] = f2_dup(m.z);
      }
      cur_si = si;
      cur_I = I;
    }
    const bool ok = mbar_wait_bounded(&full_bar[s], uint32_t((u / STAGES) & 1), stage_wait_limit(a.stage_wait_debug));
    if (__syncthreads_or(!ok)) {
      k_fail = k;
      break;
    }
    // A stopped scene's sums are not written (block-uniform).  A force
    // product's flags mark the scenes whose force comes from kept sums.
    if (!scene_done(a, sc)) {
      const bool sym = I != J;
      const int64_t rem = sc.ns - int64_t(J) * TB;
      const int cnt = int(rem < TB ? rem : TB);
      const int n_items = PairItems::items(cnt);
      const float4* __restrict__ sp = stage_pos(s);
      const float4* __restrict__ smv = stage_mom(s);
      const float near2 = BodyT::near2(sc.pc);
      const float kk = BodyT::scale();
      float2 acc[TPT][3];
#pragma unroll
      for (int t = 0; t < TPT; ++t) acc[t][0] = acc[t][1] = acc[t][2] = make_float2(0.f, 0.f);
      for (int h = 0; h < SPLIT; ++h) {
        const int j_end = min(n_items, (h + 1) * NH);
#pragma unroll 2
        for (int j0 = h * NH; j0 < j_end; j0 += P) {
          float v[NV];
#pragma unroll
          for (int q = 0; q < NV; ++q) v[q] = 0.f;
#pragma unroll
          for (int p = 0; p < P; ++p) {
            // An item past the tile's end is a zero dipole at the origin:
            // nothing on the target side; its source-side sums belong to
            // slots past the scene's end, which are never read.
            const bool in = p == 0 || j0 + p < j_end;
            const PairItems::Item it =
                in ? PairItems::load_item(sp, smv, j0 + p) : PairItems::Item{{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f},
                                                                            {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
            float2 src[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
            for (int t = 0; t < TPT; ++t) BodyT::pair(tx[t], ty[t], tz[t], tmx[t], tmy[t], tmz[t], it, near2, acc[t], src);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              v[p * 6 + 2 * c] = src[c].x;
              v[p * 6 + 2 * c + 1] = src[c].y;
            }
          }
          if (sym) {  // warp-uniform
            const float w = warp_reduce_scatter<NV>(v, lane);
            const int kv = lane / (32 / NV);
            if (lane % (32 / NV) == 0 && kv < 6 * P) s_srcf[wid][(j0 - h * NH) * 6 + kv] = w;
          }
        }
        if (sym) {
          __syncthreads();  // the phase's s_srcf is complete
          // sums for block J from block I: sources 2 h NH .. 2 (h + 1) NH - 1
          float* ps = part + (sc.tb_off + int64_t(J) * nb + I) * 3 * TB;
          const float ks = kk * BodyT::kSrcSign;
          for (int r = tid; r < 2 * NH; r += TPB) {
            const int j = r >> 1, rr = h * 2 * NH + r;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              float x = 0.f;
#pragma unroll
              for (int w = 0; w < kSymWarps; ++w) x += s_srcf[w][j * 6 + 2 * c + (r & 1)];
              ps[c * TB + rr] = x * ks;
            }
          }
          if (h + 1 < SPLIT) __syncthreads();  // read before the next phase overwrites it
        }
      }
      float* pr = part + (sc.tb_off + int64_t(I) * nb + J) * 3 * TB;  // sums for block I from block J
#pragma unroll
      for (int t = 0; t < TPT; ++t) {
        const int r = t * TPB + tid;
#pragma unroll
        for (int c = 0; c < 3; ++c) pr[c * TB + r] = (acc[t][c].x + acc[t][c].y) * kk;
      }
    }
    __syncthreads();  // every thread is done with stage s and with s_srcf
    if (tid == 0 && k + STAGES < k_end) {
      fence_proxy_async_smem();
      issue(k + STAGES, s);
    }
  }

  if (k_fail >= 0) {
    if (tid == 0) {
      atomicExch(a.err, MF_DEVERR_STAGE_TIMEOUT);
      // Copies in flight: steps k_fail .. min(k_end, k_fail + STAGES) - 1, one
      // per stage.  Wait for each (bounded) before the CTA leaves.
      const int64_t k_stop = (k_fail + STAGES < k_end) ? k_fail + STAGES : k_end;
      bool drained = true;
      for (int64_t kk = k_fail; kk < k_stop; ++kk) {
        const int64_t uu = kk - k_begin;
        if (!mbar_wait_bounded(&full_bar[uu % STAGES], uint32_t((uu / STAGES) & 1))) drained = false;
      }
      if (!drained) atomicExch(a.err, MF_DEVERR_DRAIN_TIMEOUT);
    }
    __syncthreads();
  }
}

// Per particle: the nb partner-block sums of its block, compensated FP32
// (sum and carried rounding error) in four chains over the blocks X = q
// (mod 4) -- a fixed order, with four independent chains in flight -- the
// chains combined in FP64 as (c0 + c1) + (c2 + c3); then the body's
// epilogue.  g runs over [g0, g0 + n_span), the particle indices from the
// first scene's start to the last one's end (scenes are in increasing t_off
// order; indices between scenes are skipped, and so are stopped scenes).
template <bool kForce>
__global__ void k_sym_finish(const AllPairsArgs<float> a, const float* __restrict__ part, int64_t g0,
                             int64_t n_span) {
  if (a.done_count && *a.done_count >= a.done_total) return;
  for (int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < n_span;
       g += int64_t(gridDim.x) * blockDim.x) {
    const int64_t gi = g0 + g;
    int lo = 0, hi = a.n_scenes - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.scenes[mid].t_off <= gi) lo = mid;
      else hi = mid - 1;
    }
    const SceneDesc<float>& sc = a.scenes[lo];
    const int64_t i = gi - sc.t_off;
    if (i >= sc.nt) continue;  // the padding slot after an odd scene, or a scene not in the plan
    if (scene_done(a, sc)) continue;
    const int K = int(i / kSymTB), r = int(i % kSymTB);
    const int nb = sc.n_tb;
    const float* row = part + (sc.tb_off + int64_t(K) * nb) * 3 * kSymTB;
    float s4[4][3] = {}, e4[4][3] = {};
    int X = 0;
    for (; X + 4 <= nb; X += 4) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float* p = row + int64_t(X + q) * 3 * kSymTB;
#pragma unroll
        for (int c = 0; c < 3; ++c) two_sum_acc(s4[q][c], e4[q][c], __ldcg(p + c * kSymTB + r));
      }
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      if (X + q < nb) {
        const float* p = row + int64_t(X + q) * 3 * kSymTB;
#pragma unroll
        for (int c = 0; c < 3; ++c) two_sum_acc(s4[q][c], e4[q][c], __ldcg(p + c * kSymTB + r));
      }
    }
    double v[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double w[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) w[q] = double(s4[q][c]) + double(e4[q][c]);
      v[c] = (w[0] + w[1]) + (w[2] + w[3]);
    }
    if constexpr (kForce) {
      const float4 m = a.tmom[gi];
      force_epilogue<float>(a, sc, gi, double(m.x), double(m.y), double(m.z), v);
    } else {
      FieldBody<float>::epilogue(a, sc, gi, FieldBody<float>::TData{}, v);
    }
  }
}

// ---------------------------------------------------------------------------
// The field and the Kelvin force over the same dipoles in one launch.
//
// A time step whose solve starts from a converged warm start evaluates the
// field of the magnetization (the residual) and then the force of that same
// magnetization.  Both products sweep the same unordered pairs and share the
// pair's separation, r^2 and the dots d.m_s, d.m_t, so this kernel evaluates
// both in one sweep (sym_field_force_pair2).  The field sums go through the
// field's epilogue as k_sym_finish<false> applies it; the force sums (for
// dipoles b, not yet scaled to M = c b) are kept per particle in FP64 and
// applied by k_sym_force_from_sums once the solve has confirmed that b did
// not change.  Blocks of 1,024 particles (128 threads x 8 targets) as in
// k_sym; the two bodies' sums take twice the registers of one, so the kernel
// runs at 255 registers with a few bytes spilled, and the source sums of a
// tile are reduced in four phases (a phase's per-warp buffer fits the static
// shared memory).
// ---------------------------------------------------------------------------
// Measured at N = 65,536 / 131,072 (ms per fused launch with its finish;
// targets per thread, CTAs per SM, phases): 4, 3, 2 (166 registers) 4.90 /
// 18.54; 6, 2, 2 (242) 4.63 / 17.93; 8, 2, 4 (255, 124 bytes of spills)
// 4.54 / 18.05.  The separate products take 5.36 / 21.37.
constexpr int kFfTPB = 128, kFfTPT = 8, kFfStages = 2, kFfMinBlocks = 2;
constexpr int kFfTB = kFfTPB * kFfTPT;
constexpr int kFfWarps = kFfTPB / 32;
constexpr size_t kFfSmem = size_t(kFfStages) * 2 * kFfTB * sizeof(float4);
constexpr int kFfSplit = 4;  // phases per tile: the per-warp source sums of one phase fit the static smem
constexpr int kFfNH = kFfTB / 2 / kFfSplit;  // pair items per phase
// Per item, 12 source sums: field x, y, z then force x, y, z, each for the
// item's two sources.  Row stride 13 (odd): one item's 12 lane writes, and
// the phase-end reads of 32 consecutive sources, fall in distinct banks.
constexpr int kFfRow = 13;

__global__ void __launch_bounds__(kFfTPB, kFfMinBlocks) k_sym_ff(const AllPairsArgs<float> a, float* __restrict__ partf,
                                                                float* __restrict__ partg) {
  constexpr int TPB = kFfTPB, TPT = kFfTPT, TB = kFfTB, STAGES = kFfStages, SPLIT = kFfSplit, NH = kFfNH;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ float s_src[kFfWarps][NH * kFfRow];

  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int64_t T = a.total_steps, G = gridDim.x, b = blockIdx.x;
  const int64_t k_begin = step_start(T, G, b), k_end = step_start(T, G, b + 1);
  if (k_begin >= k_end) return;
  if (a.n_scenes == 1 && scene_done(a, a.scenes[0])) return;
  if (a.done_count && *a.done_count >= a.done_total) return;
  auto stage_pos = [&](int s) { return reinterpret_cast<float4*>(smem_raw) + size_t(s) * 2 * TB; };
  auto stage_mom = [&](int s) { return stage_pos(s) + TB; };
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) mbar_init(&full_bar[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto issue = [&](int64_t k, int s) {
    const int si = find_scene(a.scenes, a.n_scenes, k);
    const SceneDesc<float>& sc = a.scenes[si];
    int I, J;
    sym_block_pair(k - sc.step_off, sc.n_tb, I, J);
    const int64_t first = sc.s_off + int64_t(J) * TB;
    const int64_t rem = sc.ns - int64_t(J) * TB;
    const int cnt = int(rem < TB ? rem : TB);
    const uint32_t bytes = PairItems::tile_bytes(cnt);
    mbar_arrive_expect_tx(&full_bar[s], 2 * bytes);
    bulk_g2s(stage_pos(s), a.spos + first, bytes, &full_bar[s]);
    bulk_g2s(stage_mom(s), a.smom + first, bytes, &full_bar[s]);
  };
  if (tid == 0)
    for (int s = 0; s < STAGES && k_begin + s < k_end; ++s) issue(k_begin + s, s);

  float2 tx[TPT], ty[TPT], tz[TPT], tmx[TPT], tmy[TPT], tmz[TPT];
  int cur_si = -1, cur_I = -1;
  int64_t k_fail = -1;
  for (int64_t k = k_begin; k < k_end; ++k) {
    const int64_t u = k - k_begin;
    const int s = int(u % STAGES);
    const int si = find_scene(a.scenes, a.n_scenes, k);
    const SceneDesc<float>& sc = a.scenes[si];
    const int nb = sc.n_tb;
    int I, J;
    sym_block_pair(k - sc.step_off, nb, I, J);
    if (si != cur_si || I != cur_I) {
#pragma unroll
      for (int t = 0; t < TPT; ++t) {
        const int64_t li = int64_t(I) * TB + t * TPB + tid;
        const bool live = li < sc.nt;
        const float3 p = pair_rec(a.spos, sc.t_off + (live ? li : 0));
        const float3 m = live ? pair_rec(a.smom, sc.t_off + li) : make_float3(0.f, 0.f, 0.f);
        tx[t] = f2_dup(p.x);
        ty[t] = f2_dup(p.y);
        tz[t] = f2_dup(p.z);
        tmx[t] = f2_dup(m.x);
        tmy[t] = f2_dup(m.y);
        tmz[t] = f2_dup(m.z);
      }
      cur_si = si;
      cur_I = I;
    }
    const bool ok = mbar_wait_bounded(&full_bar[s], uint32_t((u / STAGES) & 1), stage_wait_limit(a.stage_wait_debug));
    if (__syncthreads_or(!ok)) {
      k_fail = k;
      break;
    }
    if (!scene_done(a, sc)) {
      const bool sym = I != J;
      const int64_t rem = sc.ns - int64_t(J) * TB;
      const int cnt = int(rem < TB ? rem : TB);
      const int n_items = PairItems::items(cnt);
      const float4* __restrict__ sp = stage_pos(s);
      const float4* __restrict__ smv = stage_mom(s);
      const float nf2 = sc.pc.near2_field, ng2 = sc.pc.near2_force;
      const float kf = -float(kInv4Pi), kg = float(kForceK);
      float2 accf[TPT][3], accg[TPT][3];
#pragma unroll
      for (int t = 0; t < TPT; ++t)
#pragma unroll
        for (int c = 0; c < 3; ++c) accf[t][c] = accg[t][c] = make_float2(0.f, 0.f);
      for (int h = 0; h < SPLIT; ++h) {
        const int j_end = min(n_items, (h + 1) * NH);
#pragma unroll 2
        for (int j = h * NH; j < j_end; ++j) {
          const PairItems::Item it = PairItems::load_item(sp, smv, j);
          float2 srcf[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
          float2 srcg[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
          for (int t = 0; t < TPT; ++t)
            sym_field_force_pair2(tx[t], ty[t], tz[t], tmx[t], tmy[t], tmz[t], it, nf2, ng2, accf[t], accg[t], srcf,
                                  srcg);
          if (sym) {  // warp-uniform
            float v[16];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              v[2 * c] = srcf[c].x;
              v[2 * c + 1] = srcf[c].y;
              v[6 + 2 * c] = srcg[c].x;
              v[6 + 2 * c + 1] = srcg[c].y;
            }
            v[12] = v[13] = v[14] = v[15] = 0.f;
            const float w = warp_reduce_scatter<16>(v, lane);
            const int kv = lane >> 1;
            if ((lane & 1) == 0 && kv < 12) s_src[wid][(j - h * NH) * kFfRow + kv] = w;
          }
        }
        if (sym) {
          __syncthreads();  // the phase's s_src is complete
          // sums for block J from block I: sources 2 h NH .. 2 (h + 1) NH - 1
          const int64_t off = (sc.tb_off + int64_t(J) * nb + I) * 3 * TB;
          for (int r = tid; r < 2 * NH; r += TPB) {
            const int j = r >> 1, rr = h * 2 * NH + r;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              float xf = 0.f, xg = 0.f;
#pragma unroll
              for (int w = 0; w < kFfWarps; ++w) {
                xf += s_src[w][j * kFfRow + 2 * c + (r & 1)];
                xg += s_src[w][j * kFfRow + 6 + 2 * c + (r & 1)];
              }
              partf[off + c * TB + rr] = xf * kf;
              partg[off + c * TB + rr] = -(xg * kg);  // f_ji = -f_ij
            }
          }
          if (h + 1 < SPLIT) __syncthreads();  // read before the next phase overwrites it
        }
      }
      const int64_t off = (sc.tb_off + int64_t(I) * nb + J) * 3 * TB;  // sums for block I from block J
#pragma unroll
      for (int t = 0; t < TPT; ++t) {
        const int r = t * TPB + tid;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          partf[off + c * TB + r] = (accf[t][c].x + accf[t][c].y) * kf;
          partg[off + c * TB + r] = (accg[t][c].x + accg[t][c].y) * kg;
        }
      }
    }
    __syncthreads();  // every thread is done with stage s and with s_src
    if (tid == 0 && k + STAGES < k_end) {
      fence_proxy_async_smem();
      issue(k + STAGES, s);
    }
  }

  if (k_fail >= 0) {
    if (tid == 0) {
      atomicExch(a.err, MF_DEVERR_STAGE_TIMEOUT);
      const int64_t k_stop = (k_fail + STAGES < k_end) ? k_fail + STAGES : k_end;
      bool drained = true;
      for (int64_t kk = k_fail; kk < k_stop; ++kk) {
        const int64_t uu = kk - k_begin;
        if (!mbar_wait_bounded(&full_bar[uu % STAGES], uint32_t((uu / STAGES) & 1))) drained = false;
      }
      if (!drained) atomicExch(a.err, MF_DEVERR_DRAIN_TIMEOUT);
    }
    __syncthreads();
  }
}

// A particle's nb partner-block sums of one row of part (block size TB), in
// the fixed order and compensated arithmetic of k_sym_finish.
template <int TB>
__device__ __forceinline__ void sum_block_row(const float* __restrict__ row, int nb, int r, double* v) {
  float s4[4][3] = {}, e4[4][3] = {};
  int X = 0;
  for (; X + 4 <= nb; X += 4) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float* p = row + int64_t(X + q) * 3 * TB;
#pragma unroll
      for (int c = 0; c < 3; ++c) two_sum_acc(s4[q][c], e4[q][c], __ldcg(p + c * TB + r));
    }
  }
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    if (X + q < nb) {
      const float* p = row + int64_t(X + q) * 3 * TB;
#pragma unroll
      for (int c = 0; c < 3; ++c) two_sum_acc(s4[q][c], e4[q][c], __ldcg(p + c * TB + r));
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) w[q] = double(s4[q][c]) + double(e4[q][c]);
    v[c] = (w[0] + w[1]) + (w[2] + w[3]);
  }
}

// Per particle: the field's epilogue on its summed row of partf, and the
// force's summed row of partg kept in gsum[3 i + c] (FP64).
__global__ void k_sym_ff_finish(const AllPairsArgs<float> a, const float* __restrict__ partf,
                                const float* __restrict__ partg, double* __restrict__ gsum, int64_t g0, int64_t n_span) {
  if (a.done_count && *a.done_count >= a.done_total) return;
  for (int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < n_span;
       g += int64_t(gridDim.x) * blockDim.x) {
    const int64_t gi = g0 + g;
    int lo = 0, hi = a.n_scenes - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.scenes[mid].t_off <= gi) lo = mid;
      else hi = mid - 1;
    }
    const SceneDesc<float>& sc = a.scenes[lo];
    const int64_t i = gi - sc.t_off;
    if (i >= sc.nt) continue;
    if (scene_done(a, sc)) continue;
    const int K = int(i / kFfTB), r = int(i % kFfTB);
    const int nb = sc.n_tb;
    const int64_t row = (sc.tb_off + int64_t(K) * nb) * 3 * kFfTB;
    double v[3];
    sum_block_row<kFfTB>(partg + row, nb, r, v);
    gsum[3 * gi] = v[0];
    gsum[3 * gi + 1] = v[1];
    gsum[3 * gi + 2] = v[2];
    sum_block_row<kFfTB>(partf + row, nb, r, v);
    FieldBody<float>::epilogue(a, sc, gi, FieldBody<float>::TData{}, v);
  }
}

// The force's epilogue on kept sums: the pair sums of dipoles b scaled by
// c^2 (the force is bilinear in the dipoles, M = c b), then the correction,
// the external gradient term and the scene's scale, as k_sym_finish<true>
// applies them.  a carries the force plan's scenes and the dipoles M.
__global__ void k_sym_force_from_sums(const AllPairsArgs<float> a, const double* __restrict__ gsum, double c2,
                                      const double* __restrict__ kept, const double* __restrict__ rows,
                                      int row_stride, int c_index, int64_t g0, int64_t n_span) {
  for (int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < n_span;
       g += int64_t(gridDim.x) * blockDim.x) {
    const int64_t gi = g0 + g;
    int lo = 0, hi = a.n_scenes - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.scenes[mid].t_off <= gi) lo = mid;
      else hi = mid - 1;
    }
    const SceneDesc<float>& sc = a.scenes[lo];
    if (gi - sc.t_off >= sc.nt) continue;
    if (kept && kept[sc.flag_index] == 0.0) continue;  // this scene's force comes from its own product
    double cc = c2;
    if (rows) {
      const double c = double(float(rows[int64_t(sc.flag_index) * row_stride + c_index]));
      cc = c * c;
    }
    const double v[3] = {gsum[3 * gi] * cc, gsum[3 * gi + 1] * cc, gsum[3 * gi + 2] * cc};
    const float4 m = a.tmom[gi];
    force_epilogue<float>(a, sc, gi, double(m.x), double(m.y), double(m.z), v);
  }
}

// Resident CTAs of k_sym<kForce> on the current device (its shared-memory
// attribute set on the first call).  Plans call it when they are built, so
// a launch inside a stream capture makes no attribute or occupancy calls.
template <bool kForce>
mf_status sym_grid_max(int* out) {
  static std::mutex mu;
  static int cache[64] = {};
  const int dev = current_device();
  std::lock_guard<std::mutex> lk(mu);
  int& g = cache[dev >= 0 && dev < 64 ? dev : 0];
  if (!g) {
    MF_CUDA_TRY(cudaFuncSetAttribute(k_sym<kForce>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSymSmem)));
    int per_sm = 0;
    MF_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sym<kForce>, kSymTPB, kSymSmem));
    g = std::max(per_sm, 1) * device_sms(dev);
  }
  *out = g;
  return MF_OK;
}

mf_status sym_grid(Body body, int* out) {
  return body == Body::ForceF2 ? sym_grid_max<true>(out) : sym_grid_max<false>(out);
}

mf_status ff_grid(int* out) {
  static std::mutex mu;
  static int cache[64] = {};
  const int dev = current_device();
  std::lock_guard<std::mutex> lk(mu);
  int& g = cache[dev >= 0 && dev < 64 ? dev : 0];
  if (!g) {
    MF_CUDA_TRY(cudaFuncSetAttribute(k_sym_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kFfSmem)));
    int per_sm = 0;
    MF_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sym_ff, kFfTPB, kFfSmem));
    g = std::max(per_sm, 1) * device_sms(dev);
  }
  *out = g;
  return MF_OK;
}

AllPairsArgs<float> sym_args(const Plan<float>& plan, const LaunchIO<float>& io, int32_t* err) {
  AllPairsArgs<float> a;
  memset(&a, 0, sizeof(a));
  a.scenes = plan.d_scenes.as<SceneDesc<float>>();
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
  a.err = err;
  a.stage_wait_debug = stage_wait_debug();
  return a;
}

}  // namespace

bool sym_eligible(Body body, const std::vector<SceneSpec>& specs) {
  if (body != Body::FieldF2 && body != Body::ForceF2) return false;
  for (const SceneSpec& s : specs)
    if (s.nt <= 0 || s.nt != s.ns || s.t_off != s.s_off || s.t_off % 2) return false;
  return !specs.empty();
}

namespace {

// A pair-symmetric plan of blocks of tb particles.
mf_status build_blocks_plan(Body body, const std::vector<SceneSpec>& specs, int64_t tb, Plan<float>& plan) {
  if (!sym_eligible(body, specs))
    return fail(MF_ERR_INVALID_ARG,
                "pair-symmetric plan: packed field or force, targets equal to the sources, scenes at even indices");
  plan.body = body;
  plan.shape = kShapeSym;
  plan.host.clear();
  int64_t step = 0, blocks = 0;
  double pairs = 0, evals = 0;
  for (const SceneSpec& s : specs) {
    if (!(s.h > 0.0)) return fail(MF_ERR_INVALID_ARG, "build_plan: smoothing length must be > 0");
    SceneDesc<float> d;
    memset(&d, 0, sizeof(d));
    d.t_off = s.t_off;
    d.nt = s.nt;
    d.s_off = s.s_off;
    d.ns = s.ns;
    const int64_t nb = (s.nt + tb - 1) / tb;
    d.n_tb = int32_t(nb);
    d.n_tiles = int32_t(nb);
    d.step_off = step;
    d.tb_off = blocks;  // first block pair of this scene in the partial array
    d.flag_index = s.flag_index >= 0 ? s.flag_index : int32_t(plan.host.size());
    fill_scene_coefs<float>(s, d);
    step += nb * (nb + 1) / 2;
    blocks += nb * nb;
    pairs += double(s.nt) * double(s.ns);
    evals += double(s.nt) * double(s.nt - 1) * 0.5;
    plan.host.push_back(d);
  }
  plan.total_steps = step;
  plan.total_tb = blocks;
  plan.n_scenes = int32_t(plan.host.size());
  plan.pairs = pairs;
  plan.evals = evals;
  const size_t bytes = plan.host.size() * sizeof(SceneDesc<float>);
  MF_TRY(plan.d_scenes.reserve_grow(bytes));
  if (bytes) MF_CUDA_TRY(cudaMemcpy(plan.d_scenes.ptr, plan.host.data(), bytes, cudaMemcpyHostToDevice));
  return MF_OK;
}

}  // namespace

mf_status build_sym_plan(Body body, const std::vector<SceneSpec>& specs, Plan<float>& plan) {
  MF_TRY(build_blocks_plan(body, specs, kSymTB, plan));
  int gmax = 0;
  return sym_grid(body, &gmax);  // sets the kernel's attributes outside any stream capture
}

void sym_needs(const Plan<float>& plan, size_t* partial_doubles) {
  // FP32 block sums: 3 x TB per ordered block pair, in doubles
  *partial_doubles = (size_t(plan.total_tb) * 3 * kSymTB + 1) / 2;
}

mf_status run_sym(const Plan<float>& plan, const LaunchIO<float>& io, double* partials, int32_t* err,
                  cudaStream_t st) {
  if (plan.total_steps <= 0) return MF_OK;
  const bool force = plan.body == Body::ForceF2;
  int gmax = 0;
  MF_TRY(sym_grid(plan.body, &gmax));
  const AllPairsArgs<float> a = sym_args(plan, io, err);
  float* part = reinterpret_cast<float*>(partials);
  const int64_t g = std::min<int64_t>(plan.total_steps, gmax);
  const int64_t g0 = plan.host.front().t_off;
  const int64_t n_span = plan.host.back().t_off + plan.host.back().nt - g0;
  const int64_t fb = std::min<int64_t>((n_span + 255) / 256, 8192);
  if (force) {
    k_sym<true><<<unsigned(g), kSymTPB, kSymSmem, st>>>(a, part);
    MF_CUDA_TRY(cudaGetLastError());
    k_sym_finish<true><<<unsigned(fb), 256, 0, st>>>(a, part, g0, n_span);
  } else {
    k_sym<false><<<unsigned(g), kSymTPB, kSymSmem, st>>>(a, part);
    MF_CUDA_TRY(cudaGetLastError());
    k_sym_finish<false><<<unsigned(fb), 256, 0, st>>>(a, part, g0, n_span);
  }
  MF_CUDA_TRY(cudaGetLastError());
  return MF_OK;
}

mf_status build_symff_plan(const std::vector<SceneSpec>& specs, Plan<float>& plan) {
  MF_TRY(build_blocks_plan(Body::FieldF2, specs, kFfTB, plan));
  int gmax = 0;
  return ff_grid(&gmax);
}

void symff_needs(const Plan<float>& plan, size_t* partial_doubles) {
  // two FP32 arrays (field, force) of 3 x TB per ordered block pair, in doubles
  *partial_doubles = size_t(plan.total_tb) * 3 * kFfTB;
}

mf_status run_symff(const Plan<float>& plan, const LaunchIO<float>& io, double* partials, double* gsum,
                    int32_t* err, cudaStream_t st) {
  if (plan.total_steps <= 0) return MF_OK;
  if (plan.body != Body::FieldF2 || plan.host.empty() || plan.host.front().n_tb * int64_t(kFfTB) < plan.host.front().nt)
    return fail(MF_ERR_INVALID_ARG, "run_symff: not a field-and-force plan");
  int gmax = 0;
  MF_TRY(ff_grid(&gmax));
  const AllPairsArgs<float> a = sym_args(plan, io, err);
  float* partf = reinterpret_cast<float*>(partials);
  float* partg = partf + size_t(plan.total_tb) * 3 * kFfTB;
  const int64_t g = std::min<int64_t>(plan.total_steps, gmax);
  const int64_t g0 = plan.host.front().t_off;
  const int64_t n_span = plan.host.back().t_off + plan.host.back().nt - g0;
  const int64_t fb = std::min<int64_t>((n_span + 255) / 256, 8192);
  k_sym_ff<<<unsigned(g), kFfTPB, kFfSmem, st>>>(a, partf, partg);
  MF_CUDA_TRY(cudaGetLastError());
  k_sym_ff_finish<<<unsigned(fb), 256, 0, st>>>(a, partf, partg, gsum, g0, n_span);
  MF_CUDA_TRY(cudaGetLastError());
  return MF_OK;
}

int default_fused_mode() {
  static const int mode = [] {
    const char* e = getenv("MF_FUSED_PRODUCTS");
    return (e && (e[0] == '0' || e[0] == '2') && e[1] == 0) ? e[0] - '0' : 1;
  }();
  return mode;
}

mf_status run_sym_force_from_sums(const Plan<float>& plan, const LaunchIO<float>& io, const double* gsum, double c2,
                                  const double* kept, const double* rows, int row_stride, int c_index, int32_t* err,
                                  cudaStream_t st) {
  if (plan.host.empty()) return MF_OK;
  const AllPairsArgs<float> a = sym_args(plan, io, err);
  const int64_t g0 = plan.host.front().t_off;
  const int64_t n_span = plan.host.back().t_off + plan.host.back().nt - g0;
  const int64_t fb = std::min<int64_t>((n_span + 255) / 256, 8192);
  k_sym_force_from_sums<<<unsigned(fb), 256, 0, st>>>(a, gsum, c2, kept, rows, row_stride, c_index, g0, n_span);
  MF_CUDA_TRY(cudaGetLastError());
  return MF_OK;
}

}  // namespace mfgb
