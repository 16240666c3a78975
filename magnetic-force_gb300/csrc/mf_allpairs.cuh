// mf_allpairs.cuh -- persistent all-pairs tile kernel for sm_103a.
//
// One launch evaluates sum_j K(x_i - y_j) * s_j for every target i of one or
// more independent scenes (a scene = a contiguous target range and a
// contiguous source range with its own smoothing length and epilogue scale).
//
// Work layout.  Each scene's targets are cut into target blocks of
// TPB * TPT targets (TPT targets per thread, strided by TPB for coalescing)
// and its sources into tiles of TILE sources.  The (target block, source tile)
// pairs of all scenes form one flat "step" space that is split evenly over a
// grid of resident CTAs, so every SM gets the same number of tile-steps
// whatever the scene sizes are.  A CTA walks its contiguous step range:
//   * source tiles are staged in shared memory by 1-D bulk copies
//     (cp.async.bulk, completion on an mbarrier), STAGES deep, issued by one
//     thread, no cluster multicast;
//   * each thread keeps TPT targets in registers and sweeps the tile with
//     broadcast shared-memory reads;
//   * per target the tile's sum is formed in plain FP32 and folded into the
//     running sum with two-sum compensation (FP64 kernels add directly);
//   * a target block completely covered by one CTA is finished in place; the
//     first and last target blocks of a CTA's range may be shared with a
//     neighbour CTA, which write FP64 partials to scratch, and the last of
//     them to arrive (atomic ticket) adds the partials in CTA order, so the
//     result does not depend on scheduling.
#pragma once
#include <cstdint>

#include "mf_device.cuh"
#include "mf_pair.cuh"

namespace mfgb {

// The fitted force curves for the FP32 exact-branch body (staged into shared
// memory by each CTA).
static __constant__ float c_fit_ap[40] = MF_FITTED_CURVE_TABLE;

template <class Real>
struct SceneDesc {
  int64_t t_off, nt;     // target index range
  int64_t s_off, ns;     // source index range
  int64_t step_off;      // first flat step of this scene
  int64_t tb_off;        // first global target-block index of this scene
  int32_t n_tiles;       // ceil(ns / TILE)
  int32_t n_tb;          // ceil(nt / (TPB*TPT))
  int32_t flag_index;    // this scene's row in the launch's done_flags
  int32_t pad_;
  PairConsts<Real> pc;
  // Field epilogue: out = scale * value + coef_add * add4 + coef_add2 * add4b + cvec.
  // Force / tensor epilogues use scale only.
  Real scale;
  Real coef_add;
  Real coef_add2;
  Real cvec[3];
};

template <class Real>
struct AllPairsArgs {
  using R4 = typename Vec4T<Real>::type;
  const SceneDesc<Real>* scenes;
  int32_t n_scenes;
  int64_t total_steps;
  const R4* tpos;
  const R4* tmom;  // target dipoles (force kernel)
  const R4* spos;
  const R4* smom;
  Real* out[9];        // SoA outputs
  R4* out4;            // packed output (field kernel), optional
  const R4* add4;      // field epilogue addends (packed), optional
  const R4* add4b;
  const Real* rext[9]; // force epilogue: external gradient tensor (SoA), optional
  int32_t naive_quirks;
  // Optional per-scene stop flags (solver scalar rows): a scene whose flag is
  // non-zero is skipped (its outputs are left as they are).
  const double* done_flags;
  int32_t done_stride;
  // Optional near-field correction per target (added before the epilogue's scale).
  const R4* corr4;
  // Optional: the launch does nothing once *done_count reaches done_total
  // (every scene's solve has stopped).
  const int32_t* done_count;
  int32_t done_total;
  double* partials;    // [grid][2][TPB*TPT][kOut]
  int32_t* counters;   // [total target blocks], zero between launches
  int32_t* err;        // device error word
  // 0: staging waits take the default bound; k > 0: they give up after
  // k - 1 try-waits (debug: mf_debug_stage_wait_limit; drains keep the default).
  uint32_t stage_wait_debug;
};

// ----------------------------------------------------------------------------
// Bodies: what a pair adds and how a target's result is written.
// ----------------------------------------------------------------------------
// Source tiles as one packed record per source: item j = record j.
template <class Real>
struct RecordItems {
  using R4 = typename Vec4T<Real>::type;
  struct Item {
    R4 p, m;
  };
  __device__ static Item load_item(const R4* sp, const R4* sm, int j) { return Item{sp[j], sm[j]}; }
  __device__ static int items(int cnt) { return cnt; }
  __host__ __device__ static uint32_t tile_bytes(int cnt) { return uint32_t(cnt) * uint32_t(sizeof(R4)); }
};

// Per-target tile accumulator of kAcc scalars.
template <class Real, int N>
struct ScalarAcc {
  Real v[N];
  __device__ void zero() {
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = Real(0);
  }
};

// Adds the near-field correction of target i (if the launch has one) to v.
template <class Real>
__device__ __forceinline__ void add_correction(const AllPairsArgs<Real>& a, int64_t i, double* v) {
  if (a.corr4) {
    const typename Vec4T<Real>::type c = a.corr4[i];
    v[0] += double(c.x);
    v[1] += double(c.y);
    v[2] += double(c.z);
  }
}

template <class Real>
struct FieldBody : RecordItems<Real> {
  using R4 = typename Vec4T<Real>::type;
  static constexpr int kAcc = 6;
  static constexpr int kOut = 3;
  struct TData {
    Real x, y, z;
  };
  __device__ static void load(const AllPairsArgs<Real>& a, int64_t i, TData& t) {
    R4 p = a.tpos[i];
    t.x = p.x;
    t.y = p.y;
    t.z = p.z;
  }
  using Acc = ScalarAcc<Real, kAcc>;
  __device__ static void pair(const TData& t, const typename RecordItems<Real>::Item& it,
                              const PairConsts<Real>& pc, Acc& acc) {
    const R4& sp = it.p;
    const R4& sm = it.m;
    if constexpr (sizeof(Real) == 4)
      field_pair_sel(t.x - sp.x, t.y - sp.y, t.z - sp.z, sm.x, sm.y, sm.z, pc, acc.v, acc.v + 3);
    else
      field_pair<Real>(t.x - sp.x, t.y - sp.y, t.z - sp.z, sm.x, sm.y, sm.z, pc, acc.v, acc.v + 3);
  }
  __device__ static void tile_out(const Acc& acc, Real* o) {
    const Real c = Real(kInv4Pi);
    o[0] = (Real(3) * acc.v[0] - acc.v[3]) * c;
    o[1] = (Real(3) * acc.v[1] - acc.v[4]) * c;
    o[2] = (Real(3) * acc.v[2] - acc.v[5]) * c;
  }
  __device__ static void epilogue(const AllPairsArgs<Real>& a, const SceneDesc<Real>& sc, int64_t i,
                                  const TData&, const double* vin) {
    double v[3] = {vin[0], vin[1], vin[2]};
    add_correction(a, i, v);
    Real o[3];
    for (int k = 0; k < 3; ++k) o[k] = Real(v[k]) * sc.scale + sc.cvec[k];
    if (a.add4) {
      R4 q = a.add4[i];
      o[0] += sc.coef_add * q.x;
      o[1] += sc.coef_add * q.y;
      o[2] += sc.coef_add * q.z;
    }
    if (a.add4b) {
      R4 q = a.add4b[i];
      o[0] += sc.coef_add2 * q.x;
      o[1] += sc.coef_add2 * q.y;
      o[2] += sc.coef_add2 * q.z;
    }
    if (a.out[0]) {
      a.out[0][i] = o[0];
      a.out[1][i] = o[1];
      a.out[2][i] = o[2];
    }
    if (a.out4) {
      R4 w;
      w.x = o[0];
      w.y = o[1];
      w.z = o[2];
      w.w = Real(0);
      a.out4[i] = w;
    }
  }
};

template <class Real>
__device__ __forceinline__ void force_epilogue(const AllPairsArgs<Real>& a, const SceneDesc<Real>& sc, int64_t i,
                                               double mx, double my, double mz, const double* v);

template <class Real>
struct ForceBody : RecordItems<Real> {
  using R4 = typename Vec4T<Real>::type;
  static constexpr int kAcc = 3;
  static constexpr int kOut = 3;
  struct TData {
    Real x, y, z, mx, my, mz;
  };
  __device__ static void load(const AllPairsArgs<Real>& a, int64_t i, TData& t) {
    R4 p = a.tpos[i];
    R4 m = a.tmom[i];
    t.x = p.x;
    t.y = p.y;
    t.z = p.z;
    t.mx = m.x;
    t.my = m.y;
    t.mz = m.z;
  }
  using Acc = ScalarAcc<Real, kAcc>;
  __device__ static void pair(const TData& t, const typename RecordItems<Real>::Item& it,
                              const PairConsts<Real>& pc, Acc& acc) {
    const R4& sp = it.p;
    const R4& sm = it.m;
    if constexpr (sizeof(Real) == 4)
      force_pair_sel(t.x - sp.x, t.y - sp.y, t.z - sp.z, sm.x, sm.y, sm.z, t.mx, t.my, t.mz, pc, acc.v);
    else
      force_pair<Real>(t.x - sp.x, t.y - sp.y, t.z - sp.z, sm.x, sm.y, sm.z, t.mx, t.my, t.mz, pc, acc.v);
  }
  __device__ static void tile_out(const Acc& acc, Real* o) {
    const Real c = Real(kForceK);
    o[0] = acc.v[0] * c;
    o[1] = acc.v[1] * c;
    o[2] = acc.v[2] * c;
  }
  __device__ static void epilogue(const AllPairsArgs<Real>& a, const SceneDesc<Real>& sc, int64_t i,
                                  const TData& t, const double* v) {
    force_epilogue<Real>(a, sc, i, double(t.mx), double(t.my), double(t.mz), v);
  }
};

// F = (sum_j T_ij) m_i + external part (magnetic_force.cu:968-980 by default;
// :583-603 with the naive path's extra mu0 when naive_quirks is set).
template <class Real>
__device__ __forceinline__ void force_epilogue(const AllPairsArgs<Real>& a, const SceneDesc<Real>& sc, int64_t i,
                                               double mx, double my, double mz, const double* v) {
  {
    double f[3] = {v[0], v[1], v[2]};
    add_correction(a, i, f);
    if (a.rext[0]) {
      // rext[c*3 + r] = column c, row r; the tensor is symmetric.
      const double m[3] = {mx, my, mz};
      double e[3];
      for (int r = 0; r < 3; ++r) {
        e[r] = 0.0;
        for (int c = 0; c < 3; ++c) e[r] += double(a.rext[c * 3 + r][i]) * m[c];
      }
      const double s = a.naive_quirks ? kMu0 : 1.0;
      for (int r = 0; r < 3; ++r) f[r] += s * e[r];
    }
    a.out[0][i] = Real(f[0] * double(sc.scale));
    a.out[1][i] = Real(f[1] * double(sc.scale));
    a.out[2][i] = Real(f[2] * double(sc.scale));
  }
}

template <class Real>
struct TensorBody : RecordItems<Real> {
  using R4 = typename Vec4T<Real>::type;
  static constexpr int kAcc = 6;
  static constexpr int kOut = 6;
  struct TData {
    Real x, y, z;
  };
  __device__ static void load(const AllPairsArgs<Real>& a, int64_t i, TData& t) {
    R4 p = a.tpos[i];
    t.x = p.x;
    t.y = p.y;
    t.z = p.z;
  }
  using Acc = ScalarAcc<Real, kAcc>;
  __device__ static void pair(const TData& t, const typename RecordItems<Real>::Item& it,
                              const PairConsts<Real>& pc, Acc& acc) {
    const R4& sp = it.p;
    const R4& sm = it.m;
    tensor_pair<Real>(t.x - sp.x, t.y - sp.y, t.z - sp.z, sm.x, sm.y, sm.z, pc, acc.v);
  }
  __device__ static void tile_out(const Acc& acc, Real* o) {
    const Real c = Real(kForceK);
    for (int k = 0; k < 6; ++k) o[k] = acc.v[k] * c;
  }
  // Writes the 3x3 in the reference's layout: out[c*3 + r] = T(row r, col c).
  __device__ static void epilogue(const AllPairsArgs<Real>& a, const SceneDesc<Real>& sc, int64_t i,
                                  const TData&, const double* v) {
    const Real s = sc.scale;
    const Real xx = Real(v[0]) * s, yy = Real(v[1]) * s, zz = Real(v[2]) * s;
    const Real xy = Real(v[3]) * s, xz = Real(v[4]) * s, yz = Real(v[5]) * s;
    a.out[0][i] = xx;
    a.out[1][i] = xy;
    a.out[2][i] = xz;
    a.out[3][i] = xy;
    a.out[4][i] = yy;
    a.out[5][i] = yz;
    a.out[6][i] = xz;
    a.out[7][i] = yz;
    a.out[8][i] = zz;
  }
};

// ----------------------------------------------------------------------------
// Packed two-source bodies (FP32).  Source arrays are in pair layout: sources
// 2p and 2p+1 share two float4 records (x_a, x_b, y_a, y_b), (z_a, z_b, 0, 0),
// the same 16 bytes per source as the record layout, so tiles stage the same
// way.  A scene's sources start at an even index; an odd scene ends with a
// zero-dipole partner, which contributes exactly zero.  Every pair takes the
// far form with r^2 clamped to the near radius; the near-field correction of
// each target (mf_cells.cu) is added in the epilogue.
// ----------------------------------------------------------------------------
struct PairItems {
  struct Item {
    float2 x, y, z, mx, my, mz;
  };
  __device__ static Item load_item(const float4* sp, const float4* sm, int j) {
    const float4 p0 = sp[2 * j], p1 = sp[2 * j + 1];
    const float4 m0 = sm[2 * j], m1 = sm[2 * j + 1];
    return Item{make_float2(p0.x, p0.y), make_float2(p0.z, p0.w), make_float2(p1.x, p1.y),
                make_float2(m0.x, m0.y), make_float2(m0.z, m0.w), make_float2(m1.x, m1.y)};
  }
  __device__ static int items(int cnt) { return (cnt + 1) >> 1; }
  __host__ __device__ static uint32_t tile_bytes(int cnt) { return uint32_t((cnt + 1) >> 1) * 32u; }
};

struct FieldF2Body : PairItems {
  static constexpr int kOut = 3;
  struct TData {
    float2 x, y, z;
  };
  struct Acc {
    float2 s1[3], s2[3];
    __device__ void zero() {
#pragma unroll
      for (int k = 0; k < 3; ++k) s1[k] = s2[k] = make_float2(0.f, 0.f);
    }
  };
  __device__ static void load(const AllPairsArgs<float>& a, int64_t i, TData& t) {
    const float4 p = a.tpos[i];
    t.x = f2_dup(p.x);
    t.y = f2_dup(p.y);
    t.z = f2_dup(p.z);
  }
  __device__ static void pair(const TData& t, const Item& it, const PairConsts<float>& pc, Acc& acc) {
    field_pair2(t.x, t.y, t.z, it.x, it.y, it.z, it.mx, it.my, it.mz, pc.near2_field, acc.s1, acc.s2);
  }
  __device__ static void tile_out(const Acc& acc, float* o) {
    const float c = float(kInv4Pi);
#pragma unroll
    for (int k = 0; k < 3; ++k)
      o[k] = (3.f * (acc.s1[k].x + acc.s1[k].y) - (acc.s2[k].x + acc.s2[k].y)) * c;
  }
  __device__ static void epilogue(const AllPairsArgs<float>& a, const SceneDesc<float>& sc, int64_t i,
                                  const TData&, const double* v) {
    FieldBody<float>::epilogue(a, sc, i, FieldBody<float>::TData{}, v);
  }
};

// Outputs: the three force sums without the target-dipole term, and the
// scalar sum u of r^-5 (d.s) that the epilogue multiplies by the target's
// dipole (force_pair2).
struct ForceF2Body : PairItems {
  static constexpr int kOut = 4;
  struct TData {
    float2 x, y, z, mx, my, mz;
  };
  struct Acc {
    float2 f[3], u;
    __device__ void zero() {
#pragma unroll
      for (int k = 0; k < 3; ++k) f[k] = make_float2(0.f, 0.f);
      u = make_float2(0.f, 0.f);
    }
  };
  __device__ static void load(const AllPairsArgs<float>& a, int64_t i, TData& t) {
    const float4 p = a.tpos[i];
    const float4 m = a.tmom[i];
    t.x = f2_dup(p.x);
    t.y = f2_dup(p.y);
    t.z = f2_dup(p.z);
    t.mx = f2_dup(m.x);
    t.my = f2_dup(m.y);
    t.mz = f2_dup(m.z);
  }
  __device__ static void pair(const TData& t, const Item& it, const PairConsts<float>& pc, Acc& acc) {
    force_pair2(t.x, t.y, t.z, t.mx, t.my, t.mz, it.x, it.y, it.z, it.mx, it.my, it.mz, pc.near2_force, acc.f,
                acc.u);
  }
  __device__ static void tile_out(const Acc& acc, float* o) {
    const float c = float(kForceK);
#pragma unroll
    for (int k = 0; k < 3; ++k) o[k] = (acc.f[k].x + acc.f[k].y) * c;
    o[3] = (acc.u.x + acc.u.y) * c;
  }
  __device__ static void epilogue(const AllPairsArgs<float>& a, const SceneDesc<float>& sc, int64_t i,
                                  const TData& t, const double* v) {
    const double mx = double(t.mx.x), my = double(t.my.x), mz = double(t.mz.x);
    const double f[3] = {v[0] + mx * v[3], v[1] + my * v[3], v[2] + mz * v[3]};
    force_epilogue<float>(a, sc, i, mx, my, mz, f);
  }
};

// Packed force tensor (the FMM matrix of the Hessian kernel at separate
// targets).  The near-field correction comes as two records per target in
// corr4: (xx, yy, zz, -), (xy, xz, yz, -).
struct TensorF2Body : PairItems {
  static constexpr int kOut = 6;
  struct TData {
    float2 x, y, z;
  };
  struct Acc {
    float2 t[6];
    __device__ void zero() {
#pragma unroll
      for (int k = 0; k < 6; ++k) t[k] = make_float2(0.f, 0.f);
    }
  };
  __device__ static void load(const AllPairsArgs<float>& a, int64_t i, TData& t) {
    const float4 p = a.tpos[i];
    t.x = f2_dup(p.x);
    t.y = f2_dup(p.y);
    t.z = f2_dup(p.z);
  }
  __device__ static void pair(const TData& t, const Item& it, const PairConsts<float>& pc, Acc& acc) {
    tensor_pair2(t.x, t.y, t.z, it.x, it.y, it.z, it.mx, it.my, it.mz, pc.near2_force, acc.t);
  }
  __device__ static void tile_out(const Acc& acc, float* o) {
    const float c = float(kForceK);
#pragma unroll
    for (int k = 0; k < 6; ++k) o[k] = (acc.t[k].x + acc.t[k].y) * c;
  }
  __device__ static void epilogue(const AllPairsArgs<float>& a, const SceneDesc<float>& sc, int64_t i,
                                  const TData&, const double* vin) {
    double v[6] = {vin[0], vin[1], vin[2], vin[3], vin[4], vin[5]};
    if (a.corr4) {
      const float4 c0 = a.corr4[2 * i], c1 = a.corr4[2 * i + 1];
      v[0] += c0.x;
      v[1] += c0.y;
      v[2] += c0.z;
      v[3] += c1.x;
      v[4] += c1.y;
      v[5] += c1.z;
    }
    TensorBody<float>::epilogue(a, sc, i, TensorBody<float>::TData{}, v);
  }
};

// ----------------------------------------------------------------------------
// Step-space helpers.
// ----------------------------------------------------------------------------
__device__ __forceinline__ int64_t step_start(int64_t T, int64_t G, int64_t b) { return (T * b) / G; }
// The CTA whose range holds step x: largest b with start(b) <= x.
__device__ __forceinline__ int64_t step_owner(int64_t T, int64_t G, int64_t x) { return ((x + 1) * G - 1) / T; }

template <class Real>
__device__ __forceinline__ int find_scene(const SceneDesc<Real>* sc, int n, int64_t step) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (sc[mid].step_off <= step) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <class Real, int TILE>
struct StageLayout {
  using R4 = typename Vec4T<Real>::type;
  static constexpr int kBytes = 2 * TILE * int(sizeof(R4));
};

// ----------------------------------------------------------------------------
// The kernel.
// ----------------------------------------------------------------------------
template <class Real, class Body, int TPB, int TPT, int TILE, int STAGES>
__global__ void __launch_bounds__(TPB) allpairs_kernel(const AllPairsArgs<Real> a) {
  using R4 = typename Vec4T<Real>::type;
  constexpr int TBT = TPB * TPT;
  constexpr int kOut = Body::kOut;
  constexpr bool kComp = sizeof(Real) == 4;  // compensate FP32 running sums

  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ int s_flag;
  __shared__ float s_fit[40];

  const int tid = threadIdx.x;
  const int64_t T = a.total_steps;
  const int64_t G = gridDim.x;
  const int64_t b = blockIdx.x;
  const int64_t k_begin = step_start(T, G, b);
  const int64_t k_end = step_start(T, G, b + 1);
  if (k_begin >= k_end) return;
  // A launch whose solves have all stopped does nothing.
  if (a.done_flags && a.n_scenes == 1 && a.done_flags[int64_t(a.scenes[0].flag_index) * a.done_stride] != 0.0)
    return;
  if (a.done_count && *a.done_count >= a.done_total) return;

  // Stage s: TILE source positions, then TILE source dipoles (computed, not
  // tabulated, so a runtime stage index does not put the table in local memory).
  auto stage_pos = [&](int s) { return reinterpret_cast<R4*>(smem_raw + s * StageLayout<Real, TILE>::kBytes); };
  auto stage_mom = [&](int s) { return stage_pos(s) + TILE; };

  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) mbar_init(&full_bar[s], 1);
    fence_mbar_init();
  }
  if (tid < 40) s_fit[tid] = c_fit_ap[tid];
  __syncthreads();

  // Producer (thread 0): stage the source tile of step k into stage s.
  auto issue = [&](int64_t k, int s) {
    const int si = find_scene(a.scenes, a.n_scenes, k);
    const SceneDesc<Real>& sc = a.scenes[si];
    const int64_t local = k - sc.step_off;
    const int tile = int(local % sc.n_tiles);
    const int64_t first = sc.s_off + int64_t(tile) * TILE;
    const int64_t rem = sc.ns - int64_t(tile) * TILE;
    const uint32_t cnt = uint32_t(rem < TILE ? rem : TILE);
    const uint32_t bytes = Body::tile_bytes(cnt);
    mbar_arrive_expect_tx(&full_bar[s], 2 * bytes);
    bulk_g2s(stage_pos(s), a.spos + first, bytes, &full_bar[s]);
    bulk_g2s(stage_mom(s), a.smom + first, bytes, &full_bar[s]);
  };

  if (tid == 0) {
    for (int s = 0; s < STAGES && k_begin + s < k_end; ++s) issue(k_begin + s, s);
  }

  // Walk state.
  int si = find_scene(a.scenes, a.n_scenes, k_begin);
  int64_t local = k_begin - a.scenes[si].step_off;
  int tb = int(local / a.scenes[si].n_tiles);
  int tile = int(local % a.scenes[si].n_tiles);
  bool seg_from_start = (tile == 0);
  bool first_tb_of_cta = true;

  typename Body::TData td[TPT];
  Real run[TPT][kOut];
  Real cmp[TPT][kOut];

  auto load_targets = [&](const SceneDesc<Real>& sc, int tbl) {
#pragma unroll
    for (int t = 0; t < TPT; ++t) {
      int64_t li = int64_t(tbl) * TBT + t * TPB + tid;
      if (li >= sc.nt) li = sc.nt - 1;
      Body::load(a, sc.t_off + li, td[t]);
#pragma unroll
      for (int o = 0; o < kOut; ++o) {
        run[t][o] = Real(0);
        cmp[t][o] = Real(0);
      }
    }
  };
  load_targets(a.scenes[si], tb);

  int64_t k_fail = -1;
  for (int64_t k = k_begin; k < k_end; ++k) {
    const int64_t u = k - k_begin;
    const int s = int(u % STAGES);
    const uint32_t parity = uint32_t((u / STAGES) & 1);
    const SceneDesc<Real>& sc = a.scenes[si];
    PairConsts<Real> pc = sc.pc;
    pc.tbl = s_fit;

    const bool ok = mbar_wait_bounded(&full_bar[s], parity, stage_wait_limit(a.stage_wait_debug));
    if (__syncthreads_or(!ok)) {
      k_fail = k;
      break;
    }
    const bool skip_scene = a.done_flags && a.done_flags[int64_t(sc.flag_index) * a.done_stride] != 0.0;

    // Sweep the tile.
    if (!skip_scene) {
      const int64_t rem = sc.ns - int64_t(tile) * TILE;
      const int cnt = int(rem < TILE ? rem : TILE);
      const R4* __restrict__ sp = stage_pos(s);
      const R4* __restrict__ sm = stage_mom(s);
      typename Body::Acc acc[TPT];
#pragma unroll
      for (int t = 0; t < TPT; ++t) acc[t].zero();
      const int n_items = Body::items(cnt);
#pragma unroll 4
      for (int j = 0; j < n_items; ++j) {
        const typename Body::Item it = Body::load_item(sp, sm, j);
#pragma unroll
        for (int t = 0; t < TPT; ++t) Body::pair(td[t], it, pc, acc[t]);
      }
#pragma unroll
      for (int t = 0; t < TPT; ++t) {
        Real o[kOut];
        Body::tile_out(acc[t], o);
#pragma unroll
        for (int q = 0; q < kOut; ++q) {
          if constexpr (kComp) comp_add(run[t][q], cmp[t][q], o[q]);
          else run[t][q] += o[q];
        }
      }
    }

    __syncthreads();  // every thread is done with stage s
    if (tid == 0 && k + STAGES < k_end) {
      fence_proxy_async_smem();
      issue(k + STAGES, s);
    }

    // Advance; flush when this target block's segment ends.
    const bool last_tile = (tile == sc.n_tiles - 1);
    const bool last_step = (k == k_end - 1);
    if (last_tile || last_step) {
      const int64_t gtb = sc.tb_off + tb;
      const bool full = seg_from_start && last_tile;
      if (skip_scene) {
        // nothing to write for a stopped scene
      } else if (full) {
#pragma unroll
        for (int t = 0; t < TPT; ++t) {
          const int64_t li = int64_t(tb) * TBT + t * TPB + tid;
          if (li < sc.nt) {
            double v[kOut];
#pragma unroll
            for (int q = 0; q < kOut; ++q) v[q] = double(run[t][q]) + double(cmp[t][q]);
            Body::epilogue(a, sc, sc.t_off + li, td[t], v);
          }
        }
      } else {
        const int slot = first_tb_of_cta ? 0 : 1;
        double* part = a.partials + ((b * 2 + slot) * TBT) * kOut;
#pragma unroll
        for (int t = 0; t < TPT; ++t) {
          const int li = t * TPB + tid;
#pragma unroll
          for (int q = 0; q < kOut; ++q) part[li * kOut + q] = double(run[t][q]) + double(cmp[t][q]);
        }
        __threadfence();
        __syncthreads();
        const int64_t sa = sc.step_off + int64_t(tb) * sc.n_tiles;
        const int64_t se = sa + sc.n_tiles;
        const int64_t b_first = step_owner(T, G, sa);
        const int64_t b_last = step_owner(T, G, se - 1);
        if (tid == 0) {
          const int nseg = int(b_last - b_first + 1);
          const int ticket = atomicAdd(&a.counters[gtb], 1);
          s_flag = (ticket == nseg - 1);
        }
        __syncthreads();
        if (s_flag) {
          __threadfence();
          const bool first_split = step_start(T, G, b_first) < sa;
#pragma unroll
          for (int t = 0; t < TPT; ++t) {
            const int li = t * TPB + tid;
            double v[kOut];
#pragma unroll
            for (int q = 0; q < kOut; ++q) v[q] = 0.0;
            for (int64_t bb = b_first; bb <= b_last; ++bb) {
              const int sl = (bb == b_first && first_split) ? 1 : 0;
              const double* pp = a.partials + ((bb * 2 + sl) * TBT) * kOut;
#pragma unroll
              for (int q = 0; q < kOut; ++q) v[q] += __ldcg(&pp[li * kOut + q]);
            }
            const int64_t gi = int64_t(tb) * TBT + li;
            if (gi < sc.nt) Body::epilogue(a, sc, sc.t_off + gi, td[t], v);
          }
          if (tid == 0) a.counters[gtb] = 0;
        }
      }
      // Next target block (possibly in the next scene).
      if (!last_step) {
        first_tb_of_cta = false;
        seg_from_start = true;
        tile = 0;
        ++tb;
        if (tb == sc.n_tb) {
          tb = 0;
          ++si;
        }
        load_targets(a.scenes[si], tb);
      }
    } else {
      ++tile;
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

}  // namespace mfgb
