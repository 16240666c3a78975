// mf_vec.cuh -- vector updates and FP64 reductions of the magnetization solve.
//
// Replaces the reference's BLAS-1 layer (cuda_abstract_vector.cuh:13-161,
// :503-563): one fused launch per update instead of three per operator, no
// allocation per temporary, and inner products accumulated in FP64 with a
// deterministic two-level reduction whose last CTA also applies the solver's
// scalar step on the device (no host round trip).
//
// Vectors are packed Real4 records (x, y, z, pad) laid out scene after scene;
// every scene owns a row of 32 doubles of solver scalars.  A launch covers
// all scenes: blockIdx.y is the scene, blockIdx.x strides over its elements.
#pragma once
#include <cstdint>

#include "mf_device.cuh"

namespace mfgb {

// Solver scalars, one row of kScal doubles per scene.
enum Scal : int {
  S_DONE = 0,    // != 0: this scene's solve has stopped
  S_ITERS = 1,   // iterations completed
  S_RR = 2,      // r . r
  S_PQ = 3,      // p . q
  S_ALPHA = 4,
  S_BETA = 5,
  S_BNORM = 6,   // |Hext|
  S_RELRES = 7,  // |r| / |Hext|
  S_TOL = 8,     // relative tolerance
  S_MAXIT = 9,   // iteration cap
  S_ERR = 10,    // 0.5 |r|^2 (NLCG error)
  S_NT = 11,     // Dd . Dd
  S_DR = 12,     // Dd . r
  S_GG = 13,     // g . g
  S_DG = 14,     // d_old . (g_old - g)
  S_C = 15,      // c = V chi / (1 + chi)
  S_RESET = 16,  // NLCG: beta restart this iteration
  // Slots 20.. are kept across solves (batched scenes): per-scene constants
  // and the running total of CG iterations.
  S_CONST_C = 20,      // c = V chi / (1 + chi)
  S_CONST_INVM = 21,   // 1 / particle mass (unit density: 1 / V)
  S_CONST_H0 = 22,     // uniform external field, 3 slots
  S_ITERS_TOTAL = 25,  // CG iterations over all solves
  kScal = 32
};

struct VecRange {
  int64_t off;  // first element of the scene
  int64_t n;    // elements
};

template <class R4>
__device__ __forceinline__ double dot4(const R4& a, const R4& b) {
  return double(a.x) * double(b.x) + double(a.y) * double(b.y) + double(a.z) * double(b.z);
}

// Block-wide sum of kN doubles; result valid in thread 0.
template <int kN>
__device__ __forceinline__ void block_sum(double* v, double (*sh)[32]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kN; ++k) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[k][warp] = x;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < kN; ++k) {
      double x = lane < nw ? sh[k][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      v[k] = x;
    }
  }
}

// Per-scene reduction with a device-side scalar epilogue.
//   Op::kN                      number of sums
//   op.skip(scal_row)           uniform early exit (e.g. solve already done)
//   op.elem(i, acc, scal_row)   per element: accumulate and/or update vectors
//   op.finish(sums, scal_row)   once per scene, by the last CTA of that scene
template <class Op>
__global__ void __launch_bounds__(256) reduce_kernel(Op op, const VecRange* ranges, double* scal,
                                                     double* partials, int32_t* tickets) {
  constexpr int kN = Op::kN;
  __shared__ double sh[kN > 0 ? kN : 1][32];
  __shared__ int s_last;
  const int scene = blockIdx.y;
  double* row = scal + int64_t(scene) * kScal;
  if (op.skip(row)) return;
  const VecRange rg = ranges[scene];
  double acc[kN > 0 ? kN : 1];
#pragma unroll
  for (int k = 0; k < kN; ++k) acc[k] = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < rg.n; i += int64_t(gridDim.x) * blockDim.x)
    op.elem(rg.off + i, acc, row);
  if constexpr (kN > 0) {
    block_sum<kN>(acc, sh);
    double* part = partials + (int64_t(scene) * gridDim.x + blockIdx.x) * kN;
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < kN; ++k) part[k] = acc[k];
      __threadfence();
      const int t = atomicAdd(&tickets[scene], 1);
      s_last = (t == int(gridDim.x) - 1);
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
      __threadfence();
      double sums[kN];
#pragma unroll
      for (int k = 0; k < kN; ++k) sums[k] = 0.0;
      const double* base = partials + int64_t(scene) * gridDim.x * kN;
      for (unsigned bx = 0; bx < gridDim.x; ++bx)
#pragma unroll
        for (int k = 0; k < kN; ++k) sums[k] += __ldcg(&base[bx * kN + k]);
      op.finish(sums, row);
      tickets[scene] = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// Conjugate gradients on (I - c G) b = Hext.  The field launch before CgStart
// leaves r = c G b + Hext - b; before CgPq it leaves q = p - c G p.
// ---------------------------------------------------------------------------
// Marks a scene's solve as stopped, counting it once in *done_count (if given).
__device__ __forceinline__ void mark_done(double* row, int32_t* done_count) {
  if (row[S_DONE] == 0.0) {
    row[S_DONE] = 1.0;
    if (done_count) atomicAdd(done_count, 1);
  }
}

template <class R4>
struct CgStart {
  static constexpr int kN = 2;
  const R4* r;
  R4* p;
  const R4* hext;
  int32_t* done_count = nullptr;
  __device__ bool skip(const double*) const { return false; }
  __device__ void elem(int64_t i, double* acc, const double*) const {
    const R4 ri = r[i];
    p[i] = ri;
    acc[0] += dot4(ri, ri);
    const R4 h = hext[i];
    acc[1] += dot4(h, h);
  }
  __device__ void finish(const double* s, double* row) const {
    row[S_RR] = s[0];
    row[S_BNORM] = s[1] > 0.0 ? sqrt(s[1]) : 1.0;
    row[S_RELRES] = sqrt(s[0]) / row[S_BNORM];
    row[S_ITERS] = 0.0;
    if (row[S_RELRES] < row[S_TOL] || row[S_MAXIT] <= 0.0) mark_done(row, done_count);
  }
};

template <class R4>
struct CgPq {
  static constexpr int kN = 1;
  const R4* p;
  const R4* q;
  int32_t* done_count = nullptr;
  __device__ bool skip(const double* row) const { return row[S_DONE] != 0.0; }
  __device__ void elem(int64_t i, double* acc, const double*) const { acc[0] += dot4(p[i], q[i]); }
  __device__ void finish(const double* s, double* row) const {
    row[S_PQ] = s[0];
    if (s[0] > 0.0) {
      row[S_ALPHA] = row[S_RR] / s[0];
    } else {  // breakdown: the operator lost positive definiteness or r == 0
      row[S_ALPHA] = 0.0;
      mark_done(row, done_count);
    }
  }
};

template <class Real, class R4>
struct CgUpdate {
  static constexpr int kN = 1;
  R4* b;
  R4* r;
  const R4* p;
  const R4* q;
  int32_t* done_count = nullptr;
  __device__ bool skip(const double* row) const { return row[S_DONE] != 0.0; }
  __device__ void elem(int64_t i, double* acc, const double* row) const {
    const Real a = Real(row[S_ALPHA]);
    R4 bi = b[i], ri = r[i];
    const R4 pi = p[i], qi = q[i];
    bi.x += a * pi.x;
    bi.y += a * pi.y;
    bi.z += a * pi.z;
    ri.x -= a * qi.x;
    ri.y -= a * qi.y;
    ri.z -= a * qi.z;
    b[i] = bi;
    r[i] = ri;
    acc[0] += dot4(ri, ri);
  }
  __device__ void finish(const double* s, double* row) const {
    const double rr_old = row[S_RR];
    row[S_BETA] = rr_old > 0.0 ? s[0] / rr_old : 0.0;
    row[S_RR] = s[0];
    row[S_RELRES] = sqrt(s[0]) / row[S_BNORM];
    row[S_ITERS] += 1.0;
    row[S_ITERS_TOTAL] += 1.0;
    if (row[S_RELRES] < row[S_TOL] || row[S_ITERS] >= row[S_MAXIT]) mark_done(row, done_count);
  }
};

template <class Real, class R4>
struct CgDirection {  // p = r + beta p
  static constexpr int kN = 0;
  const R4* r;
  R4* p;
  __device__ bool skip(const double* row) const { return row[S_DONE] != 0.0; }
  __device__ void elem(int64_t i, double*, const double* row) const {
    const Real be = Real(row[S_BETA]);
    const R4 ri = r[i];
    R4 pi = p[i];
    pi.x = ri.x + be * pi.x;
    pi.y = ri.y + be * pi.y;
    pi.z = ri.z + be * pi.z;
    p[i] = pi;
  }
  __device__ void finish(const double*, double*) const {}
};

// ---------------------------------------------------------------------------
// The reference's nonlinear CG (magnetic_force.cu:1008-1095, :1287-1315).
// ---------------------------------------------------------------------------
template <class R4>
struct NlErr {  // err = 0.5 |r|^2
  static constexpr int kN = 1;
  const R4* r;
  __device__ bool skip(const double*) const { return false; }
  __device__ void elem(int64_t i, double* acc, const double*) const { acc[0] += dot4(r[i], r[i]); }
  __device__ void finish(const double* s, double* row) const { row[S_ERR] = 0.5 * s[0]; }
};

template <class R4>
struct NlAlpha {  // calc_alpha: -(Dd . r) / (Dd . Dd + 1e-10), 0 if Dd . Dd < 1e-10
  static constexpr int kN = 2;
  const R4* Dd;
  const R4* r;
  __device__ bool skip(const double*) const { return false; }
  __device__ void elem(int64_t i, double* acc, const double*) const {
    const R4 v = Dd[i];
    acc[0] += dot4(v, v);
    acc[1] += dot4(v, r[i]);
  }
  __device__ void finish(const double* s, double* row) const {
    row[S_NT] = s[0];
    row[S_DR] = s[1];
    row[S_ALPHA] = (s[0] < 1e-10) ? 0.0 : -(s[1] / (s[0] + 1e-10));
  }
};

template <class R4>
struct NlBeta {  // calc_beta: -|g|^2 / (d_old . (g_old - g) + 1e-10), clamped at 0
  static constexpr int kN = 2;
  const R4* g;
  const R4* gold;
  const R4* dold;
  __device__ bool skip(const double*) const { return false; }
  __device__ void elem(int64_t i, double* acc, const double*) const {
    const R4 gi = g[i], go = gold[i], dd = dold[i];
    acc[0] += dot4(gi, gi);
    acc[1] += double(dd.x) * (double(go.x) - double(gi.x)) + double(dd.y) * (double(go.y) - double(gi.y)) +
              double(dd.z) * (double(go.z) - double(gi.z));
  }
  __device__ void finish(const double* s, double* row) const {
    row[S_GG] = s[0];
    row[S_DG] = s[1];
    double be = -s[0] / (s[1] + 1e-10);
    if (row[S_RESET] != 0.0 || be < 0.0) be = 0.0;
    row[S_BETA] = be;
  }
};

template <class Real, class R4>
struct NlDirection {  // d = -g + beta d_old
  static constexpr int kN = 0;
  const R4* g;
  const R4* dold;
  R4* d;
  bool first;  // start(): d = -g
  __device__ bool skip(const double*) const { return false; }
  __device__ void elem(int64_t i, double*, const double* row) const {
    const R4 gi = g[i];
    R4 o;
    if (first) {
      o.x = -gi.x;
      o.y = -gi.y;
      o.z = -gi.z;
    } else {
      const Real be = Real(row[S_BETA]);
      const R4 dd = dold[i];
      o.x = -gi.x + be * dd.x;
      o.y = -gi.y + be * dd.y;
      o.z = -gi.z + be * dd.z;
    }
    o.w = Real(0);
    d[i] = o;
  }
  __device__ void finish(const double*, double*) const {}
};

template <class Real, class R4>
struct NlStep {  // b += alpha d
  static constexpr int kN = 0;
  R4* b;
  const R4* d;
  __device__ bool skip(const double*) const { return false; }
  __device__ void elem(int64_t i, double*, const double* row) const {
    const Real a = Real(row[S_ALPHA]);
    R4 bi = b[i];
    const R4 di = d[i];
    bi.x += a * di.x;
    bi.y += a * di.y;
    bi.z += a * di.z;
    b[i] = bi;
  }
  __device__ void finish(const double*, double*) const {}
};

}  // namespace mfgb
