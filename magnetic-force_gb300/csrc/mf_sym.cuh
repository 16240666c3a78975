// mf_sym.cuh -- device helpers of the products evaluated once per unordered
// pair (mf_sympair.cu for the all-pairs path, mf_fmm.cu for the FMM's near
// field): the packed pair bodies that add a pair's terms on both sides, the
// warp reduce-scatter of the sources' sums, and a compensated add.
#pragma once

#include "mf_allpairs.cuh"

namespace mfgb {

// Reduce-scatter of NV values per lane over the warp (NV a power of two,
// 8 .. 32): the value index halves at each level, lanes with bit b set keep
// the upper half; after log2(NV) levels each lane holds one value summed over
// the lanes that differ in the bits used, and the remaining levels finish the
// sum.  Value k ends in the lanes lane / (32 / NV) == k.  Fixed order: the
// result does not depend on scheduling.
template <int NV>
__device__ __forceinline__ float warp_reduce_scatter(const float (&v)[NV], int lane) {
  static_assert(NV >= 2 && NV <= 32 && (NV & (NV - 1)) == 0, "NV");
  float w[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) w[q] = v[q];
  int b = 16;
#pragma unroll
  for (int n = NV; n > 1; n >>= 1, b >>= 1) {
    const bool hi = lane & b;
#pragma unroll
    for (int q = 0; q < n / 2; ++q) {
      const float send = hi ? w[q] : w[q + n / 2];
      const float keep = hi ? w[q + n / 2] : w[q];
      w[q] = keep + __shfl_xor_sync(0xffffffffu, send, b);
    }
  }
#pragma unroll
  for (; b >= 1; b >>= 1) w[0] += __shfl_xor_sync(0xffffffffu, w[0], b);
  return w[0];
}

// Kelvin force: f_ij into the target's sums (acc), and into the sources'
// sums (src) as well: the caller negates those (f_ji = -f_ij).  Written as
//   f_ij = r^-5 g,  g = d w + m_t (d.m_s) + m_s (d.m_t),  w = m_s.m_t - 5 r^-2 (d.m_s)(d.m_t)
// with r^-5 g added into both sums by FMAs: 36 packed operations per target
// and item (forming f_ij first and adding it to both sums takes 39).
__device__ __forceinline__ void sym_force_pair2(float2 tx, float2 ty, float2 tz, float2 tmx, float2 tmy, float2 tmz,
                                                const PairItems::Item& it, float near2, float2* acc, float2* src) {
  const float2 dx = f2_sub(tx, it.x), dy = f2_sub(ty, it.y), dz = f2_sub(tz, it.z);
  const float2 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
  const float2 ri = clamp_rsqrt2(r2, near2);
  const float2 ri2 = f2_mul(ri, ri);
  const float2 ri5 = f2_mul(f2_mul(ri2, ri2), ri);
  const float2 ds = f2_fma(dz, it.mz, f2_fma(dy, it.my, f2_mul(dx, it.mx)));
  const float2 dm = f2_fma(dz, tmz, f2_fma(dy, tmy, f2_mul(dx, tmx)));
  const float2 sm = f2_fma(it.mz, tmz, f2_fma(it.my, tmy, f2_mul(it.mx, tmx)));
  const float2 e = f2_mul(f2_mul(ri2, f2_dup(-5.f)), ds);
  const float2 w = f2_fma(e, dm, sm);
  const float2 g0 = f2_fma(dx, w, f2_fma(tmx, ds, f2_mul(it.mx, dm)));
  const float2 g1 = f2_fma(dy, w, f2_fma(tmy, ds, f2_mul(it.my, dm)));
  const float2 g2 = f2_fma(dz, w, f2_fma(tmz, ds, f2_mul(it.mz, dm)));
  acc[0] = f2_fma(ri5, g0, acc[0]);
  acc[1] = f2_fma(ri5, g1, acc[1]);
  acc[2] = f2_fma(ri5, g2, acc[2]);
  src[0] = f2_fma(ri5, g0, src[0]);
  src[1] = f2_fma(ri5, g1, src[1]);
  src[2] = f2_fma(ri5, g2, src[2]);
}

// Dipole field: the target gets T m_s, the source T m_t, each accumulated as
// -(3 d (d.m) r^-5 - m r^-3) = d (d.m) (-3 r^-5) + m r^-3 with FMAs straight
// into the sums (30 packed operations per target and item).
__device__ __forceinline__ void sym_field_pair2(float2 tx, float2 ty, float2 tz, float2 tmx, float2 tmy, float2 tmz,
                                                const PairItems::Item& it, float near2, float2* acc, float2* src) {
    const float2 dx = f2_sub(tx, it.x), dy = f2_sub(ty, it.y), dz = f2_sub(tz, it.z);
    const float2 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
    const float2 ri = clamp_rsqrt2(r2, near2);
    const float2 ri2 = f2_mul(ri, ri);
    const float2 beta = f2_mul(ri2, ri);
    const float2 a3 = f2_mul(beta, f2_mul(ri2, f2_dup(-3.f)));
    const float2 ts = f2_mul(f2_fma(dz, it.mz, f2_fma(dy, it.my, f2_mul(dx, it.mx))), a3);
    const float2 tt = f2_mul(f2_fma(dz, tmz, f2_fma(dy, tmy, f2_mul(dx, tmx))), a3);
    acc[0] = f2_fma(it.mx, beta, f2_fma(dx, ts, acc[0]));
    acc[1] = f2_fma(it.my, beta, f2_fma(dy, ts, acc[1]));
    acc[2] = f2_fma(it.mz, beta, f2_fma(dz, ts, acc[2]));
    src[0] = f2_fma(tmx, beta, f2_fma(dx, tt, src[0]));
    src[1] = f2_fma(tmy, beta, f2_fma(dy, tt, src[1]));
    src[2] = f2_fma(tmz, beta, f2_fma(dz, tt, src[2]));
  }

// Field and Kelvin force of one pair item together, for a product of both
// over the same dipoles: the separation, r^2 and the two dots d.m_s, d.m_t
// are formed once (54 packed operations per target and item against 30 + 36
// apart).  Each term is the one sym_field_pair2 / sym_force_pair2 forms,
// operation for operation: the field clamped at its near radius (nf2), the
// force at its own (ng2).
__device__ __forceinline__ void sym_field_force_pair2(float2 tx, float2 ty, float2 tz, float2 tmx, float2 tmy,
                                                      float2 tmz, const PairItems::Item& it, float nf2, float ng2,
                                                      float2* accf, float2* accg, float2* srcf, float2* srcg) {
  const float2 dx = f2_sub(tx, it.x), dy = f2_sub(ty, it.y), dz = f2_sub(tz, it.z);
  const float2 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
  const float2 ds = f2_fma(dz, it.mz, f2_fma(dy, it.my, f2_mul(dx, it.mx)));
  const float2 dm = f2_fma(dz, tmz, f2_fma(dy, tmy, f2_mul(dx, tmx)));
  {
    const float2 ri = clamp_rsqrt2(r2, nf2);
    const float2 ri2 = f2_mul(ri, ri);
    const float2 beta = f2_mul(ri2, ri);
    const float2 a3 = f2_mul(beta, f2_mul(ri2, f2_dup(-3.f)));
    const float2 ts = f2_mul(ds, a3);
    const float2 tt = f2_mul(dm, a3);
    accf[0] = f2_fma(it.mx, beta, f2_fma(dx, ts, accf[0]));
    accf[1] = f2_fma(it.my, beta, f2_fma(dy, ts, accf[1]));
    accf[2] = f2_fma(it.mz, beta, f2_fma(dz, ts, accf[2]));
    srcf[0] = f2_fma(tmx, beta, f2_fma(dx, tt, srcf[0]));
    srcf[1] = f2_fma(tmy, beta, f2_fma(dy, tt, srcf[1]));
    srcf[2] = f2_fma(tmz, beta, f2_fma(dz, tt, srcf[2]));
  }
  {
    const float2 ri = clamp_rsqrt2(r2, ng2);
    const float2 ri2 = f2_mul(ri, ri);
    const float2 ri5 = f2_mul(f2_mul(ri2, ri2), ri);
    const float2 sm = f2_fma(it.mz, tmz, f2_fma(it.my, tmy, f2_mul(it.mx, tmx)));
    const float2 e = f2_mul(f2_mul(ri2, f2_dup(-5.f)), ds);
    const float2 w = f2_fma(e, dm, sm);
    const float2 g0 = f2_fma(dx, w, f2_fma(tmx, ds, f2_mul(it.mx, dm)));
    const float2 g1 = f2_fma(dy, w, f2_fma(tmy, ds, f2_mul(it.my, dm)));
    const float2 g2 = f2_fma(dz, w, f2_fma(tmz, ds, f2_mul(it.mz, dm)));
    accg[0] = f2_fma(ri5, g0, accg[0]);
    accg[1] = f2_fma(ri5, g1, accg[1]);
    accg[2] = f2_fma(ri5, g2, accg[2]);
    srcg[0] = f2_fma(ri5, g0, srcg[0]);
    srcg[1] = f2_fma(ri5, g1, srcg[1]);
    srcg[2] = f2_fma(ri5, g2, srcg[2]);
  }
}

// s + x with the rounding error of the add carried in e: Knuth's TwoSum
// (The Art of Computer Programming, vol. 2, 4.2.2), exact in round-to-
// nearest without any ordering of |s| and |x|.
__device__ __forceinline__ void two_sum_acc(float& s, float& e, float x) {
  const float t = __fadd_rn(s, x);
  const float xp = __fsub_rn(t, s);
  const float sp = __fsub_rn(t, xp);
  e = __fadd_rn(e, __fadd_rn(__fsub_rn(s, sp), __fsub_rn(x, xp)));
  s = t;
}

}  // namespace mfgb
