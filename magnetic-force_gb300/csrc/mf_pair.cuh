// mf_pair.cuh -- pair arithmetic of the SPH-smoothed dipole kernels.
//
// Field (B/mu0) of a source dipole s at offset d = target - source:
//   fmmtl_minimum/kernel/Dipole_B.kern:46-104, magnetic_force.cu:63-98
//   K_B(d) s = rhat (rhat.s)(w_avr - w_dens) - (w_avr/3 - w_dens) s.
// Written here as  (1/4pi) * (3 d (d.s) alpha - s beta)  with
//   far  (q >= 2):  alpha = r^-5,  beta = r^-3        (w_dens = 0)
//   near (q <  2):  alpha = 4pi (w_avr - w_dens) / (3 r^2),  beta = 4pi (w_avr/3 - w_dens)
// so the common far pair costs one rsqrt and a handful of FMAs.  At r = 0 the
// d-term vanishes and beta carries the self term, as in the reference.
//
// Force tensor of a source dipole s, contracted with the target dipole m:
//   fmmtl_minimum/kernel/Dipole_hessian.kern:53-253, magnetic_force.cu:239-427.
// The reference builds a rotated frame (xi, eta, zeta = rhat) and forms
// M U M^T.  Expanding that product with an orthonormal frame gives the
// frame-free form used here,
//   T_ab = P (ds delta_ab + s_a d_b + d_a s_b) + Q ds d_a d_b,   ds = d.s,
//   far  (q >  4):  P = K r^-5,            Q = -5 K r^-7,   K = 3 mu0 / (4 pi)
//   near (0<q<=4):  P = C1(q) / (h^4 r),   Q = (C2(q) - 3 C1(q)) / (h^4 r^3)
//   q == 0:         T = 0  (overlapping particles exert no force, :101-104)
// and F = T m = P (ds m + dm s + sm d) + Q ds dm d  with dm = d.m, sm = s.m.
// The far branch is the reference's analytic tensor term for term
// (A = mu0 w_avr / r^2, dAdr, dBdr of :168-206).
#pragma once
#include "mf_device.cuh"

namespace mfgb {

constexpr double kPi = 3.14159265358979323846;
constexpr double kMu0 = 1.25663706e-6;              // Dipole_hessian.kern:170
constexpr double kForceK = 3.0 * kMu0 / (4.0 * kPi);  // far-field force prefactor
constexpr double kInv4Pi = 1.0 / (4.0 * kPi);

// Per-scene constants derived from the smoothing length.
template <class Real>
struct PairConsts {
  Real inv_h;        // 1/h
  Real ih3;          // 1/h^3
  Real ih4_over_k;   // 1/(h^4 K): scales the fitted curves into the K-free form
  Real near2_field;  // (2h)^2: field pairs closer than this take the SPH branch
  Real near2_force;  // (4h)^2: force pairs at or inside this take the fitted branch
  // FP32 kernels: the fitted-curve table in shared memory (set by the kernel
  // in its own copy; null in stored scene tables).
  const float* tbl;
};

template <class Real>
__host__ __device__ inline PairConsts<Real> make_pair_consts(double h) {
  PairConsts<Real> k;
  k.inv_h = Real(1.0 / h);
  k.ih3 = Real(1.0 / (h * h * h));
  k.ih4_over_k = Real(1.0 / (h * h * h * h * kForceK));
  k.near2_field = Real(4.0 * h * h);
  k.near2_force = Real(16.0 * h * h);
  k.tbl = nullptr;
  return k;
}

template <class Real>
__device__ __forceinline__ Real rsqrt_r(Real x);
template <>
__device__ __forceinline__ float rsqrt_r<float>(float x) {
  return rsqrt_approx(x);
}
template <>
__device__ __forceinline__ double rsqrt_r<double>(double x) {
  return rsqrt(x);
}

// Near-field SPH weights of the field kernel (Dipole_B.kern:46-76), returned as
// the (alpha, beta) pair of the form above.  Only reached for r < 2h.
template <class Real>
__device__ __noinline__ void field_near_coeffs(Real r2, const PairConsts<Real>& k, Real& alpha, Real& beta) {
  Real r = sqrt(r2);
  Real q = r * k.inv_h;
  Real tmq = Real(2) - q;
  Real tmq3 = tmq * tmq * tmq;
  Real wa, wd;  // 4 pi h^3 w_avr, 4 pi h^3 w_dens
  if (q >= Real(1)) {
    Real q2 = q * q, q3 = q2 * q;
    Real P = q3 * q3 / Real(6) - Real(6) * q3 * q2 / Real(5) + Real(3) * q2 * q2 - Real(8) * q3 / Real(3) +
             Real(1) / Real(15);
    wa = Real(-3) * P / q3;
    wd = tmq3;
  } else {
    Real q2 = q * q;
    Real omq = Real(1) - q;
    wa = (Real(15) * q2 * q - Real(36) * q2 + Real(40)) / Real(10);
    wd = tmq3 - Real(4) * omq * omq * omq;
  }
  beta = (wa / Real(3) - wd) * k.ih3;
  alpha = (r2 > Real(0)) ? (wa - wd) * k.ih3 / (Real(3) * r2) : Real(0);
}

// One field pair: s1 += d (d.s) alpha, s2 += s beta.  Field = (3 s1 - s2) / 4pi.
template <class Real>
__device__ __forceinline__ void field_pair(Real dx, Real dy, Real dz, Real sx, Real sy, Real sz,
                                           const PairConsts<Real>& k, Real* s1, Real* s2) {
  Real r2 = dx * dx + dy * dy + dz * dz;
  Real alpha, beta;
  if (r2 >= k.near2_field) {
    Real ri = rsqrt_r(r2);
    Real ri2 = ri * ri;
    beta = ri2 * ri;
    alpha = beta * ri2;
  } else {
    field_near_coeffs(r2, k, alpha, beta);
  }
  Real t = (dx * sx + dy * sy + dz * sz) * alpha;
  s1[0] += dx * t;
  s1[1] += dy * t;
  s1[2] += dz * t;
  s2[0] += sx * beta;
  s2[1] += sy * beta;
  s2[2] += sz * beta;
}

// Fitted near-field curves C1(q), C2(q), q in (0, 4]
// (Dipole_hessian.kern:53-85, magnetic_force.cu:301-330).
template <class Real>
__device__ __forceinline__ void fitted_curves(Real q, Real& c1, Real& c2) {
#define MF_P4(a, b, c, d, e) (q * (q * (q * (q * Real(a) + Real(b)) + Real(c)) + Real(d)) + Real(e))
  if (q <= Real(1)) {
    c1 = MF_P4(9.97813616438174e-09, -2.97897856524718e-08, 2.38918644566813e-09, 4.53199938857366e-08,
               2.44617454752747e-11);
    c2 = MF_P4(6.69550479838731e-08, -1.61753307173877e-07, 1.68213714992711e-08, 1.34558143036838e-07,
               1.10976027980100e-10);
  } else if (q <= Real(2)) {
    c1 = MF_P4(-2.76473728643294e-09, 2.86975546540539e-08, -9.94582836806651e-08, 1.25129924573675e-07,
               -2.37010166723652e-08);
    c2 = MF_P4(-3.08460139955194e-08, 2.29192245602275e-07, -5.88399621128587e-07, 5.61170054591844e-07,
               -1.14421132829680e-07);
  } else if (q <= Real(3)) {
    c1 = MF_P4(-1.09679990621465e-09, 9.77055663264614e-09, -2.54781238661150e-08, 2.65020634884934e-09,
               5.00787562417835e-08);
    c2 = MF_P4(3.50477408060213e-09, -5.25956271895141e-08, 2.78876509535747e-07, -6.24199554212217e-07,
               4.91807818904985e-07);
  } else {
    c1 = MF_P4(3.79927162333632e-10, -6.26368404962679e-09, 3.94760528277489e-08, -1.13580541622200e-07,
               1.27491333574323e-07);
    c2 = MF_P4(7.33485346367840e-10, -9.58855788627803e-09, 4.37085309763591e-08, -7.48004594092261e-08,
               2.34161209605651e-08);
  }
#undef MF_P4
}

// (P, Q) of the force tensor for 0 <= r <= 4h, in units of K.
template <class Real>
__device__ __noinline__ void force_near_coeffs(Real r2, const PairConsts<Real>& k, Real& P, Real& Q) {
  if (r2 == Real(0)) {
    P = Real(0);
    Q = Real(0);
    return;
  }
  Real r = sqrt(r2);
  Real q = r * k.inv_h;
  q = q > Real(4) ? Real(4) : q;  // the branch test is on r^2; keep q on the fitted range
  Real c1, c2;
  fitted_curves(q, c1, c2);
  Real ir = Real(1) / r;
  Real s = k.ih4_over_k * ir;
  P = c1 * s;
  Q = (c2 - Real(3) * c1) * s * ir * ir;
}

// (P, Q) of the force tensor for any pair, in units of K.
template <class Real>
__device__ __forceinline__ void force_coeffs(Real r2, const PairConsts<Real>& k, Real& P, Real& Q) {
  if (r2 > k.near2_force) {
    Real ri = rsqrt_r(r2);
    Real ri2 = ri * ri;
    P = ri2 * ri2 * ri;
    Q = Real(-5) * P * ri2;
  } else {
    force_near_coeffs(r2, k, P, Q);
  }
}

// One force pair contracted with the target dipole m: f += T(d, s) m / K.
template <class Real>
__device__ __forceinline__ void force_pair(Real dx, Real dy, Real dz, Real sx, Real sy, Real sz, Real mx,
                                           Real my, Real mz, const PairConsts<Real>& k, Real* f) {
  Real r2 = dx * dx + dy * dy + dz * dz;
  Real ds = dx * sx + dy * sy + dz * sz;
  Real dm = dx * mx + dy * my + dz * mz;
  Real sm = sx * mx + sy * my + sz * mz;
  Real u, v, w;
  if (r2 > k.near2_force) {
    Real ri = rsqrt_r(r2);
    Real ri2 = ri * ri;
    Real ri5 = ri2 * ri2 * ri;
    u = ds * ri5;
    v = dm * ri5;
    w = (Real(-5) * ri2 * ds) * v + sm * ri5;
  } else {
    Real P, Q;
    force_near_coeffs(r2, k, P, Q);
    u = P * ds;
    v = P * dm;
    w = P * sm + Q * ds * dm;
  }
  f[0] += dx * w + mx * u + sx * v;
  f[1] += dy * w + my * u + sy * v;
  f[2] += dz * w + mz * u + sz * v;
}

// ---------------------------------------------------------------------------
// Packed two-source forms (FP32).  Lanes .x / .y hold two different sources;
// the target's values are duplicated into both lanes.  Every pair takes the
// far form with r^2 clamped to the near radius: exact beyond it, finite inside
// it (including r = 0).  The near-field correction pass (mf_cells.cu) adds,
// for each pair inside the near radius, the exact term minus this clamped one.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 clamp_rsqrt2(float2 r2, float near2) {
  return make_float2(rsqrt_approx(fmaxf(r2.x, near2)), rsqrt_approx(fmaxf(r2.y, near2)));
}

// s1 += d (d.m) r^-5, s2 += m r^-3 (field = (3 s1 - s2) / 4pi after the lanes are added).
__device__ __forceinline__ void field_pair2(float2 tx, float2 ty, float2 tz, float2 sx, float2 sy, float2 sz,
                                            float2 mx, float2 my, float2 mz, float near2, float2* s1, float2* s2) {
  const float2 dx = f2_sub(tx, sx), dy = f2_sub(ty, sy), dz = f2_sub(tz, sz);
  const float2 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
  const float2 ri = clamp_rsqrt2(r2, near2);
  const float2 ri2 = f2_mul(ri, ri);
  const float2 beta = f2_mul(ri2, ri);
  const float2 alpha = f2_mul(beta, ri2);
  const float2 dm = f2_fma(dz, mz, f2_fma(dy, my, f2_mul(dx, mx)));
  const float2 t = f2_mul(dm, alpha);
  s1[0] = f2_fma(dx, t, s1[0]);
  s1[1] = f2_fma(dy, t, s1[1]);
  s1[2] = f2_fma(dz, t, s1[2]);
  s2[0] = f2_fma(mx, beta, s2[0]);
  s2[1] = f2_fma(my, beta, s2[1]);
  s2[2] = f2_fma(mz, beta, s2[2]);
}

// f += T(d, s) m / K with the far (P, Q) = (r^-5, -5 r^-7) of the clamped
// distance, in two parts: f gets d w + s v, and u the scalar sum of
// r^-5 (d.s) whose product with the target's dipole m completes the force
// (the caller applies it once per tile: 3 packed operations fewer per pair).
__device__ __forceinline__ void force_pair2(float2 tx, float2 ty, float2 tz, float2 tmx, float2 tmy, float2 tmz,
                                            float2 sx, float2 sy, float2 sz, float2 smx, float2 smy, float2 smz,
                                            float near2, float2* f, float2& u) {
  const float2 dx = f2_sub(tx, sx), dy = f2_sub(ty, sy), dz = f2_sub(tz, sz);
  const float2 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
  const float2 ri = clamp_rsqrt2(r2, near2);
  const float2 ri2 = f2_mul(ri, ri);
  const float2 ri5 = f2_mul(f2_mul(ri2, ri2), ri);
  const float2 ds = f2_fma(dz, smz, f2_fma(dy, smy, f2_mul(dx, smx)));
  const float2 dm = f2_fma(dz, tmz, f2_fma(dy, tmy, f2_mul(dx, tmx)));
  const float2 sm = f2_fma(smz, tmz, f2_fma(smy, tmy, f2_mul(smx, tmx)));
  const float2 v = f2_mul(dm, ri5);
  const float2 e = f2_mul(f2_mul(ri2, ds), f2_dup(-5.f));
  const float2 w = f2_fma(e, v, f2_mul(sm, ri5));
  u = f2_fma(ds, ri5, u);
  f[0] = f2_fma(dx, w, f2_fma(smx, v, f[0]));
  f[1] = f2_fma(dy, w, f2_fma(smy, v, f[1]));
  f[2] = f2_fma(dz, w, f2_fma(smz, v, f[2]));
}

// Packed two-source force tensor (6 unique entries xx, yy, zz, xy, xz, yz of
// T(d, s) / K), clamped far form: P = r^-5, Q = -5 r^-7 at max(r^2, near2).
__device__ __forceinline__ void tensor_pair2(float2 tx, float2 ty, float2 tz, float2 sx, float2 sy, float2 sz,
                                             float2 smx, float2 smy, float2 smz, float near2, float2* t) {
  const float2 dx = f2_sub(tx, sx), dy = f2_sub(ty, sy), dz = f2_sub(tz, sz);
  const float2 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
  const float2 ri = clamp_rsqrt2(r2, near2);
  const float2 ri2 = f2_mul(ri, ri);
  const float2 P = f2_mul(f2_mul(ri2, ri2), ri);
  const float2 Q = f2_mul(f2_mul(ri2, P), f2_dup(-5.f));
  const float2 ds = f2_fma(dz, smz, f2_fma(dy, smy, f2_mul(dx, smx)));
  const float2 pd = f2_mul(P, ds), qd = f2_mul(Q, ds);
  const float2 ax = f2_mul(P, smx), ay = f2_mul(P, smy), az = f2_mul(P, smz);
  const float2 two = f2_dup(2.f);
  t[0] = f2_fma(f2_mul(qd, dx), dx, f2_fma(f2_mul(two, ax), dx, f2_add(pd, t[0])));
  t[1] = f2_fma(f2_mul(qd, dy), dy, f2_fma(f2_mul(two, ay), dy, f2_add(pd, t[1])));
  t[2] = f2_fma(f2_mul(qd, dz), dz, f2_fma(f2_mul(two, az), dz, f2_add(pd, t[2])));
  t[3] = f2_fma(f2_mul(qd, dx), dy, f2_fma(ax, dy, f2_fma(ay, dx, t[3])));
  t[4] = f2_fma(f2_mul(qd, dx), dz, f2_fma(ax, dz, f2_fma(az, dx, t[4])));
  t[5] = f2_fma(f2_mul(qd, dy), dz, f2_fma(ay, dz, f2_fma(az, dy, t[5])));
}

// The clamped far coefficients every near pair received in the packed loop
// (the same rsqrt and products; equal to within rounding).
__device__ __forceinline__ void clamped_field_coeffs(float near2, float& alpha, float& beta) {
  const float ri = rsqrt_approx(near2);
  const float ri2 = ri * ri;
  beta = ri2 * ri;
  alpha = beta * ri2;
}
__device__ __forceinline__ void clamped_force_coeffs(float near2, float& P, float& Q) {
  const float ri = rsqrt_approx(near2);
  const float ri2 = ri * ri;
  P = (ri2 * ri2) * ri;
  Q = ri2 * -5.f * P;
}

// Branch-free FP32 forms of the near-field coefficients for the correction
// pass, where lanes of a warp sit on different branches: both SPH pieces are
// evaluated and selected; the fitted-curve piece is looked up in a 4 x 10
// coefficient table (c1 then c2 of each piece, highest power first).
// Same mathematics as field_near_coeffs / force_near_coeffs.
__device__ __forceinline__ void field_near_coeffs_fast(float r2, float inv_h, float ih3, float& alpha, float& beta) {
  const float ri = rsqrt_approx(r2);
  const bool pos = r2 > 0.f;
  const float r = pos ? r2 * ri : 0.f;
  const float q = r * inv_h, q2 = q * q, q3 = q2 * q;
  const float tmq = 2.f - q, tmq3 = tmq * tmq * tmq;
  const float omq = 1.f - q;
  const float Pq = q3 * (q3 * (1.f / 6.f) - q2 * (6.f / 5.f) + 3.f * q - 8.f / 3.f) + 1.f / 15.f;
  float rq3;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rq3) : "f"(fmaxf(q3, 1.f)));
  const bool hi = q >= 1.f;
  const float wa = hi ? -3.f * Pq * rq3 : (15.f * q3 - 36.f * q2 + 40.f) * 0.1f;
  const float wd = hi ? tmq3 : tmq3 - 4.f * omq * omq * omq;
  beta = (wa * (1.f / 3.f) - wd) * ih3;
  alpha = pos ? (wa - wd) * ih3 * (1.f / 3.f) * (ri * ri) : 0.f;
}

__device__ __forceinline__ void force_near_coeffs_fast(float r2, const float* __restrict__ tbl, float inv_h,
                                                       float ih4_over_k, float& P, float& Q) {
  const float ri = rsqrt_approx(r2);
  const bool pos = r2 > 0.f;
  const float r = pos ? r2 * ri : 0.f;
  const float q = fminf(r * inv_h, 4.f);
  const int piece = min(max(int(ceilf(q)) - 1, 0), 3);
  const float* c = tbl + piece * 10;
  const float c1 = q * (q * (q * (q * c[0] + c[1]) + c[2]) + c[3]) + c[4];
  const float c2 = q * (q * (q * (q * c[5] + c[6]) + c[7]) + c[8]) + c[9];
  const float s = ih4_over_k * ri;
  P = pos ? c1 * s : 0.f;
  Q = pos ? (c2 - 3.f * c1) * s * (ri * ri) : 0.f;
}

// The fitted-curve table in the layout force_near_coeffs_fast reads
// (Dipole_hessian.kern:53-61): per piece, C1 then C2, highest power first.
#define MF_FITTED_CURVE_TABLE                                                                      \
  {9.97813616438174e-09f,  -2.97897856524718e-08f, 2.38918644566813e-09f,  4.53199938857366e-08f,  \
   2.44617454752747e-11f,  6.69550479838731e-08f,  -1.61753307173877e-07f, 1.68213714992711e-08f,  \
   1.34558143036838e-07f,  1.10976027980100e-10f,  -2.76473728643294e-09f, 2.86975546540539e-08f,  \
   -9.94582836806651e-08f, 1.25129924573675e-07f,  -2.37010166723652e-08f, -3.08460139955194e-08f, \
   2.29192245602275e-07f,  -5.88399621128587e-07f, 5.61170054591844e-07f,  -1.14421132829680e-07f, \
   -1.09679990621465e-09f, 9.77055663264614e-09f,  -2.54781238661150e-08f, 2.65020634884934e-09f,  \
   5.00787562417835e-08f,  3.50477408060213e-09f,  -5.25956271895141e-08f, 2.78876509535747e-07f,  \
   -6.24199554212217e-07f, 4.91807818904985e-07f,  3.79927162333632e-10f,  -6.26368404962679e-09f, \
   3.94760528277489e-08f,  -1.13580541622200e-07f, 1.27491333574323e-07f,  7.33485346367840e-10f,  \
   -9.58855788627803e-09f, 4.37085309763591e-08f,  -7.48004594092261e-08f, 2.34161209605651e-08f}

// FP32 exact pair forms without a branch: the far coefficients and the fast
// near coefficients above are both evaluated and selected by the radius, so
// warps whose lanes straddle the near radius do not diverge.  Same
// mathematics as field_pair / force_pair (the far value at r = 0 is infinite
// and discarded by the select).  The force needs k.tbl.
__device__ __forceinline__ void field_pair_sel(float dx, float dy, float dz, float sx, float sy, float sz,
                                               const PairConsts<float>& k, float* s1, float* s2) {
  const float r2 = dx * dx + dy * dy + dz * dz;
  float al, be;
  field_near_coeffs_fast(r2, k.inv_h, k.ih3, al, be);
  const float ri = rsqrt_approx(r2), ri2 = ri * ri, ri3 = ri2 * ri;
  const bool far = r2 >= k.near2_field;
  const float beta = far ? ri3 : be;
  const float alpha = far ? ri3 * ri2 : al;
  const float t = (dx * sx + dy * sy + dz * sz) * alpha;
  s1[0] += dx * t;
  s1[1] += dy * t;
  s1[2] += dz * t;
  s2[0] += sx * beta;
  s2[1] += sy * beta;
  s2[2] += sz * beta;
}

__device__ __forceinline__ void force_pair_sel(float dx, float dy, float dz, float sx, float sy, float sz, float mx,
                                               float my, float mz, const PairConsts<float>& k, float* f) {
  const float r2 = dx * dx + dy * dy + dz * dz;
  const float ds = dx * sx + dy * sy + dz * sz;
  const float dm = dx * mx + dy * my + dz * mz;
  const float sm = sx * mx + sy * my + sz * mz;
  float Pn, Qn;
  force_near_coeffs_fast(r2, k.tbl, k.inv_h, k.ih4_over_k, Pn, Qn);
  const float ri = rsqrt_approx(r2), ri2 = ri * ri, ri5 = ri2 * ri2 * ri;
  const bool far = r2 > k.near2_force;
  const float P = far ? ri5 : Pn;
  const float Q = far ? -5.f * ri5 * ri2 : Qn;
  const float u = P * ds, v = P * dm, w = P * sm + Q * ds * dm;
  f[0] += dx * w + mx * u + sx * v;
  f[1] += dy * w + my * u + sy * v;
  f[2] += dz * w + mz * u + sz * v;
}

// Correction of one near field pair (r^2 < near2): exact minus clamped,
// accumulated as s1 (d (d.m) dalpha) and s2 (m dbeta) like the packed loop.
__device__ __forceinline__ void field_near_correction(float dx, float dy, float dz, float mx, float my, float mz,
                                                      const PairConsts<float>& pc, float alpha_c, float beta_c,
                                                      float* s1, float* s2) {
  const float r2 = dx * dx + dy * dy + dz * dz;
  float alpha, beta;
  field_near_coeffs<float>(r2, pc, alpha, beta);
  const float da = alpha - alpha_c, db = beta - beta_c;
  const float t = (dx * mx + dy * my + dz * mz) * da;
  s1[0] += dx * t;
  s1[1] += dy * t;
  s1[2] += dz * t;
  s2[0] += mx * db;
  s2[1] += my * db;
  s2[2] += mz * db;
}

// Correction of one near force pair (r^2 <= near2), contracted with m.
// Tensor correction of one near pair (r^2 <= near2): exact minus clamped,
// the 6 entries (xx, yy, zz, xy, xz, yz) of T / K.
__device__ __forceinline__ void tensor_near_correction(float dx, float dy, float dz, float sx, float sy, float sz,
                                                       const PairConsts<float>& pc, float P_c, float Q_c, float* t) {
  const float r2 = dx * dx + dy * dy + dz * dz;
  float P, Q;
  force_near_coeffs<float>(r2, pc, P, Q);
  const float dP = P - P_c, dQ = Q - Q_c;
  const float ds = dx * sx + dy * sy + dz * sz;
  const float pd = dP * ds, qd = dQ * ds;
  const float ax = dP * sx, ay = dP * sy, az = dP * sz;
  t[0] += pd + 2.f * ax * dx + qd * dx * dx;
  t[1] += pd + 2.f * ay * dy + qd * dy * dy;
  t[2] += pd + 2.f * az * dz + qd * dz * dz;
  t[3] += ax * dy + ay * dx + qd * dx * dy;
  t[4] += ax * dz + az * dx + qd * dx * dz;
  t[5] += ay * dz + az * dy + qd * dy * dz;
}

__device__ __forceinline__ void force_near_correction(float dx, float dy, float dz, float sx, float sy, float sz,
                                                      float mx, float my, float mz, const PairConsts<float>& pc,
                                                      float P_c, float Q_c, float* f) {
  const float r2 = dx * dx + dy * dy + dz * dz;
  float P, Q;
  force_near_coeffs<float>(r2, pc, P, Q);
  const float dP = P - P_c, dQ = Q - Q_c;
  const float ds = dx * sx + dy * sy + dz * sz;
  const float dm = dx * mx + dy * my + dz * mz;
  const float sm = sx * mx + sy * my + sz * mz;
  const float u = dP * ds, v = dP * dm, w = dP * sm + dQ * ds * dm;
  f[0] += dx * w + mx * u + sx * v;
  f[1] += dy * w + my * u + sy * v;
  f[2] += dz * w + mz * u + sz * v;
}

// One tensor pair (6 unique entries xx, yy, zz, xy, xz, yz): t += T(d, s) / K.
template <class Real>
__device__ __forceinline__ void tensor_pair(Real dx, Real dy, Real dz, Real sx, Real sy, Real sz,
                                            const PairConsts<Real>& k, Real* t) {
  Real r2 = dx * dx + dy * dy + dz * dz;
  Real P, Q;
  force_coeffs(r2, k, P, Q);
  Real ds = dx * sx + dy * sy + dz * sz;
  Real pd = P * ds, qd = Q * ds;
  Real ax = P * sx, ay = P * sy, az = P * sz;
  t[0] += pd + Real(2) * ax * dx + qd * dx * dx;
  t[1] += pd + Real(2) * ay * dy + qd * dy * dy;
  t[2] += pd + Real(2) * az * dz + qd * dz * dz;
  t[3] += ax * dy + ay * dx + qd * dx * dy;
  t[4] += ax * dz + az * dx + qd * dx * dz;
  t[5] += ay * dz + az * dy + qd * dy * dz;
}

}  // namespace mfgb
