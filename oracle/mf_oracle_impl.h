/*
 * mf_oracle_impl.h -- TEST INFRASTRUCTURE, not product code.
 *
 * Type-generic body of the CPU oracle.  mf_oracle.c includes this file twice:
 * once with REAL=double / SFX=_f64 (the FP64 restatement every parity test
 * checks against) and once with REAL=float / SFX=_f32 (the same arithmetic in
 * the reference's own precision, used as the timed CPU baseline).
 *
 * Every function restates one piece of the reference's algorithm and cites the
 * file:line (paths within ureternalreward/magnetic-force) it follows.  Nothing
 * here is called by the shipped library.
 */
#ifndef REAL
#error "define REAL and SFX before including mf_oracle_impl.h"
#endif

#define ORC_CAT2(a, b) a##b
#define ORC_CAT(a, b) ORC_CAT2(a, b)
#define ORC(name) ORC_CAT(name, SFX)

/* ------------------------------------------------------------------------ */
/* Pair kernel for the B/mu0 field.                                          */
/* fmmtl_minimum/kernel/Dipole_B.kern:46-76 (get_weight) and :79-104          */
/* (operator*), identical in meaning to magnetic_solver/magnetic_force.cu:63-98 */
/* (cuda_Apply_G inner loop).  d = target - source, m = source dipole.        */
/* ------------------------------------------------------------------------ */
static void ORC(orc_weight)(REAL r, REAL h, REAL *w_avr, REAL *w_dens) {
  const REAL one_over_pi = (REAL)ORC_M_1_PI;
  REAL q = r * ((REAL)1 / h);
  REAL q2 = q * q;
  REAL q3 = q2 * q;
  REAL coe = one_over_pi * ((REAL)1 / (h * h * h));
  if (q >= 2) { /* Dipole_B.kern:55-59 */
    *w_avr = (REAL)0.75 * one_over_pi * ((REAL)1 / (r * r * r));
    *w_dens = 0;
    return;
  }
  if (q >= 1) { /* Dipole_B.kern:60-67 */
    *w_avr = -((REAL)3 * (q3 * q3 / (REAL)6 - ((REAL)6 * q3 * q2) / (REAL)5 +
                          (REAL)3 * q2 * q2 - ((REAL)8 * q3) / (REAL)3 + (REAL)1 / (REAL)15)) *
             one_over_pi * ((REAL)1 / ((REAL)4 * r * r * r));
    REAL tmq = (REAL)2 - q;
    *w_dens = coe * (REAL)0.25 * tmq * tmq * tmq;
    return;
  }
  { /* q < 1, Dipole_B.kern:68-75 */
    *w_avr = (q * q * ((REAL)15 / (REAL)40 * q - (REAL)36 / (REAL)40) + (REAL)1) * coe;
    REAL tmq = (REAL)2 - q;
    REAL omq = (REAL)1 - q;
    *w_dens = coe * ((REAL)0.25 * tmq * tmq * tmq - omq * omq * omq);
  }
}

void ORC(orc_pair_field)(const REAL d[3], const REAL m[3], REAL h, REAL out[3]) {
  REAL r = (REAL)sqrt((double)(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
  REAL invr = (r == 0) ? (REAL)1 : (REAL)1 / r; /* Dipole_B.kern:88 */
  REAL rx = d[0] * invr, ry = d[1] * invr, rz = d[2] * invr;
  REAL w_avr, w_dens;
  ORC(orc_weight)(r, h, &w_avr, &w_dens);
  REAL v1 = (rx * m[0] + ry * m[1] + rz * m[2]) * (w_avr - w_dens); /* :97 */
  REAL v2 = w_avr * (REAL)(1.0 / 3.0) - w_dens;                    /* :98 */
  out[0] = rx * v1 - v2 * m[0];
  out[1] = ry * v1 - v2 * m[1];
  out[2] = rz * v1 - v2 * m[2];
}

/* ------------------------------------------------------------------------ */
/* Pair force tensor.  fmmtl_minimum/kernel/Dipole_hessian.kern:53-238,       */
/* identical in meaning to magnetic_solver/magnetic_force.cu:239-427.          */
/* T is a 3x3 in glm's column-major layout: T[c*3 + r] = column c, row r, and */
/* the force on a target dipole mt is F[r] = sum_c T[c*3+r] * mt[c].           */
/* ------------------------------------------------------------------------ */
static REAL ORC(orc_poly4)(const double *c, REAL x) {
  /* DEF_POLY4_FUNC, Dipole_hessian.kern:13-17 */
  return x * (x * (x * (x * (REAL)c[0] + (REAL)c[1]) + (REAL)c[2]) + (REAL)c[3]) + (REAL)c[4];
}

static void ORC(orc_curves)(REAL q, REAL *c1, REAL *c2) {
  /* evaluate_curve1_2, Dipole_hessian.kern:63-85.  Outside (0,4] the
     reference leaves C1/C2 unset; callers only reach here with 0<q<=4. */
  int piece = -1;
  if (0 < q && q <= 1) piece = 0;
  else if (1 < q && q <= 2) piece = 1;
  else if (2 < q && q <= 3) piece = 2;
  else if (3 < q && q <= 4) piece = 3;
  if (piece < 0) { *c1 = 0; *c2 = 0; return; }
  *c1 = ORC(orc_poly4)(ORC_C1[piece], q);
  *c2 = ORC(orc_poly4)(ORC_C2[piece], q);
}

static void ORC(orc_normalize)(REAL v[3]) {
  /* glm::normalize: v * inversesqrt(dot(v, v)) */
  REAL s = (REAL)1 / (REAL)sqrt((double)(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
  v[0] *= s; v[1] *= s; v[2] *= s;
}

static void ORC(orc_cross)(const REAL a[3], const REAL b[3], REAL o[3]) {
  o[0] = a[1] * b[2] - b[1] * a[2];
  o[1] = a[2] * b[0] - b[2] * a[0];
  o[2] = a[0] * b[1] - b[0] * a[1];
}

static void ORC(orc_force_far)(REAL T[9], const REAL d[3], const REAL s[3], REAL q, REAL h) {
  /* get_far_field_force_tensor, Dipole_hessian.kern:155-207 */
  REAL r = q * h;
  REAL w_avr = (REAL)3 / ((REAL)4 * (REAL)ORC_PI * r * r * r);
  REAL invr = 1;
  if (r != 0) invr = (REAL)1 / r;
  const REAL mu_0 = (REAL)ORC_MU0;
  REAL A = mu_0 * invr * invr * (w_avr);
  REAL rdotm = d[0] * s[0] + d[1] * s[1] + d[2] * s[2];
  REAL dAdr = mu_0 * invr * invr * ((REAL)5 * invr * (-w_avr)) * rdotm * invr;
  REAL dBdr = mu_0 * invr * (-w_avr) * invr;
  /* T[c*3+r] += d_r s_c A + d_r dAdr d_c - s_r dBdr d_c  (+ rdotm*A on the diagonal) */
  for (int c = 0; c < 3; ++c)
    for (int rr = 0; rr < 3; ++rr) {
      T[c * 3 + rr] += d[rr] * s[c] * A + d[rr] * dAdr * d[c] - s[rr] * dBdr * d[c];
      if (c == rr) T[c * 3 + rr] += rdotm * A;
    }
}

static void ORC(orc_force_near)(REAL T[9], const REAL d[3], const REAL s[3], REAL q, REAL h) {
  /* get_near_field_force_tensor, Dipole_hessian.kern:88-152 */
  if (q == 0) return; /* overlapping particles: no force, :101-104 */
  REAL c1, c2;
  ORC(orc_curves)(q, &c1, &c2);
  c1 *= (REAL)1 / (h * h * h * h);
  c2 *= (REAL)1 / (h * h * h * h);
  REAL zeta[3] = {d[0], d[1], d[2]};
  ORC(orc_normalize)(zeta);
  const REAL zax[3] = {0, 0, 1};
  REAL eta[3];
  ORC(orc_cross)(zeta, zax, eta);
  eta[1] += (REAL)1e-10; /* degenerate-axis nudge, :116 */
  ORC(orc_normalize)(eta);
  REAL xi[3];
  ORC(orc_cross)(eta, zeta, xi);
  /* M = [xi eta zeta] as columns; s' = M^T s  (:122-131) */
  const REAL *Mc[3] = {xi, eta, zeta};
  REAL sp[3];
  for (int k = 0; k < 3; ++k) sp[k] = Mc[k][0] * s[0] + Mc[k][1] * s[1] + Mc[k][2] * s[2];
  /* U, symmetric, rows: (sz c1, 0, sx c1) (0, sz c1, sy c1) (sx c1, sy c1, sz c2)  (:136-139) */
  REAL U[3][3] = {{sp[2] * c1, 0, sp[0] * c1},
                  {0, sp[2] * c1, sp[1] * c1},
                  {sp[0] * c1, sp[1] * c1, sp[2] * c2}};
  /* T += M U M^T  (:151): (M U M^T)[r][c] = sum_ij M[r][i] U[i][j] M[c][j], M[r][i] = Mc[i][r] */
  for (int c = 0; c < 3; ++c)
    for (int rr = 0; rr < 3; ++rr) {
      REAL acc = 0;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) acc += Mc[i][rr] * U[i][j] * Mc[j][c];
      T[c * 3 + rr] += acc;
    }
}

void ORC(orc_pair_force_tensor)(const REAL d[3], const REAL s[3], REAL h, REAL T[9]) {
  /* get_force_Tensor, Dipole_hessian.kern:212-238; T is accumulated into. */
  REAL r = (REAL)sqrt((double)(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
  REAL q = r * ((REAL)1 / h);
  if (q > 4) ORC(orc_force_far)(T, d, s, q, h);
  else ORC(orc_force_near)(T, d, s, q, h);
}

/* ------------------------------------------------------------------------ */
/* All-pairs sums (fmmtl::direct, fmmtl_minimum/fmmtl/Direct.hpp:18-28 ->       */
/* S2T.hpp:57-79; magnetic_force.cu:8-110 for the field, :432-512 for the      */
/* tensor).  Positions / moments are AoS [n][3].  Parallel over targets.       */
/* ------------------------------------------------------------------------ */
void ORC(orc_field)(int64_t nt, const REAL *tpos, int64_t ns, const REAL *spos,
                    const REAL *smom, REAL h, REAL *out) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < nt; ++i) {
    REAL acc[3] = {0, 0, 0};
    for (int64_t j = 0; j < ns; ++j) {
      REAL d[3] = {tpos[3 * i] - spos[3 * j], tpos[3 * i + 1] - spos[3 * j + 1],
                   tpos[3 * i + 2] - spos[3 * j + 2]};
      REAL o[3];
      ORC(orc_pair_field)(d, &smom[3 * j], h, o);
      acc[0] += o[0]; acc[1] += o[1]; acc[2] += o[2];
    }
    out[3 * i] = acc[0]; out[3 * i + 1] = acc[1]; out[3 * i + 2] = acc[2];
  }
}

void ORC(orc_tensor_sum)(int64_t nt, const REAL *tpos, int64_t ns, const REAL *spos,
                         const REAL *smom, REAL h, REAL *T9) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < nt; ++i) {
    REAL T[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t j = 0; j < ns; ++j) {
      REAL d[3] = {tpos[3 * i] - spos[3 * j], tpos[3 * i + 1] - spos[3 * j + 1],
                   tpos[3 * i + 2] - spos[3 * j + 2]};
      ORC(orc_pair_force_tensor)(d, &smom[3 * j], h, T);
    }
    for (int k = 0; k < 9; ++k) T9[9 * i + k] = T[k];
  }
}

/* Kelvin force on each particle of the object.
 * naive_quirks == 0: the reference's default (FMM) path,
 *   magnetic_force.cu:968-980: F = (Rext + sum_j T_ij) . m_i.
 * naive_quirks != 0: the reference's naive CUDA path,
 *   magnetic_force.cu:583-603: F = (sum_j T_ij) . m_i + mu0 * Rext^T . m_i
 *   (the external tensor already holds mu0, so mu0 enters twice).
 * Rext is [n][9] in the column-major layout above (may be NULL = zero). */
void ORC(orc_force)(int64_t n, const REAL *pos, const REAL *mom, REAL h, const REAL *rext,
                    int naive_quirks, REAL *F) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < n; ++i) {
    REAL T[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t j = 0; j < n; ++j) {
      REAL d[3] = {pos[3 * i] - pos[3 * j], pos[3 * i + 1] - pos[3 * j + 1],
                   pos[3 * i + 2] - pos[3 * j + 2]};
      ORC(orc_pair_force_tensor)(d, &mom[3 * j], h, T);
    }
    const REAL *m = &mom[3 * i];
    REAL f[3];
    for (int rr = 0; rr < 3; ++rr) f[rr] = T[rr] * m[0] + T[3 + rr] * m[1] + T[6 + rr] * m[2];
    if (rext) {
      const REAL *R = &rext[9 * i];
      if (!naive_quirks) {
        for (int rr = 0; rr < 3; ++rr) f[rr] += R[rr] * m[0] + R[3 + rr] * m[1] + R[6 + rr] * m[2];
      } else {
        const REAL mu_0 = (REAL)ORC_MU0;
        for (int rr = 0; rr < 3; ++rr)
          f[rr] += mu_0 * (m[0] * R[rr * 3 + 0] + m[1] * R[rr * 3 + 1] + m[2] * R[rr * 3 + 2]);
      }
    }
    F[3 * i] = f[0]; F[3 * i + 1] = f[1]; F[3 * i + 2] = f[2];
  }
}

/* External field and its gradient tensor from external dipole sources plus a
 * uniform field (eval_hext, magnetic_force.cu:1102-1192; naive kernels
 * :120-237 and :432-512).  hs is the smoothing length the sources use. */
void ORC(orc_ext)(int64_t n, const REAL *pos, int64_t ns, const REAL *spos, const REAL *smom,
                  const REAL H0[3], REAL hs, REAL *hext, REAL *rext) {
  if (hext) {
    if (ns > 0) ORC(orc_field)(n, pos, ns, spos, smom, hs, hext);
    else for (int64_t i = 0; i < 3 * n; ++i) hext[i] = 0;
    for (int64_t i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) hext[3 * i + k] += H0[k];
  }
  if (rext) {
    if (ns > 0) ORC(orc_tensor_sum)(n, pos, ns, spos, smom, hs, rext);
    else for (int64_t i = 0; i < 9 * n; ++i) rext[i] = 0;
  }
}

#undef ORC
#undef ORC_CAT
#undef ORC_CAT2
