/*
 * mf_oracle.c -- TEST INFRASTRUCTURE, not product code.
 *
 * CPU restatement of the reference's magnetization-and-force step
 * (ureternalreward/magnetic-force, magnetic_solver/ + fmmtl_minimum/kernel/).
 * It is the checker for the CUDA library: only tests/, the smoke check and the
 * CPU-baseline leg of bench.py load it.  The shipped library never calls it.
 *
 * Pinning: the pair kernels and all-pairs sums here are checked against the
 * reference's own FMMTL kernels (Dipole_B.kern, Dipole_hessian.kern) compiled
 * from the reference sources by oracle/Makefile into oracle/_ref, and against
 * golden vectors that library produced (tests/golden/).  The solver loops are
 * restatements of magnetic_force.cu:874-1095 and :1275-1315; the reference
 * solver itself needs a GPU and the reference's CUDA build, so its iterates are
 * pinned through these restated loops running on the pinned kernels.
 *
 * Layout: positions, moments and fields are AoS arrays [n][3]; tensors are
 * [n][9] in glm column-major order (T[c*3+r] = column c, row r).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_M_1_PI 0.318309886183790671537767526745028724
#define ORC_PI 3.14159265358979323846264338327950288
/* mu_0 as written in Dipole_hessian.kern:170 and magnetic_force.cu:254 */
#define ORC_MU0 1.25663706e-6

/* Fitted near-field force curves, Dipole_hessian.kern:53-61 (also
 * magnetic_force.cu:301-309): four quartic pieces on (0,1], (1,2], (2,3],
 * (3,4], coefficients from the x^4 term down to the constant. */
static const double ORC_C1[4][5] = {
    {9.97813616438174e-09, -2.97897856524718e-08, 2.38918644566813e-09, 4.53199938857366e-08,
     2.44617454752747e-11},
    {-2.76473728643294e-09, 2.86975546540539e-08, -9.94582836806651e-08, 1.25129924573675e-07,
     -2.37010166723652e-08},
    {-1.09679990621465e-09, 9.77055663264614e-09, -2.54781238661150e-08, 2.65020634884934e-09,
     5.00787562417835e-08},
    {3.79927162333632e-10, -6.26368404962679e-09, 3.94760528277489e-08, -1.13580541622200e-07,
     1.27491333574323e-07}};
static const double ORC_C2[4][5] = {
    {6.69550479838731e-08, -1.61753307173877e-07, 1.68213714992711e-08, 1.34558143036838e-07,
     1.10976027980100e-10},
    {-3.08460139955194e-08, 2.29192245602275e-07, -5.88399621128587e-07, 5.61170054591844e-07,
     -1.14421132829680e-07},
    {3.50477408060213e-09, -5.25956271895141e-08, 2.78876509535747e-07, -6.24199554212217e-07,
     4.91807818904985e-07},
    {7.33485346367840e-10, -9.58855788627803e-09, 4.37085309763591e-08, -7.48004594092261e-08,
     2.34161209605651e-08}};

#define REAL double
#define SFX _f64
#include "mf_oracle_impl.h"
#undef REAL
#undef SFX

#define REAL float
#define SFX _f32
#include "mf_oracle_impl.h"
#undef REAL
#undef SFX

/* ------------------------------------------------------------------------ */
/* Solvers (FP64).                                                           */
/* ------------------------------------------------------------------------ */
static double dot3n(int64_t n, const double *a, const double *b) {
  double s = 0;
  for (int64_t i = 0; i < 3 * n; ++i) s += a[i] * b[i];
  return s;
}

/* G(in): the B/mu0 field of dipoles `in` at the object's own particles,
 * self term included (magnetic_force.cu:1196-1222). */
static void apply_G(int64_t n, const double *pos, double h, const double *in, double *out) {
  orc_field_f64(n, pos, n, pos, in, h, out);
}

/* D(x) = G(c x) - x  (magnetic_force.cu:1275-1278). */
static void apply_D(int64_t n, const double *pos, double h, double c, const double *x,
                    double *tmp, double *out) {
  for (int64_t i = 0; i < 3 * n; ++i) tmp[i] = c * x[i];
  apply_G(n, pos, h, tmp, out);
  for (int64_t i = 0; i < 3 * n; ++i) out[i] -= x[i];
}

/* D^T(x) = c G(x) - x  (magnetic_force.cu:1281-1284; G is symmetric). */
static void apply_DT(int64_t n, const double *pos, double h, double c, const double *x,
                     double *out) {
  apply_G(n, pos, h, x, out);
  for (int64_t i = 0; i < 3 * n; ++i) out[i] = c * out[i] - x[i];
}

/* The reference's least-squares nonlinear conjugate-gradient solve of
 * b = Hext + G(c b), c = V chi/(1+chi), restated step by step:
 *   solve()           magnetic_force.cu:874-888
 *   start()           :1008-1040
 *   step_iteration()  :1043-1095
 *   calc_alpha()      :1287-1302
 *   calc_beta()       :1305-1315
 * b holds the warm start on entry and the result on exit.  errors[] receives
 * the 0.5*|r|^2 history (total_error), *n_errors its length.  Returns the
 * number of step_iteration() calls made. */
int orc_solve_nlcg(int64_t n, const double *pos, double h, double volume, double chi,
                   const double *hext, double *b, double tolerance, int64_t niter,
                   int64_t max_iteration, double *errors, int64_t *n_errors) {
  const double c = volume * chi / (chi + 1);
  size_t bytes = sizeof(double) * 3 * (size_t)(n > 0 ? n : 1);
  double *r = malloc(bytes), *g = malloc(bytes), *d = malloc(bytes), *gold = malloc(bytes),
         *dold = malloc(bytes), *tmp = malloc(bytes), *tmp2 = malloc(bytes), *Dd = malloc(bytes);
  int64_t ne = 0;
  int steps = 0;
  int64_t i_step = 0;

  /* residual = G(c b) + Hext - b */
#define RESIDUAL()                                              \
  do {                                                          \
    for (int64_t k = 0; k < 3 * n; ++k) tmp[k] = c * b[k];      \
    apply_G(n, pos, h, tmp, r);                                 \
    for (int64_t k = 0; k < 3 * n; ++k) r[k] += hext[k] - b[k]; \
  } while (0)
  /* alpha = -(Dd . r) / (Dd . Dd + eps), 0 when Dd . Dd < eps */
#define ALPHA(out)                                         \
  do {                                                     \
    apply_D(n, pos, h, c, d, tmp2, Dd);                    \
    double nt = dot3n(n, Dd, Dd);                          \
    (out) = (nt < 1e-10) ? 0.0 : -(dot3n(n, Dd, r) / (nt + 1e-10)); \
  } while (0)

  /* start() */
  RESIDUAL();
  double err = 0.5 * dot3n(n, r, r);
  errors[ne++] = err;
  if (!(sqrt(err / (double)n) < tolerance)) {
    apply_DT(n, pos, h, c, r, g);
    for (int64_t k = 0; k < 3 * n; ++k) d[k] = -g[k];
    double alpha;
    ALPHA(alpha);
    for (int64_t k = 0; k < 3 * n; ++k) b[k] += alpha * d[k];
    /* solve(): step_iteration() up to min(niter, max_iteration) times */
    for (int64_t it = 0; it < niter && it < max_iteration; ++it) {
      ++steps;
      memcpy(gold, g, bytes);
      memcpy(dold, d, bytes);
      RESIDUAL();
      err = 0.5 * dot3n(n, r, r);
      errors[ne++] = err;
      if (sqrt(err / (double)n) < tolerance) break;
      if (err > errors[ne - 2]) break;
      ++i_step;
      apply_DT(n, pos, h, c, r, g);
      double beta = 0;
      if (i_step % 10 != 0) {
        /* calc_beta: -|g|^2 / (d_old . (g_old - g) + 1e-10), clamped at 0 */
        double numer = dot3n(n, g, g);
        double denom = 0;
        for (int64_t k = 0; k < 3 * n; ++k) denom += dold[k] * (gold[k] - g[k]);
        beta = -numer / (denom + 1e-10);
        if (beta < 0) beta = 0;
      }
      for (int64_t k = 0; k < 3 * n; ++k) d[k] = -g[k] + beta * dold[k];
      double alpha;
      ALPHA(alpha);
      for (int64_t k = 0; k < 3 * n; ++k) b[k] += alpha * d[k];
    }
  }
#undef RESIDUAL
#undef ALPHA
  *n_errors = ne;
  free(r); free(g); free(d); free(gold); free(dold); free(tmp); free(tmp2); free(Dd);
  return steps;
}

/* Tight solve of the same fixed point, (I - c G) b = Hext, by conjugate
 * gradients in FP64 (I - c G is symmetric positive definite for chi > -1 at
 * the densities used here).  This is the converged solution every result is
 * compared against.  Returns iterations; *rel_res gets |r|/|Hext|. */
int orc_solve_cg(int64_t n, const double *pos, double h, double c, const double *hext,
                 double *b, double rel_tol, int max_iter, double *rel_res) {
  size_t bytes = sizeof(double) * 3 * (size_t)(n > 0 ? n : 1);
  double *r = malloc(bytes), *p = malloc(bytes), *q = malloc(bytes);
  /* r = Hext - (b - c G b) */
  apply_G(n, pos, h, b, q);
  for (int64_t k = 0; k < 3 * n; ++k) r[k] = hext[k] - (b[k] - c * q[k]);
  memcpy(p, r, bytes);
  double rr = dot3n(n, r, r);
  double bnorm = sqrt(dot3n(n, hext, hext));
  if (bnorm == 0) bnorm = 1;
  int it = 0;
  while (sqrt(rr) / bnorm > rel_tol && it < max_iter) {
    apply_G(n, pos, h, p, q);
    for (int64_t k = 0; k < 3 * n; ++k) q[k] = p[k] - c * q[k];
    double alpha = rr / dot3n(n, p, q);
    for (int64_t k = 0; k < 3 * n; ++k) { b[k] += alpha * p[k]; r[k] -= alpha * q[k]; }
    double rr2 = dot3n(n, r, r);
    double beta = rr2 / rr;
    rr = rr2;
    for (int64_t k = 0; k < 3 * n; ++k) p[k] = r[k] + beta * p[k];
    ++it;
  }
  /* true residual for the report */
  apply_G(n, pos, h, b, q);
  for (int64_t k = 0; k < 3 * n; ++k) r[k] = hext[k] - (b[k] - c * q[k]);
  *rel_res = sqrt(dot3n(n, r, r)) / bnorm;
  free(r); free(p); free(q);
  return it;
}

/* Symplectic Euler step of the benchmark harness (not part of the reference):
 * v += dt F / (rho V); x += dt v, unit density. */
void orc_symplectic_euler(int64_t n, double *pos, double *vel, const double *F, double mass,
                          double dt) {
  for (int64_t i = 0; i < 3 * n; ++i) {
    vel[i] += dt * F[i] / mass;
    pos[i] += dt * vel[i];
  }
}

int orc_abi_version(void) { return 1; }
