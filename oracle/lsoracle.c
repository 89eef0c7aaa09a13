/*
 * lsoracle.c -- CPU oracle for the narrowband level-set time step.
 * TEST INFRASTRUCTURE ONLY (see lsoracle.h): the checker, never the product.
 *
 * Restates GPUTUM Level-Set's layout build, seeding, patch-scheduled fast
 * iterative method, narrowband selection and advection / curvature update
 * in serial C (patch visits of one FIM iteration are independent and run
 * under OpenMP; the result does not depend on the thread count because a
 * visit reads DT and writes only its own patch's entries of DT_out).
 */
#include "lsoracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { LSO_SEED = 0, LSO_ACTIVE = 1, LSO_ALIVE = 2, LSO_FAR = 3 };
/* per-vertex slots the reference's patch kernels keep (l_mem) */
#define LSO_SLOT_CAP(dim) ((dim) == 3 ? 32 : 16)

struct lso_layout {
  int dim, nv, ne, nparts, full, lep, lvp, lim, nadj;
  int* ele_permute;   /* full: original element id of each copy            */
  int* ele_offsets;   /* nparts+1                                          */
  int* vert_permute;  /* nv: new -> old                                    */
  int* vert_ipermute; /* nv: old -> new                                    */
  int* vert_offsets;  /* nparts+1                                          */
  int* conn;          /* full*(d+1), AoS, new vertex ids                   */
  int* vslot_off;     /* nv+1                                              */
  int* vslot;         /* per owned vertex: local slots in reference order  */
  int* block_xadj;    /* nparts+1 (reference construction)                 */
  int* block_adjncy;  /* nadj                                              */
  float* xyz_p;       /* 3*nv SoA, permuted                                */
  float* lc32;        /* full*6 (tet) AoS: FP32 local coordinates          */
  double mean_edge;
};

static double now_sec(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int lso_version(void) { return 1; }

/* ------------------------------------------------------------------------ */
/* Local tet solver, FP32 with the reference's promotions.
 * src/core3d/include/redistance_kernels3d.h:124-285.  `(x) / (2.0 * p)` and
 * `/ (h + SMALLNUM)` are evaluated in double and rounded back to float, as
 * the double literals make them in the reference. */
/* Roots of p x^2 + q x + r without cancellation (precision form): s / p
 * (root_a) and r / s (root_b) with s = -(q + sign(q) sqrt(delta)) / 2 -- the
 * reference's two roots (-q +- sqrt(delta)) / 2p, in an order that depends on
 * the sign of q (every caller takes the minimum over both). */
static float stable_s(float q, float delta) {
  float sq = sqrtf(delta);
  return -(q + (q >= 0.0f ? sq : -sq)) * 0.5f;
}
static float root_a(float p, float q, float r, float delta) { return stable_s(q, delta) / p; }
static float root_b(float p, float q, float r, float delta) { return r / stable_s(q, delta); }

/* Precision form (ill != NULL, tau > 0): a solve whose candidates cannot
 * fall below `cutoff` (the target's current value) is skipped -- every
 * candidate is at least min(TA, TB, TC) plus D's height over the plane ABC
 * (Gram determinants of AC, BC, CD; taken x 0.999); otherwise a quadratic
 * whose arrival times are all below LN and whose discriminant cancels flags
 * the solve for an FP64 repeat, and the quadratic roots are taken in the
 * cancellation-free form. */
static float tet_f32_impl(float TA, float TB, float TC, float ACAC, float ACBC,
                          float ACCD, float BCBC, float BCCD, float CDCD,
                          double eps_h, float LN, float tau, int* ill, int fdiv, float cutoff) {
  if (TA >= LN && TB >= LN && TC >= LN) return LN;
  if (ill) {
    float det2 = ACAC * BCBC - ACBC * ACBC;
    float det3 = ACAC * (BCBC * CDCD - BCCD * BCCD) - ACBC * (ACBC * CDCD - BCCD * ACCD) +
                 ACCD * (ACBC * BCCD - BCBC * ACCD);
    float lb = fminf(fminf(TA, TB), TC) + 0.999f * sqrtf(fmaxf(det3 / det2, 0.0f));
    if (lb >= cutoff) return LN;
  }
  float p, q, r, lambda1, lambda2, lambda3;
  float FaceTAC = LN, FaceTAB = LN, FaceTBC = LN;
  float delta, TE, TD = LN;
  float TAC = TC - TA, TBC = TC - TB, TAB = TB - TA;

  /* face BC (lambda1 = 0) */
  p = BCBC * TBC * TBC - BCBC * BCBC;
  q = (BCCD + BCCD) * TBC * TBC - 2 * BCBC * BCCD;
  r = TBC * TBC * CDCD - BCCD * BCCD;
  delta = q * q - 4 * p * r;
  if (ill && fmaxf(TB, TC) < LN && fabsf(delta) <= tau * (q * q + fabsf(4 * p * r))) *ill = 1;
  if (delta >= 0.0) {
    lambda1 = 0.0f;
    lambda2 = ill ? root_a(p, q, r, delta) : (float)((double)(-q + sqrtf(delta)) / (2.0 * (double)p));
    lambda3 = 1 - lambda1 - lambda2;
    if (lambda2 >= 0 && lambda2 <= 1) {
      TE = TB * lambda2 + TC * lambda3;
      FaceTBC = fminf(FaceTBC, TE + sqrtf((lambda2 * BCBC + BCCD) * lambda2 + (lambda2 * BCCD + CDCD)));
    }
    lambda1 = 0.0f;
    lambda2 = ill ? root_b(p, q, r, delta) : (float)((double)(-q - sqrtf(delta)) / (2.0 * (double)p));
    lambda3 = 1 - lambda1 - lambda2;
    if (lambda2 >= 0 && lambda2 <= 1) {
      TE = TB * lambda2 + TC * lambda3;
      FaceTBC = fminf(FaceTBC, TE + sqrtf((lambda2 * BCBC + BCCD) * lambda2 + (lambda2 * BCCD + CDCD)));
    }
  }
  FaceTBC = fminf(FaceTBC, fminf(TB + sqrtf((BCBC + BCCD) + (BCCD + CDCD)), TC + sqrtf(CDCD)));

  /* face AB (lambda3 = 0) */
  float gammax = ACAC - ACBC, gammay = ACBC - BCBC, gammaz = ACCD - BCCD;
  p = (TAB * TAB * ACAC - gammax * gammax) + (BCBC * TAB * TAB - gammay * gammay) -
      ((ACBC + ACBC) * TAB * TAB - 2 * gammax * gammay);
  q = -(BCBC * TAB * TAB - gammay * gammay) * 2 + ((ACBC + ACBC) * TAB * TAB - 2 * gammax * gammay) +
      ((ACCD + ACCD) * TAB * TAB - 2 * gammax * gammaz) - ((BCCD + BCCD) * TAB * TAB - 2 * gammay * gammaz);
  r = (TAB * TAB * BCBC - gammay * gammay) + ((BCCD + BCCD) * TAB * TAB - 2 * gammay * gammaz) +
      (TAB * TAB * CDCD - gammaz * gammaz);
  delta = q * q - 4 * p * r;
  if (ill && fmaxf(TA, TB) < LN && fabsf(delta) <= tau * (q * q + fabsf(4 * p * r))) *ill = 1;
  if (delta >= 0.0) {
    lambda1 = ill ? root_a(p, q, r, delta) : (float)((double)(-q + sqrtf(delta)) / (2.0 * (double)p));
    lambda2 = 1 - lambda1;
    if (lambda1 >= 0 && lambda1 <= 1) {
      TE = TA * lambda1 + TB * lambda2;
      FaceTAB = fminf(FaceTAB, TE + sqrtf((lambda1 * ACAC + lambda2 * ACBC + ACCD) * lambda1 +
                                          (lambda1 * ACBC + lambda2 * BCBC + BCCD) * lambda2 +
                                          (lambda1 * ACCD + lambda2 * BCCD + CDCD)));
    }
    lambda1 = ill ? root_b(p, q, r, delta) : (float)((double)(-q - sqrtf(delta)) / (2.0 * (double)p));
    lambda2 = 1 - lambda1;
    if (lambda1 >= 0 && lambda1 <= 1) {
      TE = TA * lambda1 + TB * lambda2;
      FaceTAB = fminf(FaceTAB, TE + sqrtf((lambda1 * ACAC + lambda2 * ACBC + ACCD) * lambda1 +
                                          (lambda1 * ACBC + lambda2 * BCBC + BCCD) * lambda2 +
                                          (lambda1 * ACCD + lambda2 * BCCD + CDCD)));
    }
  }
  FaceTAB = fminf(FaceTAB, fminf(TB + sqrtf((BCBC + BCCD) + (BCCD + CDCD)), TA + sqrtf((ACAC + ACCD) + (ACCD + CDCD))));

  /* face AC (lambda2 = 0) */
  p = ACAC * TAC * TAC - ACAC * ACAC;
  q = (ACCD + ACCD) * TAC * TAC - 2 * ACAC * ACCD;
  r = TAC * TAC * CDCD - ACCD * ACCD;
  delta = q * q - 4 * p * r;
  if (ill && fmaxf(TA, TC) < LN && fabsf(delta) <= tau * (q * q + fabsf(4 * p * r))) *ill = 1;
  if (delta >= 0.0) {
    lambda1 = ill ? root_a(p, q, r, delta) : (float)((double)(-q + sqrtf(delta)) / (2.0 * (double)p));
    lambda2 = 0.0f;
    lambda3 = 1 - lambda1 - lambda2;
    if (lambda1 >= 0 && lambda1 <= 1) {
      TE = TA * lambda1 + TC * lambda3;
      FaceTAC = fminf(FaceTAC, TE + sqrtf((lambda1 * ACAC + ACCD) * lambda1 + (lambda1 * ACCD + CDCD)));
    }
    lambda1 = ill ? root_b(p, q, r, delta) : (float)((double)(-q - sqrtf(delta)) / (2.0 * (double)p));
    lambda2 = 0.0f;
    lambda3 = 1 - lambda1 - lambda2;
    if (lambda1 >= 0 && lambda1 <= 1) {
      TE = TA * lambda1 + TB * lambda2 + TC * lambda3;
      FaceTAC = fminf(FaceTAC, TE + sqrtf((lambda1 * ACAC + ACCD) * lambda1 + (lambda1 * ACCD + CDCD)));
    }
  }
  FaceTAC = fminf(FaceTAC, fminf(TA + sqrtf((ACAC + ACCD) + (ACCD + CDCD)), TC + sqrtf(CDCD)));

  /* interior of face ABC */
  float s = TAC * ACBC - TBC * ACAC;
  float t = TAC * BCCD - TBC * ACCD;
  float h = -(TAC * BCBC - TBC * ACBC);
  p = (TAC * TAC * ACAC - ACAC * ACAC) * h * h + (BCBC * TAC * TAC - ACBC * ACBC) * s * s +
      ((ACBC + ACBC) * TAC * TAC - 2 * ACAC * ACBC) * s * h;
  q = (BCBC * TAC * TAC - ACBC * ACBC) * 2 * s * t + ((ACBC + ACBC) * TAC * TAC - 2 * ACAC * ACBC) * t * h +
      ((ACCD + ACCD) * TAC * TAC - 2 * ACAC * ACCD) * h * h + ((BCCD + BCCD) * TAC * TAC - 2 * ACBC * ACCD) * s * h;
  r = (TAC * TAC * BCBC - ACBC * ACBC) * t * t + ((BCCD + BCCD) * TAC * TAC - 2 * ACBC * ACCD) * t * h +
      (TAC * TAC * CDCD - ACCD * ACCD) * h * h;
  delta = q * q - 4 * p * r;
  if (ill && fmaxf(fmaxf(TA, TB), TC) < LN && fabsf(delta) <= tau * (q * q + fabsf(4 * p * r))) *ill = 1;
  if (delta >= 0.0) {
    lambda1 = ill ? root_a(p, q, r, delta) : (float)((double)(-q + sqrtf(delta)) / (2.0 * (double)p));
    lambda2 = fdiv ? (s * lambda1 + t) / (h + (float)eps_h)
                   : (float)((double)(s * lambda1 + t) / ((double)h + eps_h));
    lambda3 = 1 - lambda1 - lambda2;
    if (lambda1 >= 0 && lambda1 <= 1 && lambda2 >= 0 && lambda2 <= 1 && lambda3 >= 0 && lambda3 <= 1) {
      TE = TA * lambda1 + TB * lambda2 + TC * lambda3;
      TD = fminf(TD, TE + sqrtf((lambda1 * ACAC + lambda2 * ACBC + ACCD) * lambda1 +
                                (lambda1 * ACBC + lambda2 * BCBC + BCCD) * lambda2 +
                                (lambda1 * ACCD + lambda2 * BCCD + CDCD)));
    }
    lambda1 = ill ? root_b(p, q, r, delta) : (float)((double)(-q - sqrtf(delta)) / (2.0 * (double)p));
    lambda2 = fdiv ? (s * lambda1 + t) / (h + (float)eps_h)
                   : (float)((double)(s * lambda1 + t) / ((double)h + eps_h));
    lambda3 = 1 - lambda1 - lambda2;
    if (lambda1 >= 0 && lambda1 <= 1 && lambda2 >= 0 && lambda2 <= 1 && lambda3 >= 0 && lambda3 <= 1) {
      TE = TA * lambda1 + TB * lambda2 + TC * lambda3;
      TD = fminf(TD, TE + sqrtf((lambda1 * ACAC + lambda2 * ACBC + ACCD) * lambda1 +
                                (lambda1 * ACBC + lambda2 * BCBC + BCCD) * lambda2 +
                                (lambda1 * ACCD + lambda2 * BCCD + CDCD)));
    }
  }
  TD = fminf(TD, fminf(FaceTBC, fminf(FaceTAB, FaceTAC)));
  return TD;
}

float lso_tet_solve_f32(float TA, float TB, float TC, float ACAC, float ACBC,
                        float ACCD, float BCBC, float BCCD, float CDCD,
                        double eps_h, float LN) {
  return tet_f32_impl(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps_h, LN, 0.f, NULL, 0, INFINITY);
}

/* The same solver with every quantity in double (the FP64 oracle). */
double lso_tet_solve_f64(double TA, double TB, double TC, double ACAC,
                         double ACBC, double ACCD, double BCBC, double BCCD,
                         double CDCD, double eps_h, double LN) {
  if (TA >= LN && TB >= LN && TC >= LN) return LN;
  double p, q, r, lambda1, lambda2, lambda3;
  double FaceTAC = LN, FaceTAB = LN, FaceTBC = LN;
  double delta, TE, TD = LN;
  double TAC = TC - TA, TBC = TC - TB, TAB = TB - TA;
  p = BCBC * TBC * TBC - BCBC * BCBC;
  q = (BCCD + BCCD) * TBC * TBC - 2 * BCBC * BCCD;
  r = TBC * TBC * CDCD - BCCD * BCCD;
  delta = q * q - 4 * p * r;
  if (delta >= 0.0) {
    for (int sg = 0; sg < 2; ++sg) {
      lambda2 = (-q + (sg ? -sqrt(delta) : sqrt(delta))) / (2.0 * p);
      lambda3 = 1 - lambda2;
      if (lambda2 >= 0 && lambda2 <= 1) {
        TE = TB * lambda2 + TC * lambda3;
        FaceTBC = fmin(FaceTBC, TE + sqrt((lambda2 * BCBC + BCCD) * lambda2 + (lambda2 * BCCD + CDCD)));
      }
    }
  }
  FaceTBC = fmin(FaceTBC, fmin(TB + sqrt((BCBC + BCCD) + (BCCD + CDCD)), TC + sqrt(CDCD)));
  double gammax = ACAC - ACBC, gammay = ACBC - BCBC, gammaz = ACCD - BCCD;
  p = (TAB * TAB * ACAC - gammax * gammax) + (BCBC * TAB * TAB - gammay * gammay) -
      ((ACBC + ACBC) * TAB * TAB - 2 * gammax * gammay);
  q = -(BCBC * TAB * TAB - gammay * gammay) * 2 + ((ACBC + ACBC) * TAB * TAB - 2 * gammax * gammay) +
      ((ACCD + ACCD) * TAB * TAB - 2 * gammax * gammaz) - ((BCCD + BCCD) * TAB * TAB - 2 * gammay * gammaz);
  r = (TAB * TAB * BCBC - gammay * gammay) + ((BCCD + BCCD) * TAB * TAB - 2 * gammay * gammaz) +
      (TAB * TAB * CDCD - gammaz * gammaz);
  delta = q * q - 4 * p * r;
  if (delta >= 0.0) {
    for (int sg = 0; sg < 2; ++sg) {
      lambda1 = (-q + (sg ? -sqrt(delta) : sqrt(delta))) / (2.0 * p);
      lambda2 = 1 - lambda1;
      if (lambda1 >= 0 && lambda1 <= 1) {
        TE = TA * lambda1 + TB * lambda2;
        FaceTAB = fmin(FaceTAB, TE + sqrt((lambda1 * ACAC + lambda2 * ACBC + ACCD) * lambda1 +
                                          (lambda1 * ACBC + lambda2 * BCBC + BCCD) * lambda2 +
                                          (lambda1 * ACCD + lambda2 * BCCD + CDCD)));
      }
    }
  }
  FaceTAB = fmin(FaceTAB, fmin(TB + sqrt((BCBC + BCCD) + (BCCD + CDCD)), TA + sqrt((ACAC + ACCD) + (ACCD + CDCD))));
  p = ACAC * TAC * TAC - ACAC * ACAC;
  q = (ACCD + ACCD) * TAC * TAC - 2 * ACAC * ACCD;
  r = TAC * TAC * CDCD - ACCD * ACCD;
  delta = q * q - 4 * p * r;
  if (delta >= 0.0) {
    for (int sg = 0; sg < 2; ++sg) {
      lambda1 = (-q + (sg ? -sqrt(delta) : sqrt(delta))) / (2.0 * p);
      lambda3 = 1 - lambda1;
      if (lambda1 >= 0 && lambda1 <= 1) {
        TE = TA * lambda1 + TC * lambda3;
        FaceTAC = fmin(FaceTAC, TE + sqrt((lambda1 * ACAC + ACCD) * lambda1 + (lambda1 * ACCD + CDCD)));
      }
    }
  }
  FaceTAC = fmin(FaceTAC, fmin(TA + sqrt((ACAC + ACCD) + (ACCD + CDCD)), TC + sqrt(CDCD)));
  double s = TAC * ACBC - TBC * ACAC;
  double t = TAC * BCCD - TBC * ACCD;
  double h = -(TAC * BCBC - TBC * ACBC);
  p = (TAC * TAC * ACAC - ACAC * ACAC) * h * h + (BCBC * TAC * TAC - ACBC * ACBC) * s * s +
      ((ACBC + ACBC) * TAC * TAC - 2 * ACAC * ACBC) * s * h;
  q = (BCBC * TAC * TAC - ACBC * ACBC) * 2 * s * t + ((ACBC + ACBC) * TAC * TAC - 2 * ACAC * ACBC) * t * h +
      ((ACCD + ACCD) * TAC * TAC - 2 * ACAC * ACCD) * h * h + ((BCCD + BCCD) * TAC * TAC - 2 * ACBC * ACCD) * s * h;
  r = (TAC * TAC * BCBC - ACBC * ACBC) * t * t + ((BCCD + BCCD) * TAC * TAC - 2 * ACBC * ACCD) * t * h +
      (TAC * TAC * CDCD - ACCD * ACCD) * h * h;
  delta = q * q - 4 * p * r;
  if (delta >= 0.0) {
    for (int sg = 0; sg < 2; ++sg) {
      lambda1 = (-q + (sg ? -sqrt(delta) : sqrt(delta))) / (2.0 * p);
      lambda2 = (s * lambda1 + t) / (h + eps_h);
      lambda3 = 1 - lambda1 - lambda2;
      if (lambda1 >= 0 && lambda1 <= 1 && lambda2 >= 0 && lambda2 <= 1 && lambda3 >= 0 && lambda3 <= 1) {
        TE = TA * lambda1 + TB * lambda2 + TC * lambda3;
        TD = fmin(TD, TE + sqrt((lambda1 * ACAC + lambda2 * ACBC + ACCD) * lambda1 +
                                (lambda1 * ACBC + lambda2 * BCBC + BCCD) * lambda2 +
                                (lambda1 * ACCD + lambda2 * BCCD + CDCD)));
      }
    }
  }
  TD = fmin(TD, fmin(FaceTBC, fmin(FaceTAB, FaceTAC)));
  return TD;
}

static float tet_f32_flagged(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                             float BCBC, float BCCD, float CDCD, double eps_h, float LN, float tau,
                             int* flagged, int fdiv, float cutoff) {
  int ill = 0;
  float r = tet_f32_impl(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps_h, LN, tau, &ill, fdiv, cutoff);
  if (flagged) *flagged = ill;
  if (!ill) return r;
  return (float)lso_tet_solve_f64(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps_h, LN);
}

float lso_tet_solve_f32_flagged(float TA, float TB, float TC, float ACAC, float ACBC,
                                float ACCD, float BCBC, float BCCD, float CDCD,
                                double eps_h, float LN, float tau, int* flagged) {
  int ill = 0;
  float r = tet_f32_impl(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps_h, LN, tau, &ill, 0, INFINITY);
  if (flagged) *flagged = ill;
  if (!ill) return r;
  return (float)lso_tet_solve_f64(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps_h, LN);
}

/* ------------------------------------------------------------------------ */
/* REAL-templated sweep and update (float, then double). */
#define REAL float
#define SFX(n) n##_f32
#define RSQRT(x) sqrtf(x)
#define RABS(x) fabsf(x)
#define RMIN(a, b) fminf(a, b)
#define RMAX(a, b) fmaxf(a, b)
struct ctx_f32 {
  double eps_h, tol, largenum, dt, curv_coeff, fscale, fp64_tau;
  int ref_compat, update_kind;
  const float* vel;
  const float* lc;   /* local coordinates per copy (AoS) */
  float* sig2;       /* 2D projected velocity per copy */
  int* label;
  float *oldT, *newT;
};
static void copy_coords_f32(const lso_layout* lo, const struct ctx_f32* cx, int c, float* L) {
  int nc = lo->dim == 3 ? 6 : 3;
  for (int i = 0; i < nc; ++i) L[i] = cx->lc[(size_t)c * nc + i];
}
/* fdiv: without the reference's semantics the interior division
 * (s l1 + t) / (h + SMALLNUM) is evaluated in float (the GPU does the same);
 * with them, in double as the reference's double SMALLNUM makes it. */
static float tet_f32(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD, float BCBC,
                     float BCCD, float CDCD, double eps_h, float LN, double tau, int fdiv, float cutoff) {
  if (tau > 0)
    return tet_f32_flagged(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps_h, LN, (float)tau, NULL, fdiv,
                           cutoff);
  return tet_f32_impl(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps_h, LN, 0.f, NULL, fdiv, INFINITY);
}
#include "lso_real.inc"
#undef REAL
#undef SFX
#undef RSQRT
#undef RABS
#undef RMIN
#undef RMAX

#define REAL double
#define SFX(n) n##_f64
#define RSQRT(x) sqrt(x)
#define RABS(x) fabs(x)
#define RMIN(a, b) fmin(a, b)
#define RMAX(a, b) fmax(a, b)
struct ctx_f64 {
  double eps_h, tol, largenum, dt, curv_coeff, fscale, fp64_tau;
  int ref_compat, update_kind;
  const float* vel;
  const double* lc;
  double* sig2;
  int* label;
  double *oldT, *newT;
};
static void copy_coords_f64(const lso_layout* lo, const struct ctx_f64* cx, int c, double* L) {
  int nc = lo->dim == 3 ? 6 : 3;
  for (int i = 0; i < nc; ++i) L[i] = cx->lc[(size_t)c * nc + i];
}
static double tet_f64(double TA, double TB, double TC, double ACAC, double ACBC, double ACCD,
                      double BCBC, double BCCD, double CDCD, double eps_h, double LN, double tau, int fdiv,
                      double cutoff) {
  (void)tau;
  (void)fdiv;
  (void)cutoff;
  return lso_tet_solve_f64(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps_h, LN);
}
#include "lso_real.inc"
#undef REAL
#undef SFX
#undef RSQRT
#undef RABS
#undef RMIN
#undef RMAX

float lso_tri_solve_f32(float TA, float TB, float LenAB, float LenBC, float LenAC, float LN) {
  return tri_solve_f32(TA, TB, LenAB, LenBC, LenAC, LN);
}
double lso_tri_solve_f64(double TA, double TB, double LenAB, double LenBC, double LenAC, double LN) {
  return tri_solve_f64(TA, TB, LenAB, LenBC, LenAC, LN);
}

/* ------------------------------------------------------------------------ */
/* Layout build.
 *   element copies: one per distinct patch among an element's vertices, in
 *     vertex order (K2/K3, meshFIM_kernels.h:502-561), stably sorted by
 *     patch (thrust::sort_by_key on int keys, meshFIM3d.cu:469) so copies of
 *     a patch are in ascending element order;
 *   vertices stably sorted by patch (meshFIM3d.cu:504);
 *   slots (k*full + c) stably sorted by new vertex id (meshFIM3d.cu:537-542);
 *   patch adjacency from mesh edges, sorted unique, with the reference's
 *     leading-(-1) construction (meshFIM3d.cu:546-570, 692-710). */
void lso_layout_free(lso_layout* lo) {
  if (!lo) return;
  free(lo->ele_permute); free(lo->ele_offsets); free(lo->vert_permute);
  free(lo->vert_ipermute); free(lo->vert_offsets); free(lo->conn);
  free(lo->vslot_off); free(lo->vslot); free(lo->block_xadj);
  free(lo->block_adjncy); free(lo->xyz_p); free(lo->lc32);
  free(lo);
}

int lso_layout_build(int dim, int nv, const float* xyz, int ne, const int* elems,
                     const int* npart, int nparts, lso_layout** out) {
  *out = NULL;
  if ((dim != 2 && dim != 3) || nv <= 0 || ne <= 0 || nparts <= 0) return LSO_BAD_INPUT;
  const int d1 = dim + 1;
  for (int v = 0; v < nv; ++v)
    if (npart[v] < 0 || npart[v] >= nparts) return LSO_BAD_INPUT;
  for (long long i = 0; i < (long long)ne * d1; ++i)
    if (elems[i] < 0 || elems[i] >= nv) return LSO_BAD_INPUT;
  lso_layout* lo = (lso_layout*)calloc(1, sizeof(lso_layout));
  lo->dim = dim; lo->nv = nv; lo->ne = ne; lo->nparts = nparts;

  /* copies per element */
  int* ecnt = (int*)malloc(sizeof(int) * ne);
  long long full = 0;
  for (int e = 0; e < ne; ++e) {
    const int* ev = elems + (size_t)e * d1;
    int n = 1;
    for (int k = 1; k < d1; ++k) {
      int pk = npart[ev[k]], dup = 0;
      for (int j = 0; j < k; ++j) dup |= (npart[ev[j]] == pk);
      n += !dup;
    }
    ecnt[e] = n;
    full += n;
  }
  if (full > 0x7fffffff / 4) { free(ecnt); lso_layout_free(lo); return LSO_BAD_INPUT; }
  lo->full = (int)full;
  /* counting sort of copies by patch (stable in element order) */
  int* pc = (int*)calloc(nparts + 1, sizeof(int));
  for (int e = 0; e < ne; ++e) {
    const int* ev = elems + (size_t)e * d1;
    for (int k = 0; k < d1; ++k) {
      int pk = npart[ev[k]], dup = 0;
      for (int j = 0; j < k; ++j) dup |= (npart[ev[j]] == pk);
      if (!dup) pc[pk + 1]++;
    }
  }
  lo->ele_offsets = (int*)malloc(sizeof(int) * (nparts + 1));
  lo->ele_offsets[0] = 0;
  int lep = 0;
  for (int p = 0; p < nparts; ++p) {
    lo->ele_offsets[p + 1] = lo->ele_offsets[p] + pc[p + 1];
    if (pc[p + 1] > lep) lep = pc[p + 1];
  }
  lo->lep = lep;
  int* fillp = (int*)malloc(sizeof(int) * nparts);
  memcpy(fillp, lo->ele_offsets, sizeof(int) * nparts);
  lo->ele_permute = (int*)malloc(sizeof(int) * full);
  for (int e = 0; e < ne; ++e) {
    const int* ev = elems + (size_t)e * d1;
    for (int k = 0; k < d1; ++k) {
      int pk = npart[ev[k]], dup = 0;
      for (int j = 0; j < k; ++j) dup |= (npart[ev[j]] == pk);
      if (!dup) lo->ele_permute[fillp[pk]++] = e;
    }
  }
  free(fillp); free(ecnt);
  /* vertices by patch */
  int* vc = (int*)calloc(nparts + 1, sizeof(int));
  for (int v = 0; v < nv; ++v) vc[npart[v] + 1]++;
  lo->vert_offsets = (int*)malloc(sizeof(int) * (nparts + 1));
  lo->vert_offsets[0] = 0;
  int lvp = 0, empty = 0;
  for (int p = 0; p < nparts; ++p) {
    lo->vert_offsets[p + 1] = lo->vert_offsets[p] + vc[p + 1];
    if (vc[p + 1] > lvp) lvp = vc[p + 1];
    if (vc[p + 1] == 0 || pc[p + 1] == 0) empty = 1;
  }
  lo->lvp = lvp;
  free(pc);
  if (empty) { free(vc); lso_layout_free(lo); return LSO_BAD_INPUT; }
  lo->vert_permute = (int*)malloc(sizeof(int) * nv);
  lo->vert_ipermute = (int*)malloc(sizeof(int) * nv);
  {
    int* f = (int*)malloc(sizeof(int) * nparts);
    memcpy(f, lo->vert_offsets, sizeof(int) * nparts);
    for (int v = 0; v < nv; ++v) {
      int nvid = f[npart[v]]++;
      lo->vert_permute[nvid] = v;
      lo->vert_ipermute[v] = nvid;
    }
    free(f);
  }
  free(vc);
  /* connectivity of copies in new ids */
  lo->conn = (int*)malloc(sizeof(int) * full * d1);
  for (long long c = 0; c < full; ++c) {
    int e = lo->ele_permute[c];
    for (int k = 0; k < d1; ++k) lo->conn[c * d1 + k] = lo->vert_ipermute[elems[(size_t)e * d1 + k]];
  }
  /* permuted coordinates */
  lo->xyz_p = (float*)malloc(sizeof(float) * 3 * (size_t)nv);
  for (int v = 0; v < nv; ++v)
    for (int j = 0; j < 3; ++j) lo->xyz_p[(size_t)j * nv + v] = xyz[(size_t)lo->vert_permute[v] * 3 + j];
  /* element count per vertex (LIM) and mean edge length */
  {
    int* adj = (int*)calloc(nv, sizeof(int));
    double esum = 0;
    long long ecount = 0;
    for (int e = 0; e < ne; ++e) {
      const int* ev = elems + (size_t)e * d1;
      for (int k = 0; k < d1; ++k) adj[ev[k]]++;
      for (int a = 0; a < d1; ++a)
        for (int b = a + 1; b < d1; ++b) {
          double dx = (double)xyz[(size_t)ev[a] * 3] - xyz[(size_t)ev[b] * 3];
          double dy = (double)xyz[(size_t)ev[a] * 3 + 1] - xyz[(size_t)ev[b] * 3 + 1];
          double dz = (double)xyz[(size_t)ev[a] * 3 + 2] - xyz[(size_t)ev[b] * 3 + 2];
          esum += sqrt(dx * dx + dy * dy + dz * dz);
          ecount++;
        }
    }
    int lim = 0;
    for (int v = 0; v < nv; ++v) if (adj[v] > lim) lim = adj[v];
    lo->lim = lim;
    lo->mean_edge = esum / (double)ecount;
    free(adj);
  }
  /* owned-vertex slot lists in reference order: slots s = k*full + c sorted
   * by vertex (stable in s), restricted to the vertex's own patch; stored as
   * the local slot (c - es)*(d+1) + k */
  {
    int* vp = (int*)malloc(sizeof(int) * nv);
    for (int p = 0; p < nparts; ++p)
      for (int v = lo->vert_offsets[p]; v < lo->vert_offsets[p + 1]; ++v) vp[v] = p;
    lo->vslot_off = (int*)calloc((size_t)nv + 1, sizeof(int));
    /* the owning patch of copy c */
    int* cp = (int*)malloc(sizeof(int) * full);
    for (int p = 0; p < nparts; ++p)
      for (int c = lo->ele_offsets[p]; c < lo->ele_offsets[p + 1]; ++c) cp[c] = p;
    for (int k = 0; k < d1; ++k)
      for (long long c = 0; c < full; ++c) {
        int v = lo->conn[c * d1 + k];
        if (cp[c] == vp[v]) lo->vslot_off[v + 1]++;
      }
    for (int v = 0; v < nv; ++v) {
      if (lo->vslot_off[v + 1] == 0) { /* isolated vertex */
        free(vp); free(cp); lso_layout_free(lo); return LSO_BAD_INPUT;
      }
      lo->vslot_off[v + 1] += lo->vslot_off[v];
    }
    lo->vslot = (int*)malloc(sizeof(int) * (size_t)lo->vslot_off[nv]);
    int* f = (int*)malloc(sizeof(int) * nv);
    memcpy(f, lo->vslot_off, sizeof(int) * nv);
    for (int k = 0; k < d1; ++k)
      for (long long c = 0; c < full; ++c) {
        int v = lo->conn[c * d1 + k];
        if (cp[c] == vp[v]) lo->vslot[f[v]++] = (int)((c - lo->ele_offsets[cp[c]]) * d1 + k);
      }
    free(f);
    /* patch adjacency: every copy of p holds a vertex of p, so the patches
     * of its other vertices are exactly the patches joined to p by an edge */
    int* mark = (int*)malloc(sizeof(int) * nparts);
    for (int p = 0; p < nparts; ++p) mark[p] = -1;
    int* deg = (int*)calloc(nparts + 1, sizeof(int));
    int has_internal = 0;
    for (int p = 0; p < nparts; ++p)
      for (int c = lo->ele_offsets[p]; c < lo->ele_offsets[p + 1]; ++c) {
        int own = 0;
        for (int k = 0; k < d1; ++k) {
          int q = vp[lo->conn[(size_t)c * d1 + k]];
          if (q == p) own++;
          else if (mark[q] != p) { mark[q] = p; deg[p + 1]++; }
        }
        if (own >= 2) has_internal = 1;
      }
    for (int p = 0; p < nparts; ++p) deg[p + 1] += deg[p];
    int ntot = deg[nparts];
    int* adjl = (int*)malloc(sizeof(int) * (ntot > 0 ? ntot : 1));
    for (int p = 0; p < nparts; ++p) mark[p] = -1;
    for (int p = 0; p < nparts; ++p) {
      int w = deg[p];
      for (int c = lo->ele_offsets[p]; c < lo->ele_offsets[p + 1]; ++c)
        for (int k = 0; k < d1; ++k) {
          int q = vp[lo->conn[(size_t)c * d1 + k]];
          if (q != p && mark[q] != p) { mark[q] = p; adjl[w++] = q; }
        }
      /* insertion sort of the (short) neighbour list */
      for (int i = deg[p] + 1; i < deg[p + 1]; ++i) {
        int x = adjl[i], j = i - 1;
        while (j >= deg[p] && adjl[j] > x) { adjl[j + 1] = adjl[j]; --j; }
        adjl[j + 1] = x;
      }
    }
    /* reference construction: label/mapped pair arrays A, B, with a leading
     * (-1,-1) pair when an internal edge exists; block_xadj from the run
     * ends of A; block_adjncy = B[1:] */
    int S = ntot + (has_internal ? 1 : 0);
    if (S < 2) { free(vp); free(cp); free(mark); free(deg); free(adjl); lso_layout_free(lo); return LSO_BAD_INPUT; }
    int* A = (int*)malloc(sizeof(int) * S);
    int* B = (int*)malloc(sizeof(int) * S);
    int w = 0;
    if (has_internal) { A[w] = -1; B[w] = -1; w++; }
    for (int p = 0; p < nparts; ++p)
      for (int i = deg[p]; i < deg[p + 1]; ++i) { A[w] = p; B[w] = adjl[i]; w++; }
    int maxPart = A[S - 1];
    int nx = maxPart + 2;
    int* xadj = (int*)calloc(nx > nparts + 1 ? nx : nparts + 1, sizeof(int));
    for (int idx = 1; idx < S; ++idx) {
      int value = A[idx];
      int next = (idx + 1 < S) ? A[idx + 1] : INT32_MIN; /* the reference reads one past the end here */
      if (value != next) xadj[value + 1] = idx;
    }
    xadj[nx - 1] = S - 1;
    lo->block_xadj = xadj;
    lo->nadj = S - 1;
    lo->block_adjncy = (int*)malloc(sizeof(int) * (S - 1));
    memcpy(lo->block_adjncy, B + 1, sizeof(int) * (S - 1));
    free(A); free(B); free(adjl); free(deg); free(mark); free(vp); free(cp);
  }
  /* FP32 local coordinates (tet only; 2D local coordinates are formed in
   * the solver's precision, as the reference 2D path is double) */
  if (dim == 3) {
    lo->lc32 = (float*)malloc(sizeof(float) * 6 * full);
    for (long long c = 0; c < full; ++c) {
      float P[4][3];
      for (int k = 0; k < 4; ++k)
        for (int j = 0; j < 3; ++j) P[k][j] = lo->xyz_p[(size_t)j * nv + lo->conn[c * 4 + k]];
      local_coords_tet_f32((const float(*)[3])P, lo->lc32 + c * 6);
    }
  }
  *out = lo;
  return LSO_OK;
}

void lso_layout_info(const lso_layout* lo, long long* info) {
  info[0] = lo->nparts; info[1] = lo->full; info[2] = lo->lep; info[3] = lo->lvp;
  info[4] = lo->lim; info[5] = lo->nadj; info[6] = lo->nv; info[7] = lo->ne;
}

int lso_layout_copy(const lso_layout* lo, int which, void* dst) {
  const int d1 = lo->dim + 1;
  const long long full = lo->full;
  int* di = (int*)dst;
  switch (which) {
    case LSO_L_ELE_PERMUTE: memcpy(dst, lo->ele_permute, sizeof(int) * full); return 0;
    case LSO_L_ELE_OFFSETS: memcpy(dst, lo->ele_offsets, sizeof(int) * (lo->nparts + 1)); return 0;
    case LSO_L_VERT_PERMUTE: memcpy(dst, lo->vert_permute, sizeof(int) * lo->nv); return 0;
    case LSO_L_VERT_IPERMUTE: memcpy(dst, lo->vert_ipermute, sizeof(int) * lo->nv); return 0;
    case LSO_L_VERT_OFFSETS: memcpy(dst, lo->vert_offsets, sizeof(int) * (lo->nparts + 1)); return 0;
    case LSO_L_ELE_AFTER_PERMUTE:
      for (long long c = 0; c < full; ++c)
        for (int k = 0; k < d1; ++k) di[k * full + c] = lo->conn[c * d1 + k];
      return 0;
    case LSO_L_MEM_LOCATIONS:
    case LSO_L_MEM_LOCATION_OFFSETS: {
      /* slots k*full+c stably sorted by vertex id */
      int* off = (int*)calloc((size_t)lo->nv + 1, sizeof(int));
      for (int k = 0; k < d1; ++k)
        for (long long c = 0; c < full; ++c) off[lo->conn[c * d1 + k] + 1]++;
      for (int v = 0; v < lo->nv; ++v) off[v + 1] += off[v];
      if (which == LSO_L_MEM_LOCATION_OFFSETS) {
        memcpy(dst, off, sizeof(int) * ((size_t)lo->nv + 1));
      } else {
        for (int k = 0; k < d1; ++k)
          for (long long c = 0; c < full; ++c) di[off[lo->conn[c * d1 + k]]++] = (int)(k * full + c);
      }
      free(off);
      return 0;
    }
    case LSO_L_BLOCK_XADJ: memcpy(dst, lo->block_xadj, sizeof(int) * (lo->nparts + 1)); return 0;
    case LSO_L_BLOCK_ADJNCY: memcpy(dst, lo->block_adjncy, sizeof(int) * lo->nadj); return 0;
    case LSO_L_LOCAL_COORDS: {
      float* df = (float*)dst;
      if (lo->dim == 3) {
        for (long long c = 0; c < full; ++c)
          for (int i = 0; i < 6; ++i) df[i * full + c] = lo->lc32[c * 6 + i];
      } else {
        for (long long c = 0; c < full; ++c) {
          double P[3][3], L[3], sg[2], z[3] = {0, 0, 0};
          for (int k = 0; k < 3; ++k)
            for (int j = 0; j < 3; ++j) P[k][j] = lo->xyz_p[(size_t)j * lo->nv + lo->conn[c * 3 + k]];
          local_coords_tri_f64((const double(*)[3])P, z, L, sg);
          for (int i = 0; i < 3; ++i) df[i * full + c] = (float)L[i];
        }
      }
      return 0;
    }
  }
  return LSO_BAD_INPUT;
}

/* ------------------------------------------------------------------------ */
/* Driver.  Step order: src/core3d/cuda/meshFIM3d.cu:639-678. */
#define REAL float
#define SFX(n) n##_f32
#define RABS(x) fabsf(x)
#define RMIN(a, b) fminf(a, b)
#include "lso_driver.inc"
#undef REAL
#undef SFX
#undef RABS
#undef RMIN
#define REAL double
#define SFX(n) n##_f64
#define RABS(x) fabs(x)
#define RMIN(a, b) fmin(a, b)
#include "lso_driver.inc"
#undef REAL
#undef SFX
#undef RABS
#undef RMIN

static void fill_defaults(const lso_layout* lo, const lso_params* in, lso_params* p) {
  *p = *in;
  if (p->niter <= 0) p->niter = lo->dim == 3 ? 5 : 10;
  if (p->inside_niter <= 0) p->inside_niter = 1;
  if (p->max_fim_iters <= 0) p->max_fim_iters = 100000;
  if (p->smallnum <= 0) p->smallnum = 1e-5;
  if (p->largenum <= 0) p->largenum = 1e9;
  if (p->length_scale <= 0) p->length_scale = lo->mean_edge;
}

int lso_solve(const lso_layout* lo, const lso_params* prm_in, const float* phi0,
              const float* vel, int nsteps, float* hist, unsigned char* nb_sets,
              int* iters, lso_stats* st) {
  if (!lo || !prm_in || !phi0 || nsteps < 0) return LSO_BAD_INPUT;
  if (prm_in->dim != lo->dim) return LSO_BAD_INPUT;
  lso_params p;
  fill_defaults(lo, prm_in, &p);
#ifdef _OPENMP
  if (p.nthreads > 0) omp_set_num_threads(p.nthreads);
#endif
  lso_stats tmp;
  if (!st) st = &tmp;
  memset(st, 0, sizeof(*st));
  double t0 = now_sec();
  int rc = (p.precision == 64) ? solve_f64(lo, &p, phi0, vel, nsteps, hist, nb_sets, iters, st)
                               : solve_f32(lo, &p, phi0, vel, nsteps, hist, nb_sets, iters, st);
  st->seconds = now_sec() - t0;
  st->status = rc;
  return rc;
}

int lso_update_only(const lso_layout* lo, const lso_params* prm_in, const float* phi,
                    const float* vel, const int* nb_list, int nnb, float* phi_out) {
  if (!lo || !prm_in || !phi || !phi_out) return LSO_BAD_INPUT;
  lso_params p;
  fill_defaults(lo, prm_in, &p);
  for (int i = 0; i < nnb; ++i)
    if (nb_list[i] < 0 || nb_list[i] >= lo->nparts) return LSO_BAD_INPUT;
  return (p.precision == 64) ? update_only_f64(lo, &p, phi, vel, nb_list, nnb, phi_out)
                             : update_only_f32(lo, &p, phi, vel, nb_list, nnb, phi_out);
}
