/*
 * coord_oracle.c -- FP64 CPU restatement of PLUMED's COORDINATION hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  See coord_oracle.h.  Compile with
 * -ffp-contract=off: the reference is compiled the same way, and an FMA
 * contraction anywhere below would change the low bits of the results.
 *
 * Each routine follows the reference routine cited beside it operation for
 * operation (same association order of every + and *).
 */
#include "coord_oracle.h"
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* small 3-vector / 3x3 helpers, in the reference's evaluation order        */
/* ------------------------------------------------------------------------ */

/* LoopUnroller<3>::_sum2 (LoopUnroller.h:146-152): (d0*d0 + d1*d1) + d2*d2 */
static inline double mod2(const double d[3]) { return d[0] * d[0] + d[1] * d[1] + d[2] * d[2]; }
/* LoopUnroller<3>::_dot */
static inline double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* TensorTyped::determinant (Tensor.h:384-392) */
static double det33(const double *d) {
  return d[0] * d[4] * d[8] + d[1] * d[5] * d[6] + d[2] * d[3] * d[7] - d[0] * d[5] * d[7] -
         d[1] * d[3] * d[8] - d[2] * d[4] * d[6];
}

/* TensorTyped::inverse (Tensor.h:416-422): t(j,i) = invdet * cofactor */
static void inv33(const double *a, double *t) {
  double invdet = 1.0 / det33(a);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      t[j * 3 + i] = invdet * (a[((i + 1) % 3) * 3 + (j + 1) % 3] * a[((i + 2) % 3) * 3 + (j + 2) % 3] -
                               a[((i + 1) % 3) * 3 + (j + 2) % 3] * a[((i + 2) % 3) * 3 + (j + 1) % 3]);
}

/* matmul(Vector a, Tensor b) (Tensor.h:451-458): t(i) = sum_j a(j)*b(j,i), from 0 */
static void vecmat(const double a[3], const double *b, double t[3]) {
  for (int i = 0; i < 3; i++) {
    double s = 0.0;
    for (int j = 0; j < 3; j++) s += a[j] * b[j * 3 + i];
    t[i] = s;
  }
}
/* matmul(Tensor a, Vector b) (Tensor.h:440-447): t(i) = sum_j a(i,j)*b(j), from 0 */
static void matvec(const double *a, const double b[3], double t[3]) {
  for (int i = 0; i < 3; i++) {
    double s = 0.0;
    for (int j = 0; j < 3; j++) s += a[i * 3 + j] * b[j];
    t[i] = s;
  }
}
/* matmul(Tensor, Tensor) (Tensor.h:428-436) */
static void matmat(const double *a, const double *b, double *t) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s += a[i * 3 + k] * b[k * 3 + j];
      t[i * 3 + j] = s;
    }
}
static void transpose33(const double *a, double *t) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) t[i * 3 + j] = a[j * 3 + i];
}

/* ------------------------------------------------------------------------ */
/* Tools::pbc (Tools.h:547-571), round_toward_zero branch                    */
/* ------------------------------------------------------------------------ */
double orc_tools_pbc(double x) {
  x += 100.0;
  if (x >= 0) return x - (double)(int)(x + 0.5);
  return x - (double)(int)(x - 0.5);
}

/* ------------------------------------------------------------------------ */
/* LatticeReduction (src/tools/LatticeReduction.cpp), reduceFast path       */
/* ------------------------------------------------------------------------ */
static const double lr_one_plus_eps = 1.0 + 1e-14;

static void lr_swap(double a[3], double b[3]) {
  for (int k = 0; k < 3; k++) {
    double t = a[k];
    a[k] = b[k];
    b[k] = t;
  }
}
/* LatticeReduction::sort (LatticeReduction.cpp:31-55) */
static void lr_sort(double v[3][3]) {
  double m[3];
  for (int i = 0; i < 3; i++) m[i] = mod2(v[i]);
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++)
      if (m[i] > m[j]) {
        lr_swap(v[i], v[j]);
        double t = m[i];
        m[i] = m[j];
        m[j] = t;
      }
}
/* LatticeReduction::reduce(a,b) (LatticeReduction.cpp:57-81) */
static void lr_reduce2(double a[3], double b[3]) {
  double ma = mod2(a), mb = mod2(b);
  for (int it = 0; it < 1000000; it++) {
    if (mb > ma) {
      lr_swap(a, b);
      double t = ma;
      ma = mb;
      mb = t;
    }
    double f = floor(dot3(a, b) / mb + 0.5);
    for (int k = 0; k < 3; k++) a[k] -= b[k] * f;
    ma = mod2(a);
    if (mb <= ma * lr_one_plus_eps) break;
  }
  lr_swap(a, b);
}
/* LatticeReduction::reduceFast (LatticeReduction.cpp:139-183) */
static void lr_reduce_fast(double *t) {
  double v[3][3];
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) v[i][k] = t[i * 3 + k];
  for (int it = 0; it < 1000000; it++) {
    lr_sort(v);
    lr_reduce2(v[0], v[1]);
    double b11 = mod2(v[0]), b22 = mod2(v[1]);
    double b12 = dot3(v[0], v[1]), b13 = dot3(v[0], v[2]), b23 = dot3(v[1], v[2]);
    double z = b11 * b22 - b12 * b12;
    double y2 = -(b11 * b23 - b12 * b13) / z;
    double y1 = -(b22 * b13 - b12 * b23) / z;
    int x1min = (int)floor(y1), x1max = x1min + 1;
    int x2min = (int)floor(y2), x2max = x2min + 1;
    int first = 1;
    double mbest = 0.0, best[3] = {0, 0, 0};
    for (int x1 = x1min; x1 <= x1max; x1++)
      for (int x2 = x2min; x2 <= x2max; x2++) {
        double trial[3];
        /* v[2]+x2*v[1]+x1*v[0] evaluated left to right */
        for (int k = 0; k < 3; k++) trial[k] = (v[2][k] + (double)x2 * v[1][k]) + (double)x1 * v[0][k];
        double mtrial = mod2(trial);
        if (first || mtrial < mbest) {
          mbest = mtrial;
          memcpy(best, trial, sizeof best);
          first = 0;
        }
      }
    if (mod2(best) * lr_one_plus_eps >= mod2(v[2])) break;
    memcpy(v[2], best, sizeof best);
  }
  lr_sort(v);
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) t[i * 3 + k] = v[i][k];
}

/* Pbc::buildShifts (Pbc.cpp:59-135) */
static void pbc_build_shifts(orc_pbc *p) {
  const double small = 1e-28;
  double redT[9], rrT[9];
  transpose33(p->reduced, redT);
  matmat(p->reduced, redT, rrT);
  for (int o = 0; o < 8; o++) p->nshift[o] = 0;
  for (int l = -1; l <= 1; l++)
    for (int m = -1; m <= 1; m++)
      for (int n = -1; n <= 1; n++) {
        const int ishift[3] = {l, m, n};
        double dshift[3] = {(double)l, (double)m, (double)n};
        unsigned count = 0;
        for (int s = 0; s < 3; s++)
          if (ishift[s] != 0) count++;
        if (count == 0 || count == 3) continue;
        double cosdir[3];
        matvec(rrT, dshift, cosdir);
        double dp = dot3(dshift, cosdir);
        double ref = mod2(dshift) * mod2(cosdir);
        if (fabs(ref - dp * dp) < small) continue;
        for (int i = 0; i < 2; i++)
          for (int j = 0; j < 2; j++)
            for (int k = 0; k < 2; k++) {
              const int block[3] = {2 * i - 1, 2 * j - 1, 2 * k - 1};
              int skip = 0;
              for (int s = 0; s < 3; s++)
                if (ishift[s] * block[s] > 0) skip = 1;
              if (skip) continue;
              skip = 1;
              for (int s = 0; s < 3; s++)
                if (((1 - ishift[s] * ishift[s]) * block[s]) * cosdir[s] < -small) skip = 0;
              if (skip) continue;
              int o = 4 * i + 2 * j + k;
              double sh[3];
              matvec(redT, dshift, sh);
              if (p->nshift[o] < 32) {
                memcpy(p->shift[o][p->nshift[o]], sh, sizeof sh);
                p->nshift[o]++;
              }
            }
      }
}

/* Pbc::setBox (Pbc.cpp:165-212) */
int orc_pbc_set(orc_pbc *p, const double box[9]) {
  const double eps = 1e-28;
  memset(p, 0, sizeof *p);
  memcpy(p->box, box, 9 * sizeof(double));
  p->type = ORC_PBC_UNSET;
  double det = det33(p->box);
  if (det * det < eps) return p->type;
  const double *b = p->box;
  int cxy = (b[1] * b[1] < eps && b[3] * b[3] < eps);
  int cxz = (b[2] * b[2] < eps && b[6] * b[6] < eps);
  int cyz = (b[5] * b[5] < eps && b[7] * b[7] < eps);
  inv33(p->box, p->invbox);
  memcpy(p->reduced, p->box, sizeof p->reduced);
  if (cxy && cxz && cyz) {
    p->type = ORC_PBC_ORTHO;
    inv33(p->reduced, p->invreduced);
  } else {
    p->type = ORC_PBC_GENERIC;
    lr_reduce_fast(p->reduced);
    inv33(p->reduced, p->invreduced);
    pbc_build_shifts(p);
  }
  return p->type;
}

/* Pbc::distance(v1,v2) (Pbc.cpp:383-415) */
void orc_pbc_distance(const orc_pbc *p, const double v1[3], const double v2[3], double d[3]) {
  for (int k = 0; k < 3; k++) d[k] = v2[k] - v1[k];
  if (p->type == ORC_PBC_ORTHO) {
    for (int k = 0; k < 3; k++) d[k] = orc_tools_pbc(d[k] * p->invbox[k * 4]) * p->box[k * 4];
  } else if (p->type == ORC_PBC_GENERIC) {
    double s[3];
    vecmat(d, p->invreduced, s);
    for (int k = 0; k < 3; k++) s[k] = orc_tools_pbc(s[k]);
    vecmat(s, p->reduced, d);
    if (fabs(s[0]) + fabs(s[1]) + fabs(s[2]) > 0.5) {
      int o = 4 * (s[0] > 0 ? 1 : 0) + 2 * (s[1] > 0 ? 1 : 0) + (s[2] > 0 ? 1 : 0);
      double best[3] = {d[0], d[1], d[2]};
      double lbest = mod2(best);
      for (int i = 0; i < p->nshift[o]; i++) {
        double trial[3];
        for (int k = 0; k < 3; k++) trial[k] = d[k] + p->shift[o][i][k];
        double ltrial = mod2(trial);
        if (ltrial < lbest) {
          lbest = ltrial;
          memcpy(best, trial, sizeof best);
        }
      }
      memcpy(d, best, sizeof best);
    }
  }
}

/* ------------------------------------------------------------------------ */
/* switching functions (SwitchingFunction.cpp)                              */
/* ------------------------------------------------------------------------ */

/* Tools::fastpow(base,exp) (Tools.h:582-597); fastpow<exp> performs the same
 * multiplications in the same order. */
static double fastpow_i(double base, int exp) {
  if (exp < 0) {
    exp = -exp;
    base = 1.0 / base;
  }
  double result = 1.0;
  while (exp) {
    if (exp & 1) result *= base;
    exp >>= 1;
    base *= base;
  }
  return result;
}

/* Data::init (SwitchingFunction.cpp:84-94) */
static void data_init(orc_switch *s, double D0, double DMAX, double R0) {
  memset(s, 0, sizeof *s);
  s->d0 = D0;
  s->dmax = DMAX;
  s->dmax_2 = (s->dmax < sqrt(DBL_MAX)) ? s->dmax * s->dmax : DBL_MAX;
  s->invr0 = 1.0 / R0;
  s->invr0_2 = s->invr0 * s->invr0;
  s->stretch = 1.0;
  s->shift = 0.0;
  s->nn = 6;
  s->mm = 12;
  s->nnf = 3;
  s->mmf = 6;
  s->beta = 50.0;
  s->lambda = 1.8;
}

typedef struct {
  double f, d;
} vd_t;

/* fixedRational<N>::doRational<POW> (SwitchingFunction.cpp:191-196) */
static inline vd_t do_rational_fixed(int POW, double rdist) {
  vd_t r;
  const double rNdist = fastpow_i(rdist, POW - 1);
  r.f = 1.0 / (1.0 + rNdist * rdist);
  r.d = -POW * rNdist * r.f * r.f;
  return r;
}

/* rational<isFast,nis2m>::doRational (SwitchingFunction.cpp:253-280) */
static inline vd_t do_rational_rt(int simplified, double rdist, double secDev, int N, int M, double dfunc,
                                  double result) {
  static const double moreThanOne = 1.0 + 5.0e10 * DBL_EPSILON;
  static const double lessThanOne = 1.0 - 5.0e10 * DBL_EPSILON;
  vd_t r;
  if (simplified) {
    const double rNdist = fastpow_i(rdist, N - 1);
    result = 1.0 / (1.0 + rNdist * rdist);
    dfunc = -N * rNdist * result * result;
  } else {
    if (!((rdist > lessThanOne) && (rdist < moreThanOne))) {
      const double rNdist = fastpow_i(rdist, N - 1);
      const double rMdist = fastpow_i(rdist, M - 1);
      const double num = 1.0 - rNdist * rdist;
      const double iden = 1.0 / (1.0 - rMdist * rdist);
      result = num * iden;
      dfunc = ((M * result * rMdist) - (N * rNdist)) * iden;
    } else {
      const double x = (rdist - 1.0);
      result = result + x * (dfunc + 0.5 * x * secDev);
      dfunc = dfunc + x * secDev;
    }
  }
  r.f = result;
  r.d = dfunc;
  return r;
}

/* switching::function(rdist) for the baseSwitch types */
static vd_t sw_function(const orc_switch *s, double rdist) {
  vd_t r = {0.0, 0.0};
  switch (s->type) {
  case ORC_SW_RATFIX:
    return do_rational_fixed(s->nn, rdist);
  case ORC_SW_RATIONAL:
  case ORC_SW_RATIONAL_FAST:
    return do_rational_rt(0, rdist, s->preSecDev, s->nn, s->mm, s->preDfunc, s->preRes);
  case ORC_SW_RATIONAL_SIMPLE:
  case ORC_SW_RATIONAL_SIMPLE_FAST:
    return do_rational_rt(1, rdist, s->preSecDev, s->nn, s->mm, s->preDfunc, s->preRes);
  case ORC_SW_EXP: { /* exponentialSwitch::function (:338-341) */
    double result = exp(-rdist);
    r.f = result;
    r.d = -result;
    return r;
  }
  case ORC_SW_GAUSSIAN:
  case ORC_SW_FASTGAUSSIAN: { /* gaussianSwitch::function (:352-355) */
    double result = exp(-0.5 * rdist * rdist);
    r.f = result;
    r.d = -rdist * result;
    return r;
  }
  case ORC_SW_SMAP: { /* smapSwitch::function (:452-457) */
    const double sx = s->c * fastpow_i(rdist, s->a);
    double result = pow(1.0 + sx, s->d);
    double dfunc = -s->b * sx / rdist * result / (1.0 + sx);
    r.f = result;
    r.d = dfunc;
    return r;
  }
  case ORC_SW_CUBIC: { /* cubicSwitch::function (:466-472) */
    const double tmp1 = rdist - 1.0;
    const double tmp2 = 1.0 + 2.0 * rdist;
    double dfunc = 2 * tmp1 * tmp2 + 2 * tmp1 * tmp1;
    r.f = tmp1 * tmp1 * tmp2;
    r.d = dfunc;
    return r;
  }
  case ORC_SW_TANH: { /* tanhSwitch::function (:482-488) */
    const double tmp1 = tanh(rdist);
    double dfunc = tmp1 * tmp1 - 1.0;
    r.f = 1.0 - tmp1;
    r.d = dfunc;
    return r;
  }
  case ORC_SW_COSINUS: { /* cosinusSwitch::function (:499-509) */
    double result = 0.0, dfunc = 0.0;
    if (rdist <= 1.0) {
      const double pi = 3.141592653589793238462643383279502884197169399375105820974944592307;
      double rdistPI = rdist * pi;
      result = 0.5 * (cos(rdistPI) + 1.0);
      dfunc = -0.5 * pi * sin(rdistPI);
    }
    r.f = result;
    r.d = dfunc;
    return r;
  }
  default:
    return r;
  }
}

/* nativeqSwitch::calculate (SwitchingFunction.cpp:527-555) */
static vd_t nativeq_calculate(const orc_switch *s, double distance) {
  vd_t r;
  double res = 0.0, dfunc = 0.0;
  if (distance <= s->dmax) {
    res = 1.0;
    if (distance > s->d0) {
      const double rdist = s->beta * (distance - s->lambda * s->ref);
      double exprdist = exp(rdist);
      res = 1.0 / (1.0 + exprdist);
      dfunc = -s->beta / (exprdist + 2.0 + 1.0 / exprdist) / distance;
      dfunc *= s->stretch;
    }
    res = res * s->stretch + s->shift;
  }
  r.f = res;
  r.d = dfunc;
  return r;
}

/* leptonSwitch::calculateSqr (SwitchingFunction.cpp:730-749), FUNC of x2 */
static vd_t custom_calculate_x2(const orc_switch *s, double distance2) {
  vd_t r = {0.0, 0.0};
  if (distance2 <= s->dmax_2) {
    const double rdist_2 = distance2 * s->invr0_2;
    orc_expr_eval(&s->expr, rdist_2, &r.f, &r.d);
    r.d *= 2 * s->invr0_2;
    r.f = r.f * s->stretch + s->shift;
    r.d *= s->stretch;
  }
  return r;
}

/* leptonSwitch::calculate (SwitchingFunction.cpp:708-728) */
static vd_t custom_calculate(const orc_switch *s, double distance) {
  if (s->expr.var_x2) return custom_calculate_x2(s, distance * distance);
  vd_t r = {0.0, 0.0};
  if (distance <= s->dmax) {
    r.f = 1.0;
    const double rdist = (distance - s->d0) * s->invr0;
    if (rdist > 0.0) {
      orc_expr_eval(&s->expr, rdist, &r.f, &r.d);
      r.d *= s->invr0;
      r.d /= distance;
    }
    r.f = r.f * s->stretch + s->shift;
    r.d *= s->stretch;
  }
  return r;
}

/* baseSwitch::calculate (SwitchingFunction.cpp:130-147) with applystretch (:121-127) */
static vd_t sw_calculate(const orc_switch *s, double distance) {
  if (s->type == ORC_SW_Q) return nativeq_calculate(s, distance);
  if (s->type == ORC_SW_CUSTOM) return custom_calculate(s, distance);
  vd_t r = {0.0, 0.0};
  const double rdist = (distance - s->d0) * s->invr0;
  if (distance > s->dmax) return r;
  if (rdist > 0.0) {
    r = sw_function(s, rdist);
    r.f = r.f * s->stretch + s->shift;
    r.d *= s->stretch;
    r.d *= s->invr0;
    r.d /= distance;
    return r;
  }
  r.f = s->stretch + s->shift;
  r.d = 0.0;
  return r;
}

/* calculateSqr dispatch: fixedRational (:203-215), rational fast (:288-303),
 * fastgaussian (:410-431), else baseSwitch::calculateSqr (:177-179) */
static vd_t sw_calculate_sqr(const orc_switch *s, double distance2) {
  vd_t r = {0.0, 0.0};
  switch (s->type) {
  case ORC_SW_CUSTOM:
    if (s->expr.var_x2) return custom_calculate_x2(s, distance2);
    return custom_calculate(s, sqrt(distance2));
  case ORC_SW_RATFIX:
    if (distance2 <= s->dmax_2) {
      const double rdist = distance2 * s->invr0_2;
      r = do_rational_fixed(s->nn / 2, rdist);
      r.d *= 2 * s->invr0_2;
      r.f = r.f * s->stretch + s->shift;
      r.d *= s->stretch;
    }
    return r;
  case ORC_SW_RATIONAL_FAST:
  case ORC_SW_RATIONAL_SIMPLE_FAST:
    if (distance2 <= s->dmax_2) {
      const double rdist = distance2 * s->invr0_2;
      r = do_rational_rt(s->type == ORC_SW_RATIONAL_SIMPLE_FAST, rdist, s->preSecDevF, s->nnf, s->mmf, s->preDfuncF,
                         s->preRes);
      r.d *= 2 * s->invr0_2;
      r.f = r.f * s->stretch + s->shift;
      r.d *= s->stretch;
    }
    return r;
  case ORC_SW_FASTGAUSSIAN:
    if (distance2 < s->dmax_2) {
      r.f = 1.0;
      if (distance2 > 0.0) {
        r.f = exp(-0.5 * distance2);
        r.d = -r.f;
        r.f = r.f * s->stretch + s->shift;
        r.d *= s->stretch;
      }
    }
    return r;
  default:
    return sw_calculate(s, sqrt(distance2));
  }
}

double orc_switch_calculate(const orc_switch *s, double distance, double *dfunc) {
  vd_t r = sw_calculate(s, distance);
  *dfunc = r.d;
  return r.f;
}
double orc_switch_calculate_sqr(const orc_switch *s, double distance2, double *dfunc) {
  vd_t r = sw_calculate_sqr(s, distance2);
  *dfunc = r.d;
  return r.f;
}

/* SwitchInterface::setupStretch (SwitchingFunction.cpp:63-72) */
static void sw_setup_stretch(orc_switch *s) {
  if (s->dmax < DBL_MAX) {
    s->stretch = 1.0;
    s->shift = 0.0;
    double s0 = sw_calculate(s, 0.0).f;
    double sd = sw_calculate(s, s->dmax).f;
    s->stretch = 1.0 / (s0 - sd);
    s->shift = -sd * s->stretch;
  }
}

/* rational<>::init (SwitchingFunction.cpp:228-252) */
static void rational_init(orc_switch *s, double D0, double DMAX, double R0, int N, int M) {
  data_init(s, D0, DMAX, R0);
  s->nn = N;
  s->mm = (M == 0) ? N * 2 : M;
  s->preRes = (double)s->nn / s->mm;
  s->preDfunc = 0.5 * s->nn * (s->nn - s->mm) / (double)s->mm;
  s->preSecDev = (s->nn * (s->mm * s->mm - 3.0 * s->mm * (-1 + s->nn) + s->nn * (-3 + 2 * s->nn))) / (6.0 * s->mm);
  s->nnf = s->nn / 2;
  s->mmf = s->mm / 2;
  s->preDfuncF = 0.5 * s->nnf * (s->nnf - s->mmf) / (double)s->mmf;
  s->preSecDevF =
      (s->nnf * (s->mmf * s->mmf - 3.0 * s->mmf * (-1 + s->nnf) + s->nnf * (-3 + 2 * s->nnf))) / (6.0 * s->mmf);
}

/* rationalFactory (SwitchingFunction.cpp:306-348) */
static void rational_factory(orc_switch *s, double D0, double DMAX, double R0, int N, int M) {
  int fast = (N % 2 == 0) && (M % 2 == 0) && D0 == 0.0;
  if (((2 * N) == M || M == 0) && fast && N <= 12 &&
      (N == 12 || N == 10 || N == 8 || N == 6 || N == 4 || N == 2)) {
    data_init(s, D0, DMAX, R0);
    s->type = ORC_SW_RATFIX;
    s->nn = N;
    s->mm = 2 * N;
    return;
  }
  rational_init(s, D0, DMAX, R0, N, M);
  if (2 * N == M || M == 0)
    s->type = fast ? ORC_SW_RATIONAL_SIMPLE_FAST : ORC_SW_RATIONAL_SIMPLE;
  else
    s->type = fast ? ORC_SW_RATIONAL_FAST : ORC_SW_RATIONAL;
}

int orc_switch_set_rational(orc_switch *s, int nn, int mm, double r0, double d0) {
  if (mm == 0) mm = 2 * nn;
  double dmax = d0 + r0 * pow(0.00001, 1. / (nn - mm));
  rational_factory(s, d0, dmax, r0, nn, mm);
  sw_setup_stretch(s);
  return 0;
}

/* --- tiny word parser for SwitchingFunction::set(string) ---------------- */
#define ORC_MAXW 64
typedef struct {
  int n;
  int overflow; /* a word longer than the buffer, or more than ORC_MAXW words */
  char w[ORC_MAXW][128];
} words_t;

static void split_words(const char *def, words_t *W) {
  W->n = 0;
  W->overflow = 0;
  const char *p = def;
  while (*p) {
    while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '{' || *p == '}') p++;
    if (!*p) break;
    int len = 0;
    while (p[len] && p[len] != ' ' && p[len] != '\t' && p[len] != '\n' && p[len] != '}' && p[len] != '{') len++;
    if (W->n < ORC_MAXW && len < 127) {
      memcpy(W->w[W->n], p, len);
      W->w[W->n][len] = 0;
      W->n++;
    } else {
      W->overflow = 1;
    }
    p += len;
  }
}
static void erase_word(words_t *W, int i) {
  for (int k = i; k + 1 < W->n; k++) memcpy(W->w[k], W->w[k + 1], sizeof W->w[k]);
  W->n--;
}
/* Tools::findKeyword / Tools::parse: "KEY=value" words, removed once read.
 * Returns 1 found+parsed, 0 absent, -1 found but unparsable. */
static int parse_double(words_t *W, const char *key, double *v) {
  size_t kl = strlen(key);
  for (int i = 0; i < W->n; i++)
    if (strncmp(W->w[i], key, kl) == 0 && W->w[i][kl] == '=') {
      char *end = NULL;
      const char *val = W->w[i] + kl + 1;
      double x = strtod(val, &end);
      if (end == val || *end) return -1;
      *v = x;
      erase_word(W, i);
      return 1;
    }
  return 0;
}
static int parse_int(words_t *W, const char *key, int *v) {
  size_t kl = strlen(key);
  for (int i = 0; i < W->n; i++)
    if (strncmp(W->w[i], key, kl) == 0 && W->w[i][kl] == '=') {
      char *end = NULL;
      const char *val = W->w[i] + kl + 1;
      long x = strtol(val, &end, 10);
      if (end == val || *end) return -1;
      *v = (int)x;
      erase_word(W, i);
      return 1;
    }
  return 0;
}
/* the text after "KEY=" (removed once read); 1 found, 0 absent, -1 longer
 * than out */
static int parse_string(words_t *W, const char *key, char *out, size_t outlen) {
  size_t kl = strlen(key);
  for (int i = 0; i < W->n; i++)
    if (strncmp(W->w[i], key, kl) == 0 && W->w[i][kl] == '=') {
      const int n = snprintf(out, outlen, "%s", W->w[i] + kl + 1);
      erase_word(W, i);
      return (n < 0 || (size_t)n >= outlen) ? -1 : 1;
    }
  return 0;
}
static int parse_flag(words_t *W, const char *key) {
  for (int i = 0; i < W->n; i++)
    if (strcmp(W->w[i], key) == 0) {
      erase_word(W, i);
      return 1;
    }
  return 0;
}

/* SwitchingFunction::set(string) (SwitchingFunction.cpp:1055-1159) */
int orc_switch_set(orc_switch *s, const char *definition, char *err, int errlen) {
  words_t W;
  split_words(definition, &W);
  memset(s, 0, sizeof *s);
  if (W.overflow) {
    /* a word cut short could still parse as a different valid input */
    snprintf(err, errlen, "switching function input has a word longer than 126 characters or more than %d words "
             "(the oracle's limits)", ORC_MAXW);
    return 1;
  }
  if (W.n < 1) {
    snprintf(err, errlen, "missing all input for switching function");
    return 1;
  }
  char name[128];
  strcpy(name, W.w[0]);
  erase_word(&W, 0);
  double d0 = 0.0, dmax = DBL_MAX;
  err[0] = 0;
  if (parse_double(&W, "D_0", &d0) < 0) snprintf(err, errlen, "could not parse D_0");
  if (parse_double(&W, "D_MAX", &dmax) < 0) snprintf(err, errlen, "could not parse D_MAX");
  parse_flag(&W, "STRETCH");
  int dostretch = 1;
  if (parse_flag(&W, "NOSTRETCH")) dostretch = 0;
  if (strcmp(name, "CUBIC") == 0) {
    data_init(s, d0, dmax, dmax - d0);
    s->type = ORC_SW_CUBIC;
  } else {
    double r0 = 0.0;
    if (parse_double(&W, "R_0", &r0) != 1) snprintf(err, errlen, "R_0 is required for %s", name);
    if (strcmp(name, "RATIONAL") == 0) {
      int nn = 6, mm = 0;
      if (parse_int(&W, "NN", &nn) < 0) snprintf(err, errlen, "could not parse NN");
      if (parse_int(&W, "MM", &mm) < 0) snprintf(err, errlen, "could not parse MM");
      rational_factory(s, d0, dmax, r0, nn, mm);
    } else if (strcmp(name, "SMAP") == 0) {
      int a = 0, b = 0;
      if (parse_int(&W, "A", &a) != 1) snprintf(err, errlen, "A is required for %s", name);
      if (parse_int(&W, "B", &b) != 1) snprintf(err, errlen, "B is required for %s", name);
      data_init(s, d0, dmax, r0);
      s->type = ORC_SW_SMAP;
      s->a = a;
      s->b = b;
      s->c = pow(2., (double)s->a / (double)s->b) - 1.0;
      s->d = -(double)s->b / (double)s->a;
    } else if (strcmp(name, "Q") == 0) {
      double beta = 50.0, lambda = 1.8, ref = 0.0;
      if (parse_double(&W, "BETA", &beta) < 0) snprintf(err, errlen, "could not parse BETA");
      if (parse_double(&W, "LAMBDA", &lambda) < 0) snprintf(err, errlen, "could not parse LAMBDA");
      if (parse_double(&W, "REF", &ref) != 1) snprintf(err, errlen, "REF is required for %s", name);
      data_init(s, d0, dmax, r0);
      s->type = ORC_SW_Q;
      s->beta = beta;
      s->lambda = lambda;
      s->ref = ref;
    } else if (strcmp(name, "EXP") == 0) {
      data_init(s, d0, dmax, r0);
      s->type = ORC_SW_EXP;
    } else if (strcmp(name, "GAUSSIAN") == 0) {
      if (r0 == 1.0 && d0 == 0.0) {
        data_init(s, 0.0, dmax, 1.0);
        s->type = ORC_SW_FASTGAUSSIAN;
      } else {
        data_init(s, d0, dmax, r0);
        s->type = ORC_SW_GAUSSIAN;
      }
    } else if (strcmp(name, "TANH") == 0) {
      data_init(s, d0, dmax, r0);
      s->type = ORC_SW_TANH;
    } else if (strcmp(name, "COSINUS") == 0) {
      data_init(s, d0, dmax, r0);
      s->type = ORC_SW_COSINUS;
    } else if (strcmp(name, "CUSTOM") == 0 || strcmp(name, "MATHEVAL") == 0) {
      char func[128] = "";
      const int got = parse_string(&W, "FUNC", func, sizeof func);
      if (got <= 0) {
        snprintf(err, errlen, got < 0 ? "FUNC is longer than the oracle's expression buffer"
                                      : "CUSTOM switching function without FUNC");
        return 1;
      }
      data_init(s, d0, dmax, r0);
      s->type = ORC_SW_CUSTOM;
      if (orc_expr_compile(&s->expr, func, err, errlen)) return 1;
    } else {
      snprintf(err, errlen, "cannot understand switching function type '%s'", name);
      return 1;
    }
  }
  if (W.n > 0) {
    int off = snprintf(err, errlen, "found the following rogue keywords in switching function input : ");
    for (int i = 0; i < W.n && off < errlen; i++) off += snprintf(err + off, errlen - off, "%s ", W.w[i]);
  }
  if (err[0]) return 1;
  if (dostretch && dmax != DBL_MAX) sw_setup_stretch(s);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* neighbour lists                                                          */
/* ------------------------------------------------------------------------ */
int64_t orc_nl_nallpairs(int mode, int64_t n0, int64_t n1) {
  if (mode == ORC_NL_SINGLE) return n0 * (n0 - 1) / 2;
  if (mode == ORC_NL_TWO) return n0 * n1;
  return n0;
}

void orc_nl_index_pair(int mode, int64_t n0, int64_t n1, int64_t ipair, int64_t out[2]) {
  if (mode == ORC_NL_PAIR) {
    out[0] = ipair;
    out[1] = ipair + n0;
  } else if (mode == ORC_NL_TWO) {
    out[0] = ipair / n1;
    out[1] = ipair % n1 + n0;
  } else {
    /* row-major upper triangle: the order getIndexPair enumerates
     * (NeighborList.cpp:158-163), computed exactly in integers */
    int64_t ii = n0 * (n0 - 1) / 2 - 1 - ipair;
    int64_t K = (int64_t)floor((sqrt((double)(8 * ii + 1)) + 1) / 2);
    while (K * (K - 1) / 2 > ii) K--;
    while ((K + 1) * K / 2 <= ii) K++;
    int64_t jj = ii - K * (K - 1) / 2;
    out[0] = n0 - 1 - K;
    out[1] = n0 - 1 - jj;
  }
}

int64_t orc_nl_all_pairs(int mode, int64_t n0, int64_t n1, uint32_t *pairs, int64_t cap) {
  int64_t np = orc_nl_nallpairs(mode, n0, n1), k = 0;
  if (mode == ORC_NL_SINGLE) {
    for (int64_t a = 0; a < n0; a++)
      for (int64_t b = a + 1; b < n0; b++, k++)
        if (k < cap) {
          pairs[2 * k] = (uint32_t)a;
          pairs[2 * k + 1] = (uint32_t)b;
        }
  } else {
    for (int64_t i = 0; i < np; i++, k++) {
      int64_t ip[2];
      orc_nl_index_pair(mode, n0, n1, i, ip);
      if (k < cap) {
        pairs[2 * k] = (uint32_t)ip[0];
        pairs[2 * k + 1] = (uint32_t)ip[1];
      }
    }
  }
  return np;
}

static inline void pair_distance(const orc_pbc *pbc, int do_pbc, const double *pos, int64_t i0, int64_t i1,
                                 double d[3]) {
  if (do_pbc) {
    orc_pbc_distance(pbc, pos + 3 * i0, pos + 3 * i1, d);
  } else {
    for (int k = 0; k < 3; k++) d[k] = pos[3 * i1 + k] - pos[3 * i0 + k];
  }
}

int64_t orc_nl_classic(int mode, int64_t n0, int64_t n1, const double *pos, const orc_pbc *pbc, int do_pbc,
                       double cutoff, uint32_t *pairs, int64_t cap) {
  const double d2 = cutoff * cutoff;
  int64_t np = orc_nl_nallpairs(mode, n0, n1), k = 0;
  int64_t a = 0, b = 1; /* single list: getIndexPair order without the per-pair sqrt */
  for (int64_t i = 0; i < np; i++) {
    int64_t ip[2];
    if (mode == ORC_NL_SINGLE) {
      ip[0] = a;
      ip[1] = b;
      if (++b >= n0) {
        a++;
        b = a + 1;
      }
    } else {
      orc_nl_index_pair(mode, n0, n1, i, ip);
    }
    double d[3];
    pair_distance(pbc, do_pbc, pos, ip[0], ip[1], d);
    double value = mod2(d);
    if (value <= d2) {
      if (k < cap) {
        pairs[2 * k] = (uint32_t)ip[0];
        pairs[2 * k + 1] = (uint32_t)ip[1];
      }
      k++;
    }
  }
  return k;
}

/* Cell-accelerated search with the classic exact test.  Orthorhombic or no
 * pbc; a generic box falls back to the brute-force restatement and a final
 * sort.  Cells are at least cutoff*(1+1e-9) wide so that every pair within
 * the cutoff lies in adjacent cells despite rounding at cell borders. */
static int cmp_pair(const void *x, const void *y) {
  const uint32_t *a = (const uint32_t *)x, *b = (const uint32_t *)y;
  if (a[0] != b[0]) return a[0] < b[0] ? -1 : 1;
  if (a[1] != b[1]) return a[1] < b[1] ? -1 : 1;
  return 0;
}

int64_t orc_nl_classic_cells(int mode, int64_t n0, int64_t n1, const double *pos, const orc_pbc *pbc, int do_pbc,
                             double cutoff, uint32_t *pairs, int64_t cap) {
  int use_pbc = do_pbc && pbc->type != ORC_PBC_UNSET;
  if ((use_pbc && pbc->type == ORC_PBC_GENERIC) || mode == ORC_NL_PAIR) {
    int64_t k = orc_nl_classic(mode, n0, n1, pos, pbc, do_pbc, cutoff, pairs, cap);
    if (k <= cap) qsort(pairs, (size_t)k, 2 * sizeof(uint32_t), cmp_pair);
    return k;
  }
  const double d2 = cutoff * cutoff;
  int64_t nslots = (mode == ORC_NL_TWO) ? n0 + n1 : n0;
  int64_t bstart = (mode == ORC_NL_TWO) ? n0 : 0; /* slots binned as partners */
  int64_t nb = nslots - bstart;
  double lo[3], width[3];
  int nc[3];
  for (int k = 0; k < 3; k++) {
    if (use_pbc) {
      lo[k] = 0.0;
      width[k] = pbc->box[4 * k];
    } else {
      double mn = DBL_MAX, mx = -DBL_MAX;
      for (int64_t i = 0; i < nslots; i++) {
        double x = pos[3 * i + k];
        if (x < mn) mn = x;
        if (x > mx) mx = x;
      }
      if (nslots == 0) mn = mx = 0.0;
      lo[k] = mn;
      width[k] = (mx - mn) > 0 ? (mx - mn) : 1.0;
    }
    int n = (int)floor(width[k] / (cutoff * (1.0 + 1e-9)));
    if (n < 1) n = 1;
    if (use_pbc && n < 3) n = 1;
    if (n > 1024) n = 1024;
    nc[k] = n;
  }
  int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
  int *cellof = (int *)malloc(sizeof(int) * (size_t)(nslots > 0 ? nslots : 1));
  int64_t *start = (int64_t *)calloc((size_t)ncell + 1, sizeof(int64_t));
  int64_t *list = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nb > 0 ? nb : 1));
  for (int64_t i = 0; i < nslots; i++) {
    int c3[3];
    for (int k = 0; k < 3; k++) {
      double f;
      if (use_pbc) {
        f = pos[3 * i + k] * pbc->invbox[4 * k];
        f = f - floor(f);
      } else {
        f = (pos[3 * i + k] - lo[k]) / width[k];
      }
      int c = (int)floor(f * nc[k]);
      if (c < 0) c = 0;
      if (c >= nc[k]) c = nc[k] - 1;
      c3[k] = c;
    }
    cellof[i] = (c3[2] * nc[1] + c3[1]) * nc[0] + c3[0];
  }
  for (int64_t i = bstart; i < nslots; i++) start[cellof[i] + 1]++;
  for (int64_t c = 0; c < ncell; c++) start[c + 1] += start[c];
  {
    int64_t *fill = (int64_t *)calloc((size_t)ncell, sizeof(int64_t));
    for (int64_t i = bstart; i < nslots; i++) {
      int c = cellof[i];
      list[start[c] + fill[c]++] = i;
    }
    free(fill);
  }
  int64_t k = 0;
  int64_t amax = (mode == ORC_NL_TWO) ? n0 : nslots;
  int64_t *row = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nb > 0 ? nb : 1));
  for (int64_t a = 0; a < amax; a++) {
    int ca = cellof[a];
    int cx = ca % nc[0], cy = (ca / nc[0]) % nc[1], cz = ca / (nc[0] * nc[1]);
    int64_t nrow = 0;
    for (int dz = -1; dz <= 1; dz++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          int x = cx + dx, y = cy + dy, z = cz + dz;
          if ((nc[0] == 1 && dx) || (nc[1] == 1 && dy) || (nc[2] == 1 && dz)) continue;
          if (use_pbc) {
            x = (x + nc[0]) % nc[0];
            y = (y + nc[1]) % nc[1];
            z = (z + nc[2]) % nc[2];
          } else if (x < 0 || y < 0 || z < 0 || x >= nc[0] || y >= nc[1] || z >= nc[2]) {
            continue;
          }
          int c = (z * nc[1] + y) * nc[0] + x;
          for (int64_t q = start[c]; q < start[c + 1]; q++) {
            int64_t b = list[q];
            if (mode == ORC_NL_SINGLE && b <= a) continue;
            double d[3];
            pair_distance(pbc, do_pbc, pos, a, b, d);
            if (mod2(d) <= d2) row[nrow++] = b;
          }
        }
    /* sort the row (insertion sort, rows are short) */
    for (int64_t i = 1; i < nrow; i++) {
      int64_t v = row[i], j = i - 1;
      while (j >= 0 && row[j] > v) {
        row[j + 1] = row[j];
        j--;
      }
      row[j + 1] = v;
    }
    for (int64_t i = 0; i < nrow; i++, k++)
      if (k < cap) {
        pairs[2 * k] = (uint32_t)a;
        pairs[2 * k + 1] = (uint32_t)row[i];
      }
  }
  free(row);
  free(cellof);
  free(start);
  free(list);
  return k;
}

/* LinkCells (LinkCells.cpp): createCells (:99-122), findMyCell (:255-266),
 * addRequiredCells (:184-231). */
typedef struct {
  orc_pbc mypbc;
  int nopbc;
  double origin[3];
  int ncells[3];
  int nstride[3];
} linkcells_t;

static void lc_create(linkcells_t *lc, const double box[9], double cutoff) {
  orc_pbc_set(&lc->mypbc, box);
  for (int k = 0; k < 3; k++) {
    /* reciprocal = transpose(invBox); row k = column k of invBox */
    double r[3] = {lc->mypbc.invbox[0 * 3 + k], lc->mypbc.invbox[1 * 3 + k], lc->mypbc.invbox[2 * 3 + k]};
    int n = (int)floor(1.0 / sqrt(mod2(r)) / cutoff);
    if (n == 0) n = 1;
    lc->ncells[k] = n;
  }
  lc->nstride[0] = 1;
  lc->nstride[1] = lc->ncells[0];
  lc->nstride[2] = lc->ncells[0] * lc->ncells[1];
}

void orc_linkcells_ncells(const orc_pbc *pbc, double cutoff, int ncells[3]) {
  linkcells_t lc;
  memset(&lc, 0, sizeof lc);
  lc_create(&lc, pbc->box, cutoff);
  for (int k = 0; k < 3; k++) ncells[k] = lc.ncells[k];
}

static void lc_setup(linkcells_t *lc, const double *pos, int64_t n, const orc_pbc *pbc, double cutoff) {
  memset(lc, 0, sizeof *lc);
  int allzero = 1;
  for (int k = 0; k < 9; k++)
    if (pbc->box[k] != 0.0) allzero = 0;
  if (allzero) {
    /* LinkCells::setupCells(pos) (:48-68) */
    lc->nopbc = 1;
    double box[9] = {0};
    double minp[3], maxp[3];
    for (int k = 0; k < 3; k++) {
      minp[k] = maxp[k] = pos[k];
    }
    for (int k = 0; k < 3; k++) {
      for (int64_t i = 1; i < n; i++) {
        if (pos[3 * i + k] > maxp[k]) maxp[k] = pos[3 * i + k];
        if (pos[3 * i + k] < minp[k]) minp[k] = pos[3 * i + k];
      }
      if (cutoff < sqrt(DBL_MAX))
        box[4 * k] = cutoff * (1 + ceil((maxp[k] - minp[k]) / cutoff));
      else
        box[4 * k] = maxp[k] - minp[k] + 1;
      lc->origin[k] = (minp[k] + maxp[k]) / 2;
    }
    lc_create(lc, box, cutoff);
  } else {
    lc->nopbc = 0;
    lc_create(lc, pbc->box, cutoff);
  }
}

static int lc_find_cell(const linkcells_t *lc, const double *p) {
  double mypos[3] = {p[0], p[1], p[2]};
  if (lc->nopbc)
    for (int k = 0; k < 3; k++) mypos[k] = mypos[k] - lc->origin[k];
  /* realToScaled: matmul(invBox.transpose(), v) */
  double invT[9], fpos[3];
  transpose33(lc->mypbc.invbox, invT);
  matvec(invT, mypos, fpos);
  int idx = 0;
  for (int j = 0; j < 3; j++) {
    unsigned c = (unsigned)floor((orc_tools_pbc(fpos[j]) + 0.5) * lc->ncells[j]);
    idx += (int)c * lc->nstride[j];
  }
  return idx;
}

static int lc_min_cell(int celn, int ncells, int usePBC) {
  celn += (ncells < 2) ? 0 : -1;
  return usePBC ? celn : (celn > 0 ? celn : 0);
}
static int lc_max_cell(int celn, int ncells, int usePBC) {
  celn += (ncells < 3 && usePBC) ? 1 : 2;
  return usePBC ? celn : (celn < ncells ? celn : ncells);
}
static int lc_required(const linkcells_t *lc, int cellIndex, int usePbc, int *req) {
  int celn[3];
  int r = cellIndex;
  celn[2] = r / lc->nstride[2];
  r = r % lc->nstride[2];
  celn[1] = r / lc->nstride[1];
  celn[0] = r % lc->nstride[1];
  int nreq = 0;
  int minX = lc_min_cell(celn[0], lc->ncells[0], usePbc), maxX = lc_max_cell(celn[0], lc->ncells[0], usePbc);
  int minY = lc_min_cell(celn[1], lc->ncells[1], usePbc), maxY = lc_max_cell(celn[1], lc->ncells[1], usePbc);
  int minZ = lc_min_cell(celn[2], lc->ncells[2], usePbc), maxZ = lc_max_cell(celn[2], lc->ncells[2], usePbc);
  for (int nx = minX; nx < maxX; ++nx) {
    int xval = ((nx < 0) ? lc->ncells[0] - 1 : nx % lc->ncells[0]) * lc->nstride[0];
    for (int ny = minY; ny < maxY; ++ny) {
      int yval = ((ny < 0) ? lc->ncells[1] - 1 : ny % lc->ncells[1]) * lc->nstride[1];
      for (int nz = minZ; nz < maxZ; ++nz) {
        int zval = ((nz < 0) ? lc->ncells[2] - 1 : nz % lc->ncells[2]) * lc->nstride[2];
        req[nreq++] = xval + yval + zval;
      }
    }
  }
  return nreq;
}

/* LinkCells::addRequiredCells (LinkCells.cpp:195-240) for the cell with indices
 * cell[3] of a box (not sorted; no cell twice): returns their number. */
int orc_linkcells_required(const orc_pbc *pbc, double cutoff, const int cell[3], int use_pbc, int *req) {
  linkcells_t lc;
  memset(&lc, 0, sizeof lc);
  lc_create(&lc, pbc->box, cutoff);
  const int idx = cell[0] * lc.nstride[0] + cell[1] * lc.nstride[1] + cell[2] * lc.nstride[2];
  return lc_required(&lc, idx, use_pbc, req);
}

int64_t orc_nl_linkcells(int mode, int64_t n0, int64_t n1, const double *pos, const orc_pbc *pbc, int do_pbc,
                         double cutoff, uint32_t *pairs, int64_t cap) {
  if (mode == ORC_NL_PAIR) return -1;
  int64_t nslots = (mode == ORC_NL_TWO) ? n0 + n1 : n0;
  {
    /* LinkCells::setupCells(pbc) (LinkCells.cpp:75-83): a box that is not all
     * zero must have a volume above DBL_EPSILON */
    const double *b = pbc->box;
    int allzero = 1;
    for (int k = 0; k < 9; k++)
      if (b[k] != 0.0) allzero = 0;
    const double det = b[0] * (b[4] * b[8] - b[5] * b[7]) - b[1] * (b[3] * b[8] - b[5] * b[6]) +
                       b[2] * (b[3] * b[7] - b[4] * b[6]);
    if (!allzero && !(det > DBL_EPSILON)) return -2;
  }
  linkcells_t lc;
  lc_setup(&lc, pos, nslots, pbc, cutoff);
  int64_t ncell = (int64_t)lc.ncells[0] * lc.ncells[1] * lc.ncells[2];
  int *cellof = (int *)malloc(sizeof(int) * (size_t)(nslots > 0 ? nslots : 1));
  for (int64_t i = 0; i < nslots; i++) cellof[i] = lc_find_cell(&lc, pos + 3 * i);
  /* collections A (slots [0,na)) and B (slots [bs, nslots)); within a cell in slot order */
  int64_t na = (mode == ORC_NL_TWO) ? n0 : nslots, bs = (mode == ORC_NL_TWO) ? n0 : 0;
  int64_t *sa = (int64_t *)calloc((size_t)ncell + 1, sizeof(int64_t));
  int64_t *sb = (int64_t *)calloc((size_t)ncell + 1, sizeof(int64_t));
  int64_t *la = (int64_t *)malloc(sizeof(int64_t) * (size_t)(na > 0 ? na : 1));
  int64_t *lb = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nslots - bs > 0 ? nslots - bs : 1));
  for (int64_t i = 0; i < na; i++) sa[cellof[i] + 1]++;
  for (int64_t i = bs; i < nslots; i++) sb[cellof[i] + 1]++;
  for (int64_t c = 0; c < ncell; c++) {
    sa[c + 1] += sa[c];
    sb[c + 1] += sb[c];
  }
  {
    int64_t *fa = (int64_t *)calloc((size_t)ncell, sizeof(int64_t));
    int64_t *fb = (int64_t *)calloc((size_t)ncell, sizeof(int64_t));
    for (int64_t i = 0; i < na; i++) la[sa[cellof[i]] + fa[cellof[i]]++] = i;
    for (int64_t i = bs; i < nslots; i++) lb[sb[cellof[i]] + fb[cellof[i]]++] = i;
    free(fa);
    free(fb);
  }
  int64_t k = 0;
  int req[27];
  for (int64_t c = 0; c < ncell; c++) {
    if (sa[c + 1] == sa[c]) continue;
    int nreq = lc_required(&lc, (int)c, do_pbc, req);
    for (int64_t q = sa[c]; q < sa[c + 1]; q++) {
      int64_t A = la[q];
      for (int cb = 0; cb < nreq; cb++) {
        int cc = req[cb];
        for (int64_t t = sb[cc]; t < sb[cc + 1]; t++) {
          int64_t B = lb[t];
          if (mode == ORC_NL_SINGLE && !(B > A)) continue;
          if (k < cap) {
            pairs[2 * k] = (uint32_t)A;
            pairs[2 * k + 1] = (uint32_t)B;
          }
          k++;
        }
      }
    }
  }
  free(cellof);
  free(sa);
  free(sb);
  free(la);
  free(lb);
  return k;
}

/* ------------------------------------------------------------------------ */
/* CoordinationBase::calculate (CoordinationBase.cpp:142-231)               */
/* ------------------------------------------------------------------------ */
void orc_dhenergy_constants(double ionic, double temp, double epsilon, double unit_energy, double unit_length,
                            double unit_charge, double *k, double *constant) {
  /* DHEnergy.cpp:112-113, same operation order */
  *constant = 138.935458111 / unit_energy / unit_length * unit_charge * unit_charge;
  *k = sqrt(ionic / (epsilon * temp)) * 502.903741125 * unit_length;
}

void orc_ghbfix_constants(orc_pairing *p, double d0, double dmax, double c) {
  /* GHBFIX.cpp:111-126 */
  const double dmax2 = dmax - d0;
  p->gh_dmax_sq = dmax * dmax;
  p->gh_d0 = d0;
  p->gh_c_dmax2 = c * dmax2;
  p->gh_A = (-c * dmax2 * dmax2) / ((1 - c) * dmax2 * dmax2);
  p->gh_B = (2 * dmax2) / ((1 - c) * dmax2 * dmax2);
  p->gh_C = -1 / ((1 - c) * dmax2 * dmax2);
  p->gh_D = 1 / (c * dmax2 * dmax2);
}

double orc_pairing_eval(const orc_pairing *p, double distance2, double *dfunc, int64_t i, int64_t j) {
  if (p->kind == ORC_CV_DHENERGY) {
    /* DHEnergy::pairing (DHEnergy.cpp:128-142); self pairs never reach it */
    const double distance = sqrt(distance2);
    const double invdistance = 1.0 / distance;
    const double tmp = exp(-p->dh_k * distance) * invdistance * p->dh_constant * p->charge[i] * p->charge[j] /
                       p->dh_epsilon;
    const double dtmp = -(p->dh_k + invdistance) * tmp;
    *dfunc = dtmp * invdistance;
    return tmp;
  }
  if (p->kind == ORC_CV_GHBFIX) {
    /* GHBFIX::pairing (GHBFIX.cpp:178-218) */
    const double scale = p->eta[p->gh_ntypes * p->type[i] + p->type[j]];
    if (distance2 > p->gh_dmax_sq) {
      *dfunc = 0.0;
      return 0.;
    }
    const double distance = sqrt(distance2);
    const double rdist = distance - p->gh_d0;
    double result = -1., df = 0.0;
    if (rdist > 0.) {
      if (rdist > p->gh_c_dmax2) {
        result += (p->gh_A + p->gh_B * rdist + p->gh_C * rdist * rdist);
        df += p->gh_B + 2 * p->gh_C * rdist;
      } else {
        result += p->gh_D * (rdist * rdist);
        df += 2 * p->gh_D * rdist;
      }
      df /= distance;
    }
    result *= scale;
    df *= scale;
    *dfunc = df;
    return result;
  }
  return orc_switch_calculate_sqr(p->sw, distance2, dfunc);
}

int orc_peratom(const orc_switch *sw, const orc_pbc *pbc, int do_pbc, int64_t nslots, const int64_t *abs_index,
                const double *pos, const uint32_t *pairs, int64_t npairs, const double *g, double *cn, double *grad,
                double virial[9]) {
  for (int64_t i = 0; i < nslots; i++) cn[i] = 0.0;
  if (g) {
    for (int64_t i = 0; i < 3 * nslots; i++) grad[i] = 0.0;
    for (int k = 0; k < 9; k++) virial[k] = 0.0;
  }
  for (int64_t i = 0; i < npairs; ++i) {
    const int64_t i0 = pairs[2 * i], i1 = pairs[2 * i + 1];
    if (abs_index[i0] == abs_index[i1]) continue;
    double distance[3];
    pair_distance(pbc, do_pbc, pos, i0, i1, distance);
    const double m2 = mod2(distance);
    if (m2 < DBL_EPSILON) continue; /* ContactMatrix.h:99-101 */
    double dfunc = 0.;
    const double sig = orc_switch_calculate_sqr(sw, m2, &dfunc);
    if (sig < DBL_EPSILON) continue; /* ContactMatrix.h:104-107 */
    cn[i0] += sig;
    cn[i1] += sig;
    if (g) {
      const double w = g[i0] + g[i1];
      const double dd[3] = {w * dfunc * distance[0], w * dfunc * distance[1], w * dfunc * distance[2]};
      for (int k = 0; k < 3; k++) {
        grad[3 * i0 + k] -= dd[k];
        grad[3 * i1 + k] += dd[k];
      }
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) virial[3 * a + b] -= dd[a] * distance[b];
    }
  }
  return 0;
}

int orc_contactmap(const orc_switch *sw, int nsw, int64_t n, const double *reference, const double *weight, int mode,
                   const orc_pbc *pbc, int do_pbc, const double *pos, double *value, double *deriv, double *vir) {
  const int nv = mode == 0 ? (int)n : 1;
  for (int64_t i = 0; i < (mode == 0 ? n : 1); i++) value[i] = 0.0;
  for (int64_t i = 0; i < 6 * n; i++) deriv[i] = 0.0;
  for (int64_t i = 0; i < 9 * (int64_t)nv; i++) vir[i] = 0.0;
  double ncoord = 0.;
  for (int64_t i = 0; i < n; i++) {
    const int64_t i0 = i, i1 = n + i;
    double distance[3];
    pair_distance(pbc, do_pbc, pos, i0, i1, distance);
    double dfunc = 0.;
    const double coord = weight[i] * (orc_switch_calculate(&sw[nsw == 1 ? 0 : i], sqrt(mod2(distance)), &dfunc) -
                                      reference[i]);
    double tmpder[3], tmpvir[9];
    for (int k = 0; k < 3; k++) tmpder[k] = weight[i] * dfunc * distance[k];
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) tmpvir[3 * a + b] = weight[i] * dfunc * (distance[a] * distance[b]);
    if (mode == 2) {
      for (int k = 0; k < 3; k++) tmpder[k] *= 2. * coord;
      for (int k = 0; k < 9; k++) tmpvir[k] *= 2. * coord;
    }
    for (int k = 0; k < 3; k++) {
      deriv[3 * i0 + k] -= tmpder[k];
      deriv[3 * i1 + k] += tmpder[k];
    }
    double *v = vir + (mode == 0 ? 9 * i : 0);
    for (int k = 0; k < 9; k++) v[k] -= tmpvir[k];
    if (mode == 0)
      value[i] = coord;
    else
      ncoord += mode == 2 ? coord * coord : coord;
  }
  if (mode != 0) value[0] = ncoord;
  return 0;
}

int orc_coordination(const orc_switch *sw, const orc_pbc *pbc, int do_pbc, int64_t nslots,
                     const int64_t *abs_index, const double *pos, const uint32_t *pairs, int64_t npairs, double *s,
                     double *deriv, double virial[9], int nthreads) {
  orc_pairing p;
  memset(&p, 0, sizeof p);
  p.kind = ORC_CV_COORDINATION;
  p.sw = sw;
  return orc_cv(&p, pbc, do_pbc, nslots, abs_index, pos, pairs, npairs, s, deriv, virial, nthreads);
}

int orc_cv(const orc_pairing *pr, const orc_pbc *pbc, int do_pbc, int64_t nslots, const int64_t *abs_index,
           const double *pos, const uint32_t *pairs, int64_t npairs, double *s, double *deriv, double virial[9],
           int nthreads) {
  double ncoord = 0.;
  for (int64_t i = 0; i < 3 * nslots; i++) deriv[i] = 0.0;
  for (int k = 0; k < 9; k++) virial[k] = 0.0;
  int nt = nthreads < 1 ? 1 : nthreads;
  if ((int64_t)nt * 10 > npairs) nt = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
  {
    double *omp_deriv = NULL;
    double omp_virial[9] = {0};
    if (nt > 1) omp_deriv = (double *)calloc((size_t)(3 * nslots > 0 ? 3 * nslots : 1), sizeof(double));
    double *dv = (nt > 1) ? omp_deriv : deriv;
    double *vir = (nt > 1) ? omp_virial : virial;
#ifdef _OPENMP
#pragma omp for reduction(+ : ncoord) nowait
#endif
    for (int64_t i = 0; i < npairs; ++i) {
      const int64_t i0 = pairs[2 * i], i1 = pairs[2 * i + 1];
      if (abs_index[i0] == abs_index[i1]) continue;
      double distance[3];
      pair_distance(pbc, do_pbc, pos, i0, i1, distance);
      double dfunc = 0.;
      ncoord += orc_pairing_eval(pr, mod2(distance), &dfunc, i0, i1);
      double dd[3] = {dfunc * distance[0], dfunc * distance[1], dfunc * distance[2]};
      for (int k = 0; k < 3; k++) {
        dv[3 * i0 + k] -= dd[k];
        dv[3 * i1 + k] += dd[k];
      }
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) vir[3 * a + b] -= dd[a] * distance[b];
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    if (nt > 1) {
      for (int64_t i = 0; i < 3 * nslots; i++) deriv[i] += omp_deriv[i];
      for (int k = 0; k < 9; k++) virial[k] += omp_virial[k];
    }
    free(omp_deriv);
  }
  *s = ncoord;
  return 0;
}
