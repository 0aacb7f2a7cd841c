// switch_eval.cuh -- switching functions, value and dfunc, host and device.
//
// One templated evaluator per switch type.  Instantiated with double inside a
// translation unit compiled without FMA contraction (-fmad=false on the
// device, -ffp-contract=off on the host), every function below performs the
// reference's operations in the reference's order, so a pair's (sigma,
// dfunc) is bit-identical to SwitchingFunction::calculateSqr for the rational
// family (only +,-,*,/ and sqrt, all correctly rounded).  The exp/tanh/cos
// families call CUDA's math library, which may differ from the host libm in
// the last ulp.
//
// Semantics follow src/tools/SwitchingFunction.cpp:
//   baseSwitch::calculate (:130-147), applystretch (:121-127),
//   fixedRational<N>::calculateSqr (:203-215), rational<>::doRational
//   (:253-280) and calculateSqr (:288-303), fastgaussian calculateSqr
//   (:410-431), nativeq calculate (:527-555).
#pragma once
#include "coord_internal.h"
#include <cmath>

#ifdef __CUDACC__
#define SW_HD __host__ __device__ __forceinline__
// called, not inlined: the expression interpreter would otherwise be copied
// into every kernel that can meet a CUSTOM switch (compile time, registers)
#define SW_HD_CALL static __host__ __device__ __noinline__
#else
#define SW_HD inline
#define SW_HD_CALL static
#endif

namespace coordgpu {

template <typename T> struct VD {
  T f, d;
};

SW_HD double m_exp(double x) { return exp(x); }
SW_HD float m_exp(float x) { return expf(x); }
SW_HD double m_tanh(double x) { return tanh(x); }
SW_HD float m_tanh(float x) { return tanhf(x); }
SW_HD double m_cos(double x) { return cos(x); }
SW_HD float m_cos(float x) { return cosf(x); }
SW_HD double m_sin(double x) { return sin(x); }
SW_HD float m_sin(float x) { return sinf(x); }
SW_HD double m_pow(double x, double y) { return pow(x, y); }
SW_HD float m_pow(float x, float y) { return powf(x, y); }
SW_HD double m_sqrt(double x) { return sqrt(x); }
SW_HD float m_sqrt(float x) { return sqrtf(x); }

// Tools::fastpow(base, exp) (Tools.h:582-597); the compile-time fastpow<N>
// performs the same multiplications in the same order.
template <typename T> SW_HD T fastpow(T base, int exp) {
  if (exp < 0) {
    exp = -exp;
    base = T(1.0) / base;
  }
  T result = T(1.0);
  while (exp) {
    if (exp & 1) result *= base;
    exp >>= 1;
    base *= base;
  }
  return result;
}

// fixedRational<N>::doRational<POW> (:191-196)
template <typename T> SW_HD VD<T> rational_fixed(int POW, T rdist) {
  VD<T> r;
  const T rNdist = fastpow<T>(rdist, POW - 1);
  r.f = T(1.0) / (T(1.0) + rNdist * rdist);
  r.d = T(-POW) * rNdist * r.f * r.f;
  return r;
}

// rational<isFast,nis2m>::doRational (:253-280)
template <typename T>
SW_HD VD<T> rational_rt(bool simplified, T rdist, T secDev, int N, int M, T dfunc, T result) {
  const T moreThanOne = T(1.0 + 5.0e10 * 2.220446049250313080847263336181640625e-16);
  const T lessThanOne = T(1.0 - 5.0e10 * 2.220446049250313080847263336181640625e-16);
  if (simplified) {
    const T rNdist = fastpow<T>(rdist, N - 1);
    result = T(1.0) / (T(1.0) + rNdist * rdist);
    dfunc = T(-N) * rNdist * result * result;
  } else if (!((rdist > lessThanOne) && (rdist < moreThanOne))) {
    const T rNdist = fastpow<T>(rdist, N - 1);
    const T rMdist = fastpow<T>(rdist, M - 1);
    const T num = T(1.0) - rNdist * rdist;
    const T iden = T(1.0) / (T(1.0) - rMdist * rdist);
    result = num * iden;
    dfunc = ((T(M) * result * rMdist) - (T(N) * rNdist)) * iden;
  } else {
    const T x = (rdist - T(1.0));
    result = result + x * (dfunc + T(0.5) * x * secDev);
    dfunc = dfunc + x * secDev;
  }
  return VD<T>{result, dfunc};
}

// (1 - x^N)/(1 - x^M) for x >= 0 as a ratio of geometric sums
// P_N(x)/P_M(x), P_K = 1 + x + ... + x^(K-1): no cancellation near x = 1, so
// single precision keeps its relative accuracy there (the FP64 path uses the
// reference's closed form and Taylor window instead).
template <typename T> SW_HD VD<T> rational_geometric(T x, int N, int M) {
  T pn = T(0), dpn = T(0), pm = T(0), dpm = T(0), xk = T(1), xkm1 = T(0);
  const int K = N > M ? N : M;
  for (int k = 0; k < K; k++) {
    if (k < N) {
      pn += xk;
      dpn += T(k) * xkm1;
    }
    if (k < M) {
      pm += xk;
      dpm += T(k) * xkm1;
    }
    xkm1 = xk;
    xk *= x;
  }
  const T inv = T(1) / pm;
  const T f = pn * inv;
  return VD<T>{f, (dpn - f * dpm) * inv};
}

// switching::function(rdist) of the baseSwitch types
template <typename T> SW_HD VD<T> sw_function(const SwitchParams &s, T rdist) {
  switch (s.type) {
  case SW_RATFIX:
    return rational_fixed<T>(s.nn, rdist);
  case SW_RATIONAL:
  case SW_RATIONAL_FAST:
    if (sizeof(T) == 4 && s.nn > 0 && s.mm > 0 && rdist >= T(0)) return rational_geometric<T>(rdist, s.nn, s.mm);
    return rational_rt<T>(false, rdist, T(s.preSecDev), s.nn, s.mm, T(s.preDfunc), T(s.preRes));
  case SW_RATIONAL_SIMPLE:
  case SW_RATIONAL_SIMPLE_FAST:
    return rational_rt<T>(true, rdist, T(s.preSecDev), s.nn, s.mm, T(s.preDfunc), T(s.preRes));
  case SW_EXP: {
    T result = m_exp(-rdist);
    return VD<T>{result, -result};
  }
  case SW_GAUSSIAN:
  case SW_FASTGAUSSIAN: {
    T result = m_exp(T(-0.5) * rdist * rdist);
    return VD<T>{result, -rdist * result};
  }
  case SW_SMAP: {
    const T sx = T(s.c) * fastpow<T>(rdist, s.a);
    T result = m_pow(T(1.0) + sx, T(s.d));
    T dfunc = T(-s.b) * sx / rdist * result / (T(1.0) + sx);
    return VD<T>{result, dfunc};
  }
  case SW_CUBIC: {
    const T tmp1 = rdist - T(1.0);
    const T tmp2 = T(1.0) + T(2.0) * rdist;
    T dfunc = T(2) * tmp1 * tmp2 + T(2) * tmp1 * tmp1;
    return VD<T>{tmp1 * tmp1 * tmp2, dfunc};
  }
  case SW_TANH: {
    const T tmp1 = m_tanh(rdist);
    T dfunc = tmp1 * tmp1 - T(1.0);
    return VD<T>{T(1.0) - tmp1, dfunc};
  }
  case SW_COSINUS: {
    T result = T(0.0), dfunc = T(0.0);
    if (rdist <= T(1.0)) {
      const T pi = T(3.141592653589793238462643383279502884197169399375105820974944592307);
      T rdistPI = rdist * pi;
      result = T(0.5) * (m_cos(rdistPI) + T(1.0));
      dfunc = T(-0.5) * pi * m_sin(rdistPI);
    }
    return VD<T>{result, dfunc};
  }
  default:
    return VD<T>{T(0), T(0)};
  }
}

// ---------------------------------------------------------------------------
// CUSTOM: the compiled expression run forward on (value, derivative) pairs,
// with lepton's operations and their derivatives (src/lepton/Operation.h and
// Operation.cpp: step differentiates to delta without the chain factor, abs
// to 2 step - 1, min and max through step(a - b), select through its
// branches; a constant integer power by repeated squaring as
// PowerConstant::evaluate).  FP64 in every path.
// ---------------------------------------------------------------------------
SW_HD double expr_powc(double a, double c) {
  const int ic = (int)c;
  if ((double)ic != c) return pow(a, c);
  int n = ic < 0 ? -ic : ic;
  double base = ic < 0 ? 1.0 / a : a, r = 1.0;
  for (; n != 0; n >>= 1) {
    if (n & 1) r *= base;
    base *= base;
  }
  return r;
}

SW_HD_CALL VD<double> expr_run(const ExprProgram &p, double var) {
  double v[kExprMaxStack], d[kExprMaxStack];
  int sp = 0;
  const double two_over_sqrtpi = 1.1283791670955126;  // 2/sqrt(pi)
  for (int i = 0; i < p.n; i++) {
    const int op = p.op[i];
    if (op == EX_VAR || op == EX_CONST) {
      v[sp] = op == EX_VAR ? var : p.cst[i];
      d[sp] = op == EX_VAR ? 1.0 : 0.0;
      sp++;
      continue;
    }
    if (op == EX_SELECT) {  // select(c, a, b)
      const bool t = v[sp - 3] != 0.0;
      v[sp - 3] = t ? v[sp - 2] : v[sp - 1];
      d[sp - 3] = t ? d[sp - 2] : d[sp - 1];
      sp -= 2;
      continue;
    }
    if (op >= EX_ADD && op <= EX_POW || op >= EX_ATAN2) {  // two arguments
      const double x = v[sp - 2], dx = d[sp - 2], y = v[sp - 1], dy = d[sp - 1];
      double r, dr;
      switch (op) {
      case EX_ADD: r = x + y; dr = dx + dy; break;
      case EX_SUB: r = x - y; dr = dx - dy; break;
      case EX_MUL: r = x * y; dr = dx * y + x * dy; break;
      case EX_DIV: r = x / y; dr = dx / y - x * dy / (y * y); break;
      case EX_POW: r = pow(x, y); dr = y * pow(x, y - 1.0) * dx + log(x) * r * dy; break;
      case EX_ATAN2: r = atan2(x, y); dr = (y * dx - x * dy) / (x * x + y * y); break;
      case EX_MIN: r = (y < x) ? y : x; dr = (x - y >= 0.0) ? dy : dx; break;
      default: r = (x < y) ? y : x; dr = (x - y >= 0.0) ? dx : dy; break;  // EX_MAX
      }
      sp--;
      v[sp - 1] = r;
      d[sp - 1] = dr;
      continue;
    }
    const double x = v[sp - 1], dx = d[sp - 1];
    double r = 0.0, dr = 0.0;
    switch (op) {
    case EX_POWC: r = expr_powc(x, p.cst[i]); dr = p.cst[i] * expr_powc(x, p.cst[i] - 1.0) * dx; break;
    case EX_NEG: r = -x; dr = -dx; break;
    case EX_SQRT: r = sqrt(x); dr = 0.5 * (1.0 / r) * dx; break;
    case EX_EXP: r = exp(x); dr = r * dx; break;
    case EX_LOG: r = log(x); dr = (1.0 / x) * dx; break;
    case EX_SIN: r = sin(x); dr = cos(x) * dx; break;
    case EX_COS: r = cos(x); dr = -sin(x) * dx; break;
    case EX_SEC: r = 1.0 / cos(x); dr = r * tan(x) * dx; break;
    case EX_CSC: r = 1.0 / sin(x); dr = -r * (1.0 / tan(x)) * dx; break;
    case EX_TAN: { const double sc = 1.0 / cos(x); r = tan(x); dr = sc * sc * dx; break; }
    case EX_COT: { const double sc = 1.0 / sin(x); r = 1.0 / tan(x); dr = -sc * sc * dx; break; }
    case EX_ASIN: r = asin(x); dr = 1.0 / sqrt(1.0 - x * x) * dx; break;
    case EX_ACOS: r = acos(x); dr = -1.0 / sqrt(1.0 - x * x) * dx; break;
    case EX_ATAN: r = atan(x); dr = 1.0 / (1.0 + x * x) * dx; break;
    case EX_SINH: r = sinh(x); dr = cosh(x) * dx; break;
    case EX_COSH: r = cosh(x); dr = sinh(x) * dx; break;
    case EX_TANH: r = tanh(x); dr = (1.0 - r * r) * dx; break;
    case EX_ERF: r = erf(x); dr = two_over_sqrtpi * exp(-x * x) * dx; break;
    case EX_ERFC: r = erfc(x); dr = -two_over_sqrtpi * exp(-x * x) * dx; break;
    case EX_STEP: r = (x >= 0.0) ? 1.0 : 0.0; dr = (x == 0.0) ? INFINITY : 0.0; break;
    case EX_DELTA: r = (x == 0.0) ? INFINITY : 0.0; dr = (x == 0.0) ? NAN : 0.0; break;
    case EX_SQUARE: r = x * x; dr = 2.0 * x * dx; break;
    case EX_CUBE: r = x * x * x; dr = 3.0 * (x * x) * dx; break;
    case EX_RECIP: r = 1.0 / x; dr = -(1.0 / (x * x)) * dx; break;
    case EX_ABS: r = fabs(x); dr = (dx == 0.0) ? 0.0 : dx * (2.0 * ((x >= 0.0) ? 1.0 : 0.0) - 1.0); break;
    case EX_FLOOR: r = floor(x); break;
    case EX_CEIL: r = ceil(x); break;
    default: break;
    }
    v[sp - 1] = r;
    d[sp - 1] = dr;
  }
  return sp ? VD<double>{v[sp - 1], d[sp - 1]} : VD<double>{0.0, 0.0};
}

SW_HD const ExprProgram &expr_of(const SwitchParams &s) {
#ifdef __CUDA_ARCH__
  return *s.expr_dev;
#else
  return *s.expr_host;
#endif
}

// leptonSwitch::calculate and calculateSqr (SwitchingFunction.cpp:709-751)
// for a distance r or its square r2 (from_sqr).  With x2 the expression takes
// r^2 / r0^2 (D_0 does not enter); with x it takes (r - d0) / r0 and is 1
// (stretched) for x <= 0.
SW_HD_CALL VD<double> custom_eval(const SwitchParams &s, double r, double r2, bool from_sqr) {
  const ExprProgram &p = expr_of(s);
  VD<double> out{0.0, 0.0};
  if (p.var_x2) {
    const double distance2 = from_sqr ? r2 : r * r;
    if (distance2 <= s.dmax_2) {
      const double rdist_2 = distance2 * s.invr0_2;
      out = expr_run(p, rdist_2);
      out.d *= 2 * s.invr0_2;
      out.f = out.f * s.stretch + s.shift;
      out.d *= s.stretch;
    }
    return out;
  }
  const double distance = from_sqr ? sqrt(r2) : r;
  if (distance <= s.dmax) {
    out.f = 1.0;
    const double rdist = (distance - s.d0) * s.invr0;
    if (rdist > 0.0) {
      out = expr_run(p, rdist);
      out.d *= s.invr0;
      out.d /= distance;
    }
    out.f = out.f * s.stretch + s.shift;
    out.d *= s.stretch;
  }
  return out;
}

// nativeqSwitch::calculate (:527-555)
template <typename T> SW_HD VD<T> nativeq_calculate(const SwitchParams &s, T distance) {
  T res = T(0.0), dfunc = T(0.0);
  if (distance <= T(s.dmax)) {
    res = T(1.0);
    if (distance > T(s.d0)) {
      const T rdist = T(s.beta) * (distance - T(s.lambda) * T(s.ref));
      T exprdist = m_exp(rdist);
      res = T(1.0) / (T(1.0) + exprdist);
      dfunc = -T(s.beta) / (exprdist + T(2.0) + T(1.0) / exprdist) / distance;
      dfunc *= T(s.stretch);
    }
    res = res * T(s.stretch) + T(s.shift);
  }
  return VD<T>{res, dfunc};
}

// baseSwitch::calculate + applystretch
template <typename T> SW_HD VD<T> sw_calculate(const SwitchParams &s, T distance) {
  if (s.type == SW_Q) return nativeq_calculate<T>(s, distance);
  if (s.type == SW_CUSTOM) {
    const VD<double> r = custom_eval(s, (double)distance, 0.0, false);
    return VD<T>{T(r.f), T(r.d)};
  }
  const T rdist = (distance - T(s.d0)) * T(s.invr0);
  if (distance > T(s.dmax)) return VD<T>{T(0.0), T(0.0)};
  if (rdist > T(0.0)) {
    VD<T> r = sw_function<T>(s, rdist);
    r.f = r.f * T(s.stretch) + T(s.shift);
    r.d *= T(s.stretch);
    r.d *= T(s.invr0);
    r.d /= distance;
    return r;
  }
  return VD<T>{T(s.stretch) + T(s.shift), T(0.0)};
}

// calculateSqr dispatch
template <typename T> SW_HD VD<T> sw_calculate_sqr(const SwitchParams &s, T distance2) {
  VD<T> r{T(0.0), T(0.0)};
  switch (s.type) {
  case SW_CUSTOM: {
    const VD<double> c = custom_eval(s, 0.0, (double)distance2, true);
    return VD<T>{T(c.f), T(c.d)};
  }
  case SW_RATFIX:
    if (distance2 <= T(s.dmax_2)) {
      const T rdist = distance2 * T(s.invr0_2);
      r = rational_fixed<T>(s.nn / 2, rdist);
      r.d *= T(2) * T(s.invr0_2);
      r.f = r.f * T(s.stretch) + T(s.shift);
      r.d *= T(s.stretch);
    }
    return r;
  case SW_RATIONAL_FAST:
  case SW_RATIONAL_SIMPLE_FAST:
    if (distance2 <= T(s.dmax_2)) {
      const T rdist = distance2 * T(s.invr0_2);
      if (sizeof(T) == 4 && s.type == SW_RATIONAL_FAST && s.nnf > 0 && s.mmf > 0)
        r = rational_geometric<T>(rdist, s.nnf, s.mmf);
      else
        r = rational_rt<T>(s.type == SW_RATIONAL_SIMPLE_FAST, rdist, T(s.preSecDevF), s.nnf, s.mmf, T(s.preDfuncF),
                           T(s.preRes));
      r.d *= T(2) * T(s.invr0_2);
      r.f = r.f * T(s.stretch) + T(s.shift);
      r.d *= T(s.stretch);
    }
    return r;
  case SW_FASTGAUSSIAN:
    if (distance2 < T(s.dmax_2)) {
      r.f = T(1.0);
      if (distance2 > T(0.0)) {
        r.f = m_exp(T(-0.5) * distance2);
        r.d = -r.f;
        r.f = r.f * T(s.stretch) + T(s.shift);
        r.d *= T(s.stretch);
      }
    }
    return r;
  default:
    return sw_calculate<T>(s, m_sqrt(distance2));
  }
}

// ---------------------------------------------------------------------------
// Tools::pbc (Tools.h:547-571) and Pbc::distance (Pbc.cpp:383-415), FP64.
// ---------------------------------------------------------------------------
SW_HD double tools_pbc(double x) {
  x += 100.0;
  if (x >= 0) return x - (double)(int)(x + 0.5);
  return x - (double)(int)(x - 0.5);
}

SW_HD double mod2(const double d[3]) { return d[0] * d[0] + d[1] * d[1] + d[2] * d[2]; }

// v2 - v1 under the frame's pbc, writing d.
SW_HD void pbc_distance(const PbcParams &p, const double v1[3], const double v2[3], double d[3]) {
  for (int k = 0; k < 3; k++) d[k] = v2[k] - v1[k];
  if (p.type == PBC_ORTHO) {
    for (int k = 0; k < 3; k++) d[k] = tools_pbc(d[k] * p.invbox[k * 4]) * p.box[k * 4];
  } else if (p.type == PBC_GENERIC) {
    double s[3];
    for (int i = 0; i < 3; i++) {
      double acc = 0.0;
      for (int j = 0; j < 3; j++) acc += d[j] * p.invreduced[j * 3 + i];
      s[i] = acc;
    }
    for (int k = 0; k < 3; k++) s[k] = tools_pbc(s[k]);
    for (int i = 0; i < 3; i++) {
      double acc = 0.0;
      for (int j = 0; j < 3; j++) acc += s[j] * p.reduced[j * 3 + i];
      d[i] = acc;
    }
    if (fabs(s[0]) + fabs(s[1]) + fabs(s[2]) > 0.5) {
      const int o = 4 * (s[0] > 0 ? 1 : 0) + 2 * (s[1] > 0 ? 1 : 0) + (s[2] > 0 ? 1 : 0);
      double best[3] = {d[0], d[1], d[2]};
      double lbest = mod2(best);
      for (int i = 0; i < p.nshift[o]; i++) {
        double trial[3] = {d[0] + p.shift[o][i][0], d[1] + p.shift[o][i][1], d[2] + p.shift[o][i][2]};
        double ltrial = mod2(trial);
        if (ltrial < lbest) {
          lbest = ltrial;
          best[0] = trial[0];
          best[1] = trial[1];
          best[2] = trial[2];
        }
      }
      d[0] = best[0];
      d[1] = best[1];
      d[2] = best[2];
    }
  }
}

} // namespace coordgpu
