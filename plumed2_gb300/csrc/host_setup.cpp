// host_setup.cpp -- switching-function and pbc set-up on the host.
//
// Compiled with -ffp-contract=off: stretch, shift, inverse boxes and shift
// tables must carry the same bits as the reference's set-up code, because the
// FP64 kernels consume them.
#include "coord_internal.h"
#include "switch_eval.cuh"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace coordgpu {

double switch_host_calculate(const SwitchParams &sw, double distance, double *dfunc) {
  VD<double> r = sw_calculate<double>(sw, distance);
  *dfunc = r.d;
  return r.f;
}
double switch_host_calculate_sqr(const SwitchParams &sw, double distance2, double *dfunc) {
  VD<double> r = sw_calculate_sqr<double>(sw, distance2);
  *dfunc = r.d;
  return r.f;
}

namespace {

// switchContainers::Data::init (SwitchingFunction.cpp:84-94)
void data_init(SwitchParams *s, double D0, double DMAX, double R0) {
  std::memset(s, 0, sizeof *s);
  s->d0 = D0;
  s->dmax = DMAX;
  s->dmax_2 = (s->dmax < std::sqrt(DBL_MAX)) ? s->dmax * s->dmax : DBL_MAX;
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
  s->r0 = R0;
}

// SwitchInterface::setupStretch (SwitchingFunction.cpp:63-72): sigma(0) and
// sigma(d_max) through the non-squared calculate().
void setup_stretch(SwitchParams *s) {
  if (s->dmax < DBL_MAX) {
    s->stretch = 1.0;
    s->shift = 0.0;
    double s0 = sw_calculate<double>(*s, 0.0).f;
    double sd = sw_calculate<double>(*s, s->dmax).f;
    s->stretch = 1.0 / (s0 - sd);
    s->shift = -sd * s->stretch;
    s->stretched = 1;
  }
}

// rational<>::init (SwitchingFunction.cpp:228-252)
void rational_init(SwitchParams *s, double D0, double DMAX, double R0, int N, int M) {
  data_init(s, D0, DMAX, R0);
  s->nn = N;
  s->mm = (M == 0) ? N * 2 : M;
  s->preRes = static_cast<double>(s->nn) / s->mm;
  s->preDfunc = 0.5 * s->nn * (s->nn - s->mm) / static_cast<double>(s->mm);
  s->preSecDev = (s->nn * (s->mm * s->mm - 3.0 * s->mm * (-1 + s->nn) + s->nn * (-3 + 2 * s->nn))) / (6.0 * s->mm);
  s->nnf = s->nn / 2;
  s->mmf = s->mm / 2;
  s->preDfuncF = 0.5 * s->nnf * (s->nnf - s->mmf) / static_cast<double>(s->mmf);
  s->preSecDevF =
      (s->nnf * (s->mmf * s->mmf - 3.0 * s->mmf * (-1 + s->nnf) + s->nnf * (-3 + 2 * s->nnf))) / (6.0 * s->mmf);
}

// rationalFactory (SwitchingFunction.cpp:306-348): the precompiled
// fixedRational<N> for even N<=12 with M==2N (or 0) and D_0==0, else one of
// the four runtime rational forms.
void rational_factory(SwitchParams *s, double D0, double DMAX, double R0, int N, int M) {
  const bool fast = N % 2 == 0 && M % 2 == 0 && D0 == 0.0;
  if (((2 * N) == M || M == 0) && fast && N <= 12 && N >= 2) {
    data_init(s, D0, DMAX, R0);
    s->type = SW_RATFIX;
    s->nn = N;
    s->mm = 2 * N;
    s->nnf = N / 2;
    s->mmf = N;
    return;
  }
  rational_init(s, D0, DMAX, R0, N, M);
  if (2 * N == M || M == 0)
    s->type = fast ? SW_RATIONAL_SIMPLE_FAST : SW_RATIONAL_SIMPLE;
  else
    s->type = fast ? SW_RATIONAL_FAST : SW_RATIONAL;
}

struct Words {
  std::vector<std::string> w;
  // KEY=value; 1 found and parsed, 0 absent, -1 unparsable
  int get_double(const char *key, double *v) {
    const std::string k = std::string(key) + "=";
    for (size_t i = 0; i < w.size(); i++)
      if (w[i].compare(0, k.size(), k) == 0) {
        const char *val = w[i].c_str() + k.size();
        char *end = nullptr;
        double x = std::strtod(val, &end);
        if (end == val || *end) return -1;
        *v = x;
        w.erase(w.begin() + i);
        return 1;
      }
    return 0;
  }
  int get_int(const char *key, int *v) {
    const std::string k = std::string(key) + "=";
    for (size_t i = 0; i < w.size(); i++)
      if (w[i].compare(0, k.size(), k) == 0) {
        const char *val = w[i].c_str() + k.size();
        char *end = nullptr;
        long x = std::strtol(val, &end, 10);
        if (end == val || *end) return -1;
        *v = static_cast<int>(x);
        w.erase(w.begin() + i);
        return 1;
      }
    return 0;
  }
  bool flag(const char *key) {
    for (size_t i = 0; i < w.size(); i++)
      if (w[i] == key) {
        w.erase(w.begin() + i);
        return true;
      }
    return false;
  }
};

Words split(const char *def) {
  Words W;
  std::string cur;
  for (const char *p = def; *p; ++p) {
    const char c = *p;
    if (c == ' ' || c == '\t' || c == '\n' || c == '{' || c == '}') {
      if (!cur.empty()) W.w.push_back(cur);
      cur.clear();
    } else {
      cur.push_back(c);
    }
  }
  if (!cur.empty()) W.w.push_back(cur);
  return W;
}

// Constants of the parameter gradients (see SwitchParams::c_r0).  With the
// stretch set up from a fixed D_MAX, sigma = S*(f(x) - f(xd)), S = 1/(1 -
// f(xd)), xd = (d_max - d0)/r0, so d sigma/dp = S f'(x) dx/dp + S dsd/dp
// (sigma - 1) with dsd/dr0 = -f'(xd) xd/r0 and dsd/dd0 = -f'(xd)/r0.  In the
// R_0= syntax xd is constant (d_max moves with r0 and d0): no second term.
void setup_param_grad(SwitchParams *s) {
  s->c_r0 = 0.0;
  s->c_d0 = 0.0;
  s->grad_ok = !(s->type == SW_CUBIC || s->type == SW_Q);
  if (!s->grad_ok || !s->stretched || s->r0_syntax) return;
  const double xd = (s->dmax - s->d0) * s->invr0;
  if (!(xd > 0.0)) return;
  const double fpd = sw_function<double>(*s, xd).d;
  s->c_r0 = s->stretch * (-fpd * xd * s->invr0);
  s->c_d0 = s->stretch * (-fpd * s->invr0);
}

} // namespace

int switch_from_rational(int nn, int mm, double r0, double d0, SwitchParams *sw) {
  if (mm == 0) mm = 2 * nn;
  const double dmax = d0 + r0 * std::pow(0.00001, 1. / (nn - mm));
  rational_factory(sw, d0, dmax, r0, nn, mm);
  setup_stretch(sw);
  sw->r0 = r0;
  sw->r0_syntax = 1;
  setup_param_grad(sw);
  return 0;
}

int switch_from_string(const char *def, SwitchParams *sw, char *err, int errlen) {
  Words W = split(def);
  std::string e;
  if (W.w.empty()) {
    std::snprintf(err, errlen, "missing all input for switching function");
    return 1;
  }
  const std::string name = W.w[0];
  W.w.erase(W.w.begin());
  double d0 = 0.0, dmax = DBL_MAX;
  if (W.get_double("D_0", &d0) < 0) e = "could not parse D_0";
  if (W.get_double("D_MAX", &dmax) < 0) e = "could not parse D_MAX";
  W.flag("STRETCH");
  const bool dostretch = !W.flag("NOSTRETCH");
  if (name == "CUBIC") {
    data_init(sw, d0, dmax, dmax - d0);
    sw->type = SW_CUBIC;
  } else {
    double r0 = 0.0;
    if (W.get_double("R_0", &r0) != 1) e = "R_0 is required for " + name;
    if (name == "RATIONAL") {
      int nn = 6, mm = 0;
      if (W.get_int("NN", &nn) < 0) e = "could not parse NN";
      if (W.get_int("MM", &mm) < 0) e = "could not parse MM";
      rational_factory(sw, d0, dmax, r0, nn, mm);
    } else if (name == "SMAP") {
      int a = 0, b = 0;
      if (W.get_int("A", &a) != 1) e = "A is required for " + name;
      if (W.get_int("B", &b) != 1) e = "B is required for " + name;
      data_init(sw, d0, dmax, r0);
      sw->type = SW_SMAP;
      sw->a = a;
      sw->b = b;
      if (a != 0 && b != 0) {
        sw->c = std::pow(2., static_cast<double>(a) / static_cast<double>(b)) - 1.0;
        sw->d = -static_cast<double>(b) / static_cast<double>(a);
      }
    } else if (name == "Q") {
      double beta = 50.0, lambda = 1.8, ref = 0.0;
      if (W.get_double("BETA", &beta) < 0) e = "could not parse BETA";
      if (W.get_double("LAMBDA", &lambda) < 0) e = "could not parse LAMBDA";
      if (W.get_double("REF", &ref) != 1) e = "REF is required for " + name;
      data_init(sw, d0, dmax, r0);
      sw->type = SW_Q;
      sw->beta = beta;
      sw->lambda = lambda;
      sw->ref = ref;
    } else if (name == "EXP") {
      data_init(sw, d0, dmax, r0);
      sw->type = SW_EXP;
    } else if (name == "GAUSSIAN") {
      if (r0 == 1.0 && d0 == 0.0) {
        data_init(sw, 0.0, dmax, 1.0);
        sw->type = SW_FASTGAUSSIAN;
      } else {
        data_init(sw, d0, dmax, r0);
        sw->type = SW_GAUSSIAN;
      }
    } else if (name == "TANH") {
      data_init(sw, d0, dmax, r0);
      sw->type = SW_TANH;
    } else if (name == "COSINUS") {
      data_init(sw, d0, dmax, r0);
      sw->type = SW_COSINUS;
    } else if (name == "CUSTOM" || name == "MATHEVAL") {
      std::snprintf(err, errlen, "switching function type '%s' (a lepton expression) is not available on the GPU",
                    name.c_str());
      return 2;
    } else {
      std::snprintf(err, errlen, "cannot understand switching function type '%s'", name.c_str());
      return 1;
    }
  }
  if (!W.w.empty()) {
    e = "found the following rogue keywords in switching function input : ";
    for (auto &x : W.w) e += x + " ";
  }
  if (!e.empty()) {
    std::snprintf(err, errlen, "%s", e.c_str());
    return 1;
  }
  if (dostretch && dmax != DBL_MAX) setup_stretch(sw);
  setup_param_grad(sw);
  return 0;
}

// ---------------------------------------------------------------------------
// Pbc::setBox (Pbc.cpp:165-212) with LatticeReduction::reduceFast
// (LatticeReduction.cpp:139-183) and Pbc::buildShifts (Pbc.cpp:59-135).
// ---------------------------------------------------------------------------
namespace {
double det33(const double *d) {
  return d[0] * d[4] * d[8] + d[1] * d[5] * d[6] + d[2] * d[3] * d[7] - d[0] * d[5] * d[7] -
         d[1] * d[3] * d[8] - d[2] * d[4] * d[6];
}
void inv33(const double *a, double *t) {
  const double invdet = 1.0 / det33(a);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      t[j * 3 + i] = invdet * (a[((i + 1) % 3) * 3 + (j + 1) % 3] * a[((i + 2) % 3) * 3 + (j + 2) % 3] -
                               a[((i + 1) % 3) * 3 + (j + 2) % 3] * a[((i + 2) % 3) * 3 + (j + 1) % 3]);
}
double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
double m2(const double *a) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]; }

struct V3 {
  double v[3];
};

void lr_sort(V3 *v) {
  double m[3] = {m2(v[0].v), m2(v[1].v), m2(v[2].v)};
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++)
      if (m[i] > m[j]) {
        std::swap(v[i], v[j]);
        std::swap(m[i], m[j]);
      }
}
void lr_reduce2(V3 &a, V3 &b) {
  const double onePlusEpsilon = 1.0 + 1e-14;
  double ma = m2(a.v), mb = m2(b.v);
  for (int it = 0; it < 1000000; it++) {
    if (mb > ma) {
      std::swap(a, b);
      std::swap(ma, mb);
    }
    const double f = std::floor(dot3(a.v, b.v) / mb + 0.5);
    for (int k = 0; k < 3; k++) a.v[k] -= b.v[k] * f;
    ma = m2(a.v);
    if (mb <= ma * onePlusEpsilon) break;
  }
  std::swap(a, b);
}
void lr_reduce_fast(double *t) {
  const double onePlusEpsilon = 1.0 + 1e-14;
  V3 v[3];
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) v[i].v[k] = t[i * 3 + k];
  for (int it = 0; it < 1000000; it++) {
    lr_sort(v);
    lr_reduce2(v[0], v[1]);
    const double b11 = m2(v[0].v), b22 = m2(v[1].v);
    const double b12 = dot3(v[0].v, v[1].v), b13 = dot3(v[0].v, v[2].v), b23 = dot3(v[1].v, v[2].v);
    const double z = b11 * b22 - b12 * b12;
    const double y2 = -(b11 * b23 - b12 * b13) / z;
    const double y1 = -(b22 * b13 - b12 * b23) / z;
    const int x1min = static_cast<int>(std::floor(y1)), x2min = static_cast<int>(std::floor(y2));
    bool first = true;
    double mbest = 0.0;
    V3 best{};
    for (int x1 = x1min; x1 <= x1min + 1; x1++)
      for (int x2 = x2min; x2 <= x2min + 1; x2++) {
        V3 trial;
        for (int k = 0; k < 3; k++) trial.v[k] = (v[2].v[k] + x2 * v[1].v[k]) + x1 * v[0].v[k];
        const double mtrial = m2(trial.v);
        if (first || mtrial < mbest) {
          mbest = mtrial;
          best = trial;
          first = false;
        }
      }
    if (m2(best.v) * onePlusEpsilon >= m2(v[2].v)) break;
    v[2] = best;
  }
  lr_sort(v);
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) t[i * 3 + k] = v[i].v[k];
}
void matvec(const double *a, const double *b, double *t) {
  for (int i = 0; i < 3; i++) {
    double s = 0.0;
    for (int j = 0; j < 3; j++) s += a[i * 3 + j] * b[j];
    t[i] = s;
  }
}
void build_shifts(PbcParams *p) {
  const double small = 1e-28;
  double redT[9], rrT[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) redT[i * 3 + j] = p->reduced[j * 3 + i];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s += p->reduced[i * 3 + k] * redT[k * 3 + j];
      rrT[i * 3 + j] = s;
    }
  for (int o = 0; o < 8; o++) p->nshift[o] = 0;
  for (int l = -1; l <= 1; l++)
    for (int m = -1; m <= 1; m++)
      for (int n = -1; n <= 1; n++) {
        const int ishift[3] = {l, m, n};
        const double dshift[3] = {double(l), double(m), double(n)};
        const int count = (l != 0) + (m != 0) + (n != 0);
        if (count == 0 || count == 3) continue;
        double cosdir[3];
        matvec(rrT, dshift, cosdir);
        const double dp = dot3(dshift, cosdir);
        const double ref = m2(dshift) * m2(cosdir);
        if (std::fabs(ref - dp * dp) < small) continue;
        for (int i = 0; i < 2; i++)
          for (int j = 0; j < 2; j++)
            for (int k = 0; k < 2; k++) {
              const int block[3] = {2 * i - 1, 2 * j - 1, 2 * k - 1};
              bool skip = false;
              for (int s = 0; s < 3; s++)
                if (ishift[s] * block[s] > 0) skip = true;
              if (skip) continue;
              skip = true;
              for (int s = 0; s < 3; s++)
                if (((1 - ishift[s] * ishift[s]) * block[s]) * cosdir[s] < -small) skip = false;
              if (skip) continue;
              const int o = 4 * i + 2 * j + k;
              if (p->nshift[o] < 18) {
                matvec(redT, dshift, p->shift[o][p->nshift[o]]);
                p->nshift[o]++;
              }
            }
      }
}
} // namespace

int pbc_setup(const double box[9], PbcParams *p) {
  const double eps = 1e-28;
  std::memset(p, 0, sizeof *p);
  std::memcpy(p->box, box, 9 * sizeof(double));
  p->type = PBC_UNSET;
  const double det = det33(p->box);
  if (det * det < eps) return PBC_UNSET;
  const double *b = p->box;
  const bool cxy = b[1] * b[1] < eps && b[3] * b[3] < eps;
  const bool cxz = b[2] * b[2] < eps && b[6] * b[6] < eps;
  const bool cyz = b[5] * b[5] < eps && b[7] * b[7] < eps;
  inv33(p->box, p->invbox);
  std::memcpy(p->reduced, p->box, sizeof p->reduced);
  if (cxy && cxz && cyz) {
    p->type = PBC_ORTHO;
  } else {
    p->type = PBC_GENERIC;
    lr_reduce_fast(p->reduced);
    build_shifts(p);
  }
  inv33(p->reduced, p->invreduced);
  return p->type;
}

} // namespace coordgpu
