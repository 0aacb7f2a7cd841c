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
  // KEY=text; true when found
  bool get_string(const char *key, std::string *v) {
    const std::string k = std::string(key) + "=";
    for (size_t i = 0; i < w.size(); i++)
      if (w[i].compare(0, k.size(), k) == 0) {
        *v = w[i].substr(k.size());
        w.erase(w.begin() + i);
        return true;
      }
    return false;
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

// Tools::getWords (Tools.cpp:201-270) with its defaults: blanks separate
// words outside braces; a brace that opens or closes the outermost level is
// dropped, inner ones are kept (so FUNC={1 / (1 + x^6)} is one word).
Words split(const char *def) {
  Words W;
  std::string cur;
  int level = 0;
  for (const char *p = def; *p; ++p) {
    const char c = *p;
    if (c == '}') level = std::max(0, level - 1);
    const bool blank = c == ' ' || c == '\t' || c == '\n';
    const bool brace = c == '{' || c == '}';
    if (!(level == 0 && (blank || brace))) cur.push_back(c);
    if (c == '{') level++;
    if (level == 0 && blank && !cur.empty()) {
      W.w.push_back(cur);
      cur.clear();
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
  s->grad_ok = !(s->type == SW_CUBIC || s->type == SW_Q || s->type == SW_CUSTOM);
  if (!s->grad_ok || !s->stretched || s->r0_syntax) return;
  const double xd = (s->dmax - s->d0) * s->invr0;
  if (!(xd > 0.0)) return;
  const double fpd = sw_function<double>(*s, xd).d;
  s->c_r0 = s->stretch * (-fpd * xd * s->invr0);
  s->c_d0 = s->stretch * (-fpd * s->invr0);
}

} // namespace

// ---------------------------------------------------------------------------
// CUSTOM expressions: lepton's grammar (src/lepton/Parser.cpp) parsed into a
// tree, constant subtrees folded to numbers (as ParsedExpression::optimize
// precalculates them; a constant exponent becomes a constant power), then
// emitted as the postfix program that expr_run executes.
// ---------------------------------------------------------------------------
namespace {
struct ExprNode {
  int op;                  // ExprOp
  double c = 0.0;          // EX_CONST value, EX_POWC exponent
  int kid[3] = {-1, -1, -1};
  bool var = false;        // depends on the variable
};

struct ExprParser {
  const std::string src;
  size_t at = 0;
  std::vector<ExprNode> nodes;
  std::string err;
  bool saw_x = false, saw_x2 = false, saw_other = false;

  int add(int op, int a = -1, int b = -1, int c = -1) {
    ExprNode n;
    n.op = op;
    n.kid[0] = a;
    n.kid[1] = b;
    n.kid[2] = c;
    for (int k : n.kid)
      if (k >= 0 && nodes[k].var) n.var = true;
    nodes.push_back(n);
    return (int)nodes.size() - 1;
  }
  int constant(double v) {
    ExprNode n;
    n.op = EX_CONST;
    n.c = v;
    nodes.push_back(n);
    return (int)nodes.size() - 1;
  }
  char peek() {
    while (at < src.size() && (src[at] == ' ' || src[at] == '\t')) at++;
    return at < src.size() ? src[at] : '\0';
  }
  void fail(const std::string &m) {
    if (err.empty()) err = m + " in expression \"" + src + "\"";
  }
  static int function_op(const std::string &name, int *nargs) {
    static const struct {
      const char *name;
      int op, nargs;
    } table[] = {{"sqrt", EX_SQRT, 1},  {"exp", EX_EXP, 1},     {"log", EX_LOG, 1},     {"sin", EX_SIN, 1},
                 {"cos", EX_COS, 1},    {"sec", EX_SEC, 1},     {"csc", EX_CSC, 1},     {"tan", EX_TAN, 1},
                 {"cot", EX_COT, 1},    {"asin", EX_ASIN, 1},   {"acos", EX_ACOS, 1},   {"atan", EX_ATAN, 1},
                 {"atan2", EX_ATAN2, 2}, {"sinh", EX_SINH, 1},  {"cosh", EX_COSH, 1},   {"tanh", EX_TANH, 1},
                 {"erf", EX_ERF, 1},    {"erfc", EX_ERFC, 1},   {"step", EX_STEP, 1},   {"delta", EX_DELTA, 1},
                 {"square", EX_SQUARE, 1}, {"cube", EX_CUBE, 1}, {"recip", EX_RECIP, 1}, {"min", EX_MIN, 2},
                 {"max", EX_MAX, 2},    {"abs", EX_ABS, 1},     {"floor", EX_FLOOR, 1}, {"ceil", EX_CEIL, 1},
                 {"select", EX_SELECT, 3}};
    for (const auto &t : table)
      if (name == t.name) {
        *nargs = t.nargs;
        return t.op;
      }
    return -1;
  }
  // lepton::Constants()
  static bool named(const std::string &n, double *v) {
    const double pi = 3.14159265358979323846;
    if (n == "e") *v = std::exp(1.0);
    else if (n == "log2e") *v = 1.0 / std::log(2.0);
    else if (n == "log10e") *v = 1.0 / std::log(10.0);
    else if (n == "ln2") *v = std::log(2.0);
    else if (n == "ln10") *v = std::log(10.0);
    else if (n == "pi") *v = pi;
    else if (n == "pi_2") *v = pi * 0.5;
    else if (n == "pi_4") *v = pi * 0.25;
    else if (n == "sqrt2") *v = std::sqrt(2.0);
    else if (n == "sqrt1_2") *v = std::sqrt(0.5);
    else return false;
    return true;
  }
  int operand() {
    const char ch = peek();
    if (ch == '(') {
      at++;
      const int e = binary(0);
      if (peek() != ')') fail("unbalanced parentheses");
      else at++;
      return e;
    }
    if (ch == '-') {  // unary minus binds at precedence 2
      at++;
      return add(EX_NEG, binary(2));
    }
    if (std::isdigit((unsigned char)ch) || ch == '.') {
      const size_t start = at;
      bool exp_seen = false;
      while (at < src.size()) {
        const char d = src[at];
        if (std::isdigit((unsigned char)d) || d == '.') {
          at++;
        } else if ((d == 'e' || d == 'E') && !exp_seen) {
          exp_seen = true;
          at++;
          if (at < src.size() && (src[at] == '+' || src[at] == '-')) at++;
        } else {
          break;
        }
      }
      const std::string num = src.substr(start, at - start);
      char *end = nullptr;
      const double v = std::strtod(num.c_str(), &end);
      if (end == num.c_str() || *end) fail("could not parse the number " + num);
      return constant(v);
    }
    if (std::isalpha((unsigned char)ch) || ch == '_') {
      const size_t start = at;
      while (at < src.size() && (std::isalnum((unsigned char)src[at]) || src[at] == '_')) at++;
      const std::string name = src.substr(start, at - start);
      if (peek() == '(') {
        at++;
        int nargs = 0;
        const int op = function_op(name, &nargs);
        if (op < 0) {
          fail("unknown function: " + name);
          return constant(0.0);
        }
        int args[3] = {-1, -1, -1};
        for (int k = 0; k < nargs && err.empty(); k++) {
          if (k > 0) {
            if (peek() != ',') {
              fail("wrong number of arguments to " + name);
              break;
            }
            at++;
          }
          args[k] = binary(0);
        }
        if (peek() != ')') fail("wrong number of arguments to " + name);
        else at++;
        return add(op, args[0], args[1], args[2]);
      }
      double v;
      if (name == "x" || name == "x2") {
        (name == "x" ? saw_x : saw_x2) = true;
      } else if (named(name, &v)) {
        return constant(v);
      } else {
        saw_other = true;  // lepton takes it for a variable; the switch refuses it
      }
      ExprNode n;
      n.op = EX_VAR;
      n.var = true;
      nodes.push_back(n);
      return (int)nodes.size() - 1;
    }
    fail(std::string("unexpected character '") + ch + "'");
    at = src.size();
    return constant(0.0);
  }
  // + - * / ^ at precedences 0 0 1 1 3; ^ groups to the right
  int binary(int prec) {
    int lhs = operand();
    while (err.empty()) {
      const char ch = peek();
      const int op = ch == '+' ? EX_ADD : ch == '-' ? EX_SUB : ch == '*' ? EX_MUL : ch == '/' ? EX_DIV
                                                               : ch == '^' ? EX_POW : -1;
      if (op < 0) break;
      const int p = (op == EX_ADD || op == EX_SUB) ? 0 : (op == EX_POW ? 3 : 1);
      if (p < prec) break;
      at++;
      const int rhs = binary(op == EX_POW ? p : p + 1);
      lhs = add(op, lhs, rhs);
    }
    return lhs;
  }
};

// Postfix code of the subtree at i into prog (folding constant subtrees).
struct ExprEmitter {
  std::vector<ExprNode> &nodes;
  ExprProgram *prog;
  std::string err;
  void put(int op, double c = 0.0) {
    if (prog->n >= kExprMaxOps) {
      err = "expression too long";
      return;
    }
    prog->op[prog->n] = (unsigned char)op;
    prog->cst[prog->n] = c;
    prog->n++;
  }
  // the value of a subtree that does not depend on the variable
  double value_of(int i) {
    ExprProgram tmp{};
    ExprEmitter sub{nodes, &tmp, ""};
    sub.emit(i, false);
    if (!sub.err.empty()) err = sub.err;
    return expr_run(tmp, 0.0).f;
  }
  void emit(int i, bool fold) {
    ExprNode &n = nodes[i];
    if (fold && !n.var && n.op != EX_CONST) {
      put(EX_CONST, value_of(i));
      return;
    }
    if (n.op == EX_POW && fold && !nodes[n.kid[1]].var) {
      emit(n.kid[0], fold);
      put(EX_POWC, value_of(n.kid[1]));
      return;
    }
    for (int k : n.kid)
      if (k >= 0) emit(k, fold);
    put(n.op, n.c);
  }
};
}  // namespace

int expr_compile(const char *text, ExprProgram *prog, char *err, int errlen) {
  std::memset(prog, 0, sizeof *prog);
  ExprParser ps{text ? text : ""};
  int root = -1;
  if (ps.src.find_first_not_of(" \t") == std::string::npos) ps.fail("empty expression");
  else root = ps.binary(0);
  if (ps.err.empty() && ps.peek() != '\0') ps.fail("unexpected characters at the end");
  if (!ps.err.empty()) {
    std::snprintf(err, errlen, "Parse error: %s", ps.err.c_str());
    return 1;
  }
  // leptonSwitch::funcAndDeriv (SwitchingFunction.cpp:566-585)
  if (ps.saw_other || (ps.saw_x && ps.saw_x2)) {
    std::snprintf(err, errlen,
                  "Please declare a function with only ONE argument that can only be x or x2. Your function is: %s",
                  text);
    return 1;
  }
  ExprEmitter em{ps.nodes, prog, ""};
  em.emit(root, true);
  if (!em.err.empty()) {
    std::snprintf(err, errlen, "%s", em.err.c_str());
    return 1;
  }
  // stack depth within what expr_run holds
  int depth = 0, deepest = 0;
  for (int i = 0; i < prog->n; i++) {
    const int op = prog->op[i];
    if (op == EX_VAR || op == EX_CONST) depth++;
    else if (op == EX_SELECT) depth -= 2;
    else if ((op >= EX_ADD && op <= EX_POW) || op >= EX_ATAN2) depth--;
    deepest = std::max(deepest, depth);
  }
  if (deepest > kExprMaxStack) {
    std::snprintf(err, errlen, "expression too deeply nested for the device evaluator");
    return 1;
  }
  prog->var_x2 = ps.saw_x2 ? 1 : 0;
  return 0;
}

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

int switch_from_string(const char *def, SwitchParams *sw, char *err, int errlen, ExprProgram *prog) {
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
      // leptonSwitch (SwitchingFunction.cpp:1138-1141)
      if (!prog) {
        std::snprintf(err, errlen, "switching function type '%s' is not available here", name.c_str());
        return 2;
      }
      std::string func;
      W.get_string("FUNC", &func);
      char msg[512];
      if (expr_compile(func.c_str(), prog, msg, sizeof msg)) {
        std::snprintf(err, errlen, "%s", msg);
        return 1;
      }
      data_init(sw, d0, dmax, r0);
      sw->type = SW_CUSTOM;
      sw->expr_host = prog;
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
