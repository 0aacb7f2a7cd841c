/*
 * orc_expr.c -- lepton expressions of the CUSTOM switching function, with
 * their derivative.  TEST INFRASTRUCTURE ONLY (the oracle); see orc_expr.h.
 * Compile with -ffp-contract=off, as coord_oracle.c.
 */
#include "orc_expr.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum {
  OP_VAR, OP_CONST, OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_POW, OP_POWC, OP_NEG,
  /* one argument */
  OP_SQRT, OP_EXP, OP_LOG, OP_SIN, OP_COS, OP_SEC, OP_CSC, OP_TAN, OP_COT, OP_ASIN, OP_ACOS, OP_ATAN,
  OP_SINH, OP_COSH, OP_TANH, OP_ERF, OP_ERFC, OP_STEP, OP_DELTA, OP_SQUARE, OP_CUBE, OP_RECIP, OP_ABS,
  OP_FLOOR, OP_CEIL,
  /* two and three arguments */
  OP_ATAN2, OP_MIN, OP_MAX, OP_SELECT
};

static const struct {
  const char *name;
  int op, nargs;
} kFunctions[] = {  /* Parser::getFunctionOperation (Parser.cpp:355-410), the ones restated here */
    {"sqrt", OP_SQRT, 1},   {"exp", OP_EXP, 1},     {"log", OP_LOG, 1},     {"sin", OP_SIN, 1},
    {"cos", OP_COS, 1},     {"sec", OP_SEC, 1},     {"csc", OP_CSC, 1},     {"tan", OP_TAN, 1},
    {"cot", OP_COT, 1},     {"asin", OP_ASIN, 1},   {"acos", OP_ACOS, 1},   {"atan", OP_ATAN, 1},
    {"atan2", OP_ATAN2, 2}, {"sinh", OP_SINH, 1},   {"cosh", OP_COSH, 1},   {"tanh", OP_TANH, 1},
    {"erf", OP_ERF, 1},     {"erfc", OP_ERFC, 1},   {"step", OP_STEP, 1},   {"delta", OP_DELTA, 1},
    {"square", OP_SQUARE, 1}, {"cube", OP_CUBE, 1}, {"recip", OP_RECIP, 1}, {"min", OP_MIN, 2},
    {"max", OP_MAX, 2},     {"abs", OP_ABS, 1},     {"floor", OP_FLOOR, 1}, {"ceil", OP_CEIL, 1},
    {"select", OP_SELECT, 3}};

/* lepton::Constants() (Parser.cpp:85-101) */
static int named_constant(const char *name, double *v) {
  const double pi = 3.14159265358979323844;
  if (!strcmp(name, "e")) *v = exp(1.0);
  else if (!strcmp(name, "log2e")) *v = 1.0 / log(2.0);
  else if (!strcmp(name, "log10e")) *v = 1.0 / log(10.0);
  else if (!strcmp(name, "ln2")) *v = log(2.0);
  else if (!strcmp(name, "ln10")) *v = log(10.0);
  else if (!strcmp(name, "pi")) *v = pi;
  else if (!strcmp(name, "pi_2")) *v = pi * 0.5;
  else if (!strcmp(name, "pi_4")) *v = pi * 0.25;
  else if (!strcmp(name, "sqrt2")) *v = sqrt(2.0);
  else if (!strcmp(name, "sqrt1_2")) *v = sqrt(0.5);
  else return 0;
  return 1;
}

typedef struct {
  const char *s;
  int pos;
  orc_expr *e;
  char *err;
  int errlen;
  int failed;
  int used_x, used_x2, used_other;
} parser_t;

static void fail(parser_t *p, const char *msg) {
  if (!p->failed) snprintf(p->err, p->errlen, "%s (in '%s' at %d)", msg, p->s, p->pos);
  p->failed = 1;
}

static void emit(parser_t *p, int code) {
  if (p->e->ncode >= ORC_EXPR_MAX_CODE) {
    fail(p, "expression too long");
    return;
  }
  p->e->code[p->e->ncode++] = code;
}

static void emit_const(parser_t *p, double v) {
  if (p->e->nconst >= ORC_EXPR_MAX_CONST) {
    fail(p, "too many constants");
    return;
  }
  p->e->cst[p->e->nconst] = v;
  emit(p, OP_CONST | (p->e->nconst << 8));
  p->e->nconst++;
}

static void skip_space(parser_t *p) {
  while (p->s[p->pos] == ' ' || p->s[p->pos] == '\t') p->pos++;
}

static int parse_prec(parser_t *p, int prec);

/* A number, a variable, a named constant, a call, a parenthesis or a unary
 * minus (Parser::parsePrecedence, Parser.cpp:256-320).  Returns whether the
 * operand depends on the variable. */
static int parse_operand(parser_t *p) {
  skip_space(p);
  const char c = p->s[p->pos];
  if (c == '(') {
    p->pos++;
    const int dep = parse_prec(p, 0);
    skip_space(p);
    if (p->s[p->pos] != ')') fail(p, "unbalanced parentheses");
    else p->pos++;
    return dep;
  }
  if (c == '-') {  /* Negate(parsePrecedence(2)) */
    p->pos++;
    const int dep = parse_prec(p, 2);
    emit(p, OP_NEG);
    return dep;
  }
  if (isdigit((unsigned char)c) || c == '.') {  /* digits, '.', one exponent with its sign */
    const int start = p->pos;
    int found_exp = 0;
    while (1) {
      const char d = p->s[p->pos];
      if (isdigit((unsigned char)d) || d == '.') {
        p->pos++;
      } else if ((d == 'e' || d == 'E') && !found_exp) {
        found_exp = 1;
        p->pos++;
        if (p->s[p->pos] == '+' || p->s[p->pos] == '-') p->pos++;
      } else {
        break;
      }
    }
    char buf[64];
    const int len = p->pos - start;
    if (len >= (int)sizeof buf) {
      fail(p, "number too long");
      return 0;
    }
    memcpy(buf, p->s + start, len);
    buf[len] = 0;
    char *end = NULL;
    const double v = strtod(buf, &end);
    if (end == buf || *end) fail(p, "could not parse a number");
    emit_const(p, v);
    return 0;
  }
  if (isalpha((unsigned char)c) || c == '_') {
    const int start = p->pos;
    while (isalnum((unsigned char)p->s[p->pos]) || p->s[p->pos] == '_') p->pos++;
    char name[64];
    const int len = p->pos - start;
    if (len >= (int)sizeof name) {
      fail(p, "name too long");
      return 0;
    }
    memcpy(name, p->s + start, len);
    name[len] = 0;
    skip_space(p);
    if (p->s[p->pos] == '(') {  /* a call */
      p->pos++;
      int op = -1, nargs = 0;
      for (size_t k = 0; k < sizeof kFunctions / sizeof kFunctions[0]; k++)
        if (!strcmp(kFunctions[k].name, name)) {
          op = kFunctions[k].op;
          nargs = kFunctions[k].nargs;
        }
      if (op < 0) {  /* Parser::getFunctionOperation's message */
        if (!p->failed) snprintf(p->err, p->errlen, "Parse error in expression \"%s\": unknown function: %s", p->s, name);
        p->failed = 1;
        return 0;
      }
      int dep = 0;
      for (int a = 0; a < nargs; a++) {
        if (a > 0) {
          skip_space(p);
          if (p->s[p->pos] != ',') {
            fail(p, "wrong number of arguments");
            return 0;
          }
          p->pos++;
        }
        dep |= parse_prec(p, 0);
      }
      skip_space(p);
      if (p->s[p->pos] != ')') {
        fail(p, "wrong number of arguments");
        return 0;
      }
      p->pos++;
      emit(p, op);
      return dep;
    }
    if (!strcmp(name, "x") || !strcmp(name, "x2")) {
      if (name[1]) p->used_x2 = 1;
      else p->used_x = 1;
      emit(p, OP_VAR);
      return 1;
    }
    double v;
    if (named_constant(name, &v)) {
      emit_const(p, v);
      return 0;
    }
    /* lepton takes any other name as a variable; the switch then refuses it */
    p->used_other = 1;
    emit(p, OP_VAR);
    return 1;
  }
  fail(p, "unexpected character");
  return 0;
}

/* lepton's PowerConstant::evaluate (Operation.h): integer exponents by
 * repeated squaring, others by pow */
static double pow_const(double a, double c) {
  const int ic = (int)c;
  if ((double)ic == c) {
    int n = ic;
    double base = a, r = 1.0;
    if (n < 0) {
      n = -n;
      base = 1.0 / base;
    }
    while (n != 0) {
      if (n & 1) r *= base;
      base *= base;
      n >>= 1;
    }
    return r;
  }
  return pow(a, c);
}

#define ORC_EXPR_STACK 64

/* Runs code[a, b) on (value, derivative) pairs. */
static void run(const orc_expr *e, int a, int b, double var, double *f, double *df) {
  double v[ORC_EXPR_STACK], d[ORC_EXPR_STACK];
  int sp = 0;
  const double two_over_sqrtpi = 2.0 / sqrt(3.14159265358979323844);
  for (int i = a; i < b; i++) {
    const int op = e->code[i] & 0xff, k = e->code[i] >> 8;
    if ((op == OP_VAR || op == OP_CONST) && sp >= ORC_EXPR_STACK) {  /* deeper than the stack: no value */
      *f = *df = NAN;
      return;
    }
    if (op == OP_VAR) {
      v[sp] = var;
      d[sp++] = 1.0;
      continue;
    }
    if (op == OP_CONST) {
      v[sp] = e->cst[k];
      d[sp++] = 0.0;
      continue;
    }
    if (op == OP_SELECT) {  /* select(c, p, q): derivative select(c, p', q') */
      const double c = v[sp - 3];
      const int t = c != 0.0;
      v[sp - 3] = t ? v[sp - 2] : v[sp - 1];
      d[sp - 3] = t ? d[sp - 2] : d[sp - 1];
      sp -= 2;
      continue;
    }
    if (op == OP_ADD || op == OP_SUB || op == OP_MUL || op == OP_DIV || op == OP_POW || op == OP_ATAN2 ||
        op == OP_MIN || op == OP_MAX) {
      const double x = v[sp - 2], dx = d[sp - 2], y = v[sp - 1], dy = d[sp - 1];
      double r = 0.0, dr = 0.0;
      switch (op) {
      case OP_ADD: r = x + y; dr = dx + dy; break;
      case OP_SUB: r = x - y; dr = dx - dy; break;
      case OP_MUL: r = x * y; dr = dx * y + x * dy; break;
      case OP_DIV: r = x / y; dr = dx / y - x * dy / (y * y); break;
      case OP_POW: /* Power::differentiate: y x^(y-1) x' + log(x) x^y y' */
        r = pow(x, y);
        dr = y * pow(x, y - 1.0) * dx + log(x) * r * dy;
        break;
      case OP_ATAN2: r = atan2(x, y); dr = (y * dx - x * dy) / (x * x + y * y); break;
      case OP_MIN: /* std::min; derivative select(step(x - y), y', x') */
        r = (y < x) ? y : x;
        dr = (x - y >= 0.0) ? dy : dx;
        break;
      case OP_MAX: /* std::max; derivative select(step(x - y), x', y') */
        r = (x < y) ? y : x;
        dr = (x - y >= 0.0) ? dx : dy;
        break;
      }
      sp--;
      v[sp - 1] = r;
      d[sp - 1] = dr;
      continue;
    }
    /* one argument */
    const double x = v[sp - 1], dx = d[sp - 1];
    double r = 0.0, dr = 0.0;
    switch (op) {
    case OP_POWC: {
      const double c = e->cst[k];
      r = pow_const(x, c);
      dr = c * pow_const(x, c - 1.0) * dx;
      break;
    }
    case OP_NEG: r = -x; dr = -dx; break;
    case OP_SQRT: r = sqrt(x); dr = 0.5 * (1.0 / r) * dx; break;
    case OP_EXP: r = exp(x); dr = r * dx; break;
    case OP_LOG: r = log(x); dr = (1.0 / x) * dx; break;
    case OP_SIN: r = sin(x); dr = cos(x) * dx; break;
    case OP_COS: r = cos(x); dr = -sin(x) * dx; break;
    case OP_SEC: r = 1.0 / cos(x); dr = r * tan(x) * dx; break;
    case OP_CSC: r = 1.0 / sin(x); dr = -r * (1.0 / tan(x)) * dx; break;
    case OP_TAN: { const double s = 1.0 / cos(x); r = tan(x); dr = s * s * dx; break; }
    case OP_COT: { const double s = 1.0 / sin(x); r = 1.0 / tan(x); dr = -s * s * dx; break; }
    case OP_ASIN: r = asin(x); dr = 1.0 / sqrt(1.0 - x * x) * dx; break;
    case OP_ACOS: r = acos(x); dr = -1.0 / sqrt(1.0 - x * x) * dx; break;
    case OP_ATAN: r = atan(x); dr = 1.0 / (1.0 + x * x) * dx; break;
    case OP_SINH: r = sinh(x); dr = cosh(x) * dx; break;
    case OP_COSH: r = cosh(x); dr = sinh(x) * dx; break;
    case OP_TANH: r = tanh(x); dr = (1.0 - r * r) * dx; break;
    case OP_ERF: r = erf(x); dr = two_over_sqrtpi * exp(-x * x) * dx; break;
    case OP_ERFC: r = erfc(x); dr = -two_over_sqrtpi * exp(-x * x) * dx; break;
    case OP_STEP: /* derivative delta(x), with no chain factor (Operation.cpp) */
      r = (x >= 0.0) ? 1.0 : 0.0;
      dr = (x == 0.0) ? INFINITY : 0.0;
      break;
    case OP_DELTA: r = (x == 0.0) ? INFINITY : 0.0; dr = (x == 0.0) ? NAN : 0.0; break;
    case OP_SQUARE: r = x * x; dr = 2.0 * x * dx; break;
    case OP_CUBE: r = x * x * x; dr = 3.0 * (x * x) * dx; break;
    case OP_RECIP: r = 1.0 / x; dr = -(1.0 / (x * x)) * dx; break;
    case OP_ABS: r = fabs(x); dr = (dx == 0.0) ? 0.0 : dx * (2.0 * ((x >= 0.0) ? 1.0 : 0.0) - 1.0); break;
    case OP_FLOOR: r = floor(x); dr = 0.0; break;
    case OP_CEIL: r = ceil(x); dr = 0.0; break;
    }
    v[sp - 1] = r;
    d[sp - 1] = dr;
  }
  *f = sp ? v[sp - 1] : 0.0;
  *df = sp ? d[sp - 1] : 0.0;
}

static const int kPrec[5] = {0, 0, 1, 1, 3};  /* + - * / ^ (Parser.cpp:82) */

/* Parser::parsePrecedence's operator loop: ^ is right-associative; a
 * constant exponent is folded into one constant (PowerConstant after
 * optimize()). */
static int parse_prec(parser_t *p, int prec) {
  int dep = parse_operand(p);
  while (!p->failed) {
    skip_space(p);
    const char c = p->s[p->pos];
    const int opi = c == '+' ? 0 : c == '-' ? 1 : c == '*' ? 2 : c == '/' ? 3 : c == '^' ? 4 : -1;
    if (opi < 0 || kPrec[opi] < prec) break;
    p->pos++;
    const int rcode = p->e->ncode, rconst = p->e->nconst;
    const int rdep = parse_prec(p, opi == 4 ? kPrec[opi] : kPrec[opi] + 1);
    if (p->failed) break;
    if (opi == 4 && !rdep) {
      double ex, dex;
      run(p->e, rcode, p->e->ncode, 0.0, &ex, &dex);
      p->e->ncode = rcode;
      p->e->nconst = rconst;
      if (p->e->nconst >= ORC_EXPR_MAX_CONST) {
        fail(p, "too many constants");
        break;
      }
      p->e->cst[p->e->nconst] = ex;
      emit(p, OP_POWC | (p->e->nconst << 8));
      p->e->nconst++;
    } else {
      static const int ops[5] = {OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_POW};
      emit(p, ops[opi]);
    }
    dep |= rdep;
  }
  return dep;
}

int orc_expr_compile(orc_expr *e, const char *text, char *err, int errlen) {
  memset(e, 0, sizeof *e);
  parser_t p = {text, 0, e, err, errlen, 0, 0, 0, 0};
  parse_prec(&p, 0);
  skip_space(&p);
  if (!p.failed && p.s[p.pos]) fail(&p, "unexpected characters");
  if (!p.failed && (p.used_other || (p.used_x && p.used_x2))) {
    /* leptonSwitch::funcAndDeriv (SwitchingFunction.cpp:578-584) */
    snprintf(err, errlen,
             "Please declare a function with only ONE argument that can only be x or x2. Your function is: %s", text);
    return 1;
  }
  if (p.failed) return 1;
  /* the evaluation stack stays within ORC_EXPR_STACK */
  int depth = 0, maxd = 0;
  for (int i = 0; i < e->ncode; i++) {
    const int op = e->code[i] & 0xff;
    if (op == OP_VAR || op == OP_CONST) depth++;
    else if (op == OP_SELECT) depth -= 2;
    else if (op == OP_ADD || op == OP_SUB || op == OP_MUL || op == OP_DIV || op == OP_POW || op == OP_ATAN2 ||
             op == OP_MIN || op == OP_MAX)
      depth--;
    if (depth > maxd) maxd = depth;
  }
  if (maxd > ORC_EXPR_STACK) {
    snprintf(err, errlen, "expression too deep");
    return 1;
  }
  e->var_x2 = p.used_x2;
  return 0;
}

void orc_expr_eval(const orc_expr *e, double v, double *f, double *df) { run(e, 0, e->ncode, v, f, df); }
