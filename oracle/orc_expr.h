/*
 * orc_expr.h -- CPU restatement of the lepton expressions that PLUMED's
 * CUSTOM (MATHEVAL) switching function evaluates, with their derivative.
 *
 * TEST INFRASTRUCTURE ONLY: part of the oracle (see coord_oracle.h).
 *
 * An expression in one variable (x or x2) is compiled to a postfix program
 * of at most ORC_EXPR_MAX_CODE operations; evaluation runs it on pairs
 * (value, derivative).  Grammar, functions and constants follow
 * src/lepton/Parser.cpp (operators + - * / ^ with precedences 0 0 1 1 3,
 * unary minus at 2, ^ right-associative; Constants() at :85-101) and the
 * derivative rules of src/lepton/Operation.cpp, including the non-smooth
 * ones (step -> delta without the chain factor, abs -> 2 step - 1, min and
 * max through step(a - b), select through its branches).  The reference
 * differentiates symbolically and then simplifies, so the derivative agrees
 * with it to rounding, not bit for bit.
 */
#ifndef ORC_EXPR_H
#define ORC_EXPR_H

#define ORC_EXPR_MAX_CODE 256
#define ORC_EXPR_MAX_CONST 64

typedef struct {
  int ncode;                      /* operations in code */
  int code[ORC_EXPR_MAX_CODE];    /* op | (constant index << 8) */
  int nconst;
  double cst[ORC_EXPR_MAX_CONST];
  int var_x2;                     /* the variable is x2 (else x) */
} orc_expr;

/* Compiles text; returns 0, or 1 with a message in err. */
int orc_expr_compile(orc_expr *e, const char *text, char *err, int errlen);
/* f and df/dvar at var = v. */
void orc_expr_eval(const orc_expr *e, double v, double *f, double *df);

#endif
