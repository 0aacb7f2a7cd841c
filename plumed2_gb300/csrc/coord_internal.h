// coord_internal.h -- types shared by the host runtime and the sm_103a kernels.
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace coordgpu {

// ---------------------------------------------------------------------------
// Switching functions.  One struct carries every switch type's parameters,
// laid out like switchContainers::Data (SwitchingFunction.h:57-95) so the
// host set-up can follow SwitchingFunction::set() step by step.
// ---------------------------------------------------------------------------
enum SwitchType : int {
  SW_NONE = 0,
  SW_RATFIX,               // fixedRational<N>   (SwitchingFunction.cpp:185-216), N in nn
  SW_RATIONAL,             // rational<standard, standard>
  SW_RATIONAL_FAST,        // rational<fast, standard>
  SW_RATIONAL_SIMPLE,      // rational<standard, simplified>
  SW_RATIONAL_SIMPLE_FAST, // rational<fast, simplified>
  SW_EXP,
  SW_GAUSSIAN,
  SW_FASTGAUSSIAN,
  SW_SMAP,
  SW_CUBIC,
  SW_TANH,
  SW_COSINUS,
  SW_Q,
  SW_CUSTOM                // leptonSwitch (SwitchingFunction.cpp:553-760): an expression of x or x2
};

// A CUSTOM switching function's expression (lepton syntax, one variable: x or
// x2) as a postfix program run on (value, derivative) pairs: host_setup.cpp
// compiles it (expr_compile), switch_eval.cuh runs it (expr_run).
enum ExprOp : unsigned char {
  EX_VAR, EX_CONST, EX_ADD, EX_SUB, EX_MUL, EX_DIV, EX_POW, EX_POWC, EX_NEG,
  EX_SQRT, EX_EXP, EX_LOG, EX_SIN, EX_COS, EX_SEC, EX_CSC, EX_TAN, EX_COT, EX_ASIN, EX_ACOS, EX_ATAN,
  EX_SINH, EX_COSH, EX_TANH, EX_ERF, EX_ERFC, EX_STEP, EX_DELTA, EX_SQUARE, EX_CUBE, EX_RECIP, EX_ABS,
  EX_FLOOR, EX_CEIL, EX_ATAN2, EX_MIN, EX_MAX, EX_SELECT
};
constexpr int kExprMaxOps = 160;
constexpr int kExprMaxStack = 24;
struct ExprProgram {
  int n;                      // operations
  int var_x2;                 // the variable is x2 (else x)
  unsigned char op[kExprMaxOps];
  double cst[kExprMaxOps];    // the value of EX_CONST, the exponent of EX_POWC
};

struct SwitchParams {
  int type;
  int nn, mm, nnf, mmf;
  int a, b;
  double d0, dmax, dmax_2, invr0, invr0_2, stretch, shift;
  double preRes, preDfunc, preSecDev, preDfuncF, preSecDevF;
  double c, d;
  double beta, lambda, ref;
  double r0;               // 1/invr0 as given (for parameter gradients)
  int r0_syntax;           // set(nn,mm,r0,d0): d_max depends on R_0 and D_0
  int stretched;           // stretch/shift were set up
  // parameter gradients: dsigma/dp = (first term) + c_p * (sigma - 1) for a
  // pair inside d_max, c_p = stretch * d sigma_raw(d_max)/dp (zero when the
  // stretch constants do not depend on p); grad_ok = 0 for types whose
  // R_0/D_0 do not enter as (r - d0)/r0 (CUBIC, Q).
  double c_r0, c_d0;
  int grad_ok;
  // SW_CUSTOM: the compiled expression, host and device copies (owned by the
  // context that parsed the switch)
  const ExprProgram *expr_host;
  const ExprProgram *expr_dev;
};

// Parses SWITCH={...} (SwitchingFunction::set(string), SwitchingFunction.cpp:
// 1055-1159).  Returns 0 or writes a message into err (2: valid input the
// caller cannot take -- a CUSTOM function when prog is null).  A CUSTOM
// function is compiled into *prog, which sw->expr_host points to.
int switch_from_string(const char *def, SwitchParams *sw, char *err, int errlen, ExprProgram *prog = nullptr);
// Compiles a lepton expression of x or x2; 0, or 1 with a message.
int expr_compile(const char *text, ExprProgram *prog, char *err, int errlen);
// The R_0/NN/MM/D_0 form (SwitchingFunction::set(nn,mm,r0,d0), :1176-1184).
int switch_from_rational(int nn, int mm, double r0, double d0, SwitchParams *sw);
// Host-side evaluation (same code as the device FP64 evaluator).
double switch_host_calculate(const SwitchParams &sw, double distance, double *dfunc);
double switch_host_calculate_sqr(const SwitchParams &sw, double distance2, double *dfunc);

// ---------------------------------------------------------------------------
// Periodic boundary conditions (Pbc::setBox, Pbc.cpp:165-212).
// ---------------------------------------------------------------------------
enum PbcType : int { PBC_UNSET = 0, PBC_ORTHO = 1, PBC_GENERIC = 2 };

struct PbcParams {
  int type;
  int nshift[8];
  double box[9], invbox[9], reduced[9], invreduced[9];
  double shift[8][18][3];
};
int pbc_setup(const double box[9], PbcParams *p);

// ---------------------------------------------------------------------------
// Neighbour-list geometry for one frame (computed on the host from the box).
// ---------------------------------------------------------------------------
struct GridParams {
  int nc[3];          // cells per dimension
  int ncells;
  int wrap;           // 1: periodic cell indices
  int use_scaled;     // bin on scaled coordinates (box given)
  double lo[3];       // no-pbc bounding-box origin (device-computed when 0 box)
  double inv_width[3];
};

// Per-frame constants read by the kernels (one record per frame on device).
struct FrameConst {
  PbcParams pbc;
  GridParams grid;
  double cut2;        // NL_CUTOFF^2 (classic test, NeighborList.cpp:238)
  float  cut2_lo, cut2_hi; // FP32 prefilter band around cut2
  // fixed-point frame of the mixed path: q = frac((x - grid.lo) * inv_l) * 2^32
  double inv_l[3];
  float  scale[3];    // L / 2^32 per axis (FP32)
  int    fixed_ok;    // box is orthorhombic (or none) so fixed point applies
  // orthorhombic box with d_max below 0.45 of every side: for a pair within
  // d_max the reference's image shift round(d / L) is the integer difference
  // of the two atoms' 64-bit fixed-point positions (k_eval_nl64q)
  int    shift_ok;
  // the same q in one FMA: q = rn(x * fx_s + fx_c) mod 2^32 with
  // fx_s = inv_l * 2^32 and fx_c = -grid.lo * fx_s (fixed_frame_finish)
  double fx_s[3], fx_c[3];
  // the same q in integer arithmetic (fixed_v64): inv_l as mantissa and
  // biased exponent, and (-grid.lo * inv_l * 2^64) mod 2^64
  unsigned long long fxi_m[3], fxi_c[3];
  int fxi_e[3];
  // generic (triclinic) periodic box on the mixed path: q holds the
  // fractional coordinates in the reduced lattice, component i =
  // frac(sum_j x_j invReduced(j,i)) * 2^32 (fx_m = invReduced * 2^32), so
  // the wrapped difference of two q is Pbc::distance's Tools::pbc of the
  // scaled distance; red32 = reduced / 2^32 takes it back to Cartesian in
  // FP32 (Pbc.cpp:383-415)
  int    tric;
  double fx_m[9];
  float  red32[9];
};

#ifdef __CUDACC__
#define COORD_HD __host__ __device__
#else
#define COORD_HD
#endif
// Fixed point in integer arithmetic: (x * S * 2^64) mod 2^64 for a double x
// and a positive scale S = sm * 2^(se - 1075) (its 53-bit mantissa with the
// implicit bit, and its biased exponent).  The two mantissas' exact 106-bit
// product is shifted into place and truncated toward zero, then signed; the
// error is below one unit of 2^-64.  No FP64 instruction: the O(N) kernels
// that convert positions every step are bound by the FP64 pipe otherwise.
COORD_HD inline unsigned long long fx_bits(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long u;
  std::memcpy(&u, &x, sizeof u);
  return u;
#endif
}
// The 106-bit product of two 53-bit integers as (hi, lo) 64-bit words, from
// four 32 x 32 -> 64-bit multiplies (cheaper on the device than the generic
// 64-bit multiply and high-word multiply).
COORD_HD inline void fx_mul53(unsigned long long a, unsigned long long b, unsigned long long &lo,
                              unsigned long long &hi) {
  const unsigned long long a0 = (uint32_t)a, a1 = a >> 32, b0 = (uint32_t)b, b1 = b >> 32;
  const unsigned long long p00 = a0 * b0, mid = a0 * b1 + a1 * b0;  // mid < 2^54
  lo = p00 + (mid << 32);
  hi = a1 * b1 + (mid >> 32) + (lo < p00 ? 1ull : 0ull);
}
COORD_HD inline unsigned long long fixed_v64(double x, unsigned long long sm, int se) {
  const unsigned long long b = fx_bits(x);
  const int e = (int)((b >> 52) & 0x7ffu);
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0ull);
  unsigned long long lo, hi;
  fx_mul53(m, sm, lo, hi);
  const int sh = (e ? e : 1) + se - 2086;  // x S 2^64 = (m sm) 2^sh
  unsigned long long v;
  if (sh >= 0)
    v = sh >= 64 ? 0ull : lo << sh;
  else if (sh > -64)
    v = (lo >> -sh) | (hi << (64 + sh));
  else
    v = sh > -128 ? hi >> (-sh - 64) : 0ull;
  return (b >> 63) ? 0ull - v : v;
}

// Fills the constants of the fixed-point frame from inv_l and grid.lo: the
// one-FMA form and the integer form.
COORD_HD inline void fixed_frame_finish(FrameConst &fc) {
  for (int k = 0; k < 3; k++) {
    fc.fx_s[k] = fc.inv_l[k] * 4294967296.0;
    fc.fx_c[k] = -(fc.grid.lo[k] * fc.fx_s[k]);
    const unsigned long long sb = fx_bits(fc.inv_l[k]);
    const bool ok = fc.inv_l[k] > 0.0 && ((sb >> 52) & 0x7ffu) != 0;
    fc.fxi_e[k] = ok ? (int)((sb >> 52) & 0x7ffu) : 0;
    fc.fxi_m[k] = ok ? ((sb & 0xFFFFFFFFFFFFFull) | (1ull << 52)) : 0ull;
    fc.fxi_c[k] = fixed_v64(-fc.grid.lo[k], fc.fxi_m[k], fc.fxi_e[k]);
  }
}

// Pair modes (NeighborList::NNStyle, NeighborList.h:39).
enum PairMode : int { MODE_SINGLE = 0, MODE_TWO = 1, MODE_PAIR = 2 };

} // namespace coordgpu
