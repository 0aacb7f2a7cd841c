/*
 * coord_oracle.h -- CPU restatement of PLUMED's COORDINATION hot path (FP64).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the GPU results are
 * compared with: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it.  The
 * product (libcoordgpu.so) never links or calls it.
 *
 * Every function restates a reference routine with the same floating-point
 * operation order so that, compiled with -ffp-contract=off, a serial run
 * reproduces the reference bit for bit (pinned against oracle/_ref, the
 * reference sources compiled by oracle/Makefile, and against the reference's
 * regtest golden files in tests/golden/).  Indices are 64-bit where the
 * reference uses 32-bit `unsigned` (src/tools/NeighborList.cpp:147,244-253),
 * so sizes beyond 2^32 pairs are representable here.
 */
#ifndef COORD_ORACLE_H
#define COORD_ORACLE_H
#include <stdint.h>

#include "orc_expr.h"
#ifdef __cplusplus
extern "C" {
#endif

/* ---- periodic boundary conditions: src/tools/Pbc.{h,cpp} ---------------- */
enum { ORC_PBC_UNSET = 0, ORC_PBC_ORTHO = 1, ORC_PBC_GENERIC = 2 };

typedef struct {
  int type;
  double box[9];        /* row-major, row i = lattice vector i */
  double invbox[9];     /* Tensor::inverse (Tensor.h:416-422) */
  double reduced[9];    /* LatticeReduction::reduceFast result (generic only) */
  double invreduced[9];
  int nshift[8];        /* octant (i,j,k) -> 4i+2j+k */
  double shift[8][32][3];
} orc_pbc;

/* Pbc::setBox (Pbc.cpp:165-212).  Returns the detected type. */
int orc_pbc_set(orc_pbc *p, const double box[9]);
/* Pbc::distance(v1,v2) (Pbc.cpp:383-415): min-image of v2-v1. */
void orc_pbc_distance(const orc_pbc *p, const double v1[3], const double v2[3], double d[3]);
/* Tools::pbc (Tools.h:547-571), the round_toward_zero branch. */
double orc_tools_pbc(double x);

/* ---- switching functions: src/tools/SwitchingFunction.cpp ---------------- */
enum {
  ORC_SW_NONE = 0,
  ORC_SW_RATFIX,        /* fixedRational<N>, N stored in nn (SwitchingFunction.cpp:185-216) */
  ORC_SW_RATIONAL,      /* rational<standard,standard> */
  ORC_SW_RATIONAL_FAST, /* rational<fast,standard> */
  ORC_SW_RATIONAL_SIMPLE,      /* rational<standard,simplified> */
  ORC_SW_RATIONAL_SIMPLE_FAST, /* rational<fast,simplified> */
  ORC_SW_EXP, ORC_SW_GAUSSIAN, ORC_SW_FASTGAUSSIAN, ORC_SW_SMAP,
  ORC_SW_CUBIC, ORC_SW_TANH, ORC_SW_COSINUS, ORC_SW_Q,
  ORC_SW_CUSTOM         /* leptonSwitch (SwitchingFunction.cpp:553-760): FUNC of x or x2 */
};

typedef struct {           /* switchContainers::Data (SwitchingFunction.h:57-95) */
  int type;
  double d0, dmax, dmax_2, invr0, invr0_2, stretch, shift;
  int nn, mm;
  double preRes, preDfunc, preSecDev;
  int nnf, mmf;
  double preDfuncF, preSecDevF;
  int a, b;
  double c, d;
  double beta, lambda, ref;
  orc_expr expr;           /* CUSTOM: the compiled FUNC */
} orc_switch;

/* SwitchingFunction::set(string) (SwitchingFunction.cpp:1055-1159).
 * Returns 0 on success, else writes a message to err. */
int orc_switch_set(orc_switch *s, const char *definition, char *err, int errlen);
/* SwitchingFunction::set(nn,mm,r0,d0) (SwitchingFunction.cpp:1176-1184). */
int orc_switch_set_rational(orc_switch *s, int nn, int mm, double r0, double d0);
double orc_switch_calculate(const orc_switch *s, double distance, double *dfunc);
double orc_switch_calculate_sqr(const orc_switch *s, double distance2, double *dfunc);

/* ---- neighbour lists: src/tools/NeighborList.cpp ------------------------ */
enum { ORC_NL_SINGLE = 0, ORC_NL_TWO = 1, ORC_NL_PAIR = 2 };

/* Number of candidate pairs (nallpairs_, NeighborList.cpp:62-97). */
int64_t orc_nl_nallpairs(int mode, int64_t n0, int64_t n1);
/* NeighborList::getIndexPair (NeighborList.cpp:147-166), 64-bit and exact. */
void orc_nl_index_pair(int mode, int64_t n0, int64_t n1, int64_t ipair, int64_t out[2]);
/* All pairs in getIndexPair order (the no-NLIST list). Returns count. */
int64_t orc_nl_all_pairs(int mode, int64_t n0, int64_t n1, uint32_t *pairs, int64_t cap);
/* Classic NLIST update (NeighborList.cpp:237-308), serial order: every
 * candidate in getIndexPair order, kept when modulo2(d) <= cutoff^2.
 * pos holds n0(+n1) slots, AoS.  Returns count (may exceed cap: then only
 * cap pairs are written). */
int64_t orc_nl_classic(int mode, int64_t n0, int64_t n1, const double *pos,
                       const orc_pbc *pbc, int do_pbc, double cutoff,
                       uint32_t *pairs, int64_t cap);
/* Same pair set as orc_nl_classic with the same exact FP64 test, found
 * through a cell grid; pairs are returned sorted by (first, second). */
int64_t orc_nl_classic_cells(int mode, int64_t n0, int64_t n1, const double *pos,
                             const orc_pbc *pbc, int do_pbc, double cutoff,
                             uint32_t *pairs, int64_t cap);
/* NLISTCELLS update (NeighborList.cpp:177-236 with LinkCells.cpp:99-292):
 * every pair in neighbouring link cells, no distance test. Reference order. */
int64_t orc_nl_linkcells(int mode, int64_t n0, int64_t n1, const double *pos,
                         const orc_pbc *pbc, int do_pbc, double cutoff,
                         uint32_t *pairs, int64_t cap);
/* LinkCells::createCells cell counts for a pbc box (LinkCells.cpp:99-122). */
void orc_linkcells_ncells(const orc_pbc *pbc, double cutoff, int ncells[3]);
/* LinkCells::addRequiredCells (LinkCells.cpp:195-240): the cells searched
 * from the cell with indices cell[3], with or without PBC; returns their
 * number (at most 27) and writes them, unsorted, to req. */
int orc_linkcells_required(const orc_pbc *pbc, double cutoff, const int cell[3], int use_pbc, int *req);

/* ---- the CV: CoordinationBase::calculate (CoordinationBase.cpp:142-231) -- */
/* Loops over npairs (first,second) slot pairs, skipping pairs whose absolute
 * atom indices are equal; writes s, deriv (nslots x 3, AoS) and the 3x3
 * virial.  nthreads<=1 is the serial order; >1 mirrors the OpenMP split with
 * per-thread private accumulators merged at the end. */
int orc_coordination(const orc_switch *sw, const orc_pbc *pbc, int do_pbc,
                     int64_t nslots, const int64_t *abs_index, const double *pos,
                     const uint32_t *pairs, int64_t npairs,
                     double *s, double *deriv, double virial[9], int nthreads);

/* ---- sibling CVs of CoordinationBase: the same loop, another pairing() --- */
enum { ORC_CV_COORDINATION = 0, ORC_CV_DHENERGY = 1, ORC_CV_GHBFIX = 2 };

typedef struct {
  int kind;                 /* ORC_CV_* */
  const orc_switch *sw;     /* COORDINATION: Coordination::pairing (Coordination.cpp:159-163) */
  /* DHENERGY (DHEnergy.cpp:104-142) */
  double dh_k, dh_constant, dh_epsilon;
  const double *charge;     /* per slot */
  /* GHBFIX (GHBFIX.cpp:111-218) */
  double gh_dmax_sq, gh_d0, gh_c_dmax2, gh_A, gh_B, gh_C, gh_D;
  int gh_ntypes;
  const int *type;          /* per slot: index into the types table */
  const double *eta;        /* gh_ntypes x gh_ntypes, eta[n*t1+t2] */
} orc_pairing;

/* DHEnergy::DHEnergy (DHEnergy.cpp:112-113): screening constant k and
 * prefactor from I, TEMP, EPSILON and the energy/length/charge units. */
void orc_dhenergy_constants(double ionic, double temp, double epsilon, double unit_energy, double unit_length,
                            double unit_charge, double *k, double *constant);
/* GHBFIX::GHBFIX (GHBFIX.cpp:111-126): dmax^2, c*(dmax-d0), A, B, C, D. */
void orc_ghbfix_constants(orc_pairing *p, double d0, double dmax, double c);
/* One pairing(distance2, dfunc, i, j) of the pairing's kind, slots i, j. */
double orc_pairing_eval(const orc_pairing *p, double distance2, double *dfunc, int64_t i, int64_t j);
/* CoordinationBase::calculate with any pairing (as orc_coordination). */
int orc_cv(const orc_pairing *pr, const orc_pbc *pbc, int do_pbc, int64_t nslots, const int64_t *abs_index,
           const double *pos, const uint32_t *pairs, int64_t npairs, double *s, double *deriv, double virial[9],
           int nthreads);

/* ---- per-atom coordination ------------------------------------------------
 * COORDINATIONNUMBER (symfunc/CoordinationNumbers.cpp:268-309): the weights
 * of CONTACT_MATRIX (adjmat/ContactMatrix.h:95-120) summed per atom over the
 * given pairs, i.e. times a vector of ones.  A pair with r^2 < DBL_EPSILON or
 * sigma < DBL_EPSILON has no weight and no derivative.  cn[slot] gets sigma
 * from both atoms' sides.  With g (dV/dcn per slot) non-NULL, grad (nslots x
 * 3) and virial receive the vector-Jacobian product: each pair's derivative
 * weighted by g[i] + g[j]. */
int orc_peratom(const orc_switch *sw, const orc_pbc *pbc, int do_pbc, int64_t nslots, const int64_t *abs_index,
                const double *pos, const uint32_t *pairs, int64_t npairs, const double *g, double *cn, double *grad,
                double virial[9]);

/* ---- CONTACTMAP (colvar/ContactMap.cpp:149-365) ----------------------------
 * n contacts (first, second) = slots (i, n + i); contact i uses switch
 * sw[nsw == 1 ? 0 : i], reference[i], weight[i]:
 *   c_i = weight_i * (sigma_i(|d|) - reference_i)   (SwitchingFunction::calculate)
 * mode 0 (components): value[i] = c_i, vir[9 i..] = -tmpvir of contact i;
 * mode 1 (SUM): value[0] = sum c_i; mode 2 (CMDIST): value[0] = sum c_i^2
 * (derivatives times 2 c_i).  deriv is (2n x 3): -/+ tmpder for the two slots;
 * vir is 9 values per contact (mode 0) or 9 in total. */
int orc_contactmap(const orc_switch *sw, int nsw, int64_t n, const double *reference, const double *weight, int mode,
                   const orc_pbc *pbc, int do_pbc, const double *pos, double *value, double *deriv, double *vir);

/* Number of OpenMP threads available (1 without OpenMP). */
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
