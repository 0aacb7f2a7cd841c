// ref_harness.cpp -- a C-callable harness around the reference's own classes.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the reference's tool sources (src/tools/{Pbc,LatticeReduction,
// SwitchingFunction,LinkCells,NeighborList,...}.cpp and src/lepton/*.cpp, read
// in place, never copied) into oracle/_ref/libcoord_ref.so.  Tests use it to
// pin the C restatement in coord_oracle.c bit for bit.
//
// The pair loop below follows CoordinationBase::calculate
// (src/colvar/CoordinationBase.cpp:142-231) using the reference's Vector,
// Tensor, Pbc, SwitchingFunction and NeighborList types, so every per-pair
// operation is the reference's own code.
#include "tools/AtomNumber.h"
#include "tools/Communicator.h"
#include "tools/LinkCells.h"
#include "tools/NeighborList.h"
#include "tools/Pbc.h"
#include "tools/SwitchingFunction.h"
#include "tools/Tensor.h"
#include "tools/Vector.h"
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace PLMD;

namespace {
Tensor make_box(const double *b) {
  Tensor t;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) t(i, j) = b[3 * i + j];
  return t;
}

// spec: "R0SYNTAX nn mm r0 d0" selects SwitchingFunction::set(nn,mm,r0,d0)
// (the COORDINATION R_0= syntax); anything else goes to set(string).
int make_switch(const char *spec, SwitchingFunction &sf, char *err, int errlen) {
  std::string s(spec);
  if (s.rfind("R0SYNTAX", 0) == 0) {
    int nn = 6, mm = 0;
    double r0 = 0, d0 = 0;
    if (std::sscanf(spec + 8, "%d %d %lf %lf", &nn, &mm, &r0, &d0) != 4) return 1;
    sf.set(nn, mm, r0, d0);
    return 0;
  }
  std::string e;
  try {
    sf.set(s, e);
  } catch (std::exception &ex) {
    e = ex.what();
  }
  if (!e.empty()) {
    if (err && errlen > 0) {
      std::strncpy(err, e.c_str(), errlen - 1);
      err[errlen - 1] = 0;
    }
    return 1;
  }
  return 0;
}

std::unique_ptr<NeighborList> make_nl(int mode, int64_t n0, int64_t n1, bool do_pbc, const Pbc &pbc,
                                      Communicator &comm, double cutoff, int cells) {
  std::vector<AtomNumber> a(n0), b(n1);
  for (int64_t i = 0; i < n0; i++) a[i] = AtomNumber::index(i);
  for (int64_t i = 0; i < n1; i++) b[i] = AtomNumber::index(n0 + i);
  const bool serial = true;
  if (mode == 0) {
    if (cutoff > 0) return std::make_unique<NeighborList>(a, serial, do_pbc, pbc, comm, cutoff, 1, cells != 0);
    return std::make_unique<NeighborList>(a, serial, do_pbc, pbc, comm);
  }
  const bool dopair = (mode == 2);
  if (cutoff > 0)
    return std::make_unique<NeighborList>(a, b, serial, dopair, do_pbc, pbc, comm, cutoff, 1, cells != 0);
  return std::make_unique<NeighborList>(a, b, serial, dopair, do_pbc, pbc, comm);
}
} // namespace

#define REF_API __attribute__((visibility("default")))
extern "C" {

REF_API int ref_switch_eval(const char *spec, int n, const double *x, int squared, double *f, double *df, char *err,
                    int errlen) {
  SwitchingFunction sf;
  if (make_switch(spec, sf, err, errlen)) return 1;
  for (int i = 0; i < n; i++) {
    double d = 0;
    f[i] = squared ? sf.calculateSqr(x[i], d) : sf.calculate(x[i], d);
    df[i] = d;
  }
  return 0;
}

REF_API int ref_switch_params(const char *spec, double *out7) {
  SwitchingFunction sf;
  char err[256];
  if (make_switch(spec, sf, err, sizeof err)) return 1;
  const auto &d = sf.get_data();
  double v[7] = {d.d0, d.dmax, d.dmax_2, d.invr0, d.invr0_2, d.stretch, d.shift};
  std::memcpy(out7, v, sizeof v);
  return 0;
}

REF_API void ref_pbc(const double *box, int n, const double *v1, const double *v2, double *d, double *invbox) {
  Pbc pbc;
  pbc.setBox(make_box(box));
  for (int i = 0; i < n; i++) {
    Vector a(v1[3 * i], v1[3 * i + 1], v1[3 * i + 2]);
    Vector b(v2[3 * i], v2[3 * i + 1], v2[3 * i + 2]);
    Vector r = pbc.distance(a, b);
    for (int k = 0; k < 3; k++) d[3 * i + k] = r[k];
  }
  if (invbox) {
    const Tensor &ib = pbc.getInvBox();
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) invbox[3 * i + j] = ib(i, j);
  }
}

// LinkCells::setupCells(pbc) at the given cutoff, then addRequiredCells for the
// cell with indices cell[3]: writes the cell limits and the required cells
// (unsorted) and returns their number, or -1 when the reference refuses the
// box.
REF_API int ref_linkcells_required(const double *box, double cutoff, const unsigned *cell, int use_pbc,
                                   unsigned *limits, unsigned *req) {
  Pbc pbc;
  pbc.setBox(make_box(box));
  Communicator comm;
  LinkCells cells(comm);
  cells.setCutoff(cutoff);
  try {
    cells.setupCells(pbc);
  } catch (const std::exception &) {  // the reference's volume assertion: -1
    return -1;
  }
  const auto &lim = cells.getCellLimits();
  for (int k = 0; k < 3; k++) limits[k] = lim[k];
  std::vector<unsigned> r(27);
  unsigned n = 0;
  cells.addRequiredCells({cell[0], cell[1], cell[2]}, n, r, use_pbc != 0);
  for (unsigned i = 0; i < n; i++) req[i] = r[i];
  return (int)n;
}

// NeighborList construction + update(); returns nl.size() and writes the
// pairs (reference order) when cap allows.  cutoff<=0: no NLIST (all pairs).
REF_API int64_t ref_nl(int mode, int64_t n0, int64_t n1, const double *pos, const double *box, int do_pbc, double cutoff,
               int cells, uint32_t *pairs, int64_t cap) {
  Pbc pbc;
  pbc.setBox(make_box(box));
  Communicator comm;
  auto nl = make_nl(mode, n0, n1, do_pbc != 0, pbc, comm, cutoff, cells);
  const int64_t ns = (mode == 0) ? n0 : n0 + n1;
  if (cutoff > 0) {
    std::vector<Vector> p(ns);
    for (int64_t i = 0; i < ns; i++) p[i] = Vector(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    try {
      nl->update(p);
    } catch (const std::exception &) {  // a reference assertion (e.g. a box without volume): -2
      return -2;
    }
  }
  const int64_t n = nl->size();
  for (int64_t i = 0; i < n && i < cap; i++) {
    auto pr = nl->getClosePair(i);
    pairs[2 * i] = pr.first;
    pairs[2 * i + 1] = pr.second;
  }
  return n;
}

// The pair loop of CoordinationBase::calculate over the NeighborList built as
// in CoordinationBase's constructor.  nthreads>1 mirrors the OpenMP split
// with per-thread private derivative/virial copies merged in a critical
// section (CoordinationBase.cpp:172-216).
REF_API int ref_coordination(const char *spec, int mode, int64_t n0, int64_t n1, const int64_t *abs_index, const double *pos,
                     const double *box, int do_pbc, double nl_cutoff, int cells, int nthreads, double *s_out,
                     double *deriv_out, double *virial_out) {
  SwitchingFunction sf;
  char err[256];
  if (make_switch(spec, sf, err, sizeof err)) return 1;
  Pbc pbc;
  pbc.setBox(make_box(box));
  Communicator comm;
  auto nl = make_nl(mode, n0, n1, do_pbc != 0, pbc, comm, nl_cutoff, cells);
  const int64_t ns = (mode == 0) ? n0 : n0 + n1;
  std::vector<Vector> positions(ns);
  for (int64_t i = 0; i < ns; i++) positions[i] = Vector(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
  if (nl_cutoff > 0) nl->update(positions);

  double ncoord = 0.;
  Tensor virial;
  std::vector<Vector> deriv(ns);
  unsigned nt = nthreads < 1 ? 1 : nthreads;
  const unsigned nn = nl->size();
  if (nt * 10 > nn) nt = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
  {
    std::vector<Vector> omp_deriv(nt > 1 ? ns : 0);
    Tensor omp_virial;
#ifdef _OPENMP
#pragma omp for reduction(+ : ncoord) nowait
#endif
    for (unsigned int i = 0; i < nn; ++i) {
      Vector distance;
      const auto [i0, i1] = nl->getClosePair(i);
      if (abs_index[i0] == abs_index[i1]) continue;
      if (do_pbc)
        distance = pbc.distance(positions[i0], positions[i1]);
      else
        distance = delta(positions[i0], positions[i1]);
      double dfunc = 0.;
      ncoord += sf.calculateSqr(distance.modulo2(), dfunc);
      Vector dd(dfunc * distance);
      Tensor vv(dd, distance);
      if (nt > 1) {
        omp_deriv[i0] -= dd;
        omp_deriv[i1] += dd;
        omp_virial -= vv;
      } else {
        deriv[i0] -= dd;
        deriv[i1] += dd;
        virial -= vv;
      }
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    if (nt > 1) {
      for (int64_t i = 0; i < ns; i++) deriv[i] += omp_deriv[i];
      virial += omp_virial;
    }
  }
  *s_out = ncoord;
  for (int64_t i = 0; i < ns; i++)
    for (int k = 0; k < 3; k++) deriv_out[3 * i + k] = deriv[i][k];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) virial_out[3 * i + j] = virial(i, j);
  return 0;
}

REF_API int ref_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
}
