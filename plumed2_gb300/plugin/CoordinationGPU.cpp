// CoordinationGPU.cpp -- PLUMED plugin: COORDINATION and its CoordinationBase
// siblings DHENERGY and GHBFIX on the GPU through libcoordgpu.so
// (include/coordgpu.h).
//
// Build against an installed PLUMED and load it with LOAD (src/setup/Load.cpp):
//
//   g++ -std=c++17 -O2 -fPIC -shared CoordinationGPU.cpp -o CoordinationGPU.so
//       -I$PLUMED_PREFIX/include/plumed -I<repo>/include
//       -L<repo>/plumed2_gb300/_build -lcoordgpu -Wl,-rpath,<repo>/plumed2_gb300/_build
//   (one command line)
//
//   LOAD FILE=CoordinationGPU.so
//   c: COORDINATION GROUPA=1-1000 SWITCH={RATIONAL R_0=0.3 D_MAX=1.0}
//
// After LOAD the directives COORDINATION, DHENERGY and GHBFIX resolve to the
// classes below (the registry searches the most recently loaded images first,
// RegisterBase.h:239-253); the *_GPU names are second names so that the
// built-in and these actions can run side by side on one input.
//
// The action keeps the reference's keyword surface and per-step contract:
//   keywords    CoordinationBase::registerKeywords (CoordinationBase.cpp:30-40)
//               and Coordination::registerKeywords (Coordination.cpp:115-126),
//               plus PRECISION=FP64|MIXED and DEVICE=n
//   errors      the same checks and messages (CoordinationBase.cpp:66-84,
//               Coordination.cpp:140-148), raised with Action::error
//   requests    NeighborList::prepare (NeighborList.cpp:433-456): the full
//               list on rebuild steps, the atoms of the list otherwise
//   outputs     setValue, setAtomsDerivatives per requested atom,
//               setBoxDerivatives (CoordinationBase.cpp:226-230)
#include "core/ActionRegister.h"
#include "core/Colvar.h"
#include "tools/IFile.h"
#include "tools/Pbc.h"
#include "tools/Tensor.h"
#include "tools/Units.h"
#include "tools/Vector.h"

#include "coordgpu.h"

#include <algorithm>
#include <map>
#include <string>
#include <vector>

namespace PLMD {
namespace coordgpu_plugin {

// CoordinationBase on the GPU: the groups, PAIR/NLIST/NLISTCELLS/NOPBC
// keywords, the neighbour-list request cycle and the outputs.  A derived
// action parses its own keywords, then calls create().
class PairLoopGPU : public Colvar {
protected:
  coord_ctx *ctx = nullptr;
  coord_params p{};
  std::vector<AtomNumber> ga, gb;
  std::vector<AtomNumber> full;          // GROUPA then GROUPB (slots)
  std::vector<AtomNumber> reduced;       // sorted unique atoms of the neighbour list
  std::vector<int> slot_to_reduced;      // slot -> index in reduced (-1: not in the list)
  std::vector<double> pos_slots, deriv_slots;
  bool firsttime = true;
  bool invalidateList = true;
  int nl_stride = 0;
  bool pbc = true;
  std::string prec = "FP64";
  void check(int rc, const char *what);
  void build_reduced_list();
  void create(const char *what);
  // per-atom data of the requested atoms, on steps that request every atom
  virtual void before_forward() {}

public:
  explicit PairLoopGPU(const ActionOptions &);
  ~PairLoopGPU() override;
  static void registerKeywords(Keywords &keys);
  void prepare() override;
  void calculate() override;
};

class CoordinationGPU : public PairLoopGPU {
public:
  explicit CoordinationGPU(const ActionOptions &);
  static void registerKeywords(Keywords &keys);
};

PLUMED_REGISTER_ACTION(CoordinationGPU, "COORDINATION")
PLUMED_REGISTER_ACTION(CoordinationGPU, "COORDINATION_GPU")

// CoordinationBase::registerKeywords (CoordinationBase.cpp:30-40)
void PairLoopGPU::registerKeywords(Keywords &keys) {
  Colvar::registerKeywords(keys);
  keys.addFlag("SERIAL", false, "Perform the calculation in serial - for debug purpose");
  keys.addFlag("PAIR", false, "Pair only 1st element of the 1st group with 1st element in the second, etc");
  keys.addFlag("NLIST", false, "Use a neighbor list to speed up the calculation");
  keys.addFlag("NLISTCELLS", false, "Use a neighbor list built from link cells (every pair of neighbouring cells)");
  keys.add("optional", "NL_CUTOFF", "The cutoff for the neighbor list");
  keys.add("optional", "NL_STRIDE", "The frequency with which we are updating the atoms in the neighbor list");
  keys.add("atoms", "GROUPA", "First list of atoms");
  keys.add("atoms", "GROUPB", "Second list of atoms (if empty, N*(N-1)/2 pairs in GROUPA are counted)");
  keys.add("compulsory", "DEVICE", "0", "CUDA device");
}

// Coordination::registerKeywords (Coordination.cpp:115-126)
void CoordinationGPU::registerKeywords(Keywords &keys) {
  PairLoopGPU::registerKeywords(keys);
  keys.add("compulsory", "NN", "6", "The n parameter of the switching function ");
  keys.add("compulsory", "MM", "0", "The m parameter of the switching function; 0 implies 2*NN");
  keys.add("compulsory", "D_0", "0.0", "The d_0 parameter of the switching function");
  keys.add("compulsory", "R_0", "The r_0 parameter of the switching function");
  keys.add("optional", "SWITCH", "An alternative switching function (RATIONAL, EXP, GAUSSIAN, SMAP, CUBIC, TANH, COSINUS, Q)");
  keys.add("compulsory", "PRECISION", "FP64", "FP64 (the drop-in arithmetic) or MIXED (FP32 pairs, FP64 sums)");
  keys.setValueDescription("scalar", "the value of the coordination");
}

void PairLoopGPU::check(int rc, const char *what) {
  if (rc != COORD_OK) error(std::string(what) + ": " + coord_last_error(ctx));
}

// CoordinationBase::CoordinationBase (CoordinationBase.cpp:42-131), the
// keywords common to the three actions
PairLoopGPU::PairLoopGPU(const ActionOptions &ao) : PLUMED_COLVAR_INIT(ao) {
  bool serial = false;
  parseFlag("SERIAL", serial);
  parseAtomList("GROUPA", ga);
  parseAtomList("GROUPB", gb);
  bool nopbc = !pbc;
  parseFlag("NOPBC", nopbc);
  pbc = !nopbc;
  bool dopair = false;
  parseFlag("PAIR", dopair);
  bool nl_classic = false, nl_cells = false;
  parseFlag("NLIST", nl_classic);
  parseFlag("NLISTCELLS", nl_cells);
  if (nl_cells && nl_classic) error("Please activate only one of the two version of the NL");
  double nl_cut = 0.0;
  if (nl_cells || nl_classic) {
    parse("NL_CUTOFF", nl_cut);
    parse("NL_STRIDE", nl_stride);
  }
  coord_params_default(&p);
  parse("DEVICE", p.device);
  p.nopbc = nopbc;
  p.pair = dopair;
  p.serial = serial;
  p.nlist = nl_classic ? COORD_NL_CLASSIC : (nl_cells ? COORD_NL_CELLS : COORD_NL_NONE);
  p.nl_cutoff = nl_cut;
  p.nl_stride = nl_stride;
}

// The library context for the parsed keywords (p), the groups, the requests.
void PairLoopGPU::create(const char *what) {
  p.precision = (prec == "MIXED") ? COORD_PREC_MIXED : COORD_PREC_FP64;
  const int rc = coord_create(&p, &ctx);
  if (rc != COORD_OK) error(coord_last_error(ctx));
  full = ga;
  full.insert(full.end(), gb.begin(), gb.end());
  std::vector<int64_t> a(ga.size()), b(gb.size());
  for (size_t i = 0; i < ga.size(); i++) a[i] = ga[i].index();
  for (size_t i = 0; i < gb.size(); i++) b[i] = gb[i].index();
  check(coord_set_groups(ctx, a.data(), (int64_t)a.size(), b.data(), (int64_t)b.size()), what);
  pos_slots.assign(3 * full.size(), 0.0);
  deriv_slots.assign(3 * full.size(), 0.0);
  addValueWithDerivatives();
  setNotPeriodic();
  requestAtoms(full);
  log.printf("  between two groups of %u and %u atoms, on CUDA device %d (%s)\n", (unsigned)ga.size(),
             (unsigned)gb.size(), p.device, prec.c_str());
}

PairLoopGPU::~PairLoopGPU() { coord_destroy(ctx); }

// Coordination::Coordination (Coordination.cpp:128-157)
CoordinationGPU::CoordinationGPU(const ActionOptions &ao) : Action(ao), PairLoopGPU(ao) {
  std::string sw;
  parse("SWITCH", sw);
  if (sw.empty()) {
    parse("R_0", p.r0);
    parse("D_0", p.d0);
    parse("NN", p.nn);
    parse("MM", p.mm);
  }
  parse("PRECISION", prec);
  checkRead();
  p.switch_def = sw.empty() ? nullptr : sw.c_str();
  create("COORDINATION");
  p.switch_def = nullptr;
}

// NeighborList::prepare (NeighborList.cpp:433-456)
void PairLoopGPU::prepare() {
  if (nl_stride > 0) {
    if (nl_stride == 1) {
      invalidateList = true;
      firsttime = false;
    } else if (firsttime || (getStep() % nl_stride == 0)) {
      requestAtoms(full);
      invalidateList = true;
      firsttime = false;
    } else {
      requestAtoms(reduced);
      invalidateList = false;
      if (getExchangeStep())
        error("Neighbor lists should be updated on exchange steps - choose a NL_STRIDE which divides the exchange stride!");
    }
    if (getExchangeStep()) firsttime = true;
  }
}

// The atoms the next non-rebuild steps request (NeighborList::setRequestList,
// NeighborList.cpp:317-328), from the pair set of the rebuild.
void PairLoopGPU::build_reduced_list() {
  int64_t n = 0;
  check(coord_get_pairs(ctx, 0, nullptr, 0, &n), getName().c_str());
  std::vector<uint32_t> pairs(2 * std::max<int64_t>(n, 1));
  check(coord_get_pairs(ctx, 0, pairs.data(), n, &n), getName().c_str());
  reduced.clear();
  for (int64_t i = 0; i < 2 * n; i++) reduced.push_back(full[pairs[i]]);
  std::sort(reduced.begin(), reduced.end());
  reduced.erase(std::unique(reduced.begin(), reduced.end()), reduced.end());
  slot_to_reduced.assign(full.size(), -1);
  for (size_t s = 0; s < full.size(); s++) {
    auto it = std::lower_bound(reduced.begin(), reduced.end(), full[s]);
    if (it != reduced.end() && *it == full[s]) slot_to_reduced[s] = (int)(it - reduced.begin());
  }
}

void PairLoopGPU::calculate() {
  const auto &positions = getPositions();
  const bool full_request = (nl_stride <= 1) || invalidateList;
  if (full_request) before_forward();
  if (full_request) {
    for (size_t s = 0; s < full.size(); s++)
      for (int k = 0; k < 3; k++) pos_slots[3 * s + k] = positions[s][k];
  } else {
    for (size_t s = 0; s < full.size(); s++)
      if (slot_to_reduced[s] >= 0)
        for (int k = 0; k < 3; k++) pos_slots[3 * s + k] = positions[slot_to_reduced[s]][k];
  }
  double box[9];
  const Tensor &b = getPbc().getBox();
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) box[3 * i + j] = b(i, j);
  const unsigned flags = (nl_stride > 0 && invalidateList) ? COORD_FLAG_REBUILD : 0u;
  double s = 0.0, virial[9];
  // the step passed never triggers the library's own stride rule: prepare() decides
  check(coord_forward(ctx, pos_slots.data(), box, 1, flags, &s, deriv_slots.data(), virial), getName().c_str());
  if (nl_stride > 1 && invalidateList) build_reduced_list();
  if (full_request) {
    for (size_t i = 0; i < full.size(); i++)
      setAtomsDerivatives(i, Vector(deriv_slots[3 * i], deriv_slots[3 * i + 1], deriv_slots[3 * i + 2]));
  } else {
    std::vector<Vector> d(reduced.size());
    for (size_t s2 = 0; s2 < full.size(); s2++)
      if (slot_to_reduced[s2] >= 0)
        d[slot_to_reduced[s2]] += Vector(deriv_slots[3 * s2], deriv_slots[3 * s2 + 1], deriv_slots[3 * s2 + 2]);
    for (size_t i = 0; i < reduced.size(); i++) setAtomsDerivatives(i, d[i]);
  }
  setValue(s);
  Tensor v;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) v(i, j) = virial[3 * i + j];
  setBoxDerivatives(v);
}

// ---- DHENERGY (colvar/DHEnergy.cpp:62) -------------------------------------
class DHEnergyGPU : public PairLoopGPU {
  std::vector<double> charges;  // by absolute atom index
  void before_forward() override;

public:
  explicit DHEnergyGPU(const ActionOptions &);
  static void registerKeywords(Keywords &keys);
};

PLUMED_REGISTER_ACTION(DHEnergyGPU, "DHENERGY")
PLUMED_REGISTER_ACTION(DHEnergyGPU, "DHENERGY_GPU")

// DHEnergy::registerKeywords (DHEnergy.cpp:80-87)
void DHEnergyGPU::registerKeywords(Keywords &keys) {
  PairLoopGPU::registerKeywords(keys);
  keys.add("compulsory", "I", "1.0", "Ionic strength (M)");
  keys.add("compulsory", "TEMP", "300.0", "Simulation temperature (K)");
  keys.add("compulsory", "EPSILON", "80.0", "Dielectric constant of solvent");
  keys.setValueDescription("scalar", "the value of the DHENERGY");
}

// DHEnergy::DHEnergy (DHEnergy.cpp:98-122)
DHEnergyGPU::DHEnergyGPU(const ActionOptions &ao) : Action(ao), PairLoopGPU(ao) {
  double I = 1.0, T = 300.0, epsilon = 80.0;
  parse("I", I);
  parse("TEMP", T);
  parse("EPSILON", epsilon);
  checkRead();
  if (usingNaturalUnits()) error("DHENERGY cannot be used for calculations performed with natural units");
  p.r0 = 1.0;  // the switching function is not used by this CV
  create("DHENERGY");
  check(coord_set_dhenergy(ctx, I, T, epsilon, getUnits().getEnergy(), getUnits().getLength(), getUnits().getCharge()),
        "DHENERGY");
  log << "  with solvent dielectric constant " << epsilon << "\n";
  log << "  at temperature " << T << " K\n";
  log << "  at ionic strength " << I << "M\n";
}

// the requested atoms' charges (Atoms::getCharge) by absolute index
void DHEnergyGPU::before_forward() {
  int64_t top = 0;
  for (const auto &a : full) top = std::max<int64_t>(top, (int64_t)a.index() + 1);
  std::vector<double> q(top, 0.0);
  for (size_t i = 0; i < full.size(); i++) q[full[i].index()] = getCharge(i);
  if (q != charges) {
    charges.swap(q);
    check(coord_set_charges(ctx, charges.data(), (int64_t)charges.size()), "DHENERGY");
  }
}

// ---- GHBFIX (colvar/GHBFIX.cpp:63) -------------------------------------------
class GHBFIXGPU : public PairLoopGPU {
public:
  explicit GHBFIXGPU(const ActionOptions &);
  static void registerKeywords(Keywords &keys);
};

PLUMED_REGISTER_ACTION(GHBFIXGPU, "GHBFIX")
PLUMED_REGISTER_ACTION(GHBFIXGPU, "GHBFIX_GPU")

// GHBFIX::registerKeywords (GHBFIX.cpp:88-99)
void GHBFIXGPU::registerKeywords(Keywords &keys) {
  PairLoopGPU::registerKeywords(keys);
  keys.add("optional", "ENERGY_UNITS", "the value of ENERGY_UNITS in the switching function");
  keys.add("compulsory", "TYPES", "the value of TYPES in the switching function");
  keys.add("compulsory", "PARAMS", "the value of PARAMS in the switching function");
  keys.add("compulsory", "D_MAX", "the value of D_MAX in the switching function");
  keys.add("compulsory", "D_0", "the value of D_0 in the switching function");
  keys.add("compulsory", "C", "the value of C in the switching function");
  keys.setValueDescription("scalar", "the GHBFIX interaction energy between the atoms in GROUPA and GROUPB");
}

// GHBFIX::GHBFIX (GHBFIX.cpp:101-171): the tables are read with the same IFile
// calls; type ids in order of first appearance; a PARAMS name that TYPES
// never named takes id 0 through std::map::operator[]
GHBFIXGPU::GHBFIXGPU(const ActionOptions &ao) : Action(ao), PairLoopGPU(ao) {
  double dmax = 0.0, d0 = 0.0, c = 0.0;
  std::string types, params, energy_units = "plumed";
  parse("D_MAX", dmax);
  parse("D_0", d0);
  parse("C", c);
  parse("TYPES", types);
  parse("PARAMS", params);
  parse("ENERGY_UNITS", energy_units);
  checkRead();
  std::map<std::string, unsigned> ids;
  std::vector<int32_t> table;
  {
    IFile typesfile;
    typesfile.link(*this);
    typesfile.open(types);
    std::string itype;
    while (typesfile.scanField("itype", itype).scanField()) {
      plumed_assert(!itype.empty()) << "itype is empty";
      if (!ids.count(itype)) {
        unsigned next = 0;
        for (const auto &kv : ids) next = std::max(next, kv.second + 1);
        ids.insert({itype, next});
      }
      table.push_back((int32_t)ids[itype]);
    }
  }
  plumed_assert(!table.empty()) << "empty TYPES table";
  const int n = *std::max_element(table.begin(), table.end()) + 1;
  std::vector<double> eta((size_t)n * n, 0.0);
  {
    IFile etafile;
    etafile.open(params);
    std::string it, jt;
    double e = 0.0;
    while (etafile.scanField("itype", it).scanField("jtype", jt).scanField("eta", e).scanField()) {
      plumed_assert(!it.empty()) << "itype is empty";
      plumed_assert(!jt.empty()) << "jtype is empty";
      eta[n * ids[it] + ids[jt]] = e;
    }
  }
  if (energy_units != "plumed") {
    Units units;
    units.setEnergy(energy_units);
    for (auto &e : eta) e *= units.getEnergy() / getUnits().getEnergy();
  }
  p.r0 = 1.0;  // the switching function is not used by this CV
  create("GHBFIX");
  check(coord_set_ghbfix(ctx, d0, dmax, c, table.data(), (int64_t)table.size(), eta.data(), n), "GHBFIX");
}

// ---- CONTACTMAP (colvar/ContactMap.cpp:118-365) ------------------------------
class ContactMapGPU : public Colvar {
  coord_cmap *cm = nullptr;
  unsigned n = 0;
  bool docomp = true;
  std::vector<double> pos, value, deriv, vir;

public:
  explicit ContactMapGPU(const ActionOptions &);
  ~ContactMapGPU() override { coord_cmap_destroy(cm); }
  static void registerKeywords(Keywords &keys);
  void calculate() override;
};

PLUMED_REGISTER_ACTION(ContactMapGPU, "CONTACTMAP")
PLUMED_REGISTER_ACTION(ContactMapGPU, "CONTACTMAP_GPU")

// ContactMap::registerKeywords (ContactMap.cpp:120-145)
void ContactMapGPU::registerKeywords(Keywords &keys) {
  Colvar::registerKeywords(keys);
  keys.add("numbered", "ATOMS", "the atoms involved in each of the contacts you wish to calculate");
  keys.reset_style("ATOMS", "atoms");
  keys.add("numbered", "SWITCH", "the switching function of each contact, or one SWITCH for all");
  keys.add("numbered", "REFERENCE", "the reference value of each contact (default 0.0), or one REFERENCE for all");
  keys.add("numbered", "WEIGHT", "the weight of each contact (default 1.0), or one WEIGHT for all");
  keys.reset_style("SWITCH", "compulsory");
  keys.addFlag("SUM", false, "calculate the sum of all the contacts in the input");
  keys.addFlag("CMDIST", false, "calculate the distance with respect to the provided reference contact map");
  keys.addFlag("SERIAL", false, "Perform the calculation in serial - for debug purpose");
  keys.add("compulsory", "DEVICE", "0", "CUDA device");
  keys.addOutputComponent("contact", "default", "scalar", "By not using SUM or CMDIST each contact will be stored in a component");
  keys.setValueDescription("scalar", "the sum of all the switching function on all the distances");
}

// ContactMap::ContactMap (ContactMap.cpp:147-287): the same reading order,
// defaults and messages
ContactMapGPU::ContactMapGPU(const ActionOptions &ao) : PLUMED_COLVAR_INIT(ao) {
  bool serial = false, dosum = false, docmdist = false, nopbc = false;
  parseFlag("SERIAL", serial);
  parseFlag("SUM", dosum);
  parseFlag("CMDIST", docmdist);
  if (docmdist && dosum) error("You cannot use SUM and CMDIST together");
  parseFlag("NOPBC", nopbc);
  std::vector<AtomNumber> t, ga, gb;
  for (int i = 1;; ++i) {
    parseAtomList("ATOMS", i, t);
    if (t.empty()) break;
    if (t.size() != 2) error("ATOMS" + std::to_string(i) + " keyword has the wrong number of atoms");
    ga.push_back(t[0]);
    gb.push_back(t[1]);
    t.resize(0);
    if (!dosum && !docmdist) {
      addComponentWithDerivatives("contact-" + std::to_string(i));
      componentIsNotPeriodic("contact-" + std::to_string(i));
    }
  }
  n = ga.size();
  std::vector<std::string> sws;
  for (unsigned i = 0; i < n; ++i) {
    std::string sw1;
    if (!parseNumbered("SWITCH", i + 1, sw1)) break;
    sws.push_back(sw1);
  }
  if (sws.empty()) {
    std::string sw;
    parse("SWITCH", sw);
    if (sw.empty()) error("no switching function specified use SWITCH keyword");
    sws.push_back(sw);
  } else if (sws.size() != n) {
    error("missing SWITCH" + std::to_string(sws.size() + 1) + " keyword");
  }
  std::vector<double> reference(n, 0.), weight(n, 1.0);
  unsigned counted = 0;
  for (unsigned i = 0; i < n; ++i) {
    if (!parseNumbered("REFERENCE", i + 1, reference[i])) break;
    counted++;
  }
  if (counted == 0) {
    parse("REFERENCE", reference[0]);
    for (unsigned i = 1; i < n; ++i) {
      reference[i] = reference[0];
      counted++;
    }
  }
  if (counted == 0 && docmdist) error("with CMDIST one must use REFERENCE to setup the reference contact map");
  counted = 0;
  for (unsigned i = 0; i < n; ++i) {
    if (!parseNumbered("WEIGHT", i + 1, weight[i])) break;
    counted++;
  }
  if (counted == 0) {
    parse("WEIGHT", weight[0]);
    for (unsigned i = 1; i < n; ++i) weight[i] = weight[0];
  }
  int device = 0;
  parse("DEVICE", device);
  if (dosum || docmdist) {
    addValueWithDerivatives();
    setNotPeriodic();
  }
  docomp = !(dosum || docmdist);
  std::vector<AtomNumber> full = ga;
  full.insert(full.end(), gb.begin(), gb.end());
  requestAtoms(full);
  checkRead();
  std::vector<const char *> defs;
  for (const auto &s : sws) defs.push_back(s.c_str());
  const int mode = docmdist ? COORD_CMAP_CMDIST : (dosum ? COORD_CMAP_SUM : COORD_CMAP_COMPONENTS);
  if (coord_cmap_create((int64_t)n, defs.data(), (int)defs.size(), reference.data(), weight.data(), mode, nopbc, device,
                        &cm) != COORD_OK)
    error(coord_cmap_last_error(cm));
  const unsigned nv = docomp ? n : 1;
  pos.assign(6 * n, 0.0);
  value.assign(nv, 0.0);
  deriv.assign(6 * n, 0.0);
  vir.assign(9 * nv, 0.0);
}

void ContactMapGPU::calculate() {
  const auto &positions = getPositions();
  for (unsigned s = 0; s < 2 * n; s++)
    for (int k = 0; k < 3; k++) pos[3 * s + k] = positions[s][k];
  double box[9];
  const Tensor &b = getPbc().getBox();
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) box[3 * i + j] = b(i, j);
  if (coord_cmap_forward(cm, pos.data(), box, value.data(), deriv.data(), vir.data()) != COORD_OK)
    error(std::string("CONTACTMAP: ") + coord_cmap_last_error(cm));
  auto vec = [&](unsigned s) { return Vector(deriv[3 * s], deriv[3 * s + 1], deriv[3 * s + 2]); };
  auto ten = [&](unsigned i) {
    Tensor t;
    for (int x = 0; x < 3; x++)
      for (int y = 0; y < 3; y++) t(x, y) = vir[9 * i + 3 * x + y];
    return t;
  };
  if (docomp) {
    for (unsigned i = 0; i < n; i++) {
      Value *val = getPntrToComponent(i);
      setAtomsDerivatives(val, i, vec(i));
      setAtomsDerivatives(val, n + i, vec(n + i));
      setBoxDerivatives(val, ten(i));
      val->set(value[i]);
    }
  } else {
    for (unsigned s = 0; s < 2 * n; s++) setAtomsDerivatives(s, vec(s));
    setValue(value[0]);
    setBoxDerivatives(ten(0));
  }
}

} // namespace coordgpu_plugin
} // namespace PLMD
