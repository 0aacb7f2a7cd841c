// CoordinationGPU.cpp -- PLUMED plugin: COORDINATION on the GPU through
// libcoordgpu.so (include/coordgpu.h).
//
// Build against an installed PLUMED and load it with LOAD (src/setup/Load.cpp):
//
//   g++ -std=c++17 -O2 -fPIC -shared CoordinationGPU.cpp -o CoordinationGPU.so \
//       -I$PLUMED_PREFIX/include/plumed -I<repo>/include \
//       -L<repo>/plumed2_gb300/_build -lcoordgpu -Wl,-rpath,<repo>/plumed2_gb300/_build
//
//   LOAD FILE=CoordinationGPU.so
//   c: COORDINATION GROUPA=1-1000 SWITCH={RATIONAL R_0=0.3 D_MAX=1.0}
//
// After LOAD the directive COORDINATION resolves to this class (the registry
// searches the most recently loaded images first, RegisterBase.h:239-253);
// COORDINATION_GPU is a second name so that the built-in and this action can
// run side by side on one input.
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
#include "tools/Pbc.h"
#include "tools/Tensor.h"
#include "tools/Vector.h"

#include "coordgpu.h"

#include <algorithm>
#include <string>
#include <vector>

namespace PLMD {
namespace coordgpu_plugin {

class CoordinationGPU : public Colvar {
  coord_ctx *ctx = nullptr;
  std::vector<AtomNumber> full;          // GROUPA then GROUPB (slots)
  std::vector<AtomNumber> reduced;       // sorted unique atoms of the neighbour list
  std::vector<int> slot_to_reduced;      // slot -> index in reduced (-1: not in the list)
  std::vector<double> pos_slots, deriv_slots;
  bool firsttime = true;
  bool invalidateList = true;
  int nl_stride = 0;
  bool pbc = true;
  void check(int rc, const char *what);
  void build_reduced_list();

public:
  explicit CoordinationGPU(const ActionOptions &);
  ~CoordinationGPU() override;
  static void registerKeywords(Keywords &keys);
  void prepare() override;
  void calculate() override;
};

PLUMED_REGISTER_ACTION(CoordinationGPU, "COORDINATION")
PLUMED_REGISTER_ACTION(CoordinationGPU, "COORDINATION_GPU")

void CoordinationGPU::registerKeywords(Keywords &keys) {
  Colvar::registerKeywords(keys);
  keys.addFlag("SERIAL", false, "Perform the calculation in serial - for debug purpose");
  keys.addFlag("PAIR", false, "Pair only 1st element of the 1st group with 1st element in the second, etc");
  keys.addFlag("NLIST", false, "Use a neighbor list to speed up the calculation");
  keys.addFlag("NLISTCELLS", false, "Use a neighbor list built from link cells (every pair of neighbouring cells)");
  keys.add("optional", "NL_CUTOFF", "The cutoff for the neighbor list");
  keys.add("optional", "NL_STRIDE", "The frequency with which we are updating the atoms in the neighbor list");
  keys.add("atoms", "GROUPA", "First list of atoms");
  keys.add("atoms", "GROUPB", "Second list of atoms (if empty, N*(N-1)/2 pairs in GROUPA are counted)");
  keys.add("compulsory", "NN", "6", "The n parameter of the switching function ");
  keys.add("compulsory", "MM", "0", "The m parameter of the switching function; 0 implies 2*NN");
  keys.add("compulsory", "D_0", "0.0", "The d_0 parameter of the switching function");
  keys.add("compulsory", "R_0", "The r_0 parameter of the switching function");
  keys.add("optional", "SWITCH", "An alternative switching function (RATIONAL, EXP, GAUSSIAN, SMAP, CUBIC, TANH, COSINUS, Q)");
  keys.add("compulsory", "PRECISION", "FP64", "FP64 (the drop-in arithmetic) or MIXED (FP32 pairs, FP64 sums)");
  keys.add("compulsory", "DEVICE", "0", "CUDA device");
  keys.setValueDescription("scalar", "the value of the coordination");
}

void CoordinationGPU::check(int rc, const char *what) {
  if (rc != COORD_OK) error(std::string(what) + ": " + coord_last_error(ctx));
}

CoordinationGPU::CoordinationGPU(const ActionOptions &ao) : PLUMED_COLVAR_INIT(ao) {
  bool serial = false;
  parseFlag("SERIAL", serial);
  std::vector<AtomNumber> ga, gb;
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
  std::string sw;
  parse("SWITCH", sw);
  coord_params p;
  coord_params_default(&p);
  if (sw.empty()) {
    parse("R_0", p.r0);
    parse("D_0", p.d0);
    parse("NN", p.nn);
    parse("MM", p.mm);
  }
  std::string prec = "FP64";
  parse("PRECISION", prec);
  parse("DEVICE", p.device);
  checkRead();
  p.switch_def = sw.empty() ? nullptr : sw.c_str();
  p.nopbc = nopbc;
  p.pair = dopair;
  p.serial = serial;
  p.nlist = nl_classic ? COORD_NL_CLASSIC : (nl_cells ? COORD_NL_CELLS : COORD_NL_NONE);
  p.nl_cutoff = nl_cut;
  p.nl_stride = nl_stride;
  p.precision = (prec == "MIXED") ? COORD_PREC_MIXED : COORD_PREC_FP64;
  const int rc = coord_create(&p, &ctx);
  if (rc != COORD_OK) error(coord_last_error(ctx));
  full = ga;
  full.insert(full.end(), gb.begin(), gb.end());
  std::vector<int64_t> a(ga.size()), b(gb.size());
  for (size_t i = 0; i < ga.size(); i++) a[i] = ga[i].index();
  for (size_t i = 0; i < gb.size(); i++) b[i] = gb[i].index();
  check(coord_set_groups(ctx, a.data(), (int64_t)a.size(), b.data(), (int64_t)b.size()), "COORDINATION");
  pos_slots.assign(3 * full.size(), 0.0);
  deriv_slots.assign(3 * full.size(), 0.0);
  addValueWithDerivatives();
  setNotPeriodic();
  requestAtoms(full);
  log.printf("  between two groups of %u and %u atoms, on CUDA device %d (%s)\n", (unsigned)ga.size(),
             (unsigned)gb.size(), p.device, prec.c_str());
}

CoordinationGPU::~CoordinationGPU() { coord_destroy(ctx); }

// NeighborList::prepare (NeighborList.cpp:433-456)
void CoordinationGPU::prepare() {
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
void CoordinationGPU::build_reduced_list() {
  int64_t n = 0;
  check(coord_get_pairs(ctx, 0, nullptr, 0, &n), "COORDINATION");
  std::vector<uint32_t> pairs(2 * std::max<int64_t>(n, 1));
  check(coord_get_pairs(ctx, 0, pairs.data(), n, &n), "COORDINATION");
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

void CoordinationGPU::calculate() {
  const auto &positions = getPositions();
  const bool full_request = (nl_stride <= 1) || invalidateList;
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
  check(coord_forward(ctx, pos_slots.data(), box, 1, flags, &s, deriv_slots.data(), virial), "COORDINATION");
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

} // namespace coordgpu_plugin
} // namespace PLMD
