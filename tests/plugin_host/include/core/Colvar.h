// Test harness: a minimal restatement of the action interface PLUMED gives a
// Colvar (src/core/Action.h, ActionAtomistic.h, ActionWithValue.h, Colvar.h,
// tools/Keywords.h, tools/AtomNumber.h, tools/Log.h), written for this test
// harness only.  It holds exactly what the plugin in
// plumed2_gb300/plugin/CoordinationGPU.cpp calls, with PLUMED's meaning:
//   * keywords: KEY=value words of the input line, compulsory defaults from
//     registerKeywords, flags, numbered keywords, atom lists with PLUMED's
//     range syntax (a-b, a-b:stride, comma lists), checkRead;
//   * atoms: requestAtoms sets the atoms whose positions the next
//     calculate() receives (getPositions in request order), getPbc, getCharge;
//   * values: one value with derivatives (or named components), derivatives
//     3 per requested atom then the 9 box entries (Colvar.h layout);
//   * the step number, the log, units, errors (thrown as exceptions).
// The driver that creates actions by directive name and steps them through
// frames is host.cpp.  Not PLUMED's code.
#pragma once
#include "tools/Pbc.h"
#include "tools/Tensor.h"
#include "tools/Units.h"
#include "tools/Vector.h"

#include <cstdarg>
#include <cstdio>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace PLMD {

class AtomNumber {
  unsigned i = 0;

public:
  unsigned index() const { return i; }
  unsigned serial() const { return i + 1; }
  static AtomNumber index(unsigned k) {
    AtomNumber a;
    a.i = k;
    return a;
  }
  friend bool operator<(AtomNumber a, AtomNumber b) { return a.i < b.i; }
  friend bool operator==(AtomNumber a, AtomNumber b) { return a.i == b.i; }
};

class Log {
  std::ostringstream os;

public:
  void printf(const char *fmt, ...) {
    char buf[2048];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    os << buf;
  }
  template <typename T> Log &operator<<(const T &x) {
    os << x;
    return *this;
  }
  std::string str() const { return os.str(); }
};

// plumed_assert(condition) << "message": throws when the condition is false
struct HostAssert {
  bool ok;
  std::ostringstream os;
  ~HostAssert() noexcept(false) {
    if (!ok) throw std::runtime_error("assertion failed: " + os.str());
  }
  template <typename T> HostAssert &operator<<(const T &x) {
    os << x;
    return *this;
  }
};
#define plumed_assert(cond) ::PLMD::HostAssert{static_cast<bool>(cond), {}}

class Keywords {
public:
  std::map<std::string, std::string> defaults;  // compulsory keywords with a default
  std::map<std::string, bool> flags;
  void add(const std::string &, const std::string &, const std::string &) {}
  void add(const std::string &type, const std::string &key, const std::string &def, const std::string &) {
    if (type == "compulsory") defaults[key] = def;
  }
  void addFlag(const std::string &key, bool def, const std::string &) { flags[key] = def; }
  void reset_style(const std::string &, const std::string &) {}
  void addOutputComponent(const std::string &, const std::string &, const std::string &, const std::string &) {}
  void setValueDescription(const std::string &, const std::string &) {}
};

// What the driver provides to its actions: the step and the frame.
struct HostFrame {
  long long step = 0;
  const double *pos = nullptr;      // [n_atoms][3]
  const double *box = nullptr;      // [9]
  const double *charges = nullptr;  // [n_atoms] or null
  long long n_atoms = 0;
};

struct ActionOptions {
  std::string label, name;
  std::vector<std::string> words;  // KEY=value and flag words, braces removed
  Keywords keys;
  const HostFrame *frame = nullptr;
};

class Action {
  std::vector<std::string> words_;
  Keywords keys_;
  std::string name_, label_;
  Units units_;

protected:
  const HostFrame *frame_ = nullptr;
  Action() = default;

public:
  Log log;
  explicit Action(const ActionOptions &ao)
      : words_(ao.words), keys_(ao.keys), name_(ao.name), label_(ao.label), frame_(ao.frame) {}
  virtual ~Action() = default;
  const std::string &getName() const { return name_; }
  const std::string &getLabel() const { return label_; }
  long long getStep() const { return frame_->step; }
  bool getExchangeStep() const { return false; }
  bool usingNaturalUnits() const { return false; }
  const Units &getUnits() const { return units_; }
  [[noreturn]] void error(const std::string &msg) const {
    throw std::runtime_error("ERROR in input to action " + name_ + " with label " + label_ + " : " + msg);
  }
  virtual void prepare() {}
  virtual void calculate() = 0;

  // the value of KEY=value, removed from the line; false when absent
  bool take(const std::string &key, std::string &value) {
    for (size_t i = 0; i < words_.size(); i++) {
      const std::string &w = words_[i];
      if (w.size() > key.size() && w.compare(0, key.size(), key) == 0 && w[key.size()] == '=') {
        value = w.substr(key.size() + 1);
        words_.erase(words_.begin() + (long)i);
        return true;
      }
    }
    return false;
  }
  void convert(const std::string &key, const std::string &s, std::string &t) const { t = s; }
  void convert(const std::string &key, const std::string &s, double &t) const {
    std::size_t used = 0;
    try {
      t = std::stod(s, &used);
    } catch (...) {
      used = 0;
    }
    if (used != s.size()) error("cannot read the value of " + key + ": " + s);
  }
  void convert(const std::string &key, const std::string &s, int &t) const {
    std::size_t used = 0;
    try {
      t = std::stoi(s, &used);
    } catch (...) {
      used = 0;
    }
    if (used != s.size()) error("cannot read the value of " + key + ": " + s);
  }
  template <class T> void parse(const std::string &key, T &t) {
    std::string s;
    if (take(key, s)) {
      convert(key, s, t);
      return;
    }
    auto d = keys_.defaults.find(key);
    if (d != keys_.defaults.end()) convert(key, d->second, t);
  }
  template <class T> bool parseNumbered(const std::string &key, int no, T &t) {
    std::string s;
    if (!take(key + std::to_string(no), s)) return false;
    convert(key, s, t);
    return true;
  }
  void parseFlag(const std::string &key, bool &t) {
    for (size_t i = 0; i < words_.size(); i++)
      if (words_[i] == key) {
        words_.erase(words_.begin() + (long)i);
        t = true;
        return;
      }
    auto d = keys_.flags.find(key);
    t = (d != keys_.flags.end()) ? d->second : false;
  }
  // PLUMED's atom ranges: n, a-b, a-b:stride (stride may be negative), joined by commas
  static std::vector<AtomNumber> atoms_of(const std::string &s) {
    std::vector<AtomNumber> out;
    std::stringstream ss(s);
    std::string item;
    while (std::getline(ss, item, ',')) {
      if (item.empty()) continue;
      long long a, b, st = 1;
      const size_t colon = item.find(':');
      std::string range = item.substr(0, colon);
      if (colon != std::string::npos) st = std::stoll(item.substr(colon + 1));
      const size_t dash = range.find('-', 1);
      if (dash == std::string::npos) {
        a = b = std::stoll(range);
      } else {
        a = std::stoll(range.substr(0, dash));
        b = std::stoll(range.substr(dash + 1));
      }
      if (st == 0) throw std::runtime_error("zero stride in atom range " + item);
      for (long long k = a; st > 0 ? k <= b : k >= b; k += st) out.push_back(AtomNumber::index((unsigned)(k - 1)));
    }
    return out;
  }
  void parseAtomList(const std::string &key, std::vector<AtomNumber> &t) {
    std::string s;
    t.clear();
    if (take(key, s)) t = atoms_of(s);
  }
  void parseAtomList(const std::string &key, int num, std::vector<AtomNumber> &t) {
    parseAtomList(key + std::to_string(num), t);
  }
  void checkRead() {
    if (words_.empty()) return;
    std::string msg = "cannot understand the following words from the input line : ";
    for (const auto &w : words_) msg += w + " ";
    error(msg);
  }
};

class Value {
public:
  std::string name;
  double value = 0.0;
  std::vector<double> derivatives;  // 3 per requested atom, then the box (9)
  void set(double v) { value = v; }
  double get() const { return value; }
};

class ActionAtomistic : public virtual Action {
  std::vector<AtomNumber> requested_;
  std::vector<Vector> positions_;
  std::vector<double> charges_;
  Pbc pbc_;

public:
  void requestAtoms(const std::vector<AtomNumber> &a) { requested_ = a; }
  const std::vector<AtomNumber> &getAbsoluteIndexes() const { return requested_; }
  const std::vector<Vector> &getPositions() const { return positions_; }
  const Pbc &getPbc() const { return pbc_; }
  double getCharge(int i) const { return charges_.at((size_t)i); }
  // the driver's retrieveAtoms: the requested atoms of the current frame
  void hostRetrieve() {
    const HostFrame &fr = *frame_;
    positions_.resize(requested_.size());
    charges_.assign(requested_.size(), 0.0);
    for (size_t i = 0; i < requested_.size(); i++) {
      const long long a = requested_[i].index();
      if (a >= fr.n_atoms) error("atom " + std::to_string(a + 1) + " is beyond the frame");
      positions_[i] = Vector(fr.pos[3 * a], fr.pos[3 * a + 1], fr.pos[3 * a + 2]);
      if (fr.charges) charges_[i] = fr.charges[a];
    }
    Tensor b;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) b(i, j) = fr.box[3 * i + j];
    pbc_.setBox(b);
  }
};

class ActionWithValue : public virtual Action {
protected:
  std::vector<std::unique_ptr<Value>> values_;

public:
  void addValueWithDerivatives() { values_.emplace_back(new Value()); }
  void setNotPeriodic() {}
  void addComponentWithDerivatives(const std::string &n) {
    values_.emplace_back(new Value());
    values_.back()->name = n;
  }
  void componentIsNotPeriodic(const std::string &) {}
  Value *getPntrToComponent(int i) { return values_.at((size_t)i).get(); }
  Value *getPntrToValue() { return values_.at(0).get(); }
  int getNumberOfComponents() const { return (int)values_.size(); }
  void setValue(double v) { getPntrToValue()->set(v); }
};

class Colvar : public ActionAtomistic, public ActionWithValue {
public:
  explicit Colvar(const ActionOptions &ao) : Action(ao) {}
  static void registerKeywords(Keywords &keys) {
    keys.addFlag("NOPBC", false, "ignore the periodic boundary conditions when calculating distances");
  }
  // zeroed derivative arrays sized for the current request (before calculate)
  void hostResetDerivatives() {
    for (auto &v : values_) v->derivatives.assign(3 * getAbsoluteIndexes().size() + 9, 0.0);
  }
  void setAtomsDerivatives(Value *v, int i, const Vector &d) {
    for (int k = 0; k < 3; k++) v->derivatives.at(3 * (size_t)i + k) = d[k];
  }
  void setAtomsDerivatives(int i, const Vector &d) { setAtomsDerivatives(getPntrToValue(), i, d); }
  void setBoxDerivatives(Value *v, const Tensor &t) {
    const size_t o = 3 * getAbsoluteIndexes().size();
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) v->derivatives.at(o + 3 * a + b) = t(a, b);
  }
  void setBoxDerivatives(const Tensor &t) { setBoxDerivatives(getPntrToValue(), t); }
};

}  // namespace PLMD

#define PLUMED_COLVAR_INIT(ao) Action(ao), Colvar(ao)
