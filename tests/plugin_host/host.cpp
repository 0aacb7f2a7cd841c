// host.cpp -- test harness: drives the PLUMED plugin
// (plumed2_gb300/plugin/CoordinationGPU.cpp, compiled unchanged against the
// minimal action interface in include/) the way `plumed driver` drives an
// action (src/cltools/Driver.cpp -> PlumedMain: each step prepare(), then the
// requested atoms' positions and the box, then calculate()), and returns per
// frame the value, the derivatives summed by atom number (an atom requested
// twice gets both), the box derivatives and the number of requested atoms.
// Test infrastructure only.
#include "core/ActionRegister.h"
#include "core/Colvar.h"

#include <cstring>
#include <exception>
#include <string>
#include <vector>

namespace {

// Words of an input line; a {...} group is one word with its outer braces removed.
std::vector<std::string> split_line(const std::string &line) {
  std::vector<std::string> out;
  std::string cur;
  int depth = 0;
  for (char ch : line) {
    if (ch == '{') {
      if (depth++ == 0) continue;
    } else if (ch == '}') {
      if (--depth == 0) continue;
    } else if ((ch == ' ' || ch == '\t' || ch == '\n') && depth == 0) {
      if (!cur.empty()) out.push_back(cur);
      cur.clear();
      continue;
    }
    cur += ch;
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

void copy_out(const std::string &s, char *dst, int len) {
  if (!dst || len <= 0) return;
  std::strncpy(dst, s.c_str(), (size_t)len - 1);
  dst[len - 1] = 0;
}

}  // namespace

extern "C" int plugin_host_run(const char *line, long long n_atoms, int n_frames, long long stride,
                               const double *pos, const double *boxes, const double *charges, double *values,
                               double *deriv, double *virial, long long *n_requested, char *log_out, int log_len,
                               char *err, int err_len) {
  using namespace PLMD;
  copy_out("", err, err_len);
  try {
    std::vector<std::string> w = split_line(line);
    if (w.empty()) throw std::runtime_error("empty input line");
    ActionOptions ao;
    size_t first = 0;
    if (w[0].back() == ':') {
      ao.label = w[0].substr(0, w[0].size() - 1);
      first = 1;
    }
    if (first >= w.size()) throw std::runtime_error("no directive in the input line");
    ao.name = w[first];
    for (size_t i = first + 1; i < w.size(); i++) {
      if (w[i].compare(0, 6, "LABEL=") == 0)
        ao.label = w[i].substr(6);
      else
        ao.words.push_back(w[i]);
    }
    auto it = actionRegistry().find(ao.name);
    if (it == actionRegistry().end()) throw std::runtime_error("unknown directive " + ao.name);
    it->second.keywords(ao.keys);
    HostFrame fr;
    fr.n_atoms = n_atoms;
    fr.pos = pos;
    fr.box = boxes;
    ao.frame = &fr;
    std::unique_ptr<Action> act = it->second.create(ao);
    Colvar *cv = dynamic_cast<Colvar *>(act.get());
    if (!cv) throw std::runtime_error(ao.name + " is not a Colvar");
    for (int k = 0; k < n_frames; k++) {
      fr.step = (long long)k * stride;
      fr.pos = pos + (size_t)k * n_atoms * 3;
      fr.box = boxes + (size_t)k * 9;
      fr.charges = charges ? charges + (size_t)k * n_atoms : nullptr;
      act->prepare();
      cv->hostRetrieve();
      cv->hostResetDerivatives();
      act->calculate();
      Value *v = cv->getPntrToValue();
      const auto &idx = cv->getAbsoluteIndexes();
      if (values) values[k] = v->value;
      if (deriv)
        for (size_t i = 0; i < idx.size(); i++)
          for (int q = 0; q < 3; q++) deriv[((size_t)k * n_atoms + idx[i].index()) * 3 + q] += v->derivatives[3 * i + q];
      if (virial)
        for (int q = 0; q < 9; q++) virial[(size_t)k * 9 + q] = v->derivatives[3 * idx.size() + q];
      if (n_requested) n_requested[k] = (long long)idx.size();
    }
    copy_out(act->log.str(), log_out, log_len);
  } catch (const std::exception &e) {
    copy_out(e.what(), err, err_len);
    return 1;
  }
  return 0;
}
