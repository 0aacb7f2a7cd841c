// Test harness: the part of PLUMED's IFile (src/tools/IFile.h) that the plugin
// uses -- column files with a "#! FIELDS a b ..." header read record by
// record: scanField(name, value) reads the named column of the current record
// (reading the next line first when a record starts), scanField() closes the
// record and is false once the file has no more records.  Not PLUMED's code.
#pragma once
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace PLMD {
class Action;
class IFile {
  std::vector<std::string> fields;
  std::vector<std::vector<std::string>> rows;
  size_t next = 0;
  bool in_record = false, ok = true;
  const std::vector<std::string> *cur = nullptr;

public:
  void link(Action &) {}
  void open(const std::string &path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("IFile: cannot open " + path);
    std::string line;
    while (std::getline(in, line)) {
      std::istringstream ss(line);
      std::vector<std::string> w;
      std::string t;
      while (ss >> t) w.push_back(t);
      if (w.empty()) continue;
      if (w[0] == "#!") {
        if (w.size() > 1 && w[1] == "FIELDS") fields.assign(w.begin() + 2, w.end());
        continue;
      }
      if (w[0][0] == '#') continue;
      rows.push_back(w);
    }
  }
  template <typename T> IFile &scanField(const std::string &name, T &value) {
    if (!in_record) {
      in_record = true;
      ok = next < rows.size();
      cur = ok ? &rows[next++] : nullptr;
    }
    if (!ok) return *this;
    for (size_t i = 0; i < fields.size(); i++)
      if (fields[i] == name) {
        if (i >= cur->size()) throw std::runtime_error("IFile: record too short for field " + name);
        std::istringstream ss((*cur)[i]);
        ss >> value;
        return *this;
      }
    throw std::runtime_error("IFile: no field " + name);
  }
  IFile &scanField() {
    in_record = false;
    return *this;
  }
  explicit operator bool() const { return ok; }
};
}  // namespace PLMD
