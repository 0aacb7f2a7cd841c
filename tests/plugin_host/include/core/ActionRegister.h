// Test harness: a registry of action classes by directive name, standing in
// for PLUMED's ActionRegister (src/core/ActionRegister.h) so that the plugin's
// PLUMED_REGISTER_ACTION lines register its classes with the harness driver
// (host.cpp).  Not PLUMED's code.
#pragma once
#include <functional>
#include <map>
#include <memory>
#include <string>

namespace PLMD {
class Action;
class ActionOptions;
class Keywords;

struct ActionRegistryEntry {
  std::function<std::unique_ptr<Action>(const ActionOptions &)> create;
  std::function<void(Keywords &)> keywords;
};

inline std::map<std::string, ActionRegistryEntry> &actionRegistry() {
  static std::map<std::string, ActionRegistryEntry> m;
  return m;
}

template <class T> struct RegisterAction {
  explicit RegisterAction(const char *directive) {
    actionRegistry()[directive] = {[](const ActionOptions &ao) { return std::unique_ptr<Action>(new T(ao)); },
                                   [](Keywords &k) { T::registerKeywords(k); }};
  }
};
}  // namespace PLMD

#define PLUMED_HOST_CAT2(a, b) a##b
#define PLUMED_HOST_CAT(a, b) PLUMED_HOST_CAT2(a, b)
#define PLUMED_REGISTER_ACTION(classname, directive) \
  static ::PLMD::RegisterAction<classname> PLUMED_HOST_CAT(plumed_host_register_, __LINE__)(directive);
