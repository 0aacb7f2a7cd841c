// Test harness: the part of PLUMED's Pbc (src/tools/Pbc.h) that the plugin
// uses -- the box of the step.  Not PLUMED's code.
#pragma once
#include "tools/Tensor.h"
namespace PLMD {
class Pbc {
  Tensor box;

public:
  void setBox(const Tensor &b) { box = b; }
  const Tensor &getBox() const { return box; }
};
}  // namespace PLMD
