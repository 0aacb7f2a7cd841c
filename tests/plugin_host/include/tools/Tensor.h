// Test harness: the part of PLUMED's Tensor (src/tools/Tensor.h) that the
// plugin uses -- a 3x3 matrix with (i, j) access.  Not PLUMED's code.
#pragma once
namespace PLMD {
class Tensor {
  double m[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};

public:
  double &operator()(int i, int j) { return m[i][j]; }
  double operator()(int i, int j) const { return m[i][j]; }
};
}  // namespace PLMD
