// Test harness: the part of PLUMED's Vector (src/tools/Vector.h) that the
// plugin uses -- three doubles, indexing, +=.  Not PLUMED's code.
#pragma once
namespace PLMD {
class Vector {
  double d[3] = {0.0, 0.0, 0.0};

public:
  Vector() = default;
  Vector(double x, double y, double z) : d{x, y, z} {}
  double &operator[](int i) { return d[i]; }
  double operator[](int i) const { return d[i]; }
  Vector &operator+=(const Vector &o) {
    for (int i = 0; i < 3; i++) d[i] += o.d[i];
    return *this;
  }
};
}  // namespace PLMD
