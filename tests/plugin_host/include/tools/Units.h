// Test harness: the part of PLUMED's Units (src/tools/Units.h) that the
// plugin uses.  Energies in kJ/mol, lengths in nm, charges in e (PLUMED's
// defaults); setEnergy knows the names the plugin's tests use.  Not PLUMED's
// code.
#pragma once
#include <stdexcept>
#include <string>
namespace PLMD {
class Units {
  double energy = 1.0, length = 1.0, charge = 1.0;

public:
  void setEnergy(const std::string &s) {
    if (s == "kj/mol") energy = 1.0;
    else if (s == "kcal/mol") energy = 4.184;
    else if (s == "j/mol") energy = 0.001;
    else if (s == "eV") energy = 96.48530749925792;
    else if (s == "Ha") energy = 2625.499638;
    else {
      std::size_t used = 0;
      energy = std::stod(s, &used);
      if (used != s.size() || !(energy > 0.0)) throw std::runtime_error("Units::setEnergy: bad unit " + s);
    }
  }
  double getEnergy() const { return energy; }
  double getLength() const { return length; }
  double getCharge() const { return charge; }
};
}  // namespace PLMD
