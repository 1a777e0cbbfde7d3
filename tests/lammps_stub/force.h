#pragma once
#include "pointers.h"
namespace LAMMPS_NS {
class Force : protected Pointers {
 public:
  explicit Force(LAMMPS *lmp) : Pointers(lmp) {}
  int newton = 1, newton_pair = 1, newton_bond = 1;
};
}    // namespace LAMMPS_NS
