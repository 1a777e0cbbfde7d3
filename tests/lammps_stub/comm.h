#pragma once
#include "pointers.h"
namespace LAMMPS_NS {
class Comm : protected Pointers {
 public:
  explicit Comm(LAMMPS *lmp) : Pointers(lmp) {}
  int me = 0, nprocs = 1;
};
}    // namespace LAMMPS_NS
