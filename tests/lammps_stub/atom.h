#pragma once
#include "pointers.h"
namespace LAMMPS_NS {
class Atom : protected Pointers {
 public:
  explicit Atom(LAMMPS *lmp) : Pointers(lmp) {}
  int nlocal = 0, nghost = 0, ntypes = 0, tag_enable = 1;
  double **x = nullptr, **f = nullptr;
  int *type = nullptr;
  void set_mass(const char *file, int line, int itype, double value);
};
}    // namespace LAMMPS_NS
