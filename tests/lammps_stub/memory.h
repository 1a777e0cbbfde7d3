#pragma once
#include "pointers.h"
namespace LAMMPS_NS {
class Memory : protected Pointers {
 public:
  explicit Memory(LAMMPS *lmp) : Pointers(lmp) {}
  template <typename TYPE> TYPE **create(TYPE **&array, int n1, int n2, const char *name);
  template <typename TYPE> void destroy(TYPE **&array);
};
}    // namespace LAMMPS_NS
