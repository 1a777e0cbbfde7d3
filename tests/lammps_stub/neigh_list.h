#pragma once
#include "pointers.h"
namespace LAMMPS_NS {
class NeighList : protected Pointers {
 public:
  explicit NeighList(LAMMPS *lmp) : Pointers(lmp) {}
  int inum = 0, gnum = 0;
  int *ilist = nullptr, *numneigh = nullptr;
  int **firstneigh = nullptr;
};
}    // namespace LAMMPS_NS
