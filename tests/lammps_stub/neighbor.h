#pragma once
#include "pointers.h"
namespace LAMMPS_NS {
namespace NeighConst {
  enum { REQ_DEFAULT = 0, REQ_FULL = 1 << 0, REQ_GHOST = 1 << 1 };
}
class NeighRequest;
class Neighbor : protected Pointers {
 public:
  explicit Neighbor(LAMMPS *lmp) : Pointers(lmp) {}
  NeighRequest *add_request(class Pair *, int flags = 0);
};
}    // namespace LAMMPS_NS
