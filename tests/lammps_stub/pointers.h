#pragma once
#include "lmptype.h"
namespace LAMMPS_NS {
class Atom;
class Force;
class Comm;
class Neighbor;
class Error;
class Memory;
class LAMMPS {
 public:
  Atom *atom;
  Force *force;
  Comm *comm;
  Neighbor *neighbor;
  Error *error;
  Memory *memory;
};
class Pointers {
 public:
  explicit Pointers(LAMMPS *ptr)
      : lmp(ptr), atom(ptr->atom), force(ptr->force), comm(ptr->comm), neighbor(ptr->neighbor),
        error(ptr->error), memory(ptr->memory) {}
  virtual ~Pointers() = default;

 protected:
  LAMMPS *lmp;
  Atom *&atom;
  Force *&force;
  Comm *&comm;
  Neighbor *&neighbor;
  Error *&error;
  Memory *&memory;
};
}    // namespace LAMMPS_NS
