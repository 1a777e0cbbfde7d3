#pragma once
#include "pointers.h"
namespace LAMMPS_NS {
class NeighList;
class Pair : protected Pointers {
 public:
  explicit Pair(LAMMPS *lmp) : Pointers(lmp) {}
  ~Pair() override = default;
  double eng_vdwl = 0.0, eng_coul = 0.0;
  double virial[6] = {0, 0, 0, 0, 0, 0};
  double *eatom = nullptr;
  double **vatom = nullptr;
  int single_enable = 1, restartinfo = 1, one_coeff = 0, manybody_flag = 0;
  int no_virial_fdotr_compute = 0;
  int allocated = 0;
  int **setflag = nullptr;
  double **cutsq = nullptr;
  NeighList *list = nullptr;
  virtual void compute(int, int) = 0;
  virtual void settings(int, char **) = 0;
  virtual void coeff(int, char **) = 0;
  virtual void init_style() {}
  virtual double init_one(int, int) { return 0.0; }

 protected:
  int eflag_either = 0, eflag_global = 0, eflag_atom = 0;
  int vflag_either = 0, vflag_global = 0, vflag_atom = 0;
  void ev_init(int eflag, int vflag, int alloc = 1) { (void)eflag; (void)vflag; (void)alloc; }
};
}    // namespace LAMMPS_NS
