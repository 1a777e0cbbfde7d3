/* -*- c++ -*- ----------------------------------------------------------
   LAMMPS pair style mlip_gtinv/gpu: linearized-MLIP (gtinv) energy, forces
   and virial on one NVIDIA GB300 through the mlipg C ABI (include/mlipg.h).

   Same commands and arguments as the reference package's styles
   (pair_mlip_gtinv.h:17, pair_mlip_gtinv_kokkos.h:5-12):
     pair_style mlip_gtinv/gpu            (no arguments)
     pair_coeff * * mlp.lammps El1 ... ElN   (one element or NULL per type)
   With `-sf gpu`, `pair_style mlip_gtinv` resolves to this style.
   The same class serves `mlip_pair/gpu`, the drop-in for the reference's
   radial-only `pair_style mlip_pair` (pair_mlip_pair.h): the potential
   file's des_type line selects the descriptor.
   Requires atom IDs, `newton_pair on` and requests a full neighbour list.
------------------------------------------------------------------------- */
#ifdef PAIR_CLASS
// clang-format off
PairStyle(mlip_gtinv/gpu, PairMLIPGtinvGPU);
PairStyle(mlip_pair/gpu, PairMLIPGtinvGPU);
// clang-format on
#else

#ifndef LMP_PAIR_MLIP_GTINV_GPU_H
#define LMP_PAIR_MLIP_GTINV_GPU_H

#include "pair.h"

struct mlipg_handle;

namespace LAMMPS_NS {

class PairMLIPGtinvGPU : public Pair {
 public:
  PairMLIPGtinvGPU(class LAMMPS *);
  ~PairMLIPGtinvGPU() override;
  void compute(int, int) override;
  void settings(int, char **) override;
  void coeff(int, char **) override;
  void init_style() override;
  double init_one(int, int) override;

 protected:
  mlipg_handle *handle;
  int precision;
  void allocate();
};

}    // namespace LAMMPS_NS

#endif
#endif
