/* ----------------------------------------------------------------------
   LAMMPS pair style mlip_gtinv/gpu (see pair_mlip_gtinv_gpu.h).

   Each hook mirrors the reference Kokkos pair style
   (src/USER-MLIP/pair_mlip_gtinv_kokkos_impl.h) and hands the work to the
   mlipg C ABI; any non-zero status becomes error->all with the library's
   message instead of the reference's exit() calls.
------------------------------------------------------------------------- */
#include "pair_mlip_gtinv_gpu.h"

#include "atom.h"
#include "comm.h"
#include "error.h"
#include "force.h"
#include "memory.h"
#include "neigh_list.h"
#include "neighbor.h"

#include "mlipg.h"

#include <cstring>
#include <vector>

using namespace LAMMPS_NS;

PairMLIPGtinvGPU::PairMLIPGtinvGPU(LAMMPS *lmp) : Pair(lmp), handle(nullptr)
{
  single_enable = 0;
  restartinfo = 0;    // as the reference (pair_mlip_gtinv.cpp:43): re-read by pair_coeff
  one_coeff = 1;
  manybody_flag = 1;
  no_virial_fdotr_compute = 1;    // the library returns the virial
  // FP64 by default, as the reference pair style (which takes no precision
  // argument): the drop-in reproduces its energies; `mixed` is opt-in
  precision = MLIPG_PREC_FP64;
}

PairMLIPGtinvGPU::~PairMLIPGtinvGPU()
{
  if (handle) mlipg_destroy(handle);
  if (allocated) {
    memory->destroy(setflag);
    memory->destroy(cutsq);
  }
}

void PairMLIPGtinvGPU::allocate()
{
  allocated = 1;
  int n = atom->ntypes;
  memory->create(setflag, n + 1, n + 1, "pair:setflag");
  memory->create(cutsq, n + 1, n + 1, "pair:cutsq");
  for (int i = 1; i <= n; i++)
    for (int j = i; j <= n; j++) setflag[i][j] = 0;
}

// pair_style mlip_gtinv/gpu [fp64|fp64_native|mixed|mixed_a64]  (the reference takes no arguments,
// pair_mlip_gtinv_kokkos_impl.h:87-90; the optional keyword selects precision)
void PairMLIPGtinvGPU::settings(int narg, char **arg)
{
  if (narg > 1) error->all(FLERR, "Illegal pair_style command");
  if (narg == 1) {
    if (strcmp(arg[0], "fp64") == 0) precision = MLIPG_PREC_FP64;
    else if (strcmp(arg[0], "mixed") == 0) precision = MLIPG_PREC_MIXED;
    else if (strcmp(arg[0], "mixed_a64") == 0) precision = MLIPG_PREC_MIXED_A64;
    else if (strcmp(arg[0], "fp64_native") == 0) precision = MLIPG_PREC_FP64_NATIVE;
    else error->all(FLERR, "Illegal pair_style command");
  }
}

// pair_coeff * * file El1 ... ElN  (pair_mlip_gtinv_kokkos_impl.h:92-212)
void PairMLIPGtinvGPU::coeff(int narg, char **arg)
{
  if (!allocated) allocate();
  if (narg != 3 + atom->ntypes) error->all(FLERR, "Incorrect args for pair coefficients");
  if (strcmp(arg[0], "*") != 0 || strcmp(arg[1], "*") != 0)
    error->all(FLERR, "Incorrect args for pair coefficients");
  if (handle) mlipg_destroy(handle);
  handle = nullptr;
  if (mlipg_create(arg[2], precision, &handle) != MLIPG_OK)
    error->all(FLERR, mlipg_last_error(nullptr));
  if (mlipg_set_type_map(handle, atom->ntypes, arg + 3) != MLIPG_OK)
    error->all(FLERR, mlipg_last_error(handle));
  int count = 0;
  for (int i = 1; i <= atom->ntypes; i++) {
    for (int j = i; j <= atom->ntypes; j++) {
      if (strcmp(arg[2 + i], "NULL") != 0 && strcmp(arg[2 + j], "NULL") != 0) {
        setflag[i][j] = 1;
        count++;
      }
    }
    if (strcmp(arg[2 + i], "NULL") != 0) {
      for (int k = 0; k < mlipg_num_elements(handle); k++)
        if (strcmp(arg[2 + i], mlipg_element_name(handle, k)) == 0)
          atom->set_mass(FLERR, i, mlipg_element_mass(handle, k));
    }
  }
  if (count == 0) error->all(FLERR, "Incorrect args for pair coefficients");
}

// pair_mlip_gtinv_kokkos_impl.h:229-270: atom IDs, newton on, full list
void PairMLIPGtinvGPU::init_style()
{
  if (atom->tag_enable == 0) error->all(FLERR, "Pair style mlip_gtinv requires atom IDs");
  if (force->newton_pair == 0)
    error->all(FLERR, "Pair style mlip_gtinv requires newton pair on");
  neighbor->add_request(this, NeighConst::REQ_FULL);
}

double PairMLIPGtinvGPU::init_one(int i, int j)
{
  if (setflag[i][j] == 0) error->all(FLERR, "All pair coeffs are not set");
  return mlipg_cutoff(handle);
}

// pair_mlip_gtinv_kokkos_impl.h:272-406
void PairMLIPGtinvGPU::compute(int eflag, int vflag)
{
  ev_init(eflag, vflag);
  const int nlocal = atom->nlocal;
  const int nall = nlocal + atom->nghost;
  double energy = 0.0, vir[6] = {0, 0, 0, 0, 0, 0};
  const int rc = mlipg_compute(handle, nlocal, nall, &atom->x[0][0], atom->type, list->inum,
                               list->ilist, list->numneigh, list->firstneigh, eflag_global,
                               vflag_global, &atom->f[0][0], &energy, vir,
                               eflag_atom ? eatom : nullptr,
                               vflag_atom ? &vatom[0][0] : nullptr);
  if (rc != MLIPG_OK) error->one(FLERR, mlipg_last_error(handle));
  if (eflag_global) eng_vdwl += energy;
  if (vflag_global)
    for (int k = 0; k < 6; k++) virial[k] += vir[k];
}
