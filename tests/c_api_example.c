/* The C example of INTEGRATION.md as a program: create a handle, map the
 * LAMMPS types to elements, evaluate a two-atom system through the
 * LAMMPS-shaped entry point.  Compiled, linked against libmlipg.so and run by
 * tests/test_headers_cpu.py.  Without a GPU the evaluation returns
 * MLIPG_ENOGPU (there is no CPU fallback). */
#include <stdio.h>

#include "mlipg.h"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  mlipg_handle* h;
  if (mlipg_create(argv[1], MLIPG_PREC_MIXED, &h) != MLIPG_OK) {
    puts(mlipg_last_error(NULL));
    return 1;
  }
  const char* map[] = {"Ti", "Al"};
  if (mlipg_set_type_map(h, 2, map) != MLIPG_OK) {
    puts(mlipg_last_error(h));
    return 1;
  }
  /* two atoms 2.5 A apart, each in the other's full list, no ghosts */
  double x[6] = {0, 0, 0, 2.5, 0, 0}, f[6] = {0, 0, 0, 0, 0, 0};
  double energy = 0, virial[6], eatom[2];
  int type[2] = {1, 2}, ilist[2] = {0, 1}, numneigh[2] = {1, 1}, n0[1] = {1}, n1[1] = {0};
  const int* firstneigh[2] = {n0, n1};
  const int rc = mlipg_compute(h, 2, 2, x, type, 2, ilist, numneigh, firstneigh, 1, 1, f,
                               &energy, virial, eatom, NULL);
  printf("status %d cutoff %.3f elements %d energy %.6f\n", rc, mlipg_cutoff(h),
         mlipg_num_elements(h), energy);
  mlipg_destroy(h);
  return (rc == MLIPG_OK || rc == MLIPG_ENOGPU) ? 0 : 1;
}
