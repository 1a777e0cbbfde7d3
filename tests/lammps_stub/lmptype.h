// Minimal stand-ins for the LAMMPS declarations that the mlip_gtinv/gpu pair
// style uses (names and signatures as in LAMMPS' src/), so that the style's
// source can be syntax-checked where no LAMMPS tree exists.  Test
// infrastructure only.
#pragma once
#include <string>
#define FLERR __FILE__, __LINE__
namespace LAMMPS_NS {
class LAMMPS;
class Pair;
}
