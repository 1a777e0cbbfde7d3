#pragma once
#include "pointers.h"
namespace LAMMPS_NS {
class Error : protected Pointers {
 public:
  explicit Error(LAMMPS *lmp) : Pointers(lmp) {}
  [[noreturn]] void all(const std::string &file, int line, const std::string &str);
  [[noreturn]] void one(const std::string &file, int line, const std::string &str);
};
}    // namespace LAMMPS_NS
