// Stand-in for LIGGGHTS' Fix base class so that fix_lb_coupling_onetoone.h
// compiles (reference harness only).
#ifndef LBDEM_REF_HARNESS_FIX_H
#define LBDEM_REF_HARNESS_FIX_H
#include "lammps.h"
namespace LAMMPS_NS {
class Fix {
public:
    Fix(LAMMPS*, int, char**) {}
    virtual ~Fix() {}
};
}  // namespace LAMMPS_NS
#endif
