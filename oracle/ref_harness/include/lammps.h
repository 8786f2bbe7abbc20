// Minimal stand-in for the LIGGGHTS types the PSM headers reference (reference harness only).
#ifndef LBDEM_REF_HARNESS_LAMMPS_H
#define LBDEM_REF_HARNESS_LAMMPS_H
namespace LAMMPS_NS {
class Atom;
class Modify;
class LAMMPS {
public:
    Atom* atom;
    Modify* modify;
};
}  // namespace LAMMPS_NS
#endif
