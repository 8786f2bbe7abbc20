// Stand-in for LIGGGHTS' Atom: map(tag) is the lowest local index holding the
// tag, as LAMMPS' atom map returns the owned atom before its ghost images
// (reference harness only).
#ifndef LBDEM_REF_HARNESS_ATOM_H
#define LBDEM_REF_HARNESS_ATOM_H
#include <vector>
namespace LAMMPS_NS {
class Atom {
public:
    std::vector<int> map_array;
    int map(int tag) const { return (tag >= 0 && tag < (int)map_array.size()) ? map_array[tag] : -1; }
};
}  // namespace LAMMPS_NS
#endif
