// excludeType through the C++ shim (src/ibDataExchangeWrappers3D.hh:62-73): two
// spheres of LIGGGHTS types 1 and 2 in a periodic 32^3 lattice with a uniform
// flow; setSpheresOnLattice(lattice, wrapper, units, excludeType = {2}, false)
// must voxelize the type-1 sphere only, the sphere list must hold it alone, no
// cell may name the type-2 tag, and getForcesFromLattice must give the type-2
// atom zero force and torque and the type-1 atom a drag.  The same run without
// exclusion voxelizes both.  Exit 0 on success, 1 on a failed check, 77 without
// a GPU.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dem_standin.h"
#include "lbdem_plb.h"
#include "physunits_gpu.h"

static int run(bool exclude) {
    plb::GpuLattice3D::Options o;
    o.periodic[0] = o.periodic[1] = o.periodic[2] = true;
    o.maxParticles = 16;
    o.maxTag = 16;
    o.maxRadius = 8.0;
    plb::GpuLattice3D lattice(32, 32, 32, 1.0 / 0.6, o);
    lattice.initialize(1.0, 0.02, 0.0, 0.0);
    plb::PhysUnits3D<double> units(1.0, 1.0, 0.1 / 3.0, 32, 32, 32, 1, 1.0, 1.0);
    LiggghtsCouplingWrapper wrapper;
    const double p1[3] = {10.5, 16.5, 16.5}, p2[3] = {22.5, 16.5, 16.5}, v0[3] = {0, 0, 0};
    wrapper.atom.add(p1, v0, 4.0, 1.5, 1, 1);   // tag 1, type 1
    wrapper.atom.add(p2, v0, 4.0, 1.5, 2, 2);   // tag 2, type 2
    wrapper.sync();
    std::vector<long> excludeType;
    if (exclude) excludeType.push_back(2);
    for (int it = 0; it < 3; ++it) {
        plb::setSpheresOnLattice(lattice, wrapper, units, excludeType, false);
        lattice.collideAndStream();
        plb::getForcesFromLattice(lattice, wrapper, units);
    }
    std::vector<double> id;
    plb::getScalarQuantityFromDynamics(lattice, plb::ParticleId, id);
    long cells1 = 0, cells2 = 0;
    for (double t : id) { cells1 += t == 1.0; cells2 += t == 2.0; }
    const double f1 = std::fabs(wrapper.fix.f[0][0]), f2 = std::fabs(wrapper.fix.f[1][0]);
    const double t2 = std::fabs(wrapper.fix.t[1][0]) + std::fabs(wrapper.fix.t[1][1]) + std::fabs(wrapper.fix.t[1][2]);
    std::printf("exclude=%d list=%zu cells(tag1)=%ld cells(tag2)=%ld |Fx1|=%.6e |Fx2|=%.6e |T2|=%.6e\n", exclude,
                lattice.r.size(), cells1, cells2, f1, f2, t2);
    bool ok = cells1 > 0 && f1 > 0.0;
    if (exclude) ok = ok && lattice.r.size() == 1 && lattice.tag[0] == 1 && cells2 == 0 && f2 == 0.0 && t2 == 0.0;
    else ok = ok && lattice.r.size() == 2 && cells2 > 0 && f2 > 0.0;
    return ok ? 0 : 1;
}

int main() {
    try {
        const int a = run(true), b = run(false);
        return (a == 0 && b == 0) ? 0 : 1;
    } catch (std::exception const& e) {
        std::fprintf(stderr, "exclude_type_check: %s\n", e.what());
        return std::strstr(e.what(), "no suitable CUDA device") ? 77 : 1;
    }
}
