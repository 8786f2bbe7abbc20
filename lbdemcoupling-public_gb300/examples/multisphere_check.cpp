// Two spheres through the C++ shim with LBDEM_USE_MULTISPHERE: one belongs to a
// multisphere body (tag 1), one is free (tag 2); both spin.  After
// setSpheresOnLattice the particle surface velocity of every cell the member
// covers must equal its translation velocity (angular velocity ignored,
// src/ibDataExchangeWrappers3D.hh:88-104), while the free sphere's cells see
// v + w x (cell - centre).
//
// usage: multisphere_check    (exit 0: pass, 1: fail, 77: no suitable GPU)
#define LBDEM_USE_MULTISPHERE 1
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dem_standin.h"
#include "lbdem_plb.h"
#include "physunits_gpu.h"

int main() {
    const int n = 32;
    try {
        plb::GpuLattice3D::Options o;
        o.periodic[0] = o.periodic[1] = o.periodic[2] = true;
        o.maxParticles = 8;
        o.maxTag = 8;
        o.maxRadius = 8.0;
        plb::GpuLattice3D lattice(n, n, n, 1.0 / 0.6, o);
        plb::PhysUnits3D<double> units(1.0, 1.0, 0.1 / 3.0, n, n, n, 1, 1.0, 1.0);
        LiggghtsCouplingWrapper wrapper;
        LAMMPS_NS::FixMultisphere ms;
        ms.body_of_tag = {-1, 0, -1};   // tag 1 -> body 0, tag 2 free
        wrapper.modify.multisphere = &ms;
        const double p1[3] = {8.5, 8.5, 8.5}, v1[3] = {0.01, -0.02, 0.005};
        const double p2[3] = {22.5, 22.5, 22.5}, v2[3] = {-0.01, 0.0, 0.02};
        wrapper.atom.add(p1, v1, 4.0, 1.5, 1, 1);
        wrapper.atom.add(p2, v2, 4.0, 1.5, 2, 1);
        for (int i = 0; i < 2; ++i)
            for (int d = 0; d < 3; ++d) wrapper.atom.omega[i][d] = 0.003 * (d + 1);
        wrapper.sync();
        plb::setSpheresOnLattice(lattice, wrapper, units, false);
        const size_t N = (size_t)n * n * n;
        std::vector<double> up(3 * N);
        std::vector<int32_t> id(N);
        lattice.check(lbdem_get_field(lattice.handle(), LBDEM_FIELD_PARTICLE_VELOCITY, up.data()));
        lattice.check(lbdem_get_field(lattice.handle(), LBDEM_FIELD_PARTICLE_ID, id.data()));
        double dev1 = 0, spin2 = 0;
        long c1 = 0, c2 = 0;
        for (size_t c = 0; c < N; ++c) {
            if (id[c] == 1) {
                for (int d = 0; d < 3; ++d) dev1 = std::fmax(dev1, std::fabs(up[d * N + c] - units.getLbVel(v1[d])));
                ++c1;
            } else if (id[c] == 2) {
                for (int d = 0; d < 3; ++d) spin2 = std::fmax(spin2, std::fabs(up[d * N + c] - units.getLbVel(v2[d])));
                ++c2;
            }
        }
        std::printf("{\"member_cells\": %ld, \"member_max_dev\": %g, \"free_cells\": %ld, \"free_max_spin\": %g}\n",
                    c1, dev1, c2, spin2);
        return (c1 > 0 && c2 > 0 && dev1 == 0.0 && spin2 > 1e-3) ? 0 : 1;
    } catch (std::exception const& e) {
        std::fprintf(stderr, "multisphere_check: %s\n", e.what());
        return std::strstr(e.what(), "no suitable CUDA device") ? 77 : 1;
    }
}
