// A pressure-driven periodic channel (the loop of
// examples/showcaseRectChannel/showcaseRectChannel.cpp:253-273) through the C++
// shim: x periodic, walls in y and z, Poiseuille profile and pressure gradient at
// start, one sphere held at rest on the axis.  The reference's per-step
// computeAverageDensity + ZhangPeriodicPressureFunctional3D pair is written
// both ways: explicitly (mode "explicit") and as the fused drop (mode "fused").
//
// usage: channel [steps=300] [explicit|fused]
// Prints the mean x velocity of the fluid, the x force on the sphere and, through
// the shim's field export (the reference's Get{Scalar,Vector}QuantityFromDynamics
// functionals), the cells the sphere covers, those it owns and the largest
// surface speed (zero: the sphere is held at rest).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "dem_standin.h"
#include "lbdem_plb.h"
#include "physunits_gpu.h"

struct Box {
    long x0, x1, y0, y1, z0, z1;
};

int main(int argc, char** argv) {
    const long steps = argc > 1 ? std::atol(argv[1]) : 300;
    const bool fused = !(argc > 2 && std::strcmp(argv[2], "explicit") == 0);
    const int nx = 64, ny = 24, nz = 24;
    const double rhoHi = 1.0, rhoLo = 0.999, uMax = 0.01;
    try {
        plb::GpuLattice3D::Options o;
        o.periodic[0] = true;
        o.maxParticles = 4;
        o.maxTag = 4;
        o.maxRadius = 8.0;
        plb::GpuLattice3D lattice(nx, ny, nz, 1.0 / 0.6, o);
        lattice.initializePoiseuille(rhoHi, rhoLo, uMax, nx - 1, ny, nz, 0);
        plb::PhysUnits3D<double> units(1.0, 1.0, 0.1 / 3.0, nx, ny, nz, 1, 1.0, 1.0);
        LiggghtsCouplingWrapper wrapper;
        const double p0[3] = {32.5, 12.5, 12.5}, v0[3] = {0, 0, 0};
        wrapper.atom.add(p0, v0, 4.0, 1.5, 1, 1);
        wrapper.sync();
        const Box inlet{0, 0, 1, ny - 2, 1, nz - 2}, outlet{nx - 1, nx - 1, 1, ny - 2, 1, nz - 2};
        if (fused) lattice.setPressureDrop(inlet, outlet, rhoHi, rhoLo, 0);
        for (long iT = 0; iT < steps; ++iT) {
            plb::setSpheresOnLattice(lattice, wrapper, units, iT == 0);
            if (fused) {
                lattice.collideAndStream();
            } else {
                const double rhoAvgIn = plb::computeAverageDensity(lattice, inlet);
                const double rhoAvgOut = plb::computeAverageDensity(lattice, outlet);
                lattice.collideAndStream();
                plb::applyZhangPeriodicPressure(lattice, inlet, rhoHi, rhoAvgOut, 0, 1);
                plb::applyZhangPeriodicPressure(lattice, outlet, rhoLo, rhoAvgIn, 0, -1);
            }
            plb::getForcesFromLattice(lattice, wrapper, units);
        }
        const size_t N = (size_t)nx * ny * nz;
        std::vector<double> u(3 * N);
        lattice.check(lbdem_get_field(lattice.handle(), LBDEM_FIELD_VELOCITY, u.data()));
        double ux = 0;
        for (size_t c = 0; c < N; ++c) ux += u[c];
        std::vector<double> sf, id, up;
        plb::getScalarQuantityFromDynamics(lattice, plb::SolidFraction, sf);
        plb::getScalarQuantityFromDynamics(lattice, plb::ParticleId, id);
        plb::getVectorQuantityFromDynamics(lattice, plb::ParticleVelocity, up);
        long solid = 0, owned = 0;
        double upMax = 0;
        for (size_t c = 0; c < N; ++c) {
            solid += sf[c] > 0;
            owned += id[c] == 1.0;
            for (int d = 0; d < 3; ++d) upMax = std::max(upMax, std::abs(up[3 * c + d]));
        }
        std::printf("{\"mode\": \"%s\", \"steps\": %ld, \"mean_ux\": %.17g, \"fx\": %.17g, \"solid_cells\": %ld, "
                    "\"owned_cells\": %ld, \"max_up\": %.17g}\n",
                    fused ? "fused" : "explicit", steps, ux / (double)N, wrapper.fix.f[0][0], solid, owned, upMax);
    } catch (std::exception const& e) {
        std::fprintf(stderr, "channel: %s\n", e.what());
        return std::strstr(e.what(), "no suitable CUDA device") ? 77 : 1;
    }
    return 0;
}
