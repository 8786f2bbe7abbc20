// Sedimenting sphere (the plain-method case): D3Q19 BGK PSM lattice of
// 60 x 60 x 180 cells with half-way bounce-back walls, tau = 0.6, fluid at rest;
// one sphere of radius 5 lattice units released on the axis at z = 150 with
// density ratio 1.5 under gravity 1e-5 lattice units per step^2 (buoyancy
// reduced as in examples/sedimentingSphere/in.lbdem:41-42), 10 DEM substeps
// per lattice step (examples/sedimentingSphere/sedimentingSphere.cpp:168).
//
// The coupling loop is the reference's (sedimentingSphere.cpp:212-238) on the
// GB300 lattice through include/lbdem_gpu.h and plb/lbdem_plb.h; the particle
// is advanced by the LIGGGHTS stand-in of dem_standin.h.  Lattice units
// throughout (PhysUnits3D with unit scales; physical position = lattice + 1/2).
//
// usage: sedimenting_sphere [steps=4000] [fp64|fp32] [trace=coords.txt] [every=10]
// The trace has the columns of the reference's fix print (in2.lbdem:16-26):
// t z vz fz.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "dem_standin.h"
#include "lbdem_plb.h"
#include "physunits_gpu.h"

int main(int argc, char** argv) {
    const long steps = argc > 1 ? std::atol(argv[1]) : 4000;
    const bool fp32 = argc > 2 && std::strcmp(argv[2], "fp32") == 0;
    const char* trace = argc > 3 ? argv[3] : "coords.txt";
    const long every = argc > 4 ? std::atol(argv[4]) : 10;
    const int nx = 60, ny = 60, nz = 180;
    const double tau = 0.6, radius = 5.0, rho_s = 1.5, rho_f = 1.0, g = 1e-5;
    const int demSubsteps = 10;

    plb::GpuLattice3D::Options o;
    o.precision = fp32 ? LBDEM_PREC_FP32_DEV : LBDEM_PREC_FP64;
    o.maxParticles = 16;
    o.maxTag = 16;
    o.maxRadius = 8.0;
    try {
        plb::GpuLattice3D lattice(nx, ny, nz, 1.0 / tau, o);
        lattice.initialize();
        plb::PhysUnits3D<double> units(1.0, 1.0, (tau - 0.5) / 3.0, nx, ny, nz, 1, 1.0, rho_f);

        LiggghtsCouplingWrapper wrapper;
        wrapper.dt = 1.0 / demSubsteps;
        wrapper.gravity[2] = -g * (rho_s - rho_f) / rho_s;
        const double p0[3] = {30.5, 30.5, 150.5}, v0[3] = {0, 0, 0};
        wrapper.atom.add(p0, v0, radius, rho_s, 1, 1);
        wrapper.sync();

        std::FILE* out = std::fopen(trace, "w");
        if (!out) { std::perror(trace); return 2; }
        std::fprintf(out, "# t z vz fz\n");
        const auto t0 = std::chrono::steady_clock::now();
        for (long iT = 0; iT < steps; ++iT) {
            plb::setSpheresOnLattice(lattice, wrapper, units, false);
            lattice.collideAndStream();
            plb::getForcesFromLattice(lattice, wrapper, units);
            wrapper.run(demSubsteps);
            if (iT % every == 0)
                std::fprintf(out, "%ld %.17g %.17g %.17g\n", iT, units.getLbPosition(wrapper.atom.x[0][2]),
                             wrapper.atom.v[0][2], wrapper.fix.f[0][2]);
        }
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::fclose(out);
        std::printf("{\"steps\": %ld, \"seconds\": %.4f, \"MLUPS\": %.2f, \"z\": %.10g, \"vz\": %.10g}\n", steps,
                    secs, (double)nx * ny * nz * steps / secs / 1e6, units.getLbPosition(wrapper.atom.x[0][2]),
                    wrapper.atom.v[0][2]);
    } catch (std::exception const& e) {
        std::fprintf(stderr, "sedimenting_sphere: %s\n", e.what());
        return std::strstr(e.what(), "no suitable CUDA device") ? 77 : 1;
    }
    return 0;
}
