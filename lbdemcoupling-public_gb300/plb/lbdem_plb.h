// Host-side C++ surface of the GB300 PSM step in the reference's vocabulary.
//
// The LBDEMcoupling coupling loop (examples/sedimentingSphere/sedimentingSphere.cpp:212-238)
//
//     setSpheresOnLattice(lattice, wrapper, units, initVel);
//     lattice.collideAndStream();
//     getForcesFromLattice(lattice, wrapper, units);
//     wrapper.run(demSubsteps);
//
// compiles unchanged against this header with `lattice` a plb::GpuLattice3D.
// The particle side is read from and written to LIGGGHTS exactly as the
// reference's wrappers do (src/ibDataExchangeWrappers3D.hh:33-246): sphere list
// = local atoms then ghost images, excludeType filter, PhysUnits3D conversions,
// fix arrays zeroed then accumulated through atom->map(tag), reverse
// communication.  The wrapper and units are template parameters, so the same
// code builds against LIGGGHTS (LiggghtsCouplingWrapper, FixLbCouplingOnetoone)
// or against any stand-in with the same members.
#ifndef LBDEM_PLB_H
#define LBDEM_PLB_H

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "lbdem_gpu.h"

namespace plb {

// Construction options of GpuLattice3D.
struct GpuLatticeOptions {
    bool periodic[3] = {false, false, false};   // Palabos lattice.periodicity().toggle(d, ...)
    int32_t precision = LBDEM_PREC_FP64;         // LBDEM_PREC_FP32_DEV for the deviation form
    int32_t maxParticles = 4096;                 // list capacity, ghost images included
    int32_t maxTag = 1 << 20;
    double maxRadius = 32.0;                     // lattice units
    double bodyForce[3] = {0, 0, 0};             // Guo forcing (not part of the reference)
    int32_t device = 0;
    int32_t flags = 0;
};

// A D3Q19 PSM lattice resident on the GPU; replaces
// MultiBlockLattice3D<T, D3Q19Descriptor> populated with
// IBcompositeDynamics<T, D3Q19Descriptor>(new BGKdynamics(omega)).
class GpuLattice3D {
public:
    using Options = GpuLatticeOptions;

    GpuLattice3D(int32_t nx, int32_t ny, int32_t nz, double omega, Options const& o = Options()) {
        lbdem_config c;
        lbdem_config_default(&c);
        c.nx = nx; c.ny = ny; c.nz = nz;
        c.omega = omega;
        for (int d = 0; d < 3; ++d) { c.periodic[d] = o.periodic[d] ? 1 : 0; c.body_force[d] = o.bodyForce[d]; }
        c.precision = o.precision;
        c.max_particles = o.maxParticles;
        c.max_tag = o.maxTag;
        c.max_radius = o.maxRadius;
        c.device = o.device;
        c.flags = o.flags;
        const lbdem_status s = lbdem_create(&c, &h_);
        if (s != LBDEM_OK) throw std::runtime_error(std::string("lbdem_create: ") + lbdem_status_string(s));
        nx_ = nx; ny_ = ny; nz_ = nz;
        prec_ = o.precision;
    }
    ~GpuLattice3D() { if (h_) lbdem_destroy(h_); }
    GpuLattice3D(GpuLattice3D const&) = delete;
    GpuLattice3D& operator=(GpuLattice3D const&) = delete;

    int32_t getNx() const { return nx_; }
    int32_t getNy() const { return ny_; }
    int32_t getNz() const { return nz_; }
    size_t cells() const { return (size_t)nx_ * ny_ * nz_; }
    int32_t precision() const { return prec_; }
    lbdem_handle* handle() { return h_; }

    // lattice.initialize() of a lattice at rest, or initializeAtEquilibrium with uniform rho, u.
    void initialize(double rho = 1.0, double ux = 0, double uy = 0, double uz = 0) {
        const double u[3] = {ux, uy, uz};
        check(lbdem_init_equilibrium(h_, rho - 1.0, u));
    }
    void collideAndStream() { check(lbdem_collide_and_stream(h_)); }

    // initializeAtEquilibrium(lattice, box, PressureGradient<T>(pHi, pLo, n, dimension))
    // and (..., PoiseuilleProfileAndPressureGradient<T>(pHi, pLo, uMax, nx, ny, nz, dimension))
    // over the whole lattice (src/periodicPressureFunctionals3D.hh:238-298).
    void initializePressureGradient(double pHi, double pLo, int32_t n, int32_t dimension) {
        int32_t nn[3] = {n, n, n};
        check(lbdem_init_profile(h_, LBDEM_PROFILE_PRESSURE_GRADIENT, pHi, pLo, 0.0, nn, dimension));
    }
    void initializePoiseuille(double pHi, double pLo, double uMax, int32_t nx, int32_t ny, int32_t nz,
                              int32_t dimension) {
        const int32_t nn[3] = {nx, ny, nz};
        check(lbdem_init_profile(h_, LBDEM_PROFILE_POISEUILLE, pHi, pLo, uMax, nn, dimension));
    }

    // The pressure-driven periodic channel of examples/showcaseRectChannel (:253-273)
    // done inside every collideAndStream: inlet and outlet are Box3D-like (x0..z1).
    template <class Box>
    void setPressureDrop(Box const& inlet, Box const& outlet, double rhoIn, double rhoOut, int32_t dimension,
                         int32_t inDirection = 1, int32_t outDirection = -1) {
        lbdem_pressure_drop d;
        d.dimension = dimension;
        box6(inlet, d.inlet);
        box6(outlet, d.outlet);
        d.in_direction = inDirection;
        d.out_direction = outDirection;
        d.rho_in = rhoIn;
        d.rho_out = rhoOut;
        check(lbdem_set_pressure_drop(h_, &d));
    }

    template <class Box>
    static void box6(Box const& b, int32_t out[6]) {
        out[0] = (int32_t)b.x0; out[1] = (int32_t)b.x1; out[2] = (int32_t)b.y0;
        out[3] = (int32_t)b.y1; out[4] = (int32_t)b.z0; out[5] = (int32_t)b.z1;
    }

    void check(lbdem_status s) const {
        if (s != LBDEM_OK)
            throw std::runtime_error(std::string(lbdem_status_string(s)) + ": " + lbdem_last_error(h_));
    }

    // Particle list of the last setSpheresOnLattice (lattice units), kept for the force read.
    std::vector<double> x, v, w, r, F, T;
    std::vector<int32_t> tag;

private:
    lbdem_handle* h_ = nullptr;
    int32_t nx_ = 0, ny_ = 0, nz_ = 0;
    int32_t prec_ = LBDEM_PREC_FP64;
};

// setSpheresOnLattice, src/ibDataExchangeWrappers3D.hh:33-146.  With
// LBDEM_USE_MULTISPHERE defined (LIGGGHTS with fix multisphere, :52-115), a sphere
// that belongs to a multisphere body enters with its own velocity and no angular
// velocity (its surface velocity is then the translation of its own centre); the
// including code provides LAMMPS_NS::FixMultisphere with belongs_to(tag).
template <class Wrapper, class Units>
void setSpheresOnLattice(GpuLattice3D& lattice, Wrapper& wrapper, Units const& units,
                         std::vector<long>& excludeType, bool initVelFlag) {
    auto* atom = wrapper.lmp->atom;
    const long nPart = atom->nlocal + atom->nghost;
#ifdef LBDEM_USE_MULTISPHERE
    LAMMPS_NS::FixMultisphere* fixMultisphere = nullptr;
    if (wrapper.lmp->modify->n_fixes_style("multisphere"))
        fixMultisphere =
            static_cast<LAMMPS_NS::FixMultisphere*>(wrapper.lmp->modify->find_fix_style("multisphere", 0));
#endif
    lattice.x.clear(); lattice.v.clear(); lattice.w.clear(); lattice.r.clear(); lattice.tag.clear();
    for (long iS = 0; iS < nPart; ++iS) {
        const long type = (long)atom->type[iS];
        if (std::find(excludeType.begin(), excludeType.end(), type) != excludeType.end()) continue;
#ifdef LBDEM_USE_MULTISPHERE
        const bool member = fixMultisphere && fixMultisphere->belongs_to(atom->tag[iS]) > -1;
#else
        const bool member = false;
#endif
        for (int i = 0; i < 3; ++i) {
            lattice.x.push_back(units.getLbPosition(atom->x[iS][i]));
            lattice.v.push_back(units.getLbVel(atom->v[iS][i]));
            lattice.w.push_back(member ? 0.0 : units.getLbFreq(atom->omega[iS][i]));
        }
        lattice.r.push_back(units.getLbLength(atom->radius[iS]));
        lattice.tag.push_back((int32_t)atom->tag[iS]);
    }
    const int32_t n = (int32_t)lattice.r.size();
    lattice.check(lbdem_set_particles(lattice.handle(), n, lattice.x.data(), lattice.v.data(), lattice.w.data(),
                                      lattice.r.data(), lattice.tag.data(), initVelFlag ? 1 : 0));
}

template <class Wrapper, class Units>
void setSpheresOnLattice(GpuLattice3D& lattice, Wrapper& wrapper, Units const& units, bool initVelFlag) {
    std::vector<long> none;
    setSpheresOnLattice(lattice, wrapper, units, none, initVelFlag);
}

// Palabos computeAverageDensity(lattice, box): 1 + mean rhoBar over the box.
template <class Box>
double computeAverageDensity(GpuLattice3D& lattice, Box const& box) {
    int32_t b[6];
    GpuLattice3D::box6(box, b);
    double rho = 0;
    lattice.check(lbdem_average_density(lattice.handle(), b, &rho));
    return rho;
}

// applyProcessingFunctional(new ZhangPeriodicPressureFunctional3D<T,D>(rhoTarget, rhoAvg,
// dimension, direction), box, lattice), src/periodicPressureFunctionals3D.hh:121-159.
template <class Box>
void applyZhangPeriodicPressure(GpuLattice3D& lattice, Box const& box, double rhoTarget, double rhoAvg,
                                int32_t dimension, int32_t direction) {
    int32_t b[6];
    GpuLattice3D::box6(box, b);
    lattice.check(lbdem_zhang_rescale(lattice.handle(), b, dimension, direction, rhoTarget, rhoAvg));
}

// Per-cell quantities of the reference's field export (src/ibDataWritingFunctionals3D.h:30-31).
enum IBscalarQuantity { SolidFraction, ParticleId };
enum IBvectorQuantity { ParticleVelocity, HydrodynamicForce };

// applyProcessingFunctional(new GetScalarQuantityFromDynamicsFunctional<T, DESCRIPTOR, T>(which),
// lattice.getBoundingBox(), lattice, field), src/ibDataWritingFunctionals3D.hh:30-60, over the
// whole lattice: out[(x ny + y) nz + z] as doubles (the owner tag converted like the
// functional's cast).
inline void getScalarQuantityFromDynamics(GpuLattice3D& lattice, IBscalarQuantity which, std::vector<double>& out) {
    const size_t N = lattice.cells();
    out.assign(N, 0.0);
    if (which == SolidFraction) {
        lattice.check(lbdem_get_field(lattice.handle(), LBDEM_FIELD_SOLID_FRACTION, out.data()));
        return;
    }
    std::vector<int32_t> id(N);
    lattice.check(lbdem_get_field(lattice.handle(), LBDEM_FIELD_PARTICLE_ID, id.data()));
    for (size_t c = 0; c < N; ++c) out[c] = (double)id[c];
}

// applyProcessingFunctional(new GetVectorQuantityFromDynamicsFunctional<T, DESCRIPTOR, T, 3>(which),
// ...), src/ibDataWritingFunctionals3D.hh:68-114: out[3 cell + d], the layout of a
// TensorField3D<T, 3>.  HydrodynamicForce needs Options::flags with LBDEM_FLAG_CELL_FORCE.
inline void getVectorQuantityFromDynamics(GpuLattice3D& lattice, IBvectorQuantity which, std::vector<double>& out) {
    const size_t N = lattice.cells();
    const int32_t field = which == ParticleVelocity ? LBDEM_FIELD_PARTICLE_VELOCITY : LBDEM_FIELD_HYDRO_FORCE;
    out.assign(3 * N, 0.0);
    if (lattice.precision() == LBDEM_PREC_FP64) {
        std::vector<double> planar(3 * N);
        lattice.check(lbdem_get_field(lattice.handle(), field, planar.data()));
        for (size_t c = 0; c < N; ++c)
            for (int d = 0; d < 3; ++d) out[3 * c + d] = planar[d * N + c];
    } else {
        std::vector<float> planar(3 * N);
        lattice.check(lbdem_get_field(lattice.handle(), field, planar.data()));
        for (size_t c = 0; c < N; ++c)
            for (int d = 0; d < 3; ++d) out[3 * c + d] = (double)planar[d * N + c];
    }
}

// getForcesFromLattice, src/ibDataExchangeWrappers3D.hh:160-246.  FixType is the
// LIGGGHTS coupling fix (LAMMPS_NS::FixLbCouplingOnetoone).
template <class FixType, class Wrapper, class Units>
void getForcesFromLattice(GpuLattice3D& lattice, Wrapper& wrapper, Units const& units) {
    auto* atom = wrapper.lmp->atom;
    const long nPart = atom->nlocal + atom->nghost;
    if (nPart == 0) return;   // no particles - no work (:174)
    const int32_t n = (int32_t)lattice.r.size();
    lattice.F.assign(3 * (size_t)n, 0.0);
    lattice.T.assign(3 * (size_t)n, 0.0);
    lattice.check(lbdem_get_forces(lattice.handle(), n, lattice.F.data(), lattice.T.data()));
    FixType* couplingFix = dynamic_cast<FixType*>(wrapper.lmp->modify->find_fix_style("couple/lb/onetoone", 0));
    if (!couplingFix) throw std::runtime_error("getForcesFromLattice: fix couple/lb/onetoone not found");
    double** f_liggghts = couplingFix->get_force_ptr();
    double** t_liggghts = couplingFix->get_torque_ptr();
    for (long iPart = 0; iPart < nPart; ++iPart)
        for (int j = 0; j < 3; ++j) { f_liggghts[iPart][j] = 0; t_liggghts[iPart][j] = 0; }
    for (int32_t k = 0; k < n; ++k) {
        const int ind = atom->map(lattice.tag[k]);
        for (int j = 0; j < 3; ++j) {
            f_liggghts[ind][j] += units.getPhysForce(lattice.F[3 * (size_t)k + j]);
            t_liggghts[ind][j] += units.getPhysTorque(lattice.T[3 * (size_t)k + j]);
        }
    }
    couplingFix->comm_force_torque();
}

}  // namespace plb

#endif  // LBDEM_PLB_H
