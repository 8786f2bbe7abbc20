// Host-side C++ surface of the GB300 PSM step in the reference's vocabulary.
//
// A Palabos/LIGGGHTS case driver of LBDEMcoupling keeps its coupling code as is
// (examples/sedimentingSphere/sedimentingSphere.cpp:176-238):
//
//     defineDynamics(lattice, lattice.getBoundingBox(), new DYNAMICS);   // IBcompositeDynamics<T,D>
//     lattice.periodicity().toggleAll(false);
//     lattice.initialize();
//     for (plint iT = 0; iT < maxSteps; ++iT) {
//       setSpheresOnLattice(lattice, wrapper, units, false);
//       lattice.collideAndStream();
//       getForcesFromLattice(lattice, wrapper, units);
//       wrapper.run(demSubsteps);
//     }
//
// with `lattice` a plb::GpuLattice3D.  The reference's types are here under
// their names and template signatures: IBcompositeDynamics<T,Descriptor>
// (src/ibCompositeDynamics3D.h:32-66), IBdynamicsParticleData<T,Descriptor>
// (src/ibDynamicsParticleData.h:26-37), ParticleData<T> (src/ibProcessors3D.h:28-32),
// the processing functionals SetSingleSphere3D, SumForceTorque3D and
// AttributeFunctional (src/ibProcessors3D.h:34-94) with applyProcessingFunctional,
// and the free functions setSpheresOnLattice / getForcesFromLattice
// (src/ibDataExchangeWrappers3D.h:37-53).  The particle side is read from and
// written to LIGGGHTS exactly as the reference's wrappers do
// (src/ibDataExchangeWrappers3D.hh:33-246): sphere list = local atoms then ghost
// images, excludeType filter, PhysUnits3D conversions, fix arrays zeroed then
// accumulated through atom->map(tag), reverse communication.  The wrapper and
// units are template parameters, so the same code builds against LIGGGHTS
// (LiggghtsCouplingWrapper, LAMMPS_NS::FixLbCouplingOnetoone) or any stand-in
// with the same members.  No Palabos header is needed; where the driver
// includes Palabos, its Box3D, BGKdynamics and descriptors interoperate.
#ifndef LBDEM_PLB_H
#define LBDEM_PLB_H

#include <algorithm>
#include <array>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "lbdem_gpu.h"

// The LIGGGHTS coupling fix getForcesFromLattice writes into
// (src/ibDataExchangeWrappers3D.hh:191-195); complete where it is used.
namespace LAMMPS_NS {
class FixLbCouplingOnetoone;
}

namespace plb {

// The lattice descriptor the shim instantiates the reference's templates with
// (D3Q19 only; where Palabos is included, descriptors::D3Q19Descriptor works too).
template <typename T>
struct GpuDescriptor {
    static const int d = 3, q = 19;
};

// Palabos' Box3D as the GPU lattice reports it (inclusive cell ranges); converts
// to any box type constructible from six integers, Palabos' Box3D included.
struct GpuBox3D {
    std::ptrdiff_t x0, x1, y0, y1, z0, z1;
    template <class Box>
    operator Box() const {
        return Box(x0, x1, y0, y1, z0, z1);
    }
};

// IBdynamicsParticleData, src/ibDynamicsParticleData.h:26-37: the per-cell
// coupling state of the reference.  On the GPU this state is the voxel word
// (sub-cell count and owner tag) and the surface velocity; the struct keeps the
// reference's layout for code that names it (lbdem_get_field reads the fields).
template <typename T, template <typename U> class Descriptor>
struct IBdynamicsParticleData {
    IBdynamicsParticleData() : partId(0), solidFraction(0.), uPart{{0, 0, 0}}, hydrodynamicForce{{0, 0, 0}} {}
    std::ptrdiff_t partId;
    T solidFraction;
    std::array<T, 3> uPart;
    std::array<T, 3> hydrodynamicForce;
};

// ParticleData<T>, src/ibProcessors3D.h:28-32.
template <typename T>
struct ParticleData {
    typedef std::vector<std::array<T, 3>> ParticleDataArrayVector;
    typedef std::vector<T> ParticleDataScalarVector;
};

// IBcompositeDynamics<T,Descriptor>, src/ibCompositeDynamics3D.h:32-66: the
// Noble-Torczynski PSM dynamics around a base BGK dynamics.  Here it is the
// description a GpuLattice3D is built from or given by defineDynamics: it takes
// ownership of the base dynamics (as Palabos' CompositeDynamics does) and keeps
// its relaxation frequency; the collision itself runs on the GPU.
template <typename T, template <typename U> class Descriptor>
class IBcompositeDynamics {
public:
    template <class BaseDynamics>
    explicit IBcompositeDynamics(BaseDynamics* baseDynamics_, bool automaticPrepareCollision_ = true)
        : omega_(baseDynamics_ ? (double)baseDynamics_->getOmega() : 0.0),
          automaticPrepareCollision(automaticPrepareCollision_) {
        delete baseDynamics_;
    }
    IBcompositeDynamics(IBcompositeDynamics const&) = default;
    IBcompositeDynamics* clone() const { return new IBcompositeDynamics(*this); }
    // registered as "IBcomposite" in the reference (src/ibCompositeDynamics3D.hh:29-30)
    static const char* name() { return "IBcomposite"; }
    double getOmega() const { return omega_; }

    IBdynamicsParticleData<T, Descriptor> particleData;

private:
    double omega_;
    bool automaticPrepareCollision;
};

// SetSingleSphere3D<T,Descriptor>, src/ibProcessors3D.h:34-58: one sphere's
// voxelization.  Like the reference it holds pointers to the caller's arrays;
// applyProcessingFunctional reads them and queues the sphere on the lattice,
// whose pending list is voxelized in list order (one GPU pass, the same result
// as applying the spheres one after another) before the next collideAndStream
// or read of lattice state.
template <typename T, template <typename U> class Descriptor>
struct SetSingleSphere3D {
    SetSingleSphere3D(T* x_, T* v_, T* omega_, T* com_, T r_, int id_, bool initVelFlag_ = false)
        : x(x_), v(v_), omega(omega_), com(com_), r(r_), id(id_), initVelFlag(initVelFlag_) {}
    SetSingleSphere3D(SetSingleSphere3D const& orig) = default;
    // src/ibProcessors3D.h:43-45: the box [x - r - 2, x + r + 2], each bound converted
    // to an integer by truncation
    GpuBox3D getBoundingBox() const {
        return GpuBox3D{(std::ptrdiff_t)(x[0] - r - 2), (std::ptrdiff_t)(x[0] + r + 2),
                        (std::ptrdiff_t)(x[1] - r - 2), (std::ptrdiff_t)(x[1] + r + 2),
                        (std::ptrdiff_t)(x[2] - r - 2), (std::ptrdiff_t)(x[2] + r + 2)};
    }
    SetSingleSphere3D* clone() const { return new SetSingleSphere3D(*this); }

    T *x, *v, *omega, *com, r;   // com: centre of mass
    int id;
    bool initVelFlag;
};

// AttributeFunctional, src/ibProcessors3D.h:60-74: applied after the spheres;
// here it completes the pending voxelization.
template <typename T, template <typename U> class Descriptor>
struct AttributeFunctional {
    AttributeFunctional* clone() const { return new AttributeFunctional(*this); }
};

// SumForceTorque3D<T,Descriptor>, src/ibProcessors3D.h:76-94: per-particle force
// and torque of the last collideAndStream, added into force[3 ind + d] and
// torque[3 ind + d] with ind = atom->map(id) (src/ibProcessors3D.hh:225).  The
// GPU sums them in the collision pass, with the torque arm taken from the
// positions of the last voxelized sphere list (the values the reference's x
// vector holds: units.getLbPosition(atom->x)).
template <typename T, template <typename U> class Descriptor>
struct SumForceTorque3D {
    template <class Wrapper>
    SumForceTorque3D(typename ParticleData<T>::ParticleDataArrayVector& x_, T* force_, T* torque_, Wrapper& wrapper)
        : x(&x_), force(force_), torque(torque_), map([&wrapper](long tag) -> long {
              return (long)wrapper.lmp->atom->map((int)tag);
          }) {}
    SumForceTorque3D(SumForceTorque3D const&) = default;
    SumForceTorque3D* clone() const { return new SumForceTorque3D(*this); }

    typename ParticleData<T>::ParticleDataArrayVector* x;
    T *force, *torque;
    std::function<long(long)> map;
};

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
        create(nx, ny, nz, omega, o);
    }
    // The reference's construction with its background dynamics,
    // MultiBlockLattice3D<T,D>(..., new IBcompositeDynamics<T,D>(new BGKdynamics<T,D>(omega)))
    // (sedimentingSphere.cpp:172-178): the lattice takes ownership of the dynamics.
    template <typename T, template <typename U> class Descriptor>
    GpuLattice3D(int32_t nx, int32_t ny, int32_t nz, IBcompositeDynamics<T, Descriptor>* dynamics,
                 Options const& o = Options()) {
        const double omega = dynamics ? dynamics->getOmega() : 0.0;
        delete dynamics;
        create(nx, ny, nz, omega, o);
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
    GpuBox3D getBoundingBox() const { return GpuBox3D{0, nx_ - 1, 0, ny_ - 1, 0, nz_ - 1}; }

    // lattice.periodicity().toggle(d, flag) / toggleAll(flag)
    class Periodicity {
    public:
        explicit Periodicity(GpuLattice3D& l) : l_(l) {}
        void toggle(int d, bool flag) {
            if (d < 0 || d > 2) throw std::invalid_argument("periodicity().toggle: axis 0, 1 or 2");
            l_.per_[d] = flag ? 1 : 0;
            l_.check(lbdem_set_periodic(l_.h_, l_.per_));
        }
        void toggleAll(bool flag) {
            for (int d = 0; d < 3; ++d) l_.per_[d] = flag ? 1 : 0;
            l_.check(lbdem_set_periodic(l_.h_, l_.per_));
        }
        bool get(int d) const { return l_.per_[d] != 0; }

    private:
        GpuLattice3D& l_;
    };
    Periodicity periodicity() { return Periodicity(*this); }

    void setOmega(double omega) { check(lbdem_set_omega(h_, omega)); }

    // lattice.initialize() of a lattice at rest, or initializeAtEquilibrium with uniform rho, u.
    void initialize(double rho = 1.0, double ux = 0, double uy = 0, double uz = 0) {
        const double u[3] = {ux, uy, uz};
        check(lbdem_init_equilibrium(h_, rho - 1.0, u));
    }
    void collideAndStream() {
        flushSpheres();
        check(lbdem_collide_and_stream(h_));
    }

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

    // The sphere list of the current pass (lattice units), queued by
    // SetSingleSphere3D and voxelized in list order by flushSpheres(); it stays
    // the list the force sums refer to until the next pass starts.
    void addSphere(const double xs[3], const double vs[3], const double ws[3], double rs, int32_t tagv,
                   bool initVel) {
        if (!open_) {
            x.clear(); v.clear(); w.clear(); r.clear(); tag.clear();
            open_ = true;
            initVel_ = initVel;
        } else if (initVel != initVel_) {
            throw std::invalid_argument("SetSingleSphere3D: one pass mixes initVelFlag values");
        }
        for (int d = 0; d < 3; ++d) { x.push_back(xs[d]); v.push_back(vs[d]); w.push_back(ws[d]); }
        r.push_back(rs);
        tag.push_back(tagv);
    }
    // Voxelizes the queued spheres (SetSingleSphere3D::process for each, in order).
    void flushSpheres() {
        if (!open_) return;
        open_ = false;
        check(lbdem_set_particles(h_, (int32_t)r.size(), x.data(), v.data(), w.data(), r.data(), tag.data(),
                                  initVel_ ? 1 : 0));
    }
    // Starts a pass with no sphere yet (stays empty when every sphere of a
    // setSpheresOnLattice is excluded).
    void beginPass(bool initVel) {
        x.clear(); v.clear(); w.clear(); r.clear(); tag.clear();
        open_ = true;
        initVel_ = initVel;
    }

    // Particle list of the last pass (lattice units), and its forces and torques.
    std::vector<double> x, v, w, r, F, T;
    std::vector<int32_t> tag;

private:
    void create(int32_t nx, int32_t ny, int32_t nz, double omega, Options const& o) {
        lbdem_config c;
        lbdem_config_default(&c);
        c.nx = nx; c.ny = ny; c.nz = nz;
        c.omega = omega;
        for (int d = 0; d < 3; ++d) {
            c.periodic[d] = o.periodic[d] ? 1 : 0;
            per_[d] = c.periodic[d];
            c.body_force[d] = o.bodyForce[d];
        }
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

    lbdem_handle* h_ = nullptr;
    int32_t nx_ = 0, ny_ = 0, nz_ = 0;
    int32_t prec_ = LBDEM_PREC_FP64;
    int32_t per_[3] = {0, 0, 0};
    bool open_ = false, initVel_ = false;
};

// defineDynamics(lattice, lattice.getBoundingBox(), new IBcompositeDynamics<T,D>(...))
// (sedimentingSphere.cpp:181): the relaxation frequency of every cell.  The GPU
// lattice has one dynamics for all cells, so the box must be the whole lattice.
template <class Box, typename T, template <typename U> class Descriptor>
void defineDynamics(GpuLattice3D& lattice, Box const& domain, IBcompositeDynamics<T, Descriptor>* dynamics) {
    int32_t b[6];
    GpuLattice3D::box6(domain, b);
    const double omega = dynamics ? dynamics->getOmega() : 0.0;
    delete dynamics;
    if (b[0] != 0 || b[2] != 0 || b[4] != 0 || b[1] != lattice.getNx() - 1 || b[3] != lattice.getNy() - 1 ||
        b[5] != lattice.getNz() - 1)
        throw std::invalid_argument("defineDynamics: the GPU lattice takes one dynamics for the whole lattice");
    lattice.setOmega(omega);
}

// applyProcessingFunctional(new SetSingleSphere3D<T,D>(x, v, omega, com, r, id, initVel), box, lattice)
// (src/ibDataExchangeWrappers3D.hh:134-135): queues the sphere (the box is the
// sphere's box within the lattice; the GPU clips it the same way).  With a
// centre of mass com other than x, the sphere enters with the velocity of its
// centre, v + omega x (x - com), so that v + omega x (cell - com) is kept.
template <typename T, template <typename U> class Descriptor, class Box>
void applyProcessingFunctional(SetSingleSphere3D<T, Descriptor>* f, Box const&, GpuLattice3D& lattice) {
    double xs[3], vs[3], ws[3];
    for (int d = 0; d < 3; ++d) { xs[d] = (double)f->x[d]; vs[d] = (double)f->v[d]; ws[d] = (double)f->omega[d]; }
    if (f->com != f->x) {
        const double a[3] = {xs[0] - (double)f->com[0], xs[1] - (double)f->com[1], xs[2] - (double)f->com[2]};
        vs[0] += ws[1] * a[2] - ws[2] * a[1];
        vs[1] += ws[2] * a[0] - ws[0] * a[2];
        vs[2] += ws[0] * a[1] - ws[1] * a[0];
    }
    const double rs = (double)f->r;
    const int32_t id = (int32_t)f->id;
    const bool iv = f->initVelFlag;
    delete f;
    lattice.addSphere(xs, vs, ws, rs, id, iv);
}

// applyProcessingFunctional(new AttributeFunctional<T,D>(), box, lattice)
// (src/ibDataExchangeWrappers3D.hh:143): the end of a pass.
template <typename T, template <typename U> class Descriptor, class Box>
void applyProcessingFunctional(AttributeFunctional<T, Descriptor>* f, Box const&, GpuLattice3D& lattice) {
    delete f;
    lattice.flushSpheres();
}

// applyProcessingFunctional(new SumForceTorque3D<T,D>(x, force, torque, wrapper), box, lattice)
// (src/ibDataExchangeWrappers3D.hh:183-190): the sums of the whole lattice.
template <typename T, template <typename U> class Descriptor, class Box>
void applyProcessingFunctional(SumForceTorque3D<T, Descriptor>* f, Box const&, GpuLattice3D& lattice) {
    lattice.flushSpheres();
    const int32_t n = (int32_t)lattice.r.size();
    lattice.F.assign(3 * (size_t)n, 0.0);
    lattice.T.assign(3 * (size_t)n, 0.0);
    const lbdem_status st = lbdem_get_forces(lattice.handle(), n, lattice.F.data(), lattice.T.data());
    if (st != LBDEM_OK) {
        delete f;
        lattice.check(st);
    }
    // list entry k holds the sums of its tag at the first entry carrying it (zero at ghost images)
    for (int32_t k = 0; k < n; ++k) {
        const long ind = f->map(lattice.tag[k]);
        if (ind < 0) continue;
        for (int d = 0; d < 3; ++d) {
            f->force[3 * ind + d] += (T)lattice.F[3 * (size_t)k + d];
            f->torque[3 * ind + d] += (T)lattice.T[3 * (size_t)k + d];
        }
    }
    delete f;
}

// setSpheresOnLattice, src/ibDataExchangeWrappers3D.hh:33-146: one
// SetSingleSphere3D per LIGGGHTS sphere (locals, then ghost images) not of an
// excluded type, then AttributeFunctional.  With LBDEM_USE_MULTISPHERE defined
// (LIGGGHTS with fix multisphere, :52-115), a sphere that belongs to a
// multisphere body enters with its own velocity and no angular velocity, as
// in the reference; the including code provides LAMMPS_NS::FixMultisphere
// with belongs_to(tag).
template <class Wrapper, class Units, class Int>
void setSpheresOnLattice(GpuLattice3D& lattice, Wrapper& wrapper, Units const& units,
                         std::vector<Int>& excludeType, bool initVelFlag) {
    auto* atom = wrapper.lmp->atom;
    const long nPart = (long)atom->nlocal + (long)atom->nghost;
#ifdef LBDEM_USE_MULTISPHERE
    LAMMPS_NS::FixMultisphere* fixMultisphere = nullptr;
    if (wrapper.lmp->modify->n_fixes_style("multisphere"))
        fixMultisphere =
            static_cast<LAMMPS_NS::FixMultisphere*>(wrapper.lmp->modify->find_fix_style("multisphere", 0));
#endif
    lattice.beginPass(initVelFlag);
    const GpuBox3D all = lattice.getBoundingBox();
    for (long iS = 0; iS < nPart; ++iS) {
        const Int type = (Int)atom->type[iS];
        if (std::find(excludeType.begin(), excludeType.end(), type) != excludeType.end()) continue;
#ifdef LBDEM_USE_MULTISPHERE
        const bool member = fixMultisphere && fixMultisphere->belongs_to(atom->tag[iS]) > -1;
#else
        const bool member = false;
#endif
        double x[3], v[3], omega[3];
        for (int i = 0; i < 3; ++i) {
            x[i] = units.getLbPosition(atom->x[iS][i]);
            v[i] = units.getLbVel(atom->v[iS][i]);
            omega[i] = member ? 0.0 : units.getLbFreq(atom->omega[iS][i]);
        }
        const double r = units.getLbLength(atom->radius[iS]);
        // the sphere centre is its centre of mass, as in both branches of the reference
        applyProcessingFunctional(new SetSingleSphere3D<double, GpuDescriptor>(x, v, omega, x, r, (int)atom->tag[iS],
                                                                               initVelFlag),
                                  all, lattice);
    }
    applyProcessingFunctional(new AttributeFunctional<double, GpuDescriptor>(), all, lattice);
}

template <class Wrapper, class Units>
void setSpheresOnLattice(GpuLattice3D& lattice, Wrapper& wrapper, Units const& units, bool initVelFlag) {
    std::vector<long> none;
    setSpheresOnLattice(lattice, wrapper, units, none, initVelFlag);
}

// Palabos computeAverageDensity(lattice, box): 1 + mean rhoBar over the box.
template <class Box>
double computeAverageDensity(GpuLattice3D& lattice, Box const& box) {
    lattice.flushSpheres();
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
    lattice.flushSpheres();
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
    lattice.flushSpheres();
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
    lattice.flushSpheres();
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

// getForcesFromLattice, src/ibDataExchangeWrappers3D.hh:160-246, called as in
// the reference's drivers: getForcesFromLattice(lattice, wrapper, units).  The
// per-particle sums of SumForceTorque3D, indexed by LIGGGHTS index, go into the
// fix couple/lb/onetoone arrays (zeroed first) in physical units, then the
// reverse communication.  FixType is LAMMPS_NS::FixLbCouplingOnetoone; it is a
// defaulted template parameter only so that the fix class need not be complete
// where this header is included.
template <class Wrapper, class Units, class FixType = LAMMPS_NS::FixLbCouplingOnetoone>
void getForcesFromLattice(GpuLattice3D& lattice, Wrapper& wrapper, Units const& units) {
    static std::vector<double> force, torque;
    static ParticleData<double>::ParticleDataArrayVector x_lb;
    auto* atom = wrapper.lmp->atom;
    const long nPart = (long)atom->nlocal + (long)atom->nghost;
    if (nPart == 0) return;   // no particles - no work (:174)
    x_lb.resize((size_t)nPart);
    for (long i = 0; i < nPart; ++i)
        for (int d = 0; d < 3; ++d) x_lb[(size_t)i][d] = units.getLbPosition(atom->x[i][d]);
    force.assign(3 * (size_t)nPart, 0.0);
    torque.assign(3 * (size_t)nPart, 0.0);
    applyProcessingFunctional(new SumForceTorque3D<double, GpuDescriptor>(x_lb, force.data(), torque.data(), wrapper),
                              lattice.getBoundingBox(), lattice);
    FixType* couplingFix = dynamic_cast<FixType*>(wrapper.lmp->modify->find_fix_style("couple/lb/onetoone", 0));
    if (!couplingFix) throw std::runtime_error("getForcesFromLattice: fix couple/lb/onetoone not found");
    double** f_liggghts = couplingFix->get_force_ptr();
    double** t_liggghts = couplingFix->get_torque_ptr();
    for (long iPart = 0; iPart < nPart; ++iPart)
        for (int j = 0; j < 3; ++j) { f_liggghts[iPart][j] = 0; t_liggghts[iPart][j] = 0; }
    for (long iPart = 0; iPart < nPart; ++iPart) {
        const int ind = atom->map(atom->tag[iPart]);
        for (int j = 0; j < 3; ++j) {
            f_liggghts[ind][j] += units.getPhysForce(force[3 * (size_t)iPart + j]);
            t_liggghts[ind][j] += units.getPhysTorque(torque[3 * (size_t)iPart + j]);
        }
    }
    couplingFix->comm_force_torque();
}

}  // namespace plb

#endif  // LBDEM_PLB_H
