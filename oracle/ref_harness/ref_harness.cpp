// Reference harness -- TEST INFRASTRUCTURE.
//
// Compiles the LBDEMcoupling reference's own PSM code, from the reference tree,
// against the minimal Palabos/LIGGGHTS stand-ins in ./include:
//   src/ibCompositeDynamics3D.hh  IBcompositeDynamics::collide, prepareCollision, defineVelocity
//   src/ibProcessors3D.hh         SetSingleSphere3D::process / calcSolidFraction / setValues,
//                                 SumForceTorque3D::process
//   src/utils.h                   getParticleDataFromCell
//   src/periodicPressureFunctionals3D.hh
//                                 ZhangPeriodicPressureFunctional3D::process,
//                                 PressureGradient, PoiseuilleProfileAndPressureGradient
//   src/ibDataWritingFunctionals3D.hh
//                                 Get{Scalar,Vector}QuantityFromDynamicsFunctional (field export)
// and drives them the way src/ibDataExchangeWrappers3D.hh does (sphere loop,
// bounding box intersected with the local block, force/torque vectors), with
// push streaming on a periodic lattice standing in for Palabos' collideAndStream.
//
// It is used to check the oracle (oracle/psm_oracle.cpp) against the
// reference's statements and to generate golden fixtures; it is never part of
// the product.  Build: oracle/ref_build.py (outputs into oracle/_ref/).
#include <cstdint>
#include <cstring>
#include <vector>

#include "palabos3D.h"
#include "palabos3D.hh"

#include "ibDynamicsParticleData.h"
#include "ibCompositeDynamics3D.h"
#include "ibProcessors3D.h"
#include "periodicPressureFunctionals3D.h"
#include "ibDataWritingFunctionals3D.h"

// LIGGGHTS' coupling wrapper: only its atom map is used by SumForceTorque3D.
LiggghtsCouplingWrapper::LiggghtsCouplingWrapper(char**, MPI_Comm) : lmp(0) {}

using namespace plb;
typedef double T;
#define DESCRIPTOR descriptors::D3Q19Descriptor

namespace {

struct Harness {
    plint nx, ny, nz;
    T omega;
    BlockLattice3D<T, DESCRIPTOR> lattice;
    std::vector<T> scratch;
    Harness(plint nx_, plint ny_, plint nz_, T omega_)
        : nx(nx_), ny(ny_), nz(nz_), omega(omega_), lattice(nx_, ny_, nz_) {
        for (plint x = 1; x <= nx; ++x)
            for (plint y = 1; y <= ny; ++y)
                for (plint z = 1; z <= nz; ++z)
                    lattice.get(x, y, z).dyn =
                        new IBcompositeDynamics<T, DESCRIPTOR>(new BGKdynamics<T, DESCRIPTOR>(omega));
    }
    ~Harness() {
        for (size_t k = 0; k < lattice.cells.size(); ++k) delete lattice.cells[k].dyn;
    }
    Cell<T, DESCRIPTOR>& cell(plint x, plint y, plint z) { return lattice.get(x + 1, y + 1, z + 1); }
    size_t idx(plint x, plint y, plint z) const { return ((size_t)x * ny + y) * nz + z; }
};

// Stand-in for Palabos' iniCellAtEquilibrium, through which initializeAtEquilibrium
// applies a density/velocity functor: j = density u, rhoBar = density - 1,
// f_i = feq_i(rhoBar, 1 / (1 + rhoBar), j, |j|^2).
void ini_at_equilibrium(Cell<T, DESCRIPTOR>& c, T density, Array<T, 3> const& u) {
    Array<T, 3> j(density * u[0], density * u[1], density * u[2]);
    const T jSqr = VectorTemplateImpl<T, 3>::normSqr(j);
    const T rhoBar = density - (T)1;
    const T invRho = DESCRIPTOR<T>::invRho(rhoBar);
    for (plint i = 0; i < DESCRIPTOR<T>::q; ++i) c[i] = dynamicsTemplates<T, DESCRIPTOR>::feq(i, rhoBar, invRho, j, jSqr);
}

}  // namespace

extern "C" {

void* ref_create(int nx, int ny, int nz, double omega) { return new Harness(nx, ny, nz, omega); }
void ref_destroy(void* h) { delete (Harness*)h; }

// populations [19][nx][ny][nz]
void ref_set_pops(void* hp, const double* f) {
    Harness& h = *(Harness*)hp;
    const size_t N = (size_t)h.nx * h.ny * h.nz;
    for (plint x = 0; x < h.nx; ++x)
        for (plint y = 0; y < h.ny; ++y)
            for (plint z = 0; z < h.nz; ++z)
                for (int i = 0; i < 19; ++i) h.cell(x, y, z)[i] = f[i * N + h.idx(x, y, z)];
}

void ref_get_pops(void* hp, double* f) {
    Harness& h = *(Harness*)hp;
    const size_t N = (size_t)h.nx * h.ny * h.nz;
    for (plint x = 0; x < h.nx; ++x)
        for (plint y = 0; y < h.ny; ++y)
            for (plint z = 0; z < h.nz; ++z)
                for (int i = 0; i < 19; ++i) f[i * N + h.idx(x, y, z)] = h.cell(x, y, z)[i];
}

// The sphere loop of setSpheresOnLattice (src/ibDataExchangeWrappers3D.hh:62-139)
// with positions already in lattice units.
void ref_set_spheres(void* hp, int n, const double* xs, const double* vs, const double* ws, const double* rs,
                     const int32_t* tags, int initVel) {
    Harness& h = *(Harness*)hp;
    Box3D localBB(0, h.nx - 1, 0, h.ny - 1, 0, h.nz - 1);
    for (int s = 0; s < n; ++s) {
        T x[3], v[3], omega[3];
        for (int d = 0; d < 3; ++d) { x[d] = xs[3 * s + d]; v[d] = vs[3 * s + d]; omega[d] = ws[3 * s + d]; }
        T r = rs[s];
        plint id = tags[s];
        SetSingleSphere3D<T, DESCRIPTOR>* sss = new SetSingleSphere3D<T, DESCRIPTOR>(x, v, omega, x, r, id, initVel != 0);
        Box3D sss_box = sss->getBoundingBox();
        Box3D inter(0, 0, 0, 0, 0, 0);
        if (intersect(sss_box, localBB, inter)) {
            // global -> atomic-block coordinates (the block sits at -1, -1, -1)
            Box3D local(inter.x0 + 1, inter.x1 + 1, inter.y0 + 1, inter.y1 + 1, inter.z0 + 1, inter.z1 + 1);
            sss->process(local, h.lattice);
        }
        delete sss;
    }
}

// IBcompositeDynamics::collide in every cell, then periodic push streaming.
void ref_collide_stream(void* hp) {
    Harness& h = *(Harness*)hp;
    BlockStatistics stats;
    for (plint x = 0; x < h.nx; ++x)
        for (plint y = 0; y < h.ny; ++y)
            for (plint z = 0; z < h.nz; ++z) {
                Cell<T, DESCRIPTOR>& c = h.cell(x, y, z);
                c.getDynamics().collide(c, stats);
            }
    const size_t N = (size_t)h.nx * h.ny * h.nz;
    h.scratch.assign(19 * N, 0.0);
    for (plint x = 0; x < h.nx; ++x)
        for (plint y = 0; y < h.ny; ++y)
            for (plint z = 0; z < h.nz; ++z)
                for (int i = 0; i < 19; ++i) {
                    const plint X = (x + DESCRIPTOR<T>::c[i][0] + h.nx) % h.nx;
                    const plint Y = (y + DESCRIPTOR<T>::c[i][1] + h.ny) % h.ny;
                    const plint Z = (z + DESCRIPTOR<T>::c[i][2] + h.nz) % h.nz;
                    h.scratch[i * N + h.idx(X, Y, Z)] = h.cell(x, y, z)[i];
                }
    for (plint x = 0; x < h.nx; ++x)
        for (plint y = 0; y < h.ny; ++y)
            for (plint z = 0; z < h.nz; ++z)
                for (int i = 0; i < 19; ++i) h.cell(x, y, z)[i] = h.scratch[i * N + h.idx(x, y, z)];
}

// SumForceTorque3D over the local block with LIGGGHTS' atom map (lowest index
// per tag), as getForcesFromLattice prepares it (src/ibDataExchangeWrappers3D.hh:160-218).
void ref_sum_force_torque(void* hp, int n, const double* xs, const int32_t* tags, double* F, double* Tq) {
    Harness& h = *(Harness*)hp;
    ParticleData<T>::ParticleDataArrayVector x_lb;
    int maxTag = 0;
    for (int i = 0; i < n; ++i) {
        x_lb.push_back(Array<T, 3>(xs[3 * i], xs[3 * i + 1], xs[3 * i + 2]));
        if (tags[i] > maxTag) maxTag = tags[i];
    }
    LAMMPS_NS::Atom atom;
    atom.map_array.assign(maxTag + 1, -1);
    for (int i = n - 1; i >= 0; --i) atom.map_array[tags[i]] = i;
    LAMMPS_NS::LAMMPS lmp;
    lmp.atom = &atom;
    lmp.modify = 0;
    LiggghtsCouplingWrapper wrapper(0, 0);
    wrapper.lmp = &lmp;
    std::vector<T> force(3 * (size_t)(n > 0 ? n : 1), 0.0), torque(3 * (size_t)(n > 0 ? n : 1), 0.0);
    SumForceTorque3D<T, DESCRIPTOR> sft(x_lb, &force.front(), &torque.front(), wrapper);
    sft.process(Box3D(1, h.nx, 1, h.ny, 1, h.nz), h.lattice);
    for (int i = 0; i < 3 * n; ++i) { F[i] = force[i]; Tq[i] = torque[i]; }
}

// ZhangPeriodicPressureFunctional3D::process (src/periodicPressureFunctionals3D.hh:137-159)
// on box = {x0, x1, y0, y1, z0, z1} in lattice coordinates.
void ref_zhang_rescale(void* hp, const int32_t* b, int dim, int dir, double rhoTarget, double rhoAvg) {
    Harness& h = *(Harness*)hp;
    ZhangPeriodicPressureFunctional3D<T, DESCRIPTOR> fn(rhoTarget, rhoAvg, dim, dir);
    fn.process(Box3D(b[0] + 1, b[1] + 1, b[2] + 1, b[3] + 1, b[4] + 1, b[5] + 1), h.lattice);
}

// Every cell at equilibrium with the density and velocity of PressureGradient
// (kind 0, src/periodicPressureFunctionals3D.hh:238-256; grid size n[dim]) or
// PoiseuilleProfileAndPressureGradient (kind 1, :259-298; grid sizes n[0..2]),
// evaluated at the cell's lattice coordinates.
void ref_init_profile(void* hp, int kind, double pHi, double pLo, double uMax, const int32_t* n, int dim) {
    Harness& h = *(Harness*)hp;
    const PressureGradient<T> gradient(pHi, pLo, n[dim], dim);
    const PoiseuilleProfileAndPressureGradient<T> poiseuille(pHi, pLo, uMax, n[0], n[1], n[2], dim);
    for (plint x = 0; x < h.nx; ++x)
        for (plint y = 0; y < h.ny; ++y)
            for (plint z = 0; z < h.nz; ++z) {
                T density = 0;
                Array<T, 3> u;
                if (kind == 0) gradient(x, y, z, density, u);
                else poiseuille(x, y, z, density, u);
                ini_at_equilibrium(h.cell(x, y, z), density, u);
            }
}

// Per-cell particle data (IBdynamicsParticleData: sf, partId, uPart,
// hydrodynamicForce) exported the way the reference's case drivers export it,
// through GetScalarQuantityFromDynamicsFunctional (SolidFraction, ParticleId) and
// GetVectorQuantityFromDynamicsFunctional (ParticleVelocity, HydrodynamicForce),
// src/ibDataWritingFunctionals3D.hh:30-114, into fields of type T.
void ref_get_state(void* hp, double* sf, int32_t* id, double* up, double* cf) {
    Harness& h = *(Harness*)hp;
    const plint ex = h.nx + 2, ey = h.ny + 2, ez = h.nz + 2;
    const Box3D inner(1, h.nx, 1, h.ny, 1, h.nz);
    ScalarField3D<T> fsf(ex, ey, ez), fid(ex, ey, ez);
    TensorField3D<T, 3> fup(ex, ey, ez), fcf(ex, ey, ez);
    GetScalarQuantityFromDynamicsFunctional<T, DESCRIPTOR, T>(SolidFraction).process(inner, h.lattice, fsf);
    GetScalarQuantityFromDynamicsFunctional<T, DESCRIPTOR, T>(ParticleId).process(inner, h.lattice, fid);
    GetVectorQuantityFromDynamicsFunctional<T, DESCRIPTOR, T, 3>(ParticleVelocity).process(inner, h.lattice, fup);
    GetVectorQuantityFromDynamicsFunctional<T, DESCRIPTOR, T, 3>(HydrodynamicForce).process(inner, h.lattice, fcf);
    const size_t N = (size_t)h.nx * h.ny * h.nz;
    for (plint x = 0; x < h.nx; ++x)
        for (plint y = 0; y < h.ny; ++y)
            for (plint z = 0; z < h.nz; ++z) {
                const size_t c = h.idx(x, y, z);
                sf[c] = fsf.get(x + 1, y + 1, z + 1);
                id[c] = (int32_t)fid.get(x + 1, y + 1, z + 1);
                for (int d = 0; d < 3; ++d) {
                    up[d * N + c] = fup.get(x + 1, y + 1, z + 1)[d];
                    cf[d * N + c] = fcf.get(x + 1, y + 1, z + 1)[d];
                }
            }
}

}  // extern "C"
