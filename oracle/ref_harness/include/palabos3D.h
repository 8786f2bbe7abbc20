// Minimal stand-ins for the Palabos v1.5r1 types used by the LBDEMcoupling PSM
// headers (src/ibCompositeDynamics3D.*, src/ibProcessors3D.*, src/utils.h,
// src/physunits.h, src/periodicPressureFunctionals3D.*,
// src/ibDataWritingFunctionals3D.*) -- TEST INFRASTRUCTURE for the reference
// harness only.
//
// Palabos is not available here.  These declarations give the reference
// headers the interface they call; the lattice-Boltzmann arithmetic inside
// (moments, second-order equilibrium, BGK) restates the published definitions
// with the same expressions as oracle/psm_oracle.cpp, so that comparing the
// harness with the oracle isolates the statements the reference itself owns.
#ifndef LBDEM_REF_HARNESS_PALABOS3D_H
#define LBDEM_REF_HARNESS_PALABOS3D_H

#include <cmath>
#include <cstddef>
#include <string>
#include <vector>

typedef int MPI_Comm;

#define PLB_PRECONDITION(x)

namespace plb {

typedef long plint;
typedef unsigned long pluint;

template <typename T, int n>
class Array {
public:
    Array() { for (int i = 0; i < n; ++i) d[i] = T(); }
    Array(T a, T b, T c) { d[0] = a; d[1] = b; d[2] = c; }
    T& operator[](plint i) { return d[i]; }
    const T& operator[](plint i) const { return d[i]; }
    void resetToZero() { for (int i = 0; i < n; ++i) d[i] = T(); }
    void from_cArray(const T* a) { for (int i = 0; i < n; ++i) d[i] = a[i]; }
    Array<T, n> operator*(T s) const { Array<T, n> r; for (int i = 0; i < n; ++i) r.d[i] = d[i] * s; return r; }
    T d[n];
};

struct Dot3D {
    Dot3D() : x(0), y(0), z(0) {}
    Dot3D(plint x_, plint y_, plint z_) : x(x_), y(y_), z(z_) {}
    plint x, y, z;
};

struct Box3D {
    Box3D() : x0(0), x1(0), y0(0), y1(0), z0(0), z1(0) {}
    Box3D(plint x0_, plint x1_, plint y0_, plint y1_, plint z0_, plint z1_)
        : x0(x0_), x1(x1_), y0(y0_), y1(y1_), z0(z0_), z1(z1_) {}
    plint x0, x1, y0, y1, z0, z1;
};

inline bool intersect(Box3D const& a, Box3D const& b, Box3D& r) {
    r.x0 = a.x0 > b.x0 ? a.x0 : b.x0; r.x1 = a.x1 < b.x1 ? a.x1 : b.x1;
    r.y0 = a.y0 > b.y0 ? a.y0 : b.y0; r.y1 = a.y1 < b.y1 ? a.y1 : b.y1;
    r.z0 = a.z0 > b.z0 ? a.z0 : b.z0; r.z1 = a.z1 < b.z1 ? a.z1 : b.z1;
    return r.x0 <= r.x1 && r.y0 <= r.y1 && r.z0 <= r.z1;
}

namespace modif {
enum ModifT { nothing = 0, staticVariables, dynamicVariables, allVariables, dataStructure, undefined };
}

class BlockStatistics {};

class HierarchicSerializer {
public:
    template <typename U> void addValue(U const&) {}
};
class HierarchicUnserializer {
public:
    int getId() const { return 0; }
    template <typename U> void readValue(U&) {}
};

namespace descriptors {
// D3Q19, Palabos order: c[i + 9] = -c[i] for i = 1..9.
template <typename T>
struct D3Q19Descriptor {
    enum { q = 19, d = 3 };
    static const int c[19][3];
    static const T t[19];
    static T invRho(T rhoBar) { return (T)1 / ((T)1 + rhoBar); }
};
template <typename T>
const int D3Q19Descriptor<T>::c[19][3] = {
    {0, 0, 0}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {-1, -1, 0}, {-1, 1, 0}, {-1, 0, -1}, {-1, 0, 1}, {0, -1, -1},
    {0, -1, 1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, -1, 0}, {1, 0, 1}, {1, 0, -1}, {0, 1, 1}, {0, 1, -1}};
template <typename T>
const T D3Q19Descriptor<T>::t[19] = {(T)1 / 3,  (T)1 / 18, (T)1 / 18, (T)1 / 18, (T)1 / 36, (T)1 / 36, (T)1 / 36,
                                     (T)1 / 36, (T)1 / 36, (T)1 / 36, (T)1 / 18, (T)1 / 18, (T)1 / 18, (T)1 / 36,
                                     (T)1 / 36, (T)1 / 36, (T)1 / 36, (T)1 / 36, (T)1 / 36};
}  // namespace descriptors

template <typename T, int d>
struct VectorTemplateImpl {
    static T normSqr(Array<T, d> const& a) {
        T r = a[0] * a[0];
        for (int i = 1; i < d; ++i) r += a[i] * a[i];
        return r;
    }
};

template <typename T, template <typename U> class Descriptor>
class Cell;

// feq_i = t_i [rhoBar + 3 c.j + invRho (4.5 (c.j)^2 - 1.5 j.j)], same expression as the oracle.
template <typename T, template <typename U> class Descriptor>
struct dynamicsTemplates {
    typedef Descriptor<T> D;
    static T feq(plint i, T rhoBar, T invRho, Array<T, D::d> const& j, T jSqr) {
        T cj = (T)D::c[i][0] * j[0] + (T)D::c[i][1] * j[1] + (T)D::c[i][2] * j[2];
        return D::t[i] * (rhoBar + (T)3 * cj + invRho * ((T)4.5 * cj * cj - (T)1.5 * jSqr));
    }
    static void bgk_ma2_equilibria(T rhoBar, T invRho, Array<T, D::d> const& j, T jSqr, Array<T, D::q>& eq) {
        for (plint i = 0; i < D::q; ++i) eq[i] = feq(i, rhoBar, invRho, j, jSqr);
    }
};

template <typename T, template <typename U> class Descriptor>
struct momentTemplates {
    typedef Descriptor<T> D;
    static void get_rhoBar_j(Cell<T, Descriptor> const& cell, T& rhoBar, Array<T, D::d>& j) {
        rhoBar = 0; j[0] = j[1] = j[2] = 0;
        for (plint i = 0; i < D::q; ++i) {
            rhoBar += cell[i];
            j[0] += (T)D::c[i][0] * cell[i];
            j[1] += (T)D::c[i][1] * cell[i];
            j[2] += (T)D::c[i][2] * cell[i];
        }
    }
};

namespace meta {
inline int& dynamicsCounter() { static int n = 0; return n; }
template <typename T, template <typename U> class Descriptor, class Dyn>
int registerGeneralDynamics(std::string const&) { return ++dynamicsCounter() + 1000; }
}  // namespace meta

template <typename T, template <typename U> class Descriptor>
class Dynamics {
public:
    virtual ~Dynamics() {}
    virtual Dynamics* clone() const = 0;
    virtual int getId() const = 0;
    virtual bool isComposite() const { return false; }
    virtual void collide(Cell<T, Descriptor>& cell, BlockStatistics& stats) = 0;
    virtual void prepareCollision(Cell<T, Descriptor>&) {}
    virtual T getOmega() const { return 0; }
    virtual void computeEquilibria(Array<T, Descriptor<T>::q>& fEq, T rhoBar, Array<T, Descriptor<T>::d> const& j,
                                   T jSqr, T thetaBar = T()) const {
        dynamicsTemplates<T, Descriptor>::bgk_ma2_equilibria(rhoBar, Descriptor<T>::invRho(rhoBar), j, jSqr, fEq);
    }
    virtual void defineVelocity(Cell<T, Descriptor>&, Array<T, Descriptor<T>::d> const&) {}
    virtual void serialize(HierarchicSerializer&) const {}
    virtual void unserialize(HierarchicUnserializer&) {}
};

template <typename T, template <typename U> class Descriptor>
class NoDynamics : public Dynamics<T, Descriptor> {
public:
    NoDynamics* clone() const { return new NoDynamics(*this); }
    int getId() const { return 1; }
    void collide(Cell<T, Descriptor>&, BlockStatistics&) {}
};

// BGK collision: f_i <- f_i (1 - omega) + omega feq_i(rhoBar, j), same expression as the oracle.
template <typename T, template <typename U> class Descriptor>
class BGKdynamics : public Dynamics<T, Descriptor> {
public:
    explicit BGKdynamics(T omega_) : omega(omega_) {}
    BGKdynamics* clone() const { return new BGKdynamics(*this); }
    int getId() const { return 2; }
    T getOmega() const { return omega; }
    void collide(Cell<T, Descriptor>& cell, BlockStatistics&) {
        typedef Descriptor<T> D;
        T rhoBar; Array<T, D::d> j;
        momentTemplates<T, Descriptor>::get_rhoBar_j(cell, rhoBar, j);
        T invRho = (T)1 / ((T)1 + rhoBar);
        T jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
        for (plint i = 0; i < D::q; ++i)
            cell[i] = cell[i] * ((T)1 - omega) + omega * dynamicsTemplates<T, Descriptor>::feq(i, rhoBar, invRho, j, jSqr);
    }
private:
    T omega;
};

template <typename T, template <typename U> class Descriptor>
class CompositeDynamics : public Dynamics<T, Descriptor> {
public:
    CompositeDynamics(Dynamics<T, Descriptor>* base, bool automaticPrepareCollision_)
        : baseDynamics(base), automaticPrepareCollision(automaticPrepareCollision_) {}
    CompositeDynamics(CompositeDynamics const& o)
        : Dynamics<T, Descriptor>(o), baseDynamics(o.baseDynamics ? o.baseDynamics->clone() : 0),
          automaticPrepareCollision(o.automaticPrepareCollision) {}
    ~CompositeDynamics() { delete baseDynamics; }
    bool isComposite() const { return true; }
    Dynamics<T, Descriptor>& getBaseDynamics() { return *baseDynamics; }
    Dynamics<T, Descriptor> const& getBaseDynamics() const { return *baseDynamics; }
    T getOmega() const { return baseDynamics->getOmega(); }
    void collide(Cell<T, Descriptor>& cell, BlockStatistics& stats) {
        if (automaticPrepareCollision) this->prepareCollision(cell);
        baseDynamics->collide(cell, stats);
    }
    void serialize(HierarchicSerializer&) const {}
    void unserialize(HierarchicUnserializer&) {}
private:
    Dynamics<T, Descriptor>* baseDynamics;
    bool automaticPrepareCollision;
};

template <typename T, template <typename U> class Descriptor>
class Cell {
public:
    Cell() : dyn(0) {}
    T& operator[](plint i) { return f[i]; }
    T const& operator[](plint i) const { return f[i]; }
    Array<T, Descriptor<T>::q>& getRawPopulations() { return f; }
    Dynamics<T, Descriptor>& getDynamics() { return *dyn; }
    void defineVelocity(Array<T, Descriptor<T>::d> const& u) { dyn->defineVelocity(*this, u); }
    Array<T, Descriptor<T>::q> f;
    Dynamics<T, Descriptor>* dyn;
};

// One atomic block with an envelope of width 1, located at global (-1,-1,-1).
template <typename T, template <typename U> class Descriptor>
class BlockLattice3D {
public:
    BlockLattice3D(plint nx_, plint ny_, plint nz_) : nx(nx_ + 2), ny(ny_ + 2), nz(nz_ + 2), cells(nx * ny * nz) {}
    Cell<T, Descriptor>& get(plint x, plint y, plint z) { return cells[(x * ny + y) * nz + z]; }
    plint getNx() const { return nx; }
    plint getNy() const { return ny; }
    plint getNz() const { return nz; }
    Dot3D getLocation() const { return Dot3D(-1, -1, -1); }
    plint nx, ny, nz;
    std::vector<Cell<T, Descriptor> > cells;
};

template <typename T, template <typename U> class Descriptor>
struct BoxProcessingFunctional3D_L {
    virtual ~BoxProcessingFunctional3D_L() {}
    virtual void process(Box3D domain, BlockLattice3D<T, Descriptor>& lattice) = 0;
    virtual void getTypeOfModification(std::vector<modif::ModifT>& modified) const = 0;
};

class AtomicBlock3D {
public:
    virtual ~AtomicBlock3D() {}
};

// Scalar and tensor fields of one atomic block, indexed like BlockLattice3D
// (the caller sizes them with the lattice's envelope).
template <typename T>
class ScalarField3D : public AtomicBlock3D {
public:
    ScalarField3D(plint nx_, plint ny_, plint nz_) : nx(nx_), ny(ny_), nz(nz_), data(nx_ * ny_ * nz_) {}
    T& get(plint x, plint y, plint z) { return data[(x * ny + y) * nz + z]; }
    plint nx, ny, nz;
    std::vector<T> data;
};
template <typename T, int nDim>
class TensorField3D : public AtomicBlock3D {
public:
    TensorField3D(plint nx_, plint ny_, plint nz_) : nx(nx_), ny(ny_), nz(nz_), data(nx_ * ny_ * nz_) {}
    Array<T, nDim>& get(plint x, plint y, plint z) { return data[(x * ny + y) * nz + z]; }
    plint nx, ny, nz;
    std::vector<Array<T, nDim> > data;
};
template <typename T1, template <typename U> class Descriptor, typename T2>
struct BoxProcessingFunctional3D_LS {
    virtual ~BoxProcessingFunctional3D_LS() {}
    virtual void process(Box3D domain, BlockLattice3D<T1, Descriptor>& lattice, ScalarField3D<T2>& field) = 0;
    virtual void getTypeOfModification(std::vector<modif::ModifT>& modified) const = 0;
};
template <typename T1, template <typename U> class Descriptor, typename T2, int nDim>
struct BoxProcessingFunctional3D_LT {
    virtual ~BoxProcessingFunctional3D_LT() {}
    virtual void process(Box3D domain, BlockLattice3D<T1, Descriptor>& lattice, TensorField3D<T2, nDim>& field) = 0;
    virtual void getTypeOfModification(std::vector<modif::ModifT>& modified) const = 0;
};

// Declared only so that src/periodicPressureFunctionals3D.h parses: the Kim
// functional and PeriodicPressureManager, which use them, are never instantiated
// (the harness drives ZhangPeriodicPressureFunctional3D and the two initial-state
// functors, which need nothing beyond the types above).
class MultiBlock3D {
public:
    virtual ~MultiBlock3D() {}
};
class BoxProcessingFunctional3D {
public:
    virtual ~BoxProcessingFunctional3D() {}
};
template <typename T, template <typename U> class Descriptor> class MultiBlockLattice3D;
template <typename T> class MultiScalarField3D;
template <typename T, int nDim> class MultiTensorField3D;

// Used only so that src/physunits.h compiles.
template <typename T>
class IncomprFlowParam {
public:
    IncomprFlowParam(T uMax_, T Re_, plint N_, T lx_, T ly_, T lz_) : uMax(uMax_), N(N_) {}
    T getDeltaX() const { return (T)1 / (T)N; }
    T getDeltaT() const { return getDeltaX() * uMax; }
    T getLatticeU() const { return uMax; }
private:
    T uMax;
    plint N;
};

}  // namespace plb

#endif
