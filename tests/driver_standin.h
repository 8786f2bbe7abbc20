// The few Palabos names a LBDEMcoupling case driver's coupling code uses besides
// the coupling itself, standing in for Palabos (absent here) when the reference's
// own driver lines are compiled against plb/lbdem_plb.h: plint, pcout, Box3D,
// the D3Q19 descriptor, BGKdynamics and the flow-parameter object's getOmega.
#ifndef LBDEM_TEST_DRIVER_STANDIN_H
#define LBDEM_TEST_DRIVER_STANDIN_H

#include <cstddef>
#include <iostream>

namespace plb {

typedef std::ptrdiff_t plint;

static std::ostream& pcout = std::cout;

struct Box3D {
    Box3D(plint x0_, plint x1_, plint y0_, plint y1_, plint z0_, plint z1_)
        : x0(x0_), x1(x1_), y0(y0_), y1(y1_), z0(z0_), z1(z1_) {}
    plint x0, x1, y0, y1, z0, z1;
};

namespace descriptors {
template <typename T>
struct D3Q19Descriptor {
    static const int d = 3, q = 19;
};
}  // namespace descriptors

template <typename T, template <typename U> class Descriptor>
class BGKdynamics {
public:
    explicit BGKdynamics(T omega_) : omega(omega_) {}
    virtual ~BGKdynamics() {}
    T getOmega() const { return omega; }

private:
    T omega;
};

// IncomprFlowParam's relaxation frequency, 1 / (3 nu_lb + 1/2)
template <typename T>
class IncomprFlowParam {
public:
    explicit IncomprFlowParam(T tau_) : tau(tau_) {}
    T getOmega() const { return (T)1 / tau; }

private:
    T tau;
};

}  // namespace plb

#endif
