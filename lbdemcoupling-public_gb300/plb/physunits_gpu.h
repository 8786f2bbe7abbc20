// PhysUnits3D for builds without Palabos.
//
// Same conversions as the reference's src/physunits.h:32-77 (physical <->
// lattice units through the dimensionless flow parameters).  The reference
// takes the flow parameters from Palabos' IncomprFlowParam; without Palabos
// they are restated here from their published definitions:
//   deltaX = 1 / N, deltaT = deltaX * uLattice, nu_lattice = uLattice N / Re,
//   tau = 3 nu_lattice + 1/2, omega = 1 / tau.
// Uses the reference's include guard, so only one PhysUnits3D is ever defined.
#ifndef PHYSUNITS_H
#define PHYSUNITS_H

#include <cmath>

namespace plb {

template <typename T>
class LbdemFlowParam {
public:
    LbdemFlowParam(T latticeU_, T Re_, long N_, T lx_, T ly_, T lz_)
        : latticeU(latticeU_), Re(Re_), N(N_), lx(lx_), ly(ly_), lz(lz_) {}
    T getLatticeU() const { return latticeU; }
    T getRe() const { return Re; }
    long getResolution() const { return N; }
    T getDeltaX() const { return (T)1 / (T)N; }
    T getDeltaT() const { return getDeltaX() * latticeU; }
    T getLatticeNu() const { return latticeU * (T)N / Re; }
    T getTau() const { return (T)3 * getLatticeNu() + (T)0.5; }
    T getOmega() const { return (T)1 / getTau(); }
    long getNx() const { return (long)std::lround(lx * (T)N) + 1; }
    long getNy() const { return (long)std::lround(ly * (T)N) + 1; }
    long getNz() const { return (long)std::lround(lz * (T)N) + 1; }

private:
    T latticeU, Re;
    long N;
    T lx, ly, lz;
};

// Lattice positions are cell centres: physical position = (lattice + offset)
// deltaX l_p with offset 1/2 by default; setLbOffset changes the per-axis
// offsets used by the X/Y/Z variants (getLbPosition / getPhysPosition keep 1/2).
template <typename T>
class PhysUnits3D {
public:
    PhysUnits3D(T const l_p_, T const u_p_, T const nu_p_, T const lx_, T const ly_, T const lz_, long const N,
                T const uMax, T const rho_p_)
        : l_p(l_p_), u_p(u_p_), t_p(l_p_ / u_p_), nu_p(nu_p_), rho_p(rho_p_), Re(l_p_ * u_p_ / nu_p_),
          param(uMax, Re, N, lx_ / l_p_, ly_ / l_p_, lz_ / l_p_),
          forceFactor(std::pow(param.getDeltaX(), 4) / std::pow(param.getDeltaT(), 2) * rho_p * std::pow(l_p, 4) /
                      std::pow(t_p, 2)),
          torqueFactor(std::pow(param.getDeltaX(), 5) / std::pow(param.getDeltaT(), 2) * rho_p * std::pow(l_p, 5) /
                       std::pow(t_p, 2)),
          lbOffsetX(0.5), lbOffsetY(0.5), lbOffsetZ(0.5) {}

    T getRe() const { return Re; }
    void setLbOffset(T const ox, T const oy, T const oz) {
        lbOffsetX = ox;
        lbOffsetY = oy;
        lbOffsetZ = oz;
    }

    // physical -> lattice
    T getLbLength(T const physL) const { return physL / l_p / param.getDeltaX(); }
    T getLbPosition(T const physL) const { return physL / l_p / param.getDeltaX() - 0.5; }
    T getLbPositionX(T const physL) const { return physL / l_p / param.getDeltaX() - lbOffsetX; }
    T getLbPositionY(T const physL) const { return physL / l_p / param.getDeltaX() - lbOffsetY; }
    T getLbPositionZ(T const physL) const { return physL / l_p / param.getDeltaX() - lbOffsetZ; }
    T getLbVel(T const physVel) const { return physVel / u_p * param.getLatticeU(); }
    T getLbTime(T const physTime) const { return physTime / t_p / param.getDeltaT(); }
    T getLbDensity(T const physDensity) const { return physDensity / rho_p; }
    T getLbAccel(T const physAccel) const {
        return physAccel * (t_p * t_p / l_p) * (param.getDeltaT() * param.getDeltaT() / param.getDeltaX());
    }
    T getLbFreq(T const physFreq) const { return physFreq * t_p * param.getDeltaT(); }
    long getLbSteps(T const physTime) const { return (long)(physTime / param.getDeltaT() / t_p + 0.5); }
    // lattice density from a pressure: p = c_s^2 rho (lattice), c_s^2 = 1/3
    T getLbRho(T const physPress, T const pOffset = 0) const {
        return (physPress - pOffset) * 3. / getPhysForce(1.) * std::pow(getPhysLength(1.), 2);
    }

    // lattice -> physical
    T getPhysLength(T const lbLength) const { return lbLength * param.getDeltaX() * l_p; }
    T getPhysPosition(T const lbLength) const { return (lbLength + 0.5) * param.getDeltaX() * l_p; }
    T getPhysPositionX(T const lbLength) const { return (lbLength + lbOffsetX) * param.getDeltaX() * l_p; }
    T getPhysPositionY(T const lbLength) const { return (lbLength + lbOffsetY) * param.getDeltaX() * l_p; }
    T getPhysPositionZ(T const lbLength) const { return (lbLength + lbOffsetZ) * param.getDeltaX() * l_p; }
    T getPhysVel(T const lbVel) const { return lbVel / param.getLatticeU() * u_p; }
    T getPhysTime(T const lbTime) const { return lbTime * param.getDeltaT() * t_p; }
    T getPhysDensity(T const lbDensity) const { return lbDensity * rho_p; }
    T getPhysAccel(T const lbAccel) const { return lbAccel / getLbAccel(1.); }
    T getPhysForce(T const lbForce) const { return lbForce * forceFactor; }
    T getPhysTorque(T const lbTorque) const { return lbTorque * torqueFactor; }
    T getPhysPress(T const lbRho, T pOffset = 0) const {
        return (lbRho - 1.) / 3. * getPhysForce(1) / std::pow(getPhysLength(1.), 2) + pOffset;
    }
    LbdemFlowParam<T> const& getLbParam() const { return param; }

private:
    T const l_p, u_p, t_p, nu_p, rho_p, Re;
    LbdemFlowParam<T> param;
    T const forceFactor, torqueFactor;
    T lbOffsetX, lbOffsetY, lbOffsetZ;
};

}  // namespace plb

#endif  // PHYSUNITS_H
