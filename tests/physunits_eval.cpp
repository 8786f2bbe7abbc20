// Prints every PhysUnits3D conversion, as hexadecimal floats, for a few unit
// systems and inputs -- TEST INFRASTRUCTURE (tests/test_physunits_cpu.py).
// Compiled once against plb/physunits_gpu.h and, where the reference tree is
// present, once against the reference's src/physunits.h (with the stand-in
// flow parameters of oracle/ref_harness/include); the two outputs must agree.
#include <cstdio>

#include "physunits.h"   // whichever of the two the include path selects

using plb::PhysUnits3D;

static void line(const char* what, double v) { std::printf("%s %a\n", what, v); }

static void eval(PhysUnits3D<double>& u, const double* xs, int nx) {
    line("Re", u.getRe());
    for (int k = 0; k < nx; ++k) {
        const double x = xs[k];
        line("getLbLength", u.getLbLength(x));
        line("getLbPosition", u.getLbPosition(x));
        line("getLbPositionX", u.getLbPositionX(x));
        line("getLbPositionY", u.getLbPositionY(x));
        line("getLbPositionZ", u.getLbPositionZ(x));
        line("getLbVel", u.getLbVel(x));
        line("getLbTime", u.getLbTime(x));
        line("getLbDensity", u.getLbDensity(x));
        line("getLbAccel", u.getLbAccel(x));
        line("getLbFreq", u.getLbFreq(x));
        std::printf("getLbSteps %ld\n", (long)u.getLbSteps(x));
        line("getLbRho", u.getLbRho(x));
        line("getLbRho_off", u.getLbRho(x, 0.25 * x));
        line("getPhysLength", u.getPhysLength(x));
        line("getPhysPosition", u.getPhysPosition(x));
        line("getPhysPositionX", u.getPhysPositionX(x));
        line("getPhysPositionY", u.getPhysPositionY(x));
        line("getPhysPositionZ", u.getPhysPositionZ(x));
        line("getPhysVel", u.getPhysVel(x));
        line("getPhysTime", u.getPhysTime(x));
        line("getPhysDensity", u.getPhysDensity(x));
        line("getPhysAccel", u.getPhysAccel(x));
        line("getPhysForce", u.getPhysForce(x));
        line("getPhysTorque", u.getPhysTorque(x));
        line("getPhysPress", u.getPhysPress(x));
        line("getPhysPress_off", u.getPhysPress(x, 101325.0));
    }
    line("deltaX", u.getLbParam().getDeltaX());
    line("deltaT", u.getLbParam().getDeltaT());
    line("latticeU", u.getLbParam().getLatticeU());
}

int main() {
    const double xs[] = {0.0, 1.0, 0.37, 12.5, 1e-3, -2.75, 3.0e4};
    const int nx = (int)(sizeof(xs) / sizeof(xs[0]));
    // lattice units with a viscosity from tau = 0.6 (the sedimenting-sphere setup)
    PhysUnits3D<double> a(1.0, 1.0, 0.1 / 3.0, 60, 60, 180, 1, 1.0, 1.0);
    eval(a, xs, nx);
    // a physical system: 1 cm spheres in water, 30 cells per length unit
    PhysUnits3D<double> b(0.01, 0.1, 1e-6, 0.02, 0.02, 0.06, 30, 0.02, 1000.0);
    eval(b, xs, nx);
    b.setLbOffset(0.0, 0.25, -0.5);
    eval(b, xs, nx);
    return 0;
}
