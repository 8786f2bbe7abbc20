// The C++ binding INTEGRATION.md shows a maintainer adding on the reference side:
// GpuLattice and the two coupling functions of src/ibDataExchangeWrappers3D.h over
// the C ABI.  tests/test_abi_cpu.py compiles this file against include/lbdem_gpu.h,
// the PhysUnits3D shim and the LIGGGHTS stand-in of the example programs.
#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <vector>

#include "dem_standin.h"
#include "physunits_gpu.h"

namespace plb { typedef long plint; }
using namespace plb;

#include "lbdem_gpu.h"

struct GpuLattice {                 // replaces MultiBlockLattice3D<T,D3Q19> + IBcompositeDynamics
  lbdem_handle* h = nullptr;
  std::vector<double> x, v, w, r, F, T;
  std::vector<int32_t> tag;
  GpuLattice(int nx, int ny, int nz, double omega, bool periodic, int maxParticles) {
    lbdem_config c; lbdem_config_default(&c);
    c.nx = nx; c.ny = ny; c.nz = nz; c.omega = omega;
    c.periodic[0] = c.periodic[1] = c.periodic[2] = periodic;
    c.precision = LBDEM_PREC_FP64;   // drop-in; LBDEM_PREC_FP32_DEV for the fast form
    c.max_particles = maxParticles;
    if (lbdem_create(&c, &h) != LBDEM_OK) throw std::runtime_error("lbdem_create");
  }
  ~GpuLattice() { lbdem_destroy(h); }
  void collideAndStream() { check(lbdem_collide_and_stream(h)); }
  void check(lbdem_status s) { if (s != LBDEM_OK) throw std::runtime_error(lbdem_last_error(h)); }
};

template<typename T>
void setSpheresOnLattice(GpuLattice& lat, LiggghtsCouplingWrapper& wrapper,
                         PhysUnits3D<T> const& units, std::vector<plint>& excludeType, bool initVel) {
  LAMMPS_NS::Atom* a = wrapper.lmp->atom;
  const plint nPart = a->nlocal + a->nghost;
  lat.x.clear(); lat.v.clear(); lat.w.clear(); lat.r.clear(); lat.tag.clear();
  for (plint i = 0; i < nPart; ++i) {
    if (std::find(excludeType.begin(), excludeType.end(), (plint)a->type[i]) != excludeType.end()) continue;
    for (int d = 0; d < 3; ++d) {
      lat.x.push_back(units.getLbPosition(a->x[i][d]));
      lat.v.push_back(units.getLbVel(a->v[i][d]));
      lat.w.push_back(units.getLbFreq(a->omega[i][d]));
    }
    lat.r.push_back(units.getLbLength(a->radius[i]));
    lat.tag.push_back(a->tag[i]);
  }
  lat.check(lbdem_set_particles(lat.h, (int32_t)lat.r.size(), lat.x.data(), lat.v.data(),
                                lat.w.data(), lat.r.data(), lat.tag.data(), initVel));
}

template<typename T>
void getForcesFromLattice(GpuLattice& lat, LiggghtsCouplingWrapper& wrapper, PhysUnits3D<T> const& units) {
  const int32_t n = (int32_t)lat.r.size();
  lat.F.resize(3 * n); lat.T.resize(3 * n);
  lat.check(lbdem_get_forces(lat.h, n, lat.F.data(), lat.T.data()));   // lattice units
  LAMMPS_NS::FixLbCouplingOnetoone* fix = dynamic_cast<LAMMPS_NS::FixLbCouplingOnetoone*>(
      wrapper.lmp->modify->find_fix_style("couple/lb/onetoone", 0));
  double** f = fix->get_force_ptr();
  double** t = fix->get_torque_ptr();
  LAMMPS_NS::Atom* a = wrapper.lmp->atom;
  for (plint i = 0; i < a->nlocal + a->nghost; ++i)
    for (int d = 0; d < 3; ++d) f[i][d] = t[i][d] = 0;
  for (int32_t k = 0; k < n; ++k) {           // same index as the list passed above
    const int ind = a->map(lat.tag[k]);
    for (int d = 0; d < 3; ++d) {
      f[ind][d] += units.getPhysForce(lat.F[3 * k + d]);
      t[ind][d] += units.getPhysTorque(lat.T[3 * k + d]);
    }
  }
  fix->comm_force_torque();
}

// both templates instantiated with double
void instantiate(GpuLattice& lat, LiggghtsCouplingWrapper& w, PhysUnits3D<double> const& u,
                 std::vector<plint>& ex) {
    setSpheresOnLattice(lat, w, u, ex, true);
    getForcesFromLattice(lat, w, u);
}
