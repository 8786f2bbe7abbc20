// A host particle integrator with the LIGGGHTS members the coupling reads and
// writes, standing in for LIGGGHTS 3.1 (absent here) in the example programs.
//
// Mirrors what the reference's LIGGGHTS side does per coupling cycle
// (examples/sedimentingSphere/in.lbdem, fix_lb_coupling_onetoone.cpp:130-163):
//   fix nve/sphere        velocity-Verlet translation and rotation,
//   fix gravity           buoyancy-reduced gravity g (rho_s - rho_f) / rho_s,
//   fix couple/lb/onetoone  the hydrodynamic force/torque of the last lattice
//                         step added in every substep.
// Single process: no ghost atoms unless the calling program adds periodic images.
#ifndef LBDEM_DEM_STANDIN_H
#define LBDEM_DEM_STANDIN_H

#include <cmath>
#include <cstring>
#include <vector>

namespace LAMMPS_NS {

class Atom {
public:
    int nlocal = 0, nghost = 0;
    double **x = nullptr, **v = nullptr, **omega = nullptr;
    double* radius = nullptr;
    double* rmass = nullptr;
    int *tag = nullptr, *type = nullptr;

    void add(const double p[3], const double vel[3], double r, double density, int t, int ty) {
        px.push_back({p[0], p[1], p[2]});
        pv.push_back({vel[0], vel[1], vel[2]});
        pw.push_back({0, 0, 0});
        pr.push_back(r);
        pm.push_back(density * 4.0 / 3.0 * M_PI * r * r * r);
        ptag.push_back(t);
        ptype.push_back(ty);
        nlocal = (int)px.size();
        bind();
    }
    // atom->map(tag): index of the (owned) atom with this tag
    int map(int t) const {
        for (int i = 0; i < nlocal + nghost; ++i)
            if (ptag[i] == t) return i;
        return -1;
    }

    std::vector<std::vector<double>> px, pv, pw;
    std::vector<double> pr, pm;
    std::vector<int> ptag, ptype;

private:
    std::vector<double*> rx, rv, rw;
    void bind() {
        rx.clear(); rv.clear(); rw.clear();
        for (size_t i = 0; i < px.size(); ++i) { rx.push_back(px[i].data()); rv.push_back(pv[i].data()); rw.push_back(pw[i].data()); }
        x = rx.data(); v = rv.data(); omega = rw.data();
        radius = pr.data(); rmass = pm.data(); tag = ptag.data(); type = ptype.data();
    }
};

class Fix {
public:
    virtual ~Fix() {}
};

// The per-atom dragforce / hdtorque arrays of fix couple/lb/onetoone.
class FixLbCouplingOnetoone : public Fix {
public:
    void resize(int n) {
        f.assign(n, {0, 0, 0}); t.assign(n, {0, 0, 0});
        pf.clear(); pt.clear();
        for (int i = 0; i < n; ++i) { pf.push_back(f[i].data()); pt.push_back(t[i].data()); }
    }
    double** get_force_ptr() { return pf.data(); }
    double** get_torque_ptr() { return pt.data(); }
    void comm_force_torque() {}   // one process: nothing to reverse-communicate
    std::vector<std::vector<double>> f, t;

private:
    std::vector<double*> pf, pt;
};

// fix multisphere: which body (or -1) each tag belongs to.
class FixMultisphere : public Fix {
public:
    std::vector<int> body_of_tag;   // indexed by tag
    int belongs_to(int tag) const {
        return tag >= 0 && tag < (int)body_of_tag.size() ? body_of_tag[tag] : -1;
    }
};

class Modify {
public:
    FixLbCouplingOnetoone* coupling = nullptr;
    FixMultisphere* multisphere = nullptr;
    Fix* find_fix_style(const char* style, int) {
        if (std::strcmp(style, "couple/lb/onetoone") == 0) return coupling;
        if (std::strcmp(style, "multisphere") == 0) return multisphere;
        return nullptr;
    }
    int n_fixes_style(const char* style) { return find_fix_style(style, 0) ? 1 : 0; }
};

class LAMMPS {
public:
    Atom* atom = nullptr;
    Modify* modify = nullptr;
};

}  // namespace LAMMPS_NS

// Stand-in for LiggghtsCouplingWrapper (src/liggghtsCouplingWrapper.h:34-48):
// run(n) advances the particles by n DEM substeps of dt.
class LiggghtsCouplingWrapper {
public:
    LiggghtsCouplingWrapper() {
        lmp = &lammps;
        lammps.atom = &atom;
        lammps.modify = &modify;
        modify.coupling = &fix;
    }
    LAMMPS_NS::LAMMPS* lmp;
    LAMMPS_NS::LAMMPS lammps;
    LAMMPS_NS::Atom atom;
    LAMMPS_NS::Modify modify;
    LAMMPS_NS::FixLbCouplingOnetoone fix;
    double dt = 0.1;            // DEM time step
    double gravity[3] = {0, 0, 0};  // buoyancy-reduced gravity, applied as m g

    void sync() { fix.resize(atom.nlocal + atom.nghost); }

    // Velocity Verlet with forces constant over the substep (hydrodynamic force
    // of the last lattice step + gravity), and the rotational analogue with
    // I = 2/5 m r^2.
    void run(long nSteps) {
        for (long s = 0; s < nSteps; ++s)
            for (int i = 0; i < atom.nlocal; ++i) {
                const double m = atom.rmass[i];
                const double I = 0.4 * m * atom.radius[i] * atom.radius[i];
                for (int d = 0; d < 3; ++d) {
                    const double a = fix.f[i][d] / m + gravity[d];
                    atom.x[i][d] += atom.v[i][d] * dt + 0.5 * a * dt * dt;
                    atom.v[i][d] += a * dt;
                    atom.omega[i][d] += fix.t[i][d] / I * dt;
                }
            }
    }
};

#endif  // LBDEM_DEM_STANDIN_H
