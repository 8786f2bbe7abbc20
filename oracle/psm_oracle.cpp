// CPU restatement of the LBDEMcoupling PSM lattice step -- TEST INFRASTRUCTURE ONLY.
//
// This file is the oracle: the GPU product is checked against it, it is never
// linked into the product library and no product code path calls it.  Only the
// test-suite, the smoke check and the CPU-baseline leg of the benchmark load it.
//
// Parity status: the reference cannot be compiled here (it needs Palabos v1.5r1,
// LIGGGHTS 3.1 and MPI, none of which is present) and ships no golden vectors.
// The reference-owned arithmetic (voxelization, PSM collision, force/torque sum)
// is restated statement by statement from the reference sources cited below and
// is cross-checked against the reference headers compiled against a minimal
// Palabos/LIGGGHTS stand-in (oracle/ref_harness).  The Palabos-owned arithmetic
// (D3Q19 descriptor, BGK, second-order equilibrium, streaming) is restated from
// the published lattice-Boltzmann definitions; for that part parity is UNPINNED.
//
// Reference files followed (paths inside the LBDEMcoupling project):
//   src/ibCompositeDynamics3D.hh:109-116  prepareCollision (fPre copy when sf > SOLFRAC_MIN)
//   src/ibCompositeDynamics3D.hh:118-127  defineVelocity   (f = feq(rhoBar = 0, j = u))
//   src/ibCompositeDynamics3D.hh:130-203  collide          (BGK + B-weighted solid collision + force)
//   src/ibProcessors3D.h:43-45            SetSingleSphere3D bounding box (double -> plint truncation)
//   src/ibProcessors3D.hh:53-114          SetSingleSphere3D::process (decFlag owner resolution)
//   src/ibProcessors3D.hh:117-158         calcSolidFraction (5^3 sub-cell sampling)
//   src/ibProcessors3D.hh:163-184         setValues / setToZero
//   src/ibProcessors3D.hh:203-263         SumForceTorque3D::process (minimum image, r x F)
//   src/ibDataExchangeWrappers3D.hh:33-146  sphere order (locals then ghosts), bbox ∩ local block
//   src/ibDataExchangeWrappers3D.hh:160-246 zeroing and per-index accumulation
//   src/ibDef.h:24-27                     LBDEM_USE_WEIGHING, SOLFRAC_MIN, SOLFRAC_MAX
//
// Build with -ffp-contract=off so that no multiply-add is fused: the voxel
// counts and the particle surface velocity are bit-exact IEEE double results.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double SOLFRAC_MIN = 0.001;   // src/ibDef.h:26
constexpr double SOLFRAC_MAX = 0.999;   // src/ibDef.h:27
constexpr int Q = 19;

// Palabos D3Q19 ordering: c[i+9] = -c[i] for i = 1..9 (the reference relies on
// iOpp = iPop + q/2, src/ibCompositeDynamics3D.hh:165,189).
const int C[Q][3] = {
    {0, 0, 0},
    {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {-1, -1, 0}, {-1, 1, 0},
    {-1, 0, -1}, {-1, 0, 1}, {0, -1, -1}, {0, -1, 1},
    {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, -1, 0},
    {1, 0, 1}, {1, 0, -1}, {0, 1, 1}, {0, 1, -1}};
const double W[Q] = {1. / 3,
                     1. / 18, 1. / 18, 1. / 18, 1. / 36, 1. / 36, 1. / 36, 1. / 36, 1. / 36, 1. / 36,
                     1. / 18, 1. / 18, 1. / 18, 1. / 36, 1. / 36, 1. / 36, 1. / 36, 1. / 36, 1. / 36};
inline int opp(int i) { return i == 0 ? 0 : (i <= 9 ? i + 9 : i - 9); }

struct Base {
    virtual ~Base() {}
    int prec = 0;
};

template <class T>
struct Lattice : Base {
    int nx, ny, nz;
    int periodic[3];
    double omega;
    double g[3];
    int nthreads;
    size_t N;
    std::vector<T> f, ftmp;        // [19][N], f̄_i = f_i - t_i (Palabos storage)
    std::vector<double> sf;        // solid fraction per cell (reference keeps T = double)
    std::vector<int32_t> id;       // owner particle tag per cell
    std::vector<T> up;             // [3][N] particle surface velocity per cell
    std::vector<T> cf;             // [3][N] hydrodynamic force per cell (lattice units)

    size_t idx(int x, int y, int z) const { return ((size_t)x * ny + y) * nz + z; }
};

// Second-order equilibrium in f̄ form, written from the lattice-Boltzmann
// definition: feq_i = t_i [rhoBar + 3 c_i.j + invRho (4.5 (c_i.j)^2 - 1.5 j.j)].
// (Palabos dynamicsTemplates::bgk_ma2_equilibria, called at
// src/ibCompositeDynamics3D.hh:150-157.)
template <class T>
inline T feq(int i, T rhoBar, T invRho, const T j[3], T jSqr) {
    T cj = (T)C[i][0] * j[0] + (T)C[i][1] * j[1] + (T)C[i][2] * j[2];
    return (T)W[i] * (rhoBar + (T)3 * cj + invRho * ((T)4.5 * cj * cj - (T)1.5 * jSqr));
}

template <class T>
inline void moments(const T* f, T& rhoBar, T j[3]) {
    rhoBar = 0; j[0] = j[1] = j[2] = 0;
    for (int i = 0; i < Q; ++i) {
        rhoBar += f[i];
        j[0] += (T)C[i][0] * f[i];
        j[1] += (T)C[i][1] * f[i];
        j[2] += (T)C[i][2] * f[i];
    }
}

// BGK collision of the base dynamics (Palabos BGKdynamics::collide, invoked
// through CompositeDynamics::collide at src/ibCompositeDynamics3D.hh:139-140).
// With a non-zero body force the Guo forcing scheme is applied; the reference
// never combines a body force with the PSM dynamics, so this is an extension
// whose definition is fixed here and mirrored by the GPU kernel.
template <class T>
inline void bgk(T* f, T omega, const double gd[3], bool force) {
    T rhoBar, j[3];
    moments(f, rhoBar, j);
    T rho = (T)1 + rhoBar;
    T invRho = (T)1 / rho;
    if (!force) {
        T jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
        for (int i = 0; i < Q; ++i)
            f[i] = f[i] * ((T)1 - omega) + omega * feq(i, rhoBar, invRho, j, jSqr);
        return;
    }
    T g[3] = {(T)gd[0], (T)gd[1], (T)gd[2]};
    T jF[3], u[3];
    for (int d = 0; d < 3; ++d) {
        jF[d] = j[d] + (T)0.5 * rho * g[d];
        u[d] = jF[d] * invRho;
    }
    T jSqr = jF[0] * jF[0] + jF[1] * jF[1] + jF[2] * jF[2];
    T pre = ((T)1 - (T)0.5 * omega) * rho;
    for (int i = 0; i < Q; ++i) {
        T cu = (T)C[i][0] * u[0] + (T)C[i][1] * u[1] + (T)C[i][2] * u[2];
        T cg = (T)C[i][0] * g[0] + (T)C[i][1] * g[1] + (T)C[i][2] * g[2];
        T ug = u[0] * g[0] + u[1] * g[1] + u[2] * g[2];
        T src = (T)W[i] * pre * ((T)3 * (cg - ug) + (T)9 * cu * cg);
        f[i] = f[i] * ((T)1 - omega) + omega * feq(i, rhoBar, invRho, jF, jSqr) + src;
    }
}

// IBcompositeDynamics::collide, src/ibCompositeDynamics3D.hh:130-203.
template <class T>
inline void psm_collide(T* f, double sfd, const T up[3], T F[3], T omega, double ooo,
                        const double g[3], bool force) {
    T fPre[Q];
    if (sfd > SOLFRAC_MIN)                                   // prepareCollision :109-116
        for (int i = 0; i < Q; ++i) fPre[i] = f[i];
    F[0] = F[1] = F[2] = 0;                                  // :137
    if (sfd <= SOLFRAC_MAX) bgk(f, omega, g, force);         // :139-140
    if (sfd < SOLFRAC_MIN) return;                           // :143-144
    T rhoBar, j[3];
    moments(f, rhoBar, j);                                   // :146-148, post-collision moments
    T jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    T invRho = (T)1 / ((T)1 + rhoBar);
    T fEq[Q], fEqS[Q];
    for (int i = 0; i < Q; ++i) fEq[i] = feq(i, rhoBar, invRho, j, jSqr);
    T uP[3] = {up[0] * ((T)1 + rhoBar), up[1] * ((T)1 + rhoBar), up[2] * ((T)1 + rhoBar)};  // :154
    T uPSqr = uP[0] * uP[0] + uP[1] * uP[1] + uP[2] * uP[2];
    for (int i = 0; i < Q; ++i) fEqS[i] = feq(i, rhoBar, invRho, uP, uPSqr);
    if (sfd > SOLFRAC_MAX) {                                 // :160-175 full solid, no BGK
        T bb0 = fEq[0] - fEqS[0];
        f[0] = fPre[0] + bb0;
        for (int i = 1; i <= 9; ++i) {
            int o = i + 9;
            T bb = (fPre[o] - fEq[o]) - (fPre[i] - fEqS[i]);
            T bbOpp = (fPre[i] - fEq[i]) - (fPre[o] - fEqS[o]);
            f[i] = fPre[i] + bb;
            f[o] = fPre[o] + bbOpp;
            for (int d = 0; d < 3; ++d) F[d] -= (T)C[i][d] * (bb - bbOpp);
        }
    } else {                                                 // :177-200 partial, B-weighted
        T B = (T)(sfd * ooo / ((1. - sfd) + ooo));           // :178-179 (LBDEM_USE_WEIGHING)
        T oneMinB = (T)1 - B;
        T bb0 = fEq[0] - fEqS[0];
        f[0] = fPre[0] + oneMinB * (f[0] - fPre[0]) + B * bb0;
        for (int i = 1; i <= 9; ++i) {
            int o = i + 9;
            T bb = B * ((fPre[o] - fEq[o]) - (fPre[i] - fEqS[i]));
            T bbOpp = B * ((fPre[i] - fEq[i]) - (fPre[o] - fEqS[o]));
            f[i] = fPre[i] + oneMinB * (f[i] - fPre[i]) + bb;
            f[o] = fPre[o] + oneMinB * (f[o] - fPre[o]) + bbOpp;
            for (int d = 0; d < 3; ++d) F[d] -= (T)C[i][d] * (bb - bbOpp);
        }
    }
}

// calcSolidFraction, src/ibProcessors3D.hh:117-158, returned as the sample
// count n in [0,125] (sf = n/125; 1/125*125 == 1.0 exactly, so the early-out
// "return 1" is n = 125 and "return 0" is n = 0).
inline int solid_count(double dx_, double dy_, double dz_, double r_) {
    const double sliceWidth = 1. / 5.;
    const double sqrt3half = std::sqrt(3.1) / 2.;
    double dist = dx_ * dx_ + dy_ * dy_ + dz_ * dz_;
    double r_p = r_ + sqrt3half;
    if (dist > r_p * r_p) return 0;
    double r_m = r_ - sqrt3half;
    if (dist < r_m * r_m) return 125;
    double r_sq = r_ * r_;
    double xs[5], ys[5], zs[5];
    for (int i = 0; i < 5; ++i) {
        double delta = -0.5 + ((double)i + 0.5) * sliceWidth;
        double dx = dx_ + delta; xs[i] = dx * dx;
        double dy = dy_ + delta; ys[i] = dy * dy;
        double dz = dz_ + delta; zs[i] = dz * dz;
    }
    int n = 0;
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j)
            for (int k = 0; k < 5; ++k) n += (xs[i] + ys[j] + zs[k] < r_sq);
    return n;
}

template <class T>
void equilibrium_pops(T out[Q], double rhoBar, const double u[3]) {
    // Palabos iniCellAtEquilibrium semantics: j = rho u.
    T rb = (T)rhoBar;
    T rho = (T)1 + rb;
    T j[3] = {rho * (T)u[0], rho * (T)u[1], rho * (T)u[2]};
    T jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    T invRho = (T)1 / rho;
    for (int i = 0; i < Q; ++i) out[i] = feq(i, rb, invRho, j, jSqr);
}

template <class T>
void set_spheres(Lattice<T>& L, int n, const double* x, const double* v, const double* w,
                 const double* r, const int32_t* tag, int initVel) {
    const int dims[3] = {L.nx, L.ny, L.nz};
    for (int s = 0; s < n; ++s) {                            // ibDataExchangeWrappers3D.hh:62 order
        const double* xs = x + 3 * s;
        const double* vs = v + 3 * s;
        const double* ws = w + 3 * s;
        double rs = r[s];
        int32_t id = tag[s];
        long lo[3], hi[3];
        bool empty = false;
        for (int d = 0; d < 3; ++d) {                        // ibProcessors3D.h:43-45, plint truncation
            lo[d] = (long)(xs[d] - rs - 2);
            hi[d] = (long)(xs[d] + rs + 2);
            lo[d] = std::max<long>(lo[d], 0);                // intersect with the local block,
            hi[d] = std::min<long>(hi[d], dims[d] - 1);      // ibDataExchangeWrappers3D.hh:127-133
            if (lo[d] > hi[d]) empty = true;
        }
        if (empty) continue;
        auto body = [&](long iX) {
            for (long iY = lo[1]; iY <= hi[1]; ++iY)
                for (long iZ = lo[2]; iZ <= hi[2]; ++iZ) {
                    size_t c = L.idx((int)iX, (int)iY, (int)iZ);
                    double xG = (double)iX, yG = (double)iY, zG = (double)iZ;
                    double dx = xG - xs[0], dy = yG - xs[1], dz = zG - xs[2];
                    int nsub = solid_count(dx, dy, dz, rs);
                    double sfv = (1. / 125.) * (double)nsub;
                    double sf_old = L.sf[c];
                    int id_old = L.id[c];
                    int decFlag = (sfv > SOLFRAC_MIN) + 2 * (sf_old > SOLFRAC_MIN);
                    bool setv = false, zero = false;
                    switch (decFlag) {                       // ibProcessors3D.hh:88-105
                        case 0: zero = true; break;
                        case 1: setv = true; break;
                        case 2: if (id_old == id) zero = true; break;
                        case 3: if (sfv > sf_old || id_old == id) setv = true; break;
                    }
                    if (zero) {
                        L.sf[c] = 0; L.id[c] = 0;
                        for (int d = 0; d < 3; ++d) L.up[d * L.N + c] = 0;
                    }
                    if (setv) {                              // setValues, :163-174
                        double u0 = vs[0] + (ws[1] * dz - ws[2] * dy);
                        double u1 = vs[1] + (-ws[0] * dz + ws[2] * dx);
                        double u2 = vs[2] + (ws[0] * dy - ws[1] * dx);
                        L.up[0 * L.N + c] = (T)u0;
                        L.up[1 * L.N + c] = (T)u1;
                        L.up[2 * L.N + c] = (T)u2;
                        L.sf[c] = sfv;
                        L.id[c] = id;
                    }
                    if (initVel && sfv > SOLFRAC_MAX) {      // :107-108 -> defineVelocity :118-127
                        T u[3] = {L.up[c], L.up[L.N + c], L.up[2 * L.N + c]};
                        T uSqr = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
                        for (int i = 0; i < Q; ++i) L.f[i * L.N + c] = feq(i, (T)0, (T)1, u, uSqr);
                    }
                }
        };
#ifdef _OPENMP
        if (L.nthreads > 1) {
#pragma omp parallel for num_threads(L.nthreads) schedule(static)
            for (long iX = lo[0]; iX <= hi[0]; ++iX) body(iX);
        } else
#endif
            for (long iX = lo[0]; iX <= hi[0]; ++iX) body(iX);
    }
}

template <class T>
void collide_stream(Lattice<T>& L) {
    const T omega = (T)L.omega;
    const double ooo = 1. / L.omega - 0.5;
    const bool force = (L.g[0] != 0 || L.g[1] != 0 || L.g[2] != 0);
    const size_t N = L.N;
    auto collide_x = [&](int x) {
        for (int y = 0; y < L.ny; ++y)
            for (int z = 0; z < L.nz; ++z) {
                size_t c = L.idx(x, y, z);
                T fl[Q];
                for (int i = 0; i < Q; ++i) fl[i] = L.f[i * N + c];
                T up[3] = {L.up[c], L.up[N + c], L.up[2 * N + c]};
                T F[3];
                psm_collide(fl, L.sf[c], up, F, omega, ooo, L.g, force);
                for (int i = 0; i < Q; ++i) L.f[i * N + c] = fl[i];
                for (int d = 0; d < 3; ++d) L.cf[d * N + c] = F[d];
            }
    };
    // Push streaming f_i(x + c_i) <- f*_i(x); periodic axes wrap, other axes
    // apply half-way bounce-back: a population leaving the box returns to its
    // cell in the opposite direction.
    auto stream_x = [&](int x) {
        for (int y = 0; y < L.ny; ++y)
            for (int z = 0; z < L.nz; ++z) {
                size_t c = L.idx(x, y, z);
                for (int i = 0; i < Q; ++i) {
                    int p[3] = {x + C[i][0], y + C[i][1], z + C[i][2]};
                    const int dims[3] = {L.nx, L.ny, L.nz};
                    bool out = false;
                    for (int d = 0; d < 3; ++d) {
                        if (p[d] < 0 || p[d] >= dims[d]) {
                            if (L.periodic[d]) p[d] = (p[d] + dims[d]) % dims[d];
                            else out = true;
                        }
                    }
                    if (out) L.ftmp[opp(i) * N + c] = L.f[i * N + c];
                    else L.ftmp[i * N + L.idx(p[0], p[1], p[2])] = L.f[i * N + c];
                }
            }
    };
#ifdef _OPENMP
    if (L.nthreads > 1) {
#pragma omp parallel for num_threads(L.nthreads) schedule(static)
        for (int x = 0; x < L.nx; ++x) collide_x(x);
#pragma omp parallel for num_threads(L.nthreads) schedule(static)
        for (int x = 0; x < L.nx; ++x) stream_x(x);
    } else
#endif
    {
        for (int x = 0; x < L.nx; ++x) collide_x(x);
        for (int x = 0; x < L.nx; ++x) stream_x(x);
    }
    std::swap(L.f, L.ftmp);
}

// SumForceTorque3D::process, src/ibProcessors3D.hh:203-263, plus the zeroing
// and indexing of getForcesFromLattice, src/ibDataExchangeWrappers3D.hh:160-218.
// atom->map(tag) is LAMMPS' map: the lowest local index holding that tag (owned
// atoms precede their ghost images).  Cells whose tag has no particle are
// counted and skipped (the reference would index force[-3]).
template <class T>
long sum_force_torque(const Lattice<T>& L, int n, const double* x, const int32_t* tag,
                      double* F, double* Tq) {
    for (int i = 0; i < 3 * n; ++i) { F[i] = 0; Tq[i] = 0; }
    if (n == 0) return 0;
    int32_t maxTag = 0;
    for (int i = 0; i < n; ++i) maxTag = std::max(maxTag, tag[i]);
    std::vector<int> map((size_t)maxTag + 1, -1);
    for (int i = n - 1; i >= 0; --i) if (tag[i] >= 0) map[tag[i]] = i;
    const long nx = L.nx, ny = L.ny, nz = L.nz;
    long unmapped = 0;
    const size_t N = L.N;
    for (long iX = 0; iX < nx; ++iX)
        for (long iY = 0; iY < ny; ++iY)
            for (long iZ = 0; iZ < nz; ++iZ) {
                size_t c = L.idx((int)iX, (int)iY, (int)iZ);
                long id = L.id[c];
                if (id < 1) continue;
                long ind = (id <= maxTag) ? map[id] : -1;
                if (ind < 0) { ++unmapped; continue; }
                double dx = (double)iX - x[3 * ind + 0];
                double dy = (double)iY - x[3 * ind + 1];
                double dz = (double)iZ - x[3 * ind + 2];
                if (dx > nx / 2) dx -= nx; else if (dx < -nx / 2) dx += nx;
                if (dy > ny / 2) dy -= ny; else if (dy < -ny / 2) dy += ny;
                if (dz > nz / 2) dz -= nz; else if (dz < -nz / 2) dz += nz;
                double fX = (double)L.cf[c], fY = (double)L.cf[N + c], fZ = (double)L.cf[2 * N + c];
                double tX = dy * fZ - dz * fY;
                double tY = -dx * fZ + dz * fX;
                double tZ = dx * fY - dy * fX;
                F[3 * ind + 0] += fX; F[3 * ind + 1] += fY; F[3 * ind + 2] += fZ;
                Tq[3 * ind + 0] += tX; Tq[3 * ind + 1] += tY; Tq[3 * ind + 2] += tZ;
            }
    return unmapped;
}

// ---- periodic pressure drop and initial profiles (src/periodicPressureFunctionals3D.hh) ----
//
// box = {x0, x1, y0, y1, z0, z1}, inclusive, as Palabos' Box3D.

// Palabos computeAverageDensity(lattice, box): fullRho(sum rhoBar / nCells), with
// fullRho(rhoBar) = 1 + rhoBar for D3Q19; the sum runs in the reference's cell
// order (x outer, z inner), rhoBar of a cell summed over i = 0..18.
template <class T>
double average_density(const Lattice<T>& L, const int32_t b[6]) {
    double s = 0;
    for (int x = b[0]; x <= b[1]; ++x)
        for (int y = b[2]; y <= b[3]; ++y)
            for (int z = b[4]; z <= b[5]; ++z) {
                double rb = 0;
                for (int i = 0; i < Q; ++i) rb += (double)L.f[i * L.N + L.idx(x, y, z)];
                s += rb;
            }
    const double n = (double)(b[1] - b[0] + 1) * (double)(b[3] - b[2] + 1) * (double)(b[5] - b[4] + 1);
    return 1.0 + s / n;
}

// ZhangPeriodicPressureFunctional3D (src/periodicPressureFunctionals3D.hh:121-159):
// the populations with c_i[dimension] == direction are rescaled as
// f_i + t_i <- (f_i + t_i) * rhoTarget / rhoAvg.  The float lattice evaluates the
// same expression in double and rounds once.
template <class T>
void zhang_rescale(Lattice<T>& L, const int32_t b[6], int dim, int dir, double rhoTarget, double rhoAvg) {
    const double k = rhoTarget / rhoAvg;                              // :140
    for (int x = b[0]; x <= b[1]; ++x)
        for (int y = b[2]; y <= b[3]; ++y)
            for (int z = b[4]; z <= b[5]; ++z)
                for (int i = 0; i < Q; ++i) {
                    if (C[i][dim] != dir) continue;                   // rescalePop, :126-130
                    T& f = L.f[i * L.N + L.idx(x, y, z)];
                    double t = (double)f + W[i];                       // :151-153
                    t *= k;
                    f = (T)(t - W[i]);
                }
}

// PressureGradient (kind 0, :242-256) and PoiseuilleProfileAndPressureGradient
// (kind 1, :267-298) applied through Palabos initializeAtEquilibrium: every cell
// gets feq(rhoBar = density - 1, j = density u).  n[3] are the functor's grid
// sizes (PressureGradient uses n[dimension]).
template <class T>
void init_profile(Lattice<T>& L, int kind, double pHi, double pLo, double uMax, const int32_t n[3], int dim) {
    auto pv = [](double i, double nn) {                              // poiseuilleVelocity, :293-298
        double nHalf = nn / 2.;
        double x = (i - nHalf) / nHalf;
        return 1. - x * x;
    };
    for (int x = 0; x < L.nx; ++x)
        for (int y = 0; y < L.ny; ++y)
            for (int z = 0; z < L.nz; ++z) {
                const int ii[3] = {x, y, z};
                double density = pHi - (pHi - pLo) * (double)ii[dim] / (double)(n[dim] - 1);
                double u[3] = {0, 0, 0};
                if (kind == 1) {
                    const int a = dim == 0 ? 1 : 0, c = dim == 2 ? 1 : 2;
                    u[dim] = uMax * pv((double)ii[a], (double)n[a]) * pv((double)ii[c], (double)n[c]);
                }
                T e[Q];
                equilibrium_pops<T>(e, density - 1.0, u);
                for (int i = 0; i < Q; ++i) L.f[i * L.N + L.idx(x, y, z)] = e[i];
            }
}

template <class T>
Lattice<T>* make(int nx, int ny, int nz, const int per[3], double omega, const double g[3], int nth) {
    auto* L = new Lattice<T>();
    L->prec = sizeof(T) == 8 ? 0 : 1;
    L->nx = nx; L->ny = ny; L->nz = nz;
    for (int d = 0; d < 3; ++d) { L->periodic[d] = per[d]; L->g[d] = g[d]; }
    L->omega = omega;
    L->nthreads = nth < 1 ? 1 : nth;
    L->N = (size_t)nx * ny * nz;
    L->f.assign(Q * L->N, (T)0);
    L->ftmp.assign(Q * L->N, (T)0);
    L->sf.assign(L->N, 0.0);
    L->id.assign(L->N, 0);
    L->up.assign(3 * L->N, (T)0);
    L->cf.assign(3 * L->N, (T)0);
    return L;
}

}  // namespace

#define DISPATCH(h, CALL)                                           \
    do {                                                            \
        Base* b_ = (Base*)(h);                                      \
        if (b_->prec == 0) { auto& L = *(Lattice<double>*)b_; CALL; } \
        else { auto& L = *(Lattice<float>*)b_; CALL; }              \
    } while (0)

extern "C" {

// precision: 0 = double populations, 1 = float populations (deviation form).
void* orc_create(int precision, int nx, int ny, int nz, int px, int py, int pz, double omega,
                 double gx, double gy, double gz, int nthreads) {
    const int per[3] = {px, py, pz};
    const double g[3] = {gx, gy, gz};
    if (nx <= 0 || ny <= 0 || nz <= 0 || !(omega > 0 && omega < 2)) return nullptr;
    if (precision == 0) return make<double>(nx, ny, nz, per, omega, g, nthreads);
    return make<float>(nx, ny, nz, per, omega, g, nthreads);
}

void orc_destroy(void* h) { delete (Base*)h; }

void orc_set_threads(void* h, int nthreads) {
    DISPATCH(h, L.nthreads = nthreads < 1 ? 1 : nthreads);
}

// Populations f̄_i in [19][nx][ny][nz] order (z fastest), element type of the lattice.
void orc_set_pops(void* h, const void* f) {
    DISPATCH(h, std::memcpy(L.f.data(), f, L.f.size() * sizeof(L.f[0])));
}
void orc_get_pops(void* h, void* f) {
    DISPATCH(h, std::memcpy(f, L.f.data(), L.f.size() * sizeof(L.f[0])));
}

void orc_init_equilibrium(void* h, double rhoBar, double ux, double uy, double uz) {
    const double u[3] = {ux, uy, uz};
    DISPATCH(h, {
        using TT = typename std::remove_reference<decltype(L.f[0])>::type;
        TT e[Q];
        equilibrium_pops<TT>(e, rhoBar, u);
        for (int i = 0; i < Q; ++i) std::fill(L.f.begin() + i * L.N, L.f.begin() + (i + 1) * L.N, e[i]);
    });
}

void orc_set_spheres(void* h, int n, const double* x, const double* v, const double* w,
                     const double* r, const int32_t* tag, int initVel) {
    DISPATCH(h, set_spheres(L, n, x, v, w, r, tag, initVel));
}

void orc_collide_stream(void* h) { DISPATCH(h, collide_stream(L)); }

long orc_sum_force_torque(void* h, int n, const double* x, const int32_t* tag, double* F, double* Tq) {
    long r = 0;
    DISPATCH(h, r = sum_force_torque(L, n, x, tag, F, Tq));
    return r;
}

double orc_average_density(void* h, const int32_t* box) {
    double r = 0;
    DISPATCH(h, r = average_density(L, box));
    return r;
}

void orc_zhang_rescale(void* h, const int32_t* box, int dim, int dir, double rhoTarget, double rhoAvg) {
    DISPATCH(h, zhang_rescale(L, box, dim, dir, rhoTarget, rhoAvg));
}

void orc_init_profile(void* h, int kind, double pHi, double pLo, double uMax, const int32_t* n, int dim) {
    DISPATCH(h, init_profile(L, kind, pHi, pLo, uMax, n, dim));
}

// Per-cell coupling state.  Any pointer may be null.  sf: double[N];
// nsub: uint8[N] (sf*125); id: int32[N]; up, cf: [3][N] of the lattice type.
void orc_get_state(void* h, double* sf, uint8_t* nsub, int32_t* id, void* up, void* cf) {
    DISPATCH(h, {
        if (sf) std::memcpy(sf, L.sf.data(), L.N * sizeof(double));
        if (nsub) for (size_t c = 0; c < L.N; ++c) nsub[c] = (uint8_t)std::lround(L.sf[c] * 125.0);
        if (id) std::memcpy(id, L.id.data(), L.N * sizeof(int32_t));
        if (up) std::memcpy(up, L.up.data(), L.up.size() * sizeof(L.up[0]));
        if (cf) std::memcpy(cf, L.cf.data(), L.cf.size() * sizeof(L.cf[0]));
    });
}

// Total mass sum_cells sum_i (f̄_i + t_i), accumulated in double.
double orc_mass(void* h) {
    double m = 0;
    DISPATCH(h, {
        for (int i = 0; i < Q; ++i) {
            double s = 0;
            for (size_t c = 0; c < L.N; ++c) s += (double)L.f[i * L.N + c];
            m += s + W[i] * (double)L.N;
        }
    });
    return m;
}

// Sub-cell sample count of one cell offset (dx, dy, dz) for radius r.
int orc_solid_count(double dx, double dy, double dz, double r) { return solid_count(dx, dy, dz, r); }

// One full coupling cycle on the lattice: voxelize, collide-stream, sum forces.
long orc_cycle(void* h, int n, const double* x, const double* v, const double* w,
               const double* r, const int32_t* tag, int initVel, double* F, double* Tq) {
    orc_set_spheres(h, n, x, v, w, r, tag, initVel);
    orc_collide_stream(h);
    return orc_sum_force_torque(h, n, x, tag, F, Tq);
}

int orc_has_openmp() {
#ifdef _OPENMP
    return 1;
#else
    return 0;
#endif
}

}  // extern "C"
