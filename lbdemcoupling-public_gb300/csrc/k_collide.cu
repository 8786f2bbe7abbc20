// K1: fused D3Q19 PSM collide-stream kernel with the per-particle force and
// torque reduction folded into the same pass.
//
// Replaces, per lattice step:
//   Palabos collideAndStream with IBcompositeDynamics<T,D3Q19>(BGK) in every
//   cell  -- src/ibCompositeDynamics3D.hh:130-203 (PSM collision, per-cell force)
//   SumForceTorque3D::process -- src/ibProcessors3D.hh:203-263 (sum F, r x F per id)
//
// Streaming is the in-place "AA" pattern on one population array:
//   even phase: cell x reads f_i from slot (i, x), writes f*_i to slot (opp i, x);
//   odd phase:  cell x reads f_i from slot (opp i, x - c_i), writes f*_i to slot
//               (i, x + c_i).
// Both phases read and write exactly the same set of slots per cell, so the
// update is race-free in place.  A neighbour beyond a wall (non-periodic axis)
// is replaced by the cell itself with the direction reversed: half-way
// bounce-back.  Periodic axes wrap.
//
// One kernel implements the step: persistent CTAs of 128 threads whose warps
// walk 64-cell z-segments.  The 19 population rows of a segment (plus, in the
// odd phase, the halo element of every c_z != 0 direction), the voxel words and
// (FP64 form, single lattice) the particle surface-velocity rows are staged in
// shared memory, double-buffered, so the next segment's bytes are in flight while the
// current one is collided: per-thread 16-byte cp.async with commit groups for
// FP32 lattices with 16-byte aligned rows, cp.async.bulk on an mbarrier
// otherwise; rows that are not 16-byte aligned (nz % 4 != 0) are copied in whole
// 16-byte chunks around the row.  The staged pre-collision values double as
// fPre of the PSM update.  The FP32 form collides two cells per thread in packed
// f32x2 arithmetic (collide_segment_pairs) and recomputes the particle surface
// velocity of its solid cells from the owner particle's row of the float table
// (no per-cell velocity field); the FP64 form one cell per thread in double,
// BGK and solid correction in one pass (collide_cell_fp64; with a body force
// collide_cell), with the velocity setValues stored.  The same
// kernel steps many independent domains in one launch (batch mode).
#include "lbdem_internal.h"

#include <cstddef>
#include <type_traits>

namespace lbdem {
namespace {

constexpr unsigned FULL = 0xffffffffu;

// 1/x (the FP64 form; the FP32 form uses __frcp_rn, identical to the IEEE division 1/x).
__device__ __forceinline__ double recip(double x) { return 1.0 / x; }

// c_i . (a, b, c) with the zero terms removed at compile time (0 * x is not
// foldable under IEEE rules, so the sum is built from the non-zero components).
template <typename T>
__device__ __forceinline__ T cdot(int i, T a, T b, T c) {
    const int X = cx(i), Y = cy(i), Z = cz(i);
    T r;
    if (X != 0) {
        r = X > 0 ? a : -a;
        if (Y != 0) r = Y > 0 ? r + b : r - b;
        if (Z != 0) r = Z > 0 ? r + c : r - c;
    } else if (Y != 0) {
        r = Y > 0 ? b : -b;
        if (Z != 0) r = Z > 0 ? r + c : r - c;
    } else if (Z != 0) {
        r = Z > 0 ? c : -c;
    } else {
        r = T(0);
    }
    return r;
}

template <typename T>
__device__ __forceinline__ void moments(const T (&f)[Q], T& rhoBar, T& jx, T& jy, T& jz) {
    rhoBar = ((f[0] + (f[1] + f[10])) + ((f[2] + f[11]) + (f[3] + f[12]))) +
             (((f[4] + f[13]) + (f[5] + f[14])) + ((f[6] + f[15]) + (f[7] + f[16]))) +
             ((f[8] + f[17]) + (f[9] + f[18]));
    jx = ((f[10] + f[13]) + (f[14] + f[15]) + f[16]) - ((f[1] + f[4]) + (f[5] + f[6]) + f[7]);
    jy = ((f[11] + f[13]) + (f[17] + f[18]) + f[5]) - ((f[2] + f[4]) + (f[8] + f[9]) + f[14]);
    jz = ((f[12] + f[15]) + (f[17] + f[7]) + f[9]) - ((f[3] + f[6]) + (f[8] + f[16]) + f[18]);
}

// Zeroth and first moments of a cell, rhoBar = sum f̄, j = sum c f̄, with 1/rho.
template <typename T>
struct Mom {
    T rhoBar, jx, jy, jz, invRho;
};

template <typename T>
__device__ __forceinline__ Mom<T> cell_moments(const T (&f)[Q]) {
    Mom<T> m;
    moments(f, m.rhoBar, m.jx, m.jy, m.jz);
    m.invRho = recip(T(1) + m.rhoBar);
    return m;
}

// BGK relaxation towards the second-order equilibrium
// feq_i = t_i [rhoBar + 3 c.j + invRho (4.5 (c.j)^2 - 1.5 j.j)], written per
// opposite pair (feq_i and feq_{i+9} differ only in the sign of 3 c.j), given
// the cell's pre-collision moments.
// With FORCE the Guo scheme is used (equilibrium momentum j + rho g / 2 plus
// the forcing term t_i (1 - omega/2) rho [3 (c - u).g + 9 (c.u)(c.g)]).
template <typename T, bool FORCE>
__device__ __forceinline__ void bgk(T (&f)[Q], const Mom<T>& m, T omega, T gx, T gy, T gz) {
    const T rhoBar = m.rhoBar, invRho = m.invRho;
    T jx = m.jx, jy = m.jy, jz = m.jz;
    const T rho = T(1) + rhoBar;
    if (FORCE) {
        const T h = T(0.5) * rho;
        jx += h * gx; jy += h * gy; jz += h * gz;
    }
    const T jSqr = jx * jx + jy * jy + jz * jz;
    const T base = rhoBar - T(1.5) * invRho * jSqr;
    const T om1 = T(1) - omega;
    const T q45 = T(4.5) * invRho;
    T ux = T(0), uy = T(0), uz = T(0), pre = T(0), ug = T(0);
    if (FORCE) {
        ux = jx * invRho; uy = jy * invRho; uz = jz * invRho;
        pre = (T(1) - T(0.5) * omega) * rho;
        ug = ux * gx + uy * gy + uz * gz;
    }
    f[0] = om1 * f[0] + (omega * T(wt(0))) * base;
    if (FORCE) f[0] += T(wt(0)) * pre * (T(-3) * ug);
#pragma unroll
    for (int i = 1; i <= 9; ++i) {
        const T cj = cdot(i, jx, jy, jz);
        const T ow = omega * T(wt(i));
        const T e = base + q45 * cj * cj;
        const T s = T(3) * cj;
        f[i] = om1 * f[i] + ow * (e + s);
        f[i + 9] = om1 * f[i + 9] + ow * (e - s);
        if (FORCE) {
            const T cu = cdot(i, ux, uy, uz);
            const T cg = cdot(i, gx, gy, gz);
            const T tp = T(wt(i)) * pre;
            // direction i: c = c_i ; direction i+9: c = -c_i
            f[i] += tp * (T(3) * (cg - ug) + T(9) * cu * cg);
            f[i + 9] += tp * (T(3) * (-cg - ug) + T(9) * cu * cg);
        }
    }
}

// Solid correction of a cell with n > 0 solid sub-cells,
// src/ibCompositeDynamics3D.hh:150-200.  On entry f holds the BGK
// post-collision state (fPre itself for n == 125, where B = 1 reduces the
// weighted update to fPre + bb exactly), m its moments, and pre(i) returns
// the pre-collision value fPre_i.  With feq (m) and the solid equilibrium
// feqS (rhoBar, uPart (1 + rhoBar)) written per opposite pair,
//   bb    = B ((fPre_o - feq_o) - (fPre_i - feqS_i)) = B (D + A + S)
//   bbOpp = B ((fPre_i - feq_i) - (fPre_o - feqS_o)) = B (A - D - S)
// with D = fPre_o - fPre_i, A = t_i (eS - eE), S = 3 t_i (c.j + c.uP), so the
// force term bb - bbOpp = 2 B (D + S).
template <typename T, typename Pre>
__device__ __forceinline__ void psm(T (&f)[Q], const Mom<T>& m, T up0, T up1, T up2, T B, const Pre& pre, T& Fx,
                                    T& Fy, T& Fz) {
    const T rhoBar = m.rhoBar, jx = m.jx, jy = m.jy, jz = m.jz, invRho = m.invRho;
    const T rho = T(1) + rhoBar;
    const T ux = up0 * rho, uy = up1 * rho, uz = up2 * rho;   // uPart (1 + rhoBar), :154
    const T q45 = T(4.5) * invRho;
    // eS - eE for c = 0: -1.5 invRho (uP^2 - j^2)
    const T dB = T(-1.5) * invRho * ((ux * ux + uy * uy + uz * uz) - (jx * jx + jy * jy + jz * jz));
    const T omB = T(1) - B;
    const T B2 = B + B;
    {
        const T p0 = pre(0);
        f[0] = p0 + omB * (f[0] - p0) - B * (T(wt(0)) * dB);   // B (feq_0 - feqS_0)
    }
    Fx = T(0); Fy = T(0); Fz = T(0);
#pragma unroll
    for (int i = 1; i <= 9; ++i) {
        const int o = i + 9;
        const T t = T(wt(i));
        const T cj = cdot(i, jx, jy, jz);
        const T cu = cdot(i, ux, uy, uz);
        const T A = t * (dB + q45 * ((cu - cj) * (cu + cj)));
        const T S = (T(3) * t) * (cj + cu);
        const T pi = pre(i), po = pre(o);
        const T D = po - pi;
        const T bb = B * (D + A + S);
        const T bbOpp = B * (A - D - S);
        f[i] = pi + omB * (f[i] - pi) + bb;
        f[o] = po + omB * (f[o] - po) + bbOpp;
        const T d = B2 * (D + S);                    // bb - bbOpp; F -= c_i (bb - bbOpp), :172-174
        if (cx(i) > 0) Fx -= d; else if (cx(i) < 0) Fx += d;
        if (cy(i) > 0) Fy -= d; else if (cy(i) < 0) Fy += d;
        if (cz(i) > 0) Fz -= d; else if (cz(i) < 0) Fz += d;
    }
}

// Collision of one cell given its pre-collision populations: BGK for every
// cell below full coverage (src/ibCompositeDynamics3D.hh:139-140), then the
// solid correction for cells with n > 0.  Written as two convergent blocks so
// that a warp mixing fluid and solid cells runs the BGK once.  Without a body
// force BGK conserves rhoBar and j, so the solid correction reuses the
// pre-collision moments (the reference recomputes them from the post-collision
// populations, :146-148; the two differ by rounding only); with the Guo force
// the post-collision moments are recomputed.
// up(d) returns component d of the cell's particle surface velocity.
template <typename T, bool FORCE, typename Pre, typename Up>
__device__ __forceinline__ void collide_cell(const CollideArgs<T>& a, T (&f)[Q], uint32_t w, const Pre& pre,
                                             const Up& up, T& Fx, T& Fy, T& Fz) {
    const int n = min((int)(w & VOX_NMASK), 125);
    Fx = T(0); Fy = T(0); Fz = T(0);
    Mom<T> m = cell_moments(f);
    if (n < 125) bgk<T, FORCE>(f, m, a.omega, a.g3[0], a.g3[1], a.g3[2]);
    if (n > 0) {
        if (FORCE && n < 125) m = cell_moments(f);
        psm<T>(f, m, up(0), up(1), up(2), __ldg(a.btab + n), pre, Fx, Fy, Fz);
    }
}

// ---------------------------------------------------------------------------
// FP64 form without a body force: the base BGK (src/ibCompositeDynamics3D.hh:139-140)
// and the solid correction (:150-200) of a cell in one pass over the opposite
// pairs (i = 1..9, k = i + 9, c_k = -c_i), written around the non-equilibrium
// parts g = fPre - feq.  With the solid equilibrium feqS at P = (1 + rhoBar) uPart
// (:154), Dl = feq - feqS and alpha = omega (1 - B) + B, the reference's
//   out = fPre + (1 - B)(fBGK - fPre) + bb,  fBGK = fPre - omega g,
// becomes
//   out_i = fPre_i - alpha g_i + B (g_k - Dl_i),   out_k = fPre_k - alpha g_k + B (g_i - Dl_k),
//   out_0 = fPre_0 - omega (1 - B) g_0 + B Dl_0     (the rest-population sign, :161, :185),
//   F -= c_i (bb - bbOpp) = c_k 2 B ((fPre_k - fPre_i) - 3 t c_k.(j + P))   (:172-174),
// where, with cj = c_k.j and cP = c_k.P,
//   feq_{k,i} = C +/- 3 t cj,  C = t (rhoBar + invRho (4.5 cj^2 - 1.5 j.j)),
//   Dl_{k,i} = Qd +/- 3 t (cj - cP),  Qd = t invRho (4.5 (cj - cP)(cj + cP) - 1.5 (j.j - P.P)),
//   Dl_0 = t_0 (-1.5 invRho (j.j - P.P)).
// n = 125 gives B = 1 (no BGK, alpha = 1), n = 0 gives B = 0 (the BGK result).
// The moments are those of fPre: without a body force BGK conserves them, and the
// reference's post-collision recomputation (:146-148) differs by rounding only.
// SOLID false (a warp without solid cells) leaves out the solid terms; a fluid
// cell gets the same bits either way, so results do not depend on which cells
// share a warp.
template <int AX>
__device__ __forceinline__ double pair_sum(const double (&d)[9]) {
    // sum_k c_k[AX] d[k - 10] over the directions k = 10..18 with c_k[AX] != 0, in k order
    double r = 0.0;
    bool any = false;
#pragma unroll
    for (int k = 10; k < Q; ++k) {
        const int c = AX == 0 ? cx(k) : (AX == 1 ? cy(k) : cz(k));
        if (c == 0) continue;
        const double v = d[k - 10];
        r = any ? (c > 0 ? r + v : r - v) : (c > 0 ? v : -v);
        any = true;
    }
    return r;
}

template <bool SOLID>
__device__ __forceinline__ void collide_cell_fp64(double (&f)[Q], double omega, double B, double up0, double up1,
                                                  double up2, double& Fx, double& Fy, double& Fz) {
    double d[9];
    double rhoBar;
    {
        double s[9];
#pragma unroll
        for (int i = 1; i <= 9; ++i) {
            s[i - 1] = f[i] + f[i + 9];
            d[i - 1] = f[i + 9] - f[i];
        }
        rhoBar = f[0] + ((((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]))) + s[8]);
    }
    const double jx = pair_sum<0>(d), jy = pair_sum<1>(d), jz = pair_sum<2>(d);
    const double invRho = recip(1.0 + rhoBar);
    const double jSqr = fma(jz, jz, fma(jy, jy, jx * jx));
    const double m15 = -1.5 * invRho;
    const double base = fma(m15, jSqr, rhoBar);
    double Px = 0.0, Py = 0.0, Pz = 0.0, dd = 0.0, alpha = omega, om1B = omega;
    if (SOLID) {
        const double rho = 1.0 + rhoBar;
        Px = up0 * rho; Py = up1 * rho; Pz = up2 * rho;
        const double PSqr = fma(Pz, Pz, fma(Py, Py, Px * Px));
        dd = m15 * (jSqr - PSqr);
        alpha = fma(B, 1.0 - omega, omega);
        om1B = omega * (1.0 - B);
    }
    {
        const double g0 = f[0] - wt(0) * base;
        f[0] = SOLID ? fma(B, wt(0) * dd, fma(-om1B, g0, f[0])) : fma(-omega, g0, f[0]);
    }
    double Ex = 0.0, Ey = 0.0, Ez = 0.0;
    bool fx0 = false, fy0 = false, fz0 = false;
#pragma unroll
    for (int k = 10; k < Q; ++k) {
        const int i = k - 9;
        const double t = wt(k), t3 = 3.0 * wt(k);
        const double a45 = (4.5 * wt(k)) * invRho;
        const double cj = cdot(k, jx, jy, jz);
        const double C = fma(a45 * cj, cj, t * base);
        const double Lj = t3 * cj;
        const double gi = (f[i] - C) + Lj;
        const double gk = (f[k] - C) - Lj;
        if (SOLID) {
            const double cP = cdot(k, Px, Py, Pz);
            const double m = cj - cP, p = cj + cP;
            const double Qd = fma(a45 * m, p, t * dd);
            const double L = t3 * m;
            const double e = d[i - 1] - t3 * p;
            f[i] = fma(B, (gk - Qd) + L, fma(-alpha, gi, f[i]));
            f[k] = fma(B, (gi - Qd) - L, fma(-alpha, gk, f[k]));
            if (cx(k) != 0) { Ex = fx0 ? (cx(k) > 0 ? Ex + e : Ex - e) : (cx(k) > 0 ? e : -e); fx0 = true; }
            if (cy(k) != 0) { Ey = fy0 ? (cy(k) > 0 ? Ey + e : Ey - e) : (cy(k) > 0 ? e : -e); fy0 = true; }
            if (cz(k) != 0) { Ez = fz0 ? (cz(k) > 0 ? Ez + e : Ez - e) : (cz(k) > 0 ? e : -e); fz0 = true; }
        } else {
            f[i] = fma(-omega, gi, f[i]);
            f[k] = fma(-omega, gk, f[k]);
        }
    }
    const double B2 = B + B;
    Fx = SOLID ? B2 * Ex : 0.0;
    Fy = SOLID ? B2 * Ey : 0.0;
    Fz = SOLID ? B2 * Ez : 0.0;
}

// Per-cell force and torque added to the particle's sums (FP64 form): six
// double atomics per solid cell, resolved in L2 instead of a warp scan on the
// FP64 pipe.
__device__ __forceinline__ void add_cell_force(const CollideArgs<double>& a, int slot, const double (&v)[6]) {
    double* Fp = a.ft + 3 * (size_t)slot;
    double* Tp = a.ft + 3 * (size_t)a.nslot + 3 * (size_t)slot;
    atomicAdd(Fp + 0, v[0]); atomicAdd(Fp + 1, v[1]); atomicAdd(Fp + 2, v[2]);
    atomicAdd(Tp + 0, v[3]); atomicAdd(Tp + 1, v[4]); atomicAdd(Tp + 2, v[5]);
}

// ---------------------------------------------------------------------------
// FP32 form: two cells per thread in packed f32x2 arithmetic (sm_100 family
// add/sub/mul/fma .f32x2), the cells z and z + 1 of one row.  The same update as
// collide_cell, arranged per opposite pair around the direction k = i + 9 (every
// c_k has a non-negative first non-zero component, so c_k . v needs no
// negation), with two algebraically equal rewrites:
//   * the solid correction is applied as f + B ((fPre - f) + X), which leaves a
//     fluid cell (B = 0) exactly unchanged, so a pair mixing a fluid and a solid
//     cell runs it for both without a select;
//   * with the Guo force the solid correction's momentum is the BGK post-collision
//     momentum j + rho g (exact in arithmetic) instead of a second moment sum.
// Rounding differs from the FP64 form at the float level.
struct F2 {
    unsigned long long r;
};
__device__ __forceinline__ F2 pk(float a, float b) {
    F2 v;
    asm("mov.b64 %0, {%1, %2};" : "=l"(v.r) : "f"(a), "f"(b));
    return v;
}
__device__ __forceinline__ F2 bc(float a) { return pk(a, a); }
__device__ __forceinline__ float2 upk(F2 v) {
    float2 o;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(o.x), "=f"(o.y) : "l"(v.r));
    return o;
}
__device__ __forceinline__ F2 operator+(F2 a, F2 b) {
    F2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d.r) : "l"(a.r), "l"(b.r));
    return d;
}
__device__ __forceinline__ F2 operator-(F2 a, F2 b) {
    F2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.r) : "l"(a.r), "l"(b.r));
    return d;
}
__device__ __forceinline__ F2 operator*(F2 a, F2 b) {
    F2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d.r) : "l"(a.r), "l"(b.r));
    return d;
}
// a * b + c, one rounding
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
    F2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.r) : "l"(a.r), "l"(b.r), "l"(c.r));
    return d;
}

// c_k . (a, b, c) for k >= 10 (first non-zero component of c_k is +1)
template <int K>
__device__ __forceinline__ F2 cdotk(F2 a, F2 b, F2 c) {
    constexpr int X = cx(K), Y = cy(K), Z = cz(K);
    static_assert(X > 0 || (X == 0 && (Y > 0 || (Y == 0 && Z > 0))), "direction with a negative lead");
    if constexpr (X != 0) {
        if constexpr (Y != 0) return Y > 0 ? a + b : a - b;
        else if constexpr (Z != 0) return Z > 0 ? a + c : a - c;
        else return a;
    } else if constexpr (Y != 0) {
        if constexpr (Z != 0) return Z > 0 ? b + c : b - c;
        else return b;
    } else {
        return c;
    }
}
// the same with uniform scalars
template <int K>
__device__ __forceinline__ float cdotk_s(float a, float b, float c) {
    return (float)cx(K) * a + (float)cy(K) * b + (float)cz(K) * c;
}

struct Mom2 {
    F2 rhoBar, jx, jy, jz, invRho;
};

__device__ __forceinline__ Mom2 moments2(const F2 (&f)[Q]) {
    Mom2 m;
    m.rhoBar = ((f[0] + (f[1] + f[10])) + ((f[2] + f[11]) + (f[3] + f[12]))) +
               (((f[4] + f[13]) + (f[5] + f[14])) + ((f[6] + f[15]) + (f[7] + f[16]))) +
               ((f[8] + f[17]) + (f[9] + f[18]));
    m.jx = ((f[10] + f[13]) + (f[14] + f[15]) + f[16]) - ((f[1] + f[4]) + (f[5] + f[6]) + f[7]);
    m.jy = ((f[11] + f[13]) + (f[17] + f[18]) + f[5]) - ((f[2] + f[4]) + (f[8] + f[9]) + f[14]);
    m.jz = ((f[12] + f[15]) + (f[17] + f[7]) + f[9]) - ((f[3] + f[6]) + (f[8] + f[16]) + f[18]);
    const float2 rb = upk(m.rhoBar);
    m.invRho = pk(__frcp_rn(1.f + rb.x), __frcp_rn(1.f + rb.y));
    return m;
}

template <bool FORCE>
__device__ __forceinline__ void bgk2(F2 (&f)[Q], const Mom2& m, float omega, float gx, float gy, float gz) {
    const F2 one = bc(1.f);
    const F2 rho = one + m.rhoBar, invRho = m.invRho;
    F2 jx = m.jx, jy = m.jy, jz = m.jz;
    if (FORCE) {
        const F2 h = bc(0.5f) * rho;
        jx = fma2(h, bc(gx), jx); jy = fma2(h, bc(gy), jy); jz = fma2(h, bc(gz), jz);
    }
    const F2 jSqr = fma2(jz, jz, fma2(jy, jy, jx * jx));
    const F2 base = fma2(bc(-1.5f) * invRho, jSqr, m.rhoBar);
    const F2 om1 = bc(1.f - omega);
    const F2 q45 = bc(4.5f) * invRho;
    F2 ux{}, uy{}, uz{}, pre{}, ug{};
    if (FORCE) {
        ux = jx * invRho; uy = jy * invRho; uz = jz * invRho;
        pre = bc(1.f - 0.5f * omega) * rho;
        ug = fma2(uz, bc(gz), fma2(uy, bc(gy), ux * bc(gx)));
    }
    f[0] = fma2(om1, f[0], bc(omega * (float)wt(0)) * base);
    if (FORCE) f[0] = f[0] - bc(3.f * (float)wt(0)) * (pre * ug);
    auto pair = [&](auto kc) {
        constexpr int k = decltype(kc)::value, i = k - 9;
        const F2 cj = cdotk<k>(jx, jy, jz);          // c_k . j = -c_i . j
        const F2 ow = bc(omega * (float)wt(k));
        const F2 e = fma2(q45 * cj, cj, base);
        const F2 s = bc(3.f) * cj;
        f[i] = fma2(om1, f[i], ow * (e - s));
        f[k] = fma2(om1, f[k], ow * (e + s));
        if (FORCE) {
            const F2 cu = cdotk<k>(ux, uy, uz);
            const float cg = cdotk_s<k>(gx, gy, gz);
            const F2 tp = bc((float)wt(k)) * pre;
            const F2 X = fma2(bc(9.f * cg), cu, bc(-3.f) * ug);
            f[i] = fma2(tp, X - bc(3.f * cg), f[i]);
            f[k] = fma2(tp, X + bc(3.f * cg), f[k]);
        }
    };
    pair(std::integral_constant<int, 10>{}); pair(std::integral_constant<int, 11>{});
    pair(std::integral_constant<int, 12>{}); pair(std::integral_constant<int, 13>{});
    pair(std::integral_constant<int, 14>{}); pair(std::integral_constant<int, 15>{});
    pair(std::integral_constant<int, 16>{}); pair(std::integral_constant<int, 17>{});
    pair(std::integral_constant<int, 18>{});
}

// Solid correction of both cells (a no-op for a cell with B = 0), with the
// momentum exchange accumulated in (Fx, Fy, Fz); pre(i) returns the pair's fPre_i.
template <typename Pre>
__device__ __forceinline__ void psm2(F2 (&f)[Q], F2 rhoBar, F2 jx, F2 jy, F2 jz, F2 invRho, F2 up0, F2 up1, F2 up2,
                                     F2 B, const Pre& pre, F2& Fx, F2& Fy, F2& Fz) {
    const F2 rho = bc(1.f) + rhoBar;
    const F2 ux = up0 * rho, uy = up1 * rho, uz = up2 * rho;
    const F2 q45 = bc(4.5f) * invRho;
    const F2 dB = (bc(-1.5f) * invRho) * (fma2(uz, uz, fma2(uy, uy, ux * ux)) - fma2(jz, jz, fma2(jy, jy, jx * jx)));
    {
        const F2 p0 = pre(0);
        f[0] = fma2(B, (p0 - f[0]) - bc((float)wt(0)) * dB, f[0]);
    }
    const F2 B2 = B + B;
    Fx = bc(0.f); Fy = bc(0.f); Fz = bc(0.f);
    auto pair = [&](auto kc) {
        constexpr int k = decltype(kc)::value, i = k - 9;
        const F2 t = bc((float)wt(k));
        const F2 cj = cdotk<k>(jx, jy, jz);
        const F2 cu = cdotk<k>(ux, uy, uz);
        const F2 A = t * fma2(q45, (cu - cj) * (cu + cj), dB);
        const F2 Sk = bc(3.f * (float)wt(k)) * (cj + cu);
        const F2 pi = pre(i), pkk = pre(k);
        const F2 E = (pkk - pi) - Sk;
        f[i] = fma2(B, (pi - f[i]) + (A + E), f[i]);
        f[k] = fma2(B, (pkk - f[k]) + (A - E), f[k]);
        const F2 d = B2 * E;                          // F += c_k (bb - bbOpp)
        if constexpr (cx(k) > 0) Fx = Fx + d;
        if constexpr (cy(k) > 0) Fy = Fy + d; else if constexpr (cy(k) < 0) Fy = Fy - d;
        if constexpr (cz(k) > 0) Fz = Fz + d; else if constexpr (cz(k) < 0) Fz = Fz - d;
    };
    pair(std::integral_constant<int, 10>{}); pair(std::integral_constant<int, 11>{});
    pair(std::integral_constant<int, 12>{}); pair(std::integral_constant<int, 13>{});
    pair(std::integral_constant<int, 14>{}); pair(std::integral_constant<int, 15>{});
    pair(std::integral_constant<int, 16>{}); pair(std::integral_constant<int, 17>{});
    pair(std::integral_constant<int, 18>{});
}

// bgk2 followed by psm2 in one pass over the opposite pairs (the same operations
// in the same order, so the same bits): the pre-collision pair is still in
// registers when its correction is applied, so fPre is not re-read.  Used with a
// body force for unaligned rows (batch); aligned rows keep the two passes, which
// measured faster there (without a body force both take collide_g2).  Per pair
// k = i + 9 (c_k = -c_i), with the solid
// equilibrium at P = (1 + rhoBar) uPart and fb the BGK result:
//   A = t (dB + 4.5 invRho ((c_k.P)^2 - (c_k.j)^2)),  S = 3 t c_k.(j + P),
//   E = (fPre_k - fPre_i) - S,
//   f_i = fb_i + B ((fPre_i - fb_i) + (A + E)),  f_k = fb_k + B ((fPre_k - fb_k) + (A - E)),
//   F += c_k 2 B E      (src/ibCompositeDynamics3D.hh:150-200, regrouped).  hs = (n < 125) rho
// per cell (FORCE: the solid correction's momentum j + hs g).  A cell with B = 0
// comes out exactly as bgk2 leaves it.
template <bool FORCE>
__device__ __forceinline__ void bgk_psm2(F2 (&f)[Q], const Mom2& m, float omega, float gx, float gy, float gz, F2 hs,
                                         F2 up0, F2 up1, F2 up2, F2 B, F2& Fx, F2& Fy, F2& Fz) {
    const F2 one = bc(1.f);
    const F2 rho = one + m.rhoBar, invRho = m.invRho;
    // BGK constants (bgk2)
    F2 jx = m.jx, jy = m.jy, jz = m.jz;
    if (FORCE) {
        const F2 h = bc(0.5f) * rho;
        jx = fma2(h, bc(gx), jx); jy = fma2(h, bc(gy), jy); jz = fma2(h, bc(gz), jz);
    }
    const F2 jSqr = fma2(jz, jz, fma2(jy, jy, jx * jx));
    const F2 base = fma2(bc(-1.5f) * invRho, jSqr, m.rhoBar);
    const F2 om1 = bc(1.f - omega);
    const F2 q45 = bc(4.5f) * invRho;
    F2 ux{}, uy{}, uz{}, pre{}, ug{};
    if (FORCE) {
        ux = jx * invRho; uy = jy * invRho; uz = jz * invRho;
        pre = bc(1.f - 0.5f * omega) * rho;
        ug = fma2(uz, bc(gz), fma2(uy, bc(gy), ux * bc(gx)));
    }
    // solid-correction constants
    F2 sjx = m.jx, sjy = m.jy, sjz = m.jz;
    if (FORCE) {
        sjx = fma2(hs, bc(gx), sjx); sjy = fma2(hs, bc(gy), sjy); sjz = fma2(hs, bc(gz), sjz);
    }
    const F2 rhoS = bc(1.f) + m.rhoBar;
    const F2 px = up0 * rhoS, py = up1 * rhoS, pz = up2 * rhoS;
    const F2 q45S = bc(4.5f) * invRho;
    const F2 dB = (bc(-1.5f) * invRho) * (fma2(pz, pz, fma2(py, py, px * px)) - fma2(sjz, sjz, fma2(sjy, sjy, sjx * sjx)));
    {
        const F2 p0 = f[0];
        F2 b0 = fma2(om1, f[0], bc(omega * (float)wt(0)) * base);
        if (FORCE) b0 = b0 - bc(3.f * (float)wt(0)) * (pre * ug);
        f[0] = fma2(B, (p0 - b0) - bc((float)wt(0)) * dB, b0);
    }
    const F2 B2 = B + B;
    Fx = bc(0.f); Fy = bc(0.f); Fz = bc(0.f);
    auto pair = [&](auto kc) {
        constexpr int k = decltype(kc)::value, i = k - 9;
        const F2 pi = f[i], pkk = f[k];
        // BGK of the pair
        const F2 cj = cdotk<k>(jx, jy, jz);
        const F2 ow = bc(omega * (float)wt(k));
        const F2 e = fma2(q45 * cj, cj, base);
        const F2 s = bc(3.f) * cj;
        F2 bi = fma2(om1, pi, ow * (e - s));
        F2 bk = fma2(om1, pkk, ow * (e + s));
        if (FORCE) {
            const F2 cu = cdotk<k>(ux, uy, uz);
            const float cg = cdotk_s<k>(gx, gy, gz);
            const F2 tp = bc((float)wt(k)) * pre;
            const F2 X = fma2(bc(9.f * cg), cu, bc(-3.f) * ug);
            bi = fma2(tp, X - bc(3.f * cg), bi);
            bk = fma2(tp, X + bc(3.f * cg), bk);
        }
        // solid correction of the pair
        const F2 t = bc((float)wt(k));
        const F2 cjS = cdotk<k>(sjx, sjy, sjz);
        const F2 cu = cdotk<k>(px, py, pz);
        const F2 A = t * fma2(q45S, (cu - cjS) * (cu + cjS), dB);
        const F2 Sk = bc(3.f * (float)wt(k)) * (cjS + cu);
        const F2 E = (pkk - pi) - Sk;
        f[i] = fma2(B, (pi - bi) + (A + E), bi);
        f[k] = fma2(B, (pkk - bk) + (A - E), bk);
        const F2 d = B2 * E;
        if constexpr (cx(k) > 0) Fx = Fx + d;
        if constexpr (cy(k) > 0) Fy = Fy + d; else if constexpr (cy(k) < 0) Fy = Fy - d;
        if constexpr (cz(k) > 0) Fz = Fz + d; else if constexpr (cz(k) < 0) Fz = Fz - d;
    };
    pair(std::integral_constant<int, 10>{}); pair(std::integral_constant<int, 11>{});
    pair(std::integral_constant<int, 12>{}); pair(std::integral_constant<int, 13>{});
    pair(std::integral_constant<int, 14>{}); pair(std::integral_constant<int, 15>{});
    pair(std::integral_constant<int, 16>{}); pair(std::integral_constant<int, 17>{});
    pair(std::integral_constant<int, 18>{});
}

// FP32 form without a body force: BGK and the solid correction of both cells
// in one pass, the formulation of collide_cell_fp64 in packed pairs (around
// g = fPre - feq; alpha = omega (1 - B) + B; see there).  fPre is f itself on
// entry, so nothing is re-read from the stage.  SOLID false (no solid cell in
// the warp) leaves out the solid terms; a fluid cell (B = 0, uP = 0) gets the
// same bits either way.
template <bool SOLID>
__device__ __forceinline__ void collide_g2(F2 (&f)[Q], const Mom2& m, float omega, F2 up0, F2 up1, F2 up2, F2 B,
                                           F2& Fx, F2& Fy, F2& Fz) {
    const F2 invRho = m.invRho;
    const F2 jSqr = fma2(m.jz, m.jz, fma2(m.jy, m.jy, m.jx * m.jx));
    const F2 m15 = bc(-1.5f) * invRho;
    const F2 base = fma2(m15, jSqr, m.rhoBar);
    const F2 nom = bc(-omega);
    F2 Px = bc(0.f), Py = bc(0.f), Pz = bc(0.f), dd = bc(0.f), nalpha = nom, nom1B = nom;
    if (SOLID) {
        const F2 rho = bc(1.f) + m.rhoBar;
        Px = up0 * rho; Py = up1 * rho; Pz = up2 * rho;
        const F2 PSqr = fma2(Pz, Pz, fma2(Py, Py, Px * Px));
        dd = m15 * (jSqr - PSqr);
        nalpha = fma2(B, bc(omega - 1.f), nom);     // -(omega (1 - B) + B)
        nom1B = fma2(B, bc(omega), nom);            // -omega (1 - B)
    }
    {
        const F2 g0 = f[0] - bc((float)wt(0)) * base;
        f[0] = SOLID ? fma2(B, bc((float)wt(0)) * dd, fma2(nom1B, g0, f[0])) : fma2(nom, g0, f[0]);
    }
    F2 Ex = bc(0.f), Ey = bc(0.f), Ez = bc(0.f);
    auto pair = [&](auto kc) {
        constexpr int k = decltype(kc)::value, i = k - 9;
        const F2 t = bc((float)wt(k)), t3 = bc(3.f * (float)wt(k));
        const F2 a45 = bc(4.5f * (float)wt(k)) * invRho;
        const F2 cj = cdotk<k>(m.jx, m.jy, m.jz);
        const F2 C = fma2(a45 * cj, cj, t * base);
        const F2 Lj = t3 * cj;
        const F2 gi = (f[i] - C) + Lj;
        const F2 gk = (f[k] - C) - Lj;
        if (SOLID) {
            const F2 cP = cdotk<k>(Px, Py, Pz);
            const F2 mm = cj - cP, pp = cj + cP;
            const F2 Qd = fma2(a45 * mm, pp, t * dd);
            const F2 L = t3 * mm;
            const F2 e = (f[k] - f[i]) - t3 * pp;
            f[i] = fma2(B, (gk - Qd) + L, fma2(nalpha, gi, f[i]));
            f[k] = fma2(B, (gi - Qd) - L, fma2(nalpha, gk, f[k]));
            if constexpr (cx(k) > 0) Ex = Ex + e;
            if constexpr (cy(k) > 0) Ey = Ey + e; else if constexpr (cy(k) < 0) Ey = Ey - e;
            if constexpr (cz(k) > 0) Ez = Ez + e; else if constexpr (cz(k) < 0) Ez = Ez - e;
        } else {
            f[i] = fma2(nom, gi, f[i]);
            f[k] = fma2(nom, gk, f[k]);
        }
    };
    pair(std::integral_constant<int, 10>{}); pair(std::integral_constant<int, 11>{});
    pair(std::integral_constant<int, 12>{}); pair(std::integral_constant<int, 13>{});
    pair(std::integral_constant<int, 14>{}); pair(std::integral_constant<int, 15>{});
    pair(std::integral_constant<int, 16>{}); pair(std::integral_constant<int, 17>{});
    pair(std::integral_constant<int, 18>{});
    const F2 B2 = B + B;
    Fx = B2 * Ex; Fy = B2 * Ey; Fz = B2 * Ez;
}

// float -> double by bit manipulation (exact for normal numbers; subnormal
// floats become signed zero).  Keeps the conversion off GB300's narrow FP64 pipe.
__device__ __forceinline__ double widen(float x) {
    const uint32_t b = __float_as_uint(x);
    const uint32_t s = b & 0x80000000u, e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
    if (e == 0) return __hiloint2double((int)s, 0);
    const uint32_t ed = e == 0xffu ? 0x7ffu : e + 896u;   // rebias 127 -> 1023
    return __hiloint2double((int)(s | (ed << 20) | (m >> 3)), (int)(m << 29));
}
__device__ __forceinline__ double widen(double x) { return x; }

// Per-cell force and torque of a solid cell (SumForceTorque3D,
// src/ibProcessors3D.hh:203-263): particle slot of the owner tag and the
// terms F, r x F with the minimum-image arm of :230-243.  Returns the slot or -1.
// The terms F and r x F of a cell with arm (dx, dy, dz) before the minimum image
// (integer half extents of g, src/ibProcessors3D.hh:230-243).
template <typename T>
__device__ __forceinline__ void arm_terms(T dx, T dy, T dz, const Geom& g, T Fx, T Fy, T Fz, T (&v)[6]) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int hx = nx / 2, hy = ny / 2, hz = nz / 2;
    if (dx > T(hx)) dx -= T(nx); else if (dx < T(-hx)) dx += T(nx);
    if (dy > T(hy)) dy -= T(ny); else if (dy < T(-hy)) dy += T(ny);
    if (dz > T(hz)) dz -= T(nz); else if (dz < T(-hz)) dz += T(nz);
    v[0] = Fx; v[1] = Fy; v[2] = Fz;
    v[3] = dy * Fz - dz * Fy;
    v[4] = -dx * Fz + dz * Fx;
    v[5] = dx * Fy - dy * Fx;
}

template <typename T>
__device__ __forceinline__ int cell_force_terms(const CollideArgs<T>& a, uint32_t w, int x, int y, int z, T Fx,
                                                T Fy, T Fz, T (&v)[6]) {
    if ((w & VOX_NMASK) == 0) return -1;
    const int tag = (int)(w >> VOX_NBITS);
    const int slot = tag <= a.max_tag ? __ldg(a.tag2slot + tag) : -1;
    if (slot < 0 || slot >= a.nslot) {
        atomicOr(a.err, 0x8u);   // LBDEM_DEVERR_UNMAPPED_TAG
        return -1;
    }
    T dx, dy, dz;
    if (sizeof(T) == 8) {
        const double* p = a.rec + (size_t)slot * REC_STRIDE;
        dx = T((double)x - __ldg(p + 0));
        dy = T((double)y - __ldg(p + 1));
        dz = T((double)z - __ldg(p + 2));
    } else {
        // centre = hi + lo in float: (x - hi) - lo is the arm to ~1 ulp
        const float4* p = reinterpret_cast<const float4*>(a.xpf + (size_t)slot * XPF_STRIDE);
        const float4 h = __ldg(p), l = __ldg(p + 1);
        dx = T(((float)x - h.x) - h.w);
        dy = T(((float)y - h.y) - l.x);
        dz = T(((float)z - h.z) - l.y);
    }
    arm_terms(dx, dy, dz, a.g, Fx, Fy, Fz, v);
    return slot;
}

// Warp-segmented sum over runs of equal particle slot (consecutive cells along
// z mostly belong to the same sphere), one set of double atomics per run.
// Must be reached by all 32 lanes.
template <typename T>
__device__ __forceinline__ void reduce_forces(const CollideArgs<T>& a, int key, T (&v)[6]) {
    const unsigned solid = __ballot_sync(FULL, key >= 0);
    if (solid == 0u) return;
    const int lane = threadIdx.x & 31;
    const int first = __shfl_sync(FULL, key, __ffs(solid) - 1);
    if (__all_sync(FULL, key < 0 || key == first)) {
        // one particle in the group: butterfly sum, lane 0 adds
#pragma unroll
        for (int d = 16; d > 0; d >>= 1)
#pragma unroll
            for (int k = 0; k < 6; ++k) v[k] += __shfl_xor_sync(FULL, v[k], d);
        if (lane == 0) {
            double* Fp = a.ft + 3 * (size_t)first;
            double* Tp = a.ft + 3 * (size_t)a.nslot + 3 * (size_t)first;
            atomicAdd(Fp + 0, widen(v[0])); atomicAdd(Fp + 1, widen(v[1])); atomicAdd(Fp + 2, widen(v[2]));
            atomicAdd(Tp + 0, widen(v[3])); atomicAdd(Tp + 1, widen(v[4])); atomicAdd(Tp + 2, widen(v[5]));
        }
        return;
    }
    const int prevKey = __shfl_up_sync(FULL, key, 1);
    const bool head = (lane == 0) || (prevKey != key);
    const unsigned heads = __ballot_sync(FULL, head);
    const int segStart = 31 - __clz(heads & (FULL >> (31 - lane)));
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const T o = __shfl_up_sync(FULL, v[k], d);
            if (lane - d >= segStart) v[k] += o;
        }
    }
    const int nextKey = __shfl_down_sync(FULL, key, 1);
    const bool tail = (lane == 31) || (nextKey != key);
    if (tail && key >= 0) {
        double* Fp = a.ft + 3 * (size_t)key;
        double* Tp = a.ft + 3 * (size_t)a.nslot + 3 * (size_t)key;
        atomicAdd(Fp + 0, widen(v[0])); atomicAdd(Fp + 1, widen(v[1])); atomicAdd(Fp + 2, widen(v[2]));
        atomicAdd(Tp + 0, widen(v[3])); atomicAdd(Tp + 1, widen(v[4])); atomicAdd(Tp + 2, widen(v[5]));
    }
}

// FP32 form: force and torque of the cells of one row segment, reduced per run
// of equal owner (keyed by the owner's particle slot, which the cells' surface
// velocity already looked up).  Every cell of a
// particle lies within its radius of the particle's nearest image, so along a
// row the minimum-image arm of cell z is arm(zc) + (z - zc) e_z for any point
// zc of the segment, and
//   sum_cells arm x F = arm(zc) x sum F + sum (z - zc) e_z x F,
// with e_z x F = (-F_y, F_x, 0).  Per cell the kernel accumulates
// v = (F, -(z - zc) F_y, (z - zc) F_x); the lane that ends a run (the last
// lane of a run of equal slots, or the first solid lane when one slot covers the
// warp) takes the arm of its own cell zr from the particle's row,
// arm(zc) = arm(zr) - (zr - zc) e_z, and adds F and arm(zc) x F + (v3, v4, 0).
__device__ __forceinline__ void finish_run(const CollideArgs<float>& a, int slot, const float (&v)[5], int sx, int sy,
                                           int zr, int zc, const float4& rh, float rl0, float rl1, bool have) {
    // the lane's own table row when it is the run's owner's (loaded for the velocity)
    float4 h = rh, l = make_float4(rl0, rl1, 0.f, 0.f);
    if (!have) {
        const float4* p = reinterpret_cast<const float4*>(a.xpf + (size_t)slot * XPF_STRIDE);
        h = __ldg(p);
        l = __ldg(p + 1);
    }
    float dx = ((float)sx - h.x) - h.w;
    float dy = ((float)sy - h.y) - l.x;
    float dz = ((float)zr - h.z) - l.y;
    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const int hx = nx / 2, hy = ny / 2, hz = nz / 2;
    if (dx > (float)hx) dx -= (float)nx; else if (dx < (float)-hx) dx += (float)nx;
    if (dy > (float)hy) dy -= (float)ny; else if (dy < (float)-hy) dy += (float)ny;
    if (dz > (float)hz) dz -= (float)nz; else if (dz < (float)-hz) dz += (float)nz;
    dz -= (float)(zr - zc);
    double* Fp = a.ft + 3 * (size_t)slot;
    double* Tp = a.ft + 3 * (size_t)a.nslot + 3 * (size_t)slot;
    // few lanes get here: the hardware conversion is cheaper than widen()
    atomicAdd(Fp + 0, (double)v[0]); atomicAdd(Fp + 1, (double)v[1]); atomicAdd(Fp + 2, (double)v[2]);
    atomicAdd(Tp + 0, (double)((dy * v[2] - dz * v[1]) + v[3]));
    atomicAdd(Tp + 1, (double)((dz * v[0] - dx * v[2]) + v[4]));
    atomicAdd(Tp + 2, (double)(dx * v[1] - dy * v[0]));
}

// Warp reduction of v over runs of equal key (owner slot, -1: no solid cell);
// zr is a cell of the lane's run.  Must be reached by all 32 lanes.
__device__ __forceinline__ void reduce_runs(const CollideArgs<float>& a, int key, float (&v)[5], int zr, int sx,
                                            int sy, int zc, const float4& rh, float rl0, float rl1, int rslot) {
    const unsigned solid = __ballot_sync(FULL, key >= 0);
    if (solid == 0u) return;
    const int lane = threadIdx.x & 31;
    const int lead = __ffs(solid) - 1;
    const int first = __shfl_sync(FULL, key, lead);
    if (__all_sync(FULL, key < 0 || key == first)) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1)
#pragma unroll
            for (int k = 0; k < 5; ++k) v[k] += __shfl_xor_sync(FULL, v[k], d);
        if (lane == lead) finish_run(a, first, v, sx, sy, zr, zc, rh, rl0, rl1, rslot == first);
        return;
    }
    const int prevKey = __shfl_up_sync(FULL, key, 1);
    const bool head = (lane == 0) || (prevKey != key);
    const unsigned heads = __ballot_sync(FULL, head);
    const int segStart = 31 - __clz(heads & (FULL >> (31 - lane)));
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const float o = __shfl_up_sync(FULL, v[k], d);
            if (lane - d >= segStart) v[k] += o;
        }
    }
    const int nextKey = __shfl_down_sync(FULL, key, 1);
    const bool tail = (lane == 31) || (nextKey != key);
    if (tail && key >= 0) finish_run(a, key, v, sx, sy, zr, zc, rh, rl0, rl1, rslot == key);
}

__device__ __forceinline__ int wrap_minus(int v, int n, int per) { return v > 0 ? v - 1 : (per ? n - 1 : -1); }
__device__ __forceinline__ int wrap_plus(int v, int n, int per) { return v < n - 1 ? v + 1 : (per ? 0 : -1); }
__device__ __forceinline__ int pick(int c, int m, int v, int p) { return c < 0 ? m : (c > 0 ? p : v); }

// ---------------------------------------------------------------------------
// Staged persistent kernel: every warp runs its own double-buffered pipeline
// over SEGW-cell z-segments (no block-wide barriers, so a warp with solid
// cells does not hold up the others).
constexpr int WARPS = COLLIDE_BLOCK / 32;    // warps per CTA
// Per-CTA tables in dynamic shared memory behind the warps' stages.
// FP32 form, single lattice: a copy of the tag -> slot map when the tags fit below
// TAGMAP_SMEM - 1, holding -1 for a tag with no particle in the list and for every entry
// past max_tag (the last one included), so that a lookup is one shared load at
// min(tag, TAGMAP_SMEM - 1) with no tests between the cell's voxel word and the owner's
// table row; then B(n) (128 floats).
constexpr int TAGMAP_SMEM = 2048;
template <typename T, bool BATCH>
__host__ __device__ constexpr bool smem_tagmap() { return sizeof(T) == 4 && !BATCH; }
template <typename T, bool BATCH>
__host__ __device__ constexpr size_t tagmap_bytes() {
    return smem_tagmap<T, BATCH>() ? sizeof(int) * TAGMAP_SMEM + sizeof(float) * 128 : 0;
}
// Batch mode: each CTA keeps the first segment of every domain in shared memory when
// there are at most SEG0_SMEM domains (the per-segment domain search reads it there).
constexpr int SEG0_SMEM = 2048;
template <bool BATCH>
__host__ __device__ constexpr size_t seg0_bytes() { return BATCH ? sizeof(int) * SEG0_SMEM : 0; }
constexpr int SEGW = COLLIDE_SEGW;          // cells per warp segment (2 per lane)
constexpr int WAIT_LIMIT = 1 << 22;         // bounded mbarrier wait (iterations of try_wait)
constexpr int PROBE_WAIT = 64;              // the timeout test hook's wait (iterations)

// Surface-velocity rows are staged by the FP64 form of a single lattice only.
template <typename T, bool BATCH>
__host__ __device__ constexpr bool stage_up() { return !BATCH && sizeof(T) == 8; }

// 16-byte aligned, so that every warp's stage (at warp * sizeof) keeps the bulk
// copies' shared-memory destinations on 16-byte boundaries.
template <typename T, bool STAGE_UP = true>
struct alignas(16) WarpStage {
    static constexpr int V = 16 / (int)sizeof(T);   // elements per 16 bytes
    static constexpr int UW = STAGE_UP ? SEGW + V : 1;
    static constexpr int W = SEGW + 2 * V;          // row: V halo | (lead) SEGW core | V halo
    T f[2][Q][W];
    uint32_t vox[2][SEGW + 4];
    T up[2][3][UW];        // particle surface velocity rows of the segment (when staged)
    long long row[2][9];   // element offset of row (x + dx, y + dy) at [3 (dx + 1) + dy + 1]; -1 beyond a wall
    int geo[2][8];         // x, y, z0, len, domain of the segment held in buffer b
    unsigned long long lead[2];   // unaligned rows: lead elements of row i at bits 2i, voxel row at bits 38,
                                  // surface-velocity row d at bits 40 + 2d
    unsigned long long bar[2];
};

static_assert(sizeof(WarpStage<float, true>) % 16 == 0 && sizeof(WarpStage<float, false>) % 16 == 0 &&
                  sizeof(WarpStage<double, true>) % 16 == 0 && sizeof(WarpStage<double, false>) % 16 == 0,
              "per-warp stages must keep 16-byte alignment");
static_assert(offsetof(WarpStage<float>, vox) % 16 == 0 && offsetof(WarpStage<float>, up) % 16 == 0 &&
                  offsetof(WarpStage<double>, vox) % 16 == 0 && offsetof(WarpStage<double>, up) % 16 == 0,
              "bulk-copy destinations on 16-byte boundaries");

// The per-CTA tables behind the warps' stages.
template <typename T, bool STAGE_UP>
__device__ __forceinline__ unsigned char* cta_tables() {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    return smem_raw + WARPS * sizeof(WarpStage<T, STAGE_UP>);
}

__device__ __forceinline__ constexpr int row_slot(int dx, int dy) { return 3 * (dx + 1) + dy + 1; }

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false if the phase did not complete within `limit` tries.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity, int limit = WAIT_LIMIT) {
    for (int k = 0; k < limit; ++k)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// Global -> shared bulk copy completing on an mbarrier (16-byte aligned, size % 16 == 0).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Directions with c_z != 0 (they need a halo element in the odd phase).
__device__ __forceinline__ int zdir(int k) {
    // {3, 6, 7, 8, 9, 12, 15, 16, 17, 18} packed in 5-bit fields
    constexpr unsigned long long D = 3ull | 6ull << 5 | 7ull << 10 | 8ull << 15 | 9ull << 20 | 12ull << 25 |
                                     15ull << 30 | 16ull << 35 | 17ull << 40 | 18ull << 45;
    return (int)((D >> (5 * k)) & 31u);
}

struct SegGeo {
    int x, y, z0, len;
    int xm, xp, ym, yp;     // neighbour rows along x and y (-1: beyond a wall)
};

// dz divides by the z-segments per row, dy by ny (CollideArgs::dz, dy).  PER: all
// axes periodic (known at compile time).
template <bool PER = false>
__device__ __forceinline__ SegGeo seg_geo(const Geom& g, long long seg, const DivMagic& dz, const DivMagic& dy) {
    SegGeo s;
    // 32-bit arithmetic: a lattice holds fewer than 2^31 segments (launch checks)
    const unsigned sg = (unsigned)seg;
    const unsigned row = fast_div(sg, dz);
    const int zs = (int)(sg - row * dz.d);
    s.x = (int)fast_div(row, dy);
    s.y = (int)(row - (unsigned)s.x * dy.d);
    s.z0 = zs * SEGW;
    s.len = min(SEGW, g.nz - s.z0);
    s.xm = wrap_minus(s.x, g.nx, PER ? 1 : g.per[0]); s.xp = wrap_plus(s.x, g.nx, PER ? 1 : g.per[0]);
    s.ym = wrap_minus(s.y, g.ny, PER ? 1 : g.per[1]); s.yp = wrap_plus(s.y, g.ny, PER ? 1 : g.per[1]);
    return s;
}

// Row (x + dx, y + dy) as an element offset, or -1 beyond a wall.
template <bool PER = false>
__device__ __forceinline__ long long row_off(const Geom& g, const SegGeo& s, int dx, int dy) {
    const int X = pick(dx, s.xm, s.x, s.xp), Y = pick(dy, s.ym, s.y, s.yp);
    if (!PER && (X < 0 || Y < 0)) return -1;
    return ((long long)X * g.ny + Y) * g.nz;
}

// Issued by one warp for its segment into buffer b:
//   lanes 0..18:  population rows (even: own row, slot i; odd: row x - c_i,
//                 slot opp i, or own row slot i when that row is beyond a wall);
//   lanes 19..28: odd phase, aligned rows: the 16-byte chunk holding the halo
//                 element of the (lane-19)-th c_z != 0 direction (none beyond a z wall);
//   lane 29:      voxel words of the segment;
//   lanes 29-31:  (second copy) the segment's particle surface-velocity rows.
// MIS (rows not 16-byte aligned, nz % 4 != 0): each row copy starts at the
// 16-byte boundary below the row and is rounded up to whole chunks (the
// allocations carry 64 bytes of tail padding); the lead of every row is
// published in st.lead.  The odd-phase halo elements are then read by lanes
// 0..9 with plain loads and returned, to be put in place once the copy has
// landed: the cell that reads and writes such a slot in this step lies in
// this segment, so no other warp touches it meanwhile.
// Lanes 0..9 also publish the segment geometry for the compute pass.
template <typename T, bool ODD, bool MIS, bool STAGE_UP>
__device__ __forceinline__ T issue_segment(const CollideArgs<T>& a, WarpStage<T, STAGE_UP>& st, int b, long long seg,
                                           int dom) {
    constexpr int V = WarpStage<T>::V;
    const int lane = threadIdx.x & 31;
    const Geom& g = a.g;
    const SegGeo s = seg_geo(g, seg, a.dz, a.dy);
    const size_t N = g.N;
    const long long own = ((long long)s.x * g.ny + s.y) * g.nz;
    if (lane < 9) st.row[b][lane] = row_off(g, s, lane / 3 - 1, lane % 3 - 1);

    if (lane == 9) {
        st.geo[b][0] = s.x; st.geo[b][1] = s.y; st.geo[b][2] = s.z0; st.geo[b][3] = s.len; st.geo[b][4] = dom;
    }
    const T* src = nullptr;
    void* dst = nullptr;
    uint32_t bytes = 0;
    uint32_t lead = 0;
    T halo = T(0);
    if (lane < Q) {
        const int i = lane;
        size_t off = (size_t)i * N + (size_t)own + s.z0;
        if (ODD && i != 0) {
            const long long r = row_off(g, s, -cx(i), -cy(i));
            if (r >= 0) off = (size_t)opp(i) * N + (size_t)r + s.z0;
        }
        src = a.f + off;
        dst = &st.f[b][i][V];
        if (MIS) {
            lead = (uint32_t)(((uintptr_t)src & 15u) / sizeof(T));
            src -= lead;
            bytes = (uint32_t)(((lead + (uint32_t)s.len + V - 1) / V) * 16u);
        } else {
            bytes = (uint32_t)(s.len * sizeof(T));
        }
    } else if (ODD && !MIS && lane < Q + 10) {
        const int i = zdir(lane - Q);
        const long long r = row_off(g, s, -cx(i), -cy(i));
        if (r >= 0) {
            int zc;      // first element of the 16-byte chunk (-1: beyond a z wall)
            if (cz(i) > 0) {
                zc = s.z0 - V;
                if (zc < 0) zc = g.per[2] ? zc + g.nz : -1;
                dst = &st.f[b][i][0];
            } else {
                zc = s.z0 + s.len;
                if (zc >= g.nz) zc = g.per[2] ? zc - g.nz : -1;
                dst = &st.f[b][i][V + s.len];
            }
            if (zc >= 0) {
                src = a.f + (size_t)opp(i) * N + (size_t)r + zc;
                bytes = 16;
            }
        }
    } else if (lane == Q + 10) {
        const uint32_t* vs = a.vox + own + s.z0;
        if (MIS) {
            lead = (uint32_t)(((uintptr_t)vs & 15u) / 4u);
            vs -= lead;
            bytes = ((lead + (uint32_t)s.len + 3u) / 4u) * 16u;
        } else {
            bytes = (uint32_t)(s.len * sizeof(uint32_t));
        }
        src = reinterpret_cast<const T*>(vs);
        dst = &st.vox[b][0];
    }
    // lanes 29, 30, 31: the surface-velocity rows (components 2, 0, 1) as a second copy
    const T* src2 = nullptr;
    void* dst2 = nullptr;
    uint32_t bytes2 = 0, lead2 = 0;
    const int ud = lane == Q + 10 ? 2 : lane - (Q + 11);
    if (STAGE_UP && lane >= Q + 10) {
        src2 = a.up + (size_t)ud * N + own + s.z0;
        dst2 = &st.up[b][ud][0];
        if (MIS) {
            lead2 = (uint32_t)(((uintptr_t)src2 & 15u) / sizeof(T));
            src2 -= lead2;
            bytes2 = (uint32_t)(((lead2 + (uint32_t)s.len + V - 1) / V) * 16u);
        } else {
            bytes2 = (uint32_t)(s.len * sizeof(T));
        }
    }
    if (MIS) {
        const uint32_t lo = __reduce_or_sync(FULL, lane < 16 ? lead << (2 * lane) : 0u);
        const uint32_t hi = __reduce_or_sync(
            FULL, ((lane >= 16 && lane < Q) ? lead << (2 * (lane - 16)) : (lane == Q + 10 ? lead << 6 : 0u)) |
                      ((STAGE_UP && lane >= Q + 10) ? lead2 << (8 + 2 * ud) : 0u));
        if (lane == 0) st.lead[b] = (unsigned long long)lo | ((unsigned long long)hi << 32);
        if (ODD && lane < 10) {
            const int i = zdir(lane);
            const long long r = row_off(g, s, -cx(i), -cy(i));
            if (r >= 0) {
                if (cz(i) > 0) {
                    const int zs = s.z0 > 0 ? s.z0 - 1 : (g.per[2] ? g.nz - 1 : -1);
                    halo = zs >= 0 ? a.f[(size_t)opp(i) * N + (size_t)r + zs] : a.f[(size_t)i * N + (size_t)own];
                } else {
                    const int ze = s.z0 + s.len;
                    const int zs = ze < g.nz ? ze : (g.per[2] ? 0 : -1);
                    halo = zs >= 0 ? a.f[(size_t)opp(i) * N + (size_t)r + zs]
                                   : a.f[(size_t)i * N + (size_t)own + g.nz - 1];
                }
            }
        }
    }
    const uint32_t total = __reduce_add_sync(FULL, bytes + bytes2);
    if (lane == 0) mbar_arrive_expect_tx(&st.bar[b], total);
    __syncwarp();
    if (bytes) bulk_g2s(dst, src, bytes, &st.bar[b]);
    if (bytes2) bulk_g2s(dst2, src2, bytes2, &st.bar[b]);
    return halo;
}

// ---------------------------------------------------------------------------
// Staging of aligned rows (nz % 4 == 0) with per-thread 16-byte cp.async
// through the load/store path: a segment's rows go out as many small copies
// (19 population rows, the voxel row, the surface-velocity rows and up to 10
// halo chunks), and bulk copies of that size are bounded by the per-operation
// rate of the bulk-copy unit rather than by DRAM.  Completion is tracked per
// thread with commit groups (one group per segment).
__device__ __forceinline__ void cp16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int P>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(P) : "memory");
}

template <typename Fn, int... Ts>
__device__ __forceinline__ void unroll_seq(std::integer_sequence<int, Ts...>, Fn&& fn) {
    (fn(std::integral_constant<int, Ts>{}), ...);
}

// Element offset of the source row of direction I (even: slot I of the own row;
// odd: slot opp I of row x - c_I, or slot I of the own row beyond a wall).
// PER: every axis periodic, the row x - c_I always exists.
template <bool ODD, bool PER, int I>
__device__ __forceinline__ size_t src_row(const long long* row, size_t N, size_t own) {
    if constexpr (!ODD || I == 0) {
        return (size_t)I * N + own;
    } else {
        const long long r = row[row_slot(-cx(I), -cy(I))];
        if constexpr (PER) return (size_t)opp(I) * N + (size_t)r;
        else return r >= 0 ? (size_t)opp(I) * N + (size_t)r : (size_t)I * N + own;
    }
}

template <typename T, bool ODD, bool PER, bool STAGE_UP>
__device__ __forceinline__ void issue_segment_lsu(const CollideArgs<T>& a, WarpStage<T, STAGE_UP>& st, int b,
                                                  long long seg) {
    constexpr int V = WarpStage<T>::V;   // elements per 16-byte chunk
    constexpr int CPR = SEGW / V;        // chunks per row of a segment
    constexpr int RPI = 32 / CPR;        // rows per warp pass
    static_assert(CPR * RPI == 32, "a warp pass covers whole rows");
    const int lane = threadIdx.x & 31;
    const Geom& g = a.g;
    const SegGeo s = seg_geo<PER>(g, seg, a.dz, a.dy);
    const size_t N = g.N;
    const size_t own = ((size_t)s.x * g.ny + s.y) * g.nz;
    if (lane < 9) st.row[b][lane] = row_off<PER>(g, s, lane / 3 - 1, lane % 3 - 1);
    if (lane == 9) {
        st.geo[b][0] = s.x; st.geo[b][1] = s.y; st.geo[b][2] = s.z0; st.geo[b][3] = s.len; st.geo[b][4] = 0;
    }
    __syncwarp();
    const long long* row = st.row[b];
    const int c = lane % CPR, sub = lane / CPR;
    const bool cin = c * V < s.len;   // rows of aligned lattices end on a chunk boundary
    const T* f = a.f;
    // population rows: pass t covers directions t * RPI + sub
    unroll_seq(std::make_integer_sequence<int, (Q + RPI - 1) / RPI>{}, [&](auto tc) {
        constexpr int t = decltype(tc)::value;
        constexpr int i0 = t * RPI, i1 = t * RPI + 1;
        if constexpr (RPI == 1 || i1 >= Q) {
            if (sub == 0 && cin) cp16(&st.f[b][i0][V + c * V], f + src_row<ODD, PER, i0>(row, N, own) + s.z0 + c * V);
        } else {
            size_t off;
            if constexpr (ODD && PER && i0 != 0) {
                // one row lookup per pass: the lane's direction picks slot and array
                constexpr int s0 = row_slot(-cx(i0), -cy(i0)), s1 = row_slot(-cx(i1), -cy(i1));
                const long long r = row[sub == 0 ? s0 : s1];
                off = (size_t)(sub == 0 ? opp(i0) : opp(i1)) * N + (size_t)r;
            } else {
                off = sub == 0 ? src_row<ODD, PER, i0>(row, N, own) : src_row<ODD, PER, i1>(row, N, own);
            }
            if (cin) cp16(&st.f[b][sub == 0 ? i0 : i1][V + c * V], f + off + s.z0 + c * V);
        }
    });
    // then: voxel row (SEGW / 4 chunks), surface-velocity rows (3 CPR), halo chunks
    // (odd phase, 10) -- in that order, so that only the first pass mixes two kinds
    constexpr int NH = ODD ? 10 : 0, NV = SEGW / 4, NU = STAGE_UP ? 3 * CPR : 0;
    constexpr int NX = NH + NV + NU;
#pragma unroll
    for (int kk = lane; kk < ((NX + 31) / 32) * 32; kk += 32) {
        // item order voxel, velocity, halo, mapped onto the halo-first numbering below
        const int k = kk < NV + NU ? kk + NH : kk - (NV + NU);
        if (kk >= NX) continue;
        if (k < NH) {
            const int i = zdir(k);
            const long long r = row[row_slot(-cx(i), -cy(i))];
            if (!PER && r < 0) continue;
            int zc;     // first element of the chunk holding the halo (-1: beyond a z wall)
            T* dst;
            if (cz(i) > 0) {
                zc = s.z0 - V;
                if (zc < 0) zc = (PER || g.per[2]) ? zc + g.nz : -1;
                dst = &st.f[b][i][0];
            } else {
                zc = s.z0 + s.len;
                if (zc >= g.nz) zc = (PER || g.per[2]) ? zc - g.nz : -1;
                dst = &st.f[b][i][V + s.len];
            }
            if (zc >= 0) cp16(dst, f + (size_t)opp(i) * N + (size_t)r + zc);
        } else if (k < NH + NV) {
            const int cv = k - NH;
            if (cv * 4 < s.len) cp16(&st.vox[b][cv * 4], a.vox + own + s.z0 + cv * 4);
        } else if (k < NX) {
            const int u = k - NH - NV, d = u / CPR, cu = u % CPR;
            if (STAGE_UP && cu * V < s.len)
                cp16(&st.up[b][d][cu * V], a.up + (size_t)d * N + own + s.z0 + cu * V);
        }
    }
    cp_commit();
}

// Force and torque of a segment that is a whole z-periodic row (per-cell arms),
// kept out of line: the bench lattices never take it.
__device__ __noinline__ void whole_row_forces(const CollideArgs<float>& a, uint32_t w0, uint32_t w1, bool v0, bool v1,
                                              int sx, int sy, int za, int zb, float2 fx, float2 fy, float2 fz) {
    float va[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, vb[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const int ka = v0 ? cell_force_terms(a, w0, sx, sy, za, fx.x, fy.x, fz.x, va) : -1;
    const int kb = v1 ? cell_force_terms(a, w1, sx, sy, zb, fx.y, fy.y, fz.y, vb) : -1;
    if (__all_sync(FULL, ka < 0 || kb < 0 || ka == kb)) {
        const int key = ka >= 0 ? ka : kb;
#pragma unroll
        for (int q = 0; q < 6; ++q) va[q] += vb[q];
        reduce_forces(a, key, va);
    } else {
        reduce_forces(a, ka, va);
        reduce_forces(a, kb, vb);
    }
}

// FP32 compute pass over one staged segment, two cells per lane in packed
// pairs.  Aligned rows (!MIS): lane l takes the adjacent cells j = 2 l, 2 l + 1,
// whose staged values and destination slots are 8-byte aligned pairs, so loads
// and stores are 64-bit (in the odd phase the c_z != 0 directions land one slot
// over and are moved one lane over with a shuffle).  Unaligned rows (MIS): lane
// l takes j = l and l + 32 (32-bit accesses, conflict-free and coalesced).
// Force and torque are reduced per run of equal owner (reduce_runs); the two
// cells of a lane go through one warp reduction when their owners agree.
// FLAT (even phase of the FP32 batch): the segment is 64 cells of an x-plane
// taken in memory order across its z-rows (a.g is the plane view, see
// CollideArgs); a solid cell's true (y, z) is recovered from its index in the
// plane, and force and torque take per-cell arms (a run may cross rows).  The
// even phase touches only the cell's own slots, so a cell's populations do
// not depend on how the cells are grouped into segments.  FOLD (batch): one
// force-reduction site instead of three (the batch kernels' loop bodies miss the
// instruction cache).
template <bool ODD, bool FORCE, bool PER, bool MIS, bool STAGE_UP, bool FLAT = false, bool FOLD = false>
__device__ __forceinline__ void collide_segment_pairs(const CollideArgs<float>& a, WarpStage<float, STAGE_UP>& st,
                                                      int b, int sx, int sy, int z0, int len, uint32_t srcrow,
                                                      unsigned long long lead, bool smap_ok, bool sbtab_ok) {
    static_assert(!FLAT || (!ODD && MIS), "plane segments: even phase, unaligned-row staging");
    constexpr int V = WarpStage<float>::V;
    constexpr bool ADJ = !MIS;
    const int lane = threadIdx.x & 31;
    const Geom& g = a.g;
    const size_t N = g.N;
    float* F = a.fo;
    const size_t own = (size_t)st.row[b][row_slot(0, 0)];
    const int j0 = ADJ ? 2 * lane : lane, j1 = ADJ ? j0 + 1 : lane + 32;
    const bool v0 = j0 < len, v1 = j1 < len;
    const int za = z0 + j0, zb = z0 + j1;
    const size_t ca = own + za, cb = own + zb;
    // the cells' true geometry and coordinates (y, z) (FLAT: from the plane index;
    // otherwise gt is g itself, not a copy that would hold its fields in registers)
    Geom gflat;
    if constexpr (FLAT) {
        gflat = g;
        gflat.ny = a.flat_ny;
        gflat.nz = a.flat_nz;
    }
    const Geom& gt = FLAT ? gflat : g;
    int ya = sy, yb = sy, zta = za, ztb = zb;
    if constexpr (FLAT) {
        ya = (int)fast_div((unsigned)za, a.dnz);
        yb = (int)fast_div((unsigned)zb, a.dnz);
        zta = za - ya * a.flat_nz;
        ztb = zb - yb * a.flat_nz;
    }

    // staged values of direction i for the lane's two cells
    auto at2 = [&](int i) -> F2 {
        const int shift = (ODD && cz(i) != 0 && (PER || ((srcrow >> i) & 1u))) ? cz(i) : 0;
        const int m = MIS ? (int)((lead >> (2 * i)) & 3u) : 0;
        const float* p = &st.f[b][i][V + m - shift];
        if (ADJ && (shift & 1) == 0) {
            const float2 t = *reinterpret_cast<const float2*>(p + j0);
            return pk(t.x, t.y);
        }
        return pk(p[j0], p[j1]);
    };
    F2 f[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) f[i] = at2(i);
    const int vlead = MIS ? (int)((lead >> 38) & 3u) : 0;
    const uint32_t w0 = v0 ? st.vox[b][vlead + j0] : 0u, w1 = v1 ? st.vox[b][vlead + j1] : 0u;
    const int n0 = min((int)(w0 & VOX_NMASK), 125), n1 = min((int)(w1 & VOX_NMASK), 125);
    const int* smap = reinterpret_cast<const int*>(cta_tables<float, STAGE_UP>());
    const float* sbtab = reinterpret_cast<const float*>(smap + TAGMAP_SMEM);
    const F2 B = sbtab_ok ? pk(sbtab[n0], sbtab[n1]) : pk(__ldg(a.btab + n0), __ldg(a.btab + n1));

    // BGK runs for every cell, the fully covered ones included (their solid
    // correction with B = 1 returns fPre + bb up to rounding), so that a cell's
    // result does not depend on the cell it is paired with.
    const Mom2 m = moments2(f);
    F2 Fx = bc(0.f), Fy = bc(0.f), Fz = bc(0.f);
    // particle surface velocity of the lane's solid cells, recomputed from the
    // owner particle's row of the float table (one row when both cells belong to
    // the same particle), read after the BGK arithmetic.  (Looking the owners up
    // before the moment sums, or prefetching the rows, measured slower.)
    // owner slots (from the CTA's shared copy of the map when it has one)
    auto owner = [&](uint32_t w) -> int {
        const int tag = (int)(w >> VOX_NBITS);
        if (smap_ok) return smap[min(tag, TAGMAP_SMEM - 1)];
        // global map: an unconditional load at the clamped tag, tested afterwards
        const int slot = __ldg(a.tag2slot + min(tag, a.max_tag));
        return (tag <= a.max_tag && slot >= 0 && slot < a.nslot) ? slot : -1;
    };
    const int s0 = n0 > 0 ? owner(w0) : -1;
    const int s1 = n1 > 0 ? owner(w1) : -1;
    F2 up[3] = {bc(0.f), bc(0.f), bc(0.f)};
    // the centre part of the row the velocity read (slot vslot), kept for the force flush
    float4 vrh = make_float4(0.f, 0.f, 0.f, 0.f);
    float vrl0 = 0.f, vrl1 = 0.f;
    int vslot = -1;
    auto solid_velocity = [&]() {
        float ua[3] = {0.f, 0.f, 0.f}, ub[3] = {0.f, 0.f, 0.f};
        const int sl = s0 >= 0 ? s0 : s1;
        {
            // every lane of the warp loads a row (slot 0 for a lane without a solid
            // cell, whose velocities stay zero): no branch ahead of the load
            const TableRow r = load_row(a.xpf, max(sl, 0));
            vrh = r.a; vrl0 = r.b.x; vrl1 = r.b.y; vslot = sl;
            const RowPart rp = row_part(r, sx, ya, gt);
            if (s0 >= 0) cell_part(r, rp, zta, gt, ua[0], ua[1], ua[2]);
            if (sl >= 0 && s1 == sl) {
                if (FLAT && yb != ya) cell_part(r, row_part(r, sx, yb, gt), ztb, gt, ub[0], ub[1], ub[2]);
                else cell_part(r, rp, ztb, gt, ub[0], ub[1], ub[2]);
            }
        }
        if (s1 >= 0 && s1 != sl) row_velocity(load_row(a.xpf, s1), sx, yb, ztb, gt, ub[0], ub[1], ub[2]);
#pragma unroll
        for (int d = 0; d < 3; ++d) up[d] = pk(ua[d], ub[d]);
    };
    // FORCE: the solid correction's momentum is the BGK post-collision one, j + rho g,
    // for the cells that ran BGK
    auto hsol = [&]() -> F2 {
        return FORCE ? pk(n0 < 125 ? 1.f : 0.f, n1 < 125 ? 1.f : 0.f) * (bc(1.f) + m.rhoBar) : bc(0.f);
    };
    if constexpr (!FORCE) {
        // one pass; the solid terms only in warps that hold a solid cell
        if (__any_sync(FULL, n0 > 0 || n1 > 0)) {
            solid_velocity();
            collide_g2<true>(f, m, a.omega, up[0], up[1], up[2], B, Fx, Fy, Fz);
        } else {
            collide_g2<false>(f, m, a.omega, up[0], up[1], up[2], B, Fx, Fy, Fz);
        }
    } else if constexpr (MIS) {
        if (__any_sync(FULL, n0 > 0 || n1 > 0)) {   // one pass; a no-op for the lanes' fluid cells
            if (n0 > 0 || n1 > 0) solid_velocity();
            bgk_psm2<FORCE>(f, m, a.omega, a.g3[0], a.g3[1], a.g3[2], hsol(), up[0], up[1], up[2], B, Fx, Fy, Fz);
        } else
            bgk2<FORCE>(f, m, a.omega, a.g3[0], a.g3[1], a.g3[2]);
    } else {
        bgk2<FORCE>(f, m, a.omega, a.g3[0], a.g3[1], a.g3[2]);
        if (n0 > 0 || n1 > 0) {
            const F2 hs = hsol();
            const F2 sjx = fma2(hs, bc(a.g3[0]), m.jx), sjy = fma2(hs, bc(a.g3[1]), m.jy),
                     sjz = fma2(hs, bc(a.g3[2]), m.jz);
            solid_velocity();
            if (FORCE) psm2(f, m.rhoBar, sjx, sjy, sjz, m.invRho, up[0], up[1], up[2], B, at2, Fx, Fy, Fz);
            else psm2(f, m.rhoBar, m.jx, m.jy, m.jz, m.invRho, up[0], up[1], up[2], B, at2, Fx, Fy, Fz);
        }
    }

    // Stores.  put(off, x, y, vx, vy): values x, y into slots off, off + 1 (ADJ:
    // one 64-bit store when both are valid and the pair is aligned).
    auto put = [&](size_t off, float x, float y, bool vx, bool vy) {
        // aligned rows only (the launcher sends arrays that are not 16-byte aligned
        // to the unaligned-row path): an even slot offset is an 8-byte aligned pair
        if (vx && vy) {
            *reinterpret_cast<float2*>(F + off) = make_float2(x, y);
        } else {
            if (vx) F[off] = x;
            if (vy) F[off + 1] = y;
        }
    };
    // the lane's two cells into slots (i, base + j0) and (i, base + j1)
    auto put_cells = [&](size_t base, F2 v) {
        const float2 t = upk(v);
        if (ADJ) {
            // aligned rows: segments hold a multiple of 4 cells, so both cells of a pair
            // are valid together, and every pair of slots is 8-byte aligned
            if (v0) *reinterpret_cast<float2*>(F + base + j0) = t;
        } else {
            if (v0) F[base + j0] = t.x;
            if (v1) F[base + j1] = t.y;
        }
    };
    if (!ODD) {
#pragma unroll
        for (int i = 0; i < Q; ++i) put_cells((size_t)opp(i) * N + own + z0, f[i]);
    } else {
        put_cells(own + z0, f[0]);
        const int per_z = PER ? 1 : g.per[2];
#pragma unroll
        for (int i = 1; i < Q; ++i) {
            const long long r = st.row[b][row_slot(cx(i), cy(i))];
            if (!PER && r < 0) {            // beyond an x / y wall: bounce back in place
                put_cells((size_t)opp(i) * N + own + z0, f[i]);
                continue;
            }
            const size_t dst = (size_t)i * N + (size_t)r;   // row x + c_i
            if (cz(i) == 0) {
                put_cells(dst + z0, f[i]);
                continue;
            }
            // c_z != 0: each cell to slot z + c_z (wrapped, or bounced back at a z wall)
            const float2 t = upk(f[i]);
            if (ADJ) {
                // slots (j0, j0 + 1) of this lane receive cells (j0 - 1, j0) (c_z = +1)
                // or (j0 + 1, j0 + 2) (c_z = -1), one lane over; the cell whose slot
                // lies outside the segment (je) is stored on its own
                if (cz(i) > 0) put(dst + z0 + j0, __shfl_up_sync(FULL, t.y, 1), t.x, lane > 0 && v0, v1);
                else put(dst + z0 + j0, t.y, __shfl_down_sync(FULL, t.x, 1), v1, j0 + 2 < len);
                const int je = cz(i) > 0 ? len - 1 : 0;
                const int ze = z0 + je;
                const int zd = cz(i) > 0 ? wrap_plus(ze, g.nz, per_z) : wrap_minus(ze, g.nz, per_z);
                const size_t eoff = (PER || zd >= 0) ? dst + zd : (size_t)opp(i) * N + own + ze;
                const float ev = (je & 1) ? t.y : t.x;
                if (lane == (je >> 1)) F[eoff] = ev;
            } else {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (h == 0 ? !v0 : !v1) continue;
                    const int zz = h == 0 ? za : zb;
                    const int zd = cz(i) > 0 ? wrap_plus(zz, g.nz, per_z) : wrap_minus(zz, g.nz, per_z);
                    const float val = h == 0 ? t.x : t.y;
                    if (PER || zd >= 0) F[dst + zd] = val;
                    else F[(size_t)opp(i) * N + own + zz] = val;
                }
            }
        }
    }

    const float2 fx = upk(Fx), fy = upk(Fy), fz = upk(Fz);
    if (a.cf) {
        if (v0) { a.cf[ca] = fx.x; a.cf[N + ca] = fy.x; a.cf[2 * N + ca] = fz.x; }
        if (v1) { a.cf[cb] = fx.y; a.cf[N + cb] = fy.y; a.cf[2 * N + cb] = fz.y; }
    }
    if constexpr (FLAT) {
        // per-cell arms (a run of one owner may cross rows here), keyed by the owner
        // slots of the velocity lookup; the arm reads the centre from the table row
        // that lookup kept (a second owner in the lane reads its own row)
        if ((v0 && n0 > 0 && s0 < 0) || (v1 && n1 > 0 && s1 < 0)) atomicOr(a.err, 0x8u);   // LBDEM_DEVERR_UNMAPPED_TAG
        const int ka = v0 ? s0 : -1;
        const int kb = v1 ? s1 : -1;
        if (!__any_sync(FULL, ka >= 0 || kb >= 0)) return;
        auto terms = [&](int slot, int y, int z, float cfx, float cfy, float cfz, float (&v)[6]) {
            float4 h = vrh;
            float lx = vrl0, lz = vrl1;
            if (slot != vslot) {
                const float4* p = reinterpret_cast<const float4*>(a.xpf + (size_t)slot * XPF_STRIDE);
                h = __ldg(p);
                const float4 l = __ldg(p + 1);
                lx = l.x;
                lz = l.y;
            }
            // centre = hi + lo in float: (x - hi) - lo is the arm to ~1 ulp
            arm_terms(((float)sx - h.x) - h.w, ((float)y - h.y) - lx, ((float)z - h.z) - lz, gt, cfx, cfy, cfz, v);
        };
        float va[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, vb[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (ka >= 0) terms(ka, ya, zta, fx.x, fy.x, fz.x, va);
        if (kb >= 0) terms(kb, yb, ztb, fx.y, fy.y, fz.y, vb);
        const bool one = __all_sync(FULL, ka < 0 || kb < 0 || ka == kb);   // one reduction for both cells
        if (one) {
#pragma unroll
            for (int q = 0; q < 6; ++q) va[q] += vb[q];
        }
        // a single reduction site: this kernel's loop body is large enough for
        // instruction-cache misses to cost more than the loop
#pragma unroll 1
        for (int pass = 0; pass < (one ? 1 : 2); ++pass) {
            float v[6];
#pragma unroll
            for (int q = 0; q < 6; ++q) v[q] = pass == 0 ? va[q] : vb[q];
            reduce_forces(a, pass == 0 ? (one && ka < 0 ? kb : ka) : kb, v);
        }
        return;
    }
    if ((PER || g.per[2]) && len == g.nz) {
        // the segment is a whole z-periodic row: a particle's chord may wrap
        // around inside it, so the arms are taken per cell
        whole_row_forces(a, w0, w1, v0, v1, sx, sy, za, zb, fx, fy, fz);
        return;
    }
    // runs of equal owner, arms from the segment's middle point zc
    const int zc = z0 + SEGW / 2;
    // keys: the owners' particle slots; a solid cell whose tag names no particle is
    // reported and left out
    const int ka = v0 ? s0 : -1;
    const int kb = v1 ? s1 : -1;
    if ((v0 && n0 > 0 && s0 < 0) || (v1 && n1 > 0 && s1 < 0)) atomicOr(a.err, 0x8u);   // LBDEM_DEVERR_UNMAPPED_TAG
    const float da = (float)(za - zc), db = (float)(zb - zc);
    float va[5] = {fx.x, fy.x, fz.x, -da * fy.x, da * fx.x};
    float vb[5] = {fx.y, fy.y, fz.y, -db * fy.y, db * fx.y};
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        if (ka < 0) va[q] = 0.f;
        if (kb < 0) vb[q] = 0.f;
    }
    if constexpr (FOLD) {
        const bool one = __all_sync(FULL, ka < 0 || kb < 0 || ka == kb);   // one reduction for both cells
        if (one) {
#pragma unroll
            for (int q = 0; q < 5; ++q) va[q] += vb[q];
        }
#pragma unroll 1
        for (int pass = 0; pass < (one ? 1 : 2); ++pass) {
            float v[5];
#pragma unroll
            for (int q = 0; q < 5; ++q) v[q] = pass == 0 ? va[q] : vb[q];
            const bool second = pass == 1 || (one && ka < 0);   // the run's cells are the b cells
            reduce_runs(a, second ? kb : ka, v, second ? zb : za, sx, sy, zc, vrh, vrl0, vrl1, vslot);
        }
    } else if (__all_sync(FULL, ka < 0 || kb < 0 || ka == kb)) {
        const int key = ka >= 0 ? ka : kb;
#pragma unroll
        for (int q = 0; q < 5; ++q) va[q] += vb[q];
        reduce_runs(a, key, va, ka >= 0 ? za : zb, sx, sy, zc, vrh, vrl0, vrl1, vslot);
    } else {
        reduce_runs(a, ka, va, za, sx, sy, zc, vrh, vrl0, vrl1, vslot);
        reduce_runs(a, kb, vb, zb, sx, sy, zc, vrh, vrl0, vrl1, vslot);
    }
}

// PER: every axis periodic (no wall cases; shifts and neighbour rows are fixed).
// MIS: rows not 16-byte aligned (see issue_segment).
// BATCH: segments of many domains, numbered domain after domain (seg0[d] is
// the first segment of domain d); every domain has its own CollideArgs.
template <typename T, bool ODD, bool FORCE, bool PER, bool MIS, bool BATCH>
__global__ void __launch_bounds__(COLLIDE_BLOCK, sizeof(T) == 4 ? 4 : 2)
k_collide_staged(const CollideArgs<T> a1, long long nseg, const CollideArgs<T>* __restrict__ dargs,
                 const int* __restrict__ seg0, int ndom) {
    constexpr int V = WarpStage<T>::V;
    // FP64 form: surface-velocity rows staged with the populations for a single
    // lattice; the many short rows of a batch read them directly (three more small
    // copies per segment cost more there than the loads they replace).  The FP32
    // form keeps no velocity field (it recomputes the velocity per solid cell).
    constexpr bool STAGE_UP = stage_up<T, BATCH>();
    // FP32 form, aligned rows of a single lattice: staging by per-thread cp.async
    constexpr bool LSU = sizeof(T) == 4 && !MIS && !BATCH;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    WarpStage<T, STAGE_UP>& st = reinterpret_cast<WarpStage<T, STAGE_UP>*>(smem_raw)[warp];
    __shared__ unsigned long long probe[WARPS];   // the test hook's barrier (never completes)
    if (lane == 0) {
        mbar_init(&st.bar[0], 1);
        mbar_init(&st.bar[1], 1);
        mbar_init(&probe[warp], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    bool smap_ok = false;   // the CTA holds a copy of the tag -> slot map (FP32, single lattice)
    if constexpr (smem_tagmap<T, BATCH>()) {
        int* m = reinterpret_cast<int*>(cta_tables<T, STAGE_UP>());
        smap_ok = a1.max_tag < TAGMAP_SMEM - 1;
        if (smap_ok)
            for (int k = threadIdx.x; k < TAGMAP_SMEM; k += blockDim.x) {
                const int v = k <= a1.max_tag ? __ldg(a1.tag2slot + k) : -1;
                m[k] = (v >= 0 && v < a1.nslot) ? v : -1;
            }
        float* sb = reinterpret_cast<float*>(m + TAGMAP_SMEM);
        for (int k = threadIdx.x; k < 126; k += blockDim.x) sb[k] = __ldg(a1.btab + k);
        __syncthreads();   // every warp of the CTA reaches it (before any leaves)
    }
    const int* sseg0 = nullptr;   // batch: the CTA's copy of seg0 (ndom <= SEG0_SMEM)
    if constexpr (BATCH) {
        int* m = reinterpret_cast<int*>(cta_tables<T, STAGE_UP>());
        if (ndom <= SEG0_SMEM) {
            for (int k = threadIdx.x; k < ndom; k += blockDim.x) m[k] = __ldg(seg0 + k);
            sseg0 = m;
        }
        __syncthreads();   // every warp of the CTA reaches it (before any leaves)
    }
    const long long stride = (long long)gridDim.x * WARPS;
    long long seg = (long long)blockIdx.x * WARPS + warp;
    if (seg >= nseg) return;
    auto issue = [&](int buf, long long sg) -> T {
        if constexpr (LSU) {
            issue_segment_lsu<T, ODD, PER, STAGE_UP>(a1, st, buf, sg);
            return T(0);
        }
        if (BATCH) {
            int d, first;
            if (sseg0) {
                int lo = 0, hi = ndom - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (sseg0[mid] <= (int)sg) lo = mid;
                    else hi = mid - 1;
                }
                d = lo;
                first = sseg0[d];
            } else {
                d = find_domain(seg0, ndom, (int)sg);
                first = __ldg(seg0 + d);
            }
            const CollideArgs<T>& A = dargs[d];
            return issue_segment<T, ODD, MIS, STAGE_UP>(A, st, buf, sg - first, d);
        }
        return issue_segment<T, ODD, MIS, STAGE_UP>(a1, st, buf, sg, 0);
    };
    T hcur = issue(0, seg);
    uint32_t phase = 0;   // bit b: parity expected next on buffer b
    bool first = true;
    int b = 0;
    for (; seg < nseg; seg += stride, b ^= 1) {
        const long long next = seg + stride;
        T hnext = T(0);
        if (next < nseg) hnext = issue(b ^ 1, next);
        if constexpr (LSU) {
            // this thread's copies of the current segment (all groups but the newest)
            if (next < nseg) cp_wait<1>();
            else cp_wait<0>();
            __syncwarp();   // and every other lane's
        } else {
            const uint32_t pb = (phase >> b) & 1u;
            bool ok;
            if (!BATCH && a1.probe_timeout && first) {
                // test hook: wait on a barrier nothing arrives on, as for a copy that never lands
                ok = mbar_wait(&probe[warp], 0u, PROBE_WAIT);
            } else {
                ok = mbar_wait(&st.bar[b], pb);
            }
            phase ^= 1u << b;
            first = false;
            if (__any_sync(FULL, !ok)) {
                // a copy did not land: report, let this warp's copies in flight land
                // (both buffers, bounded), leave
                if (lane == 0) atomicOr(BATCH ? dargs[0].err : a1.err, 0x20u);   // LBDEM_DEVERR_TIMEOUT
                mbar_wait(&st.bar[b], pb);
                if (next < nseg) mbar_wait(&st.bar[b ^ 1], (phase >> (b ^ 1)) & 1u);
                return;
            }
        }
        const int sx = st.geo[b][0], sy = st.geo[b][1], z0 = st.geo[b][2], len = st.geo[b][3];
        const CollideArgs<T>& a = BATCH ? dargs[st.geo[b][4]] : a1;
        const Geom& g = a.g;
        const size_t N = g.N;
        const T* Fin = a.f;   // input populations
        T* F = a.fo;          // output populations (== a.f in place)
        const size_t own = (size_t)st.row[b][row_slot(0, 0)];
        const unsigned long long lead = MIS ? st.lead[b] : 0ull;
        if (MIS && ODD) {
            if (lane < 10) {
                const int i = zdir(lane);
                if (st.row[b][row_slot(-cx(i), -cy(i))] >= 0) {
                    const int m = (int)((lead >> (2 * i)) & 3u);
                    if (cz(i) > 0) st.f[b][i][V + m - 1] = hcur;
                    else st.f[b][i][V + m + len] = hcur;
                }
            }
            __syncwarp();
        }
        // Odd phase with walls along z, aligned rows: the halo element of an edge
        // cell is its own slot i (half-way bounce-back).
        if (!MIS && ODD && !PER && !g.per[2] && (z0 == 0 || z0 + len == g.nz)) {
            if (lane < 10) {
                const int i = zdir(lane);
                if (st.row[b][row_slot(-cx(i), -cy(i))] >= 0) {
                    if (cz(i) > 0 && z0 == 0) st.f[b][i][V - 1] = Fin[(size_t)i * N + own];
                    if (cz(i) < 0 && z0 + len == g.nz) st.f[b][i][V + len] = Fin[(size_t)i * N + own + g.nz - 1];
                }
            }
            __syncwarp();
        }
        uint32_t srcrow = 0;   // bit i: source row of direction i lies inside the lattice
        if (ODD && !PER) {
#pragma unroll
            for (int i = 1; i < Q; ++i)
                if (cz(i) != 0 && st.row[b][row_slot(-cx(i), -cy(i))] >= 0) srcrow |= 1u << i;
        }
        if constexpr (sizeof(T) == 4) {
            // FP32 form: packed pairs of cells (batch, even phase: plane segments)
            collide_segment_pairs<ODD, FORCE, PER, MIS, STAGE_UP, BATCH && !ODD, BATCH>(
                a, st, b, sx, sy, z0, len, srcrow, lead, smap_ok, smem_tagmap<T, BATCH>());
        } else {
            // FP64 form: one cell per lane at a time; force and torque per cell with
            // double atomics.  The segment's solid cells are taken first (pass 0
            // holds as many of them as fit): a pass whose warp holds a solid cell
            // runs the solid terms for every lane, so gathering them leaves more
            // passes on the BGK-only path.  A cell's result does not depend on
            // its pass.
            static_assert(SEGW == 64, "two passes of 32 cells per segment");
            const int vlead = MIS ? (int)((lead >> 38) & 3u) : 0;
            const uint32_t wl0 = lane < len ? st.vox[b][vlead + lane] : 0u;
            const uint32_t wl1 = lane + 32 < len ? st.vox[b][vlead + lane + 32] : 0u;
            const unsigned sol0 = __ballot_sync(FULL, (wl0 & VOX_NMASK) != 0u);
            const unsigned sol1 = __ballot_sync(FULL, (wl1 & VOX_NMASK) != 0u);
            const unsigned flu0 = __ballot_sync(FULL, lane < len) & ~sol0;
            const unsigned flu1 = __ballot_sync(FULL, lane + 32 < len) & ~sol1;
            const int ns0 = __popc(sol0), ns = ns0 + __popc(sol1);
            const int nf0 = __popc(flu0), nf = nf0 + __popc(flu1);
#pragma unroll 1
            for (int p = 0; p < 2; ++p) {
                const int slot = 32 * p + lane;
                int j = -1;   // the cell this lane takes in pass p
                if (slot < ns) j = slot < ns0 ? nth_bit(sol0, slot) : 32 + nth_bit(sol1, slot - ns0);
                else if (slot - ns < nf) j = slot - ns < nf0 ? nth_bit(flu0, slot - ns) : 32 + nth_bit(flu1, slot - ns - nf0);
                const bool any_solid = ns > 32 * p;   // warp-uniform
                T v[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
                if (j >= 0) {
                    const uint32_t w = st.vox[b][vlead + j];
                    const int z = z0 + j;
                    const size_t c = own + z;
                    // smem index of direction i: V + lead_i + j - shift_i, shift_i = c_z,i
                    // when the source row x - c_i exists (odd phase)
                    auto at = [&](int i) -> const T& {
                        const int shift = (ODD && cz(i) != 0 && (PER || ((srcrow >> i) & 1u))) ? cz(i) : 0;
                        const int m = MIS ? (int)((lead >> (2 * i)) & 3u) : 0;
                        return st.f[b][i][V + m + j - shift];
                    };
                    T f[Q];
#pragma unroll
                    for (int i = 0; i < Q; ++i) f[i] = at(i);
                    T Fx, Fy, Fz;
                    auto upv = [&](int d) -> T {
                        if (!STAGE_UP) return __ldg(a.up + (size_t)d * N + c);
                        const int m = MIS ? (int)((lead >> (40 + 2 * d)) & 3u) : 0;
                        return st.up[b][d][m + j];
                    };
                    if constexpr (!FORCE) {
                        const int n = min((int)(w & VOX_NMASK), 125);
                        if (any_solid) {
                            const bool s = n > 0;   // a fluid cell's velocity slot is not read
                            collide_cell_fp64<true>(f, a.omega, __ldg(a.btab + n), s ? upv(0) : T(0),
                                                    s ? upv(1) : T(0), s ? upv(2) : T(0), Fx, Fy, Fz);
                        } else {
                            collide_cell_fp64<false>(f, a.omega, T(0), T(0), T(0), T(0), Fx, Fy, Fz);
                        }
                    } else {
                        collide_cell<T, FORCE>(a, f, w, [&](int i) { return at(i); }, upv, Fx, Fy, Fz);
                    }
                    if (!ODD) {
#pragma unroll
                        for (int i = 0; i < Q; ++i) F[(size_t)opp(i) * N + c] = f[i];
                    } else {
                        F[c] = f[0];
                        const int zm = wrap_minus(z, g.nz, PER ? 1 : g.per[2]);
                        const int zp = wrap_plus(z, g.nz, PER ? 1 : g.per[2]);
#pragma unroll
                        for (int i = 1; i < Q; ++i) {
                            const long long r = st.row[b][row_slot(cx(i), cy(i))];
                            const int zd = pick(cz(i), zm, z, zp);
                            if (PER || (r >= 0 && zd >= 0)) F[(size_t)i * N + (size_t)r + zd] = f[i];
                            else F[(size_t)opp(i) * N + c] = f[i];
                        }
                    }
                    if (a.cf) { a.cf[c] = Fx; a.cf[N + c] = Fy; a.cf[2 * N + c] = Fz; }
                    const int key = cell_force_terms(a, w, sx, sy, z, Fx, Fy, Fz, v);
                    if (key >= 0) add_cell_force(a, key, v);
                }
            }
        }
        __syncwarp();   // buffer b is free for the segment after next
        hcur = hnext;
    }
}

template <typename T, bool ODD, bool FORCE, bool PER, bool MIS, bool BATCH>
cudaError_t launch_staged(const CollideArgs<T>& a, long long nseg, const CollideArgs<T>* dargs,
                          const int* seg0, int ndom, int blocks_per_sm, cudaStream_t s) {
    constexpr size_t smem =
        WARPS * sizeof(WarpStage<T, stage_up<T, BATCH>()>) + tagmap_bytes<T, BATCH>() + seg0_bytes<BATCH>();
    if (nseg >= (1LL << 31)) return cudaErrorInvalidValue;   // segment indices are split in 32 bits
    // per device: (resident blocks per SM << 16) | SM count, 0 until first use there
    static std::atomic<int> shape[LBDEM_MAX_DEVICES];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= LBDEM_MAX_DEVICES) return cudaErrorInvalidDevice;
    int packed = shape[dev].load(std::memory_order_relaxed);
    if (packed == 0) {
        int sms = 0, per_sm = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_collide_staged<T, ODD, FORCE, PER, MIS, BATCH>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_collide_staged<T, ODD, FORCE, PER, MIS, BATCH>,
                                                              COLLIDE_BLOCK, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        packed = (per_sm << 16) | (sms & 0xffff);
        shape[dev].store(packed, std::memory_order_relaxed);
    }
    const int per_sm = packed >> 16, sms = packed & 0xffff;
    if (nseg <= 0) return cudaSuccess;
    const int use = (blocks_per_sm > 0 && blocks_per_sm < per_sm) ? blocks_per_sm : per_sm;
    const long long want = (long long)sms * use;
    const long long blocks = (nseg + WARPS - 1) / WARPS;
    const unsigned grid = (unsigned)(blocks < want ? blocks : want);
    k_collide_staged<T, ODD, FORCE, PER, MIS, BATCH><<<grid, COLLIDE_BLOCK, smem, s>>>(a, nseg, dargs, seg0, ndom);
    return cudaGetLastError();
}

template <typename T, bool ODD, bool FORCE>
cudaError_t launch_one(const CollideArgs<T>& args, cudaStream_t s) {
    const int nzseg = (args.g.nz + SEGW - 1) / SEGW;
    CollideArgs<T> a = args;
    a.dz = div_magic((unsigned)nzseg);
    a.dy = div_magic((unsigned)a.g.ny);
    const long long nseg = (long long)a.g.nx * a.g.ny * nzseg;
    // Aligned bulk copies need every row start and length 16-byte aligned:
    // population rows (nz * sizeof(T)) and voxel-word rows (nz * 4), i.e. nz % 4 == 0,
    // and 16-byte aligned arrays (device allocations are; a caller's out-of-place
    // target that is not takes the unaligned-row path)
    const bool arrays_aligned = (((uintptr_t)a.f | (uintptr_t)a.fo | (uintptr_t)a.vox | (uintptr_t)a.up) & 15u) == 0;
    if (a.g.nz % 4 == 0 && arrays_aligned) {
        if (a.g.per[0] && a.g.per[1] && a.g.per[2])
            return launch_staged<T, ODD, FORCE, true, false, false>(a, nseg, nullptr, nullptr, 0, 0, s);
        return launch_staged<T, ODD, FORCE, false, false, false>(a, nseg, nullptr, nullptr, 0, 0, s);
    }
    return launch_staged<T, ODD, FORCE, false, true, false>(a, nseg, nullptr, nullptr, 0, 0, s);
}

template <typename T, bool ODD, bool FORCE>
cudaError_t launch_batch(const CollideArgs<T>* dargs, const int* seg0, int ndom, long long nseg, int blocks_per_sm,
                         cudaStream_t s) {
    CollideArgs<T> none{};
    return launch_staged<T, ODD, FORCE, false, true, true>(none, nseg, dargs, seg0, ndom, blocks_per_sm, s);
}

}  // namespace

template <typename T>
cudaError_t launch_collide_stream(const CollideArgs<T>& a, bool odd, bool force, cudaStream_t s) {
    if (odd) return force ? launch_one<T, true, true>(a, s) : launch_one<T, true, false>(a, s);
    return force ? launch_one<T, false, true>(a, s) : launch_one<T, false, false>(a, s);
}

template <typename T>
cudaError_t launch_collide_batch(const CollideArgs<T>* dargs, const int* seg0, int ndom, long long nseg, bool odd,
                                 bool force, int blocks_per_sm, cudaStream_t s) {
    if (odd)
        return force ? launch_batch<T, true, true>(dargs, seg0, ndom, nseg, blocks_per_sm, s)
                     : launch_batch<T, true, false>(dargs, seg0, ndom, nseg, blocks_per_sm, s);
    return force ? launch_batch<T, false, true>(dargs, seg0, ndom, nseg, blocks_per_sm, s)
                 : launch_batch<T, false, false>(dargs, seg0, ndom, nseg, blocks_per_sm, s);
}

template cudaError_t launch_collide_stream<float>(const CollideArgs<float>&, bool, bool, cudaStream_t);
template cudaError_t launch_collide_stream<double>(const CollideArgs<double>&, bool, bool, cudaStream_t);
template cudaError_t launch_collide_batch<float>(const CollideArgs<float>*, const int*, int, long long, bool, bool,
                                                 int, cudaStream_t);
template cudaError_t launch_collide_batch<double>(const CollideArgs<double>*, const int*, int, long long, bool, bool,
                                                  int, cudaStream_t);

}  // namespace lbdem
