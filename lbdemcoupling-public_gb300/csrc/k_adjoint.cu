// Reverse-mode (adjoint) step of the PSM lattice: gradients of a loss built
// from the per-particle forces and torques of a window of steps, with respect
// to the populations, the per-step particle velocities and angular velocities,
// the body force and the relaxation time tau.  The solid fraction and owner of
// every cell are held fixed over the window and are not differentiated.
//
// Forward map of one cell (what K1 computes, src/ibCompositeDynamics3D.hh:130-203,
// written as one function of the pre-collision populations f):
//   BGK with Guo forcing (n < 125):
//     rhoBar = sum f, j = sum c f, rho = 1 + rhoBar, r = 1/rho,
//     J = j + rho g / 2, u = J r, pre = (1 - omega/2) rho,
//     feq_k = t_k [rhoBar + 3 c_k.J + r (4.5 (c_k.J)^2 - 1.5 J.J)],
//     src_k = t_k pre [3 (c_k.g - u.g) + 9 (c_k.u)(c_k.g)],
//     f*_k = (1 - omega) f_k + omega feq_k + src_k          (f* = f when n = 125)
//   PSM (n > 0), moments rhoBar*, j* of f*, P = (1 + rhoBar*) uP:
//     out_k = (1 - B) f*_k + B (f_opp(k) - feq_opp(k)(j*) + feq_k(P))   k != 0
//     out_0 = (1 - B) f*_0 + B (f_0 + feq_0(j*) - feq_0(P))
//     F = -sum_{k=1..9} c_k (bb_k - bbOpp_k) = B (2 j - j* - P)
//   (feq(.) at rhoBar*, 1/(1 + rhoBar*)), and push streaming with half-way
//   bounce-back.  With uP = v + w x d (d: cell minus particle centre, minimum
//   image), tau entering through omega = 1/tau and B = sf ooo / ((1 - sf) + ooo),
//   ooo = tau - 1/2.
//
// The adjoint step, per cell x, given lambda_{t+1} (natural layout):
//   mu_k   = lambda_{t+1,k}(x + c_k), or lambda_{t+1,opp k}(x) beyond a wall
//            (transpose of push streaming),
//   a      = dL/dF of the owner particle at this step (+ w_T x arm for torques),
//   lambda_t(x) = (d out / d f)^T mu + (dF/df)^T a, and the parameter
//   gradients (d out / d theta)^T mu + (dF/d theta)^T a,
// evaluated by hand-written reverse differentiation of the formulas above.
#include "lbdem_internal.h"

namespace lbdem {
namespace {

constexpr unsigned FULLMASK = 0xffffffffu;
constexpr int ADJ_THREADS = 256;

template <typename T>
__device__ __forceinline__ T cdotT(int k, T a, T b, T c) {
    const int X = cx(k), Y = cy(k), Z = cz(k);
    T r = T(0);
    if (X) r = X > 0 ? a : -a;
    if (Y) r = Y > 0 ? r + b : r - b;
    if (Z) r = Z > 0 ? r + c : r - c;
    return r;
}

// 1/x: IEEE division in float; in double a float reciprocal refined by two
// Newton-Raphson steps r <- r (2 - x r) (relative error ~2^-23 -> ~2^-46 -> below
// double rounding), far cheaper than a double division on the narrow FP64 pipe.
__device__ __forceinline__ float recipT(float x) { return 1.0f / x; }
__device__ __forceinline__ double recipT(double x) {
    double r = (double)(1.0f / (float)x);
    r = r * (2.0 - x * r);
    return r * (2.0 - x * r);
}

template <typename T>
__device__ __forceinline__ T feqT(int k, T rb, T r, T c_dot, T sq) {
    return T(wt(k)) * (rb + T(3) * c_dot + r * (T(4.5) * c_dot * c_dot - T(1.5) * sq));
}

// Scalars of one cell's reverse pass; with them lambda_k (the adjoint of f_k) is
//   psm_k + (n == 125 ? phi_k : (1 - omega) phi_k + grb + c_k . gJ),
//   psm_k = B mu_opp(k) + 2 B (a . c_k),  phi_k = sB mu_k + grbs + c_k . gjs
// (n == 0: B = 0, sB = 1, grbs = gjs = 0), so the 19 values are formed while
// they are stored and never held together.
template <typename T>
struct CellAdj {
    T B, sB, grbs, gjs0, gjs1, gjs2;   // PSM part: adjoint of f* = sB mu + grbs + c . gjs
    T grb, gJ0, gJ1, gJ2;              // BGK part
};

// Reverse of one cell.  f: pre-collision populations; mu: adjoint of the
// post-collision populations; a: adjoint of the cell force.  Accumulates
// d/duP, d/dtau, d/dg and returns the scalars lambda is built from.
// general (warp-uniform: the warp holds a solid cell): a fluid cell takes the
// solid cells' path too, with B = 0, where it yields B = 0, sB = 1 and zero
// grbs, gjs, guP, so phi = mu and the same bits as the fluid path; the warp
// then runs one path instead of both.
template <typename T>
__device__ __forceinline__ CellAdj<T> adjoint_cell(const T (&f)[Q], const T (&mu)[Q], int n, bool general, T B,
                                                   T dBdtau, const T (&uP)[3], const T (&a)[3], T omega,
                                                   const T (&g)[3], T (&guP)[3], T& gtau, T (&gg)[3]) {
    CellAdj<T> R;
    // pre-collision moments
    T rb = T(0), j0 = T(0), j1 = T(0), j2 = T(0);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        rb += f[k];
        if (cx(k)) j0 += cx(k) > 0 ? f[k] : -f[k];
        if (cy(k)) j1 += cy(k) > 0 ? f[k] : -f[k];
        if (cz(k)) j2 += cz(k) > 0 ? f[k] : -f[k];
    }
    const T rho = T(1) + rb, r = recipT(rho);
    const T J0 = j0 + T(0.5) * rho * g[0], J1 = j1 + T(0.5) * rho * g[1], J2v = j2 + T(0.5) * rho * g[2];
    const T u0 = J0 * r, u1 = J1 * r, u2 = J2v * r;
    const T JJ = J0 * J0 + J1 * J1 + J2v * J2v;
    const T pre = (T(1) - T(0.5) * omega) * rho;
    const T ug = u0 * g[0] + u1 * g[1] + u2 * g[2];

    R.B = T(0); R.sB = T(1); R.grbs = T(0); R.gjs0 = T(0); R.gjs1 = T(0); R.gjs2 = T(0);
    guP[0] = guP[1] = guP[2] = T(0);
    if (n > 0 || general) {
        // moments of f* and S1 = sum mu_k f*_k
        T rbs = T(0), js0 = T(0), js1 = T(0), js2 = T(0), S1 = T(0);
        if (n == 125) {
            rbs = rb; js0 = j0; js1 = j1; js2 = j2;
#pragma unroll
            for (int k = 0; k < Q; ++k) S1 += mu[k] * f[k];
        } else {
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                const T cJ = cdotT<T>(k, J0, J1, J2v);
                const T cu = cdotT<T>(k, u0, u1, u2), cg = cdotT<T>(k, g[0], g[1], g[2]);
                const T src = T(wt(k)) * pre * (T(3) * (cg - ug) + T(9) * cu * cg);
                const T fs = (T(1) - omega) * f[k] + omega * feqT<T>(k, rb, r, cJ, JJ) + src;
                rbs += fs;
                if (cx(k)) js0 += cx(k) > 0 ? fs : -fs;
                if (cy(k)) js1 += cy(k) > 0 ? fs : -fs;
                if (cz(k)) js2 += cz(k) > 0 ? fs : -fs;
                S1 += mu[k] * fs;
            }
        }
        R.B = B;
        R.sB = T(1) - B;
        const T rhos = T(1) + rbs, rs = recipT(rhos);
        const T Jq = js0 * js0 + js1 * js1 + js2 * js2;
        const T P0 = rhos * uP[0], P1 = rhos * uP[1], P2v = rhos * uP[2];
        const T PP = P0 * P0 + P1 * P1 + P2v * P2v;
        // F = B (2 j - j* - P)
        T gB = -S1 + a[0] * (T(2) * j0 - js0 - P0) + a[1] * (T(2) * j1 - js1 - P1) + a[2] * (T(2) * j2 - js2 - P2v);
        T gjs0 = -B * a[0], gjs1 = -B * a[1], gjs2 = -B * a[2];
        T gP0 = -B * a[0], gP1 = -B * a[1], gP2 = -B * a[2];
        // seeds e (of feq at j*) and E (of feq at P) of the B-weighted terms of out,
        // folded into the equilibria's reverse as they are formed
        T se = T(0), sE = T(0), grs = T(0);
        {
            const T q0 = feqT<T>(0, rbs, rs, T(0), Jq), s0 = feqT<T>(0, rbs, rs, T(0), PP);
            gB += mu[0] * (f[0] + q0 - s0);
            const T w = T(wt(0)), e0 = B * mu[0], E0 = -B * mu[0];
            se += w * e0;
            sE += w * E0;
            grs += w * (e0 * (-T(1.5) * Jq) + E0 * (-T(1.5) * PP));
        }
#pragma unroll
        for (int i = 1; i <= 9; ++i) {
            const int o = i + 9;
            const T w = T(wt(i));
            const T ci = cdotT<T>(i, js0, js1, js2);
            const T pi = cdotT<T>(i, P0, P1, P2v);
            const T qi = feqT<T>(i, rbs, rs, ci, Jq), qo = feqT<T>(o, rbs, rs, -ci, Jq);
            const T si = feqT<T>(i, rbs, rs, pi, PP), so = feqT<T>(o, rbs, rs, -pi, PP);
            gB += mu[i] * (f[o] - qo + si) + mu[o] * (f[i] - qi + so);
            const T ei = -B * mu[o], eo = -B * mu[i], Ei = B * mu[i], Eo = B * mu[o];
            se += w * (ei + eo);
            sE += w * (Ei + Eo);
            const T cq = T(4.5) * ci * ci - T(1.5) * Jq, pq = T(4.5) * pi * pi - T(1.5) * PP;
            grs += w * ((ei + eo) * cq + (Ei + Eo) * pq);
            // c_i w (e_i (3 + 9 rs c_i.j*) - e_o (3 - 9 rs c_i.j*)), c_o = -c_i
            const T aj = w * (ei * (T(3) + T(9) * rs * ci) - eo * (T(3) - T(9) * rs * ci));
            const T ap = w * (Ei * (T(3) + T(9) * rs * pi) - Eo * (T(3) - T(9) * rs * pi));
            if (cx(i)) { gjs0 += cx(i) > 0 ? aj : -aj; gP0 += cx(i) > 0 ? ap : -ap; }
            if (cy(i)) { gjs1 += cy(i) > 0 ? aj : -aj; gP1 += cy(i) > 0 ? ap : -ap; }
            if (cz(i)) { gjs2 += cz(i) > 0 ? aj : -aj; gP2 += cz(i) > 0 ? ap : -ap; }
        }
        // the -3 rs j* (resp. P) part of d feq / d j*, summed over k
        gjs0 -= T(3) * rs * se * js0; gjs1 -= T(3) * rs * se * js1; gjs2 -= T(3) * rs * se * js2;
        gP0 -= T(3) * rs * sE * P0; gP1 -= T(3) * rs * sE * P1; gP2 -= T(3) * rs * sE * P2v;
        // P = rho* uP, rs = 1/rho*, rho* = 1 + rbs
        T grhos = gP0 * uP[0] + gP1 * uP[1] + gP2 * uP[2];
        guP[0] = rhos * gP0; guP[1] = rhos * gP1; guP[2] = rhos * gP2;
        grhos -= rs * rs * grs;
        R.grbs = se + sE + grhos;
        R.gjs0 = gjs0; R.gjs1 = gjs1; R.gjs2 = gjs2;
        gtau += gB * dBdtau;
    }

    R.grb = T(0); R.gJ0 = T(0); R.gJ1 = T(0); R.gJ2 = T(0);
    if (n == 125) return R;   // no BGK: f* = f
    // BGK reverse with phi_k = sB mu_k + grbs + c_k . gjs.  Every term is a
    // weighted moment of phi of order <= 2 in c_k (feq and src are quadratic in
    // c_k), so the sums over k reduce to m0 = sum t_k phi_k, m1 = sum t_k phi_k c_k,
    // m2 = sum t_k phi_k c_k c_k^T, and sum phi_k f_k.
    T m0 = T(0), m1x = T(0), m1y = T(0), m1z = T(0);
    T mxx = T(0), myy = T(0), mzz = T(0), mxy = T(0), mxz = T(0), myz = T(0), sphf = T(0);
    auto moments = [&](auto phi_of) {
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const T phi = phi_of(k);
            sphf += phi * f[k];
            const T wp = T(wt(k)) * phi;
            m0 += wp;
            const int X = cx(k), Y = cy(k), Z = cz(k);
            if (X) { m1x += X > 0 ? wp : -wp; mxx += wp; }
            if (Y) { m1y += Y > 0 ? wp : -wp; myy += wp; }
            if (Z) { m1z += Z > 0 ? wp : -wp; mzz += wp; }
            if (X && Y) mxy += X * Y > 0 ? wp : -wp;
            if (X && Z) mxz += X * Z > 0 ? wp : -wp;
            if (Y && Z) myz += Y * Z > 0 ? wp : -wp;
        }
    };
    if (!general) moments([&](int k) { return mu[k]; });   // fluid cells only: phi = mu
    else moments([&](int k) { return R.sB * mu[k] + R.grbs + cdotT<T>(k, R.gjs0, R.gjs1, R.gjs2); });
    // m2 applied to J, u, g
    const T aJ0 = mxx * J0 + mxy * J1 + mxz * J2v, aJ1 = mxy * J0 + myy * J1 + myz * J2v,
            aJ2 = mxz * J0 + myz * J1 + mzz * J2v;
    const T ag0 = mxx * g[0] + mxy * g[1] + mxz * g[2], ag1 = mxy * g[0] + myy * g[1] + myz * g[2],
            ag2 = mxz * g[0] + myz * g[1] + mzz * g[2];
    const T au0 = mxx * u0 + mxy * u1 + mxz * u2, au1 = mxy * u0 + myy * u1 + myz * u2,
            au2 = mxz * u0 + myz * u1 + mzz * u2;
    const T JmJ = J0 * aJ0 + J1 * aJ1 + J2v * aJ2;
    const T quad = T(4.5) * JmJ - T(1.5) * JJ * m0;            // sum t phi (4.5 (c.J)^2 - 1.5 J.J)
    // sum phi_k feq_k - sum phi_k f_k
    T gom = rb * m0 + T(3) * (m1x * J0 + m1y * J1 + m1z * J2v) + r * quad - sphf;
    const T sh = omega * m0;                                       // sum t_k h_k, h = omega phi
    T gr = omega * quad;
    T gJ0 = omega * (T(3) * m1x + T(9) * r * aJ0), gJ1 = omega * (T(3) * m1y + T(9) * r * aJ1),
      gJ2 = omega * (T(3) * m1z + T(9) * r * aJ2);
    const T gpre = T(3) * (m1x * g[0] + m1y * g[1] + m1z * g[2]) - T(3) * ug * m0 +
                   T(9) * (u0 * ag0 + u1 * ag1 + u2 * ag2);
    const T swp = pre * m0;                                        // sum t_k pre phi_k
    T gu0 = T(9) * pre * ag0, gu1 = T(9) * pre * ag1, gu2 = T(9) * pre * ag2;
    T gg0 = pre * (T(3) * m1x + T(9) * au0), gg1 = pre * (T(3) * m1y + T(9) * au1),
      gg2 = pre * (T(3) * m1z + T(9) * au2);
    // the k-independent parts: -3 r J (sum t h), -3 g (sum t pre phi), -3 u (sum t pre phi)
    gJ0 -= T(3) * r * sh * J0; gJ1 -= T(3) * r * sh * J1; gJ2 -= T(3) * r * sh * J2v;
    gu0 -= T(3) * swp * g[0]; gu1 -= T(3) * swp * g[1]; gu2 -= T(3) * swp * g[2];
    gg0 -= T(3) * swp * u0; gg1 -= T(3) * swp * u1; gg2 -= T(3) * swp * u2;
    // pre = (1 - omega/2) rho
    gom -= T(0.5) * rho * gpre;
    T grho = (T(1) - T(0.5) * omega) * gpre;
    // u = J r
    gJ0 += r * gu0; gJ1 += r * gu1; gJ2 += r * gu2;
    gr += J0 * gu0 + J1 * gu1 + J2v * gu2;
    // J = j + rho g / 2
    grho += T(0.5) * (g[0] * gJ0 + g[1] * gJ1 + g[2] * gJ2);
    gg0 += T(0.5) * rho * gJ0; gg1 += T(0.5) * rho * gJ1; gg2 += T(0.5) * rho * gJ2;
    grho -= r * r * gr;
    R.grb = sh + grho;
    R.gJ0 = gJ0; R.gJ1 = gJ1; R.gJ2 = gJ2;
    gtau -= gom * omega * omega;   // omega = 1/tau
    gg[0] += gg0; gg[1] += gg1; gg[2] += gg2;
    return R;
}

// Warp-segmented sum of six values per particle slot into out[key][6]
// (consecutive cells mostly share the owner).  All 32 lanes must call.
template <typename T>
__device__ __forceinline__ void reduce6(int key, T (&v)[6], double* __restrict__ out) {
    const unsigned solid = __ballot_sync(FULLMASK, key >= 0);
    if (solid == 0u) return;
    const int lane = threadIdx.x & 31;
    const int prevKey = __shfl_up_sync(FULLMASK, key, 1);
    const bool head = (lane == 0) || (prevKey != key);
    const unsigned heads = __ballot_sync(FULLMASK, head);
    const int segStart = 31 - __clz(heads & (FULLMASK >> (31 - lane)));
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const T o = __shfl_up_sync(FULLMASK, v[q], d);
            if (lane - d >= segStart) v[q] += o;
        }
    }
    const int nextKey = __shfl_down_sync(FULLMASK, key, 1);
    const bool tail = (lane == 31) || (nextKey != key);
    if (tail && key >= 0)
#pragma unroll
        for (int q = 0; q < 6; ++q) atomicAdd(out + 6 * (size_t)key + q, (double)v[q]);
}

// PER: every axis periodic (no wall cases in the neighbour lookups).
template <typename T, bool PER>
__global__ void __launch_bounds__(ADJ_THREADS, sizeof(T) == 4 ? 2 : 1) k_adjoint_step(const AdjointArgs<T> A) {
    __shared__ double s_red[ADJ_THREADS / 32][4];
    const Geom g = A.g;
    const size_t N = g.N;
    T gtau = T(0), gg[3] = {T(0), T(0), T(0)};   // per-thread sums, widened once
    // one warp per 64-cell run of a z-row, in two passes of 32 cells: rows * runs
    // < 2^31 (nx * ny < 2^31 is checked at creation), so all index arithmetic
    // stays in 32 bits.  The run's solid cells are taken first (pass 0 holds as
    // many as fit): a pass with a solid cell runs the solid cells' path for every
    // lane, so gathering them leaves more passes on the fluid path.  A cell's
    // result does not depend on its pass.
    const int lane = threadIdx.x & 31;
    const int nzc = (g.nz + 63) >> 6;
    const long long nchunks = (long long)g.nx * g.ny * nzc;
    const long long wstride = (long long)gridDim.x * (ADJ_THREADS / 32);
    for (long long q = (long long)blockIdx.x * (ADJ_THREADS / 32) + (threadIdx.x >> 5); q < nchunks; q += wstride) {
        const int qi = (int)q;   // runs of 64 cells: < 2^31 for any lattice that fits in memory
        const int row = qi / nzc;
        const int zb = (qi - row * nzc) * 64;
        const int len = min(64, g.nz - zb);
        const size_t rowc = (size_t)row * g.nz + zb;
        const uint32_t wl0 = lane < len ? A.vox[rowc + lane] : 0u;
        const uint32_t wl1 = lane + 32 < len ? A.vox[rowc + lane + 32] : 0u;
        const unsigned sol0 = __ballot_sync(FULLMASK, (wl0 & VOX_NMASK) != 0u);
        const unsigned sol1 = __ballot_sync(FULLMASK, (wl1 & VOX_NMASK) != 0u);
        const unsigned flu0 = __ballot_sync(FULLMASK, lane < len) & ~sol0;
        const unsigned flu1 = __ballot_sync(FULLMASK, lane + 32 < len) & ~sol1;
        const int ns0 = __popc(sol0), ns = ns0 + __popc(sol1);
        const int nf0 = __popc(flu0), nf = nf0 + __popc(flu1);
#pragma unroll 1
        for (int pass = 0; pass < 2; ++pass) {
            const int slot_l = 32 * pass + lane;
            int jr = -1;   // the cell of the run this lane takes in this pass
            if (slot_l < ns) jr = slot_l < ns0 ? nth_bit(sol0, slot_l) : 32 + nth_bit(sol1, slot_l - ns0);
            else if (slot_l - ns < nf)
                jr = slot_l - ns < nf0 ? nth_bit(flu0, slot_l - ns) : 32 + nth_bit(flu1, slot_l - ns - nf0);
            const bool general = ns > 32 * pass;   // warp-uniform: the pass holds a solid cell
            const int z = zb + jr;
            int key = -1;
            T pv[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
            if (jr >= 0) {
                const int x = row / g.ny;
                const int y = row - x * g.ny;
                const size_t c = (size_t)row * g.nz + z;
                // neighbour coordinates (-1 beyond a wall) and the nine row offsets
                const bool p0 = PER || g.per[0], p1 = PER || g.per[1], p2 = PER || g.per[2];
                const int xs[3] = {x > 0 ? x - 1 : (p0 ? g.nx - 1 : -1), x, x < g.nx - 1 ? x + 1 : (p0 ? 0 : -1)};
                const int ys[3] = {y > 0 ? y - 1 : (p1 ? g.ny - 1 : -1), y, y < g.ny - 1 ? y + 1 : (p1 ? 0 : -1)};
                const int zs[3] = {z > 0 ? z - 1 : (p2 ? g.nz - 1 : -1), z, z < g.nz - 1 ? z + 1 : (p2 ? 0 : -1)};
                long long rowoff[9];
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int b = 0; b < 3; ++b)
                        rowoff[3 * a + b] =
                            (PER || (xs[a] >= 0 && ys[b] >= 0)) ? ((long long)xs[a] * g.ny + ys[b]) * g.nz : -1;
                // cell x + (dx, dy, dz) as a linear index, or -1 beyond a wall
                auto nb = [&](int dx, int dy, int dz) -> long long {
                    const long long r = rowoff[3 * (dx + 1) + dy + 1];
                    const int zz = zs[dz + 1];
                    return (PER || (r >= 0 && zz >= 0)) ? r + zz : -1;
                };
                T f[Q], mu[Q];
                if (A.phase == 0) {
#pragma unroll
                    for (int k = 0; k < Q; ++k) f[k] = A.f[(size_t)k * N + c];
                } else {
                    // odd layout: f_k(x) in slot (opp k, x - c_k), or (k, x) when x - c_k is beyond a wall
                    f[0] = A.f[c];
#pragma unroll
                    for (int k = 1; k < Q; ++k) {
                        const long long s2 = nb(-cx(k), -cy(k), -cz(k));
                        f[k] = s2 >= 0 ? A.f[(size_t)opp(k) * N + (size_t)s2] : A.f[(size_t)k * N + c];
                    }
                }
                // transpose of push streaming: mu_k = lambda_k(x + c_k), or lambda_opp k(x) beyond a wall
#pragma unroll
                for (int k = 0; k < Q; ++k) {
                    const long long s2 = k == 0 ? (long long)c : nb(cx(k), cy(k), cz(k));
                    mu[k] = s2 >= 0 ? A.lam_in[(size_t)k * N + (size_t)s2] : A.lam_in[(size_t)opp(k) * N + c];
                }
                const uint32_t w = A.vox[c];
                int n = min((int)(w & VOX_NMASK), 125);
                T uP[3] = {T(0), T(0), T(0)}, a[3] = {T(0), T(0), T(0)}, d[3] = {T(0), T(0), T(0)};
                T B = T(0), dBdtau = T(0);
                int slot = -1;
                if (n > 0) {
                    const int tag = (int)(w >> VOX_NBITS);
                    slot = tag <= A.max_tag ? A.tag2slot[tag] : -1;
                    if (slot < 0 || slot >= A.nslot) {
                        atomicOr(A.err, 0x8u);   // LBDEM_DEVERR_UNMAPPED_TAG
                        slot = -1;
                    } else {
                        const double* p = A.rec + (size_t)slot * REC_STRIDE;
                        // arm d = cell - centre, minimum image as in the force arm
                        // (src/ibProcessors3D.hh:230-243); the float form takes the
                        // centre's hi/lo split as the forward pass does
                        if (sizeof(T) == 8) {
                            d[0] = T((double)x - p[0]); d[1] = T((double)y - p[1]); d[2] = T((double)z - p[2]);
                        } else {
                            const float4* q4 = reinterpret_cast<const float4*>(A.xpf + (size_t)slot * XPF_STRIDE);
                            const float4 hq = q4[0], lq = q4[1];
                            d[0] = T(((float)x - hq.x) - hq.w);
                            d[1] = T(((float)y - hq.y) - lq.x);
                            d[2] = T(((float)z - hq.z) - lq.y);
                        }
                        const int ext[3] = {g.nx, g.ny, g.nz};
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            const int h = ext[q] / 2;
                            if (d[q] > T(h)) d[q] -= T(ext[q]);
                            else if (d[q] < T(-h)) d[q] += T(ext[q]);
                        }
                        const T v0 = T(p[3]), v1 = T(p[4]), v2 = T(p[5]);
                        const T w0 = T(p[6]), w1 = T(p[7]), w2 = T(p[8]);
                        // uP = v + w x d (setValues, src/ibProcessors3D.hh:163-174)
                        uP[0] = v0 + (w1 * d[2] - w2 * d[1]);
                        uP[1] = v1 + (-w0 * d[2] + w2 * d[0]);
                        uP[2] = v2 + (w0 * d[1] - w1 * d[0]);
                        const double* wgt = A.w + (size_t)slot * 6;
                        const T wf0 = T(wgt[0]), wf1 = T(wgt[1]), wf2 = T(wgt[2]);
                        const T wt0 = T(wgt[3]), wt1 = T(wgt[4]), wt2 = T(wgt[5]);
                        // dL/dF_cell = w_F + w_T x d
                        a[0] = wf0 + (wt1 * d[2] - wt2 * d[1]);
                        a[1] = wf1 + (wt2 * d[0] - wt0 * d[2]);
                        a[2] = wf2 + (wt0 * d[1] - wt1 * d[0]);
                        B = A.btab[n];
                        const T sf = T(1.0 / 125.0) * T(n), den = (T(1) - sf) + (A.tauT - T(0.5));
                        dBdtau = n < 125 ? sf * (T(1) - sf) / (den * den) : T(0);
                    }
                }
                if (n > 0 && slot < 0) n = 0;
                T guP[3];
                const T gvec[3] = {A.g3[0], A.g3[1], A.g3[2]};
                const CellAdj<T> R = adjoint_cell<T>(f, mu, n, general, B, dBdtau, uP, a, A.omega, gvec, guP, gtau, gg);
                const T om1 = n == 125 ? T(1) : T(1) - A.omega;
                if (!general) {   // fluid cells only: phi = mu, no solid terms
#pragma unroll
                    for (int k = 0; k < Q; ++k)
                        A.lam_out[(size_t)k * N + c] = om1 * mu[k] + (R.grb + cdotT<T>(k, R.gJ0, R.gJ1, R.gJ2));
                } else {
                    // the fluid path's expression plus the solid terms (exactly zero for a fluid cell)
#pragma unroll
                    for (int k = 0; k < Q; ++k) {
                        const T phi = R.sB * mu[k] + R.grbs + cdotT<T>(k, R.gjs0, R.gjs1, R.gjs2);
                        T l = om1 * phi + (R.grb + cdotT<T>(k, R.gJ0, R.gJ1, R.gJ2));
                        l += R.B * mu[opp(k)] + T(2) * R.B * cdotT<T>(k, a[0], a[1], a[2]);
                        A.lam_out[(size_t)k * N + c] = l;
                    }
                }
                if (slot >= 0) {
                    key = slot;
                    pv[0] = guP[0]; pv[1] = guP[1]; pv[2] = guP[2];
                    // d/dw of w x d: d x guP
                    pv[3] = d[1] * guP[2] - d[2] * guP[1];
                    pv[4] = d[2] * guP[0] - d[0] * guP[2];
                    pv[5] = d[0] * guP[1] - d[1] * guP[0];
                }
            }
            reduce6(key, pv, A.gvel);
        }
    }
    // block sums of d/dg and d/dtau, one atomic per block and value
    const int warp = threadIdx.x >> 5;
    double v4[4] = {(double)gg[0], (double)gg[1], (double)gg[2], (double)gtau};
#pragma unroll
    for (int q = 0; q < 4; ++q)
        for (int o = 16; o > 0; o >>= 1) v4[q] += __shfl_down_sync(FULLMASK, v4[q], o);
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < 4; ++q) s_red[warp][q] = v4[q];
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0;
        for (int k = 0; k < ADJ_THREADS / 32; ++k) s += s_red[k][threadIdx.x];
        atomicAdd(A.gglob + threadIdx.x, s);
    }
}

// loss += sum_p w[p] . (F_p, T_p) for one step (ft: F (3 nslot) then T (3 nslot)).
__global__ void k_loss_step(const double* __restrict__ ft, const double* __restrict__ w, int n, int nslot,
                            double* __restrict__ loss) {
    double s = 0.0;
    for (int p = threadIdx.x; p < n; p += blockDim.x)
#pragma unroll
        for (int q = 0; q < 3; ++q)
            s += w[6 * (size_t)p + q] * ft[3 * (size_t)p + q] + w[6 * (size_t)p + 3 + q] * ft[3 * (size_t)nslot + 3 * (size_t)p + q];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(FULLMASK, s, o);
    __shared__ double part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += part[k];
        *loss += t;
    }
}

}  // namespace

template <typename T>
cudaError_t launch_adjoint_step(const AdjointArgs<T>& a, cudaStream_t s) {
    static std::atomic<int> cached[LBDEM_MAX_DEVICES];   // per device: grid size
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= LBDEM_MAX_DEVICES) return cudaErrorInvalidDevice;
    int blocks = cached[dev].load(std::memory_order_relaxed);
    if (blocks == 0) {
        int sms = 0, per_sm = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adjoint_step<T, false>, ADJ_THREADS, 0);
        if (e != cudaSuccess) return e;
        blocks = sms * (per_sm > 0 ? per_sm : 1);
        cached[dev].store(blocks, std::memory_order_relaxed);
    }
    const size_t need = (a.g.N + ADJ_THREADS - 1) / ADJ_THREADS;
    const unsigned grid = (unsigned)(need < (size_t)blocks ? (need > 0 ? need : 1) : (size_t)blocks);
    if (a.g.per[0] && a.g.per[1] && a.g.per[2])
        k_adjoint_step<T, true><<<grid, ADJ_THREADS, 0, s>>>(a);
    else
        k_adjoint_step<T, false><<<grid, ADJ_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_loss_step(const double* ft, const double* w, int n, int nslot, double* loss, cudaStream_t s) {
    k_loss_step<<<1, 256, 0, s>>>(ft, w, n, nslot, loss);
    return cudaGetLastError();
}

template cudaError_t launch_adjoint_step<float>(const AdjointArgs<float>&, cudaStream_t);
template cudaError_t launch_adjoint_step<double>(const AdjointArgs<double>&, cudaStream_t);

}  // namespace lbdem
