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
// One thread per cell, a block spans 128 consecutive cells of one z-row, so
// every population access of a warp is one contiguous 128-float / 256-double
// segment (shifted by one element for c_z != 0 in the odd phase).
#include "lbdem_internal.h"

namespace lbdem {
namespace {

constexpr unsigned FULL = 0xffffffffu;

// 1/x rounded to nearest (identical to the IEEE division 1/x).
__device__ __forceinline__ float recip(float x) { return __frcp_rn(x); }
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

// BGK relaxation towards the second-order equilibrium
// feq_i = t_i [rhoBar + 3 c.j + invRho (4.5 (c.j)^2 - 1.5 j.j)], written per
// opposite pair (feq_i and feq_{i+9} differ only in the sign of 3 c.j).
// With FORCE the Guo scheme is used (equilibrium momentum j + rho g / 2 plus
// the forcing term t_i (1 - omega/2) rho [3 (c - u).g + 9 (c.u)(c.g)]).
template <typename T, bool FORCE>
__device__ __forceinline__ void bgk(T (&f)[Q], T omega, T gx, T gy, T gz) {
    T rhoBar, jx, jy, jz;
    moments(f, rhoBar, jx, jy, jz);
    const T rho = T(1) + rhoBar;
    const T invRho = recip(rho);
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

// PSM collision of a cell with n > 0 solid sub-cells,
// src/ibCompositeDynamics3D.hh:130-203.  n == 125 is the full-solid branch
// (no BGK, B = 1, which reduces the weighted update to fPre + bb exactly).
template <typename T, bool FORCE>
__device__ __forceinline__ void psm(T (&f)[Q], int n, T up0, T up1, T up2, T B, T omega,
                                    T gx, T gy, T gz, T& Fx, T& Fy, T& Fz) {
    T fPre[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) fPre[i] = f[i];
    if (n < 125) bgk<T, FORCE>(f, omega, gx, gy, gz);
    T rhoBar, jx, jy, jz;
    moments(f, rhoBar, jx, jy, jz);                  // post-collision moments, :146-148
    const T rho = T(1) + rhoBar;
    const T invRho = recip(rho);
    const T ux = up0 * rho, uy = up1 * rho, uz = up2 * rho;   // uPart (1 + rhoBar), :154
    const T q45 = T(4.5) * invRho;
    const T baseE = rhoBar - T(1.5) * invRho * (jx * jx + jy * jy + jz * jz);
    const T baseS = rhoBar - T(1.5) * invRho * (ux * ux + uy * uy + uz * uz);
    const T omB = T(1) - B;
    f[0] = fPre[0] + omB * (f[0] - fPre[0]) + B * (T(wt(0)) * baseE - T(wt(0)) * baseS);
    Fx = T(0); Fy = T(0); Fz = T(0);
#pragma unroll
    for (int i = 1; i <= 9; ++i) {
        const int o = i + 9;
        const T t = T(wt(i));
        const T cj = cdot(i, jx, jy, jz);
        const T cu = cdot(i, ux, uy, uz);
        const T eE = baseE + q45 * cj * cj, sE = T(3) * cj;
        const T eS = baseS + q45 * cu * cu, sS = T(3) * cu;
        const T fEq_i = t * (eE + sE), fEq_o = t * (eE - sE);
        const T fEqS_i = t * (eS + sS), fEqS_o = t * (eS - sS);
        const T bb = B * ((fPre[o] - fEq_o) - (fPre[i] - fEqS_i));
        const T bbOpp = B * ((fPre[i] - fEq_i) - (fPre[o] - fEqS_o));
        f[i] = fPre[i] + omB * (f[i] - fPre[i]) + bb;
        f[o] = fPre[o] + omB * (f[o] - fPre[o]) + bbOpp;
        const T d = bb - bbOpp;                      // F -= c_i (bb - bbOpp), :172-174
        if (cx(i) > 0) Fx -= d; else if (cx(i) < 0) Fx += d;
        if (cy(i) > 0) Fy -= d; else if (cy(i) < 0) Fy += d;
        if (cz(i) > 0) Fz -= d; else if (cz(i) < 0) Fz += d;
    }
}

__device__ __forceinline__ int wrap_minus(int v, int n, int per) { return v > 0 ? v - 1 : (per ? n - 1 : -1); }
__device__ __forceinline__ int wrap_plus(int v, int n, int per) { return v < n - 1 ? v + 1 : (per ? 0 : -1); }
__device__ __forceinline__ int pick(int c, int m, int v, int p) { return c < 0 ? m : (c > 0 ? p : v); }

template <typename T, bool ODD, bool FORCE>
__global__ void __launch_bounds__(COLLIDE_BLOCK)
k_collide_stream(const CollideArgs<T> a) {
    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const size_t N = a.g.N;
    const int row = blockIdx.x;
    const int x = row / ny;
    const int y = row - x * ny;
    const int z = blockIdx.y * COLLIDE_BLOCK + threadIdx.x;
    const bool valid = z < nz;
    const size_t c = ((size_t)x * ny + y) * nz + (valid ? z : 0);
    T* __restrict__ F = a.f;

    // Per-cell force and torque, summed over a warp in the population type
    // (double for the FP64 form) and accumulated per particle in double.
    int key = -1;
    T v[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};

    if (valid) {
        // neighbour coordinates along each axis (-1: beyond a wall)
        int xm = 0, xp = 0, ym = 0, yp = 0, zm = 0, zp = 0;
        if (ODD) {
            xm = wrap_minus(x, nx, a.g.per[0]); xp = wrap_plus(x, nx, a.g.per[0]);
            ym = wrap_minus(y, ny, a.g.per[1]); yp = wrap_plus(y, ny, a.g.per[1]);
            zm = wrap_minus(z, nz, a.g.per[2]); zp = wrap_plus(z, nz, a.g.per[2]);
        }
        auto nb = [&](int i) -> long long {
            const int X = pick(cx(i), xm, x, xp), Y = pick(cy(i), ym, y, yp), Z = pick(cz(i), zm, z, zp);
            if (X < 0 || Y < 0 || Z < 0) return -1;
            return ((long long)X * ny + Y) * nz + Z;
        };

        T f[Q];
        if (!ODD) {
#pragma unroll
            for (int i = 0; i < Q; ++i) f[i] = __ldcs(F + (size_t)i * N + c);
        } else {
            f[0] = __ldcs(F + c);
#pragma unroll
            for (int i = 1; i < Q; ++i) {
                const long long s = nb(opp(i));
                f[i] = s >= 0 ? __ldcs(F + (size_t)opp(i) * N + (size_t)s) : __ldcs(F + (size_t)i * N + c);
            }
        }

        const uint32_t w = __ldg(a.vox + c);
        const int n = min((int)(w & VOX_NMASK), 125);
        const T omega = T(a.omega);
        const T gx = T(a.g3[0]), gy = T(a.g3[1]), gz = T(a.g3[2]);
        T Fx = T(0), Fy = T(0), Fz = T(0);
        if (n == 0) {
            bgk<T, FORCE>(f, omega, gx, gy, gz);
        } else {
            const T up0 = __ldg(a.up + c), up1 = __ldg(a.up + N + c), up2 = __ldg(a.up + 2 * N + c);
            const T B = T(__ldg(a.btab + n));
            psm<T, FORCE>(f, n, up0, up1, up2, B, omega, gx, gy, gz, Fx, Fy, Fz);
        }

        if (!ODD) {
#pragma unroll
            for (int i = 0; i < Q; ++i) __stcs(F + (size_t)opp(i) * N + c, f[i]);
        } else {
            __stcs(F + c, f[0]);
#pragma unroll
            for (int i = 1; i < Q; ++i) {
                const long long d = nb(i);
                if (d >= 0) __stcs(F + (size_t)i * N + (size_t)d, f[i]);
                else __stcs(F + (size_t)opp(i) * N + c, f[i]);
            }
        }

        if (a.cf) {
            a.cf[c] = Fx; a.cf[N + c] = Fy; a.cf[2 * N + c] = Fz;
        }

        if (n > 0) {
            const int tag = (int)(w >> VOX_NBITS);
            const int slot = tag <= a.max_tag ? __ldg(a.tag2slot + tag) : -1;
            if (slot < 0 || slot >= a.nslot) {
                atomicOr(a.err, 0x8u);   // LBDEM_DEVERR_UNMAPPED_TAG
            } else {
                key = slot;
                // torque arm with the minimum image of src/ibProcessors3D.hh:230-243
                T dx, dy, dz;
                if (sizeof(T) == 8) {
                    const double* p = a.rec + (size_t)slot * REC_STRIDE;
                    dx = T((double)x - __ldg(p + 0));
                    dy = T((double)y - __ldg(p + 1));
                    dz = T((double)z - __ldg(p + 2));
                } else {
                    // centre = hi + lo in float: (x - hi) - lo is the arm to ~1 ulp
                    const float4* p = reinterpret_cast<const float4*>(a.xpf) + 2 * (size_t)slot;
                    const float4 h = __ldg(p), l = __ldg(p + 1);
                    dx = T(((float)x - h.x) - h.w);
                    dy = T(((float)y - h.y) - l.x);
                    dz = T(((float)z - h.z) - l.y);
                }
                const int hx = nx / 2, hy = ny / 2, hz = nz / 2;
                if (dx > T(hx)) dx -= T(nx); else if (dx < T(-hx)) dx += T(nx);
                if (dy > T(hy)) dy -= T(ny); else if (dy < T(-hy)) dy += T(ny);
                if (dz > T(hz)) dz -= T(nz); else if (dz < T(-hz)) dz += T(nz);
                v[0] = Fx; v[1] = Fy; v[2] = Fz;
                v[3] = dy * Fz - dz * Fy;
                v[4] = -dx * Fz + dz * Fx;
                v[5] = dx * Fy - dy * Fx;
            }
        }
    }

    // Warp-segmented sum over runs of equal particle slot (consecutive cells
    // along z mostly belong to the same sphere), one set of double atomics per run.
    if (__ballot_sync(FULL, key >= 0) == 0u) return;
    const int lane = threadIdx.x & 31;
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
        atomicAdd(Fp + 0, (double)v[0]); atomicAdd(Fp + 1, (double)v[1]); atomicAdd(Fp + 2, (double)v[2]);
        atomicAdd(Tp + 0, (double)v[3]); atomicAdd(Tp + 1, (double)v[4]); atomicAdd(Tp + 2, (double)v[5]);
    }
}

template <typename T, bool ODD, bool FORCE>
cudaError_t launch_one(const CollideArgs<T>& a, cudaStream_t s) {
    dim3 grid((unsigned)((size_t)a.g.nx * a.g.ny), (unsigned)((a.g.nz + COLLIDE_BLOCK - 1) / COLLIDE_BLOCK));
    k_collide_stream<T, ODD, FORCE><<<grid, COLLIDE_BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t launch_collide_stream(const CollideArgs<T>& a, bool odd, bool force, cudaStream_t s) {
    if (odd) return force ? launch_one<T, true, true>(a, s) : launch_one<T, true, false>(a, s);
    return force ? launch_one<T, false, true>(a, s) : launch_one<T, false, false>(a, s);
}

template cudaError_t launch_collide_stream<float>(const CollideArgs<float>&, bool, bool, cudaStream_t);
template cudaError_t launch_collide_stream<double>(const CollideArgs<double>&, bool, bool, cudaStream_t);

}  // namespace lbdem
