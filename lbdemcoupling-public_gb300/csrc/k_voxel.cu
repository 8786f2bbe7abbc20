// K2: sphere voxelization, bit-exact with SetSingleSphere3D.
//
// Replaces setSpheresOnLattice -> SetSingleSphere3D::process for every sphere
// (src/ibDataExchangeWrappers3D.hh:33-146, src/ibProcessors3D.hh:53-184).
//
// Order.  The reference applies spheres one after another, and a cell's new
// state depends on its previous state and on the order of the spheres whose
// bounding box covers it (decFlag, src/ibProcessors3D.hh:85-105).  The GPU
// keeps that order per cell: every sphere is binned to the 8^3-cell tiles its
// box overlaps, each tile's bin is sorted by sphere index in shared memory, and
// every cell folds the sorted list through the same state machine.  Cells are
// independent, so the result equals the sequential sweep.  A bin holds
// TILE_BIN spheres; a tile overlapped by more re-collects its spheres by
// testing every box (slow but exact).
//
// Exactness of the sub-cell count.  The reference decides, in IEEE double,
//   dist = (dx^2 + dy^2) + dz^2  against (r + sqrt(3.1)/2)^2 and (r - sqrt(3.1)/2)^2,
//   (xs_i + ys_j) + zs_k < r^2   for the 125 sub-cell centres of shell cells.
// GB300 executes double arithmetic at two lanes per clock per SM, so each
// comparison is first made in float with a margin M = 2^-19 (r + 4)^2.  For a
// cell inside the box (|dx| < r + 3, centre split x = xh + xl with |x| < 2^24)
// the float value differs from the double one by at most 27 u (r + 3.5)^2,
// u = 2^-24 (sample sums), resp. 22 u (r + 3.2)^2 (dist), so a float result
// farther than M from the threshold decides the comparison as the double
// computation does.  Only comparisons inside the band are evaluated with the
// reference's double sequence (__dadd_rn/__dmul_rn: no fused multiply-add).
// Counts n and owner tags are identical to the sequential CPU result; the
// FP64 form also reproduces the particle surface velocity bit for bit.
#include "lbdem_internal.h"

#include <climits>

namespace lbdem {
namespace {

constexpr unsigned FULL_MASK = 0xffffffffu;

constexpr double SQRT3HALF = 0.8803408430829505;  // sqrt(3.1)/2, src/ibProcessors3D.hh:128-130
// -0.5 + (i + 0.5) * (1./5.), src/ibProcessors3D.hh:141-147, evaluated in double:
__device__ __forceinline__ double sub_delta(int i) {
    return i == 0 ? -0.4 : i == 1 ? -0.19999999999999996 : i == 2 ? 0.0 : i == 3 ? 0.20000000000000007 : 0.4;
}
__device__ __forceinline__ float sub_delta_f(int i) {
    return i == 0 ? -0.4f : i == 1 ? -0.2f : i == 2 ? 0.0f : i == 3 ? 0.2f : 0.4f;
}

// Single operations with round-to-nearest and no contraction into fused
// multiply-adds (results independent of how the compiler schedules a kernel).
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }

// Region of a cell against the early-out thresholds in the reference's double
// arithmetic: 0 outside (dist > rp2), 1 inside (dist < rm2), 2 shell.
__device__ __noinline__ int region_exact(int X, int Y, int Z, const SphereDev& s) {
    const double dx = __dsub_rn((double)X, s.x[0]);
    const double dy = __dsub_rn((double)Y, s.x[1]);
    const double dz = __dsub_rn((double)Z, s.x[2]);
    const double dist = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    if (dist > s.rp2) return 0;
    if (dist < s.rm2) return 1;
    return 2;
}

__device__ __forceinline__ int tiles_along(int n) { return (n + TILE - 1) / TILE; }

// Per sphere: bounding box (double -> integer truncation toward zero,
// src/ibProcessors3D.h:43-45) intersected with the lattice
// (src/ibDataExchangeWrappers3D.hh:127-133), thresholds, the float split of
// the centre, and the tag -> lowest list index map (LAMMPS atom->map keeps the
// owned atom, which precedes its ghost images).  Returns the cell box that the
// sphere's tiles are binned by (lo > hi: the sphere reaches no cell).
__device__ __forceinline__ void prepare_sphere(const double* __restrict__ p, int i, int il, const Geom& g,
                                               int max_tag, double max_radius, SphereDev* __restrict__ sph,
                                               SphereFast* __restrict__ fast, float* __restrict__ xpf,
                                               int* __restrict__ tag2slot, unsigned* __restrict__ err, int box[6]) {
    SphereDev s;
    SphereFast q;
    for (int d = 0; d < 3; ++d) { s.x[d] = p[d]; s.v[d] = p[3 + d]; s.w[d] = p[6 + d]; }
    s.r = p[9];
    const double tagd = p[10];
    s.valid = 1;
    if (!(tagd >= 1.0 && tagd <= (double)max_tag)) {
        atomicOr(err, 0x4u);  // LBDEM_DEVERR_TAG_RANGE
        s.valid = 0;
        s.tag = 0;
    } else {
        s.tag = (int)tagd;
    }
    if (!(s.r > 0.0 && s.r <= max_radius)) {
        atomicOr(err, 0x10u);  // LBDEM_DEVERR_RADIUS
        s.valid = 0;
    }
    const int dims[3] = {g.nx, g.ny, g.nz};
    for (int d = 0; d < 3; ++d) {
        const double xd = s.x[d];
        q.xh[d] = 0.f; q.xl[d] = 0.f;
        // |x| < 2^24 keeps the integer conversions defined and the float split
        // accurate; a sphere farther out cannot reach the lattice.
        if (!(xd > -16777216.0 && xd < 16777216.0)) { s.valid = 0; s.lo[d] = 1; s.hi[d] = 0; continue; }
        q.xh[d] = (float)xd;
        q.xl[d] = (float)(xd - (double)q.xh[d]);
        long long lo = (long long)(__dsub_rn(__dsub_rn(xd, s.r), 2.0));
        long long hi = (long long)(__dadd_rn(__dadd_rn(xd, s.r), 2.0));
        if (lo < 0) lo = 0;
        if (hi > dims[d] - 1) hi = dims[d] - 1;
        s.lo[d] = (int)(lo < (long long)dims[d] ? lo : dims[d]);
        s.hi[d] = (int)(hi > -1 ? hi : -1);
        if (s.lo[d] > s.hi[d]) s.valid = 0;
    }
    const double rp = __dadd_rn(s.r, SQRT3HALF), rm = __dsub_rn(s.r, SQRT3HALF);
    s.rp2 = __dmul_rn(rp, rp);
    s.rm2 = __dmul_rn(rm, rm);
    s.rsq = __dmul_rn(s.r, s.r);
    q.rp2 = (float)s.rp2;
    q.rm2 = (float)s.rm2;
    q.rsq = (float)s.rsq;
    const float r4 = (float)s.r + 4.0f;
    q.margin = ldexpf(r4 * r4, -19);
    for (int d = 0; d < 3; ++d) {
        q.lo[d] = s.valid ? s.lo[d] : 1;
        q.hi[d] = s.valid ? s.hi[d] : 0;
        q.v[d] = (float)s.v[d];
        q.w[d] = (float)s.w[d];
        box[2 * d] = q.lo[d];
        box[2 * d + 1] = q.hi[d];
    }
    q.tag = s.tag;
    q.pad = 0;
    sph[i] = s;
    fast[i] = q;
    float4* xp = reinterpret_cast<float4*>(xpf + (size_t)i * XPF_STRIDE);
    xp[0] = make_float4(q.xh[0], q.xh[1], q.xh[2], q.xl[0]);
    xp[1] = make_float4(q.xl[1], q.xl[2], q.v[0], q.v[1]);
    xp[2] = make_float4(q.v[2], q.w[0], q.w[1], q.w[2]);
    xp[3] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (s.tag >= 1) atomicMin(tag2slot + s.tag, il);
}

// One warp per sphere: lane 0 prepares the sphere (prepare_sphere), then the
// lanes stride over the tiles its box overlaps and append the sphere to each
// tile's bin (entries past TILE_BIN are dropped; the voxelization of such a
// tile re-collects its spheres; a tile's bin is rank-sorted there, so the
// append order does not matter).  The first sphere of a tile also appends the
// tile to the work list.
// BATCH: slot i belongs to the domain d with soff[d] <= i; slots past the
// domain's particle count are skipped; the map stores domain-local slots.
// ft_zero (may be null): the 6 n force/torque sums of the coming collide-stream
// step, zeroed here instead of by a separate memset launch.  rec_copy (may be
// null, never overlapping rec): receives a copy of the n records.
template <bool BATCH>
__global__ void k_prepare_bin(const double* __restrict__ rec, int n, SphereDev* __restrict__ sph,
                              SphereFast* __restrict__ fast, float* __restrict__ xpf, int* __restrict__ tag2slot,
                              unsigned* __restrict__ err, Geom g, int max_tag, double max_radius,
                              const DomView* __restrict__ doms, const int* __restrict__ soff, int ndom,
                              const int* __restrict__ ncur, double* __restrict__ ft_zero,
                              double* __restrict__ rec_copy, int* __restrict__ tile_cnt, int* __restrict__ bins,
                              int* __restrict__ work, int* __restrict__ work_n) {
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n) return;   // warp-uniform from here on
    if (ft_zero && lane < 6) ft_zero[(size_t)lane * n + i] = 0.0;
    int il = i, t0 = 0;
    if (BATCH) {
        const int d = find_domain(soff, ndom, i);
        il = i - __ldg(soff + d);
        if (il >= __ldg(ncur + d)) return;
        g = doms[d].g;
        tag2slot += doms[d].tag0;
        t0 = doms[d].t0;
    }
    const double* p = rec + (size_t)i * REC_STRIDE;
    if (rec_copy && lane < REC_STRIDE) rec_copy[(size_t)i * REC_STRIDE + lane] = p[lane];
    int box[6] = {1, 0, 1, 0, 1, 0};
    if (lane == 0) prepare_sphere(p, i, il, g, max_tag, max_radius, sph, fast, xpf, tag2slot, err, box);
#pragma unroll
    for (int k = 0; k < 6; ++k) box[k] = __shfl_sync(0xffffffffu, box[k], 0);
    if (box[0] > box[1] || box[2] > box[3] || box[4] > box[5]) return;
    const int tx0 = box[0] / TILE, ty0 = box[2] / TILE, tz0 = box[4] / TILE;
    const int ex = box[1] / TILE - tx0 + 1, ey = box[3] / TILE - ty0 + 1, ez = box[5] / TILE - tz0 + 1;
    const int tny = tiles_along(g.ny), tnz = tiles_along(g.nz);
    const int total = ex * ey * ez;
    for (int k = lane; k < total; k += 32) {
        const int kz = k % ez, kr = k / ez;
        const int ky = kr % ey, kx = kr / ey;
        const size_t t = (size_t)t0 + ((size_t)(tx0 + kx) * tny + (ty0 + ky)) * tnz + (tz0 + kz);
        const int pos = atomicAdd(tile_cnt + t, 1);
        if (pos == 0) work[atomicAdd(work_n, 1)] = (int)t;
        if (pos < TILE_BIN) bins[t * TILE_BIN + pos] = il;
    }
}

// Location of population i of cell c in the AA layout (phase = completed steps mod 2).
template <typename T>
__device__ __forceinline__ T* pop_slot(T* f, int i, int x, int y, int z, int phase, const Geom& g) {
    if (phase == 0 || i == 0) return f + (size_t)i * g.N + ((size_t)x * g.ny + y) * g.nz + z;
    // odd layout: f_i(x) sits in slot (opp i, x - c_i), or (i, x) when x - c_i is beyond a wall
    int X = x - cx(i), Y = y - cy(i), Z = z - cz(i);
    bool out = false;
    if (X < 0 || X >= g.nx) { if (g.per[0]) X = (X + g.nx) % g.nx; else out = true; }
    if (Y < 0 || Y >= g.ny) { if (g.per[1]) Y = (Y + g.ny) % g.ny; else out = true; }
    if (Z < 0 || Z >= g.nz) { if (g.per[2]) Z = (Z + g.nz) % g.nz; else out = true; }
    if (out) return f + (size_t)i * g.N + ((size_t)x * g.ny + y) * g.nz + z;
    return f + (size_t)opp(i) * g.N + ((size_t)X * g.ny + Y) * g.nz + Z;
}

// setValues, src/ibProcessors3D.hh:163-174 (com == x for single spheres):
// u = v + omega x (cell - com), in the reference's double operation order.
__device__ __forceinline__ void surface_velocity(const SphereDev& s, int X, int Y, int Z, double& u0, double& u1,
                                                 double& u2) {
    const double dx = __dsub_rn((double)X, s.x[0]);
    const double dy = __dsub_rn((double)Y, s.x[1]);
    const double dz = __dsub_rn((double)Z, s.x[2]);
    u0 = __dadd_rn(s.v[0], __dsub_rn(__dmul_rn(s.w[1], dz), __dmul_rn(s.w[2], dy)));
    u1 = __dadd_rn(s.v[1], __dadd_rn(__dmul_rn(-s.w[0], dz), __dmul_rn(s.w[2], dx)));
    u2 = __dadd_rn(s.v[2], __dsub_rn(__dmul_rn(s.w[0], dy), __dmul_rn(s.w[1], dx)));
}

// Packed pairs of floats for the sample sums.
__device__ __forceinline__ unsigned long long pk2(float a, float b) {
    unsigned long long v;
    asm("mov.b64 %0, {%1, %2};" : "=l"(v) : "f"(a), "f"(b));
    return v;
}
__device__ __forceinline__ unsigned long long add2(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long sub2(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// Sub-cell count of one x-slice (i fixed: 25 of the 125 samples) of a shell
// cell in float, every operation rounded on its own (the error bound of the
// header holds for this form): the sums t = (xs + ys_j) + zs_k are formed two
// at a time in packed f32x2 arithmetic, d = t - r^2 (exact near r^2), and a
// sample is inside when the sign bit of d is set.  *unsure is set when some
// |d| <= M (a sample inside the decision band).
__device__ __forceinline__ int slice_count_fast(float dxf, float dyf, float dzf, int i, float rsq, float M,
                                                bool* unsure) {
    const float ax = __fadd_rn(dxf, sub_delta_f(i));
    const float xs = __fmul_rn(ax, ax);
    float ys[5], zs[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const float d = sub_delta_f(j);
        const float ay = __fadd_rn(dyf, d); ys[j] = __fmul_rn(ay, ay);
        const float az = __fadd_rn(dzf, d); zs[j] = __fmul_rn(az, az);
    }
    const unsigned long long z01 = pk2(zs[0], zs[1]), z23 = pk2(zs[2], zs[3]), r2 = pk2(rsq, rsq);
    unsigned neg = 0u;
    float mind = 3.0e38f;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const float a = __fadd_rn(xs, ys[j]);
        const unsigned long long a2 = pk2(a, a);
        const unsigned long long d01 = sub2(add2(a2, z01), r2), d23 = sub2(add2(a2, z23), r2);
        const float d4 = __fsub_rn(__fadd_rn(a, zs[4]), rsq);
        const unsigned u0 = (unsigned)d01, u1 = (unsigned)(d01 >> 32), u2 = (unsigned)d23, u3 = (unsigned)(d23 >> 32);
        neg += (u0 >> 31) + (u1 >> 31) + (u2 >> 31) + (u3 >> 31) + (__float_as_uint(d4) >> 31);
        mind = fminf(mind, fminf(fminf(fabsf(__uint_as_float(u0)), fabsf(__uint_as_float(u1))),
                                 fminf(fminf(fabsf(__uint_as_float(u2)), fabsf(__uint_as_float(u3))), fabsf(d4))));
    }
    *unsure = !(mind > M);
    return (int)neg;
}

// The same slice with the samples inside the band decided by the reference's
// double sequence ((xs_i + ys_j) + zs_k < r^2, src/ibProcessors3D.hh:141-155).
// Inlined into the count loop (a call there cost its register saves and restores on
// every pass, 0.235 against 0.227 ms; the cell-distance routine region_exact stays out
// of line, inlining it measured slower).
__device__ __forceinline__ int slice_count_resolve(float dxf, float dyf, float dzf, int i, float rsq, float M, int X,
                                                int Y, int Z, const SphereDev& s) {
    const double dx = __dsub_rn((double)X, s.x[0]);
    const double dy = __dsub_rn((double)Y, s.x[1]);
    const double dz = __dsub_rn((double)Z, s.x[2]);
    const double axd = __dadd_rn(dx, sub_delta(i));
    const double xsd = __dmul_rn(axd, axd);
    const float ax = dxf + sub_delta_f(i);
    const float xs = ax * ax;
    const float lo = rsq - M, hi = rsq + M;
    int n = 0;
    for (int j = 0; j < 5; ++j) {
        const float ay = dyf + sub_delta_f(j);
        const float a = xs + ay * ay;
        double ad = 0.0;
        bool have_ad = false;
        for (int k = 0; k < 5; ++k) {
            const float az = dzf + sub_delta_f(k);
            const float t = a + az * az;
            if (t < lo) {
                ++n;
            } else if (t < hi) {
                if (!have_ad) {
                    const double ayd = __dadd_rn(dy, sub_delta(j));
                    ad = __dadd_rn(xsd, __dmul_rn(ayd, ayd));
                    have_ad = true;
                }
                const double azd = __dadd_rn(dz, sub_delta(k));
                n += (__dadd_rn(ad, __dmul_rn(azd, azd)) < s.rsq) ? 1 : 0;
            }
        }
    }
    return n;
}

// ---------------------------------------------------------------------------
// Voxelization, one warp per 8^3 tile.
//
// The tile's cell state (voxel words, and per cell the list index of the
// sphere that last set or cleared it) lives in per-warp shared memory while
// the tile's spheres are applied in list order.  Lane `lane` handles cells
// l = lane + 32 j (j = 0..15): the half x-plane j holds x = j >> 1,
// y = (lane >> 3) + 4 (j & 1), z = lane & 7.  Per sphere (apply_sphere):
//  1  the half-planes that meet the sphere's box are classified in float
//     (outside: n = 0, inside: n = 125, shell); comparisons within the float
//     error band are decided in the reference's double arithmetic; outside and
//     inside cells are folded through decFlag at once, shell cells queued;
//  2  all lanes take the queued cells' sub-cell counts, five x-slices (25
//     samples) per cell, added into per-cell bytes with shared-memory atomics;
//  3  the queued cells are folded through decFlag.
// No block-wide barrier is involved, so the warps of a block work on
// unrelated tiles.  The spheres of a tile come from its bin (at most
// TILE_BIN, put in ascending list order by repeated warp minima), or, for a
// tile whose bin overflowed, from a scan of every sphere's box in list order.
constexpr int VOX_WARPS = 8;                        // warps per block
constexpr int VOX_THREADS = 32 * VOX_WARPS;
constexpr int VOX_STAGE = 32;                       // sphere records staged at a time
constexpr int TOFF_SMEM = 512;                      // batch: domains whose first tiles a CTA keeps
constexpr uint32_t SETTER_ZERO = 0xffffffffu;       // the cell was set to zero (setToZero)
constexpr uint32_t SETTER_KEEP = 0xfffffffeu;       // the cell keeps its state (and velocity)

// Per-warp shared memory.  setter: the list index of the sphere that last set
// the cell in this pass (or SETTER_ZERO / SETTER_KEEP); defv (INIT_VEL): the
// setter code at the cell's last full coverage (defineVelocity), SETTER_ZERO
// + SETTER_KEEP markers as for setter, DEFV_NONE without full coverage.
constexpr uint32_t DEFV_NONE = 0xfffffffdu;
template <bool INIT_VEL>
struct alignas(16) WarpVox {
    SphereFast q[VOX_STAGE];                        // staged sphere records
    int list[TILE_BIN];                             // the tile's spheres in list order
    uint32_t w[TILE_CELLS];                         // voxel words (n | tag << 7)
    uint32_t setter[TILE_CELLS];
    uint32_t defv[INIT_VEL ? TILE_CELLS : 1];
    uint32_t cnt4[TILE_CELLS / 4];                  // shell sub-cell counts, one byte per cell
    uint16_t queue[TILE_CELLS];                     // shell cells of the current sphere
    uint16_t items[5 * 32];                         // x-slices left to count: tile cell << 3 | slice
};

// decFlag, src/ibProcessors3D.hh:85-105 (sf > 0.001 <=> n > 0; sf > sf_old <=>
// n > n_old), for cell l with the sub-cell count n of sphere m.
template <bool INIT_VEL>
__device__ __forceinline__ void fold_cell(WarpVox<INIT_VEL>& S, int l, uint32_t n, uint32_t tag, int m) {
    const uint32_t w = S.w[l];
    const uint32_t nold = w & VOX_NMASK, idold = w >> VOX_NBITS;
    const int dec = (n > 0u ? 1 : 0) + (nold > 0u ? 2 : 0);
    if (dec == 2 && idold == tag) {
        S.w[l] = 0u;
        S.setter[l] = SETTER_ZERO;
    } else if (dec == 1 || (dec == 3 && ((n > nold) || (idold == tag)))) {
        S.w[l] = n | (tag << VOX_NBITS);
        S.setter[l] = (uint32_t)m;
    }
    // dec == 0 is setToZero on a cell that is already empty
    // the velocity the cell holds right after this sphere (src/ibProcessors3D.hh:107-108)
    if (INIT_VEL && n == 125u) S.defv[l] = S.setter[l];
}

// Steps 1-3 above for sphere m (float record q in shared memory) on the tile at
// (X0, Y0, Z0).  Inlined at both sphere sources (an out-of-line routine measured
// 5 % slower: the call's register saves and restores).
template <bool INIT_VEL>
__device__ __forceinline__ void apply_sphere(WarpVox<INIT_VEL>& S, const SphereFast& q, int m,
                                          const SphereDev* __restrict__ sph, int X0, int Y0, int Z0) {
    const int lane = threadIdx.x & 31;
    const int bx0 = max(q.lo[0] - X0, 0), bx1 = min(q.hi[0] - X0, TILE - 1);
    const int by0 = max(q.lo[1] - Y0, 0), by1 = min(q.hi[1] - Y0, TILE - 1);
    const int bz0 = max(q.lo[2] - Z0, 0), bz1 = min(q.hi[2] - Z0, TILE - 1);
    if (bx0 > bx1 || by0 > by1 || bz0 > bz1) return;
    const float M = q.margin, rp2 = q.rp2, rm2 = q.rm2;
    const uint32_t tag = (uint32_t)q.tag;
    const int z = lane & 7, yl = lane >> 3;
    const bool zin = z >= bz0 && z <= bz1;
    const float dzf = ((float)(Z0 + z) - q.xh[2]) - q.xl[2];
    uint8_t* cnt8 = reinterpret_cast<uint8_t*>(S.cnt4);
    const unsigned below = (1u << lane) - 1u;
    int qn = 0;
    // 1: the box's cells of the tile, x-plane by x-plane in the half-planes h
    // (rows y = yl + 4 h) that meet the box's y range.  The squared distance is
    // formed as dx^2 + (dy^2 + dz^2), every rounding explicit, the x-free part
    // once per lane and half-plane.
    const float dz2 = __fmul_rn(dzf, dzf);
    float sh[2];
    bool inh[2], meet[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int y = yl + 4 * h;
        const float dyf = ((float)(Y0 + y) - q.xh[1]) - q.xl[1];
        sh[h] = __fmaf_rn(dyf, dyf, dz2);
        inh[h] = zin && y >= by0 && y <= by1;
        meet[h] = !(4 * h > by1 || 4 * h + 3 < by0);   // warp-uniform
    }
    // A sphere whose shell stays clear of the box's cells in this tile (about half
    // of the (tile, sphere) pairs at r = 8) only clears the cells that hold its tag
    // (decFlag 2, setToZero): the box's squared distance from the centre, formed
    // like a cell's, is more than 2 M beyond (r + sqrt(3.1)/2)^2, so every cell of the
    // box is outside in the reference's double arithmetic too.
    {
        auto gap = [](float lo, float hi) { return fmaxf(0.f, fmaxf(lo, -hi)); };
        const float ex = gap(((float)(X0 + bx0) - q.xh[0]) - q.xl[0], ((float)(X0 + bx1) - q.xh[0]) - q.xl[0]);
        const float ey = gap(((float)(Y0 + by0) - q.xh[1]) - q.xl[1], ((float)(Y0 + by1) - q.xh[1]) - q.xl[1]);
        const float ez = gap(((float)(Z0 + bz0) - q.xh[2]) - q.xl[2], ((float)(Z0 + bz1) - q.xh[2]) - q.xl[2]);
        const float d2 = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, __fmul_rn(ez, ez)));
        if (d2 > rp2 + 2.f * M) {   // warp-uniform
            for (int x = bx0; x <= bx1; ++x) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (!meet[h] || !inh[h]) continue;
                    const int l = lane + 64 * x + 32 * h;
                    const uint32_t w = S.w[l];
                    if ((w & VOX_NMASK) != 0u && (w >> VOX_NBITS) == tag) {
                        S.w[l] = 0u;
                        S.setter[l] = SETTER_ZERO;
                    }
                }
            }
            return;
        }
    }
    for (int x = bx0; x <= bx1; ++x) {
        const float dxf = ((float)(X0 + x) - q.xh[0]) - q.xl[0];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (!meet[h]) continue;
            int region = -1;
            if (inh[h]) {
                const float distf = __fmaf_rn(dxf, dxf, sh[h]);
                if (fabsf(distf - rp2) <= M || fabsf(distf - rm2) <= M)
                    region = region_exact(X0 + x, Y0 + yl + 4 * h, Z0 + z, sph[m]);
                else
                    region = distf > rp2 ? 0 : (distf < rm2 ? 1 : 2);
            }
            const int l = lane + 64 * x + 32 * h;
            const unsigned bal = __ballot_sync(FULL_MASK, region == 2);
            if (region == 2) {
                S.queue[qn + __popc(bal & below)] = (uint16_t)l;
            } else if (region >= 0) {
                fold_cell(S, l, region == 1 ? 125u : 0u, tag, m);
            }
            qn += __popc(bal);
        }
    }
    if (qn == 0) return;
    __syncwarp();
    // 2: counts of the queued cells, 32 at a time.  Lane `lane` takes queued
    // cell c0 + lane and decides each x-slice from its largest and smallest
    // sample sums, (xs_i + max ys) + max zs and (xs_i + min ys) + min zs: these
    // are samples of the slice, and the rounded sums are monotone in every term,
    // so a bound farther than M from r^2 decides all 25 samples as the
    // per-sample rule would (25 inside, or none).  The slices left are queued
    // and counted sample by sample, one slice per lane.
    for (int c0 = 0; c0 < qn; c0 += 32) {
        uint32_t mixed = 0u;
        int l = 0;
        if (c0 + lane < qn) {
            l = S.queue[c0 + lane];
            const int X = X0 + (l >> 6), Y = Y0 + ((l >> 3) & 7), Z = Z0 + (l & 7);
            const float dxf = ((float)X - q.xh[0]) - q.xl[0];
            const float dyf = ((float)Y - q.xh[1]) - q.xl[1];
            const float dzq = ((float)Z - q.xh[2]) - q.xl[2];
            float ymin = 3.0e38f, ymax = 0.f, zmin = 3.0e38f, zmax = 0.f;
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                const float d = sub_delta_f(j);
                const float ay = __fadd_rn(dyf, d), az = __fadd_rn(dzq, d);
                const float ys = __fmul_rn(ay, ay), zs = __fmul_rn(az, az);
                ymin = fminf(ymin, ys); ymax = fmaxf(ymax, ys);
                zmin = fminf(zmin, zs); zmax = fmaxf(zmax, zs);
            }
            int inside = 0;
#pragma unroll
            for (int i = 0; i < 5; ++i) {
                const float ax = __fadd_rn(dxf, sub_delta_f(i));
                const float xs = __fmul_rn(ax, ax);
                const float hi = __fsub_rn(__fadd_rn(__fadd_rn(xs, ymax), zmax), q.rsq);
                const float lo = __fsub_rn(__fadd_rn(__fadd_rn(xs, ymin), zmin), q.rsq);
                if (hi < -M) inside += 25;
                else if (!(lo > M)) mixed |= 1u << i;
            }
            cnt8[l] = (uint8_t)inside;
        }
        const int k = __popc(mixed);
        int incl = k;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int o = __shfl_up_sync(FULL_MASK, incl, d);
            if (lane >= d) incl += o;
        }
        const int total = __shfl_sync(FULL_MASK, incl, 31);
        for (int pos = incl - k; mixed; mixed &= mixed - 1u) S.items[pos++] = (uint16_t)((l << 3) | (__ffs(mixed) - 1));
        __syncwarp();
        for (int u = lane; u < total; u += 32) {
            const int it = S.items[u];
            const int l = it >> 3, i = it & 7;
            const int X = X0 + (l >> 6), Y = Y0 + ((l >> 3) & 7), Z = Z0 + (l & 7);
            const float dxf = ((float)X - q.xh[0]) - q.xl[0];
            const float dyf = ((float)Y - q.xh[1]) - q.xl[1];
            const float dzq = ((float)Z - q.xh[2]) - q.xl[2];
            bool unsure;
            int cs = slice_count_fast(dxf, dyf, dzq, i, q.rsq, M, &unsure);
            if (unsure) cs = slice_count_resolve(dxf, dyf, dzq, i, q.rsq, M, X, Y, Z, sph[m]);
            if (cs) atomicAdd(&S.cnt4[l >> 2], (uint32_t)cs << (8 * (l & 3)));
        }
        __syncwarp();
    }
    // 3
    for (int e = lane; e < qn; e += 32) {
        const int l = S.queue[e];
        fold_cell(S, l, (uint32_t)cnt8[l], tag, m);
    }
    __syncwarp();
}

// Surface velocity of a cell set by sphere `code` (SETTER_ZERO: zero).
template <typename T>
__device__ __forceinline__ void setter_velocity(uint32_t code, const SphereDev* __restrict__ sph,
                                                const SphereFast* __restrict__ fast, int X, int Y, int Z, T& u0,
                                                T& u1, T& u2) {
    if (code == SETTER_ZERO) {
        u0 = u1 = u2 = T(0);
    } else if (sizeof(T) == 8) {
        // setValues, src/ibProcessors3D.hh:163-174 (com == x for single spheres)
        double a0, a1, a2;
        surface_velocity(sph[code], X, Y, Z, a0, a1, a2);
        u0 = T(a0); u1 = T(a1); u2 = T(a2);
    } else {
        const SphereFast& q = fast[code];
        const float dxf = ((float)X - q.xh[0]) - q.xl[0];
        const float dyf = ((float)Y - q.xh[1]) - q.xl[1];
        const float dzf = ((float)Z - q.xh[2]) - q.xl[2];
        u0 = T(add_rn(q.v[0], sub_rn(mul_rn(q.w[1], dzf), mul_rn(q.w[2], dyf))));
        u1 = T(add_rn(q.v[1], add_rn(mul_rn(-q.w[0], dzf), mul_rn(q.w[2], dxf))));
        u2 = T(add_rn(q.v[2], sub_rn(mul_rn(q.w[0], dyf), mul_rn(q.w[1], dxf))));
    }
}

// One tile by one warp.  up == nullptr: no surface-velocity field is kept.
// INIT_VEL: defineVelocity (src/ibCompositeDynamics3D.hh:118-127) with the
// velocity a fully covered cell holds right after the last sphere covering it.
template <typename T, bool INIT_VEL>
__device__ __forceinline__ void voxelize_tile(WarpVox<INIT_VEL>& S, int t, const SphereDev* __restrict__ sph,
                                              const SphereFast* __restrict__ fast, int nsph,
                                              int* __restrict__ tile_cnt, const int* __restrict__ bins,
                                              uint32_t* __restrict__ vox, T* __restrict__ up, T* __restrict__ f,
                                              int phase, const Geom& g, const OwnerTable& ot) {
    const int lane = threadIdx.x & 31;
    const int tny = tiles_along(g.ny), tnz = tiles_along(g.nz);
    const int tx = t / (tny * tnz);
    const int rem = t - tx * tny * tnz;
    const int ty = rem / tnz;
    const int tz = rem - ty * tnz;
    const int X0 = tx * TILE, Y0 = ty * TILE, Z0 = tz * TILE;
    // The tile's count, both bin slots of the lane (read whatever the count; the
    // slots past it are ignored) and its 16 voxel words are independent loads,
    // issued together so that the tile waits for one memory latency, not four.
    const int cnt = tile_cnt[t];
    const int a0 = bins[(size_t)t * TILE_BIN + lane];
    const int b0 = bins[(size_t)t * TILE_BIN + lane + 32];
    // cell state; a lane's cells share z and, per plane half, the row
    const int z = lane & 7, Z = Z0 + z;
    const bool zok = Z < g.nz;
    uint32_t wv[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const int X = X0 + (j >> 1), Y = Y0 + (lane >> 3) + 4 * (j & 1);
        wv[j] = (zok && X < g.nx && Y < g.ny) ? vox[((size_t)X * g.ny + Y) * g.nz + Z] : 0u;
    }
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const int l = lane + 32 * j;
        S.w[l] = wv[j];
        S.setter[l] = SETTER_KEEP;
        if (INIT_VEL) S.defv[l] = DEFV_NONE;
    }
    // the lane's bin entries (list indices)
    int a = (cnt <= TILE_BIN && lane < cnt) ? a0 : INT_MAX;
    int b = (cnt <= TILE_BIN && lane + 32 < cnt) ? b0 : INT_MAX;
    if (cnt <= 0) return;
    if (lane == 0) tile_cnt[t] = 0;    // the bins are reused by the next voxelization
    constexpr int W4 = (int)(sizeof(SphereFast) / 16);
    const uint4* src = reinterpret_cast<const uint4*>(fast);
    uint4* dst = reinterpret_cast<uint4*>(S.q);
    if (cnt <= TILE_BIN) {
        for (int k = 0; k < cnt; ++k) {
            const int m = __reduce_min_sync(FULL_MASK, min(a, b));
            if (a == m) a = INT_MAX;
            if (b == m) b = INT_MAX;
            if (lane == 0) S.list[k] = m;
        }
        for (int base = 0; base < cnt; base += VOX_STAGE) {
            const int nst = min(VOX_STAGE, cnt - base);
            __syncwarp();
            for (int i = lane; i < W4 * nst; i += 32) {
                const int e = i / W4;
                dst[i] = __ldg(src + (size_t)S.list[base + e] * W4 + (i - W4 * e));
            }
            __syncwarp();
            for (int k = 0; k < nst; ++k) apply_sphere(S, S.q[k], S.list[base + k], sph, X0, Y0, Z0);
        }
    } else {
        // bin overflow: every sphere whose box reaches the tile, in list order
        for (int base = 0; base < nsph; base += 32) {
            const int i = base + lane;
            bool hit = false;
            if (i < nsph) {
                const SphereFast& q = fast[i];
                hit = q.lo[0] <= q.hi[0] && q.lo[1] <= q.hi[1] && q.lo[2] <= q.hi[2] && q.lo[0] <= X0 + TILE - 1 &&
                      q.hi[0] >= X0 && q.lo[1] <= Y0 + TILE - 1 && q.hi[1] >= Y0 && q.lo[2] <= Z0 + TILE - 1 &&
                      q.hi[2] >= Z0;
            }
            unsigned bal = __ballot_sync(FULL_MASK, hit);
            while (bal) {
                const int m = base + __ffs(bal) - 1;
                bal &= bal - 1u;
                __syncwarp();
                if (lane < W4) dst[lane] = __ldg(src + (size_t)m * W4 + lane);
                __syncwarp();
                apply_sphere(S, S.q[0], m, sph, X0, Y0, Z0);
            }
        }
    }
    __syncwarp();

    // defineVelocity first: it may need the surface velocity a cell held before this pass
    if (INIT_VEL) {
#pragma unroll 1
        for (int j = 0; j < 16; ++j) {
            const int l = lane + 32 * j;
            const uint32_t code = S.defv[l];
            if (code == DEFV_NONE) continue;
            const int X = X0 + (j >> 1), Y = Y0 + (lane >> 3) + 4 * (j & 1);
            const size_t c = ((size_t)X * g.ny + Y) * g.nz + Z;
            T d0, d1, d2;
            if (code == SETTER_KEEP && up != nullptr) {
                d0 = up[c]; d1 = up[g.N + c]; d2 = up[2 * g.N + c];
            } else if (code == SETTER_KEEP) {
                // no velocity field (float form): the velocity of the cell's
                // unchanged owner, recomputed as the collision does
                d0 = d1 = d2 = T(0);
                if constexpr (sizeof(T) == 4) {
                    const int slot = owner_slot(vox[c], ot.tag2slot, ot.max_tag, nsph);
                    if (slot >= 0) table_velocity(ot.xpf + (size_t)slot * XPF_STRIDE, X, Y, Z, g, d0, d1, d2);
                }
            } else {
                setter_velocity<T>(code, sph, fast, X, Y, Z, d0, d1, d2);
            }
            // f̄_i = feq_i(rhoBar = 0, invRho = 1, j = u), rounded operation by operation
            // (no contraction), so that every kernel variant writes the same bits
            const T uSqr = add_rn(add_rn(mul_rn(d0, d0), mul_rn(d1, d1)), mul_rn(d2, d2));
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                const T cu = add_rn(add_rn(mul_rn(T(cx(i)), d0), mul_rn(T(cy(i)), d1)), mul_rn(T(cz(i)), d2));
                const T e = mul_rn(T(wt(i)), add_rn(mul_rn(T(3), cu),
                                                    sub_rn(mul_rn(mul_rn(T(4.5), cu), cu), mul_rn(T(1.5), uSqr))));
                *pop_slot(f, i, X, Y, Z, phase, g) = e;
            }
        }
    }
    // write back the changed cells
#pragma unroll 2
    for (int j = 0; j < 16; ++j) {
        const int l = lane + 32 * j;
        const uint32_t code = S.setter[l];
        if (code == SETTER_KEEP) continue;
        const int X = X0 + (j >> 1), Y = Y0 + (lane >> 3) + 4 * (j & 1);
        const size_t c = ((size_t)X * g.ny + Y) * g.nz + Z;
        vox[c] = S.w[l];
        if (up != nullptr) {
            T u0, u1, u2;
            setter_velocity<T>(code, sph, fast, X, Y, Z, u0, u1, u2);
            up[c] = u0; up[g.N + c] = u1; up[2 * g.N + c] = u2;
        }
    }
}

// Persistent voxelization: warps claim tiles of the work list one at a time
// (work_n[0] tiles listed, work_n[1] claim counter, work_n[2] finished warps;
// the last warp to finish zeroes all three for the next voxelization).
// BATCH: a listed tile belongs to the domain d with toff[d] <= tile.
template <typename T, bool INIT_VEL, bool BATCH>
__global__ void __launch_bounds__(VOX_THREADS, INIT_VEL ? 2 : 3)
k_voxelize(const SphereDev* __restrict__ sph, const SphereFast* __restrict__ fast, int nsph,
           int* __restrict__ tile_cnt, const int* __restrict__ bins, const int* __restrict__ work,
           int* __restrict__ work_n, uint32_t* __restrict__ vox, T* __restrict__ up, T* __restrict__ f, int phase,
           Geom g, const DomView* __restrict__ doms, const int* __restrict__ toff, int ndom,
           const int* __restrict__ ncur, OwnerTable ot) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WarpVox<INIT_VEL>& S = reinterpret_cast<WarpVox<INIT_VEL>*>(smem_raw)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    // batch: the CTA's copy of the domains' first tiles (ndom <= TOFF_SMEM), for the
    // per-tile domain search
    const int* stoff = nullptr;
    if constexpr (BATCH) {
        int* m = reinterpret_cast<int*>(smem_raw + sizeof(WarpVox<INIT_VEL>) * VOX_WARPS);
        if (ndom <= TOFF_SMEM) {
            for (int k = threadIdx.x; k < ndom; k += blockDim.x) m[k] = __ldg(toff + k);
            stoff = m;
        }
        __syncthreads();   // every thread of the CTA reaches it (before any leaves)
    }
    const int nwork = *(volatile int*)work_n;
    // the next tile is claimed and its index read while the current one is worked on
    auto claim = [&]() -> int {
        int w = 0;
        if (lane == 0) w = atomicAdd(work_n + 1, 1);
        w = __shfl_sync(FULL_MASK, w, 0);
        return w < nwork ? work[w] : -1;
    };
    int next = claim();
    while (next >= 0) {
        const int tg = next;
        next = claim();
        if (BATCH) {
            int d;
            if (stoff) {
                int lo = 0, hi = ndom - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (stoff[mid] <= tg) lo = mid;
                    else hi = mid - 1;
                }
                d = lo;
            } else {
                d = find_domain(toff, ndom, tg);
            }
            const DomView& D = doms[d];
            const OwnerTable od{ot.xpf + (size_t)XPF_STRIDE * D.s0, ot.tag2slot + D.tag0, ot.max_tag};
            voxelize_tile<T, INIT_VEL>(S, tg - D.t0, sph + D.s0, fast + D.s0, __ldg(ncur + d), tile_cnt + D.t0,
                                       bins + (size_t)D.t0 * TILE_BIN, vox + D.cell0, up ? up + D.up0 : up,
                                       f ? f + D.f0 : f, phase, D.g, od);
        } else {
            voxelize_tile<T, INIT_VEL>(S, tg, sph, fast, nsph, tile_cnt, bins, vox, up, f, phase, g, ot);
        }
        __syncwarp();
    }
    if (lane == 0) {
        __threadfence();
        if (atomicAdd(work_n + 2, 1) == (int)(gridDim.x * VOX_WARPS) - 1) {
            work_n[0] = 0;
            work_n[1] = 0;
            work_n[2] = 0;
        }
    }
}

}  // namespace

cudaError_t launch_prepare_bin(const double* rec, int n, SphereDev* sph, SphereFast* fast, float* xpf,
                               int* tag2slot, unsigned* err, Geom g, int max_tag, double max_radius,
                               double* ft_zero, double* rec_copy, int* tile_cnt, int* bins, int* work, int* work_n,
                               cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_prepare_bin<false><<<(n + 7) / 8, 256, 0, s>>>(rec, n, sph, fast, xpf, tag2slot, err, g, max_tag, max_radius,
                                                     nullptr, nullptr, 0, nullptr, ft_zero, rec_copy, tile_cnt, bins,
                                                     work, work_n);
    return cudaGetLastError();
}

cudaError_t launch_prepare_bin_batch(const double* rec, int nslots, SphereDev* sph, SphereFast* fast, float* xpf,
                                     int* tag2slot, unsigned* err, int max_tag, double max_radius,
                                     const DomView* doms, const int* soff, int ndom, const int* ncur,
                                     double* ft_zero, int* tile_cnt, int* bins, int* work, int* work_n,
                                     cudaStream_t s) {
    if (nslots <= 0) return cudaSuccess;
    k_prepare_bin<true><<<(nslots + 7) / 8, 256, 0, s>>>(rec, nslots, sph, fast, xpf, tag2slot, err, Geom{}, max_tag,
                                                         max_radius, doms, soff, ndom, ncur, ft_zero, nullptr,
                                                         tile_cnt, bins, work, work_n);
    return cudaGetLastError();
}

namespace {

template <typename T, bool INIT_VEL, bool BATCH>
cudaError_t launch_vox(const SphereDev* sph, const SphereFast* fast, int n, int* tile_cnt, const int* bins,
                       const int* work, int* work_n, int ntiles, uint32_t* vox, T* up, T* f, int phase, Geom g,
                       const DomView* doms, const int* toff, int ndom, const int* ncur, const OwnerTable& ot,
                       cudaStream_t s) {
    constexpr size_t smem = sizeof(WarpVox<INIT_VEL>) * VOX_WARPS + (BATCH ? sizeof(int) * TOFF_SMEM : 0);
    static std::atomic<int> cached[LBDEM_MAX_DEVICES];   // per device: persistent grid size
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= LBDEM_MAX_DEVICES) return cudaErrorInvalidDevice;
    int blocks = cached[dev].load(std::memory_order_relaxed);
    if (blocks == 0) {
        int sms = 0, per_sm = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_voxelize<T, INIT_VEL, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_voxelize<T, INIT_VEL, BATCH>, VOX_THREADS,
                                                              smem);
        if (e != cudaSuccess) return e;
        blocks = sms * (per_sm > 0 ? per_sm : 1);
        cached[dev].store(blocks, std::memory_order_relaxed);
    }
    const int need = (ntiles + VOX_WARPS - 1) / VOX_WARPS;
    const int grid = need < blocks ? need : blocks;
    k_voxelize<T, INIT_VEL, BATCH><<<grid, VOX_THREADS, smem, s>>>(sph, fast, n, tile_cnt, bins, work, work_n, vox, up,
                                                                  f, phase, g, doms, toff, ndom, ncur, ot);
    return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t launch_voxelize(const SphereDev* sph, const SphereFast* fast, int n, int* tile_cnt, const int* bins,
                            const int* work, int* work_n, int ntiles, uint32_t* vox, T* up, T* f, int init_vel,
                            int odd_phase, Geom g, const OwnerTable& ot, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    if (init_vel)
        return launch_vox<T, true, false>(sph, fast, n, tile_cnt, bins, work, work_n, ntiles, vox, up, f, odd_phase, g,
                                          nullptr, nullptr, 0, nullptr, ot, s);
    return launch_vox<T, false, false>(sph, fast, n, tile_cnt, bins, work, work_n, ntiles, vox, up, f, odd_phase, g,
                                       nullptr, nullptr, 0, nullptr, ot, s);
}

template <typename T>
cudaError_t launch_voxelize_batch(const SphereDev* sph, const SphereFast* fast, int* tile_cnt, const int* bins,
                                  const int* work, int* work_n, int ntiles, uint32_t* vox, T* up, T* f, int init_vel,
                                  int odd_phase, const DomView* doms, const int* toff, int ndom, const int* ncur,
                                  const OwnerTable& ot, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    if (init_vel)
        return launch_vox<T, true, true>(sph, fast, 0, tile_cnt, bins, work, work_n, ntiles, vox, up, f, odd_phase,
                                         Geom{}, doms, toff, ndom, ncur, ot, s);
    return launch_vox<T, false, true>(sph, fast, 0, tile_cnt, bins, work, work_n, ntiles, vox, up, f, odd_phase,
                                      Geom{}, doms, toff, ndom, ncur, ot, s);
}

#define INST(T)                                                                                                    \
    template cudaError_t launch_voxelize<T>(const SphereDev*, const SphereFast*, int, int*, const int*, const int*, \
                                            int*, int, uint32_t*, T*, T*, int, int, Geom, const OwnerTable&,       \
                                            cudaStream_t);                                                         \
    template cudaError_t launch_voxelize_batch<T>(const SphereDev*, const SphereFast*, int*, const int*,          \
                                                  const int*, int*, int, uint32_t*, T*, T*, int, int,              \
                                                  const DomView*, const int*, int, const int*, const OwnerTable&,  \
                                                  cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace lbdem
