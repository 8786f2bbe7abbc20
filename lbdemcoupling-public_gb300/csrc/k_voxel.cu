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
// comparison is first made in float with a margin M = 2^-18 (r + 4)^2.  For a
// cell inside the box (|dx| < r + 3, centre split x = xh + xl with |x| < 2^24)
// the float value differs from the double one by at most 27 u (r + 3.5)^2,
// u = 2^-24 (sample sums), resp. 22 u (r + 3.2)^2 (dist), so a float result
// farther than M from the threshold decides the comparison as the double
// computation does.  Only comparisons inside the band are evaluated with the
// reference's double sequence (__dadd_rn/__dmul_rn: no fused multiply-add).
// Counts n and owner tags are identical to the sequential CPU result; the
// FP64 form also reproduces the particle surface velocity bit for bit.
#include "lbdem_internal.h"

namespace lbdem {
namespace {

constexpr double SQRT3HALF = 0.8803408430829505;  // sqrt(3.1)/2, src/ibProcessors3D.hh:128-130
// -0.5 + (i + 0.5) * (1./5.), src/ibProcessors3D.hh:141-147, evaluated in double:
__device__ __forceinline__ double sub_delta(int i) {
    return i == 0 ? -0.4 : i == 1 ? -0.19999999999999996 : i == 2 ? 0.0 : i == 3 ? 0.20000000000000007 : 0.4;
}
__device__ __forceinline__ float sub_delta_f(int i) {
    return i == 0 ? -0.4f : i == 1 ? -0.2f : i == 2 ? 0.0f : i == 3 ? 0.2f : 0.4f;
}

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
    q.margin = ldexpf(r4 * r4, -18);
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
    float* xp = xpf + (size_t)i * 8;
    xp[0] = q.xh[0]; xp[1] = q.xh[1]; xp[2] = q.xh[2]; xp[3] = q.xl[0];
    xp[4] = q.xl[1]; xp[5] = q.xl[2]; xp[6] = 0.f; xp[7] = 0.f;
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

// Sub-cell count of one x-slice (i fixed: 25 of the 125 samples) of a shell
// cell in float; *unsure is set when a sample falls inside the decision band.
__device__ __forceinline__ int slice_count_fast(float dxf, float dyf, float dzf, int i, float rsq, float M,
                                                bool* unsure) {
    const float ax = dxf + sub_delta_f(i);
    const float xs = ax * ax;
    float ys[5], zs[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const float d = sub_delta_f(j);
        const float ay = dyf + d; ys[j] = ay * ay;
        const float az = dzf + d; zs[j] = az * az;
    }
    const float lo = rsq - M, hi = rsq + M;
    int n_lo = 0, n_hi = 0;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const float a = xs + ys[j];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const float t = a + zs[k];
            n_lo += t < lo ? 1 : 0;
            n_hi += t < hi ? 1 : 0;
        }
    }
    *unsure = n_lo != n_hi;
    return n_lo;
}

// The same slice with the samples inside the band decided by the reference's
// double sequence ((xs_i + ys_j) + zs_k < r^2, src/ibProcessors3D.hh:141-155).
__device__ __noinline__ int slice_count_resolve(float dxf, float dyf, float dzf, int i, float rsq, float M, int X,
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

// Sub-cell count of a shell cell by one thread (all five x-slices), out of line:
// only taken when a chunk's shell queue is full.
__device__ __noinline__ uint32_t shell_count_direct(float dxf, float dyf, float dzf, float rsq, float M, int X, int Y,
                                                    int Z, const SphereDev& s) {
    uint32_t n = 0;
#pragma unroll 1
    for (int i = 0; i < 5; ++i) {
        bool unsure;
        int c = slice_count_fast(dxf, dyf, dzf, i, rsq, M, &unsure);
        if (unsure) c = slice_count_resolve(dxf, dyf, dzf, i, rsq, M, X, Y, Z, s);
        n += (uint32_t)c;
    }
    return n;
}

// Shared memory of one voxelization block.
constexpr int VOX_THREADS = 256;            // two cells of the 8^3 tile per thread
constexpr int VOX_CHUNK = 32;               // spheres classified per pass
constexpr int VOX_QUEUE = 2048;             // shell (sphere, cell) pairs per pass
constexpr uint32_t N_NONE = 255;            // cell outside the sphere's box

template <typename T, bool INIT_VEL>
struct VoxSmem {
    int raw[TILE_LIST_MAX];
    int sorted[TILE_LIST_MAX];
    SphereFast q[VOX_CHUNK];
    uint32_t bm[VOX_CHUNK];                   // tile-local box of sphere k: x, y, z cell masks (8 bits each)
    uint32_t n4[VOX_CHUNK][TILE_CELLS / 4];   // count of (sphere k, cell), one byte per cell
    uint16_t queue[VOX_QUEUE];                // (k << 9) | cell of the queued shell pairs
    T u[3][TILE_CELLS];                       // cell state carried across chunks
    T d[INIT_VEL ? 3 : 1][INIT_VEL ? TILE_CELLS : 1];
    uint32_t id[TILE_CELLS];
    uint8_t n[TILE_CELLS];
    uint8_t flags[TILE_CELLS];                // bit 0: state changed, bit 1: define velocity
    int qcount;
    int cnt;
};

__device__ __forceinline__ uint32_t get_n(const uint32_t* row, int l) { return (row[l >> 2] >> (8 * (l & 3))) & 0xffu; }
__device__ __forceinline__ void set_n(uint32_t* row, int l, uint32_t n) {
    uint8_t* b = reinterpret_cast<uint8_t*>(row);
    b[l] = (uint8_t)n;
}

// One block per 8^3 tile, 256 threads.  Spheres are taken in sorted chunks of
// VOX_CHUNK; each chunk runs three phases separated by block barriers:
//  A  classify every (sphere, cell) pair in float: outside the box, outside
//     (n = 0) and inside (n = 125) are final, shell pairs are queued with n = 0;
//  B  the queue is split into x-slices (25 samples each) and drained by all
//     threads, slice counts added into the pair's byte with shared atomics;
//  C  every cell folds the chunk's counts, in sphere order, through decFlag.
// INIT_VEL: defineVelocity (src/ibCompositeDynamics3D.hh:118-127) is applied
// with the uPart the cell holds right after each sphere that covers it fully
// (src/ibProcessors3D.hh:107-108); it depends only on that uPart, so the last
// such sphere decides the populations written.
template <typename T, bool INIT_VEL>
__device__ __forceinline__ void voxelize_tile(VoxSmem<T, INIT_VEL>& S, int t, const SphereDev* __restrict__ sph,
                                              const SphereFast* __restrict__ fast, int nsph,
                                              int* __restrict__ tile_cnt, const int* __restrict__ bins,
                                              uint32_t* __restrict__ vox, T* __restrict__ up, T* __restrict__ f,
                                              int phase, const Geom& g, unsigned* __restrict__ err) {
    const int tid = threadIdx.x;
    const int tny = tiles_along(g.ny), tnz = tiles_along(g.nz);
    const int tx = t / (tny * tnz);
    const int rem = t - tx * tny * tnz;
    const int ty = rem / tnz;
    const int tz = rem - ty * tnz;
    const int X0 = tx * TILE, Y0 = ty * TILE, Z0 = tz * TILE;

    // the cell-state loads go out first: their latency overlaps the list loads
    uint32_t wv[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int l = tid + h * VOX_THREADS;
        const int X = X0 + (l >> 6), Y = Y0 + ((l >> 3) & 7), Z = Z0 + (l & 7);
        wv[h] = (X < g.nx && Y < g.ny && Z < g.nz) ? vox[((size_t)X * g.ny + Y) * g.nz + Z] : 0u;
    }
    int cnt = tile_cnt[t];
    if (cnt <= 0) return;
    __syncthreads();
    if (tid == 0) tile_cnt[t] = 0;   // bins are reused by the next voxelization
    if (cnt <= TILE_BIN) {
        for (int k = tid; k < cnt; k += VOX_THREADS) S.raw[k] = bins[(size_t)t * TILE_BIN + k];
    } else {
        // bin overflow: collect every sphere whose box overlaps this tile
        if (tid == 0) S.cnt = 0;
        __syncthreads();
        for (int i = tid; i < nsph; i += VOX_THREADS) {
            const SphereFast& q = fast[i];
            if (q.lo[0] <= X0 + TILE - 1 && q.hi[0] >= X0 && q.lo[1] <= Y0 + TILE - 1 && q.hi[1] >= Y0 &&
                q.lo[2] <= Z0 + TILE - 1 && q.hi[2] >= Z0 && q.lo[0] <= q.hi[0] && q.lo[1] <= q.hi[1] &&
                q.lo[2] <= q.hi[2]) {
                const int pos = atomicAdd(&S.cnt, 1);
                if (pos < TILE_LIST_MAX) S.raw[pos] = i;
            }
        }
        __syncthreads();
        cnt = S.cnt;
        if (cnt > TILE_LIST_MAX) {
            if (tid == 0) atomicOr(err, 0x1u);  // LBDEM_DEVERR_TILE_LIST
            return;
        }
    }
    // cell state into shared memory
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int l = tid + h * VOX_THREADS;
        const int X = X0 + (l >> 6), Y = Y0 + ((l >> 3) & 7), Z = Z0 + (l & 7);
        const uint32_t w0 = wv[h];
        S.n[l] = (uint8_t)(w0 & VOX_NMASK);
        S.id[l] = w0 >> VOX_NBITS;
        S.flags[l] = 0;
        // The surface velocity a cell holds is only read back by defineVelocity
        // (a fully covered cell that no sphere of this pass sets keeps it); the
        // velocity written back is always the one a set or zero of this pass made.
        T u0 = T(0), u1 = T(0), u2 = T(0);
        if (INIT_VEL && (w0 & VOX_NMASK) > 0) {
            const size_t c = ((size_t)X * g.ny + Y) * g.nz + Z;
            u0 = up[c]; u1 = up[g.N + c]; u2 = up[2 * g.N + c];
        }
        S.u[0][l] = u0; S.u[1][l] = u1; S.u[2][l] = u2;
    }
    __syncthreads();
    // rank sort by sphere index (the indices of one list are distinct)
    for (int k = tid; k < cnt; k += VOX_THREADS) {
        const int vk = S.raw[k];
        int rank = 0;
        for (int m = 0; m < cnt; ++m) rank += (S.raw[m] < vk) ? 1 : 0;
        S.sorted[rank] = vk;
    }

    for (int base = 0; base < cnt; base += VOX_CHUNK) {
        const int m = min(VOX_CHUNK, cnt - base);
        __syncthreads();   // sorted list ready / previous chunk finished with S.q and S.n4
        {
            const int words = (int)(sizeof(SphereFast) / 4);
            for (int k = tid; k < m * words; k += VOX_THREADS) {
                const int e = k / words, wd = k - e * words;
                reinterpret_cast<int*>(&S.q[e])[wd] = reinterpret_cast<const int*>(&fast[S.sorted[base + e]])[wd];
            }
            if (tid < m) {   // the sphere's box within this tile and the lattice, as cell masks
                const SphereFast& qs = fast[S.sorted[base + tid]];
                const int o[3] = {X0, Y0, Z0}, dims[3] = {g.nx, g.ny, g.nz};
                uint32_t bm = 0;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const int lo = max(qs.lo[a] - o[a], 0);
                    const int hi = min(min(qs.hi[a] - o[a], TILE - 1), dims[a] - 1 - o[a]);
                    const uint32_t mk = lo <= hi ? ((0xffu >> (TILE - 1 - hi)) & (0xffu << lo)) & 0xffu : 0u;
                    bm |= mk << (8 * a);
                }
                S.bm[tid] = bm;
            }
        }
        if (tid == 0) S.qcount = 0;
        __syncthreads();
        // Phase A
        for (int k = 0; k < m; ++k) {
            const SphereFast& q = S.q[k];
#pragma unroll 1
            for (int h = 0; h < 2; ++h) {
                const int l = tid + h * VOX_THREADS;
                const int X = X0 + (l >> 6), Y = Y0 + ((l >> 3) & 7), Z = Z0 + (l & 7);
                uint32_t n = N_NONE;
                const uint32_t bm = S.bm[k];
                if ((bm >> (l >> 6)) & (bm >> (8 + ((l >> 3) & 7))) & (bm >> (16 + (l & 7))) & 1u) {
                    const float dxf = ((float)X - q.xh[0]) - q.xl[0];
                    const float dyf = ((float)Y - q.xh[1]) - q.xl[1];
                    const float dzf = ((float)Z - q.xh[2]) - q.xl[2];
                    const float distf = (dxf * dxf + dyf * dyf) + dzf * dzf;
                    const float M = q.margin;
                    int region;
                    if (fabsf(distf - q.rp2) <= M || fabsf(distf - q.rm2) <= M)
                        region = region_exact(X, Y, Z, sph[S.sorted[base + k]]);
                    else
                        region = distf > q.rp2 ? 0 : (distf < q.rm2 ? 1 : 2);
                    if (region == 0) {
                        n = 0;
                    } else if (region == 1) {
                        n = 125;
                    } else {
                        n = 0;   // the queued slice counts are added to it
                        const int pos = atomicAdd(&S.qcount, 1);
                        if (pos < VOX_QUEUE) {
                            S.queue[pos] = (uint16_t)((k << 9) | l);
                        } else {
                            n = shell_count_direct(dxf, dyf, dzf, q.rsq, M, X, Y, Z, sph[S.sorted[base + k]]);
                        }
                    }
                }
                set_n(S.n4[k], l, n);
            }
        }
        __syncthreads();
        // Phase B: five x-slices per queued pair
        {
            const int qn = min(S.qcount, VOX_QUEUE);
            for (int wi = tid; wi < 5 * qn; wi += VOX_THREADS) {
                const int e = wi / 5, i = wi - 5 * e;
                const int k = S.queue[e] >> 9, l = S.queue[e] & 511;
                const SphereFast& q = S.q[k];
                const int X = X0 + (l >> 6), Y = Y0 + ((l >> 3) & 7), Z = Z0 + (l & 7);
                const float dxf = ((float)X - q.xh[0]) - q.xl[0];
                const float dyf = ((float)Y - q.xh[1]) - q.xl[1];
                const float dzf = ((float)Z - q.xh[2]) - q.xl[2];
                bool unsure;
                int c = slice_count_fast(dxf, dyf, dzf, i, q.rsq, q.margin, &unsure);
                if (unsure) c = slice_count_resolve(dxf, dyf, dzf, i, q.rsq, q.margin, X, Y, Z, sph[S.sorted[base + k]]);
                if (c) atomicAdd(&S.n4[k][l >> 2], (uint32_t)c << (8 * (l & 3)));
            }
        }
        __syncthreads();
        // Phase C: decFlag, src/ibProcessors3D.hh:85-105 (sf > 0.001 <=> n > 0; sf > sf_old <=> n > n_old)
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
            const int l = tid + h * VOX_THREADS;
            const int X = X0 + (l >> 6), Y = Y0 + ((l >> 3) & 7), Z = Z0 + (l & 7);
            uint32_t nold = S.n[l], idold = S.id[l];
            T u0 = S.u[0][l], u1 = S.u[1][l], u2 = S.u[2][l];
            uint32_t fl = S.flags[l];
            for (int k = 0; k < m; ++k) {
                const uint32_t n = get_n(S.n4[k], l);
                if (n == N_NONE) continue;
                const SphereFast& q = S.q[k];
                const int dec = (n > 0 ? 1 : 0) + (nold > 0 ? 2 : 0);
                bool set = false, zero = false;
                if (dec == 1) set = true;
                else if (dec == 2) zero = (idold == (uint32_t)q.tag);
                else if (dec == 3) set = (n > nold) || (idold == (uint32_t)q.tag);
                // dec == 0 is setToZero on a cell that is already empty
                if (zero) {
                    nold = 0; idold = 0; u0 = u1 = u2 = T(0); fl |= 1u;
                } else if (set) {
                    // setValues, src/ibProcessors3D.hh:163-174 (com == x for single spheres)
                    if (sizeof(T) == 8) {
                        double a0, a1, a2;
                        surface_velocity(sph[S.sorted[base + k]], X, Y, Z, a0, a1, a2);
                        u0 = T(a0); u1 = T(a1); u2 = T(a2);
                    } else {
                        const float dxf = ((float)X - q.xh[0]) - q.xl[0];
                        const float dyf = ((float)Y - q.xh[1]) - q.xl[1];
                        const float dzf = ((float)Z - q.xh[2]) - q.xl[2];
                        u0 = T(q.v[0] + (q.w[1] * dzf - q.w[2] * dyf));
                        u1 = T(q.v[1] + (-q.w[0] * dzf + q.w[2] * dxf));
                        u2 = T(q.v[2] + (q.w[0] * dyf - q.w[1] * dxf));
                    }
                    nold = n; idold = (uint32_t)q.tag; fl |= 1u;
                }
                if (INIT_VEL && n == 125) {
                    fl |= 2u;
                    S.d[0][l] = u0; S.d[1][l] = u1; S.d[2][l] = u2;
                }
            }
            S.n[l] = (uint8_t)nold; S.id[l] = idold; S.flags[l] = (uint8_t)fl;
            S.u[0][l] = u0; S.u[1][l] = u1; S.u[2][l] = u2;
        }
    }

    // write back (each thread its own two cells; no barrier needed)
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
        const int l = tid + h * VOX_THREADS;
        const int X = X0 + (l >> 6), Y = Y0 + ((l >> 3) & 7), Z = Z0 + (l & 7);
        if (X >= g.nx || Y >= g.ny || Z >= g.nz) continue;
        const size_t c = ((size_t)X * g.ny + Y) * g.nz + Z;
        const uint32_t fl = S.flags[l];
        if (fl & 1u) {
            vox[c] = (uint32_t)S.n[l] | (S.id[l] << VOX_NBITS);
            up[c] = S.u[0][l]; up[g.N + c] = S.u[1][l]; up[2 * g.N + c] = S.u[2][l];
        }
        if (INIT_VEL && (fl & 2u)) {
            // f̄_i = feq_i(rhoBar = 0, invRho = 1, j = u)
            const T d0 = S.d[0][l], d1 = S.d[1][l], d2 = S.d[2][l];
            const T uSqr = d0 * d0 + d1 * d1 + d2 * d2;
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                const T cu = T(cx(i)) * d0 + T(cy(i)) * d1 + T(cz(i)) * d2;
                const T e = T(wt(i)) * (T(3) * cu + (T(4.5) * cu * cu - T(1.5) * uSqr));
                *pop_slot(f, i, X, Y, Z, phase, g) = e;
            }
        }
    }
}

// Persistent voxelization: blocks claim tiles of the work list one at a time
// (work_n[0] tiles listed, work_n[1] claim counter, work_n[2] finished blocks;
// the last block to finish zeroes all three for the next voxelization).
// BATCH: a listed tile belongs to the domain d with toff[d] <= tile.
template <typename T, bool INIT_VEL, bool BATCH>
__global__ void __launch_bounds__(VOX_THREADS, 4)   // 4 blocks per SM (measured best; a few spills)
k_voxelize(const SphereDev* __restrict__ sph, const SphereFast* __restrict__ fast, int nsph,
           int* __restrict__ tile_cnt, const int* __restrict__ bins, const int* __restrict__ work,
           int* __restrict__ work_n, uint32_t* __restrict__ vox, T* __restrict__ up, T* __restrict__ f, int phase,
           Geom g, unsigned* __restrict__ err, const DomView* __restrict__ doms, const int* __restrict__ toff,
           int ndom, const int* __restrict__ ncur) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    VoxSmem<T, INIT_VEL>& S = *reinterpret_cast<VoxSmem<T, INIT_VEL>*>(smem_raw);
    __shared__ int s_item;
    const int nwork = *(volatile int*)work_n;
    for (;;) {
        __syncthreads();   // previous tile done with S
        if (threadIdx.x == 0) s_item = atomicAdd(work_n + 1, 1);
        __syncthreads();
        const int w = s_item;
        if (w >= nwork) break;
        const int tg = work[w];
        if (BATCH) {
            const int d = find_domain(toff, ndom, tg);
            const DomView& D = doms[d];
            voxelize_tile<T, INIT_VEL>(S, tg - D.t0, sph + D.s0, fast + D.s0, __ldg(ncur + d), tile_cnt + D.t0,
                                       bins + (size_t)D.t0 * TILE_BIN, vox + D.cell0, up + D.up0, f ? f + D.f0 : f,
                                       phase, D.g, err);
        } else {
            voxelize_tile<T, INIT_VEL>(S, tg, sph, fast, nsph, tile_cnt, bins, vox, up, f, phase, g, err);
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(work_n + 2, 1) == (int)gridDim.x - 1) {
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
                       unsigned* err, const DomView* doms, const int* toff, int ndom, const int* ncur,
                       cudaStream_t s) {
    constexpr size_t smem = sizeof(VoxSmem<T, INIT_VEL>);
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
    const int grid = ntiles < blocks ? ntiles : blocks;
    k_voxelize<T, INIT_VEL, BATCH><<<grid, VOX_THREADS, smem, s>>>(sph, fast, n, tile_cnt, bins, work, work_n, vox, up,
                                                                  f, phase, g, err, doms, toff, ndom, ncur);
    return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t launch_voxelize(const SphereDev* sph, const SphereFast* fast, int n, int* tile_cnt, const int* bins,
                            const int* work, int* work_n, int ntiles, uint32_t* vox, T* up, T* f, int init_vel,
                            int odd_phase, Geom g, unsigned* err, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    if (init_vel)
        return launch_vox<T, true, false>(sph, fast, n, tile_cnt, bins, work, work_n, ntiles, vox, up, f, odd_phase, g,
                                          err, nullptr, nullptr, 0, nullptr, s);
    return launch_vox<T, false, false>(sph, fast, n, tile_cnt, bins, work, work_n, ntiles, vox, up, f, odd_phase, g,
                                       err, nullptr, nullptr, 0, nullptr, s);
}

template <typename T>
cudaError_t launch_voxelize_batch(const SphereDev* sph, const SphereFast* fast, int* tile_cnt, const int* bins,
                                  const int* work, int* work_n, int ntiles, uint32_t* vox, T* up, T* f, int init_vel,
                                  int odd_phase, const DomView* doms, const int* toff, int ndom, const int* ncur,
                                  unsigned* err, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    if (init_vel)
        return launch_vox<T, true, true>(sph, fast, 0, tile_cnt, bins, work, work_n, ntiles, vox, up, f, odd_phase,
                                         Geom{}, err, doms, toff, ndom, ncur, s);
    return launch_vox<T, false, true>(sph, fast, 0, tile_cnt, bins, work, work_n, ntiles, vox, up, f, odd_phase,
                                      Geom{}, err, doms, toff, ndom, ncur, s);
}

#define INST(T)                                                                                                    \
    template cudaError_t launch_voxelize<T>(const SphereDev*, const SphereFast*, int, int*, const int*, const int*, \
                                            int*, int, uint32_t*, T*, T*, int, int, Geom, unsigned*, cudaStream_t); \
    template cudaError_t launch_voxelize_batch<T>(const SphereDev*, const SphereFast*, int*, const int*,          \
                                                  const int*, int*, int, uint32_t*, T*, T*, int, int,              \
                                                  const DomView*, const int*, int, const int*, unsigned*,          \
                                                  cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace lbdem
