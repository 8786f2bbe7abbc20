// K2: sphere voxelization, bit-exact with SetSingleSphere3D.
//
// Replaces setSpheresOnLattice -> SetSingleSphere3D::process for every sphere
// (src/ibDataExchangeWrappers3D.hh:33-146, src/ibProcessors3D.hh:53-184).
//
// The reference applies spheres one after another, and each cell's new state
// depends on its previous state and on the order of the spheres whose bounding
// box covers it (decFlag, src/ibProcessors3D.hh:85-105).  The GPU version keeps
// that order per cell: spheres are binned to 8^3-cell tiles, each tile's list
// is sorted by sphere index in shared memory, and every cell folds the sorted
// list through the same state machine.  Cells are independent, so the result
// equals the sequential sweep exactly.
//
// Arithmetic is IEEE double with every multiply and add rounded separately
// (__dmul_rn / __dadd_rn: no fused multiply-add), in the reference's operation
// order, so the sub-cell counts n, the owner tags and the surface velocities
// are bit-identical to the CPU result.
#include "lbdem_internal.h"

namespace lbdem {
namespace {

constexpr double SQRT3HALF = 0.8803408430829505;  // sqrt(3.1)/2, src/ibProcessors3D.hh:128-130
// -0.5 + (i + 0.5) * (1./5.), src/ibProcessors3D.hh:141-147, evaluated in double:
__device__ __forceinline__ double sub_delta(int i) {
    return i == 0 ? -0.4 : i == 1 ? -0.19999999999999996 : i == 2 ? 0.0 : i == 3 ? 0.20000000000000007 : 0.4;
}

// calcSolidFraction as a sub-cell count n in [0,125]; sf = n / 125 exactly
// (the early-outs return 0 and 1, i.e. n = 0 and n = 125).
__device__ __forceinline__ int solid_count(double dx_, double dy_, double dz_, double r_) {
    const double dist = __dadd_rn(__dadd_rn(__dmul_rn(dx_, dx_), __dmul_rn(dy_, dy_)), __dmul_rn(dz_, dz_));
    const double r_p = __dadd_rn(r_, SQRT3HALF);
    if (dist > __dmul_rn(r_p, r_p)) return 0;
    const double r_m = __dsub_rn(r_, SQRT3HALF);
    if (dist < __dmul_rn(r_m, r_m)) return 125;
    const double r_sq = __dmul_rn(r_, r_);
    double xs[5], ys[5], zs[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const double d = sub_delta(i);
        const double ax = __dadd_rn(dx_, d); xs[i] = __dmul_rn(ax, ax);
        const double ay = __dadd_rn(dy_, d); ys[i] = __dmul_rn(ay, ay);
        const double az = __dadd_rn(dz_, d); zs[i] = __dmul_rn(az, az);
    }
    int n = 0;
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            const double a = __dadd_rn(xs[i], ys[j]);
#pragma unroll
            for (int k = 0; k < 5; ++k) n += (__dadd_rn(a, zs[k]) < r_sq) ? 1 : 0;
        }
    return n;
}

__device__ __forceinline__ int tiles_along(int n) { return (n + TILE - 1) / TILE; }

// Per sphere: bounding box (double -> integer truncation toward zero,
// src/ibProcessors3D.h:43-45) intersected with the lattice
// (src/ibDataExchangeWrappers3D.hh:127-133), tile overlap counts, and the
// tag -> lowest list index map (LAMMPS atom->map keeps the owned atom).
__global__ void k_prepare_spheres(const double* __restrict__ rec, int n, SphereDev* __restrict__ sph,
                                  int* __restrict__ tile_count, int* __restrict__ tag2slot,
                                  unsigned* __restrict__ err, Geom g, int max_tag, double max_radius) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* p = rec + (size_t)i * REC_STRIDE;
    SphereDev s;
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
        // |x| bounded so that the integer conversions below are defined; such
        // a sphere cannot reach the lattice anyway.
        if (!(xd > -1.0e9 && xd < 1.0e9)) { s.valid = 0; s.lo[d] = 1; s.hi[d] = 0; continue; }
        long long lo = (long long)(__dsub_rn(__dsub_rn(xd, s.r), 2.0));
        long long hi = (long long)(__dadd_rn(__dadd_rn(xd, s.r), 2.0));
        if (lo < 0) lo = 0;
        if (hi > dims[d] - 1) hi = dims[d] - 1;
        s.lo[d] = (int)(lo < (long long)dims[d] ? lo : dims[d]);
        s.hi[d] = (int)(hi > -1 ? hi : -1);
        if (s.lo[d] > s.hi[d]) s.valid = 0;
    }
    sph[i] = s;
    if (s.tag >= 1) atomicMin(tag2slot + s.tag, i);
    if (!s.valid) return;
    const int tny = tiles_along(g.ny), tnz = tiles_along(g.nz);
    for (int tx = s.lo[0] / TILE; tx <= s.hi[0] / TILE; ++tx)
        for (int ty = s.lo[1] / TILE; ty <= s.hi[1] / TILE; ++ty)
            for (int tz = s.lo[2] / TILE; tz <= s.hi[2] / TILE; ++tz)
                atomicAdd(tile_count + ((size_t)tx * tny + ty) * tnz + tz, 1);
}

// Exclusive scan of the tile counts (one block): tile_count[t] becomes the
// offset of tile t's list, tile_count[ntiles] the total.  Also clears the fill
// cursors.
constexpr int SCAN_THREADS = 1024;
__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_tiles(int* __restrict__ cnt, int ntiles, int pair_capacity, int* __restrict__ cursor,
             unsigned* __restrict__ err) {
    __shared__ long long s_sum[SCAN_THREADS];
    const int t = threadIdx.x;
    const int per = (ntiles + SCAN_THREADS - 1) / SCAN_THREADS;
    const int beg = t * per;
    const int end = min(beg + per, ntiles);
    long long local = 0;
    for (int k = beg; k < end; ++k) local += cnt[k];
    s_sum[t] = local;
    __syncthreads();
    for (int off = 1; off < SCAN_THREADS; off <<= 1) {
        long long add = t >= off ? s_sum[t - off] : 0;
        __syncthreads();
        s_sum[t] += add;
        __syncthreads();
    }
    long long run = s_sum[t] - local;  // exclusive prefix
    for (int k = beg; k < end; ++k) {
        const int c = cnt[k];
        cnt[k] = (int)(run < (long long)pair_capacity ? run : pair_capacity);
        cursor[k] = 0;
        run += c;
    }
    if (t == SCAN_THREADS - 1) {
        const long long total = s_sum[t];
        if (total > pair_capacity) atomicOr(err, 0x2u);  // LBDEM_DEVERR_PAIR_CAPACITY
        cnt[ntiles] = (int)(total < (long long)pair_capacity ? total : pair_capacity);
    }
}

__global__ void k_fill_pairs(const SphereDev* __restrict__ sph, int n, const int* __restrict__ off,
                             int* __restrict__ cursor, int* __restrict__ list, int pair_capacity, Geom g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SphereDev& s = sph[i];
    if (!s.valid) return;
    const int tny = tiles_along(g.ny), tnz = tiles_along(g.nz);
    for (int tx = s.lo[0] / TILE; tx <= s.hi[0] / TILE; ++tx)
        for (int ty = s.lo[1] / TILE; ty <= s.hi[1] / TILE; ++ty)
            for (int tz = s.lo[2] / TILE; tz <= s.hi[2] / TILE; ++tz) {
                const size_t t = ((size_t)tx * tny + ty) * tnz + tz;
                const int pos = off[t] + atomicAdd(cursor + t, 1);
                if (pos < pair_capacity) list[pos] = i;
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

// One block per tile; 512 threads, one per cell of the 8^3 tile.
// INIT_VEL: defineVelocity (src/ibCompositeDynamics3D.hh:118-127) is applied
// with the uPart the cell holds right after each sphere that covers it fully
// (src/ibProcessors3D.hh:107-108); it depends only on that uPart, so the last
// such sphere decides the populations written.
template <typename T, bool INIT_VEL>
__global__ void __launch_bounds__(TILE_CELLS)
k_voxelize(const SphereDev* __restrict__ sph, const int* __restrict__ off, const int* __restrict__ list,
           uint32_t* __restrict__ vox, T* __restrict__ up, T* __restrict__ f, int phase, Geom g,
           unsigned* __restrict__ err) {
    __shared__ int s_raw[TILE_LIST_MAX];
    __shared__ int s_sorted[TILE_LIST_MAX];
    const int t = blockIdx.x;
    const int beg = off[t];
    const int cnt = off[t + 1] - beg;
    if (cnt <= 0) return;
    if (cnt > TILE_LIST_MAX) {
        if (threadIdx.x == 0) atomicOr(err, 0x1u);  // LBDEM_DEVERR_TILE_LIST
        return;
    }
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) s_raw[k] = list[beg + k];
    __syncthreads();
    // rank sort by sphere index (the indices of one list are distinct)
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
        const int vk = s_raw[k];
        int rank = 0;
        for (int m = 0; m < cnt; ++m) rank += (s_raw[m] < vk) ? 1 : 0;
        s_sorted[rank] = vk;
    }
    __syncthreads();

    const int tny = tiles_along(g.ny), tnz = tiles_along(g.nz);
    const int tx = t / (tny * tnz);
    const int rem = t - tx * tny * tnz;
    const int ty = rem / tnz;
    const int tz = rem - ty * tnz;
    const int lx = threadIdx.x >> 6, ly = (threadIdx.x >> 3) & 7, lz = threadIdx.x & 7;
    const int X = tx * TILE + lx, Y = ty * TILE + ly, Z = tz * TILE + lz;
    if (X >= g.nx || Y >= g.ny || Z >= g.nz) return;
    const size_t c = ((size_t)X * g.ny + Y) * g.nz + Z;

    const uint32_t w0 = vox[c];
    int n_old = (int)(w0 & VOX_NMASK);
    int id_old = (int)(w0 >> VOX_NBITS);
    T u0 = T(0), u1 = T(0), u2 = T(0);
    if (n_old > 0) { u0 = up[c]; u1 = up[g.N + c]; u2 = up[2 * g.N + c]; }
    bool dirty = false, define_vel = false;
    T d0 = T(0), d1 = T(0), d2 = T(0);
    const double xG = (double)X, yG = (double)Y, zG = (double)Z;

    for (int k = 0; k < cnt; ++k) {
        const SphereDev& s = sph[s_sorted[k]];
        if (X < s.lo[0] || X > s.hi[0] || Y < s.lo[1] || Y > s.hi[1] || Z < s.lo[2] || Z > s.hi[2]) continue;
        const double dx = __dsub_rn(xG, s.x[0]);
        const double dy = __dsub_rn(yG, s.x[1]);
        const double dz = __dsub_rn(zG, s.x[2]);
        const int n = solid_count(dx, dy, dz, s.r);
        // decFlag, src/ibProcessors3D.hh:85-105 (sf > 0.001 <=> n > 0; sf > sf_old <=> n > n_old)
        const int dec = (n > 0 ? 1 : 0) + (n_old > 0 ? 2 : 0);
        bool set = false, zero = false;
        if (dec == 1) set = true;
        else if (dec == 2) zero = (id_old == s.tag);
        else if (dec == 3) set = (n > n_old) || (id_old == s.tag);
        // dec == 0 is setToZero on a cell that is already empty
        if (zero) {
            n_old = 0; id_old = 0; u0 = u1 = u2 = T(0); dirty = true;
        } else if (set) {
            // setValues, src/ibProcessors3D.hh:163-174 (com == x for single spheres)
            const double a0 = __dadd_rn(s.v[0], __dsub_rn(__dmul_rn(s.w[1], dz), __dmul_rn(s.w[2], dy)));
            const double a1 = __dadd_rn(s.v[1], __dadd_rn(__dmul_rn(-s.w[0], dz), __dmul_rn(s.w[2], dx)));
            const double a2 = __dadd_rn(s.v[2], __dsub_rn(__dmul_rn(s.w[0], dy), __dmul_rn(s.w[1], dx)));
            u0 = T(a0); u1 = T(a1); u2 = T(a2);
            n_old = n; id_old = s.tag; dirty = true;
        }
        if (INIT_VEL && n == 125) { define_vel = true; d0 = u0; d1 = u1; d2 = u2; }
    }
    if (dirty) {
        vox[c] = (uint32_t)n_old | ((uint32_t)id_old << VOX_NBITS);
        up[c] = u0; up[g.N + c] = u1; up[2 * g.N + c] = u2;
    }
    if (INIT_VEL && define_vel) {
        // f̄_i = feq_i(rhoBar = 0, invRho = 1, j = u)
        const T uSqr = d0 * d0 + d1 * d1 + d2 * d2;
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const T cu = T(cx(i)) * d0 + T(cy(i)) * d1 + T(cz(i)) * d2;
            const T e = T(wt(i)) * (T(3) * cu + (T(4.5) * cu * cu - T(1.5) * uSqr));
            *pop_slot(f, i, X, Y, Z, phase, g) = e;
        }
    }
}

}  // namespace

cudaError_t launch_prepare_spheres(const double* rec, int n, SphereDev* sph, int* tile_count,
                                   int* tag2slot, unsigned* err, Geom g, int max_tag,
                                   double max_radius, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_prepare_spheres<<<(n + 127) / 128, 128, 0, s>>>(rec, n, sph, tile_count, tag2slot, err, g, max_tag,
                                                     max_radius);
    return cudaGetLastError();
}

cudaError_t launch_scan_tiles(int* tile_count, int ntiles, int pair_capacity, int* cursor, unsigned* err,
                              cudaStream_t s) {
    k_scan_tiles<<<1, SCAN_THREADS, 0, s>>>(tile_count, ntiles, pair_capacity, cursor, err);
    return cudaGetLastError();
}

cudaError_t launch_fill_pairs(const SphereDev* sph, int n, const int* tile_off, int* cursor, int* list,
                              int pair_capacity, Geom g, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_fill_pairs<<<(n + 127) / 128, 128, 0, s>>>(sph, n, tile_off, cursor, list, pair_capacity, g);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_voxelize(const SphereDev* sph, const int* tile_off, const int* list, int ntiles,
                            int pair_capacity, uint32_t* vox, T* up, T* f, int init_vel, int odd_phase,
                            Geom g, unsigned* err, cudaStream_t s) {
    (void)pair_capacity;
    if (ntiles <= 0) return cudaSuccess;
    if (init_vel)
        k_voxelize<T, true><<<ntiles, TILE_CELLS, 0, s>>>(sph, tile_off, list, vox, up, f, odd_phase, g, err);
    else
        k_voxelize<T, false><<<ntiles, TILE_CELLS, 0, s>>>(sph, tile_off, list, vox, up, f, odd_phase, g, err);
    return cudaGetLastError();
}

template cudaError_t launch_voxelize<float>(const SphereDev*, const int*, const int*, int, int, uint32_t*,
                                            float*, float*, int, int, Geom, unsigned*, cudaStream_t);
template cudaError_t launch_voxelize<double>(const SphereDev*, const int*, const int*, int, int, uint32_t*,
                                             double*, double*, int, int, Geom, unsigned*, cudaStream_t);

}  // namespace lbdem
