// Internal declarations shared by the CUDA translation units of liblbdem_gb300.
//
// D3Q19 in Palabos ordering (c[i+9] = -c[i], i = 1..9), populations stored as
// f̄_i = f_i - t_i, fields laid out [component][x][y][z] with z fastest.
#pragma once

#include <cstddef>
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

namespace lbdem {

constexpr int Q = 19;
constexpr int TILE = 8;                 // voxelization tile edge (cells)
constexpr int TILE_CELLS = TILE * TILE * TILE;
constexpr int TILE_BIN = 64;            // sphere slots per tile bin
constexpr int TILE_LIST_MAX = 1024;     // spheres per tile when a bin overflows (shared memory)
constexpr int REC_STRIDE = 12;          // doubles per particle record {x3, v3, w3, r, tag, 0}
constexpr int XPF_STRIDE = 16;          // floats per particle of the float table (xpf, see below)
constexpr int VOX_NBITS = 7;            // voxel word: sub-cell count n (7 bits) | tag << 7
constexpr uint32_t VOX_NMASK = (1u << VOX_NBITS) - 1u;
constexpr int32_t MAX_TAG_LIMIT = (1 << 25) - 1;
constexpr int COLLIDE_BLOCK = 128;      // threads per block along z in the collide-stream kernel
constexpr int COLLIDE_SEGW = 64;        // cells per z-segment of the collide-stream kernel

// Lattice velocities, Palabos D3Q19 order.  Each component is stored as
// c + 1 in two bits per direction of a 64-bit constant, so that a lookup with a
// run-time index is a shift and a mask.
namespace lattice_table {
constexpr int cx_of(int i) {
    return (i == 1 || i == 4 || i == 5 || i == 6 || i == 7) ? -1
         : (i == 10 || i == 13 || i == 14 || i == 15 || i == 16) ? 1 : 0;
}
constexpr int cy_of(int i) {
    return (i == 2 || i == 4 || i == 8 || i == 9 || i == 14) ? -1
         : (i == 5 || i == 11 || i == 13 || i == 17 || i == 18) ? 1 : 0;
}
constexpr int cz_of(int i) {
    return (i == 3 || i == 6 || i == 8 || i == 16 || i == 18) ? -1
         : (i == 7 || i == 9 || i == 12 || i == 15 || i == 17) ? 1 : 0;
}
constexpr unsigned long long pack(int axis) {
    unsigned long long p = 0;
    for (int i = 0; i < 19; ++i)
        p |= (unsigned long long)((axis == 0 ? cx_of(i) : axis == 1 ? cy_of(i) : cz_of(i)) + 1) << (2 * i);
    return p;
}
constexpr unsigned long long CX = pack(0), CY = pack(1), CZ = pack(2);
}  // namespace lattice_table
__host__ __device__ constexpr int cx(int i) { return (int)((lattice_table::CX >> (2 * i)) & 3u) - 1; }
__host__ __device__ constexpr int cy(int i) { return (int)((lattice_table::CY >> (2 * i)) & 3u) - 1; }
__host__ __device__ constexpr int cz(int i) { return (int)((lattice_table::CZ >> (2 * i)) & 3u) - 1; }
namespace lattice_table {
constexpr bool same(int i) {
    return i == 19 || (cx(i) == cx_of(i) && cy(i) == cy_of(i) && cz(i) == cz_of(i) && same(i + 1));
}
static_assert(same(0), "packed lattice velocities");
}  // namespace lattice_table
__host__ __device__ constexpr int opp(int i) { return i == 0 ? 0 : (i <= 9 ? i + 9 : i - 9); }
__host__ __device__ constexpr double wt(int i) {
    return i == 0 ? 1.0 / 3.0 : ((i == 1 || i == 2 || i == 3 || i == 10 || i == 11 || i == 12) ? 1.0 / 18.0 : 1.0 / 36.0);
}

struct Geom {
    int nx, ny, nz;
    int per[3];
    size_t N;
};

// Index of the slot that holds population i of cell (x,y,z) in the AA layout.
// phase 0 (even number of completed steps): slot (i, x).
// phase 1: slot (opp i, x - c_i), or (i, x) when x - c_i is beyond a wall.
__device__ __forceinline__ size_t slot_index(int i, int x, int y, int z, int phase, const Geom& g) {
    if (phase == 0 || i == 0) return (size_t)i * g.N + ((size_t)x * g.ny + y) * g.nz + z;
    int X = x - cx(i), Y = y - cy(i), Z = z - cz(i);
    bool out = false;
    if (X < 0 || X >= g.nx) { if (g.per[0]) X = X < 0 ? X + g.nx : X - g.nx; else out = true; }
    if (Y < 0 || Y >= g.ny) { if (g.per[1]) Y = Y < 0 ? Y + g.ny : Y - g.ny; else out = true; }
    if (Z < 0 || Z >= g.nz) { if (g.per[2]) Z = Z < 0 ? Z + g.nz : Z - g.nz; else out = true; }
    if (out) return (size_t)i * g.N + ((size_t)x * g.ny + y) * g.nz + z;
    return (size_t)opp(i) * g.N + ((size_t)X * g.ny + Y) * g.nz + Z;
}

// Position of the k-th set bit (k = 0: the lowest) of m; k < popc(m).
__device__ __forceinline__ int nth_bit(unsigned m, int k) {
    int pos = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const unsigned lo = m & ((1u << w) - 1u);
        const int c = __popc(lo);
        if (k >= c) {
            k -= c;
            m >>= w;
            pos += w;
        } else {
            m = lo;
        }
    }
    return pos;
}

// Arguments of one collide-stream launch.
// Launch shapes cached per device (the SM count, the resident blocks of a kernel
// and its dynamic shared-memory opt-in are properties of one device).
constexpr int LBDEM_MAX_DEVICES = 64;

// Division by an invariant divisor d >= 1 as a multiply-high and a shift, exact
// for numerators below 2^31: with l = ceil(log2 d), s = l - 1 and
// m = ceil(2^(32+s) / d) (< 2^32), n / d = umulhi(n, m) >> s, because
// n m / 2^(31+l) - n / d < n / 2^(31+l) < 2^-l <= 1 / d  (Granlund and
// Montgomery, "Division by invariant integers using multiplication", 1994).
struct DivMagic {
    unsigned m;
    int s;
    unsigned d;
};
inline DivMagic div_magic(unsigned d) {
    DivMagic r{0u, 0, d};
    if (d <= 1) return r;
    int l = 0;
    while ((1ull << l) < d) ++l;
    r.s = l - 1;
    r.m = (unsigned)(((1ull << (32 + r.s)) + d - 1) / d);
    return r;
}
__device__ __forceinline__ unsigned fast_div(unsigned n, const DivMagic& q) {
    return q.d <= 1 ? n : (__umulhi(n, q.m) >> q.s);
}

template <typename T>
struct CollideArgs {
    Geom g;
    T* f;                    // [19][N] populations, AA in-place layout
    T* fo;                   // where the step's output goes: f itself (in place) or a second
                             // array of the same layout (an out-of-place step)
    const uint32_t* vox;     // [N] n | tag << 7
    const T* up;             // [3][N] particle surface velocity
    T* cf;                   // [3][N] per-cell force (nullptr: not kept)
    const int* tag2slot;     // [max_tag + 1] lowest particle index per tag
    const double* rec;       // [n][12] particle records (positions for the torque arm)
    const float* xpf;        // [n][XPF_STRIDE] float table: centre hi/lo, v, omega (float form)
    int nslot;               // particles in the current list
    int max_tag;             // tag2slot has max_tag + 1 entries
    double* ft;              // [6][n]: F (3n) then T (3n)
    unsigned* err;
    const T* btab;           // [126] B(n) = sf ooo / ((1 - sf) + ooo), evaluated in double
    T omega;                 // BGK relaxation frequency
    T g3[3];                 // Guo body-force acceleration
    DivMagic dz, dy;         // division by the z-segments per row and by ny (set by the launchers)
    int probe_timeout;       // test hook: the first wait of every warp runs out (LBDEM_FLAG_PROBE_TIMEOUT)
    // Plane view (FP32 batch, even phase): g describes the domain as nx rows of
    // ny nz cells, so that 64-cell segments run across the z-rows of an x-plane;
    // flat_ny, flat_nz are the true extents and dnz divides by flat_nz.  0: no view.
    int flat_ny, flat_nz;
    DivMagic dnz;
};

// Float table of a particle list, one row of XPF_STRIDE floats per particle:
//   {xh0, xh1, xh2, xl0 | xl1, xl2, v0, v1 | v2, w0, w1, w2 | 0, 0, 0, 0},
// centre = xh + xl (hi/lo split), velocity and angular velocity rounded to float.
// It gives the float form its torque arms and its particle surface velocities.
struct TableRow {
    float4 a, b, c;
};
__device__ __forceinline__ TableRow load_row(const float* __restrict__ xpf, int slot) {
    const float4* p = reinterpret_cast<const float4*>(xpf + (size_t)slot * XPF_STRIDE);
    return TableRow{__ldg(p), __ldg(p + 1), __ldg(p + 2)};
}
//
// Particle surface velocity of cell (x, y, z) in the float form, recomputed from
// the owner particle's row instead of being stored per cell: v + omega x arm,
// arm = cell - centre taken to the nearest image along periodic axes with the
// minimum-image rule of the force sum (integer half extent,
// src/ibProcessors3D.hh:230-243).  setValues (src/ibProcessors3D.hh:163-174)
// stores the same velocity from the image that set the cell; ghost images
// carry their owner's v and omega, and the nearest image is the one that set
// the cell whenever the periodic extent exceeds the sphere's diameter plus
// two cells.  Every operation is rounded on its own, so that all kernels
// that form this velocity agree bit for bit.
__host__ __device__ __forceinline__ float min_image_f(float d, int n, int per) {
    if (!per) return d;
    const int h = n / 2;
    if (d > (float)h) return d - (float)n;
    if (d < (float)-h) return d + (float)n;
    return d;
}
// The row part (x, y fixed) of the velocity: c = v + omega x (dx, dy, 0).
struct RowPart {
    float c0, c1, c2;
};
__device__ __forceinline__ RowPart row_part(const TableRow& r, int x, int y, const Geom& g) {
    const float dx = min_image_f(__fsub_rn(__fsub_rn((float)x, r.a.x), r.a.w), g.nx, g.per[0]);
    const float dy = min_image_f(__fsub_rn(__fsub_rn((float)y, r.a.y), r.b.x), g.ny, g.per[1]);
    // v = (b.z, b.w, c.x), omega = (c.y, c.z, c.w)
    return RowPart{__fsub_rn(r.b.z, __fmul_rn(r.c.w, dy)), __fadd_rn(r.b.w, __fmul_rn(r.c.w, dx)),
                   __fadd_rn(r.c.x, __fsub_rn(__fmul_rn(r.c.y, dy), __fmul_rn(r.c.z, dx)))};
}
// ... plus the z part omega x (0, 0, dz)
__device__ __forceinline__ void cell_part(const TableRow& r, const RowPart& p, int z, const Geom& g, float& u0,
                                          float& u1, float& u2) {
    const float dz = min_image_f(__fsub_rn(__fsub_rn((float)z, r.a.z), r.b.y), g.nz, g.per[2]);
    u0 = __fadd_rn(p.c0, __fmul_rn(r.c.z, dz));
    u1 = __fsub_rn(p.c1, __fmul_rn(r.c.y, dz));
    u2 = p.c2;
}
__device__ __forceinline__ void row_velocity(const TableRow& r, int x, int y, int z, const Geom& g, float& u0,
                                             float& u1, float& u2) {
    cell_part(r, row_part(r, x, y, g), z, g, u0, u1, u2);
}
__device__ __forceinline__ void table_velocity(const float* __restrict__ row, int x, int y, int z, const Geom& g,
                                               float& u0, float& u1, float& u2) {
    const float4* p = reinterpret_cast<const float4*>(row);
    row_velocity(TableRow{__ldg(p), __ldg(p + 1), __ldg(p + 2)}, x, y, z, g, u0, u1, u2);
}
// The owner slot of a voxel word (-1: no solid fraction, or a tag with no particle).
__device__ __forceinline__ int owner_slot(uint32_t w, const int* __restrict__ tag2slot, int max_tag, int nslot) {
    if ((w & VOX_NMASK) == 0u) return -1;
    const int tag = (int)(w >> VOX_NBITS);
    const int slot = tag <= max_tag ? __ldg(tag2slot + tag) : -1;
    return (slot >= 0 && slot < nslot) ? slot : -1;
}

// Exact (double) description of one sphere of the list, for the decisions
// that need the reference's double arithmetic.
struct SphereDev {
    double x[3], v[3], w[3], r;
    double rp2, rm2, rsq;    // (r + sqrt(3.1)/2)^2, (r - sqrt(3.1)/2)^2, r^2 in double
    int tag, valid;
    int lo[3], hi[3];        // bounding box clipped to the lattice (lo > hi: empty)
};

// Float description read by every cell of the voxelization fold.
struct SphereFast {
    float xh[3], xl[3];      // centre = xh + xl
    float rp2, rm2, rsq;     // thresholds rounded to float
    float margin;            // decision band half-width, 2^-19 (r + 4)^2
    int lo[3], hi[3];        // empty box: lo > hi
    int tag;
    float v[3], w[3];        // velocity and angular velocity rounded to float
    int pad;
};
static_assert(sizeof(SphereFast) == 96, "SphereFast is staged as 24 words");

// One domain of a batch as the voxelization kernels see it: its geometry and
// where its data starts in the batch arenas.
struct DomView {
    Geom g;
    int s0;          // first particle slot (slots s0 .. s0 + capacity - 1)
    int t0;          // first voxelization tile
    size_t cell0;    // first cell in the voxel-word arena
    size_t up0;      // first element of the domain's [3][N] particle-velocity block
    size_t f0;       // first element of the domain's [19][N] population block
    size_t tag0;     // first entry of the domain's tag -> slot map
};

// Largest d in [0, n) with off[d] <= idx (off ascending, off[0] <= idx).
__device__ __forceinline__ int find_domain(const int* __restrict__ off, int n, int idx) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= idx) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Population, voxel-word and surface-velocity allocations carry this many bytes
// past their end: the staged collide kernel copies whole 16-byte chunks around
// unaligned rows.
constexpr size_t ALLOC_TAIL = 64;

// Test hook of lbdem_debug_fail_allocation: when positive, the allocation that
// brings it to zero reports failure without being made (device and pinned
// allocations of lbdem_create and lbdem_batch_create).
extern std::atomic<int> g_alloc_fail_countdown;
inline bool alloc_should_fail() {
    int c = g_alloc_fail_countdown.load(std::memory_order_relaxed);
    while (c > 0) {
        if (g_alloc_fail_countdown.compare_exchange_weak(c, c - 1, std::memory_order_relaxed)) return c == 1;
    }
    return false;
}

// Launchers (return cudaGetLastError() of the launch).
template <typename T>
cudaError_t launch_collide_stream(const CollideArgs<T>& a, bool odd, bool force, cudaStream_t s);
// Many domains in one persistent launch: dargs[d] describes domain d, its
// segments (rows of nz cells cut into 64-cell pieces, x-major) are numbered
// from seg0[d]; nseg segments in all.  blocks_per_sm <= 0: as many as fit.
// The FP32 even phase takes plane views (CollideArgs::flat_nz != 0: rows of
// ny nz cells, one per x-plane) with their own seg0 and nseg.
template <typename T>
cudaError_t launch_collide_batch(const CollideArgs<T>* dargs, const int* seg0, int ndom, long long nseg, bool odd,
                                 bool force, int blocks_per_sm, cudaStream_t s);

// Sphere tables (sph, fast, xpf), the tag -> lowest slot map (tag2slot must
// hold "no slot" on entry) and the tile bins, in one launch.  tile_cnt must be
// zero on entry; launch_voxelize leaves it zero again.  Every tile that receives
// a sphere is appended to work[] (work_n counts them; zero on entry, left zero
// by launch_voxelize).  ft_zero (may be null): 6 n doubles set to zero by the
// same launch (the force and torque sums of the next collide-stream step).
// rec_copy (may be null, never overlapping rec): receives a copy of the n records.
cudaError_t launch_prepare_bin(const double* rec, int n, SphereDev* sph, SphereFast* fast, float* xpf,
                               int* tag2slot, unsigned* err, Geom g, int max_tag, double max_radius,
                               double* ft_zero, double* rec_copy, int* tile_cnt, int* bins, int* work, int* work_n,
                               cudaStream_t s);
// The float table and tag map of the list being voxelized (the prepare launch
// fills both); used by defineVelocity in the float form, which keeps no
// surface-velocity field (up == nullptr).
struct OwnerTable {
    const float* xpf;
    const int* tag2slot;
    int max_tag;
};
template <typename T>
cudaError_t launch_voxelize(const SphereDev* sph, const SphereFast* fast, int n, int* tile_cnt, const int* bins,
                            const int* work, int* work_n, int ntiles, uint32_t* vox, T* up, T* f, int init_vel,
                            int odd_phase, Geom g, const OwnerTable& ot, cudaStream_t s);

// Batch forms: particle slots and tiles of all domains in one index space;
// soff[d] = doms[d].s0, toff[d] = doms[d].t0 (ascending); ncur[d] particles of
// domain d are in use (slots s0 .. s0 + ncur[d] - 1); tag2slot holds a
// (max_tag + 1)-entry map per domain, with domain-local slots.
cudaError_t launch_prepare_bin_batch(const double* rec, int nslots, SphereDev* sph, SphereFast* fast, float* xpf,
                                     int* tag2slot, unsigned* err, int max_tag, double max_radius,
                                     const DomView* doms, const int* soff, int ndom, const int* ncur,
                                     double* ft_zero, int* tile_cnt, int* bins, int* work, int* work_n,
                                     cudaStream_t s);
template <typename T>
cudaError_t launch_voxelize_batch(const SphereDev* sph, const SphereFast* fast, int* tile_cnt, const int* bins,
                                  const int* work, int* work_n, int ntiles, uint32_t* vox, T* up, T* f, int init_vel,
                                  int odd_phase, const DomView* doms, const int* toff, int ndom, const int* ncur,
                                  const OwnerTable& ot, cudaStream_t s);

// Field helpers.  phase: number of completed steps mod 2 (storage layout).
template <typename T>
cudaError_t launch_pop_gather(const T* f, T* out, int i, int phase, Geom g, cudaStream_t s);
template <typename T>
cudaError_t launch_pop_scatter(T* f, const T* in, int i, int phase, Geom g, cudaStream_t s);
template <typename T>
cudaError_t launch_fill_equilibrium(T* f, double rho_bar, const double* u, int phase, Geom g, cudaStream_t s);
template <typename T>
cudaError_t launch_macro(const T* f, int phase, double* rho, double* u, Geom g, cudaStream_t s);
template <typename T>
cudaError_t launch_mass(const T* f, double* out, Geom g, cudaStream_t s);
cudaError_t launch_vox_fields(const uint32_t* vox, double* sf, int32_t* id, uint8_t* nsub, Geom g,
                              cudaStream_t s);
// Float form: the particle surface velocity of every cell, [3][N], as the
// collision recomputes it (owner rows of the float table; zero in free cells).
cudaError_t launch_owner_velocity(const uint32_t* vox, const int* tag2slot, int max_tag, int nslot, const float* xpf,
                                  Geom g, float* out, cudaStream_t s);

// One plane (box) of the periodic pressure drop: average density of the box and,
// optionally, the Zhang rescale of the populations entering it.
struct PlaneJob {
    void* f;                 // populations of the domain the box lies in
    Geom g;
    int box[6];              // x0, x1, y0, y1, z0, z1 (inclusive)
    int dim, dir;            // rescaled populations: c_i[dim] == dir
    double target;           // target density of the box
    int read;                // average slot giving rhoAvg of the rescale
    int write;               // average slot receiving this box's average
};
constexpr int PLANE_BLOCKS_MAX = 64;    // blocks per job (partial sums per job)
constexpr int PLANE_THREADS = 256;

// jobs: device table; partial: [njobs][PLANE_BLOCKS_MAX]; count: [njobs], zero on
// entry and left zero; avg_in / avg_out: average slots before / after.  rescale = 0
// only computes the averages (into avg_out).
template <typename T>
cudaError_t launch_plane_pressure(const PlaneJob* jobs, int njobs, int blocks_per_job, int phase, int rescale,
                                  const double* avg_in, double* avg_out, double* partial, unsigned* count,
                                  cudaStream_t s);
// One adjoint step (k_adjoint.cu).
template <typename T>
struct AdjointArgs {
    Geom g;
    const T* f;              // pre-collision populations of the step, AA layout of `phase`
    int phase;
    const T* lam_in;         // adjoint of the populations after the step, natural [19][N]
    T* lam_out;              // adjoint of the populations before the step, natural [19][N]
    const uint32_t* vox;     // voxel words (fixed over the window)
    const int* tag2slot;
    int max_tag, nslot;
    const double* rec;       // [nslot][12] particle records of the step
    const float* xpf;        // [nslot][XPF_STRIDE] float table (float form's arm)
    const double* w;         // [nslot][6] dL/dF, dL/dT of the step
    double* gvel;            // [nslot][6] += dL/dv, dL/domega of the step
    double* gglob;           // [4] += dL/dg, dL/dtau
    const T* btab;           // B(n)
    T omega;
    T tauT;                  // tau = 1 / omega in the lattice type
    T g3[3];
    unsigned* err;
};
template <typename T>
cudaError_t launch_adjoint_step(const AdjointArgs<T>& a, cudaStream_t s);
// loss += sum_p w[p] . (F_p, T_p) of one step
cudaError_t launch_loss_step(const double* ft, const double* w, int n, int nslot, double* loss, cudaStream_t s);

// Equilibrium initial profiles, src/periodicPressureFunctionals3D.hh:242-298:
// kind 0 pressure gradient, kind 1 Poiseuille profile plus pressure gradient.
template <typename T>
cudaError_t launch_init_profile(T* f, int phase, int kind, double p_hi, double p_lo, double u_max, int n0, int n1,
                                int n2, int dim, Geom g, cudaStream_t s);

}  // namespace lbdem
