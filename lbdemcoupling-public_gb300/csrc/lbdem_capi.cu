// C ABI of liblbdem_gb300: handle life cycle, device memory, staging buffers
// and the launch sequence of one coupling cycle.  See include/lbdem_gpu.h.
#include "lbdem_gpu.h"
#include "lbdem_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <utility>
#include <vector>

using namespace lbdem;

namespace lbdem {
std::atomic<int> g_alloc_fail_countdown{0};
}

namespace {
// Pinned host allocation through the allocation-failure test hook.
template <typename P>
cudaError_t halloc(P** p, size_t bytes) {
    if (alloc_should_fail()) return cudaErrorMemoryAllocation;
    return cudaMallocHost((void**)p, bytes);
}
}  // namespace

struct lbdem_handle {
    lbdem_config cfg{};
    Geom g{};
    int prec = 0;
    size_t esz = 8;
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;

    void* f = nullptr;          // [19][N] populations
    uint32_t* vox = nullptr;    // [N] n | tag << 7
    void* up = nullptr;         // [3][N] particle surface velocity (FP64 form only; the FP32
                                // form recomputes it from the owner particle)
    void* cf = nullptr;         // [3][N] optional
    double* btab = nullptr;     // [126] B(n), double
    float* btabf = nullptr;     // [126] B(n) rounded to float

    int cap = 0;
    double* d_rec = nullptr;    // [cap][12]
    SphereDev* d_sph = nullptr; // [cap]
    SphereFast* d_fast = nullptr; // [cap]
    float* d_xpf = nullptr;     // [cap][XPF_STRIDE]
    int* d_tag2slot = nullptr;  // [max_tag + 1]
    int ntiles = 0;
    int* d_tile_cnt = nullptr;  // [ntiles] spheres binned per tile (zero between calls)
    int* d_bins = nullptr;      // [ntiles][TILE_BIN]
    int* d_work = nullptr;      // [ntiles] tiles with spheres (voxelization work list)
    int* d_work_n = nullptr;    // [4] work-list counters (zero between calls)
    double* d_ft = nullptr;     // [6][cap]
    unsigned* d_err = nullptr;
    double* d_mass = nullptr;

    double* h_rec = nullptr;    // pinned staging
    double* h_ft = nullptr;
    unsigned* h_err = nullptr;
    cudaEvent_t ev_staged = nullptr;
    bool staged_pending = false;

    // periodic pressure drop: plane jobs 0 (inlet) and 1 (outlet) of the fused
    // mode, job 2 for the single-box calls; average slots [2 parities][4]:
    // 0 inlet, 1 outlet, 2 single-box result, 3 single-box given average
    PlaneJob* d_jobs = nullptr;
    double* d_pavg = nullptr;
    double* d_ppart = nullptr;  // [3][PLANE_BLOCKS_MAX]
    unsigned* d_pcount = nullptr; // [3]
    double* h_pavg = nullptr;   // pinned
    bool pdrop_on = false;
    bool pavg_valid = false;
    bool ft_dirty = false;      // d_ft holds sums of a step (zeroed by the next voxelization)
    int pdrop_bpj = 1;

    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    size_t dev_bytes = 0;

    float adj_fwd_ms = 0.f, adj_bwd_ms = 0.f;

    int n_cur = 0;
    int64_t step = 0;
    int64_t launches = 0;
    std::string last_error;
};

namespace {

// Restores the caller's current device on scope exit.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

lbdem_status fail(lbdem_handle* h, lbdem_status s, const std::string& msg) {
    if (h) h->last_error = msg;
    return s;
}

lbdem_status fail_cuda(lbdem_handle* h, const char* what, cudaError_t e) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(h, e == cudaErrorMemoryAllocation ? LBDEM_ERR_OUT_OF_MEMORY : LBDEM_ERR_CUDA, m);
}

#define CK(h, call)                                              \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return fail_cuda((h), #call, e_); \
    } while (0)

template <typename P>
cudaError_t dalloc(lbdem_handle* h, P** p, size_t bytes) {
    void* q = nullptr;
    if (alloc_should_fail()) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(&q, bytes == 0 ? 16 : bytes);
    if (e == cudaSuccess) {
        *p = (P*)q;
        h->dev_bytes += bytes;
    }
    return e;
}

void release(lbdem_handle* h) {
    void* dev[] = {h->f, h->vox, h->up, h->cf, h->btab, h->btabf, h->d_rec, h->d_sph, h->d_fast, h->d_xpf, h->d_tag2slot,
                   h->d_tile_cnt, h->d_bins, h->d_work, h->d_work_n, h->d_ft, h->d_err, h->d_mass, h->scratch, h->d_jobs, h->d_pavg,
                   h->d_ppart, h->d_pcount};
    for (void* p : dev)
        if (p) cudaFree(p);
    void* host[] = {h->h_rec, h->h_ft, h->h_err, h->h_pavg};
    for (void* p : host)
        if (p) cudaFreeHost(p);
    if (h->ev_staged) cudaEventDestroy(h->ev_staged);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
}

lbdem_status ensure_scratch(lbdem_handle* h, size_t bytes) {
    if (h->scratch_bytes >= bytes) return LBDEM_OK;
    if (h->scratch) {
        cudaFree(h->scratch);
        h->dev_bytes -= h->scratch_bytes;
        h->scratch = nullptr;
        h->scratch_bytes = 0;
    }
    CK(h, dalloc(h, &h->scratch, bytes));
    h->scratch_bytes = bytes;
    return LBDEM_OK;
}

lbdem_status wait_staging(lbdem_handle* h) {
    if (h->staged_pending) {
        CK(h, cudaEventSynchronize(h->ev_staged));
        h->staged_pending = false;
    }
    return LBDEM_OK;
}

// Voxelization of n records read from src (h->d_rec, or a device table of the
// caller that the prepare launch copies into h->d_rec as it reads it).
lbdem_status voxelize(lbdem_handle* h, int n, int init_vel, const double* src) {
    cudaStream_t s = h->stream;
    // defineVelocity reads the velocity a covered cell held before this pass.  The
    // FP32 form keeps no velocity field: rebuild it, as the collision saw it, from
    // the previous list's tables before the prepare launch replaces them.
    float* up_before = nullptr;
    if (init_vel && n > 0 && h->prec == LBDEM_PREC_FP32_DEV) {
        lbdem_status st = ensure_scratch(h, 3 * h->g.N * sizeof(float));
        if (st != LBDEM_OK) return st;
        up_before = (float*)h->scratch;
        CK(h, launch_owner_velocity(h->vox, h->d_tag2slot, h->cfg.max_tag, h->n_cur, h->d_xpf, h->g, up_before, s));
        h->launches += 1;
    }
    CK(h, cudaMemsetAsync(h->d_tag2slot, 0x7F, sizeof(int) * ((size_t)h->cfg.max_tag + 1), s));
    if (n > 0) {
        CK(h, launch_prepare_bin(src, n, h->d_sph, h->d_fast, h->d_xpf, h->d_tag2slot, h->d_err, h->g,
                                 h->cfg.max_tag, h->cfg.max_radius, h->d_ft, src == h->d_rec ? nullptr : h->d_rec,
                                 h->d_tile_cnt, h->d_bins, h->d_work, h->d_work_n, s));
        h->ft_dirty = false;   // the prepare launch zeroed the 6 n sums
        const int phase = (int)(h->step & 1);
        if (h->prec == LBDEM_PREC_FP64)
            CK(h, launch_voxelize<double>(h->d_sph, h->d_fast, n, h->d_tile_cnt, h->d_bins, h->d_work, h->d_work_n,
                                          h->ntiles, h->vox, (double*)h->up, (double*)h->f, init_vel, phase, h->g,
                                          OwnerTable{h->d_xpf, h->d_tag2slot, h->cfg.max_tag}, s));
        else
            CK(h, launch_voxelize<float>(h->d_sph, h->d_fast, n, h->d_tile_cnt, h->d_bins, h->d_work, h->d_work_n,
                                         h->ntiles, h->vox, up_before, (float*)h->f, init_vel, phase, h->g,
                                         OwnerTable{h->d_xpf, h->d_tag2slot, h->cfg.max_tag}, s));
        h->launches += 2;
        if (init_vel) h->pavg_valid = false;
    }
    h->n_cur = n;
    return LBDEM_OK;
}

// B(n) = sf ooo / ((1 - sf) + ooo), sf = n/125, ooo = 1/omega - 1/2
// (src/ibCompositeDynamics3D.hh:178-179); n = 125 is the full-solid branch, B = 1.
// Synchronous copies of the handle's omega into both tables.
cudaError_t upload_btab(lbdem_handle* h) {
    double bt[126];
    const double ooo = 1. / h->cfg.omega - 0.5;
    for (int n = 0; n < 126; ++n) {
        const double sf = (1. / 125.) * (double)n;
        bt[n] = sf * ooo / ((1. - sf) + ooo);
    }
    bt[0] = 0.0;
    bt[125] = 1.0;
    cudaError_t e = cudaMemcpy(h->btab, bt, sizeof(bt), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    float btf[126];
    for (int n = 0; n < 126; ++n) btf[n] = (float)bt[n];
    return cudaMemcpy(h->btabf, btf, sizeof(btf), cudaMemcpyHostToDevice);
}

bool box_ok(const lbdem_handle* h, const int32_t* b) {
    const int ext[3] = {h->g.nx, h->g.ny, h->g.nz};
    for (int d = 0; d < 3; ++d)
        if (b[2 * d] < 0 || b[2 * d + 1] >= ext[d] || b[2 * d] > b[2 * d + 1]) return false;
    return true;
}

long long box_cells(const int32_t* b) {
    return (long long)(b[1] - b[0] + 1) * (b[3] - b[2] + 1) * (b[5] - b[4] + 1);
}

int plane_blocks(long long cells) {
    long long b = (cells + 2 * PLANE_THREADS - 1) / (2 * PLANE_THREADS);
    return (int)std::max(1LL, std::min<long long>(b, PLANE_BLOCKS_MAX));
}

PlaneJob make_job(const lbdem_handle* h, const int32_t* box, int dim, int dir, double target, int read, int write) {
    PlaneJob j;
    j.f = h->f;
    j.g = h->g;
    for (int k = 0; k < 6; ++k) j.box[k] = box[k];
    j.dim = dim;
    j.dir = dir;
    j.target = target;
    j.read = read;
    j.write = write;
    return j;
}

// One collide-stream launch of the handle reading populations fin and writing
// fout (fin == fout: the in-place step; otherwise an out-of-place step into an
// array of the same layout).  Particle state, force sums and the step parity
// are the handle's.
cudaError_t k1_launch(lbdem_handle* h, void* fin, void* fout) {
    h->ft_dirty = true;
    const bool odd = (h->step & 1) != 0;
    const bool force = h->cfg.body_force[0] != 0.0 || h->cfg.body_force[1] != 0.0 || h->cfg.body_force[2] != 0.0;
    const int n = h->n_cur;
    if (h->prec == LBDEM_PREC_FP64) {
        CollideArgs<double> a;
        a.g = h->g; a.f = (double*)fin; a.fo = (double*)fout; a.vox = h->vox; a.up = (const double*)h->up;
        a.cf = (double*)h->cf; a.tag2slot = h->d_tag2slot; a.rec = h->d_rec; a.xpf = h->d_xpf; a.nslot = n;
        a.max_tag = h->cfg.max_tag; a.ft = h->d_ft; a.err = h->d_err; a.btab = h->btab; a.omega = h->cfg.omega;
        a.probe_timeout = (h->cfg.flags & LBDEM_FLAG_PROBE_TIMEOUT) ? 1 : 0;
        for (int d = 0; d < 3; ++d) a.g3[d] = h->cfg.body_force[d];
        return launch_collide_stream<double>(a, odd, force, h->stream);
    }
    CollideArgs<float> a;
    a.g = h->g; a.f = (float*)fin; a.fo = (float*)fout; a.vox = h->vox; a.up = nullptr;
    a.cf = (float*)h->cf; a.tag2slot = h->d_tag2slot; a.rec = h->d_rec; a.xpf = h->d_xpf; a.nslot = n;
    a.max_tag = h->cfg.max_tag; a.ft = h->d_ft; a.err = h->d_err; a.btab = h->btabf; a.omega = (float)h->cfg.omega;
    a.probe_timeout = (h->cfg.flags & LBDEM_FLAG_PROBE_TIMEOUT) ? 1 : 0;
    for (int d = 0; d < 3; ++d) a.g3[d] = (float)h->cfg.body_force[d];
    return launch_collide_stream<float>(a, odd, force, h->stream);
}

cudaError_t plane_launch(lbdem_handle* h, const PlaneJob* jobs, int njobs, int bpj, int phase, int rescale,
                         const double* avg_in, double* avg_out) {
    if (h->prec == LBDEM_PREC_FP64)
        return launch_plane_pressure<double>(jobs, njobs, bpj, phase, rescale, avg_in, avg_out, h->d_ppart,
                                             h->d_pcount, h->stream);
    return launch_plane_pressure<float>(jobs, njobs, bpj, phase, rescale, avg_in, avg_out, h->d_ppart, h->d_pcount,
                                        h->stream);
}

}  // namespace

extern "C" {

void lbdem_debug_fail_allocation(int32_t nth) { g_alloc_fail_countdown.store(nth > 0 ? nth : 0); }

void lbdem_config_default(lbdem_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->nx = c->ny = c->nz = 32;
    c->periodic[0] = c->periodic[1] = c->periodic[2] = 1;
    c->omega = 1.0;
    c->precision = LBDEM_PREC_FP64;
    c->device = 0;
    c->max_particles = 1024;
    c->max_tag = 1 << 20;
    c->max_radius = 16.0;
    c->flags = 0;
}

const char* lbdem_status_string(lbdem_status s) {
    switch (s) {
        case LBDEM_OK: return "ok";
        case LBDEM_ERR_INVALID_ARG: return "invalid argument";
        case LBDEM_ERR_CUDA: return "CUDA error";
        case LBDEM_ERR_OUT_OF_MEMORY: return "out of memory";
        case LBDEM_ERR_CAPACITY: return "capacity exceeded";
        case LBDEM_ERR_DEVICE: return "device error word set";
        case LBDEM_ERR_NO_DEVICE: return "no suitable CUDA device";
    }
    return "unknown status";
}

const char* lbdem_last_error(const lbdem_handle* h) { return h ? h->last_error.c_str() : "null handle"; }

lbdem_status lbdem_create(const lbdem_config* cfg, lbdem_handle** out) {
    if (!cfg || !out) return LBDEM_ERR_INVALID_ARG;
    *out = nullptr;
    const lbdem_config& c = *cfg;
    if (c.nx <= 0 || c.ny <= 0 || c.nz <= 0) return LBDEM_ERR_INVALID_ARG;
    if (!(c.omega > 0.0 && c.omega < 2.0)) return LBDEM_ERR_INVALID_ARG;
    if (c.precision != LBDEM_PREC_FP64 && c.precision != LBDEM_PREC_FP32_DEV) return LBDEM_ERR_INVALID_ARG;
    if (c.max_particles < 0 || c.max_tag < 1 || c.max_tag > MAX_TAG_LIMIT) return LBDEM_ERR_INVALID_ARG;
    if (!(c.max_radius > 0.0 && c.max_radius <= 1024.0)) return LBDEM_ERR_INVALID_ARG;
    for (int d = 0; d < 3; ++d)
        if (c.periodic[d] != 0 && c.periodic[d] != 1) return LBDEM_ERR_INVALID_ARG;
    if (!std::isfinite(c.body_force[0]) || !std::isfinite(c.body_force[1]) || !std::isfinite(c.body_force[2]))
        return LBDEM_ERR_INVALID_ARG;
    const size_t N = (size_t)c.nx * c.ny * c.nz;
    if ((size_t)c.nx * c.ny > 0x7fffffffu) return LBDEM_ERR_INVALID_ARG;
    // cell coordinates must be exact in float (voxelization filter, float torque arm)
    if (c.nx >= (1 << 24) || c.ny >= (1 << 24) || c.nz >= (1 << 24)) return LBDEM_ERR_INVALID_ARG;

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0 || c.device < 0 || c.device >= ndev) {
        cudaGetLastError();
        return LBDEM_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, c.device) != cudaSuccess) return LBDEM_ERR_NO_DEVICE;
    // The library carries sm_103a code only.
    if (!(prop.major == 10 && prop.minor == 3)) return LBDEM_ERR_NO_DEVICE;

    lbdem_handle* h = new (std::nothrow) lbdem_handle();
    if (!h) return LBDEM_ERR_OUT_OF_MEMORY;
    h->cfg = c;
    h->device = c.device;
    h->prec = c.precision;
    h->esz = c.precision == LBDEM_PREC_FP64 ? 8 : 4;
    h->g.nx = c.nx; h->g.ny = c.ny; h->g.nz = c.nz;
    for (int d = 0; d < 3; ++d) h->g.per[d] = c.periodic[d];
    h->g.N = N;
    h->cap = c.max_particles;
    const int tnx = (c.nx + TILE - 1) / TILE, tny = (c.ny + TILE - 1) / TILE, tnz = (c.nz + TILE - 1) / TILE;
    if ((long long)tnx * tny * tnz > 0x7fffffffLL) {
        delete h;
        return LBDEM_ERR_INVALID_ARG;
    }
    h->ntiles = tnx * tny * tnz;

    DeviceGuard dg(h->device);
    auto bail = [&](lbdem_status s) {
        release(h);
        delete h;
        return s;
    };
    cudaError_t e;
#define TRY(call)                                   \
    if ((e = (call)) != cudaSuccess) {              \
        cudaGetLastError();                         \
        return bail(e == cudaErrorMemoryAllocation ? LBDEM_ERR_OUT_OF_MEMORY : LBDEM_ERR_CUDA); \
    }
    TRY(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking));
    h->stream = h->own_stream;
    TRY(cudaEventCreateWithFlags(&h->ev_staged, cudaEventDisableTiming));
    TRY(dalloc(h, &h->f, (size_t)Q * N * h->esz + ALLOC_TAIL));
    TRY(dalloc(h, &h->vox, N * sizeof(uint32_t) + ALLOC_TAIL));
    if (h->prec == LBDEM_PREC_FP64) TRY(dalloc(h, &h->up, 3 * N * h->esz + ALLOC_TAIL));
    if (c.flags & LBDEM_FLAG_CELL_FORCE) TRY(dalloc(h, &h->cf, 3 * N * h->esz));
    TRY(dalloc(h, &h->btab, 126 * sizeof(double)));
    TRY(dalloc(h, &h->btabf, 126 * sizeof(float)));
    const size_t capn = (size_t)(h->cap > 0 ? h->cap : 1);
    TRY(dalloc(h, &h->d_rec, capn * REC_STRIDE * sizeof(double)));
    TRY(dalloc(h, &h->d_sph, capn * sizeof(SphereDev)));
    TRY(dalloc(h, &h->d_fast, capn * sizeof(SphereFast)));
    TRY(dalloc(h, &h->d_xpf, capn * XPF_STRIDE * sizeof(float)));
    TRY(dalloc(h, &h->d_tag2slot, ((size_t)c.max_tag + 1) * sizeof(int)));
    TRY(dalloc(h, &h->d_tile_cnt, (size_t)h->ntiles * sizeof(int)));
    TRY(dalloc(h, &h->d_bins, (size_t)h->ntiles * TILE_BIN * sizeof(int)));
    TRY(cudaMemset(h->d_tile_cnt, 0, (size_t)h->ntiles * sizeof(int)));
    TRY(dalloc(h, &h->d_work, (size_t)h->ntiles * sizeof(int)));
    TRY(dalloc(h, &h->d_work_n, 4 * sizeof(int)));
    TRY(cudaMemset(h->d_work_n, 0, 4 * sizeof(int)));
    TRY(dalloc(h, &h->d_ft, 6 * capn * sizeof(double)));
    TRY(dalloc(h, &h->d_err, sizeof(unsigned)));
    TRY(dalloc(h, &h->d_mass, sizeof(double)));
    TRY(halloc(&h->h_rec, capn * REC_STRIDE * sizeof(double)));
    TRY(halloc(&h->h_ft, 6 * capn * sizeof(double)));
    TRY(halloc(&h->h_err, sizeof(unsigned)));
    TRY(dalloc(h, &h->d_jobs, 3 * sizeof(PlaneJob)));
    TRY(dalloc(h, &h->d_pavg, 8 * sizeof(double)));
    TRY(dalloc(h, &h->d_ppart, 3 * PLANE_BLOCKS_MAX * sizeof(double)));
    TRY(dalloc(h, &h->d_pcount, 3 * sizeof(unsigned)));
    TRY(cudaMemset(h->d_pcount, 0, 3 * sizeof(unsigned)));
    TRY(cudaMemset(h->d_pavg, 0, 8 * sizeof(double)));
    TRY(halloc(&h->h_pavg, sizeof(double)));

    TRY(upload_btab(h));
    TRY(cudaMemset(h->f, 0, (size_t)Q * N * h->esz));   // f̄ = 0: rho = 1, u = 0
    TRY(cudaMemset(h->vox, 0, N * sizeof(uint32_t)));
    if (h->up) TRY(cudaMemset(h->up, 0, 3 * N * h->esz));
    if (h->cf) TRY(cudaMemset(h->cf, 0, 3 * N * h->esz));
    TRY(cudaMemset(h->d_tag2slot, 0x7F, ((size_t)c.max_tag + 1) * sizeof(int)));
    TRY(cudaMemset(h->d_ft, 0, 6 * capn * sizeof(double)));
    TRY(cudaMemset(h->d_err, 0, sizeof(unsigned)));
    TRY(cudaDeviceSynchronize());
#undef TRY
    *out = h;
    return LBDEM_OK;
}

lbdem_status lbdem_destroy(lbdem_handle* h) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    {
        DeviceGuard dg(h->device);
        cudaStreamSynchronize(h->stream);
        release(h);
    }
    delete h;
    return LBDEM_OK;
}

lbdem_status lbdem_set_stream(lbdem_handle* h, void* stream) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    DeviceGuard dg(h->device);
    CK(h, cudaStreamSynchronize(h->stream));
    h->stream = stream ? (cudaStream_t)stream : h->own_stream;
    return LBDEM_OK;
}

lbdem_status lbdem_synchronize(lbdem_handle* h) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    DeviceGuard dg(h->device);
    CK(h, cudaStreamSynchronize(h->stream));
    return LBDEM_OK;
}

lbdem_status lbdem_init_equilibrium(lbdem_handle* h, double rho_bar, const double u[3]) {
    if (!h || !u) return fail(h, LBDEM_ERR_INVALID_ARG, "init_equilibrium: null argument");
    if (!(rho_bar > -1.0) || !std::isfinite(rho_bar)) return fail(h, LBDEM_ERR_INVALID_ARG, "rho_bar <= -1");
    DeviceGuard dg(h->device);
    const int phase = (int)(h->step & 1);
    if (h->prec == LBDEM_PREC_FP64)
        CK(h, launch_fill_equilibrium<double>((double*)h->f, rho_bar, u, phase, h->g, h->stream));
    else
        CK(h, launch_fill_equilibrium<float>((float*)h->f, rho_bar, u, phase, h->g, h->stream));
    h->launches += 1;
    h->pavg_valid = false;
    return LBDEM_OK;
}

lbdem_status lbdem_set_populations(lbdem_handle* h, const void* host_f) {
    if (!h || !host_f) return fail(h, LBDEM_ERR_INVALID_ARG, "set_populations: null argument");
    DeviceGuard dg(h->device);
    lbdem_status st = ensure_scratch(h, h->g.N * h->esz);
    if (st != LBDEM_OK) return st;
    const int phase = (int)(h->step & 1);
    for (int i = 0; i < Q; ++i) {
        const char* src = (const char*)host_f + (size_t)i * h->g.N * h->esz;
        CK(h, cudaMemcpyAsync(h->scratch, src, h->g.N * h->esz, cudaMemcpyHostToDevice, h->stream));
        if (h->prec == LBDEM_PREC_FP64)
            CK(h, launch_pop_scatter<double>((double*)h->f, (const double*)h->scratch, i, phase, h->g, h->stream));
        else
            CK(h, launch_pop_scatter<float>((float*)h->f, (const float*)h->scratch, i, phase, h->g, h->stream));
        h->launches += 1;
    }
    CK(h, cudaStreamSynchronize(h->stream));
    h->pavg_valid = false;
    return LBDEM_OK;
}

lbdem_status lbdem_get_populations(lbdem_handle* h, void* host_f) {
    return lbdem_get_field(h, LBDEM_FIELD_POPULATIONS, host_f);
}

lbdem_status lbdem_set_particles(lbdem_handle* h, int32_t n, const double* x, const double* v, const double* w,
                                 const double* r, const int32_t* tag, int32_t init_vel) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    if (n < 0) return fail(h, LBDEM_ERR_INVALID_ARG, "set_particles: n < 0");
    if (n > h->cap) return fail(h, LBDEM_ERR_CAPACITY, "set_particles: n exceeds max_particles");
    if (n > 0 && (!x || !v || !w || !r || !tag)) return fail(h, LBDEM_ERR_INVALID_ARG, "set_particles: null array");
    DeviceGuard dg(h->device);
    lbdem_status st = wait_staging(h);
    if (st != LBDEM_OK) return st;
    for (int i = 0; i < n; ++i) {
        double* p = h->h_rec + (size_t)i * REC_STRIDE;
        p[0] = x[3 * i]; p[1] = x[3 * i + 1]; p[2] = x[3 * i + 2];
        p[3] = v[3 * i]; p[4] = v[3 * i + 1]; p[5] = v[3 * i + 2];
        p[6] = w[3 * i]; p[7] = w[3 * i + 1]; p[8] = w[3 * i + 2];
        p[9] = r[i];
        p[10] = (double)tag[i];
        p[11] = 0.0;
    }
    if (n > 0) {
        CK(h, cudaMemcpyAsync(h->d_rec, h->h_rec, (size_t)n * REC_STRIDE * sizeof(double), cudaMemcpyHostToDevice,
                              h->stream));
        CK(h, cudaEventRecord(h->ev_staged, h->stream));
        h->staged_pending = true;
    }
    return voxelize(h, n, init_vel, h->d_rec);
}

lbdem_status lbdem_set_particles_device(lbdem_handle* h, int32_t n, const double* rec, int32_t init_vel) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    if (n < 0) return fail(h, LBDEM_ERR_INVALID_ARG, "set_particles_device: n < 0");
    if (n > h->cap) return fail(h, LBDEM_ERR_CAPACITY, "set_particles_device: n exceeds max_particles");
    if (n > 0 && !rec) return fail(h, LBDEM_ERR_INVALID_ARG, "set_particles_device: null table");
    DeviceGuard dg(h->device);
    // a table overlapping the handle's own (other than being it) cannot be read and copied in one pass
    const uintptr_t a = (uintptr_t)rec, b = (uintptr_t)h->d_rec, len = (uintptr_t)n * REC_STRIDE * sizeof(double);
    if (n > 0 && a != b && a < b + len && b < a + len)
        return fail(h, LBDEM_ERR_INVALID_ARG, "set_particles_device: table overlaps the handle's particle table");
    return voxelize(h, n, init_vel, rec);
}

lbdem_status lbdem_collide_and_stream(lbdem_handle* h) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    DeviceGuard dg(h->device);
    const int n = h->n_cur;
    // the sums start from zero: the voxelization of this list zeroed them unless
    // a step has run since
    if (n > 0 && h->ft_dirty) CK(h, cudaMemsetAsync(h->d_ft, 0, 6 * (size_t)n * sizeof(double), h->stream));
    const int P = (int)(h->step & 1);
    if (h->pdrop_on && !h->pavg_valid) {
        // averages of the state before the step (computeAverageDensity before collideAndStream)
        CK(h, plane_launch(h, h->d_jobs, 2, h->pdrop_bpj, P, 0, nullptr, h->d_pavg + 4 * P));
        h->launches += 1;
    }
    CK(h, k1_launch(h, h->f, h->f));
    h->launches += 1;
    if (h->pdrop_on) {
        // rescale of the streamed populations with the pre-step averages; the same
        // pass leaves the averages of the new state for the next step
        CK(h, plane_launch(h, h->d_jobs, 2, h->pdrop_bpj, P ^ 1, 1, h->d_pavg + 4 * P, h->d_pavg + 4 * (P ^ 1)));
        h->launches += 1;
        h->pavg_valid = true;
    }
    h->step += 1;
    return LBDEM_OK;
}

lbdem_status lbdem_get_forces(lbdem_handle* h, int32_t n, double* force, double* torque) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    if (n != h->n_cur) return fail(h, LBDEM_ERR_INVALID_ARG, "get_forces: n differs from the particle list");
    if (n > 0 && (!force || !torque)) return fail(h, LBDEM_ERR_INVALID_ARG, "get_forces: null output");
    DeviceGuard dg(h->device);
    if (n > 0)
        CK(h, cudaMemcpyAsync(h->h_ft, h->d_ft, 6 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(h->h_err, h->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->staged_pending = false;
    if (n > 0) {
        std::memcpy(force, h->h_ft, 3 * (size_t)n * sizeof(double));
        std::memcpy(torque, h->h_ft + 3 * (size_t)n, 3 * (size_t)n * sizeof(double));
    }
    if (*h->h_err) {
        char buf[96];
        std::snprintf(buf, sizeof(buf), "device error word 0x%x", *h->h_err);
        return fail(h, LBDEM_ERR_DEVICE, buf);
    }
    return LBDEM_OK;
}

lbdem_status lbdem_get_forces_device(lbdem_handle* h, int32_t n, double* dev_ft) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    if (n != h->n_cur) return fail(h, LBDEM_ERR_INVALID_ARG, "get_forces_device: n differs from the particle list");
    if (n > 0 && !dev_ft) return fail(h, LBDEM_ERR_INVALID_ARG, "get_forces_device: null output");
    DeviceGuard dg(h->device);
    if (n > 0)
        CK(h, cudaMemcpyAsync(dev_ft, h->d_ft, 6 * (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    return LBDEM_OK;
}

lbdem_status lbdem_cycle(lbdem_handle* h, int32_t n, const double* x, const double* v, const double* w,
                         const double* r, const int32_t* tag, int32_t init_vel, double* force, double* torque) {
    lbdem_status s = lbdem_set_particles(h, n, x, v, w, r, tag, init_vel);
    if (s != LBDEM_OK) return s;
    s = lbdem_collide_and_stream(h);
    if (s != LBDEM_OK) return s;
    return lbdem_get_forces(h, n, force, torque);
}

lbdem_status lbdem_get_field(lbdem_handle* h, int32_t which, void* host_buf) {
    if (!h || !host_buf) return fail(h, LBDEM_ERR_INVALID_ARG, "get_field: null argument");
    DeviceGuard dg(h->device);
    const size_t N = h->g.N;
    const int phase = (int)(h->step & 1);
    cudaStream_t s = h->stream;
    lbdem_status st;
    switch (which) {
        case LBDEM_FIELD_POPULATIONS:
            if ((st = ensure_scratch(h, N * h->esz)) != LBDEM_OK) return st;
            for (int i = 0; i < Q; ++i) {
                if (h->prec == LBDEM_PREC_FP64)
                    CK(h, launch_pop_gather<double>((const double*)h->f, (double*)h->scratch, i, phase, h->g, s));
                else
                    CK(h, launch_pop_gather<float>((const float*)h->f, (float*)h->scratch, i, phase, h->g, s));
                h->launches += 1;
                CK(h, cudaMemcpyAsync((char*)host_buf + (size_t)i * N * h->esz, h->scratch, N * h->esz,
                                      cudaMemcpyDeviceToHost, s));
            }
            break;
        case LBDEM_FIELD_SOLID_FRACTION:
        case LBDEM_FIELD_PARTICLE_ID:
        case LBDEM_FIELD_SUBCELL_COUNT: {
            if ((st = ensure_scratch(h, N * sizeof(double))) != LBDEM_OK) return st;
            double* sf = which == LBDEM_FIELD_SOLID_FRACTION ? (double*)h->scratch : nullptr;
            int32_t* id = which == LBDEM_FIELD_PARTICLE_ID ? (int32_t*)h->scratch : nullptr;
            uint8_t* ns = which == LBDEM_FIELD_SUBCELL_COUNT ? (uint8_t*)h->scratch : nullptr;
            CK(h, launch_vox_fields(h->vox, sf, id, ns, h->g, s));
            h->launches += 1;
            const size_t bytes = which == LBDEM_FIELD_SOLID_FRACTION ? N * 8 : which == LBDEM_FIELD_PARTICLE_ID ? N * 4 : N;
            CK(h, cudaMemcpyAsync(host_buf, h->scratch, bytes, cudaMemcpyDeviceToHost, s));
            break;
        }
        case LBDEM_FIELD_PARTICLE_VELOCITY:
            if (h->up) {
                CK(h, cudaMemcpyAsync(host_buf, h->up, 3 * N * h->esz, cudaMemcpyDeviceToHost, s));
            } else {   // FP32 form: recomputed from the owner particles of the current list
                if ((st = ensure_scratch(h, 3 * N * sizeof(float))) != LBDEM_OK) return st;
                CK(h, launch_owner_velocity(h->vox, h->d_tag2slot, h->cfg.max_tag, h->n_cur, h->d_xpf, h->g,
                                            (float*)h->scratch, s));
                h->launches += 1;
                CK(h, cudaMemcpyAsync(host_buf, h->scratch, 3 * N * sizeof(float), cudaMemcpyDeviceToHost, s));
            }
            break;
        case LBDEM_FIELD_HYDRO_FORCE:
            if (!h->cf) return fail(h, LBDEM_ERR_INVALID_ARG, "get_field: create with LBDEM_FLAG_CELL_FORCE");
            CK(h, cudaMemcpyAsync(host_buf, h->cf, 3 * N * h->esz, cudaMemcpyDeviceToHost, s));
            break;
        case LBDEM_FIELD_DENSITY:
        case LBDEM_FIELD_VELOCITY: {
            const bool vel = which == LBDEM_FIELD_VELOCITY;
            if ((st = ensure_scratch(h, (vel ? 3 : 1) * N * sizeof(double))) != LBDEM_OK) return st;
            if (h->prec == LBDEM_PREC_FP64)
                CK(h, launch_macro<double>((const double*)h->f, phase, vel ? nullptr : (double*)h->scratch,
                                           vel ? (double*)h->scratch : nullptr, h->g, s));
            else
                CK(h, launch_macro<float>((const float*)h->f, phase, vel ? nullptr : (double*)h->scratch,
                                          vel ? (double*)h->scratch : nullptr, h->g, s));
            h->launches += 1;
            CK(h, cudaMemcpyAsync(host_buf, h->scratch, (vel ? 3 : 1) * N * sizeof(double), cudaMemcpyDeviceToHost, s));
            break;
        }
        default:
            return fail(h, LBDEM_ERR_INVALID_ARG, "get_field: unknown field");
    }
    CK(h, cudaStreamSynchronize(s));
    return LBDEM_OK;
}

lbdem_status lbdem_mass(lbdem_handle* h, double* mass) {
    if (!h || !mass) return fail(h, LBDEM_ERR_INVALID_ARG, "mass: null argument");
    DeviceGuard dg(h->device);
    CK(h, cudaMemsetAsync(h->d_mass, 0, sizeof(double), h->stream));
    if (h->prec == LBDEM_PREC_FP64) CK(h, launch_mass<double>((const double*)h->f, h->d_mass, h->g, h->stream));
    else CK(h, launch_mass<float>((const float*)h->f, h->d_mass, h->g, h->stream));
    h->launches += 1;
    double m = 0;
    CK(h, cudaMemcpyAsync(h->h_ft, h->d_mass, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    m = h->h_ft[0];
    *mass = m + (double)h->g.N;   // sum_i t_i = 1 per cell
    return LBDEM_OK;
}

lbdem_status lbdem_get_device_errors(lbdem_handle* h, uint32_t* bits) {
    if (!h || !bits) return fail(h, LBDEM_ERR_INVALID_ARG, "get_device_errors: null argument");
    DeviceGuard dg(h->device);
    CK(h, cudaMemcpyAsync(h->h_err, h->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemsetAsync(h->d_err, 0, sizeof(unsigned), h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    *bits = *h->h_err;
    return LBDEM_OK;
}

lbdem_status lbdem_get_step(lbdem_handle* h, int64_t* step) {
    if (!h || !step) return LBDEM_ERR_INVALID_ARG;
    *step = h->step;
    return LBDEM_OK;
}

lbdem_status lbdem_device_bytes(lbdem_handle* h, size_t* bytes) {
    if (!h || !bytes) return LBDEM_ERR_INVALID_ARG;
    *bytes = h->dev_bytes;
    return LBDEM_OK;
}

lbdem_status lbdem_get_launch_count(lbdem_handle* h, int64_t* count) {
    if (!h || !count) return LBDEM_ERR_INVALID_ARG;
    *count = h->launches;
    return LBDEM_OK;
}

lbdem_status lbdem_average_density(lbdem_handle* h, const int32_t box[6], double* rho) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    if (!box || !rho) return fail(h, LBDEM_ERR_INVALID_ARG, "average_density: null argument");
    if (!box_ok(h, box)) return fail(h, LBDEM_ERR_INVALID_ARG, "average_density: box outside the lattice or empty");
    DeviceGuard dg(h->device);
    const PlaneJob j = make_job(h, box, 0, 0, 1.0, 2, 2);
    CK(h, cudaMemcpyAsync(h->d_jobs + 2, &j, sizeof(j), cudaMemcpyHostToDevice, h->stream));
    CK(h, plane_launch(h, h->d_jobs + 2, 1, plane_blocks(box_cells(box)), (int)(h->step & 1), 0, nullptr, h->d_pavg));
    h->launches += 1;
    CK(h, cudaMemcpyAsync(h->h_pavg, h->d_pavg + 2, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    *rho = *h->h_pavg;
    return LBDEM_OK;
}

lbdem_status lbdem_zhang_rescale(lbdem_handle* h, const int32_t box[6], int32_t dimension, int32_t direction,
                                 double rho_target, double rho_avg) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    if (!box || !box_ok(h, box)) return fail(h, LBDEM_ERR_INVALID_ARG, "zhang_rescale: box outside the lattice or empty");
    if (dimension < 0 || dimension > 2 || (direction != 1 && direction != -1))
        return fail(h, LBDEM_ERR_INVALID_ARG, "zhang_rescale: dimension must be 0..2 and direction +-1");
    if (!(rho_target > 0.0) || !(rho_avg > 0.0) || !std::isfinite(rho_target) || !std::isfinite(rho_avg))
        return fail(h, LBDEM_ERR_INVALID_ARG, "zhang_rescale: densities must be positive and finite");
    DeviceGuard dg(h->device);
    const PlaneJob j = make_job(h, box, dimension, direction, rho_target, 3, 2);
    CK(h, cudaMemcpyAsync(h->d_jobs + 2, &j, sizeof(j), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->d_pavg + 3, &rho_avg, sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(h, plane_launch(h, h->d_jobs + 2, 1, plane_blocks(box_cells(box)), (int)(h->step & 1), 1, h->d_pavg,
                       h->d_pavg));
    h->launches += 1;
    CK(h, cudaStreamSynchronize(h->stream));   // the host-side source of the copies is the caller's stack
    h->pavg_valid = false;
    return LBDEM_OK;
}

lbdem_status lbdem_set_pressure_drop(lbdem_handle* h, const lbdem_pressure_drop* d) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    if (!d) {
        h->pdrop_on = false;
        return LBDEM_OK;
    }
    if (d->dimension < 0 || d->dimension > 2) return fail(h, LBDEM_ERR_INVALID_ARG, "pressure_drop: dimension");
    if (!box_ok(h, d->inlet) || !box_ok(h, d->outlet))
        return fail(h, LBDEM_ERR_INVALID_ARG, "pressure_drop: box outside the lattice or empty");
    bool overlap = true;
    for (int k = 0; k < 3; ++k)
        if (d->inlet[2 * k + 1] < d->outlet[2 * k] || d->outlet[2 * k + 1] < d->inlet[2 * k]) overlap = false;
    if (overlap) return fail(h, LBDEM_ERR_INVALID_ARG, "pressure_drop: inlet and outlet boxes overlap");
    if ((d->in_direction != 1 && d->in_direction != -1) || (d->out_direction != 1 && d->out_direction != -1))
        return fail(h, LBDEM_ERR_INVALID_ARG, "pressure_drop: directions must be +-1");
    if (!(d->rho_in > 0.0) || !(d->rho_out > 0.0) || !std::isfinite(d->rho_in) || !std::isfinite(d->rho_out))
        return fail(h, LBDEM_ERR_INVALID_ARG, "pressure_drop: densities must be positive and finite");
    DeviceGuard dg(h->device);
    PlaneJob j[2] = {make_job(h, d->inlet, d->dimension, d->in_direction, d->rho_in, 1, 0),
                     make_job(h, d->outlet, d->dimension, d->out_direction, d->rho_out, 0, 1)};
    CK(h, cudaMemcpyAsync(h->d_jobs, j, sizeof(j), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->pdrop_bpj = plane_blocks(std::max(box_cells(d->inlet), box_cells(d->outlet)));
    h->pdrop_on = true;
    h->pavg_valid = false;
    return LBDEM_OK;
}

lbdem_status lbdem_set_omega(lbdem_handle* h, double omega) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    if (!(omega > 0.0 && omega < 2.0)) return fail(h, LBDEM_ERR_INVALID_ARG, "set_omega: omega outside (0, 2)");
    DeviceGuard dg(h->device);
    CK(h, cudaStreamSynchronize(h->stream));   // queued steps use the old tables
    h->cfg.omega = omega;
    CK(h, upload_btab(h));
    return LBDEM_OK;
}

lbdem_status lbdem_set_periodic(lbdem_handle* h, const int32_t periodic[3]) {
    if (!h || !periodic) return LBDEM_ERR_INVALID_ARG;
    for (int d = 0; d < 3; ++d)
        if (periodic[d] != 0 && periodic[d] != 1) return fail(h, LBDEM_ERR_INVALID_ARG, "set_periodic: 0 or 1");
    if (h->pdrop_on)
        return fail(h, LBDEM_ERR_INVALID_ARG, "set_periodic: set the periodicity before the pressure drop");
    DeviceGuard dg(h->device);
    CK(h, cudaStreamSynchronize(h->stream));
    for (int d = 0; d < 3; ++d) h->cfg.periodic[d] = h->g.per[d] = periodic[d];
    return LBDEM_OK;
}

lbdem_status lbdem_init_profile(lbdem_handle* h, int32_t kind, double rho_hi, double rho_lo, double u_max,
                                const int32_t n[3], int32_t dimension) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    if (!n || (kind != LBDEM_PROFILE_PRESSURE_GRADIENT && kind != LBDEM_PROFILE_POISEUILLE) || dimension < 0 ||
        dimension > 2)
        return fail(h, LBDEM_ERR_INVALID_ARG, "init_profile: kind, dimension or n");
    if (n[dimension] < 2) return fail(h, LBDEM_ERR_INVALID_ARG, "init_profile: n[dimension] < 2");
    if (kind == LBDEM_PROFILE_POISEUILLE)
        for (int d = 0; d < 3; ++d)
            if (n[d] < 1) return fail(h, LBDEM_ERR_INVALID_ARG, "init_profile: n < 1");
    if (!std::isfinite(rho_hi) || !std::isfinite(rho_lo) || !std::isfinite(u_max))
        return fail(h, LBDEM_ERR_INVALID_ARG, "init_profile: non-finite parameter");
    const int ext[3] = {h->g.nx, h->g.ny, h->g.nz};
    const double slope = (rho_hi - rho_lo) / (double)(n[dimension] - 1);
    if (!(rho_hi > 0.0) || !(rho_hi - slope * (ext[dimension] - 1) > 0.0))
        return fail(h, LBDEM_ERR_INVALID_ARG, "init_profile: density not positive on the lattice");
    DeviceGuard dg(h->device);
    const int phase = (int)(h->step & 1);
    if (h->prec == LBDEM_PREC_FP64)
        CK(h, launch_init_profile<double>((double*)h->f, phase, kind, rho_hi, rho_lo, u_max, n[0], n[1], n[2],
                                          dimension, h->g, h->stream));
    else
        CK(h, launch_init_profile<float>((float*)h->f, phase, kind, rho_hi, rho_lo, u_max, n[0], n[1], n[2],
                                         dimension, h->g, h->stream));
    h->launches += 1;
    h->pavg_valid = false;
    return LBDEM_OK;
}

}  // extern "C"

namespace {

// Device buffers of one adjoint window, released on every exit path.
struct AdjointBuffers {
    std::vector<void*> ptrs;
    ~AdjointBuffers() {
        for (void* p : ptrs)
            if (p) cudaFree(p);
    }
    template <typename P>
    cudaError_t get(P** p, size_t bytes) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, bytes == 0 ? 16 : bytes);
        if (e == cudaSuccess) {
            ptrs.push_back(q);
            *p = (P*)q;
        }
        return e;
    }
};

struct EventPair {
    cudaEvent_t e[3] = {nullptr, nullptr, nullptr};
    ~EventPair() {
        for (auto& x : e)
            if (x) cudaEventDestroy(x);
    }
};

template <typename T>
cudaError_t adjoint_launch(lbdem_handle* h, const T* f, int phase, const T* lam_in, T* lam_out, const double* rec,
                           const double* w, double* gvel, double* gglob, int n) {
    AdjointArgs<T> a;
    a.g = h->g;
    a.f = f;
    a.phase = phase;
    a.lam_in = lam_in;
    a.lam_out = lam_out;
    a.vox = h->vox;
    a.tag2slot = h->d_tag2slot;
    a.max_tag = h->cfg.max_tag;
    a.nslot = n;
    a.rec = rec;
    a.xpf = h->d_xpf;
    a.w = w;
    a.gvel = gvel;
    a.gglob = gglob;
    a.btab = sizeof(T) == 8 ? (const T*)h->btab : (const T*)h->btabf;
    a.omega = (T)h->cfg.omega;
    a.tauT = (T)(1.0 / h->cfg.omega);
    for (int d = 0; d < 3; ++d) a.g3[d] = (T)h->cfg.body_force[d];
    a.err = h->d_err;
    return launch_adjoint_step<T>(a, h->stream);
}

}  // namespace

extern "C" {

lbdem_status lbdem_adjoint_window(lbdem_handle* h, int32_t nsteps, int32_t K, int32_t n, const double* rec,
                                  const double* weights, double* loss, double* grad_vel, double* grad_body_force,
                                  double* grad_tau, void* grad_f0) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    if (nsteps < 1 || K < 1 || K > nsteps) return fail(h, LBDEM_ERR_INVALID_ARG, "adjoint: need 1 <= checkpoint_every <= nsteps");
    if (n < 0) return fail(h, LBDEM_ERR_INVALID_ARG, "adjoint: n < 0");
    if (n > h->cap) return fail(h, LBDEM_ERR_CAPACITY, "adjoint: n exceeds max_particles");
    if (!loss || !grad_body_force || !grad_tau || (n > 0 && (!rec || !weights || !grad_vel)))
        return fail(h, LBDEM_ERR_INVALID_ARG, "adjoint: null argument");
    if (h->pdrop_on) return fail(h, LBDEM_ERR_INVALID_ARG, "adjoint: the pressure drop is not differentiated");
    for (int t = 1; t < nsteps; ++t)
        for (int k = 0; k < n; ++k) {
            const double* a = rec + ((size_t)t * n + k) * REC_STRIDE;
            const double* b = rec + (size_t)k * REC_STRIDE;
            if (std::memcmp(a, b, 3 * sizeof(double)) != 0 || std::memcmp(a + 9, b + 9, 2 * sizeof(double)) != 0)
                return fail(h, LBDEM_ERR_INVALID_ARG, "adjoint: positions, radii and tags must stay fixed");
        }
    DeviceGuard dg(h->device);
    cudaStream_t s = h->stream;
    const size_t N = h->g.N;
    const size_t pop = (size_t)Q * N * h->esz;
    const int nseg = (nsteps + K - 1) / K;
    const size_t nrec = (size_t)nsteps * n;
    AdjointBuffers buf;
    double *d_recs = nullptr, *d_w = nullptr, *d_gv = nullptr, *d_glob = nullptr, *d_loss = nullptr, *d_ft = nullptr;
    unsigned char *ckpt = nullptr, *tape = nullptr, *lam = nullptr;
    CK(h, buf.get(&d_recs, nrec * REC_STRIDE * sizeof(double)));
    CK(h, buf.get(&d_w, nrec * 6 * sizeof(double)));
    CK(h, buf.get(&d_gv, nrec * 6 * sizeof(double)));
    CK(h, buf.get(&d_glob, 4 * sizeof(double)));
    CK(h, buf.get(&d_loss, sizeof(double)));
    CK(h, buf.get(&d_ft, 6 * (size_t)std::max(n, 1) * sizeof(double)));
    CK(h, buf.get(&ckpt, (size_t)nseg * pop));
    CK(h, buf.get(&tape, (size_t)K * pop + ALLOC_TAIL));
    CK(h, buf.get(&lam, 2 * pop));
    EventPair ev;
    for (auto& e : ev.e) CK(h, cudaEventCreate(&e));
    if (n > 0) {
        CK(h, cudaMemcpyAsync(d_recs, rec, nrec * REC_STRIDE * sizeof(double), cudaMemcpyHostToDevice, s));
        CK(h, cudaMemcpyAsync(d_w, weights, nrec * 6 * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    CK(h, cudaMemsetAsync(d_gv, 0, nrec * 6 * sizeof(double) + 0, s));
    CK(h, cudaMemsetAsync(d_glob, 0, 4 * sizeof(double), s));
    CK(h, cudaMemsetAsync(d_loss, 0, sizeof(double), s));
    CK(h, cudaMemsetAsync(lam, 0, pop, s));        // lambda after the window = 0
    CK(h, cudaMemsetAsync(tape + (size_t)K * pop, 0, ALLOC_TAIL, s));
    const int64_t step0 = h->step;
    lbdem_status st;
    // A step whose particle table equals the one voxelized last needs no new
    // voxelization: with positions fixed the update is idempotent (every cell's
    // owner re-sets itself, no other sphere can displace it), so the voxel
    // words, surface velocities and tag map are already those of the step.
    int vox_t = -1;   // step whose table the voxel state holds
    auto same_table = [&](int a, int b) {
        return a >= 0 && b >= 0 &&
               std::memcmp(rec + (size_t)a * n * REC_STRIDE, rec + (size_t)b * n * REC_STRIDE,
                           (size_t)n * REC_STRIDE * sizeof(double)) == 0;
    };
    auto voxelize_for = [&](int t) -> lbdem_status {
        if (same_table(vox_t, t)) return LBDEM_OK;
        const lbdem_status r = lbdem_set_particles_device(h, n, d_recs + (size_t)t * n * REC_STRIDE, 0);
        if (r == LBDEM_OK) vox_t = t;
        return r;
    };

    // forward pass with checkpoints
    CK(h, cudaEventRecord(ev.e[0], s));
    for (int t = 0; t < nsteps; ++t) {
        if (t % K == 0) CK(h, cudaMemcpyAsync(ckpt + (size_t)(t / K) * pop, h->f, pop, cudaMemcpyDeviceToDevice, s));
        if ((st = voxelize_for(t)) != LBDEM_OK) return st;
        if ((st = lbdem_collide_and_stream(h)) != LBDEM_OK) return st;
        if (n > 0) {
            CK(h, launch_loss_step(h->d_ft, d_w + (size_t)t * n * 6, n, n, d_loss, s));
            h->launches += 1;
        }
    }
    CK(h, cudaEventRecord(ev.e[1], s));
    if (n > 0) CK(h, cudaMemcpyAsync(d_ft, h->d_ft, 6 * (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));

    // backward pass: recompute each segment into the tape, then reverse steps
    unsigned char* lam_in = lam;
    unsigned char* lam_out = lam + pop;
    lbdem_status bst = LBDEM_OK;
    for (int seg = nseg - 1; seg >= 0 && bst == LBDEM_OK; --seg) {
        const int t0 = seg * K, t1 = std::min(t0 + K, nsteps);
        // tape[0] = the segment's checkpoint; every recomputed step writes its
        // output straight into the next tape slot (out-of-place collide-stream)
        cudaError_t e = cudaMemcpyAsync(tape, ckpt + (size_t)seg * pop, pop, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) { bst = fail_cuda(h, "adjoint checkpoint restore", e); break; }
        h->step = step0 + t0;
        for (int t = t0; t + 1 < t1 && bst == LBDEM_OK; ++t) {
            if ((bst = voxelize_for(t)) != LBDEM_OK) break;
            if (n > 0) {
                e = cudaMemsetAsync(h->d_ft, 0, 6 * (size_t)n * sizeof(double), s);
                if (e != cudaSuccess) { bst = fail_cuda(h, "adjoint force reset", e); break; }
            }
            e = k1_launch(h, tape + (size_t)(t - t0) * pop, tape + (size_t)(t - t0 + 1) * pop);
            if (e != cudaSuccess) { bst = fail_cuda(h, "adjoint recompute", e); break; }
            h->launches += 1;
            h->step += 1;
        }
        for (int t = t1 - 1; t >= t0 && bst == LBDEM_OK; --t) {
            const int phase = (int)((step0 + t) & 1);
            const unsigned char* ft = tape + (size_t)(t - t0) * pop;
            if (h->prec == LBDEM_PREC_FP64)
                e = adjoint_launch<double>(h, (const double*)ft, phase, (const double*)lam_in, (double*)lam_out,
                                           d_recs + (size_t)t * n * REC_STRIDE, d_w + (size_t)t * n * 6,
                                           d_gv + (size_t)t * n * 6, d_glob, n);
            else
                e = adjoint_launch<float>(h, (const float*)ft, phase, (const float*)lam_in, (float*)lam_out,
                                          d_recs + (size_t)t * n * REC_STRIDE, d_w + (size_t)t * n * 6,
                                          d_gv + (size_t)t * n * 6, d_glob, n);
            if (e != cudaSuccess) { bst = fail_cuda(h, "adjoint step", e); break; }
            h->launches += 1;
            std::swap(lam_in, lam_out);
        }
    }
    h->step = step0 + nsteps;
    if (bst != LBDEM_OK) return bst;
    CK(h, cudaEventRecord(ev.e[2], s));
    // the voxel state and the forces of the window's last step
    if ((st = voxelize_for(nsteps - 1)) != LBDEM_OK) return st;
    if (n > 0) CK(h, cudaMemcpyAsync(h->d_ft, d_ft, 6 * (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));

    double glob[4];
    CK(h, cudaMemcpyAsync(loss, d_loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(h, cudaMemcpyAsync(glob, d_glob, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (n > 0) CK(h, cudaMemcpyAsync(grad_vel, d_gv, nrec * 6 * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (grad_f0) CK(h, cudaMemcpyAsync(grad_f0, lam_in, pop, cudaMemcpyDeviceToHost, s));
    CK(h, cudaMemcpyAsync(h->h_err, h->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(h, cudaStreamSynchronize(s));
    grad_body_force[0] = glob[0];
    grad_body_force[1] = glob[1];
    grad_body_force[2] = glob[2];
    *grad_tau = glob[3];
    CK(h, cudaEventElapsedTime(&h->adj_fwd_ms, ev.e[0], ev.e[1]));
    CK(h, cudaEventElapsedTime(&h->adj_bwd_ms, ev.e[1], ev.e[2]));
    if (*h->h_err) {
        char msg[96];
        std::snprintf(msg, sizeof(msg), "device error word 0x%x", *h->h_err);
        return fail(h, LBDEM_ERR_DEVICE, msg);
    }
    return LBDEM_OK;
}

lbdem_status lbdem_adjoint_timing(lbdem_handle* h, float* forward_ms, float* backward_ms) {
    if (!h) return LBDEM_ERR_INVALID_ARG;
    if (forward_ms) *forward_ms = h->adj_fwd_ms;
    if (backward_ms) *backward_ms = h->adj_bwd_ms;
    return LBDEM_OK;
}

}  // extern "C"

namespace {

struct CheckpointHeader {
    char magic[8];           // "LBDEMCK1"
    int32_t version;         // 1
    int32_t nx, ny, nz;
    int32_t periodic[3];
    int32_t precision;
    double omega;
    double body_force[3];
    int64_t step;
};

struct FileCloser {
    std::FILE* f = nullptr;
    ~FileCloser() {
        if (f) std::fclose(f);
    }
};

}  // namespace

extern "C" {

lbdem_status lbdem_save_state(lbdem_handle* h, const char* path) {
    if (!h || !path) return fail(h, LBDEM_ERR_INVALID_ARG, "save_state: null argument");
    const size_t N = h->g.N;
    std::vector<unsigned char> pops((size_t)Q * N * h->esz);
    lbdem_status st = lbdem_get_populations(h, pops.data());
    if (st != LBDEM_OK) return st;
    std::vector<uint32_t> vox(N);
    std::vector<unsigned char> up(3 * N * h->esz);
    if ((st = lbdem_get_field(h, LBDEM_FIELD_PARTICLE_VELOCITY, up.data())) != LBDEM_OK) return st;
    {
        DeviceGuard dg(h->device);
        CK(h, cudaMemcpyAsync(vox.data(), h->vox, N * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    CheckpointHeader hd{};
    std::memcpy(hd.magic, "LBDEMCK1", 8);
    hd.version = 1;
    hd.nx = h->g.nx; hd.ny = h->g.ny; hd.nz = h->g.nz;
    for (int d = 0; d < 3; ++d) { hd.periodic[d] = h->g.per[d]; hd.body_force[d] = h->cfg.body_force[d]; }
    hd.precision = h->prec;
    hd.omega = h->cfg.omega;
    hd.step = h->step;
    FileCloser fc;
    fc.f = std::fopen(path, "wb");
    if (!fc.f) return fail(h, LBDEM_ERR_INVALID_ARG, std::string("save_state: cannot open ") + path);
    bool ok = std::fwrite(&hd, sizeof(hd), 1, fc.f) == 1 && std::fwrite(pops.data(), 1, pops.size(), fc.f) == pops.size() &&
              std::fwrite(vox.data(), sizeof(uint32_t), N, fc.f) == N && std::fwrite(up.data(), 1, up.size(), fc.f) == up.size();
    ok = (std::fclose(fc.f) == 0) && ok;
    fc.f = nullptr;
    if (!ok) return fail(h, LBDEM_ERR_INVALID_ARG, std::string("save_state: write failed: ") + path);
    return LBDEM_OK;
}

lbdem_status lbdem_load_state(lbdem_handle* h, const char* path) {
    if (!h || !path) return fail(h, LBDEM_ERR_INVALID_ARG, "load_state: null argument");
    FileCloser fc;
    fc.f = std::fopen(path, "rb");
    if (!fc.f) return fail(h, LBDEM_ERR_INVALID_ARG, std::string("load_state: cannot open ") + path);
    CheckpointHeader hd{};
    if (std::fread(&hd, sizeof(hd), 1, fc.f) != 1 || std::memcmp(hd.magic, "LBDEMCK1", 8) != 0 || hd.version != 1)
        return fail(h, LBDEM_ERR_INVALID_ARG, "load_state: not a checkpoint of this library");
    if (hd.nx != h->g.nx || hd.ny != h->g.ny || hd.nz != h->g.nz || hd.precision != h->prec)
        return fail(h, LBDEM_ERR_INVALID_ARG, "load_state: lattice extent or precision differs");
    const size_t N = h->g.N;
    std::vector<unsigned char> pops((size_t)Q * N * h->esz);
    std::vector<uint32_t> vox(N);
    std::vector<unsigned char> up(3 * N * h->esz);
    if (std::fread(pops.data(), 1, pops.size(), fc.f) != pops.size() ||
        std::fread(vox.data(), sizeof(uint32_t), N, fc.f) != N || std::fread(up.data(), 1, up.size(), fc.f) != up.size())
        return fail(h, LBDEM_ERR_INVALID_ARG, "load_state: file truncated");
    // the step count first: it fixes the in-place layout the populations are scattered into
    h->step = hd.step;
    lbdem_status st = lbdem_set_populations(h, pops.data());
    if (st != LBDEM_OK) return st;
    DeviceGuard dg(h->device);
    CK(h, cudaMemcpyAsync(h->vox, vox.data(), N * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
    // the FP32 form keeps no velocity field: it recomputes the velocity from the
    // particle list of the next lbdem_set_particles
    if (h->up) CK(h, cudaMemcpyAsync(h->up, up.data(), 3 * N * h->esz, cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->pavg_valid = false;
    return LBDEM_OK;
}

}  // extern "C"
