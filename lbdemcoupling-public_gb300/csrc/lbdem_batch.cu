// Batched independent domains: the lbdem_batch_* entry points of
// include/lbdem_gpu.h.
//
// Every array of the single-lattice handle becomes one arena with per-domain
// offsets (populations, voxel words, particle velocities, particle slots, tag
// maps, voxelization tiles, collide-stream segments, force sums), so that each
// stage of a coupling cycle is one launch over all domains:
//   prepare spheres -> bin spheres -> voxelize work list -> collide-stream
//   (persistent, segments of all domains) -> pressure-drop planes.
// The device part of a cycle, including the upload of the particle table and
// the download of the force sums, is captured into one CUDA graph per
// streaming phase and replayed.
#include "lbdem_gpu.h"
#include "lbdem_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

using namespace lbdem;

struct lbdem_batch {
    lbdem_batch_config cfg{};
    int ndom = 0;
    int prec = 0;
    size_t esz = 8;
    int device = 0;
    cudaStream_t stream = nullptr;

    std::vector<lbdem_domain> dom;
    std::vector<DomView> views;          // host copy of d_views
    std::vector<int> soff, toff, seg0;   // per-domain first slot / tile / segment; seg0 holds the row
                                         // segments, then (FP32 even phase) the plane segments
    std::vector<int> cap;
    int nslots = 0, ntiles = 0;
    long long nseg = 0, nseg_plane = 0;
    size_t ncells = 0, f_elems = 0, up_elems = 0, vox_elems = 0;

    void* f = nullptr;
    uint32_t* vox = nullptr;
    void* up = nullptr;
    void* btab = nullptr;                // [ndom][126] of the lattice type
    unsigned char* d_stage = nullptr;    // [ndom] int counts (padded) then [nslots][12] doubles
    int* d_ncur = nullptr;
    double* d_rec = nullptr;
    SphereDev* d_sph = nullptr;
    SphereFast* d_fast = nullptr;
    float* d_xpf = nullptr;
    int* d_tag2slot = nullptr;           // [ndom][max_tag + 1]
    int* d_tile_cnt = nullptr;
    int* d_bins = nullptr;
    int* d_work = nullptr;
    int* d_work_n = nullptr;
    double* d_ft = nullptr;              // per domain [6][cap]
    unsigned* d_err = nullptr;
    DomView* d_views = nullptr;
    int* d_soff = nullptr;
    int* d_toff = nullptr;
    int* d_seg0 = nullptr;               // [2][ndom]: row segments, plane segments
    void* d_dargs = nullptr;             // CollideArgs<T>[2][ndom]: row views, plane views
    void* scratch = nullptr;
    size_t scratch_bytes = 0;

    // periodic pressure drop: jobs 2k (inlet) and 2k + 1 (outlet) of the k-th
    // domain with a drop; averages [2 parities][njobs]
    int njobs = 0;
    int plane_bpj = 1;
    PlaneJob* d_jobs = nullptr;
    double* d_pavg = nullptr;
    double* d_ppart = nullptr;
    unsigned* d_pcount = nullptr;
    bool pavg_valid = false;

    unsigned char* h_stage = nullptr;    // pinned mirror of d_stage
    size_t stage_bytes = 0, rec_off = 0;
    double* h_ft = nullptr;              // pinned mirror of d_ft
    unsigned* h_err = nullptr;
    std::vector<int> counts;             // staged per-domain counts
    int init_vel = 0;

    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    int collide_bps = 0;                 // CTAs per SM of the collide-stream grid (0: all that fit)
    float collide_ms = 0.f;
    bool tuned = false;

    size_t dev_bytes = 0;
    int64_t step = 0;
    int64_t launches = 0;
    std::string last_error;
};

namespace {

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

lbdem_status fail(lbdem_batch* b, lbdem_status s, const std::string& msg) {
    if (b) b->last_error = msg;
    return s;
}

lbdem_status fail_cuda(lbdem_batch* b, const char* what, cudaError_t e) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(b, e == cudaErrorMemoryAllocation ? LBDEM_ERR_OUT_OF_MEMORY : LBDEM_ERR_CUDA, m);
}

#define BK(b, call)                                              \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return fail_cuda((b), #call, e_); \
    } while (0)

template <typename P>
cudaError_t dalloc(lbdem_batch* b, P** p, size_t bytes) {
    void* q = nullptr;
    if (alloc_should_fail()) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(&q, bytes == 0 ? 16 : bytes);
    if (e == cudaSuccess) {
        *p = (P*)q;
        b->dev_bytes += bytes;
    }
    return e;
}

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

void release(lbdem_batch* b) {
    for (auto& g : b->gexec)
        if (g) cudaGraphExecDestroy(g);
    void* dev[] = {b->f, b->vox, b->up, b->btab, b->d_stage, b->d_sph, b->d_fast, b->d_xpf, b->d_tag2slot,
                   b->d_tile_cnt, b->d_bins, b->d_work, b->d_work_n, b->d_ft, b->d_err, b->d_views, b->d_soff,
                   b->d_toff, b->d_seg0, b->d_dargs, b->scratch, b->d_jobs, b->d_pavg, b->d_ppart, b->d_pcount};
    for (void* p : dev)
        if (p) cudaFree(p);
    void* host[] = {b->h_stage, b->h_ft, b->h_err};
    for (void* p : host)
        if (p) cudaFreeHost(p);
    if (b->stream) cudaStreamDestroy(b->stream);
}

bool domain_ok(const lbdem_domain& d) {
    if (d.nx <= 0 || d.ny <= 0 || d.nz <= 0 || d.nx >= (1 << 24) || d.ny >= (1 << 24) || d.nz >= (1 << 24))
        return false;
    if ((size_t)d.nx * d.ny > 0x7fffffffu) return false;
    if (!(d.omega > 0.0 && d.omega < 2.0)) return false;
    for (int k = 0; k < 3; ++k) {
        if (d.periodic[k] != 0 && d.periodic[k] != 1) return false;
        if (!std::isfinite(d.body_force[k])) return false;
    }
    if (d.max_particles < 0) return false;
    return true;
}

bool box_in(const lbdem_domain& d, const int32_t* b) {
    const int ext[3] = {d.nx, d.ny, d.nz};
    for (int k = 0; k < 3; ++k)
        if (b[2 * k] < 0 || b[2 * k + 1] >= ext[k] || b[2 * k] > b[2 * k + 1]) return false;
    return true;
}

bool drop_ok(const lbdem_domain& d) {
    const lbdem_pressure_drop& p = d.drop;
    if (p.dimension < 0 || p.dimension > 2 || !box_in(d, p.inlet) || !box_in(d, p.outlet)) return false;
    bool overlap = true;
    for (int k = 0; k < 3; ++k)
        if (p.inlet[2 * k + 1] < p.outlet[2 * k] || p.outlet[2 * k + 1] < p.inlet[2 * k]) overlap = false;
    if (overlap) return false;
    if ((p.in_direction != 1 && p.in_direction != -1) || (p.out_direction != 1 && p.out_direction != -1)) return false;
    return p.rho_in > 0.0 && p.rho_out > 0.0 && std::isfinite(p.rho_in) && std::isfinite(p.rho_out);
}

long long box_cells(const int32_t* b) {
    return (long long)(b[1] - b[0] + 1) * (b[3] - b[2] + 1) * (b[5] - b[4] + 1);
}

template <typename T>
T* fptr(lbdem_batch* b, int d) { return (T*)b->f + b->views[d].f0; }

// out[d]: domain d as rows of nz cells; out[ndom + d]: the same domain as nx rows
// of ny nz cells (the plane view of the FP32 even phase, whose update touches
// only each cell's own slots).
template <typename T>
void fill_dargs(lbdem_batch* b, std::vector<CollideArgs<T>>& out, T* f_base, double* ft_base) {
    out.resize(2 * (size_t)b->ndom);
    for (int d = 0; d < b->ndom; ++d) {
        const DomView& v = b->views[d];
        CollideArgs<T>& a = out[d];
        a = CollideArgs<T>{};
        a.g = v.g;
        a.f = f_base + v.f0;
        a.fo = a.f;
        a.vox = b->vox + v.cell0;
        a.up = b->up ? (const T*)b->up + v.up0 : nullptr;   // FP64 form only
        a.cf = nullptr;
        a.tag2slot = b->d_tag2slot + v.tag0;
        a.rec = b->d_rec + (size_t)REC_STRIDE * v.s0;
        a.xpf = b->d_xpf + (size_t)XPF_STRIDE * v.s0;
        a.nslot = b->cap[d];
        a.max_tag = b->cfg.max_tag;
        a.ft = ft_base + (size_t)6 * v.s0;
        a.err = b->d_err;
        a.btab = (const T*)b->btab + (size_t)126 * d;
        a.omega = (T)b->dom[d].omega;
        for (int k = 0; k < 3; ++k) a.g3[k] = (T)b->dom[d].body_force[k];
        a.dz = div_magic((unsigned)((v.g.nz + COLLIDE_SEGW - 1) / COLLIDE_SEGW));
        a.dy = div_magic((unsigned)v.g.ny);
        CollideArgs<T>& p = out[b->ndom + d];
        p = a;
        const int plane = v.g.ny * v.g.nz;
        p.g.ny = 1;
        p.g.nz = plane;
        p.dz = div_magic((unsigned)((plane + COLLIDE_SEGW - 1) / COLLIDE_SEGW));
        p.dy = div_magic(1u);
        p.flat_ny = v.g.ny;
        p.flat_nz = v.g.nz;
        p.dnz = div_magic((unsigned)v.g.nz);
    }
}

bool any_force(const lbdem_batch* b) {
    for (const auto& d : b->dom)
        if (d.body_force[0] != 0.0 || d.body_force[1] != 0.0 || d.body_force[2] != 0.0) return true;
    return false;
}

// dargs: the [2][ndom] table of fill_dargs on the device.
cudaError_t launch_k1(lbdem_batch* b, const void* dargs, bool odd, int bps) {
    const bool force = any_force(b);
    if (b->prec == LBDEM_PREC_FP64)
        return launch_collide_batch<double>((const CollideArgs<double>*)dargs, b->d_seg0, b->ndom, b->nseg, odd,
                                            force, bps, b->stream);
    if (!odd)   // plane segments
        return launch_collide_batch<float>((const CollideArgs<float>*)dargs + b->ndom, b->d_seg0 + b->ndom, b->ndom,
                                           b->nseg_plane, false, force, bps, b->stream);
    return launch_collide_batch<float>((const CollideArgs<float>*)dargs, b->d_seg0, b->ndom, b->nseg, true, force,
                                       bps, b->stream);
}

cudaError_t launch_planes(lbdem_batch* b, int phase, int rescale, const double* avg_in, double* avg_out) {
    if (b->prec == LBDEM_PREC_FP64)
        return launch_plane_pressure<double>(b->d_jobs, b->njobs, b->plane_bpj, phase, rescale, avg_in, avg_out,
                                             b->d_ppart, b->d_pcount, b->stream);
    return launch_plane_pressure<float>(b->d_jobs, b->njobs, b->plane_bpj, phase, rescale, avg_in, avg_out,
                                        b->d_ppart, b->d_pcount, b->stream);
}

// The device part of one step, queued on b->stream (capturable: no
// synchronization, no allocation).  Averages of the pressure-drop boxes must
// be current (pavg_valid) when `capture` is set.
cudaError_t enqueue_step(lbdem_batch* b, bool odd, int init_vel) {
    cudaStream_t s = b->stream;
    const int P = odd ? 1 : 0;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(b->d_stage, b->h_stage, b->stage_bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(b->d_tag2slot, 0x7F, sizeof(int) * ((size_t)b->cfg.max_tag + 1) * b->ndom, s)) !=
        cudaSuccess)
        return e;
    if ((e = launch_prepare_bin_batch(b->d_rec, b->nslots, b->d_sph, b->d_fast, b->d_xpf, b->d_tag2slot, b->d_err,
                                      b->cfg.max_tag, b->cfg.max_radius, b->d_views, b->d_soff, b->ndom, b->d_ncur,
                                      b->d_ft, b->d_tile_cnt, b->d_bins, b->d_work, b->d_work_n, s)) !=
        cudaSuccess)   // also zeroes the force/torque sums
        return e;
    if (b->prec == LBDEM_PREC_FP64)
        e = launch_voxelize_batch<double>(b->d_sph, b->d_fast, b->d_tile_cnt, b->d_bins, b->d_work, b->d_work_n,
                                          b->ntiles, b->vox, (double*)b->up, (double*)b->f, init_vel, P, b->d_views,
                                          b->d_toff, b->ndom, b->d_ncur,
                                          OwnerTable{b->d_xpf, b->d_tag2slot, b->cfg.max_tag}, s);
    else
        e = launch_voxelize_batch<float>(b->d_sph, b->d_fast, b->d_tile_cnt, b->d_bins, b->d_work, b->d_work_n,
                                         b->ntiles, b->vox, nullptr, (float*)b->f, init_vel, P, b->d_views,
                                         b->d_toff, b->ndom, b->d_ncur,
                                         OwnerTable{b->d_xpf, b->d_tag2slot, b->cfg.max_tag}, s);
    if (e != cudaSuccess) return e;
    if (b->njobs > 0 && !b->pavg_valid) {
        if ((e = launch_planes(b, P, 0, nullptr, b->d_pavg + (size_t)b->njobs * P)) != cudaSuccess) return e;
    }
    if ((e = launch_k1(b, b->d_dargs, odd, b->collide_bps)) != cudaSuccess) return e;
    if (b->njobs > 0) {
        if ((e = launch_planes(b, P ^ 1, 1, b->d_pavg + (size_t)b->njobs * P, b->d_pavg + (size_t)b->njobs * (P ^ 1))) !=
            cudaSuccess)
            return e;
    }
    if ((e = cudaMemcpyAsync(b->h_ft, b->d_ft, sizeof(double) * 6 * (size_t)b->nslots, cudaMemcpyDeviceToHost, s)) !=
        cudaSuccess)
        return e;
    return cudaMemcpyAsync(b->h_err, b->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
}

int launches_per_step(const lbdem_batch* b, bool stale) {
    return 3 + (b->njobs > 0 ? (stale ? 2 : 1) : 0);   // prepare + bin, voxelize, collide-stream, planes
}

// Collide-stream grid shapes timed on a copy of the populations (the state is
// not advanced): each candidate runs an even and an odd pass three times, the
// first pair discarded; the fastest candidate is kept.
template <typename T>
lbdem_status autotune(lbdem_batch* b) {
    const size_t fbytes = b->f_elems * sizeof(T) + ALLOC_TAIL;
    const size_t ftbytes = sizeof(double) * 6 * (size_t)std::max(b->nslots, 1);
    void* fcopy = nullptr;
    double* ftcopy = nullptr;
    void* dcopy = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
        if (fcopy) cudaFree(fcopy);
        if (ftcopy) cudaFree(ftcopy);
        if (dcopy) cudaFree(dcopy);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    cudaError_t e = cudaMalloc(&fcopy, fbytes);
    if (e == cudaSuccess) e = cudaMalloc((void**)&ftcopy, ftbytes);
    if (e == cudaSuccess) e = cudaMalloc(&dcopy, sizeof(CollideArgs<T>) * 2 * (size_t)b->ndom);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fcopy, b->f, fbytes, cudaMemcpyDeviceToDevice, b->stream);
    std::vector<CollideArgs<T>> args;
    if (e == cudaSuccess) {
        fill_dargs<T>(b, args, (T*)fcopy, ftcopy);
        e = cudaMemcpyAsync(dcopy, args.data(), sizeof(CollideArgs<T>) * args.size(), cudaMemcpyHostToDevice,
                            b->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        cleanup();
        cudaGetLastError();
        return fail_cuda(b, "autotune setup", e);
    }
    const int cand[] = {0, 1, 2, 3};
    float best = 1e30f;
    int best_bps = 0;
    for (int c : cand) {
        float total = 0.f;
        for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
            e = cudaEventRecord(e0, b->stream);
            if (e == cudaSuccess) e = launch_k1(b, dcopy, false, c);
            if (e == cudaSuccess) e = launch_k1(b, dcopy, true, c);
            if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0) total += ms;   // first repetition warms up
            b->launches += 2;
        }
        if (e != cudaSuccess) break;
        if (total < best) {
            best = total;
            best_bps = c;
        }
    }
    cleanup();
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail_cuda(b, "autotune", e);
    }
    b->collide_bps = best_bps;
    b->collide_ms = best / 4.f;   // per pass
    b->tuned = true;
    return LBDEM_OK;
}

void drop_graphs(lbdem_batch* b) {
    for (auto& g : b->gexec)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

lbdem_status capture(lbdem_batch* b, int P) {
    cudaGraph_t g = nullptr;
    BK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_step(b, P != 0, 0);
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return fail_cuda(b, "capture", e != cudaSuccess ? e : e2);
    }
    e = cudaGraphInstantiate(&b->gexec[P], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->gexec[P] = nullptr;
        return fail_cuda(b, "cudaGraphInstantiate", e);
    }
    return LBDEM_OK;
}

}  // namespace

extern "C" {

void lbdem_batch_config_default(lbdem_batch_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->precision = LBDEM_PREC_FP32_DEV;
    c->device = 0;
    c->max_tag = 1024;
    c->max_radius = 16.0;
    c->use_graph = 1;
    c->autotune = 1;
}

const char* lbdem_batch_last_error(const lbdem_batch* b) { return b ? b->last_error.c_str() : "null batch"; }

lbdem_status lbdem_batch_create(const lbdem_batch_config* cfg, int32_t ndomains, const lbdem_domain* domains,
                                lbdem_batch** out) {
    if (!cfg || !out || !domains || ndomains <= 0) return LBDEM_ERR_INVALID_ARG;
    *out = nullptr;
    const lbdem_batch_config& c = *cfg;
    if (c.precision != LBDEM_PREC_FP64 && c.precision != LBDEM_PREC_FP32_DEV) return LBDEM_ERR_INVALID_ARG;
    if (c.max_tag < 1 || c.max_tag > MAX_TAG_LIMIT) return LBDEM_ERR_INVALID_ARG;
    if (!(c.max_radius > 0.0 && c.max_radius <= 1024.0)) return LBDEM_ERR_INVALID_ARG;
    for (int d = 0; d < ndomains; ++d) {
        if (!domain_ok(domains[d])) return LBDEM_ERR_INVALID_ARG;
        if (domains[d].has_pressure_drop && !drop_ok(domains[d])) return LBDEM_ERR_INVALID_ARG;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0 || c.device < 0 || c.device >= ndev) {
        cudaGetLastError();
        return LBDEM_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, c.device) != cudaSuccess) return LBDEM_ERR_NO_DEVICE;
    if (!(prop.major == 10 && prop.minor == 3)) return LBDEM_ERR_NO_DEVICE;

    lbdem_batch* b = new (std::nothrow) lbdem_batch();
    if (!b) return LBDEM_ERR_OUT_OF_MEMORY;
    b->cfg = c;
    b->ndom = ndomains;
    b->prec = c.precision;
    b->esz = c.precision == LBDEM_PREC_FP64 ? 8 : 4;
    b->device = c.device;
    b->dom.assign(domains, domains + ndomains);

    // layout
    long long slots = 0, tiles = 0, segs = 0, psegs = 0;
    size_t fo = 0, co = 0, uo = 0;
    b->views.resize(ndomains);
    b->soff.resize(ndomains);
    b->toff.resize(ndomains);
    b->seg0.resize(2 * (size_t)ndomains);
    b->cap.resize(ndomains);
    for (int d = 0; d < ndomains; ++d) {
        const lbdem_domain& dm = domains[d];
        DomView& v = b->views[d];
        v.g.nx = dm.nx; v.g.ny = dm.ny; v.g.nz = dm.nz;
        for (int k = 0; k < 3; ++k) v.g.per[k] = dm.periodic[k];
        v.g.N = (size_t)dm.nx * dm.ny * dm.nz;
        v.s0 = (int)slots;
        v.t0 = (int)tiles;
        v.f0 = fo;
        v.cell0 = co;
        v.up0 = uo;
        v.tag0 = (size_t)d * ((size_t)c.max_tag + 1);
        b->soff[d] = v.s0;
        b->toff[d] = v.t0;
        b->seg0[d] = (int)segs;
        b->seg0[ndomains + d] = (int)psegs;
        b->cap[d] = dm.max_particles;
        slots += dm.max_particles;
        tiles += (long long)((dm.nx + TILE - 1) / TILE) * ((dm.ny + TILE - 1) / TILE) * ((dm.nz + TILE - 1) / TILE);
        segs += (long long)dm.nx * dm.ny * ((dm.nz + COLLIDE_SEGW - 1) / COLLIDE_SEGW);
        psegs += (long long)dm.nx * (((long long)dm.ny * dm.nz + COLLIDE_SEGW - 1) / COLLIDE_SEGW);
        fo += round_up((size_t)Q * v.g.N, 32);
        co += round_up(v.g.N, 32);
        uo += round_up(3 * v.g.N, 32);
        b->ncells += v.g.N;
        if (slots > 0x7fffffffLL || tiles > 0x7fffffffLL || segs > 0x7fffffffLL || psegs > 0x7fffffffLL ||
            (long long)dm.ny * dm.nz > 0x7fffffffLL) {
            delete b;
            return LBDEM_ERR_INVALID_ARG;
        }
    }
    b->nslots = (int)slots;
    b->ntiles = (int)tiles;
    b->nseg = segs;
    b->nseg_plane = psegs;
    b->f_elems = fo;
    b->vox_elems = co;
    b->up_elems = uo;
    b->counts.assign(ndomains, 0);
    for (int d = 0; d < ndomains; ++d)
        if (domains[d].has_pressure_drop) b->njobs += 2;

    DeviceGuard dg(b->device);
    auto bail = [&](lbdem_status s) {
        release(b);
        delete b;
        return s;
    };
    cudaError_t e;
#define TRY(call)                                                                               \
    if ((e = (call)) != cudaSuccess) {                                                          \
        cudaGetLastError();                                                                     \
        return bail(e == cudaErrorMemoryAllocation ? LBDEM_ERR_OUT_OF_MEMORY : LBDEM_ERR_CUDA); \
    }
    TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    const size_t capn = (size_t)std::max(b->nslots, 1);
    TRY(dalloc(b, &b->f, b->f_elems * b->esz + ALLOC_TAIL));
    TRY(dalloc(b, &b->vox, b->vox_elems * sizeof(uint32_t) + ALLOC_TAIL));
    if (b->prec == LBDEM_PREC_FP64) TRY(dalloc(b, &b->up, b->up_elems * b->esz + ALLOC_TAIL));
    TRY(dalloc(b, &b->btab, (size_t)126 * ndomains * b->esz));
    b->rec_off = round_up(sizeof(int) * (size_t)ndomains, 16);
    b->stage_bytes = b->rec_off + capn * REC_STRIDE * sizeof(double);
    TRY(dalloc(b, &b->d_stage, b->stage_bytes));
    b->d_ncur = (int*)b->d_stage;
    b->d_rec = (double*)(b->d_stage + b->rec_off);
    TRY(dalloc(b, &b->d_sph, capn * sizeof(SphereDev)));
    TRY(dalloc(b, &b->d_fast, capn * sizeof(SphereFast)));
    TRY(dalloc(b, &b->d_xpf, capn * XPF_STRIDE * sizeof(float)));
    TRY(dalloc(b, &b->d_tag2slot, sizeof(int) * ((size_t)c.max_tag + 1) * ndomains));
    TRY(dalloc(b, &b->d_tile_cnt, sizeof(int) * (size_t)std::max(b->ntiles, 1)));
    TRY(dalloc(b, &b->d_bins, sizeof(int) * TILE_BIN * (size_t)std::max(b->ntiles, 1)));
    TRY(dalloc(b, &b->d_work, sizeof(int) * (size_t)std::max(b->ntiles, 1)));
    TRY(dalloc(b, &b->d_work_n, sizeof(int) * 4));
    TRY(dalloc(b, &b->d_ft, sizeof(double) * 6 * capn));
    TRY(dalloc(b, &b->d_err, sizeof(unsigned)));
    TRY(dalloc(b, &b->d_views, sizeof(DomView) * ndomains));
    TRY(dalloc(b, &b->d_soff, sizeof(int) * ndomains));
    TRY(dalloc(b, &b->d_toff, sizeof(int) * ndomains));
    TRY(dalloc(b, &b->d_seg0, sizeof(int) * 2 * (size_t)ndomains));
    TRY(dalloc(b, &b->d_dargs, (b->prec == LBDEM_PREC_FP64 ? sizeof(CollideArgs<double>) : sizeof(CollideArgs<float>)) *
                                   2 * (size_t)ndomains));
    TRY(alloc_should_fail() ? cudaErrorMemoryAllocation : cudaMallocHost((void**)&b->h_stage, b->stage_bytes));
    TRY(alloc_should_fail() ? cudaErrorMemoryAllocation : cudaMallocHost((void**)&b->h_ft, sizeof(double) * 6 * capn));
    TRY(alloc_should_fail() ? cudaErrorMemoryAllocation : cudaMallocHost((void**)&b->h_err, sizeof(unsigned)));
    std::memset(b->h_stage, 0, b->stage_bytes);

    TRY(cudaMemset(b->f, 0, b->f_elems * b->esz + ALLOC_TAIL));
    TRY(cudaMemset(b->vox, 0, b->vox_elems * sizeof(uint32_t) + ALLOC_TAIL));
    if (b->up) TRY(cudaMemset(b->up, 0, b->up_elems * b->esz));
    TRY(cudaMemset(b->d_tile_cnt, 0, sizeof(int) * (size_t)std::max(b->ntiles, 1)));
    TRY(cudaMemset(b->d_work_n, 0, sizeof(int) * 4));
    TRY(cudaMemset(b->d_err, 0, sizeof(unsigned)));
    TRY(cudaMemset(b->d_ft, 0, sizeof(double) * 6 * capn));
    TRY(cudaMemset(b->d_stage, 0, b->stage_bytes));

    // B(n) per domain, src/ibCompositeDynamics3D.hh:178-179 (as lbdem_create)
    std::vector<double> bt((size_t)126 * ndomains);
    for (int d = 0; d < ndomains; ++d) {
        const double ooo = 1. / domains[d].omega - 0.5;
        for (int n = 0; n < 126; ++n) {
            const double sf = (1. / 125.) * (double)n;
            bt[(size_t)126 * d + n] = sf * ooo / ((1. - sf) + ooo);
        }
        bt[(size_t)126 * d] = 0.0;
        bt[(size_t)126 * d + 125] = 1.0;
    }
    if (b->prec == LBDEM_PREC_FP64) {
        TRY(cudaMemcpy(b->btab, bt.data(), bt.size() * sizeof(double), cudaMemcpyHostToDevice));
    } else {
        std::vector<float> bf(bt.begin(), bt.end());
        TRY(cudaMemcpy(b->btab, bf.data(), bf.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    TRY(cudaMemcpy(b->d_views, b->views.data(), sizeof(DomView) * ndomains, cudaMemcpyHostToDevice));
    TRY(cudaMemcpy(b->d_soff, b->soff.data(), sizeof(int) * ndomains, cudaMemcpyHostToDevice));
    TRY(cudaMemcpy(b->d_toff, b->toff.data(), sizeof(int) * ndomains, cudaMemcpyHostToDevice));
    TRY(cudaMemcpy(b->d_seg0, b->seg0.data(), sizeof(int) * b->seg0.size(), cudaMemcpyHostToDevice));
    if (b->prec == LBDEM_PREC_FP64) {
        std::vector<CollideArgs<double>> a;
        fill_dargs<double>(b, a, (double*)b->f, b->d_ft);
        TRY(cudaMemcpy(b->d_dargs, a.data(), sizeof(a[0]) * a.size(), cudaMemcpyHostToDevice));
    } else {
        std::vector<CollideArgs<float>> a;
        fill_dargs<float>(b, a, (float*)b->f, b->d_ft);
        TRY(cudaMemcpy(b->d_dargs, a.data(), sizeof(a[0]) * a.size(), cudaMemcpyHostToDevice));
    }

    if (b->njobs > 0) {
        std::vector<PlaneJob> jobs;
        long long maxcells = 1;
        for (int d = 0; d < ndomains; ++d) {
            if (!domains[d].has_pressure_drop) continue;
            const lbdem_pressure_drop& p = domains[d].drop;
            const int k = (int)jobs.size();
            for (int side = 0; side < 2; ++side) {
                PlaneJob j;
                j.f = (char*)b->f + b->views[d].f0 * b->esz;
                j.g = b->views[d].g;
                const int32_t* box = side == 0 ? p.inlet : p.outlet;
                for (int q = 0; q < 6; ++q) j.box[q] = box[q];
                j.dim = p.dimension;
                j.dir = side == 0 ? p.in_direction : p.out_direction;
                j.target = side == 0 ? p.rho_in : p.rho_out;
                j.read = side == 0 ? k + 1 : k;   // inlet rescaled with the outlet average and vice versa
                j.write = k + side;
                jobs.push_back(j);
                maxcells = std::max(maxcells, box_cells(box));
            }
        }
        b->plane_bpj = (int)std::max(1LL, std::min<long long>((maxcells + 2 * PLANE_THREADS - 1) / (2 * PLANE_THREADS),
                                                              PLANE_BLOCKS_MAX));
        TRY(dalloc(b, &b->d_jobs, sizeof(PlaneJob) * b->njobs));
        TRY(dalloc(b, &b->d_pavg, sizeof(double) * 2 * b->njobs));
        TRY(dalloc(b, &b->d_ppart, sizeof(double) * PLANE_BLOCKS_MAX * b->njobs));
        TRY(dalloc(b, &b->d_pcount, sizeof(unsigned) * b->njobs));
        TRY(cudaMemcpy(b->d_jobs, jobs.data(), sizeof(PlaneJob) * b->njobs, cudaMemcpyHostToDevice));
        TRY(cudaMemset(b->d_pavg, 0, sizeof(double) * 2 * b->njobs));
        TRY(cudaMemset(b->d_pcount, 0, sizeof(unsigned) * b->njobs));
    }
    TRY(cudaDeviceSynchronize());
#undef TRY
    *out = b;
    return LBDEM_OK;
}

lbdem_status lbdem_batch_destroy(lbdem_batch* b) {
    if (!b) return LBDEM_ERR_INVALID_ARG;
    {
        DeviceGuard dg(b->device);
        cudaStreamSynchronize(b->stream);
        release(b);
    }
    delete b;
    return LBDEM_OK;
}

lbdem_status lbdem_batch_init_equilibrium(lbdem_batch* b, double rho_bar, const double u[3]) {
    if (!b || !u) return fail(b, LBDEM_ERR_INVALID_ARG, "batch_init_equilibrium: null argument");
    if (!(rho_bar > -1.0) || !std::isfinite(rho_bar)) return fail(b, LBDEM_ERR_INVALID_ARG, "rho_bar <= -1");
    DeviceGuard dg(b->device);
    const int phase = (int)(b->step & 1);
    for (int d = 0; d < b->ndom; ++d) {
        if (b->prec == LBDEM_PREC_FP64)
            BK(b, launch_fill_equilibrium<double>(fptr<double>(b, d), rho_bar, u, phase, b->views[d].g, b->stream));
        else
            BK(b, launch_fill_equilibrium<float>(fptr<float>(b, d), rho_bar, u, phase, b->views[d].g, b->stream));
        b->launches += 1;
    }
    b->pavg_valid = false;
    return LBDEM_OK;
}

lbdem_status lbdem_batch_init_profile(lbdem_batch* b, int32_t domain, int32_t kind, double rho_hi, double rho_lo,
                                      double u_max, const int32_t n[3], int32_t dimension) {
    if (!b) return LBDEM_ERR_INVALID_ARG;
    if (domain < 0 || domain >= b->ndom) return fail(b, LBDEM_ERR_INVALID_ARG, "batch_init_profile: domain");
    if (!n || (kind != LBDEM_PROFILE_PRESSURE_GRADIENT && kind != LBDEM_PROFILE_POISEUILLE) || dimension < 0 ||
        dimension > 2 || n[dimension] < 2)
        return fail(b, LBDEM_ERR_INVALID_ARG, "batch_init_profile: kind, dimension or n");
    if (kind == LBDEM_PROFILE_POISEUILLE)
        for (int k = 0; k < 3; ++k)
            if (n[k] < 1) return fail(b, LBDEM_ERR_INVALID_ARG, "batch_init_profile: n < 1");
    if (!std::isfinite(rho_hi) || !std::isfinite(rho_lo) || !std::isfinite(u_max))
        return fail(b, LBDEM_ERR_INVALID_ARG, "batch_init_profile: non-finite parameter");
    const Geom& g = b->views[domain].g;
    const int ext[3] = {g.nx, g.ny, g.nz};
    const double slope = (rho_hi - rho_lo) / (double)(n[dimension] - 1);
    if (!(rho_hi > 0.0) || !(rho_hi - slope * (ext[dimension] - 1) > 0.0))
        return fail(b, LBDEM_ERR_INVALID_ARG, "batch_init_profile: density not positive on the lattice");
    DeviceGuard dg(b->device);
    const int phase = (int)(b->step & 1);
    if (b->prec == LBDEM_PREC_FP64)
        BK(b, launch_init_profile<double>(fptr<double>(b, domain), phase, kind, rho_hi, rho_lo, u_max, n[0], n[1],
                                          n[2], dimension, g, b->stream));
    else
        BK(b, launch_init_profile<float>(fptr<float>(b, domain), phase, kind, rho_hi, rho_lo, u_max, n[0], n[1], n[2],
                                         dimension, g, b->stream));
    b->launches += 1;
    b->pavg_valid = false;
    return LBDEM_OK;
}

lbdem_status lbdem_batch_set_particles(lbdem_batch* b, const int32_t* counts, const double* rec, int32_t init_vel) {
    if (!b || !counts) return fail(b, LBDEM_ERR_INVALID_ARG, "batch_set_particles: null argument");
    long long total = 0;
    for (int d = 0; d < b->ndom; ++d) {
        if (counts[d] < 0) return fail(b, LBDEM_ERR_INVALID_ARG, "batch_set_particles: negative count");
        if (counts[d] > b->cap[d]) return fail(b, LBDEM_ERR_CAPACITY, "batch_set_particles: count exceeds capacity");
        total += counts[d];
    }
    if (total > 0 && !rec) return fail(b, LBDEM_ERR_INVALID_ARG, "batch_set_particles: null records");
    DeviceGuard dg(b->device);
    // the pinned table may still be read by a queued upload
    BK(b, cudaStreamSynchronize(b->stream));
    int* hn = (int*)b->h_stage;
    double* hr = (double*)(b->h_stage + b->rec_off);
    size_t k = 0;
    for (int d = 0; d < b->ndom; ++d) {
        hn[d] = counts[d];
        if (counts[d] > 0)
            std::memcpy(hr + (size_t)REC_STRIDE * b->soff[d], rec + (size_t)REC_STRIDE * k,
                        sizeof(double) * REC_STRIDE * counts[d]);
        k += counts[d];
    }
    b->counts.assign(counts, counts + b->ndom);
    b->init_vel = init_vel ? 1 : 0;
    return LBDEM_OK;
}

lbdem_status lbdem_batch_step(lbdem_batch* b) {
    if (!b) return LBDEM_ERR_INVALID_ARG;
    DeviceGuard dg(b->device);
    if (b->cfg.autotune && !b->tuned && b->step >= 1) {   // after one step: particles voxelized
        const lbdem_status st = b->prec == LBDEM_PREC_FP64 ? autotune<double>(b) : autotune<float>(b);
        if (st != LBDEM_OK) return st;
        drop_graphs(b);
    }
    const int P = (int)(b->step & 1);
    const bool stale = b->njobs > 0 && !b->pavg_valid;
    // the first step runs eagerly: it also performs the launchers' one-time
    // attribute and occupancy setup outside any capture
    if (b->cfg.use_graph && !b->init_vel && !stale && b->step >= 1) {
        if (!b->gexec[P]) {
            const lbdem_status st = capture(b, P);
            if (st != LBDEM_OK) return st;
        }
        BK(b, cudaGraphLaunch(b->gexec[P], b->stream));
    } else {
        BK(b, enqueue_step(b, P != 0, b->init_vel));
    }
    b->launches += launches_per_step(b, stale);
    if (b->njobs > 0) b->pavg_valid = true;
    if (b->init_vel) b->init_vel = 0;   // defineVelocity applies to the step it was staged for
    b->step += 1;
    return LBDEM_OK;
}

lbdem_status lbdem_batch_get_forces(lbdem_batch* b, double* force, double* torque) {
    if (!b) return LBDEM_ERR_INVALID_ARG;
    long long total = 0;
    for (int d = 0; d < b->ndom; ++d) total += b->counts[d];
    if (total > 0 && (!force || !torque)) return fail(b, LBDEM_ERR_INVALID_ARG, "batch_get_forces: null output");
    DeviceGuard dg(b->device);
    BK(b, cudaStreamSynchronize(b->stream));
    size_t k = 0;
    for (int d = 0; d < b->ndom; ++d) {
        const double* ft = b->h_ft + (size_t)6 * b->soff[d];
        const int n = b->counts[d], cap = b->cap[d];
        if (n > 0) {
            std::memcpy(force + 3 * k, ft, sizeof(double) * 3 * n);
            std::memcpy(torque + 3 * k, ft + 3 * (size_t)cap, sizeof(double) * 3 * n);
        }
        k += n;
    }
    if (*b->h_err) {
        char buf[96];
        std::snprintf(buf, sizeof(buf), "device error word 0x%x", *b->h_err);
        return fail(b, LBDEM_ERR_DEVICE, buf);
    }
    return LBDEM_OK;
}

lbdem_status lbdem_batch_cycle(lbdem_batch* b, const int32_t* counts, const double* rec, int32_t init_vel,
                               double* force, double* torque) {
    lbdem_status s = lbdem_batch_set_particles(b, counts, rec, init_vel);
    if (s != LBDEM_OK) return s;
    s = lbdem_batch_step(b);
    if (s != LBDEM_OK) return s;
    return lbdem_batch_get_forces(b, force, torque);
}

lbdem_status lbdem_batch_get_field(lbdem_batch* b, int32_t domain, int32_t which, void* host_buf) {
    if (!b || !host_buf) return fail(b, LBDEM_ERR_INVALID_ARG, "batch_get_field: null argument");
    if (domain < 0 || domain >= b->ndom) return fail(b, LBDEM_ERR_INVALID_ARG, "batch_get_field: domain");
    DeviceGuard dg(b->device);
    const DomView& v = b->views[domain];
    const size_t N = v.g.N;
    const int phase = (int)(b->step & 1);
    cudaStream_t s = b->stream;
    const size_t need = std::max(N * b->esz, 3 * N * sizeof(double));
    if (b->scratch_bytes < need) {
        if (b->scratch) cudaFree(b->scratch);
        b->scratch = nullptr;
        b->dev_bytes -= b->scratch_bytes;
        b->scratch_bytes = 0;
        BK(b, dalloc(b, &b->scratch, need));
        b->scratch_bytes = need;
    }
    switch (which) {
        case LBDEM_FIELD_POPULATIONS:
            for (int i = 0; i < Q; ++i) {
                if (b->prec == LBDEM_PREC_FP64)
                    BK(b, launch_pop_gather<double>(fptr<double>(b, domain), (double*)b->scratch, i, phase, v.g, s));
                else
                    BK(b, launch_pop_gather<float>(fptr<float>(b, domain), (float*)b->scratch, i, phase, v.g, s));
                b->launches += 1;
                BK(b, cudaMemcpyAsync((char*)host_buf + (size_t)i * N * b->esz, b->scratch, N * b->esz,
                                      cudaMemcpyDeviceToHost, s));
            }
            break;
        case LBDEM_FIELD_SOLID_FRACTION:
        case LBDEM_FIELD_PARTICLE_ID:
        case LBDEM_FIELD_SUBCELL_COUNT: {
            double* sf = which == LBDEM_FIELD_SOLID_FRACTION ? (double*)b->scratch : nullptr;
            int32_t* id = which == LBDEM_FIELD_PARTICLE_ID ? (int32_t*)b->scratch : nullptr;
            uint8_t* ns = which == LBDEM_FIELD_SUBCELL_COUNT ? (uint8_t*)b->scratch : nullptr;
            BK(b, launch_vox_fields(b->vox + v.cell0, sf, id, ns, v.g, s));
            b->launches += 1;
            const size_t bytes =
                which == LBDEM_FIELD_SOLID_FRACTION ? N * 8 : which == LBDEM_FIELD_PARTICLE_ID ? N * 4 : N;
            BK(b, cudaMemcpyAsync(host_buf, b->scratch, bytes, cudaMemcpyDeviceToHost, s));
            break;
        }
        case LBDEM_FIELD_PARTICLE_VELOCITY:
            if (b->up) {
                BK(b, cudaMemcpyAsync(host_buf, (char*)b->up + v.up0 * b->esz, 3 * N * b->esz, cudaMemcpyDeviceToHost,
                                      s));
            } else {   // FP32 form: recomputed from the owner particles of the domain's list
                BK(b, launch_owner_velocity(b->vox + v.cell0, b->d_tag2slot + v.tag0, b->cfg.max_tag, b->cap[domain],
                                            b->d_xpf + (size_t)XPF_STRIDE * v.s0, v.g, (float*)b->scratch, s));
                b->launches += 1;
                BK(b, cudaMemcpyAsync(host_buf, b->scratch, 3 * N * sizeof(float), cudaMemcpyDeviceToHost, s));
            }
            break;
        case LBDEM_FIELD_DENSITY:
        case LBDEM_FIELD_VELOCITY: {
            const bool vel = which == LBDEM_FIELD_VELOCITY;
            if (b->prec == LBDEM_PREC_FP64)
                BK(b, launch_macro<double>(fptr<double>(b, domain), phase, vel ? nullptr : (double*)b->scratch,
                                           vel ? (double*)b->scratch : nullptr, v.g, s));
            else
                BK(b, launch_macro<float>(fptr<float>(b, domain), phase, vel ? nullptr : (double*)b->scratch,
                                          vel ? (double*)b->scratch : nullptr, v.g, s));
            b->launches += 1;
            BK(b, cudaMemcpyAsync(host_buf, b->scratch, (vel ? 3 : 1) * N * sizeof(double), cudaMemcpyDeviceToHost, s));
            break;
        }
        default:
            return fail(b, LBDEM_ERR_INVALID_ARG, "batch_get_field: field not kept per domain");
    }
    BK(b, cudaStreamSynchronize(s));
    return LBDEM_OK;
}

lbdem_status lbdem_batch_synchronize(lbdem_batch* b) {
    if (!b) return LBDEM_ERR_INVALID_ARG;
    DeviceGuard dg(b->device);
    BK(b, cudaStreamSynchronize(b->stream));
    return LBDEM_OK;
}

lbdem_status lbdem_batch_get_step(lbdem_batch* b, int64_t* step) {
    if (!b || !step) return LBDEM_ERR_INVALID_ARG;
    *step = b->step;
    return LBDEM_OK;
}

lbdem_status lbdem_batch_get_launch_count(lbdem_batch* b, int64_t* count) {
    if (!b || !count) return LBDEM_ERR_INVALID_ARG;
    *count = b->launches;
    return LBDEM_OK;
}

lbdem_status lbdem_batch_device_bytes(lbdem_batch* b, size_t* bytes) {
    if (!b || !bytes) return LBDEM_ERR_INVALID_ARG;
    *bytes = b->dev_bytes;
    return LBDEM_OK;
}

lbdem_status lbdem_batch_cells(lbdem_batch* b, int64_t* cells) {
    if (!b || !cells) return LBDEM_ERR_INVALID_ARG;
    *cells = (int64_t)b->ncells;
    return LBDEM_OK;
}

lbdem_status lbdem_batch_get_tuning(lbdem_batch* b, int32_t* collide_blocks_per_sm, float* collide_ms) {
    if (!b) return LBDEM_ERR_INVALID_ARG;
    if (collide_blocks_per_sm) *collide_blocks_per_sm = b->collide_bps;
    if (collide_ms) *collide_ms = b->collide_ms;
    return LBDEM_OK;
}

lbdem_status lbdem_batch_set_tuning(lbdem_batch* b, int32_t collide_blocks_per_sm) {
    if (!b || collide_blocks_per_sm < 0) return LBDEM_ERR_INVALID_ARG;
    DeviceGuard dg(b->device);
    BK(b, cudaStreamSynchronize(b->stream));
    b->collide_bps = collide_blocks_per_sm;
    b->tuned = true;
    drop_graphs(b);
    return LBDEM_OK;
}

}  // extern "C"
