// lbdem_voxelize_static: sphere voxelization into caller-owned cell arrays with
// no device allocation.
//
// Some callers cannot let a library allocate device memory: a host application
// that hands the whole GPU to its own pool allocator, or a coupling loop that
// must not pay the implicit device synchronisation of cudaMalloc/cudaFree.
// This entry point runs the same kernels as lbdem_set_particles (prepare,
// bin, voxelize) but takes its scratch -- sphere tables, tile bins and the tag
// map -- from one file-scope device array of fixed size, which every GPU that
// loads the library holds until the process exits.
//
// The array is shared by every call: calls whose GPU work overlaps (different
// streams, or different threads on one device) race on it.  The tile counters
// and the tag map are cleared by each call before use.
#include "lbdem_gpu.h"
#include "lbdem_internal.h"

#include <cstring>

using namespace lbdem;

namespace {

constexpr int STATIC_MAX_DEVICES = 64;
constexpr size_t ALIGN = 256;

constexpr size_t up_align(size_t b) { return (b + ALIGN - 1) / ALIGN * ALIGN; }

// Scratch regions, in order.
constexpr size_t OFF_SPH = 0;
constexpr size_t OFF_FAST = OFF_SPH + up_align(sizeof(SphereDev) * LBDEM_STATIC_MAX_SPHERES);
constexpr size_t OFF_XPF = OFF_FAST + up_align(sizeof(SphereFast) * LBDEM_STATIC_MAX_SPHERES);
constexpr size_t OFF_TAG = OFF_XPF + up_align(sizeof(float) * XPF_STRIDE * LBDEM_STATIC_MAX_SPHERES);
constexpr size_t OFF_CNT = OFF_TAG + up_align(sizeof(int) * ((size_t)LBDEM_STATIC_MAX_TAG + 1));
constexpr size_t OFF_BINS = OFF_CNT + up_align(sizeof(int) * LBDEM_STATIC_MAX_TILES);
constexpr size_t OFF_WORK = OFF_BINS + up_align(sizeof(int) * TILE_BIN * (size_t)LBDEM_STATIC_MAX_TILES);
constexpr size_t OFF_WORKN = OFF_WORK + up_align(sizeof(int) * LBDEM_STATIC_MAX_TILES);
constexpr size_t SCRATCH_BYTES = OFF_WORKN + up_align(sizeof(int) * 4);

static_assert(SCRATCH_BYTES <= LBDEM_STATIC_SCRATCH_BYTES, "static scratch regions exceed the stated size");

// The scratch.  In host code this name only stands for the symbol; its device
// address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_scratch[LBDEM_STATIC_SCRATCH_BYTES];


}  // namespace

extern "C" lbdem_status lbdem_voxelize_static(int32_t nx, int32_t ny, int32_t nz, int32_t precision, int32_t n,
                                              const double* dev_rec, uint32_t* dev_vox, void* dev_up,
                                              uint32_t* dev_err, void* cuda_stream) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || nx >= (1 << 24) || ny >= (1 << 24) || nz >= (1 << 24))
        return LBDEM_ERR_INVALID_ARG;
    if (precision != LBDEM_PREC_FP64 && precision != LBDEM_PREC_FP32_DEV) return LBDEM_ERR_INVALID_ARG;
    if (n < 0) return LBDEM_ERR_INVALID_ARG;
    const long long tnx = (nx + TILE - 1) / TILE, tny = (ny + TILE - 1) / TILE, tnz = (nz + TILE - 1) / TILE;
    const long long ntiles = tnx * tny * tnz;
    if (ntiles > LBDEM_STATIC_MAX_TILES || n > LBDEM_STATIC_MAX_SPHERES) return LBDEM_ERR_CAPACITY;
    if (!dev_vox || !dev_up || !dev_err || (n > 0 && !dev_rec)) return LBDEM_ERR_INVALID_ARG;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return LBDEM_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= STATIC_MAX_DEVICES) return LBDEM_ERR_NO_DEVICE;
    // The array's device address on the current device, looked up on every call
    // (a host-side lookup, no GPU work): nothing is cached that a device reset
    // or a second thread could invalidate.
    void* addr = nullptr;
    if (cudaGetSymbolAddress(&addr, g_scratch) != cudaSuccess || !addr) {
        cudaGetLastError();
        return LBDEM_ERR_CUDA;
    }
    unsigned char* base = static_cast<unsigned char*>(addr);
    SphereDev* sph = reinterpret_cast<SphereDev*>(base + OFF_SPH);
    SphereFast* fast = reinterpret_cast<SphereFast*>(base + OFF_FAST);
    float* xpf = reinterpret_cast<float*>(base + OFF_XPF);
    int* tag2slot = reinterpret_cast<int*>(base + OFF_TAG);
    int* tile_cnt = reinterpret_cast<int*>(base + OFF_CNT);
    int* bins = reinterpret_cast<int*>(base + OFF_BINS);
    int* work = reinterpret_cast<int*>(base + OFF_WORK);
    int* work_n = reinterpret_cast<int*>(base + OFF_WORKN);

    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    Geom g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.per[0] = g.per[1] = g.per[2] = 1;   // used only when populations are initialised
    g.N = (size_t)nx * ny * nz;

    // what must start from zero (the tile counters, the work-list counters) or
    // from "no particle" (the tag map)
    if (cudaMemsetAsync(tile_cnt, 0, sizeof(int) * (size_t)ntiles, s) != cudaSuccess ||
        cudaMemsetAsync(work_n, 0, sizeof(int) * 4, s) != cudaSuccess ||
        cudaMemsetAsync(tag2slot, 0x7F, sizeof(int) * ((size_t)LBDEM_STATIC_MAX_TAG + 1), s) != cudaSuccess)
        return LBDEM_ERR_CUDA;
    if (n == 0) return LBDEM_OK;   // no sphere touches a cell (as in the reference)
    cudaError_t e = launch_prepare_bin(dev_rec, n, sph, fast, xpf, tag2slot, dev_err, g, LBDEM_STATIC_MAX_TAG,
                                       LBDEM_STATIC_MAX_RADIUS, nullptr, nullptr, tile_cnt, bins, work, work_n, s);
    const OwnerTable ot{xpf, tag2slot, LBDEM_STATIC_MAX_TAG};
    if (e == cudaSuccess) {
        if (precision == LBDEM_PREC_FP64) {
            e = launch_voxelize<double>(sph, fast, n, tile_cnt, bins, work, work_n, (int)ntiles, dev_vox,
                                        static_cast<double*>(dev_up), nullptr, 0, 0, g, ot, s);
        } else {
            // FP32 form: the velocity field is the one the handle's collision
            // recomputes from the owner particles (lbdem_get_field)
            e = launch_voxelize<float>(sph, fast, n, tile_cnt, bins, work, work_n, (int)ntiles, dev_vox, nullptr,
                                       nullptr, 0, 0, g, ot, s);
            if (e == cudaSuccess)
                e = launch_owner_velocity(dev_vox, tag2slot, LBDEM_STATIC_MAX_TAG, n, xpf, g,
                                          static_cast<float*>(dev_up), s);
        }
    }
    return e == cudaSuccess ? LBDEM_OK : LBDEM_ERR_CUDA;
}
