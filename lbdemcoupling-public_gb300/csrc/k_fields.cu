// Field export and initialisation kernels: population layout conversion for the
// in-place AA storage, uniform equilibrium, density/velocity, total mass and the
// voxel-word fields (the data of GetScalar/VectorQuantityFromDynamicsFunctional,
// src/ibDataWritingFunctionals3D.hh:32-114).
#include "lbdem_internal.h"

namespace lbdem {
namespace {

__device__ __forceinline__ void decompose(size_t c, const Geom& g, int& x, int& y, int& z) {
    z = (int)(c % g.nz);
    const size_t r = c / g.nz;
    y = (int)(r % g.ny);
    x = (int)(r / g.ny);
}

template <typename T>
__global__ void k_pop_gather(const T* __restrict__ f, T* __restrict__ out, int i, int phase, Geom g) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.N; c += (size_t)gridDim.x * blockDim.x) {
        int x, y, z;
        decompose(c, g, x, y, z);
        size_t s;
        switch (i) {
#define CASE(k) case k: s = slot_index(k, x, y, z, phase, g); break;
            CASE(0) CASE(1) CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8) CASE(9)
            CASE(10) CASE(11) CASE(12) CASE(13) CASE(14) CASE(15) CASE(16) CASE(17) CASE(18)
#undef CASE
            default: s = c;
        }
        out[c] = f[s];
    }
}

template <typename T>
__global__ void k_pop_scatter(T* __restrict__ f, const T* __restrict__ in, int i, int phase, Geom g) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.N; c += (size_t)gridDim.x * blockDim.x) {
        int x, y, z;
        decompose(c, g, x, y, z);
        size_t s;
        switch (i) {
#define CASE(k) case k: s = slot_index(k, x, y, z, phase, g); break;
            CASE(0) CASE(1) CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8) CASE(9)
            CASE(10) CASE(11) CASE(12) CASE(13) CASE(14) CASE(15) CASE(16) CASE(17) CASE(18)
#undef CASE
            default: s = c;
        }
        f[s] = in[c];
    }
}

template <typename T>
struct EqVals { T v[Q]; };

template <typename T>
__global__ void k_fill_equilibrium(T* __restrict__ f, EqVals<T> e, int phase, Geom g) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.N; c += (size_t)gridDim.x * blockDim.x) {
        if (phase == 0) {
#pragma unroll
            for (int i = 0; i < Q; ++i) f[(size_t)i * g.N + c] = e.v[i];
        } else {   // odd layout: f_i of a cell sits in slot (opp i, x - c_i), or (i, x) beyond a wall
            int x, y, z;
            decompose(c, g, x, y, z);
#pragma unroll
            for (int i = 0; i < Q; ++i) f[slot_index(i, x, y, z, phase, g)] = e.v[i];
        }
    }
}

template <typename T>
__global__ void k_macro(const T* __restrict__ f, int phase, double* __restrict__ rho, double* __restrict__ u,
                        Geom g) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.N; c += (size_t)gridDim.x * blockDim.x) {
        int x, y, z;
        decompose(c, g, x, y, z);
        double rb = 0, jx = 0, jy = 0, jz = 0;
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const double v = (double)f[slot_index(i, x, y, z, phase, g)];
            rb += v;
            if (cx(i)) jx += cx(i) * v;
            if (cy(i)) jy += cy(i) * v;
            if (cz(i)) jz += cz(i) * v;
        }
        const double r = 1.0 + rb;
        if (rho) rho[c] = r;
        if (u) { u[c] = jx / r; u[g.N + c] = jy / r; u[2 * g.N + c] = jz / r; }
    }
}

constexpr int MASS_THREADS = 256;
template <typename T>
__global__ void __launch_bounds__(MASS_THREADS) k_mass(const T* __restrict__ f, double* __restrict__ out, Geom g) {
    __shared__ double s_part[MASS_THREADS / 32];
    const size_t total = (size_t)Q * g.N;
    double acc = 0;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x)
        acc += (double)f[k];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < MASS_THREADS / 32 ? s_part[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) atomicAdd(out, v);
    }
}

__global__ void k_vox_fields(const uint32_t* __restrict__ vox, double* __restrict__ sf, int32_t* __restrict__ id,
                             uint8_t* __restrict__ nsub, Geom g) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.N; c += (size_t)gridDim.x * blockDim.x) {
        const uint32_t w = vox[c];
        const uint32_t n = w & VOX_NMASK;
        if (sf) sf[c] = (1.0 / 125.0) * (double)n;   // fraction * n, src/ibProcessors3D.hh:157
        if (id) id[c] = (int32_t)(w >> VOX_NBITS);
        if (nsub) nsub[c] = (uint8_t)n;
    }
}

inline unsigned grid_for(size_t n, int threads) {
    size_t b = (n + threads - 1) / threads;
    const size_t cap = 152 * 32;
    return (unsigned)(b < cap ? (b > 0 ? b : 1) : cap);
}

// Particle surface velocity field of the float form, [3][N]: the velocity the
// collision uses, recomputed per solid cell from its owner's float-table row
// (zero in free cells and in cells whose tag has no particle).
__global__ void k_owner_velocity(const uint32_t* __restrict__ vox, const int* __restrict__ tag2slot, int max_tag,
                                 int nslot, const float* __restrict__ xpf, Geom g, float* __restrict__ out) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.N; c += (size_t)gridDim.x * blockDim.x) {
        float u0 = 0.f, u1 = 0.f, u2 = 0.f;
        const int slot = owner_slot(vox[c], tag2slot, max_tag, nslot);
        if (slot >= 0) {
            int x, y, z;
            decompose(c, g, x, y, z);
            table_velocity(xpf + (size_t)slot * XPF_STRIDE, x, y, z, g, u0, u1, u2);
        }
        out[c] = u0;
        out[g.N + c] = u1;
        out[2 * g.N + c] = u2;
    }
}

}  // namespace

template <typename T>
cudaError_t launch_pop_gather(const T* f, T* out, int i, int phase, Geom g, cudaStream_t s) {
    k_pop_gather<T><<<grid_for(g.N, 256), 256, 0, s>>>(f, out, i, phase, g);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_pop_scatter(T* f, const T* in, int i, int phase, Geom g, cudaStream_t s) {
    k_pop_scatter<T><<<grid_for(g.N, 256), 256, 0, s>>>(f, in, i, phase, g);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_fill_equilibrium(T* f, double rho_bar, const double* u, int phase, Geom g, cudaStream_t s) {
    // Palabos iniCellAtEquilibrium: j = rho u; feq_i = t_i [rhoBar + 3 c.j + invRho (4.5 (c.j)^2 - 1.5 j.j)]
    EqVals<T> e;
    const T rb = T(rho_bar);
    const T rho = T(1) + rb;
    const T j[3] = {rho * T(u[0]), rho * T(u[1]), rho * T(u[2])};
    const T jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    const T invRho = T(1) / rho;
    for (int i = 0; i < Q; ++i) {
        const T cj = T(cx(i)) * j[0] + T(cy(i)) * j[1] + T(cz(i)) * j[2];
        e.v[i] = T(wt(i)) * (rb + T(3) * cj + invRho * (T(4.5) * cj * cj - T(1.5) * jSqr));
    }
    k_fill_equilibrium<T><<<grid_for(g.N, 256), 256, 0, s>>>(f, e, phase, g);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_macro(const T* f, int phase, double* rho, double* u, Geom g, cudaStream_t s) {
    k_macro<T><<<grid_for(g.N, 256), 256, 0, s>>>(f, phase, rho, u, g);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_mass(const T* f, double* out, Geom g, cudaStream_t s) {
    k_mass<T><<<grid_for((size_t)Q * g.N, MASS_THREADS), MASS_THREADS, 0, s>>>(f, out, g);
    return cudaGetLastError();
}
cudaError_t launch_owner_velocity(const uint32_t* vox, const int* tag2slot, int max_tag, int nslot, const float* xpf,
                                  Geom g, float* out, cudaStream_t s) {
    k_owner_velocity<<<grid_for(g.N, 256), 256, 0, s>>>(vox, tag2slot, max_tag, nslot, xpf, g, out);
    return cudaGetLastError();
}
cudaError_t launch_vox_fields(const uint32_t* vox, double* sf, int32_t* id, uint8_t* nsub, Geom g, cudaStream_t s) {
    k_vox_fields<<<grid_for(g.N, 256), 256, 0, s>>>(vox, sf, id, nsub, g);
    return cudaGetLastError();
}

#define INST(T)                                                                                      \
    template cudaError_t launch_pop_gather<T>(const T*, T*, int, int, Geom, cudaStream_t);           \
    template cudaError_t launch_pop_scatter<T>(T*, const T*, int, int, Geom, cudaStream_t);          \
    template cudaError_t launch_fill_equilibrium<T>(T*, double, const double*, int, Geom, cudaStream_t);  \
    template cudaError_t launch_macro<T>(const T*, int, double*, double*, Geom, cudaStream_t);       \
    template cudaError_t launch_mass<T>(const T*, double*, Geom, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace lbdem
