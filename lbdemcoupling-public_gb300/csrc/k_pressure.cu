// Periodic pressure drop across a periodic boundary and the equilibrium initial
// profiles of the channel cases.
//
// The pressure drop follows Zhang & Kwok, Phys. Rev. E 73, 047702 (2006), as the
// reference applies it (examples/showcaseRectChannel/showcaseRectChannel.cpp:253-273):
// the average densities of the inlet and outlet boxes are taken before
// collideAndStream (Palabos computeAverageDensity), and after it the populations
// entering each box through the periodic wrap are rescaled,
//   f_i + t_i <- (f_i + t_i) * rhoTarget / rhoAvg(other box),
// for the i with c_i[dimension] == direction
// (src/periodicPressureFunctionals3D.hh:121-159).
//
// One launch handles every box of every domain (one job per box).  Each thread
// owns whole cells: it rescales the cell's incoming populations and adds the
// cell's rhoBar (after the rescale) to the box sum, so the same launch also
// leaves the averages the next step's rescale needs.  The box sums are
// deterministic: per-block partial sums, added in block order by the last block
// of each job.
#include "lbdem_internal.h"

namespace lbdem {
namespace {

// Double operations without contraction, so that the rescale and the profiles are
// the correctly rounded sequence the CPU restatement evaluates.
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float tadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double tadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float tsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double tsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float tmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double tmul(double a, double b) { return __dmul_rn(a, b); }

// (v + t) k - t evaluated in double; the float lattice rounds the result once.
template <typename T>
__device__ __forceinline__ T rescale_pop(T v, double t, double k) {
    return (T)dsub(dmul(dadd((double)v, t), k), t);
}

__device__ __forceinline__ int comp(int i, int dim) { return dim == 0 ? cx(i) : (dim == 1 ? cy(i) : cz(i)); }

template <typename T, bool RESCALE>
__global__ void __launch_bounds__(PLANE_THREADS)
    k_plane_pressure(const PlaneJob* __restrict__ jobs, int phase, const double* __restrict__ avg_in,
                     double* __restrict__ avg_out, double* __restrict__ partial, unsigned* __restrict__ count) {
    __shared__ double s_warp[PLANE_THREADS / 32];
    __shared__ bool s_last;
    __shared__ double s_k;
    const PlaneJob J = jobs[blockIdx.y];
    T* __restrict__ f = (T*)J.f;
    const int ey = J.box[3] - J.box[2] + 1, ez = J.box[5] - J.box[4] + 1;
    const long long ncell = (long long)(J.box[1] - J.box[0] + 1) * ey * ez;
    if (RESCALE && threadIdx.x == 0) s_k = J.target / avg_in[J.read];   // one division per block
    __syncthreads();
    const double k = RESCALE ? s_k : 1.0;

    double acc = 0;
    auto cell = [&](int x, int y, int z) {
        T rb = T(0);   // the cell's rhoBar in the lattice type, widened once
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const size_t s = slot_index(i, x, y, z, phase, J.g);
            T v = f[s];
            if (RESCALE && comp(i, J.dim) == J.dir) {
                v = rescale_pop<T>(v, wt(i), k);
                f[s] = v;
            }
            rb += v;
        }
        acc += (double)rb;
    };
    if (ncell < 0x7fffffffLL) {   // planes: 32-bit index arithmetic
        const int nc = (int)ncell;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
            const int r = c / ez;
            const int yy = r % ey;
            cell(J.box[0] + r / ey, J.box[2] + yy, J.box[4] + (c - r * ez));
        }
    } else {
        for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell;
             c += (long long)gridDim.x * blockDim.x) {
            const long long r = c / ez;
            cell(J.box[0] + (int)(r / ey), J.box[2] + (int)(r % ey), J.box[4] + (int)(c % ez));
        }
    }

    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0;
        for (int w = 0; w < PLANE_THREADS / 32; ++w) b += s_warp[w];
        partial[(size_t)blockIdx.y * PLANE_BLOCKS_MAX + blockIdx.x] = b;
        __threadfence();
        s_last = atomicAdd(&count[blockIdx.y], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        const volatile double* p = partial + (size_t)blockIdx.y * PLANE_BLOCKS_MAX;
        double sum = 0;
        for (unsigned b = 0; b < gridDim.x; ++b) sum += p[b];
        avg_out[J.write] = 1.0 + sum / (double)ncell;       // fullRho(mean rhoBar)
        count[blockIdx.y] = 0;
    }
}

// Palabos iniCellAtEquilibrium with the functor's (density, velocity):
// rhoBar = density - 1, j = density u, f̄_i = feq_i(rhoBar, j), evaluated in the
// lattice type without contraction.
template <typename T>
__global__ void k_init_profile(T* __restrict__ f, int phase, int kind, double p_hi, double p_lo, double u_max,
                               int n0, int n1, int n2, int dim, Geom g) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.N; c += (size_t)gridDim.x * blockDim.x) {
        const int z = (int)(c % g.nz);
        const size_t r = c / g.nz;
        const int y = (int)(r % g.ny);
        const int x = (int)(r / g.ny);
        const int ii[3] = {x, y, z};
        const int nn[3] = {n0, n1, n2};
        // density = pHi - (pHi - pLo) * i / (n - 1)     (:250, :272)
        const double density = dsub(p_hi, dmul(dsub(p_hi, p_lo), (double)ii[dim]) / (double)(nn[dim] - 1));
        double u[3] = {0.0, 0.0, 0.0};
        if (kind == 1) {
            const int a = dim == 0 ? 1 : 0, b = dim == 2 ? 1 : 2;
            double pv[2];
            const int ia[2] = {ii[a], ii[b]}, na[2] = {nn[a], nn[b]};
#pragma unroll
            for (int q = 0; q < 2; ++q) {                    // poiseuilleVelocity, :293-298
                const double nHalf = (double)na[q] / 2.;
                const double xx = dsub((double)ia[q], nHalf) / nHalf;
                pv[q] = dsub(1., dmul(xx, xx));
            }
            u[dim] = dmul(dmul(u_max, pv[0]), pv[1]);
        }
        const T rb = (T)dsub(density, 1.0);
        const T rho = tadd(T(1), rb);
        const T j[3] = {tmul(rho, (T)u[0]), tmul(rho, (T)u[1]), tmul(rho, (T)u[2])};
        const T jSqr = tadd(tadd(tmul(j[0], j[0]), tmul(j[1], j[1])), tmul(j[2], j[2]));
        const T invRho = T(1) / rho;
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const T cj = tadd(tadd(tmul((T)cx(i), j[0]), tmul((T)cy(i), j[1])), tmul((T)cz(i), j[2]));
            const T quad = tsub(tmul(tmul(T(4.5), cj), cj), tmul(T(1.5), jSqr));
            const T e = tmul((T)wt(i), tadd(tadd(rb, tmul(T(3), cj)), tmul(invRho, quad)));
            f[slot_index(i, x, y, z, phase, g)] = e;
        }
    }
}

}  // namespace

template <typename T>
cudaError_t launch_plane_pressure(const PlaneJob* jobs, int njobs, int blocks_per_job, int phase, int rescale,
                                  const double* avg_in, double* avg_out, double* partial, unsigned* count,
                                  cudaStream_t s) {
    if (njobs <= 0) return cudaSuccess;
    if (blocks_per_job < 1) blocks_per_job = 1;
    if (blocks_per_job > PLANE_BLOCKS_MAX) blocks_per_job = PLANE_BLOCKS_MAX;
    const dim3 grid(blocks_per_job, njobs);
    if (rescale)
        k_plane_pressure<T, true><<<grid, PLANE_THREADS, 0, s>>>(jobs, phase, avg_in, avg_out, partial, count);
    else
        k_plane_pressure<T, false><<<grid, PLANE_THREADS, 0, s>>>(jobs, phase, avg_in, avg_out, partial, count);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_init_profile(T* f, int phase, int kind, double p_hi, double p_lo, double u_max, int n0, int n1,
                                int n2, int dim, Geom g, cudaStream_t s) {
    size_t b = (g.N + 255) / 256;
    if (b > 152 * 32) b = 152 * 32;
    k_init_profile<T><<<(unsigned)(b > 0 ? b : 1), 256, 0, s>>>(f, phase, kind, p_hi, p_lo, u_max, n0, n1, n2, dim, g);
    return cudaGetLastError();
}

#define INST(T)                                                                                                  \
    template cudaError_t launch_plane_pressure<T>(const PlaneJob*, int, int, int, int, const double*, double*,    \
                                                  double*, unsigned*, cudaStream_t);                             \
    template cudaError_t launch_init_profile<T>(T*, int, int, double, double, double, int, int, int, int, Geom,  \
                                                cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace lbdem
