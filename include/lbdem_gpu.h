/*
 * lbdem_gpu.h -- C ABI of the GB300 partially-saturated-cells (PSM) lattice step.
 *
 * One handle owns one D3Q19 lattice resident in GPU memory together with its
 * per-cell coupling state (solid fraction, owner particle tag, particle surface
 * velocity) and the per-particle force/torque accumulators.  A coupling cycle
 * of the LBDEMcoupling reference maps onto three calls:
 *
 *   reference (LBDEMcoupling)                         this ABI
 *   setSpheresOnLattice(...)                          lbdem_set_particles
 *     src/ibDataExchangeWrappers3D.hh:33-146            (voxelization kernel)
 *   lattice.collideAndStream() with IBcompositeDynamics lbdem_collide_and_stream
 *     src/ibCompositeDynamics3D.hh:130-203              (fused collide-stream kernel,
 *                                                       force/torque reduction fused)
 *   getForcesFromLattice(...)                         lbdem_get_forces
 *     src/ibDataExchangeWrappers3D.hh:160-246           (reads back F and T)
 *
 * Conventions
 *  - Every call returns lbdem_status; LBDEM_OK is 0.  lbdem_last_error() gives
 *    a human-readable message for the last failing call on a handle.
 *  - Lattice units throughout (the caller converts with PhysUnits3D, exactly as
 *    the reference's wrappers do before calling SetSingleSphere3D).
 *  - Fields are laid out [component][x][y][z] with z fastest (Palabos order).
 *  - Populations are stored as f̄_i = f_i - t_i (Palabos' storage convention),
 *    in double (LBDEM_PREC_FP64, the drop-in form) or float
 *    (LBDEM_PREC_FP32_DEV, deviation form; force/torque still accumulate in
 *    double).
 *  - A handle is not thread-safe: one host thread per handle.  All GPU work of
 *    a handle is ordered on one CUDA stream (its own, or one set with
 *    lbdem_set_stream).  Host buffers belong to the caller; device memory
 *    belongs to the handle.
 *  - Functions ending in _device take device pointers and do not synchronize.
 */
#ifndef LBDEM_GPU_H
#define LBDEM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    LBDEM_OK = 0,
    LBDEM_ERR_INVALID_ARG = 1,  /* null handle/pointer, bad size, bad enum        */
    LBDEM_ERR_CUDA = 2,         /* a CUDA runtime call failed                      */
    LBDEM_ERR_OUT_OF_MEMORY = 3,/* device or pinned allocation failed              */
    LBDEM_ERR_CAPACITY = 4,     /* more particles / tags / overlaps than reserved  */
    LBDEM_ERR_DEVICE = 5,       /* the device error word is non-zero (see below)   */
    LBDEM_ERR_NO_DEVICE = 6     /* no CUDA device, or not a GB300-class device     */
} lbdem_status;

/* Bits of the device error word (lbdem_get_device_errors). */
#define LBDEM_DEVERR_TILE_LIST     0x1u  /* kept for compatibility; no longer raised (a tile's
                                            spheres are re-collected without a limit)        */
#define LBDEM_DEVERR_TAG_RANGE     0x4u  /* a particle tag is < 1 or > max_tag              */
#define LBDEM_DEVERR_UNMAPPED_TAG  0x8u  /* a solid cell names a tag with no particle       */
#define LBDEM_DEVERR_RADIUS        0x10u /* a radius is not finite, <= 0 or > max_radius    */
#define LBDEM_DEVERR_TIMEOUT       0x20u /* a bounded wait for staged data gave up           */

typedef enum {
    LBDEM_PREC_FP64 = 0,     /* populations in double: the drop-in form            */
    LBDEM_PREC_FP32_DEV = 1  /* populations f̄ = f - t_i in float, F/T in double   */
} lbdem_precision;

typedef enum {
    LBDEM_FIELD_POPULATIONS = 0,      /* f̄_i, [19][N], lattice element type           */
    LBDEM_FIELD_SOLID_FRACTION = 1,   /* double[N]  (IBscalarQuantity SolidFraction)   */
    LBDEM_FIELD_PARTICLE_ID = 2,      /* int32[N]   (IBscalarQuantity ParticleId)      */
    LBDEM_FIELD_PARTICLE_VELOCITY = 3,/* [3][N] lattice type (IBvectorQuantity ParticleVelocity) */
    LBDEM_FIELD_HYDRO_FORCE = 4,      /* [3][N] lattice type (IBvectorQuantity HydrodynamicForce);
                                         needs LBDEM_FLAG_CELL_FORCE                       */
    LBDEM_FIELD_DENSITY = 5,          /* double[N]  rho = 1 + sum f̄_i                    */
    LBDEM_FIELD_VELOCITY = 6,         /* double[3][N]  u = j / rho                        */
    LBDEM_FIELD_SUBCELL_COUNT = 7     /* uint8[N]   solid sub-cell count n, sf = n/125    */
} lbdem_field;

/* Keep the per-cell hydrodynamic force field (for export).  Off by default: the
 * force/torque sum is fused into the collide-stream kernel and needs no field. */
#define LBDEM_FLAG_CELL_FORCE 0x1
/* Failure-path test hook: in every collide-stream step of the handle, each warp's
 * first wait for its staged data waits on a barrier that nothing completes
 * (bounded), so the step takes the path of a copy that never lands: the kernel
 * sets LBDEM_DEVERR_TIMEOUT, lets its copies in flight land and returns early
 * (the step's populations are then not valid).  Applies to the FP64 form and to
 * rows that are not 16-byte aligned (the staging that waits on barriers). */
#define LBDEM_FLAG_PROBE_TIMEOUT 0x2

typedef struct {
    int32_t nx, ny, nz;       /* lattice extent in cells                              */
    int32_t periodic[3];      /* 1 = periodic axis, 0 = half-way bounce-back walls    */
    double omega;             /* BGK relaxation frequency 1/tau, 0 < omega < 2        */
    double body_force[3];     /* Guo body-force acceleration; zero = reference form   */
    int32_t precision;        /* lbdem_precision                                      */
    int32_t device;           /* CUDA device ordinal                                  */
    int32_t max_particles;    /* capacity of one particle list, ghosts included       */
    int32_t max_tag;          /* largest particle tag that may appear (< 2^25)        */
    double max_radius;        /* largest sphere radius in lattice units               */
    int32_t flags;            /* LBDEM_FLAG_*                                         */
    int32_t reserved;
} lbdem_config;

typedef struct lbdem_handle lbdem_handle;

/* Failure-path test hook: the nth device or pinned allocation made by
 * lbdem_create or lbdem_batch_create from now on (process-wide) reports failure
 * without being made; nth <= 0 switches the hook off.  A creation that meets it
 * returns LBDEM_ERR_OUT_OF_MEMORY after releasing what it had allocated. */
void lbdem_debug_fail_allocation(int32_t nth);

/* Fills cfg with defaults: 32^3 periodic, omega 1, FP64, device 0,
 * 1024 particles, max_tag 1<<20, max_radius 16. */
void lbdem_config_default(lbdem_config* cfg);

/* Creates a lattice at rest (f̄ = 0, i.e. rho = 1, u = 0; Palabos
 * lattice.initialize()) with every cell free of particles. */
lbdem_status lbdem_create(const lbdem_config* cfg, lbdem_handle** out);
lbdem_status lbdem_destroy(lbdem_handle* h);
const char* lbdem_last_error(const lbdem_handle* h);
const char* lbdem_status_string(lbdem_status s);

/* BGK relaxation frequency of every cell, 0 < omega < 2: what
 * defineDynamics(lattice, lattice.getBoundingBox(), new IBcompositeDynamics<T,D>(
 * new BGKdynamics<T,D>(omega))) sets in the reference's case drivers
 * (examples/sedimentingSphere/sedimentingSphere.cpp:181).  Waits for the
 * handle's queued work. */
lbdem_status lbdem_set_omega(lbdem_handle* h, double omega);

/* Periodicity per axis (1 periodic, 0 half-way bounce-back walls): Palabos'
 * lattice.periodicity().toggle(d, flag) / toggleAll(flag)
 * (sedimentingSphere.cpp:183, showcaseRectChannel.cpp:201).  Not allowed
 * while a pressure drop is set.  Waits for the handle's queued work. */
lbdem_status lbdem_set_periodic(lbdem_handle* h, const int32_t periodic[3]);

/* Orders the handle's GPU work on the given cudaStream_t (NULL: back to the
 * handle's own stream). */
lbdem_status lbdem_set_stream(lbdem_handle* h, void* cuda_stream);
lbdem_status lbdem_synchronize(lbdem_handle* h);

/* Uniform equilibrium: f̄_i = feq_i(rhoBar, j = (1 + rhoBar) u) in every cell
 * (Palabos initializeAtEquilibrium). */
lbdem_status lbdem_init_equilibrium(lbdem_handle* h, double rho_bar, const double u[3]);

/* Whole population field, [19][N] of the lattice element type, natural order
 * (f̄_i at cell x), independent of the in-place streaming phase. */
lbdem_status lbdem_set_populations(lbdem_handle* h, const void* host_f);
lbdem_status lbdem_get_populations(lbdem_handle* h, void* host_f);

/* setSpheresOnLattice / SetSingleSphere3D::process for n spheres applied in
 * index order (LIGGGHTS local atoms first, then ghost images, which repeat the
 * owner's tag).  x, v, omega: [n][3] doubles; r: [n]; tag: [n] int32 >= 1.
 * init_vel != 0 sets the populations of fully covered cells to the equilibrium
 * at the particle surface velocity (initVelFlag, src/ibProcessors3D.hh:107-108).
 * Host buffers; returns after the data has been staged (work is queued).
 * Replaces src/ibDataExchangeWrappers3D.hh:33-146 and src/ibProcessors3D.hh:53-184. */
lbdem_status lbdem_set_particles(lbdem_handle* h, int32_t n, const double* x, const double* v,
                                 const double* omega, const double* r, const int32_t* tag,
                                 int32_t init_vel);

/* Same, with the particle table already in device memory: rec is [n][12]
 * doubles {x0,x1,x2, v0,v1,v2, w0,w1,w2, r, tag, 0} (tag stored as a double).
 * The handle keeps its own copy, taken on its stream: rec may be reused once
 * the work queued so far on that stream has run. */
lbdem_status lbdem_set_particles_device(lbdem_handle* h, int32_t n, const double* rec,
                                        int32_t init_vel);

/* One lattice time step: PSM collision in every cell
 * (IBcompositeDynamics::collide, src/ibCompositeDynamics3D.hh:130-203)
 * followed by streaming, with the per-particle force and torque of
 * SumForceTorque3D (src/ibProcessors3D.hh:203-263) accumulated in double in
 * the same pass.  The sums refer to the particle list of the last
 * lbdem_set_particles call. */
lbdem_status lbdem_collide_and_stream(lbdem_handle* h);

/* Forces and torques of the last lbdem_collide_and_stream, lattice units,
 * [n][3] doubles indexed like the particle list: the entry of the first list
 * index carrying a tag holds that tag's sum, ghost-image entries are zero
 * (the reference's force/torque vectors, src/ibDataExchangeWrappers3D.hh:194-218).
 * Zero between an lbdem_set_particles and the step that follows it.
 * Synchronizes; returns LBDEM_ERR_DEVICE if the device error word is set. */
lbdem_status lbdem_get_forces(lbdem_handle* h, int32_t n, double* force, double* torque);

/* Device-pointer variant: copies 3n forces then 3n torques into dev_ft
 * (6n doubles) on the handle's stream; does not synchronize. */
lbdem_status lbdem_get_forces_device(lbdem_handle* h, int32_t n, double* dev_ft);

/* One coupling cycle (set particles, step, read forces) with host buffers. */
lbdem_status lbdem_cycle(lbdem_handle* h, int32_t n, const double* x, const double* v,
                         const double* omega, const double* r, const int32_t* tag,
                         int32_t init_vel, double* force, double* torque);

/* Copies one field to host memory (see lbdem_field for types and sizes). */
lbdem_status lbdem_get_field(lbdem_handle* h, int32_t which, void* host_buf);

/* Total mass sum_x sum_i (f̄_i + t_i), accumulated in double on the GPU. */
lbdem_status lbdem_mass(lbdem_handle* h, double* mass);

/* Reads and clears the device error word (LBDEM_DEVERR_* bits). */
lbdem_status lbdem_get_device_errors(lbdem_handle* h, uint32_t* bits);

/* Number of completed lattice steps. */
lbdem_status lbdem_get_step(lbdem_handle* h, int64_t* step);

/* Bytes of device memory held by the handle. */
lbdem_status lbdem_device_bytes(lbdem_handle* h, size_t* bytes);

/* Kernel launches issued by this handle since creation (all kernels of this
 * library; memset/memcpy not counted). */
lbdem_status lbdem_get_launch_count(lbdem_handle* h, int64_t* count);

/* ---- Checkpoint / resume ----------------------------------------------------
 * The per-cell coupling state IBcompositeDynamics::serialize writes
 * (src/ibCompositeDynamics3D.hh:77-107: solid fraction and owner as the voxel
 * word, particle surface velocity) together with the populations and the step
 * count, as one binary file: a header (magic "LBDEMCK1", format version,
 * nx, ny, nz, periodicity, precision, omega, body force, step), the populations
 * [19][N] in natural order, the voxel words [N] and the surface velocities
 * [3][N].  Loading needs a handle of the same extent and precision; the run
 * then continues exactly as the saved one would have (call lbdem_set_particles
 * before the next step, as after any step).  Both synchronize. */
lbdem_status lbdem_save_state(lbdem_handle* h, const char* path);
lbdem_status lbdem_load_state(lbdem_handle* h, const char* path);

/* ---- Periodic pressure drop and initial profiles ---------------------------
 * Boxes are Palabos Box3D: {x0, x1, y0, y1, z0, z1}, inclusive. */

/* Palabos computeAverageDensity(lattice, box) = 1 + mean rhoBar over the box.
 * Synchronizes. */
lbdem_status lbdem_average_density(lbdem_handle* h, const int32_t box[6], double* rho);

/* ZhangPeriodicPressureFunctional3D(rho_target, rho_avg, dimension, direction)
 * applied on box: f_i + t_i <- (f_i + t_i) rho_target / rho_avg for the
 * populations with c_i[dimension] == direction
 * (src/periodicPressureFunctionals3D.hh:121-159). */
lbdem_status lbdem_zhang_rescale(lbdem_handle* h, const int32_t box[6], int32_t dimension,
                                 int32_t direction, double rho_target, double rho_avg);

/* The pressure-driven periodic channel of examples/showcaseRectChannel
 * (showcaseRectChannel.cpp:253-273) done inside every lbdem_collide_and_stream:
 * the inlet and outlet average densities are those of the state before the
 * step, and after streaming the inlet populations with c[dimension] ==
 * in_direction are rescaled towards rho_in with the outlet average, the outlet
 * populations with c[dimension] == out_direction towards rho_out with the inlet
 * average.  One fused plane launch per step, no host synchronization. */
typedef struct {
    int32_t dimension;        /* 0 = x, 1 = y, 2 = z */
    int32_t inlet[6];         /* Box3D */
    int32_t outlet[6];        /* Box3D, disjoint from the inlet */
    int32_t in_direction;     /* +1 in the reference */
    int32_t out_direction;    /* -1 in the reference */
    double rho_in, rho_out;   /* rhoHi, rhoLo */
} lbdem_pressure_drop;

/* NULL switches the pressure drop off. */
lbdem_status lbdem_set_pressure_drop(lbdem_handle* h, const lbdem_pressure_drop* drop);

/* Equilibrium initial profiles (Palabos initializeAtEquilibrium over the whole
 * lattice with the reference's functors, src/periodicPressureFunctionals3D.hh):
 *   LBDEM_PROFILE_PRESSURE_GRADIENT: PressureGradient(rho_hi, rho_lo, n[dimension], dimension)
 *   LBDEM_PROFILE_POISEUILLE: PoiseuilleProfileAndPressureGradient(rho_hi, rho_lo, u_max,
 *                             n[0], n[1], n[2], dimension)
 * density = rho_hi - (rho_hi - rho_lo) i / (n - 1) along dimension; the Poiseuille
 * velocity u_max (1 - a^2)(1 - b^2), a = (i - n/2) / (n/2) in each other direction. */
typedef enum { LBDEM_PROFILE_PRESSURE_GRADIENT = 0, LBDEM_PROFILE_POISEUILLE = 1 } lbdem_profile;
lbdem_status lbdem_init_profile(lbdem_handle* h, int32_t kind, double rho_hi, double rho_lo,
                                double u_max, const int32_t n[3], int32_t dimension);

/* ---- Voxelization that allocates nothing ---------------------------------
 * No counterpart in the reference.  For callers that cannot have a library
 * allocate device memory: an application that gives the whole GPU to its own
 * pool allocator, or a coupling loop that must not pay the device-wide
 * synchronisation of cudaMalloc/cudaFree.  Applies SetSingleSphere3D for n
 * spheres, in list order, to cell state the caller owns -- exactly what
 * lbdem_set_particles does to a handle's state -- without a handle and
 * without any allocation: its scratch (sphere tables, tile bins, tag map) is
 * one static device array of LBDEM_STATIC_SCRATCH_BYTES that every GPU which
 * loads the library keeps until the process exits.
 *   nx, ny, nz   lattice extent; at most LBDEM_STATIC_MAX_TILES tiles of 8^3
 *                cells (e.g. 128^3 cells)
 *   precision    element type of dev_up (lbdem_precision)
 *   n, dev_rec   particle table in device memory, [n][12] doubles as for
 *                lbdem_set_particles_device; n <= LBDEM_STATIC_MAX_SPHERES,
 *                tags 1..LBDEM_STATIC_MAX_TAG, radii up to LBDEM_STATIC_MAX_RADIUS
 *                (a larger radius sets LBDEM_DEVERR_RADIUS and the sphere is
 *                skipped, as on a handle)
 *   dev_vox      [N] voxel words (count n | tag << 7), read and updated
 *   dev_up       [3][N] particle surface velocity.  FP64: read and updated
 *                (setValues of the reference).  FP32: written in full with the
 *                velocity the FP32 form's collision recomputes per cell from the
 *                owner particle (lbdem_get_field of a handle), the arm taken to
 *                the nearest image along every axis
 *   dev_err      one device word; LBDEM_DEVERR_* bits are OR-ed into it
 *   cuda_stream  stream of the work (NULL: the legacy default stream)
 * Sizes beyond the limits return LBDEM_ERR_CAPACITY before any GPU work.
 * The work is queued and not synchronized.  Every call looks up the array's
 * device address on the current device (cudaGetSymbolAddress, no GPU work);
 * the first call on a device may load the library's device code there, so
 * make that first call before any stream capture.  Every call uses the same
 * array: calls whose GPU work overlaps (on different streams or threads) race
 * on it.  Each call clears the tile counters and the tag map before using them. */
#define LBDEM_STATIC_MAX_SPHERES 4096
#define LBDEM_STATIC_MAX_TILES 4096
#define LBDEM_STATIC_MAX_TAG 65535
#define LBDEM_STATIC_MAX_RADIUS 1024.0
#define LBDEM_STATIC_SCRATCH_BYTES (3u << 20)
lbdem_status lbdem_voxelize_static(int32_t nx, int32_t ny, int32_t nz, int32_t precision, int32_t n,
                                   const double* dev_rec, uint32_t* dev_vox, void* dev_up, uint32_t* dev_err,
                                   void* cuda_stream);

/* ---- Adjoint ---------------------------------------------------------------
 * No counterpart in the reference.  Reverse-mode gradients of a loss built
 * from the per-particle forces and torques of a window of steps,
 *     L = sum_t sum_p weights[t][p] . (F_p(t), T_p(t)),
 * with respect to the per-step particle velocities and angular velocities,
 * the body force and tau.  Every cell's solid fraction and owner are held
 * fixed over the window and are not differentiated.  The call runs the window
 * forward from the handle's state exactly as nsteps calls of
 * lbdem_set_particles_device + lbdem_collide_and_stream would, keeps the
 * populations every checkpoint_every steps, then sweeps back segment by
 * segment, recomputing each segment once into a tape and applying the
 * hand-written reverse of collide-stream (transposed streaming, reverse
 * B-weighted PSM collision, reverse BGK with Guo forcing) step by step.
 *   rec        [nsteps][n][12] particle tables (host) as for
 *              lbdem_set_particles_device; positions, radii and tags must be
 *              identical in every step, velocities may change
 *   weights    [nsteps][n][6] dL/dF_p and dL/dT_p of every step (host)
 *   loss       out: L
 *   grad_vel   out [nsteps][n][6]: dL/dv_p(t), dL/domega_p(t), at the first
 *              list index of each tag (ghost-image entries zero)
 *   grad_body_force out [3], grad_tau out [1]
 *   grad_f0    optional out [19][N] of the lattice type, natural order: dL/d
 *              populations before the window
 * On return the handle holds the state after the window and the forces of its
 * last step.  Not available with a pressure drop set (not differentiated). */
lbdem_status lbdem_adjoint_window(lbdem_handle* h, int32_t nsteps, int32_t checkpoint_every, int32_t n,
                                  const double* rec, const double* weights, double* loss, double* grad_vel,
                                  double* grad_body_force, double* grad_tau, void* grad_f0);
/* Device time of the last lbdem_adjoint_window: forward pass and backward
 * pass (segment recomputation + adjoint steps), CUDA events. */
lbdem_status lbdem_adjoint_timing(lbdem_handle* h, float* forward_ms, float* backward_ms);

/* ---- Batched independent domains ------------------------------------------
 * No counterpart in the reference, which couples one lattice per process.
 * Many independent lattices of uneven size -- each with its own extent,
 * periodicity, omega, body force, particle list and optional periodic pressure
 * drop -- step together: each voxelization stage, the collide-stream pass and
 * the pressure-drop planes are one launch over all domains.  The device part of
 * a cycle (upload of the staged particle table, voxelization, collide-stream,
 * planes, download of the forces) is captured once per streaming phase into a
 * CUDA graph and replayed.  Every domain behaves exactly as an lbdem_handle
 * with the same configuration fed the same calls. */
typedef struct lbdem_batch lbdem_batch;

typedef struct {
    int32_t nx, ny, nz;
    int32_t periodic[3];
    double omega;
    double body_force[3];
    int32_t max_particles;          /* list capacity of this domain, ghost images included */
    int32_t has_pressure_drop;      /* 1: `drop` is applied in every step */
    lbdem_pressure_drop drop;
} lbdem_domain;

typedef struct {
    int32_t precision;              /* lbdem_precision, shared by all domains */
    int32_t device;
    int32_t max_tag;                /* tags 1..max_tag within every domain */
    double max_radius;
    int32_t use_graph;              /* 1: replay the device part of a cycle as a CUDA graph */
    int32_t autotune;               /* 1: time the collide-stream grid shapes on the first step */
    int32_t reserved[2];
} lbdem_batch_config;

void lbdem_batch_config_default(lbdem_batch_config* cfg);
lbdem_status lbdem_batch_create(const lbdem_batch_config* cfg, int32_t ndomains, const lbdem_domain* domains,
                                lbdem_batch** out);
lbdem_status lbdem_batch_destroy(lbdem_batch* b);
const char* lbdem_batch_last_error(const lbdem_batch* b);

/* Uniform equilibrium in every domain (as lbdem_init_equilibrium). */
lbdem_status lbdem_batch_init_equilibrium(lbdem_batch* b, double rho_bar, const double u[3]);
/* lbdem_init_profile on one domain. */
lbdem_status lbdem_batch_init_profile(lbdem_batch* b, int32_t domain, int32_t kind, double rho_hi, double rho_lo,
                                      double u_max, const int32_t n[3], int32_t dimension);

/* Stages the particles of every domain: counts[d] records for domain d, the
 * records of all domains back to back in domain order, [sum counts][12] doubles
 * as for lbdem_set_particles_device (host memory).  init_vel as for
 * lbdem_set_particles.  The table is uploaded by the next lbdem_batch_step. */
lbdem_status lbdem_batch_set_particles(lbdem_batch* b, const int32_t* counts, const double* rec, int32_t init_vel);

/* One coupling step of every domain: voxelization of the staged particles,
 * collide-stream with the force/torque sums, pressure-drop planes.  Queued,
 * not synchronized. */
lbdem_status lbdem_batch_step(lbdem_batch* b);

/* Forces and torques of the last step, [sum counts][3] each, indexed like the
 * staged records (per domain as lbdem_get_forces).  Synchronizes; returns
 * LBDEM_ERR_DEVICE if the device error word is set. */
lbdem_status lbdem_batch_get_forces(lbdem_batch* b, double* force, double* torque);

/* set_particles + step + get_forces. */
lbdem_status lbdem_batch_cycle(lbdem_batch* b, const int32_t* counts, const double* rec, int32_t init_vel,
                               double* force, double* torque);

/* Field of one domain (lbdem_field), host memory. */
lbdem_status lbdem_batch_get_field(lbdem_batch* b, int32_t domain, int32_t which, void* host_buf);

lbdem_status lbdem_batch_synchronize(lbdem_batch* b);
lbdem_status lbdem_batch_get_step(lbdem_batch* b, int64_t* step);
lbdem_status lbdem_batch_get_launch_count(lbdem_batch* b, int64_t* count);
lbdem_status lbdem_batch_device_bytes(lbdem_batch* b, size_t* bytes);
/* Total cells of all domains. */
lbdem_status lbdem_batch_cells(lbdem_batch* b, int64_t* cells);

/* Launch shape of the collide-stream pass: CTAs per SM of the persistent grid
 * (0: as many as fit).  Set by the autotuner or by hand. */
lbdem_status lbdem_batch_get_tuning(lbdem_batch* b, int32_t* collide_blocks_per_sm, float* collide_ms);
lbdem_status lbdem_batch_set_tuning(lbdem_batch* b, int32_t collide_blocks_per_sm);

#ifdef __cplusplus
}
#endif

#endif /* LBDEM_GPU_H */
