/*
 * pica_gb300.h -- C ABI of the GB300 particle-in-cell step.
 *
 * pica (the reference) is a header-only C++ library whose hot path is a set of
 * per-particle operators driven by a host loop: the Yee grid, the Yee solver,
 * the CIC field interpolator, the Boris pusher, the CIC current depositor and
 * the supercell ensemble.  Per-particle calls cannot be fast on a GPU, so this
 * ABI exposes the same operators at ensemble granularity: one call advances
 * every particle of every supercell.  A host loop that used the reference
 * classes calls these entry points once per step instead; pica_gb300.hpp is
 * the header-level C++ mirror of pica's class names over them.
 *
 * Conventions
 *  - Every function returns a status (PICA_OK = 0, negative = error); no C++
 *    exception crosses this boundary.  pica_last_error() gives the message.
 *  - The context owns all device memory.  Calls on one context are
 *    single-threaded and are enqueued on the context's stream.
 *  - Host arrays use pica's layouts: grid arrays are N^3, z fastest,
 *    index (i*ny + j)*nz + k (utility/Array.h:140-144); particles are SoA
 *    with positions in cm and momenta normalised as u = p/(m c)
 *    (particles/Particle.h:68-72, particles/ParticleArray.h:195-199).
 *  - Units are CGS, with pica's constants (math/Constants.h:10-18), including
 *    pi = 3.14159265358.
 */
#ifndef PICA_GB300_H
#define PICA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PICA_ABI_VERSION 1

/* Status codes. */
#define PICA_OK 0
#define PICA_ERR_INVALID (-1)   /* bad argument or configuration          */
#define PICA_ERR_CUDA (-2)      /* CUDA runtime error                     */
#define PICA_ERR_OOM (-3)       /* device or host allocation failed       */
#define PICA_ERR_OVERFLOW (-4)  /* supercell capacity could not be grown  */
#define PICA_ERR_MIGRATION (-5) /* a particle crossed more than one supercell in one step */
#define PICA_ERR_STATE (-6)     /* call out of order (e.g. push twice without migrate) */
#define PICA_ERR_NOT_BUILT (-7) /* form / shape / depositor combination not compiled */
#define PICA_ERR_LIMIT (-8)     /* size beyond a documented fixed limit   */
#define PICA_ERR_TIMEOUT (-9)   /* a bounded wait on the device gave up (an asynchronous copy never completed) */

/* Precision forms. */
#define PICA_FORM_FP64_PLAIN 0  /* FP64 absolute positions; pica's own arithmetic */
#define PICA_FORM_FP32_CELL 1   /* int cell index + FP32 in-cell offset, FP32 push */

/* Form factors (field interpolation and charge shape). */
#define PICA_SHAPE_CIC 1
#define PICA_SHAPE_TSC 2

/* Current depositors. */
#define PICA_DEPOSIT_DIRECT 0     /* pica CurrentDepositorCIC: q w v at the new position */
#define PICA_DEPOSIT_ESIRKEPOV 1  /* charge-conserving (Esirkepov 2001) */

typedef struct pica_config {
    int32_t n[3];        /* grid cells per dimension (periodic domain [0, n h))         */
    int32_t sc[3];       /* cells per supercell per dimension; n % sc == 0, sc <= 8      */
    double h[3];         /* cell size, cm                                                */
    double dt;           /* time step, s                                                 */
    int32_t form;        /* PICA_FORM_*                                                  */
    int32_t shape;       /* PICA_SHAPE_*                                                 */
    int32_t deposit;     /* PICA_DEPOSIT_*                                               */
    int32_t nspecies;    /* 1..4 (pica ParticleTypes table, particles/Particle.h:21-31)  */
    double mass[4];      /* g                                                            */
    double charge[4];    /* statC                                                        */
    double slack;        /* spare slots per supercell as a fraction of its count (0 -> 0.15) */
    int32_t resort_every;/* re-balance supercell capacities every k steps (0 = on overflow only) */
    int32_t threads;     /* host threads for upload/download/generation (0 = hardware) */
} pica_config;

typedef struct pica_diag {
    double field_energy;   /* sum over nodes of (E^2 + B^2) h^3 / (8 pi)         */
    double kinetic_energy; /* sum over particles of w m c^2 (gamma - 1)          */
    double total_charge;   /* sum over particles of q w                           */
    double gauss_max;      /* max over cells |div E - 4 pi (rho + bg)|            */
    double rho_max;        /* max over cells |rho| of the particles               */
    double pad_[3];
} pica_diag;

/* Synthetic plasma description for pica_plasma_generate (host-side set-up). */
typedef struct pica_plasma_spec {
    int32_t n[3];          /* cells                                              */
    int32_t species;       /* species index written for every particle           */
    double h[3];           /* cell size, cm                                      */
    double ppc;            /* mean particles per cell                            */
    double density_mod;    /* a: per-cell count = round(ppc (1 + a cos(2 pi (i+1/2)/nx)))  */
    double drift_u;        /* beam drift u = gamma beta along drift_axis         */
    double sigma_u;        /* Maxwellian spread of each u component              */
    double weight;         /* macro-particle factor                              */
    uint64_t seed;
    int32_t nbeams;        /* 1: one thermal population; 2: beams at +drift_u and -drift_u */
    int32_t drift_axis;    /* 0, 1, 2                                            */
} pica_plasma_spec;

typedef struct pica_ctx pica_ctx;

int         pica_abi_version(void);
const char* pica_status_string(int status);

/* Context.  Replaces constructing YeeGrid<Three,Real>(origin, step, size)
 * (grid/YeeGrid.h:193-256) together with EnsembleSupercells<PA>(min, max,
 * numCells, numCellsPerSupercell) (particles/EnsembleSupercells.h:25-34) and
 * BorisPusher<Particle,Real>(dt) (particlePush/BorisPusher.h:23-30). */
int         pica_ctx_create(const pica_config* cfg, pica_ctx** out);
int         pica_ctx_destroy(pica_ctx* ctx);
/* Stream for all work of this context (a cudaStream_t; NULL = legacy default stream). */
int         pica_set_stream(pica_ctx* ctx, void* stream);
int         pica_synchronize(pica_ctx* ctx);
const char* pica_last_error(pica_ctx* ctx);
/* Kernels this context has launched since creation (for launch accounting). */
int64_t     pica_launch_count(pica_ctx* ctx);
/* Launch shape of the FP32 charge-conserving push kernel (no counterpart in pica,
 * which has no GPU path): 0..count-1, chosen by pica_gb300.autotune.  All variants
 * give bit-identical results.  Variant 4 stages the E/B tile of interior
 * supercells with tensor-memory-accelerator copies (supercells of 4^3 cells on
 * grids of at least 12 cells per side; elsewhere, and in the batching form, it
 * launches as variant 0). */
int         pica_set_variant(pica_ctx* ctx, int32_t variant);
int         pica_get_variant(pica_ctx* ctx, int32_t* variant, int32_t* count);

/* Particles.  Replaces EnsembleSupercells::add (EnsembleSupercells.h:41-45) for
 * every particle: particles are routed to supercells by
 * floor(x / supercellSize) in input order.  species may be NULL (all 0). */
int     pica_upload_particles(pica_ctx* ctx, int64_t n, const double* x, const double* y, const double* z,
                              const double* ux, const double* uy, const double* uz, const double* w,
                              const int32_t* species);
int64_t pica_num_particles(pica_ctx* ctx);
/* Download in ensemble order: species, then supercell (linear (sx*nsy+sy)*nsz+sz),
 * then slot -- the order of EnsembleSupercells::getParticles(idx)[i].  Any pointer may be NULL. */
int     pica_download_particles(pica_ctx* ctx, double* x, double* y, double* z, double* ux, double* uy,
                                double* uz, double* w, int32_t* species, int32_t* supercell);
/* Per-supercell particle counts, counts[species * nsupercells + s]. */
int     pica_get_counts(pica_ctx* ctx, int32_t* counts);

/* Migration lists.  pica routes a particle by floor((x - min) / supercellSize)
 * (particles/EnsembleSupercells.h:54-57) and has no step that moves particles
 * between supercells; a host loop over it pops a particle whose route changed and
 * adds it to its new supercell.  With recording on (enable = 1; off by default),
 * every pica_migrate keeps the list of its moves: one entry per particle that
 * changed supercell, (species, source supercell, slot in the source supercell
 * before the move, destination supercell), ordered by species, then source
 * supercell, then slot.  pica_num_migrations gives the length of the last step's
 * list (0 before the first recorded step, -1 for a NULL context) and
 * pica_get_migrations copies it out (each pointer may be NULL).  Recording reads
 * the leaver lists back to the host once per step, so it is for checks and
 * debugging, not for timed runs.  Steps of a batch (pica_batch_step) are not
 * recorded. */
int     pica_record_migrations(pica_ctx* ctx, int32_t enable);
int64_t pica_num_migrations(pica_ctx* ctx);
int     pica_get_migrations(pica_ctx* ctx, int32_t* species, int32_t* src, int32_t* slot, int32_t* dst);

/* Domain decomposition of one plasma into slabs along x, each slab a context whose
 * grid holds its own cells plus guard layers on both x faces (pica reserves the
 * fields of a domain decomposition in Parameters.h:16-27 and plans one in
 * README.md:21; it has none).  All device buffers below are the caller's device
 * memory on this context's device; the copies run on the context stream.
 *
 * pica_field_slab: x-layers [x0, x0 + nx) of field component comp (0..8 = ex ey ez
 *   bx by bz jx jy jz; double in the FP64 form, float in the FP32 form) to the
 *   buffer (mode 0), from it (mode 1), or the buffer added to them (mode 2: the
 *   current a neighbour deposited into its guard layers).  A run of x-layers is
 *   contiguous (z fastest), so each call is one copy or one add kernel.  Allowed
 *   while a migration is pending (after push_deposit the FP32 form's J holds the
 *   step's current).
 * pica_take_supercells: moves the particles of supercells [sc_begin, sc_end) of one
 *   species out of the context: their slots, supercell by supercell, packed into
 *   the component buffers dev[0..ncomp) (components as for pica_state_copy), and
 *   those supercells left empty.  counts (host, may be NULL) receives each
 *   supercell's number.  Returns the total (>= 0) or a status.  dev == NULL
 *   returns the total and counts without taking anything.  PICA_ERR_LIMIT when the
 *   total exceeds capacity; PICA_ERR_STATE for supercells holding dead slots
 *   (the guard supercells a migration has just filled hold none).
 * pica_append_to_supercells: appends counts[i] packed particles (the layout
 *   pica_take_supercells writes) to the end of supercell sc_begin + i, shifting
 *   the FP32 form's cell x (or the FP64 form's x) by dx_cells cells into this
 *   context's frame.  PICA_ERR_OVERFLOW, with nothing written, when the arrivals
 *   exceed a supercell's spare slots (the caller then re-uploads the ensemble).
 * Both particle calls return PICA_ERR_STATE between push_deposit and migrate. */
int     pica_field_slab(pica_ctx* ctx, int32_t comp, int32_t x0, int32_t nx, void* dev, int32_t mode);
int64_t pica_take_supercells(pica_ctx* ctx, int32_t species, int32_t sc_begin, int32_t sc_end, void* const* dev,
                             int64_t capacity, int32_t* counts);
int     pica_append_to_supercells(pica_ctx* ctx, int32_t species, int32_t sc_begin, int32_t sc_end,
                                  const int32_t* counts, const void* const* dev, int32_t dx_cells);

/* Fields: f9 = {ex, ey, ez, bx, by, bz, jx, jy, jz}, each N^3 doubles.
 * Replaces element access YeeGrid::ex(i,j,k) ... (grid/YeeGrid.h:293-333). */
int     pica_upload_fields(pica_ctx* ctx, const double* const* f9);
int     pica_download_fields(pica_ctx* ctx, double* const* f9);

/* Operators.
 * pica_push_deposit: for every supercell, FieldInterpolatorCICSupercell::get
 *   (fieldInterpolation/FieldInterpolatorYeeGrid.h:197-242) or its TSC form,
 *   BorisPusher::push (particlePush/BorisPusher.h:33-47) and
 *   CurrentDepositorCICSupercell::deposit + flush (currentDeposition/
 *   CurrentDepositorYeeGrid.h:178-226) or Esirkepov deposition.  J is cleared
 *   first; the deposit is periodic.  Leaves the ensemble awaiting pica_migrate.
 * pica_update_b / pica_update_e: YeeSolver::updateB / updateE
 *   (fieldSolver/YeeSolver.h:177-213 / 132-175) on the periodic grid.
 * pica_migrate: wraps positions periodically and moves particles whose
 *   supercell changed (pica has no migration; order: stayers in slot order,
 *   then arrivals by direction code, each in source-slot order).
 * pica_step: push_deposit; update_b(dt/2); update_e(dt); update_b(dt/2); migrate. */
int     pica_push_deposit(pica_ctx* ctx);
/* Sort every supercell by cell now, dropping its dead slots (what the periodic
 * resort does every resort_every steps): the supercell layout's counterpart of
 * EnsembleOrdered::reorder (particles/EnsembleOrdered.h:61-71); here the order is
 * (species, supercell, cell, slot).  PICA_ERR_STATE between push_deposit and migrate. */
int     pica_reorder(pica_ctx* ctx);

/* Flat particle arrays: pica's EnsembleUnordered / EnsembleOrdered layouts
 * (particles/EnsembleUnordered.h:14-40, EnsembleOrdered.h:17-71), one SoA array of
 * FP64 particles in caller-owned device memory instead of supercells.
 *
 * pica_order_by_position: EnsembleOrdered::reorder on the device.  order[i] (device)
 *   is the index of the i-th particle in lexicographic position order over the
 *   first dims coordinates of x, y, z (device; y, z may be NULL below dims 2, 3),
 *   with pica's comparator (EnsembleOrdered.h:31-41; -0.0 equals +0.0).  Stable:
 *   ties keep input order, where pica's std::sort leaves them unspecified.
 *   Positions must not be NaN.  stream: a cudaStream_t (NULL: legacy default
 *   stream); allocates about 16 bytes per particle of scratch and frees it, and
 *   synchronises the stream.
 * pica_push_flat: one push of a flat array in any order, on the context's fields
 *   (FP64 plain form, direct deposition).  Per particle: the grid-level gather of
 *   FieldInterpolatorCIC<YeeGrid<Three,Real>> (fieldInterpolation/
 *   FieldInterpolatorYeeGrid.h:23-38, 137-183) for a pica grid whose origin is
 *   -guard cells (pica node g = context node g - guard, periodic), or the TSC
 *   gather on the nearest nodes; BorisPusher::push (particlePush/BorisPusher.h:
 *   33-47); CurrentDepositorCIC<YeeGrid<Three,Real>>::deposit (currentDeposition/
 *   CurrentDepositorYeeGrid.h:23-38, 126-163) of the current v (q w) / (hx hy hz)
 *   at the new position, added to J (zeroed first) with FP64 global atomics, whose
 *   order varies from run to run.  Positions then wrap periodically; the array
 *   order never changes.  The caller then runs pica_update_b / pica_update_e.
 *   species may be NULL (all 0).  Synchronises the context stream.
 *   PICA_ERR_NOT_BUILT for the FP32 form or the Esirkepov depositor; PICA_ERR_STATE
 *   between push_deposit and migrate; PICA_ERR_INVALID for a species out of range. */
int     pica_order_by_position(int64_t n, int32_t dims, const double* x, const double* y, const double* z,
                               int64_t* order, void* stream);
/* pica_order_by_position on host arrays (copied to the device and back); for host
 * containers such as the C++ mirror's EnsembleOrdered. */
int     pica_order_by_position_host(int64_t n, int32_t dims, const double* x, const double* y, const double* z,
                                    int64_t* order);
int     pica_push_flat(pica_ctx* ctx, int64_t n, double* x, double* y, double* z, double* ux, double* uy,
                       double* uz, const double* w, const int32_t* species, int32_t guard);
/* pica_push_flat on host arrays (copied to the device and back, x..uz updated in
 * place); for host containers such as the C++ mirror's EnsembleUnordered. */
int     pica_push_flat_host(pica_ctx* ctx, int64_t n, double* x, double* y, double* z, double* ux, double* uy,
                            double* uz, const double* w, const int32_t* species, int32_t guard);
/* pica_push_deposit as nchunks launches over consecutive ranges of supercells
 * (range r: linear supercells [nscTot r / nchunks, nscTot (r+1) / nchunks)), the
 * launch of range r enqueued on the context stream after a wait for
 * wait_events[r] (a cudaEvent_t; NULL entries and a NULL array wait for nothing).
 * A host loop that uploads the packed state range by range
 * (pica_state_copy_packed_range) records one event per range, and the push of
 * each range starts as soon as its particles are in.  Results equal those of
 * pica_push_deposit bit for bit (FP32 form).  Forms other than the FP32
 * Esirkepov one push in one launch after all the waits. */
int     pica_push_deposit_chunked(pica_ctx* ctx, int32_t nchunks, void* const* wait_events);
/* pica_push_deposit_chunked over ranges of the caller's choice: range r is
 * supercells [bounds[r], bounds[r+1]) (nranges + 1 bounds, not decreasing, from 0
 * to the supercell count; empty ranges launch nothing but still wait).  A host
 * loop that moves small ranges first and last keeps the link busy at the ends of
 * a step.  PICA_ERR_INVALID for bounds that do not cover the supercells. */
int     pica_push_deposit_ranges(pica_ctx* ctx, int32_t nranges, const int32_t* bounds, void* const* wait_events);
int     pica_update_b(pica_ctx* ctx, double dt);
int     pica_update_e(pica_ctx* ctx, double dt);
int     pica_migrate(pica_ctx* ctx);
int     pica_step(pica_ctx* ctx, int32_t nsteps);

/* FP64 reductions on the device.  bg_density is a uniform background charge
 * density (statC/cm^3) added to rho, e.g. immobile neutralising ions. */
int     pica_diagnostics(pica_ctx* ctx, double bg_density, pica_diag* out);
/* Charge density at cell centres (N^3 doubles, host), shape of the configured form factor. */
int     pica_charge_density(pica_ctx* ctx, double* rho);
/* Field energy sum over the grid (FP64, deterministic two-pass reduction). */
int     pica_field_energy(pica_ctx* ctx, double* out);

/* Field energy of six caller-owned device arrays (ex ey ez bx by bz, Array3d
 * order, n[0] x n[1] x n[2] nodes, double if fp64 else float) with no context
 * and no allocation, for callers that must not allocate: a diagnostics hook
 * beside a live step (cudaMalloc and cudaFree synchronise the device), an
 * application whose memory pool has reserved the device, or a component that
 * owns its fields but has no pica context.  The scratch is one static device
 * array of 16384 partial sums (128 KB), so grids above 512^3 = 134,217,728
 * nodes return PICA_ERR_LIMIT.  The first call on each device looks the
 * scratch address up (cudaGetSymbolAddress) with that device current.  With
 * CUDA's lazy module loading, the first call of
 * each precision on a device also loads its kernels and the static array, which
 * is an allocation: make one call per precision used at start-up; later calls
 * allocate nothing.  The address is kept for the life of the process, so a
 * process that resets the device (cudaDeviceReset) must not call this again.
 * Calls that can overlap on the GPU (other streams, other host threads) race on
 * the one scratch: serialise them.  Runs on `stream` (a cudaStream_t of the
 * current device, 0 for the legacy stream) and synchronises it; an error left
 * by earlier unrelated work surfaces here as PICA_ERR_CUDA.
 * No counterpart in the reference. */
int     pica_field_energy_noalloc(const void* const* fields, int32_t fp64, const int32_t* n, const double* h,
                                  void* stream, double* out);

/* Device state, for host loops that keep the particle state in host memory
 * between steps: raw copies of the current particle buffer (the device
 * layout, slot arrays of pica_state_slots() entries per species and
 * component) with cudaMemcpyAsync on the context stream.  comp: FP64 form
 * 0..6 = x y z ux uy uz w (double); FP32 form 0 = packed cell (uint32),
 * 1..7 = ox oy oz ux uy uz w (float). */
int64_t pica_state_slots(pica_ctx* ctx, int32_t species);
int     pica_state_copy(pica_ctx* ctx, int32_t species, int32_t comp, void* host, int32_t to_device);
/* The raw slots of supercells [sc_begin, sc_end) (one contiguous run of the layout,
 * slack included: [start[sc_begin], start[sc_end]) of pica_state_slots() entries,
 * at the same offset in host) with one cudaMemcpyAsync on copy_stream (a
 * cudaStream_t; NULL: the context stream), ordered against the context stream by
 * an event: an upload before the context stream's next work, a download after the
 * context stream's work so far.  No kernel: for host loops whose copies must not
 * wait for SMs.  The layout is valid until the next step (a resort or capacity
 * rebuild changes it; pica_state_slots() gives the host buffer size after each step). */
int     pica_state_copy_range_on(pica_ctx* ctx, int32_t species, int32_t comp, void* host, int32_t to_device,
                                 int32_t sc_begin, int32_t sc_end, void* copy_stream);
/* Packed particle state: the used slots of every supercell (dead ones
 * included), back to back in supercell order -- the slot state without the
 * layout's slack.  pica_state_packed_slots() reads the current counts
 * (synchronising the context stream), lays the image out and returns its size in
 * slots; pica_state_copy_packed() then moves one component of the image between
 * the device and host memory on the context stream (a gather or scatter kernel
 * and one copy; the device keeps a staging copy of the image).  The image is
 * valid until the next step or change of layout: pica_state_copy_packed returns
 * PICA_ERR_STATE once it is out of date.  Components as for pica_state_copy. */
int64_t pica_state_packed_slots(pica_ctx* ctx, int32_t species);
int     pica_state_copy_packed(pica_ctx* ctx, int32_t species, int32_t comp, void* host, int32_t to_device);
/* The part of the image that belongs to supercells [sc_begin, sc_end) (linear
 * supercell index, z fastest); host is still the start of the whole image. */
int     pica_state_copy_packed_range(pica_ctx* ctx, int32_t species, int32_t comp, void* host, int32_t to_device,
                                     int32_t sc_begin, int32_t sc_end);
/* pica_state_copy_packed_range with the host copy enqueued on copy_stream (a
 * cudaStream_t; NULL: the context stream) and the gather / scatter kernel on the
 * context stream, ordered by an event: an upload's scatter waits for its copy,
 * a download's copy for its gather.  A host loop that keeps its copies on streams
 * of their own runs them back to back instead of behind each range's kernels.
 * The caller orders later work against the copy stream (a download is complete
 * once the copy stream has passed it). */
int     pica_state_copy_packed_range_on(pica_ctx* ctx, int32_t species, int32_t comp, void* host,
                                        int32_t to_device, int32_t sc_begin, int32_t sc_end, void* copy_stream);

/* Batching form: many independent plasmas advanced together (FP32 cell form,
 * Esirkepov deposition, one shape and one supercell size for all members; grids,
 * particle counts and species may differ).  The push of every member is one
 * persistent launch over all members' supercells; the device part of the step
 * (flag reset, push, current conversion, B(dt/2) E(dt) B(dt/2), leaver sort,
 * arrival count, fill) is captured once as a CUDA graph and replayed while its
 * launch arguments stay the same (a resort or a capacity rebuild changes them
 * and the graph is captured again).  After every step the host reads all
 * members' flags and finishes their migrations (error, rebuild, resort).
 * Results equal those of the members stepped one by one with pica_step.
 * No counterpart in the reference (pica has no batched driver). */
typedef struct pica_batch pica_batch;
int       pica_batch_create(const pica_config* cfgs, int32_t count, pica_batch** out);
int       pica_batch_destroy(pica_batch* batch);
/* Member k: an ordinary context owned by the batch (upload, download, diagnostics;
 * do not destroy it or change its stream).  Calling this marks the work order for
 * recomputation from the members' particle counts at the next step. */
pica_ctx* pica_batch_member(pica_batch* batch, int32_t k);
/* use_graph: replay a captured CUDA graph (1) or enqueue every launch (0);
 * variant: launch shape of the batched push, as pica_set_variant. */
int       pica_batch_set_options(pica_batch* batch, int32_t use_graph, int32_t variant);
int       pica_batch_step(pica_batch* batch, int32_t nsteps);
/* out[0] graph captures, out[1] graph launches, out[2] kernel launches, out[3] steps. */
int       pica_batch_stats(pica_batch* batch, int64_t* out4);
const char* pica_batch_last_error(pica_batch* batch);

/* Checkpoint of the context between steps: configuration, fields, every
 * species' slot layout and particle buffer, step counter and fixed-point scale.
 * A context created with the same configuration and loaded from it continues like
 * the original (the building block of a host loop's restart): bit for bit in the
 * FP32 form; in the FP64 form to the rounding of its FP64 atomic current sums,
 * whose order differs from run to run.
 * Errors: PICA_ERR_INVALID for an unreadable file or a different configuration,
 * PICA_ERR_STATE between push_deposit and migrate.  pica has no checkpoints. */
int     pica_checkpoint_save(pica_ctx* ctx, const char* path);
/* Steps completed since upload (restored by pica_checkpoint_load; drives the resort cadence). */
int64_t pica_step_count(pica_ctx* ctx);
int     pica_checkpoint_load(pica_ctx* ctx, const char* path);

/* Synthetic plasma generated on the device, in place of pica_upload_particles
 * (FP32 cell form): the populations `specs[0..nspecs)` (grid and cell size equal
 * to the context's; at most 8 per species) replace the particle state.  The
 * particles are those pica_plasma_generate draws for the same specifications,
 * each in the cell it was drawn in, with the in-cell offset the FP32 rounding
 * of the uniform draw; they are stored in the order pica_upload_particles gives
 * that output (supercell, cell, population, particle).  No host memory holds the
 * ensemble.  pica has no generator; this replaces a host loop of
 * EnsembleSupercells::add (particles/EnsembleSupercells.h:41-45) over generated
 * particles.  PICA_ERR_INVALID for the FP64 form or a bad specification. */
int     pica_generate_plasma(pica_ctx* ctx, const pica_plasma_spec* specs, int32_t nspecs);

/* Host-side plasma set-up (no device work). */
int64_t pica_plasma_count(const pica_plasma_spec* spec);
int     pica_plasma_generate(const pica_plasma_spec* spec, int32_t threads, double* x, double* y, double* z,
                             double* ux, double* uy, double* uz, double* w, int32_t* species);

#ifdef __cplusplus
}
#endif
#endif
