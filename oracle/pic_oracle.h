/*
 * pic_oracle.h -- C API of the CPU restatement of pica's particle-in-cell step.
 *
 * TEST INFRASTRUCTURE ONLY.  The product (pica_gb300) never links, loads or
 * calls anything under oracle/.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py use it, and only as the checker / the timed CPU
 * baseline.
 *
 * Two implementations share this API:
 *   orc_*  : oracle/pic_oracle.cpp, a restatement written for this project
 *            (CIC and TSC form factors, direct and Esirkepov deposition,
 *            FP64 absolute-position form and FP32 cell+offset form).
 *   ref_*  : oracle/ref_harness.cpp, a driver around pica's own headers
 *            (FP64, CIC, direct deposition only); it pins the restatement.
 *
 * Ensemble order (both implement it identically):
 *   - load: particles are routed to supercells and, within a supercell, put
 *     in cell order (stable: local cell (lx*Sy + ly)*Sz + lz, then input order);
 *   - step: a particle that leaves its supercell leaves a dead slot behind;
 *     each destination receives its arrivals in canonical order (direction
 *     code 0..26 of the move, then source slot) into the slots its own
 *     leavers vacated in this step (ascending), then appended at the end;
 *   - every resort_every steps: each supercell drops its dead slots and is
 *     re-sorted by cell (stable).
 * Downloads list the live particles in slot order.
 */
#ifndef PICA_ORACLE_H
#define PICA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_FORM_FP64_PLAIN = 0, ORC_FORM_FP32_CELL = 1 };
enum { ORC_SHAPE_CIC = 1, ORC_SHAPE_TSC = 2 };
enum { ORC_DEPOSIT_DIRECT = 0, ORC_DEPOSIT_ESIRKEPOV = 1 };

typedef struct orc_config {
    int32_t n[3];        /* cells per dimension                          */
    int32_t sc[3];       /* cells per supercell per dimension            */
    double h[3];         /* cell size, cm                                */
    double dt;           /* time step, s                                 */
    int32_t form;        /* ORC_FORM_*                                   */
    int32_t shape;       /* ORC_SHAPE_*                                  */
    int32_t deposit;     /* ORC_DEPOSIT_*                                */
    int32_t nspecies;    /* <= 4                                         */
    double mass[4];      /* g                                            */
    double charge[4];    /* statC                                        */
    int32_t threads;     /* OpenMP threads, 0 = runtime default          */
    int32_t resort_every;/* compact + sort each supercell by cell every k steps (0 = never) */
} orc_config;

/* Diagnostics, all FP64 sums (see orc_diagnostics). */
typedef struct orc_diag {
    double field_energy;     /* sum (E^2+B^2) h^3 / 8pi over the N^3 nodes   */
    double kinetic_energy;   /* sum w m c^2 (gamma-1)                        */
    double total_charge;     /* sum q w                                      */
    double gauss_max;        /* max |div E - 4 pi (rho + rho_bg)|            */
    double rho_max;          /* max |rho| of the particles (statC/cm^3)      */
    double pad_[3];
} orc_diag;

void*   orc_create(const orc_config* cfg);
void    orc_destroy(void* sim);
/* Load particles (any order); they are routed to supercells stably. */
int     orc_load(void* sim, int64_t n, const double* x, const double* y, const double* z,
                 const double* ux, const double* uy, const double* uz,
                 const double* w, const int32_t* species);
/* Fields are N^3 arrays, z fastest: index (i*ny + j)*nz + k.  order: ex ey ez bx by bz jx jy jz */
int     orc_set_fields(void* sim, const double* const* f9);
int     orc_get_fields(void* sim, double* const* f9);
int     orc_step(void* sim, int32_t nsteps);
int64_t orc_num_particles(void* sim);
/* Particles in ensemble order: species-major, then supercell (linear), then slot. */
int     orc_get_particles(void* sim, double* x, double* y, double* z, double* ux, double* uy,
                          double* uz, double* w, int32_t* species, int32_t* supercell);
/* FP32 cell form raw state in ensemble order; cell is the linear cell (i*ny+j)*nz+k. */
int     orc_get_particles_cell(void* sim, int32_t* cell, float* ox, float* oy, float* oz,
                               float* ux, float* uy, float* uz, float* w);
/* counts[species * nsupercells + s] */
int     orc_get_counts(void* sim, int32_t* counts);
/* Migrations of the last step, ordered by (species, source supercell, source slot). */
int64_t orc_num_migrations(void* sim);
int     orc_get_migrations(void* sim, int32_t* species, int32_t* src, int32_t* slot, int32_t* dst);
/* rho at cell centres (N^3), shape of the configured form factor, FP64. */
int     orc_charge_density(void* sim, double* rho);
/* bg_density: neutralising background charge density (statC/cm^3) added to rho. */
int     orc_diagnostics(void* sim, double bg_density, orc_diag* out);

/* Flat particle arrays (pica's EnsembleOrdered / EnsembleUnordered).
 * orc_order_by_position: order[i] = index of the i-th particle in lexicographic
 *   position order over the first `dims` coordinates, ties in input order.
 * orc_push_flat: one push of a flat FP64 array in array order with the grid-level
 *   CIC (or TSC) gather and direct deposit on a periodic grid viewed with `guard`
 *   layers below the domain; the current v (q w) / (hx hy hz) is added to j3;
 *   positions and momenta are updated in place and wrapped periodically.
 *   ref_push_flat does the same through pica's own classes (guard 2, CIC only), and
 *   ref_order_by_position through EnsembleOrdered::reorder (std::sort: ties unordered). */
int     orc_order_by_position(int64_t n, int32_t dims, const double* x, const double* y, const double* z,
                              int64_t* order);
int     orc_push_flat(const orc_config* cfg, int32_t guard, int64_t n, double* x, double* y, double* z,
                      double* ux, double* uy, double* uz, const double* w, const int32_t* species,
                      const double* const* f6, double* const* j3);
int     ref_order_by_position(int64_t n, int32_t dims, const double* x, const double* y, const double* z,
                              int64_t* order);
int     ref_push_flat(const orc_config* cfg, int32_t guard, int64_t n, double* x, double* y, double* z,
                      double* ux, double* uy, double* uz, const double* w, const int32_t* species,
                      const double* const* f6, double* const* j3);
/* Synthetic plasma: the particles the product's host generator draws for the
 * same description (same counter-based draws, same order), so that the timed
 * CPU baseline needs no product code.  Layout equal to pica_plasma_spec. */
typedef struct orc_plasma {
    int32_t n[3];          /* cells                                              */
    int32_t species;       /* species index written for every particle           */
    double h[3];           /* cell size, cm                                      */
    double ppc;            /* mean particles per cell                            */
    double density_mod;    /* per-cell count round(ppc (1 + a cos(2 pi (i+1/2)/nx)))  */
    double drift_u;        /* beam drift u along drift_axis                      */
    double sigma_u;        /* Maxwellian spread of each u component              */
    double weight;         /* macro-particle factor                              */
    uint64_t seed;
    int32_t nbeams;        /* 1 or 2 (beams at +drift_u and -drift_u)            */
    int32_t drift_axis;    /* 0, 1, 2                                            */
} orc_plasma;
int64_t orc_plasma_count(const orc_plasma* spec);
/* Order: x-plane, y, z, then particle in the cell.  threads 0 = OpenMP default. */
int     orc_plasma_generate(const orc_plasma* spec, int32_t threads, double* x, double* y, double* z,
                            double* ux, double* uy, double* uz, double* w, int32_t* species);

/* The same API over pica's own headers (oracle/ref_harness.cpp). */
void*   ref_create(const orc_config* cfg);
void    ref_destroy(void* sim);
int     ref_load(void* sim, int64_t n, const double* x, const double* y, const double* z,
                 const double* ux, const double* uy, const double* uz,
                 const double* w, const int32_t* species);
int     ref_set_fields(void* sim, const double* const* f9);
int     ref_get_fields(void* sim, double* const* f9);
int     ref_step(void* sim, int32_t nsteps);
int64_t ref_num_particles(void* sim);
int     ref_get_particles(void* sim, double* x, double* y, double* z, double* ux, double* uy,
                          double* uz, double* w, int32_t* species, int32_t* supercell);
int     ref_get_counts(void* sim, int32_t* counts);
int64_t ref_num_migrations(void* sim);
int     ref_get_migrations(void* sim, int32_t* species, int32_t* src, int32_t* slot, int32_t* dst);

#ifdef __cplusplus
}
#endif
#endif
