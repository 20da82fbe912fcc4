// Internal declarations shared by the pica_gb300 translation units.
//
// Data layout in HBM (one context):
//   fields  : 9 arrays (ex ey ez bx by bz jx jy jz) of N^3 Real, z fastest,
//             index (i*ny + j)*nz + k -- pica's Array3d layout without guards
//             (periodicity is handled by index wrap in every kernel).
//   particles, per species: two SoA buffers A/B of `slots` entries.  Supercell
//             s owns slots [start[s], start[s] + cap[s]); its count[s] live
//             particles are packed at the front, in ensemble order.
//             FP64 plain form : x y z ux uy uz w            (double, 56 B)
//             FP32 cell form  : cell(uint32 packed) ox oy oz ux uy uz w (4 B each, 32 B)
//             The push kernel reads buffer `cur` and writes the other one:
//             stayers packed at the front of the supercell's range, leavers
//             packed backwards from its end with a direction byte each; the
//             migrate kernel then appends arrivals after the stayers in place.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pica_gb300.h"

namespace pgb {

constexpr int kMaxSpecies = 4;
constexpr int kG = 2;      // tile guard: a supercell tile starts at node m - 2
constexpr int kMaxS = 8;   // largest supported supercell edge (tile edge S + 5)
constexpr int kPushThreads = 256;
// FP32 form: current is accumulated in 64-bit two's-complement fixed point: one unit =
// kmax * 2^-F, where kmax (a power of two) bounds |q w| max(c, h/dt) over the
// particles, so every contribution is at most 2^F units.  F (at most 48) is
// chosen from the layout so that the largest number of contributions one node
// can receive in a step (all particles of the supercells whose tiles cover
// it) times 2^F stays below 2^62.  Integer sums are exact and independent of
// the order of the atomic adds, so the deposit is deterministic.
constexpr int kJFracBitsMax = 48;

// Packed FP32-form cell index: x (11 bits) | y (11 bits) | z (10 bits).
__host__ __device__ inline uint32_t packCell(int x, int y, int z) {
    return ((uint32_t)x << 21) | ((uint32_t)y << 10) | (uint32_t)z;
}
__host__ __device__ inline void unpackCell(uint32_t c, int& x, int& y, int& z) {
    x = (int)(c >> 21); y = (int)((c >> 10) & 0x7FFu); z = (int)(c & 0x3FFu);
}

struct PlainPtrs {  // FP64 plain form particle SoA
    double *x, *y, *z, *ux, *uy, *uz, *w;
};
struct CellPtrs {   // FP32 cell form particle SoA
    uint32_t* cell;
    float *ox, *oy, *oz, *ux, *uy, *uz, *w;
};

template <class P>
struct SpeciesArgs {
    P in, out;
    const int64_t* start;
    const int32_t* cap;
    const int32_t* count;
    int32_t* nstay;
    int32_t* nleave;
    uint8_t* dir;      // direction byte per slot of the output buffer
    double ec;         // q dt / (2 m c)   (BorisPusher.h:29)
    double q;          // charge
    double kq[3];      // -q h_d / dt      (Esirkepov current factor per unit weight)
    double qc;         // q c              (FP32 direct current per unit weight and u/gamma)
};

template <class P>
struct PushArgs {
    int n[3], S[3], nsc[3], T[3];
    int nspecies;
    double h[3], invh[3], L[3], scInv[3], dt;
    double cdth[3];     // c dt / h (FP32 form position update in cell units)
    const void* eb[6];  // ex ey ez bx by bz (Real)
    unsigned long long* jacc[3];  // FP32 form: J accumulators, fixed point (unit kmax * 2^-F)
    double invUnit;     // FP32 form: 2^F / kmax, current contribution -> fixed-point units
    void* j[3];         // FP64 form: jx jy jz (double), summed with FP64 atomics
    double norm;        // FP64 form: 1 / (hx hy hz)
    int* flags;         // flags[0]: error code (0 = ok)
    SpeciesArgs<P> sp[kMaxSpecies];
};

template <class P>
struct MigrateSpecies {
    P buf;                  // the buffer written by the push kernel
    P dst;                  // rebuild destination (new layout)
    const int64_t* start;
    const int32_t* cap;
    const int32_t* nstay;
    const int32_t* nleave;
    const uint8_t* dir;
    int32_t* count;         // in-place migrate: new counts
    int32_t* needed;        // stayers + arrivals (always written)
    const int64_t* newStart;// rebuild: new layout starts
};

template <class P>
struct MigrateArgs {
    int nsc[3];
    int nspecies;
    int* flags;             // flags[0] error code, flags[1] overflow
    MigrateSpecies<P> sp[kMaxSpecies];
};

// Push launchers (push_fp64.cu / push_fp32.cu).  Return cudaError_t as int.
int launchPushPlain(const PushArgs<PlainPtrs>& a, int shape, int deposit, cudaStream_t s);
int launchPushCell(const PushArgs<CellPtrs>& a, int shape, int deposit, cudaStream_t s);
int launchMigratePlain(const MigrateArgs<PlainPtrs>& a, bool rebuild, cudaStream_t s);
int launchMigrateCell(const MigrateArgs<CellPtrs>& a, bool rebuild, cudaStream_t s);

// Grid launchers (grid_kernels.cu).  `fp64` selects double vs float arrays.
// J = Jacc * scale (Real), then Jacc = 0.
int launchConvertJ(bool fp64, void* const* j, unsigned long long* const* jacc, int64_t nodes, double scale,
                   cudaStream_t s);
int launchUpdateB(bool fp64, void* const* f, const int* n, const double* coeff, cudaStream_t s);
int launchUpdateE(bool fp64, void* const* f, const int* n, double cc, const double* coeff, cudaStream_t s);
// Field energy: sum over nodes of sum_c f_c^2 (FP64) into *out (device); partial: scratch of
// at least kReduceBlocks doubles.
constexpr int kReduceBlocks = 1216;  // 8 x 152 SMs
int launchFieldEnergy(bool fp64, void* const* f, int64_t nodes, double* partial, double* out, cudaStream_t s);
// Particle sums per supercell block: kinetic (w m c^2 (gamma-1)) and charge; partial: 2*nscTot doubles.
struct ParticleSumArgs {
    bool fp64;
    int nspecies, nscTot;
    const void* ux[kMaxSpecies];
    const void* uy[kMaxSpecies];
    const void* uz[kMaxSpecies];
    const void* w[kMaxSpecies];
    const int64_t* start[kMaxSpecies];
    const int32_t* count[kMaxSpecies];
    double mc2[kMaxSpecies], q[kMaxSpecies];
};
int launchParticleSums(const ParticleSumArgs& a, double* partial, double* out2, cudaStream_t s);
// Charge density (FP64 atomics) at cell centres.
struct RhoArgs {
    bool fp64;
    int shape, nspecies, nscTot;
    int n[3], S[3], nsc[3];
    double invh[3], norm;
    const void* p0[kMaxSpecies];  // plain: x ; cell: packed cell
    const void* p1[kMaxSpecies];  // plain: y ; cell: ox
    const void* p2[kMaxSpecies];  // plain: z ; cell: oy
    const void* p3[kMaxSpecies];  // cell: oz
    const void* w[kMaxSpecies];
    const int64_t* start[kMaxSpecies];
    const int32_t* count[kMaxSpecies];
    double q[kMaxSpecies];
};
int launchRho(const RhoArgs& a, double* rho, cudaStream_t s);
// Gauss residual: max |div E - 4 pi (rho + bg)| and max |rho|; partial: 2*kReduceBlocks doubles.
int launchGauss(bool fp64, void* const* f, const double* rho, const int* n, const double* h, double bg,
                double* partial, double* out2, cudaStream_t s);

}  // namespace pgb
