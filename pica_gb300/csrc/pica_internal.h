// Internal declarations shared by the pica_gb300 translation units.
//
// Data layout in HBM (one context):
//   fields  : 9 arrays (ex ey ez bx by bz jx jy jz) of N^3 Real, z fastest,
//             index (i*ny + j)*nz + k -- pica's Array3d layout without guards
//             (periodicity is handled by index wrap in every kernel).
//   particles, per species: SoA buffers A (current) and B (side buffer) of
//             `slots` entries.  Supercell s owns slots [start[s], start[s] +
//             cap[s]); slots [0, count[s]) of it are used, some of them dead.
//             FP64 plain form : x y z ux uy uz w            (double, 56 B; dead: x = -1e300)
//             FP32 cell form  : cell(uint32 packed) ox oy oz ux uy uz w (4 B each, 32 B;
//                               dead: cell = 0xFFFFFFFF)
//   A step: the push kernel updates A in place; a particle that leaves its
//   supercell is the supercell's k-th leaver (k from a shared-memory counter):
//   its record goes to B at start + k, so a supercell's leaver records are
//   packed; its slot in A becomes dead and joins the leaver list, and the slot's
//   direction word holds the move's direction code and k.  Migration fills
//   each destination's fresh holes with its arrivals (canonical order), then
//   appends.  Every resort_every steps each supercell is compacted and
//   sorted by cell into B, and A and B swap.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda.h>   // CUtensorMap (types only; the encoder is reached through the runtime's driver entry point)
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

// Counter-based draws of the synthetic plasma generator, shared by the host
// generator and the device generator: draw `draw` of particle p of cell `cell`
// is the splitmix64 finaliser (S. Vigna) of the seed's hash xor a key made
// from (cell, p, draw), so any particle can be drawn alone, in any order.
__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// Uniform in [0, 1) with 53 random bits.
__host__ __device__ inline double uniDraw(uint64_t seed, int64_t cell, int64_t p, int draw) {
    const uint64_t key = ((uint64_t)cell << 24) ^ ((uint64_t)p << 4) ^ (uint64_t)draw;
    return (double)(mix64(mix64(seed) ^ key) >> 11) * 0x1.0p-53;
}
// Standard normal by Box-Muller from draws `draw` and `draw + 1`.
__host__ __device__ inline double normalDraw(uint64_t seed, int64_t cell, int64_t p, int draw) {
    const double u1 = 1.0 - uniDraw(seed, cell, p, draw), u2 = uniDraw(seed, cell, p, draw + 1);
    return sqrt(-2.0 * log(u1)) * cos(2.0 * 3.14159265358979323846 * u2);
}

struct PlainPtrs {  // FP64 plain form particle SoA
    double *x, *y, *z, *ux, *uy, *uz, *w;
};
struct CellPtrs {   // FP32 cell form particle SoA
    uint32_t* cell;
    float *ox, *oy, *oz, *ux, *uy, *uz, *w;
};

// Dead-slot markers.
constexpr double kDeadX = -1.0e300;          // FP64 form: x of a dead slot
constexpr uint32_t kDeadCell = 0xFFFFFFFFu;  // FP32 form: cell of a dead slot
__host__ __device__ inline bool aliveX(double x) { return x > -1.0e299; }

template <class P>
struct SpeciesArgs {
    P buf;             // A: updated in place
    P out;             // B: leaver records, packed at start + k
    const int64_t* start;
    const int32_t* cap;
    const int32_t* count;
    int32_t* nleave;   // leavers per supercell (this step)
    int32_t* llist;    // leaver slots, list of supercell s at [start[s], start[s] + nleave[s])
    uint32_t* dir;     // per slot, valid for leavers: direction code | (packed record index << 5)
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
    int tileSplit;      // FP32 form: low bits L of the split shared-memory tile sums
    void* j[3];         // FP64 form: jx jy jz (double), summed with FP64 atomics
    double norm;        // FP64 form: 1 / (hx hy hz)
    int* flags;         // flags[0]: error code (0 = ok)
    int scBegin, scEnd; // FP32 Esirkepov push: supercells [scBegin, scEnd) (scEnd 0: all)
    const struct TmaFieldMaps* tmaps;   // FP32 form, host: tensor maps of ex..bz (nullptr: none)
    SpeciesArgs<P> sp[kMaxSpecies];
};
// Tensor maps of the six E/B arrays for the TMA-staged push (launch variant 4): a
// 3D tiled map per component over (nz, ny, nx) floats, box (kTmaBoxZ, S+3, S+3).
// The box starts 4 nodes below the supercell in z, so that its innermost
// coordinate is a multiple of 4 floats (16 bytes), and covers nodes m-4 .. m+7.
constexpr int kTmaS = 4;          // supercell edge of the TMA variant
constexpr int kTmaBoxZ = 12;      // z extent of the box (48 bytes)
constexpr int kTmaZOff = 3;       // tile node m-1 sits at box index 3
constexpr int kTmaCompFloats = 608;   // (S+3)^2 x 12 = 588 floats, padded to a multiple of 128 bytes
struct TmaFieldMaps {   // aligned as CUtensorMap itself requires
    CUtensorMap m[6];
};

// Arguments of the FP32 Esirkepov push: only the fields it reads, FP64 factors
// rounded to FP32.  The single-plasma kernel takes one; the batching form takes
// those of up to batchMembers<NSP>() plasmas of at most NSP species in its kernel
// parameters, work item w (one supercell) belonging to plasma k with
// base[k] <= w < base[k + 1].
struct SpeciesArgsSlim {
    CellPtrs buf;
    CellPtrs out;
    const int64_t* start;
    const int32_t* count;
    int32_t* nleave;
    int32_t* llist;
    uint32_t* dir;
    float ec;
    float kq[3];
};
template <int NSP>
struct PushArgsSlim {
    int n[3], S[3], nsc[3], T[3];
    int nspecies;
    int tileSplit;
    int scOffset;       // first supercell of the launch (block b works on supercell scOffset + b)
    float cdth[3];
    float invUnit;
    const void* eb[6];
    unsigned long long* jacc[3];
    int* flags;
    SpeciesArgsSlim sp[NSP];
};
// The FP32 push arguments of one plasma, FP64 factors rounded to FP32 on the
// host (the FP32 kernels read only these; a conversion from FP64 in the kernel
// would run on the narrow FP64 pipe).
template <int NSP>
inline void slimArgs(const PushArgs<CellPtrs>& a, PushArgsSlim<NSP>& o) {
    std::memset(&o, 0, sizeof o);
    for (int d = 0; d < 3; d++) {
        o.n[d] = a.n[d]; o.S[d] = a.S[d]; o.nsc[d] = a.nsc[d]; o.T[d] = a.T[d];
        o.cdth[d] = (float)a.cdth[d]; o.jacc[d] = a.jacc[d];
    }
    o.nspecies = a.nspecies;
    o.tileSplit = a.tileSplit;
    o.scOffset = a.scBegin;
    o.invUnit = (float)a.invUnit;
    for (int k = 0; k < 6; k++) o.eb[k] = a.eb[k];
    o.flags = a.flags;
    for (int q = 0; q < a.nspecies && q < NSP; q++) {
        const auto& x = a.sp[q];
        auto& y = o.sp[q];
        y.buf = x.buf; y.out = x.out; y.start = x.start; y.count = x.count;
        y.nleave = x.nleave; y.llist = x.llist; y.dir = x.dir; y.ec = (float)x.ec;
        for (int d = 0; d < 3; d++) y.kq[d] = (float)x.kq[d];
    }
}

constexpr int kBatchParamBytes = 31 * 1024;
template <int NSP>
constexpr int batchMembers() { return (int)((kBatchParamBytes - 64) / (sizeof(PushArgsSlim<NSP>) + sizeof(int))); }
template <int NSP>
struct BatchPushArgs {
    int count;
    int total;
    int* counter;      // next work item; zero before the launch
    int base[batchMembers<NSP>() + 1];
    PushArgsSlim<NSP> members[batchMembers<NSP>()];
};
static_assert(sizeof(BatchPushArgs<1>) <= 32000 && sizeof(BatchPushArgs<2>) <= 32000,
              "batched push arguments exceed the kernel parameter space");
constexpr int kBatchSpecies = 2;

constexpr int kDirBuckets = 28;  // 27 direction codes + end

template <class P>
struct MigrateSpecies {
    P a;                    // A (current)
    P b;                    // B (leaver records, packed at start + k)
    P dst;                  // rebuild / resort destination (new layout)
    P outbox;               // rebuild: leaver copies gathered per source supercell
    const int64_t* start;
    const int32_t* cap;
    int32_t* count;         // used slots (incl. dead)
    int32_t* alive;         // live particles
    const int32_t* nleave;
    int32_t* llist;         // leaver slots by slot (the holes, in fill order)
    int32_t* lbydir;        // leaver record indices k, by (direction code, slot)
    int32_t* dirOff;        // per supercell: kDirBuckets offsets into lbydir (code c: [dirOff[c], dirOff[c+1]))
    const uint32_t* dir;
    int32_t* needed;        // count after migration
    int32_t* neededAlive;   // live particles after migration
    const int64_t* newStart;// rebuild / resort: new layout
    const int64_t* outOff;  // rebuild: first outbox entry of each source supercell
};

template <class P>
struct MigrateArgs {
    int nsc[3], S[3];
    int nspecies;
    double invh[3];         // FP64 resort: local cell from x
    int bitmapWords;        // leaver sort: 32-bit words covering the largest count
    int srcMaxCap;          // resort: largest capacity of the source layout (any species)
    int* flags;             // flags[0] error code, flags[1] overflow
    MigrateSpecies<P> sp[kMaxSpecies];
};

// Push launchers (push_fp64.cu / push_fp32.cu).  Return cudaError_t as int.
int launchPushPlain(const PushArgs<PlainPtrs>& a, int shape, int deposit, cudaStream_t s);
// Flat particle arrays (flat.cu): stable lexicographic position order of n particles
// (dims coordinates, key[d] device arrays) into order (device), and one push of a
// flat FP64 array (xu: x y z ux uy uz, device) on a grid seen with `guard` layers.
int orderByPosition(int64_t n, int dims, const double* const* key, int64_t* order, cudaStream_t s);
int launchPushFlat(const pica_config& c, void* const* f, int guard, int64_t n, double* const* xu, const double* w,
                   const int32_t* species, int* flags, cudaStream_t s);

// variant: launch shape of the FP32 Esirkepov kernel (0..kPushVariants-1), see push_fp32.cu.
constexpr int kPushVariants = 5;
int launchPushCell(const PushArgs<CellPtrs>& a, int shape, int deposit, int variant, cudaStream_t s);
// Persistent push over a batch (FP32 cell form, Esirkepov; S = supercell edges shared
// by every plasma).  grid <= 0: one CTA per resident slot on every SM.
template <int NSP>
int launchPushBatch(const BatchPushArgs<NSP>& b, int shape, const int* S, int variant, cudaStream_t s);
// Migration stages.
enum MigrateStage { kSortLeavers = 0, kCountArrivals = 1, kFill = 2, kGatherOutbox = 3, kRebuild = 4, kResort = 5 };
int launchMigratePlain(const MigrateArgs<PlainPtrs>& a, int stage, cudaStream_t s);
int launchMigrateCell(const MigrateArgs<CellPtrs>& a, int stage, cudaStream_t s);

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
    const void* key[kMaxSpecies];   // x (FP64) or packed cell (FP32): dead-slot test
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
// Device generator of a synthetic plasma (pica_generate_plasma): the populations
// of one species, written in the FP32 cell form's layout (one CTA per supercell).
constexpr int kGenMaxSpecs = 8;
struct GenSpec {
    double sigma, drift, weight;
    uint64_t seed;
    int nbeams, axis;
};
struct GenArgs {
    int n[3], S[3], nsc[3];
    int nspecs;                 // populations of this species, in the caller's order
    GenSpec sp[kGenMaxSpecs];
    const int32_t* per;         // particles per cell of x-plane i of population k at [k * n[0] + i]
    const int64_t* start;       // first slot of each supercell
    CellPtrs buf;
};
int launchGenerate(const GenArgs& a, int nscTot, cudaStream_t s);
// Packed state image: supercell s's used slots [start[s], start[s] + count[s]) of a
// component (words 4-byte words per slot) to or from image offset off[s] (slots).
// gather: slots -> image (src = slot array, dst = image); else image -> slots
// (src = image, dst = slot array).
int launchPackCopy(const void* src, void* dst, const int64_t* start, const int32_t* count, const int64_t* off,
                   int scBegin, int scEnd, int words, bool gather, cudaStream_t s);
// Domain decomposition (domain_kernels.cu): dst += src over n elements (double if fp64
// else float); the position component of packed arrivals into supercells [scBegin,
// scEnd) (slots from start[s], count[s] of them from image offset off[s]), the FP32
// form's cell x shifted by dxCells (wrapped into [0, nx)), the FP64 form's x by dxLength.
int launchAddSlab(bool fp64, void* dst, const void* src, int64_t n, cudaStream_t s);
int launchAppendPositions(bool fp64, const void* src, void* dst, const int64_t* start, const int32_t* count,
                          const int64_t* off, int scBegin, int scEnd, int dxCells, int nx, double dxLength,
                          cudaStream_t s);
// Gauss residual: max |div E - 4 pi (rho + bg)| and max |rho|; partial: 2*kReduceBlocks doubles.
int launchGauss(bool fp64, void* const* f, const double* rho, const int* n, const double* h, double bg,
                double* partial, double* out2, cudaStream_t s);

}  // namespace pgb
