// C ABI of pica_gb300 (include/pica_gb300.h): context, particle/field transfer,
// step orchestration and host-side plasma generation.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "pica_internal.h"

using namespace pgb;

namespace {

constexpr double kC = 29979245800.0;     // pica math/Constants.h:11
constexpr double kPiRef = 3.14159265358; // pica math/Constants.h:10

inline int wrapHost(int a, int n) { a %= n; return a < 0 ? a + n : a; }

struct SpeciesState {
    void* buf[2][8] = {};        // A = buf[cur], B = buf[1 - cur]
    int64_t slots[2] = {0, 0};   // allocated slots of each buffer
    uint32_t* dir = nullptr;     // per slot: direction code | (packed leaver record index << 5)
    int32_t* llist = nullptr;    // leaver slots per supercell (at [start, start + nleave)), by slot
    int32_t* lbydir = nullptr;   // the same slots by (direction code, slot)
    int32_t* d_dirOff = nullptr; // per supercell, 28 bucket offsets of lbydir
    int64_t slotArrays = 0;      // allocated entries of dir / llist
    void* outbox[8] = {};        // overflow rebuild: leavers gathered per source supercell
    int64_t outSlots = 0;
    int64_t* d_start = nullptr;
    int32_t* d_cap = nullptr;
    int32_t* d_count = nullptr;  // used slots, dead ones included
    int32_t* d_alive = nullptr;  // live particles
    int32_t* d_nleave = nullptr;
    int32_t* d_needed = nullptr;
    int32_t* d_neededAlive = nullptr;
    int64_t* d_start2 = nullptr;
    int32_t* d_cap2 = nullptr;
    int64_t* d_outOff = nullptr;
    std::vector<int64_t> h_start;
    std::vector<int32_t> h_cap;
    int64_t layoutSlots = 0;     // sum of caps of the current layout
    // Pinned staging of the resort's host round trip (live counts in, new layout out).
    // Packed state image (pica_state_packed_slots / pica_state_copy_packed): supercell
    // offsets of the image, its size, the epoch it was laid out for, and one device
    // staging buffer per component.
    int64_t* d_packOff = nullptr;
    std::vector<int64_t> h_packOff;   // host copy, nscTot + 1 entries
    int64_t packSlots = -1;
    int64_t packEpoch = -1;
    int64_t packCap = 0;
    void* d_pack[8] = {};
    int32_t* h_pinAlive = nullptr;
    int64_t* h_pinStart = nullptr;
    int32_t* h_pinCap = nullptr;
};

}  // namespace

struct pica_ctx {
    pica_config cfg;
    bool fp64 = true;
    int ncomp = 7;
    size_t compBytes[8] = {};
    int nsc[3] = {}, nscTot = 0, T[3] = {};
    cudaStream_t stream = nullptr;
    void* f[9] = {};
    SpeciesState sp[kMaxSpecies];
    int cur = 0;
    bool pending = false;
    int* d_flags = nullptr;
    int* h_flags = nullptr;
    double* d_red = nullptr;
    int64_t redCount = 0;
    double* d_out = nullptr;
    double* h_out = nullptr;
    double* d_rho = nullptr;
    unsigned long long* jacc[3] = {};
    double kmax = 1.0;      // power of two bounding |q w| max(c, h/dt) (sets the J fixed-point unit)
    int jfrac = 40;         // fraction bits of the J fixed point (see pica_internal.h)
    int tileSplit = 16;     // low bits of the split shared-memory tile sums (FP32 form)
    int variant = 0;        // launch variant of the FP32 Esirkepov push kernel
    std::string err;
    int64_t launches = 0;
    int64_t steps = 0;
    int64_t epoch = 0;      // bumped by every step and every change of layout (packed-image validity)
    int threads = 1;
    cudaEvent_t copyOrder = nullptr;   // orders a host copy on a caller's copy stream against the context stream
    bool recordMig = false;            // keep each step's migration list (pica_record_migrations)
    std::vector<int32_t> mig;          // last step's list: (species, src, slot, dst) per entry
    TmaFieldMaps tmaps{};              // tensor maps of ex..bz for push variant 4 (FP32 form, supercells 4^3)
    bool hasTmaps = false;
};

namespace {

int fail(pica_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                               \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? PICA_ERR_OOM : PICA_ERR_CUDA,   \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                   \
    } while (0)

#define CKL(expr)                                                                              \
    do {                                                                                       \
        int e_ = (expr);                                                                       \
        if (e_ != 0)                                                                           \
            return fail(ctx, PICA_ERR_CUDA, std::string(#expr) + ": " +                        \
                        cudaGetErrorString((cudaError_t)e_));                                  \
    } while (0)

int scLinear(const pica_ctx* c, int x, int y, int z) { return (x * c->nsc[1] + y) * c->nsc[2] + z; }

int32_t capacityFor(const pica_ctx* c, int32_t count) {
    const double sl = c->cfg.slack > 0 ? c->cfg.slack : 0.15;
    int64_t extra = std::max<int64_t>(32, (int64_t)std::ceil(count * sl));
    int64_t cap = (count + extra + 31) / 32 * 32;
    return (int32_t)cap;
}

void layoutFrom(const pica_ctx* c, const std::vector<int32_t>& counts, std::vector<int64_t>& start,
                std::vector<int32_t>& cap, int64_t& total) {
    start.resize(c->nscTot);
    cap.resize(c->nscTot);
    total = 0;
    for (int s = 0; s < c->nscTot; s++) {
        start[s] = total;
        cap[s] = capacityFor(c, counts[s]);
        total += cap[s];
    }
}

// Largest particle count of one supercell and species: its capacity (count plus
// slack) stays an int32.
constexpr int64_t kMaxSupercellCount = 1ll << 30;

// Particles per cell of x-plane i of a synthetic population (host generator and
// device generator alike): round(ppc (1 + a cos(2 pi (i + 1/2) / nx))).
int cellCount(const pica_plasma_spec* s, int i) {
    const double f = 1.0 + s->density_mod * std::cos(2.0 * 3.14159265358979323846 * (i + 0.5) / s->n[0]);
    return (int)std::lround(s->ppc * f);
}

// Fixed-point unit of the J accumulators: kmax = 2^ceil(log2 max |q w| max(c, h/dt)).
void setCurrentUnit(pica_ctx* ctx, double maxQW) {
    const pica_config& c = ctx->cfg;
    const double hmax = std::max(std::max(c.h[0], c.h[1]), c.h[2]);
    const double bound = maxQW * std::max(kC, hmax / c.dt);
    ctx->kmax = bound > 0 ? std::ldexp(1.0, (int)std::ceil(std::log2(bound))) : 1.0;
}

// Fraction bits of the J fixed point for the current layout: a node can receive one
// contribution per particle of every supercell whose tile covers it.
void updateJFrac(pica_ctx* ctx) {
    int64_t maxCaps = 0;
    for (int q = 0; q < ctx->cfg.nspecies; q++) {
        int32_t m = 0;
        for (int32_t v : ctx->sp[q].h_cap) m = std::max(m, v);
        maxCaps += m;
    }
    int64_t cover = 1;
    for (int d = 0; d < 3; d++) cover *= (ctx->cfg.sc[d] + 2 * kG + 1 + ctx->cfg.sc[d] - 1) / ctx->cfg.sc[d];
    const double worst = (double)cover * (double)std::max<int64_t>(maxCaps, 1) + 1.0;
    // Shared-memory tile: a node receives at most one addition per particle of its
    // supercell (all species), each below 2^F in magnitude.  With maxCaps < 2^b the
    // unsigned low part (L bits per addition) stays below 2^32 for L <= 32 - b, and
    // the signed high part, |sum floor(v / 2^L)| <= 2^(F+b-L) + 2^b, below 2^31 for
    // F <= 29 + L - b.  L <= 23 keeps the split exact in FP32 (FixTile::add).
    const int b = (int)std::ceil(std::log2((double)std::max<int64_t>(maxCaps, 1) + 1.0));
    ctx->tileSplit = std::min(31 - b, 23);
    ctx->jfrac = std::min(std::min(kJFracBitsMax, 62 - (int)std::ceil(std::log2(worst))), 29 + ctx->tileSplit - b);
}

// Slot arrays grow with 1/16 headroom, so that layouts that grow by a few slots
// at a resort or rebuild do not reallocate (and synchronise the device) each time.
int64_t withHeadroom(int64_t slots) { return std::max<int64_t>(slots, 1) + slots / 16 + 1024; }

int ensureBuffer(pica_ctx* ctx, int spi, int b, int64_t slots) {
    SpeciesState& S = ctx->sp[spi];
    if (S.slots[b] >= slots) return PICA_OK;
    for (int k = 0; k < ctx->ncomp; k++) {
        if (S.buf[b][k]) CK(cudaFree(S.buf[b][k]));
        S.buf[b][k] = nullptr;
    }
    S.slots[b] = 0;
    const int64_t grown = withHeadroom(slots);
    for (int k = 0; k < ctx->ncomp; k++) CK(cudaMalloc(&S.buf[b][k], grown * ctx->compBytes[k]));
    S.slots[b] = grown;
    return PICA_OK;
}

int ensureSlotArrays(pica_ctx* ctx, int spi, int64_t slots) {
    SpeciesState& S = ctx->sp[spi];
    if (S.slotArrays >= slots) return PICA_OK;
    if (S.dir) CK(cudaFree(S.dir));
    if (S.llist) CK(cudaFree(S.llist));
    if (S.lbydir) CK(cudaFree(S.lbydir));
    S.dir = nullptr;
    S.llist = nullptr;
    S.lbydir = nullptr;
    S.slotArrays = 0;
    const int64_t grown = withHeadroom(slots);
    CK(cudaMalloc(&S.dir, grown * 4));
    CK(cudaMalloc(&S.llist, grown * 4));
    CK(cudaMalloc(&S.lbydir, grown * 4));
    S.slotArrays = grown;
    return PICA_OK;
}

int ensureOutbox(pica_ctx* ctx, int spi, int64_t slots) {
    SpeciesState& S = ctx->sp[spi];
    if (S.outSlots >= slots) return PICA_OK;
    for (int k = 0; k < ctx->ncomp; k++) {
        if (S.outbox[k]) CK(cudaFree(S.outbox[k]));
        S.outbox[k] = nullptr;
    }
    S.outSlots = 0;
    const int64_t grown = withHeadroom(slots);
    for (int k = 0; k < ctx->ncomp; k++) CK(cudaMalloc(&S.outbox[k], grown * ctx->compBytes[k]));
    S.outSlots = grown;
    return PICA_OK;
}

// Fresh layout of species q for the given per-supercell counts (slots
// [start, start + count) used, none dead), in host and device copies.
int installLayout(pica_ctx* ctx, int q, const std::vector<int32_t>& counts) {
    SpeciesState& S = ctx->sp[q];
    int64_t total;
    layoutFrom(ctx, counts, S.h_start, S.h_cap, total);
    S.layoutSlots = total;
    int rc;
    if ((rc = ensureBuffer(ctx, q, 0, total)) || (rc = ensureBuffer(ctx, q, 1, total)) ||
        (rc = ensureSlotArrays(ctx, q, total)))
        return rc;
    // Ordered on the context's stream (which may be a non-blocking stream), and
    // complete before return.
    CK(cudaMemcpyAsync(S.d_start, S.h_start.data(), ctx->nscTot * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(S.d_cap, S.h_cap.data(), ctx->nscTot * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(S.d_count, counts.data(), ctx->nscTot * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(S.d_alive, counts.data(), ctx->nscTot * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(S.d_nleave, 0, ctx->nscTot * 4, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->epoch++;
    return PICA_OK;
}

template <class P>
P ptrsOf(void* const* p);
template <>
PlainPtrs ptrsOf<PlainPtrs>(void* const* p) {
    return PlainPtrs{(double*)p[0], (double*)p[1], (double*)p[2], (double*)p[3], (double*)p[4], (double*)p[5], (double*)p[6]};
}
template <>
CellPtrs ptrsOf<CellPtrs>(void* const* p) {
    return CellPtrs{(uint32_t*)p[0], (float*)p[1], (float*)p[2], (float*)p[3], (float*)p[4], (float*)p[5], (float*)p[6], (float*)p[7]};
}

PlainPtrs plainPtrs(pica_ctx* c, int spi, int b) {
    void* const* p = c->sp[spi].buf[b];
    return PlainPtrs{(double*)p[0], (double*)p[1], (double*)p[2], (double*)p[3], (double*)p[4], (double*)p[5], (double*)p[6]};
}
CellPtrs cellPtrs(pica_ctx* c, int spi, int b) {
    void* const* p = c->sp[spi].buf[b];
    return CellPtrs{(uint32_t*)p[0], (float*)p[1], (float*)p[2], (float*)p[3], (float*)p[4], (float*)p[5], (float*)p[6], (float*)p[7]};
}

// Run fn over [0, n) split into contiguous chunks on `threads` host threads.
void parallelFor(int threads, int64_t n, const std::function<void(int64_t, int64_t)>& fn) {
    if (threads <= 1 || n < 65536) { fn(0, n); return; }
    std::vector<std::thread> th;
    int64_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; t++) {
        int64_t a = t * chunk, b = std::min(n, a + chunk);
        if (a >= b) break;
        th.emplace_back(fn, a, b);
    }
    for (auto& t : th) t.join();
}
}  // namespace

// Tensor maps of the six FP32 E/B arrays for push variant 4: a 3D tiled map over
// (nz, ny, nx) floats per component, box (kTmaBoxZ, 7, 7), no swizzle, zero fill
// outside the grid (the kernel copies only boxes whose used nodes lie inside).
// The encoder is the driver's cuTensorMapEncodeTiled, reached through the runtime.
// False, and no maps, for other supercell shapes, grids narrower than 12 cells, or
// a driver without the encoder: variant 4 then launches as variant 0.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static bool encodeFieldMaps(pica_ctx* ctx) {
    const pica_config& c = ctx->cfg;
    for (int d = 0; d < 3; d++)
        if (c.sc[d] != kTmaS || c.n[d] < 12) return false;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return false;
    }
    const cuuint64_t dims[3] = {(cuuint64_t)c.n[2], (cuuint64_t)c.n[1], (cuuint64_t)c.n[0]};
    const cuuint64_t strides[2] = {(cuuint64_t)c.n[2] * 4, (cuuint64_t)c.n[1] * c.n[2] * 4};
    const cuuint32_t box[3] = {kTmaBoxZ, kTmaS + 3, kTmaS + 3}, unit[3] = {1, 1, 1};
    for (int k = 0; k < 6; k++)
        if (reinterpret_cast<EncodeTiledFn>(fn)(&ctx->tmaps.m[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, ctx->f[k], dims,
                                                 strides, box, unit, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                                 CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    return true;
}

// Kernel arguments of the push for the context's current layout (the buffers
// themselves are set by the caller).
template <class A>
static void fillPushArgs(pica_ctx* ctx, A& a) {
    const pica_config& c = ctx->cfg;
    for (int d = 0; d < 3; d++) {
        a.n[d] = c.n[d]; a.S[d] = c.sc[d]; a.nsc[d] = ctx->nsc[d]; a.T[d] = ctx->T[d];
        a.h[d] = c.h[d]; a.invh[d] = 1.0 / c.h[d]; a.L[d] = (double)c.n[d] * c.h[d];
        a.scInv[d] = 1.0 / ((double)c.sc[d] * ((a.L[d] - 0.0) / (double)c.n[d]));
        a.cdth[d] = kC * c.dt / c.h[d];
    }
    a.dt = c.dt;
    a.nspecies = c.nspecies;
    for (int k = 0; k < 6; k++) a.eb[k] = ctx->f[k];
    for (int k = 0; k < 3; k++) { a.jacc[k] = ctx->jacc[k]; a.j[k] = ctx->f[6 + k]; }
    a.invUnit = std::ldexp(1.0, ctx->jfrac) / ctx->kmax;
    a.tileSplit = ctx->tileSplit;
    a.norm = 1.0 / (c.h[0] * c.h[1] * c.h[2]);   // CurrentDepositorYeeGrid.h:203
    a.flags = ctx->d_flags;
    if constexpr (std::is_same<A, PushArgs<CellPtrs>>::value) a.tmaps = ctx->hasTmaps ? &ctx->tmaps : nullptr;
    for (int q = 0; q < c.nspecies; q++) {
        SpeciesState& S = ctx->sp[q];
        auto& sa = a.sp[q];
        sa.start = S.d_start; sa.cap = S.d_cap; sa.count = S.d_count;
        sa.nleave = S.d_nleave; sa.llist = S.llist; sa.dir = S.dir;
        sa.ec = c.charge[q] * c.dt / (2.0 * c.mass[q] * kC);   // BorisPusher.h:29
        sa.q = c.charge[q];
        for (int d = 0; d < 3; d++) sa.kq[d] = -c.charge[q] * (c.h[d] / c.dt);
        sa.qc = c.charge[q] * kC;
    }
}

extern "C" {

int pica_abi_version(void) { return PICA_ABI_VERSION; }

const char* pica_status_string(int s) {
    switch (s) {
        case PICA_OK: return "ok";
        case PICA_ERR_INVALID: return "invalid argument or configuration";
        case PICA_ERR_CUDA: return "CUDA runtime error";
        case PICA_ERR_OOM: return "out of memory";
        case PICA_ERR_OVERFLOW: return "supercell capacity overflow";
        case PICA_ERR_MIGRATION: return "particle crossed more than one supercell in one step";
        case PICA_ERR_STATE: return "call out of order";
        case PICA_ERR_NOT_BUILT: return "combination not built";
        case PICA_ERR_LIMIT: return "size beyond a fixed limit";
        case PICA_ERR_TIMEOUT: return "a bounded device wait gave up";
        default: return "unknown status";
    }
}

const char* pica_last_error(pica_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }
int64_t pica_launch_count(pica_ctx* ctx) { return ctx ? ctx->launches : -1; }

int pica_ctx_create(const pica_config* cfg, pica_ctx** out) {
    pica_ctx* ctx = nullptr;
    if (!cfg || !out) return PICA_ERR_INVALID;
    *out = nullptr;
    if (cfg->form != PICA_FORM_FP64_PLAIN && cfg->form != PICA_FORM_FP32_CELL) return PICA_ERR_INVALID;
    if (cfg->shape != PICA_SHAPE_CIC && cfg->shape != PICA_SHAPE_TSC) return PICA_ERR_INVALID;
    if (cfg->deposit != PICA_DEPOSIT_DIRECT && cfg->deposit != PICA_DEPOSIT_ESIRKEPOV) return PICA_ERR_INVALID;
    if (cfg->nspecies < 1 || cfg->nspecies > kMaxSpecies) return PICA_ERR_INVALID;
    if (!(cfg->dt > 0)) return PICA_ERR_INVALID;
    for (int d = 0; d < 3; d++) {
        if (cfg->n[d] <= 0 || cfg->sc[d] <= 0 || cfg->sc[d] > kMaxS || cfg->n[d] % cfg->sc[d] != 0) return PICA_ERR_INVALID;
        if (!(cfg->h[d] > 0)) return PICA_ERR_INVALID;
    }
    if (cfg->form == PICA_FORM_FP32_CELL && (cfg->n[0] > 2048 || cfg->n[1] > 2048 || cfg->n[2] > 1024)) return PICA_ERR_LIMIT;
    // No CUDA device (or no driver): a CUDA error, not an allocation failure.  There is no CPU path.
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return PICA_ERR_CUDA;
    }
    ctx = new pica_ctx();
    ctx->cfg = *cfg;
    ctx->fp64 = cfg->form == PICA_FORM_FP64_PLAIN;
    ctx->ncomp = ctx->fp64 ? 7 : 8;
    for (int k = 0; k < 8; k++) ctx->compBytes[k] = ctx->fp64 ? 8 : 4;
    ctx->nscTot = 1;
    for (int d = 0; d < 3; d++) {
        ctx->nsc[d] = cfg->n[d] / cfg->sc[d];
        ctx->nscTot *= ctx->nsc[d];
        ctx->T[d] = cfg->sc[d] + 2 * kG + 1;
    }
    ctx->threads = cfg->threads > 0 ? cfg->threads : std::max(1u, std::thread::hardware_concurrency());
    const int64_t nodes = (int64_t)cfg->n[0] * cfg->n[1] * cfg->n[2];
    const size_t rb = ctx->fp64 ? 8 : 4;
    int rc = PICA_OK;
    auto bail = [&](int code) { pica_ctx_destroy(ctx); return code; };
    for (int c = 0; c < 9; c++) {
        if (cudaMalloc(&ctx->f[c], nodes * rb) != cudaSuccess) return bail(PICA_ERR_OOM);
        if (cudaMemset(ctx->f[c], 0, nodes * rb) != cudaSuccess) return bail(PICA_ERR_CUDA);
    }
    for (int c = 0; c < 3; c++) {
        if (cudaMalloc(&ctx->jacc[c], nodes * 8) != cudaSuccess) return bail(PICA_ERR_OOM);
        if (cudaMemset(ctx->jacc[c], 0, nodes * 8) != cudaSuccess) return bail(PICA_ERR_CUDA);
    }
    for (int s = 0; s < cfg->nspecies; s++) {
        SpeciesState& S = ctx->sp[s];
        const size_t n = ctx->nscTot;
        if (cudaMalloc(&S.d_start, n * 8) || cudaMalloc(&S.d_cap, n * 4) || cudaMalloc(&S.d_count, n * 4) ||
            cudaMalloc(&S.d_alive, n * 4) || cudaMalloc(&S.d_nleave, n * 4) || cudaMalloc(&S.d_needed, n * 4) ||
            cudaMalloc(&S.d_neededAlive, n * 4) || cudaMalloc(&S.d_start2, n * 8) || cudaMalloc(&S.d_cap2, n * 4) ||
            cudaMalloc(&S.d_outOff, n * 8) || cudaMalloc(&S.d_dirOff, n * kDirBuckets * 4) ||
            cudaMallocHost(&S.h_pinAlive, n * 4) || cudaMallocHost(&S.h_pinStart, n * 8) || cudaMallocHost(&S.h_pinCap, n * 4))
            return bail(PICA_ERR_OOM);
        std::vector<int32_t> zero(n, 0);
        int64_t total;
        layoutFrom(ctx, zero, S.h_start, S.h_cap, total);
        S.layoutSlots = total;
        if ((rc = ensureBuffer(ctx, s, 0, total)) || (rc = ensureBuffer(ctx, s, 1, total)) ||
            (rc = ensureSlotArrays(ctx, s, total)))
            return bail(rc);
        if (cudaMemcpy(S.d_start, S.h_start.data(), n * 8, cudaMemcpyHostToDevice) ||
            cudaMemcpy(S.d_cap, S.h_cap.data(), n * 4, cudaMemcpyHostToDevice) || cudaMemset(S.d_count, 0, n * 4) ||
            cudaMemset(S.d_alive, 0, n * 4) || cudaMemset(S.d_nleave, 0, n * 4))
            return bail(PICA_ERR_CUDA);
    }
    ctx->redCount = std::max<int64_t>(2 * kReduceBlocks, 2 * (int64_t)ctx->nscTot) + 8;
    if (cudaMalloc(&ctx->d_flags, 4 * sizeof(int)) || cudaMallocHost(&ctx->h_flags, 4 * sizeof(int)) ||
        cudaMalloc(&ctx->d_red, ctx->redCount * 8) || cudaMalloc(&ctx->d_out, 8 * 8) || cudaMallocHost(&ctx->h_out, 8 * 8))
        return bail(PICA_ERR_OOM);
    cudaMemset(ctx->d_flags, 0, 4 * sizeof(int));
    if (!ctx->fp64) ctx->hasTmaps = encodeFieldMaps(ctx);
    if (cudaDeviceSynchronize() != cudaSuccess) return bail(PICA_ERR_CUDA);
    *out = ctx;
    return PICA_OK;
}

int pica_ctx_destroy(pica_ctx* ctx) {
    if (!ctx) return PICA_ERR_INVALID;
    cudaDeviceSynchronize();
    for (auto p : ctx->f) if (p) cudaFree(p);
    for (auto p : ctx->jacc) if (p) cudaFree(p);
    for (auto& S : ctx->sp) {
        for (auto& b : S.buf) for (auto p : b) if (p) cudaFree(p);
        for (auto p : S.outbox) if (p) cudaFree(p);
        for (void* p : {(void*)S.dir, (void*)S.llist, (void*)S.d_start, (void*)S.d_cap, (void*)S.d_count,
                        (void*)S.d_alive, (void*)S.d_nleave, (void*)S.d_needed, (void*)S.d_neededAlive,
                        (void*)S.d_start2, (void*)S.d_cap2, (void*)S.d_outOff, (void*)S.lbydir, (void*)S.d_dirOff})
            if (p) cudaFree(p);
        for (void* p : {(void*)S.h_pinAlive, (void*)S.h_pinStart, (void*)S.h_pinCap})
            if (p) cudaFreeHost(p);
        if (S.d_packOff) cudaFree(S.d_packOff);
        for (auto p : S.d_pack) if (p) cudaFree(p);
    }
    if (ctx->d_flags) cudaFree(ctx->d_flags);
    if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
    if (ctx->d_red) cudaFree(ctx->d_red);
    if (ctx->d_out) cudaFree(ctx->d_out);
    if (ctx->h_out) cudaFreeHost(ctx->h_out);
    if (ctx->d_rho) cudaFree(ctx->d_rho);
    if (ctx->copyOrder) cudaEventDestroy(ctx->copyOrder);
    delete ctx;
    return PICA_OK;
}

int pica_set_variant(pica_ctx* ctx, int32_t variant) {
    if (!ctx || variant < 0 || variant >= kPushVariants) return fail(ctx, PICA_ERR_INVALID, "no such push variant");
    ctx->variant = variant;
    return PICA_OK;
}

int pica_get_variant(pica_ctx* ctx, int32_t* variant, int32_t* count) {
    if (!ctx) return PICA_ERR_INVALID;
    if (variant) *variant = ctx->variant;
    if (count) *count = kPushVariants;
    return PICA_OK;
}

int pica_set_stream(pica_ctx* ctx, void* stream) {
    if (!ctx) return PICA_ERR_INVALID;
    ctx->stream = (cudaStream_t)stream;
    return PICA_OK;
}

int pica_synchronize(pica_ctx* ctx) {
    if (!ctx) return PICA_ERR_INVALID;
    CK(cudaStreamSynchronize(ctx->stream));
    return PICA_OK;
}

int pica_upload_particles(pica_ctx* ctx, int64_t n, const double* x, const double* y, const double* z,
                          const double* ux, const double* uy, const double* uz, const double* w,
                          const int32_t* species) {
    if (!ctx || n < 0 || (n > 0 && (!x || !y || !z || !ux || !uy || !uz || !w))) return fail(ctx, PICA_ERR_INVALID, "null array");
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "upload while a migration is pending");
    CK(cudaStreamSynchronize(ctx->stream));
    const pica_config& c = ctx->cfg;
    const int nsp = c.nspecies;
    double scInv[3], invh[3];
    for (int d = 0; d < 3; d++) {
        const double L = (double)c.n[d] * c.h[d];
        scInv[d] = 1.0 / ((double)c.sc[d] * ((L - 0.0) / (double)c.n[d]));  // EnsembleSupercells.h:31-33
        invh[d] = 1.0 / c.h[d];
    }
    // Route: key = species * nscTot + supercell and the local cell inside the supercell
    // (particles are stored by supercell, then cell, stably); FP32 form also converts
    // to cell + offset.
    const int S3 = c.sc[0] * c.sc[1] * c.sc[2];
    std::vector<int32_t> key(n), lcell(n);
    std::vector<uint32_t> cell(ctx->fp64 ? 0 : n);
    std::vector<float> off(ctx->fp64 ? 0 : 3 * n);
    int bad = 0;
    parallelFor(ctx->threads, n, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; i++) {
            const int q = species ? species[i] : 0;
            if (q < 0 || q >= nsp) { bad = 1; key[i] = 0; continue; }
            const double p[3] = {x[i], y[i], z[i]};
            const double uu[4] = {ux[i], uy[i], uz[i], w[i]};
            bool ok = true;
            for (int d = 0; d < 3; d++) ok = ok && std::isfinite(p[d]) && p[d] >= 0.0 && p[d] < (double)c.n[d] * c.h[d];
            for (double v : uu) ok = ok && std::isfinite(v);
            if (!ok) { bad = 2; key[i] = 0; continue; }
            int s3[3];
            int l3[3];
            if (ctx->fp64) {
                for (int d = 0; d < 3; d++) {
                    s3[d] = (int)std::floor((p[d] - 0.0) * scInv[d]);
                    s3[d] = std::min(std::max(s3[d], 0), ctx->nsc[d] - 1);
                    l3[d] = std::min(std::max((int)std::floor(p[d] * invh[d]) - s3[d] * c.sc[d], 0), c.sc[d] - 1);
                }
            } else {
                int cc[3];
                for (int d = 0; d < 3; d++) {
                    const double xi = p[d] * invh[d];
                    const double fl = std::floor(xi);
                    cc[d] = (int)fl;
                    float o = (float)(xi - fl);
                    if (o >= 1.0f) { o = 0.0f; cc[d] += 1; }
                    cc[d] = wrapHost(cc[d], c.n[d]);
                    off[3 * i + d] = o;
                    s3[d] = cc[d] / c.sc[d];
                    l3[d] = cc[d] - s3[d] * c.sc[d];
                }
                cell[i] = packCell(cc[0], cc[1], cc[2]);
            }
            key[i] = q * ctx->nscTot + scLinear(ctx, s3[0], s3[1], s3[2]);
            lcell[i] = (l3[0] * c.sc[1] + l3[1]) * c.sc[2] + l3[2];
        }
    });
    if (bad == 1) return fail(ctx, PICA_ERR_INVALID, "species index out of range");
    if (bad == 2) return fail(ctx, PICA_ERR_INVALID, "non-finite value or position outside [0, n h)");
    {
        double maxQW = 0.0;
        for (int64_t i = 0; i < n; i++) maxQW = std::max(maxQW, std::fabs(c.charge[species ? species[i] : 0] * w[i]));
        setCurrentUnit(ctx, maxQW);
    }
    const int64_t nkeys = (int64_t)nsp * ctx->nscTot;
    std::vector<int64_t> cnt(nkeys + 1, 0);
    for (int64_t i = 0; i < n; i++) cnt[key[i] + 1]++;
    // Per species layout.
    for (int q = 0; q < nsp; q++) {
        std::vector<int32_t> counts(ctx->nscTot);
        for (int s = 0; s < ctx->nscTot; s++) {
            const int64_t v = cnt[(int64_t)q * ctx->nscTot + s + 1];
            if (v > kMaxSupercellCount) return fail(ctx, PICA_ERR_LIMIT, "too many particles in one supercell");
            counts[s] = (int32_t)v;
        }
        int rc;
        if ((rc = installLayout(ctx, q, counts))) return rc;
    }
    updateJFrac(ctx);
    ctx->steps = 0;
    // Slot of each particle: start of its supercell + its rank by (local cell, input order).
    std::vector<int64_t> base2((size_t)nkeys * S3 + 1, 0);
    for (int64_t i = 0; i < n; i++) base2[(size_t)key[i] * S3 + lcell[i] + 1]++;
    for (int64_t k = 0; k < nkeys; k++) {
        int64_t run = ctx->sp[k / ctx->nscTot].h_start[k % ctx->nscTot];
        for (int l = 0; l < S3; l++) {
            const int64_t c2 = base2[(size_t)k * S3 + l + 1];
            base2[(size_t)k * S3 + l] = run;
            run += c2;
        }
    }
    std::vector<int64_t> slot(n);
    for (int64_t i = 0; i < n; i++) slot[i] = base2[(size_t)key[i] * S3 + lcell[i]]++;
    std::vector<int32_t> spOf(n);
    for (int64_t i = 0; i < n; i++) spOf[i] = key[i] / ctx->nscTot;
    ctx->cur = 0;
    for (int q = 0; q < nsp; q++) {
        SpeciesState& S = ctx->sp[q];
        const int64_t total = S.layoutSlots;
        for (int k = 0; k < ctx->ncomp; k++) {
            std::vector<unsigned char> host(total * ctx->compBytes[k], 0);
            parallelFor(ctx->threads, n, [&](int64_t a, int64_t b) {
                for (int64_t i = a; i < b; i++) {
                    if (spOf[i] != q) continue;
                    const int64_t o = slot[i];
                    if (ctx->fp64) {
                        const double* src[7] = {x, y, z, ux, uy, uz, w};
                        ((double*)host.data())[o] = src[k][i];
                    } else if (k == 0) {
                        ((uint32_t*)host.data())[o] = cell[i];
                    } else if (k <= 3) {
                        ((float*)host.data())[o] = off[3 * i + (k - 1)];
                    } else {
                        const double* src[4] = {ux, uy, uz, w};
                        ((float*)host.data())[o] = (float)src[k - 4][i];
                    }
                }
            });
            // From pageable memory: staged before the call returns, ordered on the stream.
            CK(cudaMemcpyAsync(S.buf[0][k], host.data(), total * ctx->compBytes[k], cudaMemcpyHostToDevice,
                               ctx->stream));
        }
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return PICA_OK;
}

int pica_generate_plasma(pica_ctx* ctx, const pica_plasma_spec* specs, int32_t nspecs) {
    if (!ctx) return PICA_ERR_INVALID;
    if (!specs || nspecs < 1) return fail(ctx, PICA_ERR_INVALID, "no plasma specification");
    if (ctx->fp64) return fail(ctx, PICA_ERR_INVALID, "the device generator writes the FP32 cell form only");
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "generate while a migration is pending");
    const pica_config& c = ctx->cfg;
    const int nx = c.n[0];
    std::vector<int> perSpecies(c.nspecies, 0);
    double maxQW = 0.0;
    for (int k = 0; k < nspecs; k++) {
        const pica_plasma_spec& g = specs[k];
        if (pica_plasma_count(&g) < 0) return fail(ctx, PICA_ERR_INVALID, "invalid plasma specification");
        for (int d = 0; d < 3; d++)
            if (g.n[d] != c.n[d] || g.h[d] != c.h[d])
                return fail(ctx, PICA_ERR_INVALID, "plasma specification on another grid than the context's");
        if (g.species < 0 || g.species >= c.nspecies) return fail(ctx, PICA_ERR_INVALID, "species index out of range");
        if ((g.nbeams != 1 && g.nbeams != 2) || g.drift_axis < 0 || g.drift_axis > 2)
            return fail(ctx, PICA_ERR_INVALID, "beams must be 1 or 2 and the drift axis 0, 1 or 2");
        if (!std::isfinite(g.sigma_u) || !std::isfinite(g.drift_u) || !std::isfinite(g.weight) ||
            !std::isfinite(g.ppc) || !std::isfinite(g.density_mod))
            return fail(ctx, PICA_ERR_INVALID, "non-finite plasma parameter");
        if (++perSpecies[g.species] > kGenMaxSpecs)
            return fail(ctx, PICA_ERR_LIMIT, "more than 8 plasma specifications for one species");
        maxQW = std::max(maxQW, std::fabs(c.charge[g.species] * g.weight));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    // Particles per cell of every x-plane, from the host's count rule (the layout
    // below and the device kernel both read this table).
    std::vector<int32_t> per((size_t)nspecs * nx);
    for (int k = 0; k < nspecs; k++)
        for (int i = 0; i < nx; i++) {
            const int v = cellCount(&specs[k], i);
            if (v < 0) return fail(ctx, PICA_ERR_INVALID, "negative particle count");
            per[(size_t)k * nx + i] = v;
        }
    const int64_t cellsYZ = (int64_t)c.sc[1] * c.sc[2];
    for (int q = 0; q < c.nspecies; q++) {
        std::vector<int32_t> counts(ctx->nscTot);
        for (int s = 0; s < ctx->nscTot; s++) {
            const int sx = s / (ctx->nsc[1] * ctx->nsc[2]);
            int64_t v = 0;
            for (int k = 0; k < nspecs; k++)
                if (specs[k].species == q)
                    for (int lx = 0; lx < c.sc[0]; lx++) v += (int64_t)per[(size_t)k * nx + sx * c.sc[0] + lx] * cellsYZ;
            if (v > kMaxSupercellCount) return fail(ctx, PICA_ERR_LIMIT, "too many particles in one supercell");
            counts[s] = (int32_t)v;
        }
        int rc;
        if ((rc = installLayout(ctx, q, counts))) return rc;
    }
    setCurrentUnit(ctx, maxQW);
    updateJFrac(ctx);
    ctx->cur = 0;
    ctx->steps = 0;
    int32_t* d_per = nullptr;
    CK(cudaMalloc(&d_per, per.size() * 4));
    int err = 0;
    for (int q = 0; q < c.nspecies && !err; q++) {
        SpeciesState& S = ctx->sp[q];
        for (int k = 0; k < ctx->ncomp && !err; k++)   // unused slots read as zero, as after an upload
            err = cudaMemsetAsync(S.buf[0][k], 0, S.layoutSlots * ctx->compBytes[k], ctx->stream);
        if (err || perSpecies[q] == 0) continue;
        GenArgs a{};
        for (int d = 0; d < 3; d++) {
            a.n[d] = c.n[d];
            a.S[d] = c.sc[d];
            a.nsc[d] = ctx->nsc[d];
        }
        std::vector<int32_t> mine;
        for (int k = 0; k < nspecs; k++) {
            if (specs[k].species != q) continue;
            const pica_plasma_spec& g = specs[k];
            a.sp[a.nspecs] = GenSpec{g.sigma_u, g.drift_u, g.weight, g.seed, g.nbeams, g.drift_axis};
            mine.insert(mine.end(), per.begin() + (size_t)k * nx, per.begin() + (size_t)(k + 1) * nx);
            a.nspecs++;
        }
        // This species' rows of the table, in the order of its populations (a copy from
        // pageable memory: staged before the call returns).
        err = cudaMemcpyAsync(d_per, mine.data(), mine.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
        if (err) break;
        a.per = d_per;
        a.start = S.d_start;
        CellPtrs& b = a.buf;
        b.cell = (uint32_t*)S.buf[0][0];
        b.ox = (float*)S.buf[0][1]; b.oy = (float*)S.buf[0][2]; b.oz = (float*)S.buf[0][3];
        b.ux = (float*)S.buf[0][4]; b.uy = (float*)S.buf[0][5]; b.uz = (float*)S.buf[0][6];
        b.w = (float*)S.buf[0][7];
        err = launchGenerate(a, (int)ctx->nscTot, ctx->stream);
        ctx->launches++;
        if (!err) err = cudaStreamSynchronize(ctx->stream);   // d_per is rewritten for the next species
    }
    if (!err) err = cudaStreamSynchronize(ctx->stream);
    cudaFree(d_per);
    if (err) return fail(ctx, PICA_ERR_CUDA, std::string("device generation: ") + cudaGetErrorString((cudaError_t)err));
    return PICA_OK;
}

int64_t pica_num_particles(pica_ctx* ctx) {
    if (!ctx) return PICA_ERR_INVALID;
    int64_t total = 0;
    std::vector<int32_t> counts(ctx->nscTot);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return fail(ctx, PICA_ERR_CUDA, "synchronize failed");
    for (int q = 0; q < ctx->cfg.nspecies; q++) {
        if (cudaMemcpy(counts.data(), ctx->sp[q].d_alive, ctx->nscTot * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            return fail(ctx, PICA_ERR_CUDA, "count download failed");
        for (int32_t v : counts) total += v;
    }
    return total;
}

int pica_get_counts(pica_ctx* ctx, int32_t* counts) {
    if (!ctx || !counts) return PICA_ERR_INVALID;
    CK(cudaStreamSynchronize(ctx->stream));
    for (int q = 0; q < ctx->cfg.nspecies; q++)
        CK(cudaMemcpy(counts + (size_t)q * ctx->nscTot, ctx->sp[q].d_alive, ctx->nscTot * 4, cudaMemcpyDeviceToHost));
    return PICA_OK;
}

int pica_download_particles(pica_ctx* ctx, double* x, double* y, double* z, double* ux, double* uy, double* uz,
                            double* w, int32_t* species, int32_t* supercell) {
    if (!ctx) return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "download while a migration is pending");
    CK(cudaStreamSynchronize(ctx->stream));
    const pica_config& c = ctx->cfg;
    double* out[7] = {x, y, z, ux, uy, uz, w};
    int64_t o = 0;
    for (int q = 0; q < c.nspecies; q++) {
        SpeciesState& S = ctx->sp[q];
        std::vector<int32_t> counts(ctx->nscTot);
        CK(cudaMemcpy(counts.data(), S.d_count, ctx->nscTot * 4, cudaMemcpyDeviceToHost));
        const int64_t total = S.layoutSlots;
        std::vector<std::vector<unsigned char>> host(ctx->ncomp);
        for (int k = 0; k < ctx->ncomp; k++) {
            host[k].resize(total * ctx->compBytes[k]);
            CK(cudaMemcpy(host[k].data(), S.buf[ctx->cur][k], total * ctx->compBytes[k], cudaMemcpyDeviceToHost));
        }
        for (int s = 0; s < ctx->nscTot; s++) {
            const int64_t st = S.h_start[s];
            for (int i = 0; i < counts[s]; i++) {
                const int64_t slot = st + i;
                if (ctx->fp64 ? !aliveX(((double*)host[0].data())[slot])
                              : ((uint32_t*)host[0].data())[slot] == kDeadCell)
                    continue;
                if (ctx->fp64) {
                    for (int k = 0; k < 7; k++)
                        if (out[k]) out[k][o] = ((double*)host[k].data())[slot];
                } else {
                    int cx, cy, cz;
                    unpackCell(((uint32_t*)host[0].data())[slot], cx, cy, cz);
                    const float* f[7];
                    for (int k = 0; k < 7; k++) f[k] = (const float*)host[k + 1].data();
                    if (x) x[o] = ((double)cx + (double)f[0][slot]) * c.h[0];
                    if (y) y[o] = ((double)cy + (double)f[1][slot]) * c.h[1];
                    if (z) z[o] = ((double)cz + (double)f[2][slot]) * c.h[2];
                    for (int k = 3; k < 7; k++)
                        if (out[k]) out[k][o] = (double)f[k][slot];
                }
                if (species) species[o] = q;
                if (supercell) supercell[o] = s;
                o++;
            }
        }
    }
    return PICA_OK;
}

int pica_upload_fields(pica_ctx* ctx, const double* const* f9) {
    if (!ctx || !f9) return PICA_ERR_INVALID;
    const int64_t nodes = (int64_t)ctx->cfg.n[0] * ctx->cfg.n[1] * ctx->cfg.n[2];
    CK(cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < 9; c++) {
        if (!f9[c]) return fail(ctx, PICA_ERR_INVALID, "null field array");
        if (ctx->fp64) CK(cudaMemcpy(ctx->f[c], f9[c], nodes * 8, cudaMemcpyHostToDevice));
        else {
            std::vector<float> tmp(nodes);
            for (int64_t i = 0; i < nodes; i++) tmp[i] = (float)f9[c][i];
            CK(cudaMemcpy(ctx->f[c], tmp.data(), nodes * 4, cudaMemcpyHostToDevice));
        }
    }
    return PICA_OK;
}

int pica_download_fields(pica_ctx* ctx, double* const* f9) {
    if (!ctx || !f9) return PICA_ERR_INVALID;
    const int64_t nodes = (int64_t)ctx->cfg.n[0] * ctx->cfg.n[1] * ctx->cfg.n[2];
    CK(cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < 9; c++) {
        if (!f9[c]) continue;
        if (ctx->fp64) CK(cudaMemcpy(f9[c], ctx->f[c], nodes * 8, cudaMemcpyDeviceToHost));
        else {
            std::vector<float> tmp(nodes);
            CK(cudaMemcpy(tmp.data(), ctx->f[c], nodes * 4, cudaMemcpyDeviceToHost));
            for (int64_t i = 0; i < nodes; i++) f9[c][i] = tmp[i];
        }
    }
    return PICA_OK;
}

}  // extern "C"

// The push over all supercells, as nchunks launches over consecutive supercell
// ranges [bounds[r], bounds[r+1]) (FP32 Esirkepov kernel; the other kernels take
// one launch after all waits), the launch of range r enqueued after a wait for
// events[r] when given.  bounds == nullptr: one launch over all supercells.
static int pushImpl(pica_ctx* ctx, int nchunks, const int32_t* bounds, void* const* events) {
    if (!ctx) return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "push_deposit called twice without migrate");
    const pica_config& c = ctx->cfg;
    const int64_t nodes = (int64_t)c.n[0] * c.n[1] * c.n[2];
    CK(cudaMemsetAsync(ctx->d_flags, 0, 4 * sizeof(int), ctx->stream));
    if (ctx->fp64)
        for (int k = 6; k < 9; k++) CK(cudaMemsetAsync(ctx->f[k], 0, nodes * 8, ctx->stream));
    const bool ranges = !ctx->fp64 && c.deposit == PICA_DEPOSIT_ESIRKEPOV && nchunks > 1 && bounds;
    if (!ranges)
        for (int r = 0; r < nchunks; r++)
            if (events && events[r]) CK(cudaStreamWaitEvent(ctx->stream, static_cast<cudaEvent_t>(events[r]), 0));
    if (ctx->fp64) {
        PushArgs<PlainPtrs> a{};
        fillPushArgs(ctx, a);
        for (int q = 0; q < c.nspecies; q++) { a.sp[q].buf = plainPtrs(ctx, q, ctx->cur); a.sp[q].out = plainPtrs(ctx, q, 1 - ctx->cur); }
        CKL(launchPushPlain(a, c.shape, c.deposit, ctx->stream));
        ctx->launches++;
    } else {
        PushArgs<CellPtrs> a{};
        fillPushArgs(ctx, a);
        for (int q = 0; q < c.nspecies; q++) { a.sp[q].buf = cellPtrs(ctx, q, ctx->cur); a.sp[q].out = cellPtrs(ctx, q, 1 - ctx->cur); }
        if (!ranges) {
            CKL(launchPushCell(a, c.shape, c.deposit, ctx->variant, ctx->stream));
            ctx->launches++;
        } else {
            for (int r = 0; r < nchunks; r++) {
                if (events && events[r]) CK(cudaStreamWaitEvent(ctx->stream, static_cast<cudaEvent_t>(events[r]), 0));
                a.scBegin = bounds[r];
                a.scEnd = bounds[r + 1];
                if (a.scEnd <= a.scBegin) continue;
                CKL(launchPushCell(a, c.shape, c.deposit, ctx->variant, ctx->stream));
                ctx->launches++;
            }
        }
    }
    if (!ctx->fp64) {
        // J = sum / h^3 (CurrentDepositorYeeGrid.h:203), from the exact fixed-point sums.
        const double scale = (ctx->kmax * std::ldexp(1.0, -ctx->jfrac)) * (1.0 / (c.h[0] * c.h[1] * c.h[2]));
        CKL(launchConvertJ(false, ctx->f + 6, ctx->jacc, nodes, scale, ctx->stream));
        ctx->launches++;
    }
    ctx->pending = true;
    return PICA_OK;
}

extern "C" {

int pica_push_deposit(pica_ctx* ctx) { return pushImpl(ctx, 1, nullptr, nullptr); }

int pica_push_deposit_chunked(pica_ctx* ctx, int32_t nchunks, void* const* wait_events) {
    if (!ctx) return PICA_ERR_INVALID;
    if (nchunks < 1 || nchunks > 4096) return fail(ctx, PICA_ERR_INVALID, "chunk count out of range (1..4096)");
    std::vector<int32_t> bounds(nchunks + 1);
    for (int r = 0; r <= nchunks; r++) bounds[r] = (int32_t)((int64_t)ctx->nscTot * r / nchunks);
    return pushImpl(ctx, nchunks, bounds.data(), wait_events);
}

int pica_push_deposit_ranges(pica_ctx* ctx, int32_t nranges, const int32_t* bounds, void* const* wait_events) {
    if (!ctx) return PICA_ERR_INVALID;
    if (nranges < 1 || nranges > 4096 || !bounds)
        return fail(ctx, PICA_ERR_INVALID, "range count out of range (1..4096) or no bounds");
    if (bounds[0] != 0 || bounds[nranges] != ctx->nscTot)
        return fail(ctx, PICA_ERR_INVALID, "ranges must start at supercell 0 and end at the supercell count");
    for (int r = 0; r < nranges; r++)
        if (bounds[r + 1] < bounds[r]) return fail(ctx, PICA_ERR_INVALID, "range bounds must not decrease");
    return pushImpl(ctx, nranges, bounds, wait_events);
}

int pica_order_by_position(int64_t n, int32_t dims, const double* x, const double* y, const double* z, int64_t* order,
                           void* stream) {
    if (n < 0 || dims < 1 || dims > 3) return PICA_ERR_INVALID;
    if (n == 0) return PICA_OK;
    if (!x || (dims > 1 && !y) || (dims > 2 && !z) || !order) return PICA_ERR_INVALID;
    if (n > ((int64_t)1 << 40)) return PICA_ERR_LIMIT;
    const double* key[3] = {x, y, z};
    const int e = orderByPosition(n, dims, key, order, static_cast<cudaStream_t>(stream));
    if (e == (int)cudaErrorMemoryAllocation) { cudaGetLastError(); return PICA_ERR_OOM; }
    return e ? PICA_ERR_CUDA : PICA_OK;
}

int pica_order_by_position_host(int64_t n, int32_t dims, const double* x, const double* y, const double* z,
                                int64_t* order) {
    if (n < 0 || dims < 1 || dims > 3 || (n > 0 && (!x || (dims > 1 && !y) || (dims > 2 && !z) || !order)))
        return PICA_ERR_INVALID;
    if (n == 0) return PICA_OK;
    if (n > ((int64_t)1 << 40)) return PICA_ERR_LIMIT;
    const double* host[3] = {x, y, z};
    double* dev[3] = {nullptr, nullptr, nullptr};
    int64_t* dorder = nullptr;
    int rc = PICA_OK;
    for (int d = 0; d < dims && rc == PICA_OK; d++) {
        if (cudaMalloc(&dev[d], (size_t)n * 8) != cudaSuccess) rc = PICA_ERR_OOM;
        else if (cudaMemcpy(dev[d], host[d], (size_t)n * 8, cudaMemcpyHostToDevice) != cudaSuccess) rc = PICA_ERR_CUDA;
    }
    if (rc == PICA_OK && cudaMalloc(&dorder, (size_t)n * 8) != cudaSuccess) rc = PICA_ERR_OOM;
    if (rc == PICA_OK) rc = pica_order_by_position(n, dims, dev[0], dev[1], dev[2], dorder, nullptr);
    if (rc == PICA_OK && cudaMemcpy(order, dorder, (size_t)n * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = PICA_ERR_CUDA;
    for (double* p : dev) cudaFree(p);
    cudaFree(dorder);
    if (rc != PICA_OK) cudaGetLastError();
    return rc;
}

int pica_push_flat(pica_ctx* ctx, int64_t n, double* x, double* y, double* z, double* ux, double* uy, double* uz,
                   const double* w, const int32_t* species, int32_t guard) {
    if (!ctx || n < 0 || guard < 0 || guard > 1024) return fail(ctx, PICA_ERR_INVALID, "bad flat push arguments");
    if (n > 0 && (!x || !y || !z || !ux || !uy || !uz || !w))
        return fail(ctx, PICA_ERR_INVALID, "a flat particle array is missing");
    if (!ctx->fp64) return fail(ctx, PICA_ERR_NOT_BUILT, "flat particle arrays hold FP64 positions: the plain form only");
    if (ctx->cfg.deposit != PICA_DEPOSIT_DIRECT)
        return fail(ctx, PICA_ERR_NOT_BUILT, "flat particle arrays deposit directly (no charge-conserving form)");
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "the context's own push awaits its migration");
    const int64_t nodes = (int64_t)ctx->cfg.n[0] * ctx->cfg.n[1] * ctx->cfg.n[2];
    for (int k = 6; k < 9; k++) CK(cudaMemsetAsync(ctx->f[k], 0, nodes * 8, ctx->stream));
    CK(cudaMemsetAsync(ctx->d_flags, 0, 4 * sizeof(int), ctx->stream));
    double* xu[6] = {x, y, z, ux, uy, uz};
    CKL(launchPushFlat(ctx->cfg, ctx->f, guard, n, xu, w, species, ctx->d_flags, ctx->stream));
    ctx->launches += n > 0 ? 1 : 0;
    CK(cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->h_flags[0]) return fail(ctx, ctx->h_flags[0], "a particle's species is outside the configuration");
    return PICA_OK;
}

int pica_push_flat_host(pica_ctx* ctx, int64_t n, double* x, double* y, double* z, double* ux, double* uy, double* uz,
                        const double* w, const int32_t* species, int32_t guard) {
    if (!ctx || n < 0) return fail(ctx, PICA_ERR_INVALID, "bad flat push arguments");
    if (n > 0 && (!x || !y || !z || !ux || !uy || !uz || !w))
        return fail(ctx, PICA_ERR_INVALID, "a flat particle array is missing");
    double* host[7] = {x, y, z, ux, uy, uz, const_cast<double*>(w)};
    double* dev[7] = {};
    int32_t* dsp = nullptr;
    int rc = PICA_OK;
    const size_t bytes = (size_t)std::max<int64_t>(n, 1) * 8;
    for (int k = 0; k < 7 && rc == PICA_OK; k++) {
        if (cudaMalloc(&dev[k], bytes) != cudaSuccess) rc = fail(ctx, PICA_ERR_OOM, "flat push staging");
        else if (n > 0 && cudaMemcpy(dev[k], host[k], (size_t)n * 8, cudaMemcpyHostToDevice) != cudaSuccess)
            rc = fail(ctx, PICA_ERR_CUDA, "flat push upload");
    }
    if (rc == PICA_OK && species) {
        if (cudaMalloc(&dsp, bytes / 2) != cudaSuccess) rc = fail(ctx, PICA_ERR_OOM, "flat push staging");
        else if (n > 0 && cudaMemcpy(dsp, species, (size_t)n * 4, cudaMemcpyHostToDevice) != cudaSuccess)
            rc = fail(ctx, PICA_ERR_CUDA, "flat push upload");
    }
    if (rc == PICA_OK) rc = pica_push_flat(ctx, n, dev[0], dev[1], dev[2], dev[3], dev[4], dev[5], dev[6], dsp, guard);
    for (int k = 0; k < 6 && rc == PICA_OK && n > 0; k++)
        if (cudaMemcpy(host[k], dev[k], (size_t)n * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = fail(ctx, PICA_ERR_CUDA, "flat push download");
    for (double* p : dev) cudaFree(p);
    cudaFree(dsp);
    if (rc != PICA_OK) cudaGetLastError();
    return rc;
}

int pica_update_b(pica_ctx* ctx, double dt) {
    if (!ctx) return PICA_ERR_INVALID;
    const pica_config& c = ctx->cfg;
    double coeff[3];
    for (int d = 0; d < 3; d++) coeff[d] = (kC * dt) / c.h[d];   // YeeSolver.h:181-182
    CKL(launchUpdateB(ctx->fp64, ctx->f, c.n, coeff, ctx->stream));
    ctx->launches++;
    return PICA_OK;
}

int pica_update_e(pica_ctx* ctx, double dt) {
    if (!ctx) return PICA_ERR_INVALID;
    const pica_config& c = ctx->cfg;
    double coeff[3];
    for (int d = 0; d < 3; d++) coeff[d] = (kC * dt) / c.h[d];   // YeeSolver.h:137-138
    const double cc = -4.0 * kPiRef * dt;                         // YeeSolver.h:135
    CKL(launchUpdateE(ctx->fp64, ctx->f, c.n, cc, coeff, ctx->stream));
    ctx->launches++;
    return PICA_OK;
}

}  // extern "C"

// Upload a new layout (start/cap per supercell) into the *2 arrays; returns its slot total.
static int stageLayout(pica_ctx* ctx, int q, const std::vector<int32_t>& counts, int64_t& total) {
    SpeciesState& S = ctx->sp[q];
    std::vector<int64_t> nstart;
    std::vector<int32_t> ncap;
    layoutFrom(ctx, counts, nstart, ncap, total);
    // From pageable memory: staged before the calls return, ordered on the stream.
    CK(cudaMemcpyAsync(S.d_start2, nstart.data(), ctx->nscTot * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(S.d_cap2, ncap.data(), ctx->nscTot * 4, cudaMemcpyHostToDevice, ctx->stream));
    S.h_start.swap(nstart);
    S.h_cap.swap(ncap);
    S.layoutSlots = total;
    return PICA_OK;
}

template <class P>
static void migrateArgs(pica_ctx* ctx, MigrateArgs<P>& a) {
    const pica_config& c = ctx->cfg;
    const int A = ctx->cur, B = 1 - ctx->cur;
    for (int d = 0; d < 3; d++) { a.nsc[d] = ctx->nsc[d]; a.S[d] = c.sc[d]; a.invh[d] = 1.0 / c.h[d]; }
    a.nspecies = c.nspecies;
    a.flags = ctx->d_flags;
    int32_t maxCap = 0;
    for (int q = 0; q < c.nspecies; q++) {
        SpeciesState& S = ctx->sp[q];
        for (int32_t v : S.h_cap) maxCap = std::max(maxCap, v);
        auto& m = a.sp[q];
        m.a = ptrsOf<P>(S.buf[A]); m.b = ptrsOf<P>(S.buf[B]); m.dst = ptrsOf<P>(S.buf[B]);
        m.outbox = ptrsOf<P>(S.outbox);
        m.start = S.d_start; m.cap = S.d_cap; m.count = S.d_count; m.alive = S.d_alive;
        m.nleave = S.d_nleave; m.llist = S.llist; m.dir = S.dir;
        m.needed = S.d_needed; m.neededAlive = S.d_neededAlive;
        m.newStart = S.d_start2; m.outOff = S.d_outOff;
        m.lbydir = S.lbydir; m.dirOff = S.d_dirOff;
    }
    a.bitmapWords = (maxCap + 31) / 32;
}

template <class P>
static int launchMigrate(pica_ctx* ctx, MigrateArgs<P>& m, int stage) {
    if constexpr (std::is_same<P, PlainPtrs>::value) return launchMigratePlain(m, stage, ctx->stream);
    else return launchMigrateCell(m, stage, ctx->stream);
}

// Device part of the migration, enqueued without waiting: sort the leaver lists,
// count arrivals (flags[1] set on a capacity overflow), fill the holes (the fill
// returns at once when flags[0] or flags[1] is set).
template <class P>
static int migrateDevice(pica_ctx* ctx) {
    MigrateArgs<P> a{};
    migrateArgs(ctx, a);
    if ((size_t)a.bitmapWords * 4 > 200 * 1024) return fail(ctx, PICA_ERR_LIMIT, "supercell capacity too large for the leaver sort");
    CKL(launchMigrate(ctx, a, kSortLeavers));
    CKL(launchMigrate(ctx, a, kCountArrivals));
    CKL(launchMigrate(ctx, a, kFill));
    ctx->launches += 3;
    return PICA_OK;
}

// Host part, after the device part has finished and ctx->h_flags holds its flags:
// report a migration error, or rebuild on a capacity overflow; count the step.
template <class P>
static int migrateFinish(pica_ctx* ctx) {
    const pica_config& c = ctx->cfg;
    const int A = ctx->cur, B = 1 - ctx->cur;
    if (ctx->h_flags[0])
        return fail(ctx, ctx->h_flags[0],
                    ctx->h_flags[0] == PICA_ERR_TIMEOUT ? "the push's tensor copies of the E/B tile never completed"
                                                         : "a particle crossed more than one supercell in one step");
    if (ctx->h_flags[1]) {
        // Overflow (the fill did nothing): gather the leavers into the outbox (B is then
        // free), rebuild A + arrivals into B with capacities for the new counts, and swap.
        MigrateArgs<P> a{};
        for (int q = 0; q < c.nspecies; q++) {
            SpeciesState& S = ctx->sp[q];
            std::vector<int32_t> nl(ctx->nscTot);
            CK(cudaMemcpy(nl.data(), S.d_nleave, ctx->nscTot * 4, cudaMemcpyDeviceToHost));
            std::vector<int64_t> off(ctx->nscTot);
            int64_t tot = 0;
            for (int k = 0; k < ctx->nscTot; k++) { off[k] = tot; tot += nl[k]; }
            int rc;
            if ((rc = ensureOutbox(ctx, q, tot))) return rc;
            CK(cudaMemcpy(S.d_outOff, off.data(), ctx->nscTot * 8, cudaMemcpyHostToDevice));
        }
        migrateArgs(ctx, a);
        CKL(launchMigrate(ctx, a, kGatherOutbox));
        ctx->launches++;
        CK(cudaStreamSynchronize(ctx->stream));
        for (int q = 0; q < c.nspecies; q++) {
            SpeciesState& S = ctx->sp[q];
            std::vector<int32_t> needed(ctx->nscTot);
            CK(cudaMemcpy(needed.data(), S.d_needed, ctx->nscTot * 4, cudaMemcpyDeviceToHost));
            int64_t total;
            int rc;
            if ((rc = stageLayout(ctx, q, needed, total)) || (rc = ensureBuffer(ctx, q, B, total))) return rc;
        }
        migrateArgs(ctx, a);   // buffer B may have been reallocated
        CKL(launchMigrate(ctx, a, kRebuild));
        ctx->launches++;
        CK(cudaStreamSynchronize(ctx->stream));
        for (int q = 0; q < c.nspecies; q++) {
            SpeciesState& S = ctx->sp[q];
            std::swap(S.d_start, S.d_start2);
            std::swap(S.d_cap, S.d_cap2);
            int rc;
            if ((rc = ensureBuffer(ctx, q, A, S.layoutSlots)) || (rc = ensureSlotArrays(ctx, q, S.layoutSlots))) return rc;
        }
        ctx->cur = B;
        updateJFrac(ctx);
    }
    ctx->steps++;
    ctx->epoch++;
    return PICA_OK;
}

// The periodic resort, in three parts so that a batch can do each part for all its
// members before waiting: enqueue the copy of the live counts; once they have
// arrived, lay out the new capacities, upload them and launch the resort into the
// other buffer; once that has finished, swap layouts and buffers.
static bool resortDue(const pica_ctx* ctx) {
    return ctx->cfg.resort_every > 0 && ctx->steps > 0 && ctx->steps % ctx->cfg.resort_every == 0;
}

static int resortFetchCounts(pica_ctx* ctx) {
    for (int q = 0; q < ctx->cfg.nspecies; q++)
        CK(cudaMemcpyAsync(ctx->sp[q].h_pinAlive, ctx->sp[q].d_alive, ctx->nscTot * 4, cudaMemcpyDeviceToHost, ctx->stream));
    return PICA_OK;
}

template <class P>
static int resortLaunch(pica_ctx* ctx) {
    const int B2 = 1 - ctx->cur;
    const size_t n = ctx->nscTot;
    int32_t srcMaxCap = 0;   // of the layout being resorted
    for (int q = 0; q < ctx->cfg.nspecies; q++)
        for (int32_t v : ctx->sp[q].h_cap) srcMaxCap = std::max(srcMaxCap, v);
    for (int q = 0; q < ctx->cfg.nspecies; q++) {
        SpeciesState& S = ctx->sp[q];
        std::vector<int32_t> alive(S.h_pinAlive, S.h_pinAlive + n);
        std::vector<int64_t> nstart;
        std::vector<int32_t> ncap;
        int64_t total;
        layoutFrom(ctx, alive, nstart, ncap, total);
        std::copy(nstart.begin(), nstart.end(), S.h_pinStart);
        std::copy(ncap.begin(), ncap.end(), S.h_pinCap);
        int rc;
        if ((rc = ensureBuffer(ctx, q, B2, total)) || (rc = ensureSlotArrays(ctx, q, total))) return rc;
        CK(cudaMemcpyAsync(S.d_start2, S.h_pinStart, n * 8, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(S.d_cap2, S.h_pinCap, n * 4, cudaMemcpyHostToDevice, ctx->stream));
        S.h_start.swap(nstart);
        S.h_cap.swap(ncap);
        S.layoutSlots = total;
    }
    MigrateArgs<P> r{};
    migrateArgs(ctx, r);   // a = current buffer, dst = the other one, newStart = the uploaded layout
    r.srcMaxCap = srcMaxCap;
    CKL(launchMigrate(ctx, r, kResort));
    ctx->launches++;
    return PICA_OK;
}

static int resortFinish(pica_ctx* ctx) {
    const int A2 = ctx->cur;
    for (int q = 0; q < ctx->cfg.nspecies; q++) {
        SpeciesState& S = ctx->sp[q];
        std::swap(S.d_start, S.d_start2);
        std::swap(S.d_cap, S.d_cap2);
        int rc;
        if ((rc = ensureBuffer(ctx, q, A2, S.layoutSlots))) return rc;
    }
    ctx->cur = 1 - A2;
    updateJFrac(ctx);
    ctx->epoch++;
    return PICA_OK;
}

// Compact every supercell and sort it by cell into the other buffer, with
// capacities recomputed from the live counts.
template <class P>
static int resortNow(pica_ctx* ctx) {
    int rc = resortFetchCounts(ctx);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    if ((rc = resortLaunch<P>(ctx))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return resortFinish(ctx);
}

// The migration list of the step whose device part has just finished: the leaver
// lists (slots sorted ascending by the leaver sort) and the direction code of each
// leaver's slot, read back and expanded to (species, src, slot, dst).  Runs before
// a rebuild or resort changes the layout the lists refer to.
static int recordMigrations(pica_ctx* ctx) {
    ctx->mig.clear();
    const int n = ctx->nscTot;
    for (int q = 0; q < ctx->cfg.nspecies; q++) {
        SpeciesState& S = ctx->sp[q];
        std::vector<int32_t> nl(n), ll(S.layoutSlots);
        std::vector<uint32_t> dir(S.layoutSlots);
        CK(cudaMemcpy(nl.data(), S.d_nleave, (size_t)n * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(ll.data(), S.llist, (size_t)S.layoutSlots * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(dir.data(), S.dir, (size_t)S.layoutSlots * 4, cudaMemcpyDeviceToHost));
        for (int s = 0; s < n; s++) {
            const int sz = s % ctx->nsc[2], sy = (s / ctx->nsc[2]) % ctx->nsc[1], sx = s / (ctx->nsc[1] * ctx->nsc[2]);
            const int64_t st = S.h_start[s];
            for (int k = 0; k < nl[s]; k++) {
                const int slot = ll[st + k];
                const int code = (int)(dir[st + slot] & 31u);
                if (code == 13) continue;
                const int dx = code / 9 - 1, dy = (code / 3) % 3 - 1, dz = code % 3 - 1;
                const int nx = (sx + dx + ctx->nsc[0]) % ctx->nsc[0], ny = (sy + dy + ctx->nsc[1]) % ctx->nsc[1],
                          nz = (sz + dz + ctx->nsc[2]) % ctx->nsc[2];
                ctx->mig.insert(ctx->mig.end(), {q, s, slot, scLinear(ctx, nx, ny, nz)});
            }
        }
    }
    return PICA_OK;
}

template <class P>
static int migrateImpl(pica_ctx* ctx) {
    int rc = migrateDevice<P>(ctx);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->recordMig && !ctx->h_flags[0] && (rc = recordMigrations(ctx))) return rc;
    if ((rc = migrateFinish<P>(ctx))) return rc;
    return resortDue(ctx) ? resortNow<P>(ctx) : PICA_OK;
}

extern "C" {

int pica_migrate(pica_ctx* ctx) {
    if (!ctx) return PICA_ERR_INVALID;
    if (!ctx->pending) return fail(ctx, PICA_ERR_STATE, "migrate without push_deposit");
    ctx->pending = false;
    return ctx->fp64 ? migrateImpl<PlainPtrs>(ctx) : migrateImpl<CellPtrs>(ctx);
}

int pica_record_migrations(pica_ctx* ctx, int32_t enable) {
    if (!ctx) return PICA_ERR_INVALID;
    ctx->recordMig = enable != 0;
    ctx->mig.clear();
    return PICA_OK;
}

int64_t pica_num_migrations(pica_ctx* ctx) { return ctx ? (int64_t)(ctx->mig.size() / 4) : -1; }

int pica_get_migrations(pica_ctx* ctx, int32_t* species, int32_t* src, int32_t* slot, int32_t* dst) {
    if (!ctx) return PICA_ERR_INVALID;
    int32_t* out[4] = {species, src, slot, dst};
    const size_t m = ctx->mig.size() / 4;
    for (int c = 0; c < 4; c++)
        if (out[c])
            for (size_t i = 0; i < m; i++) out[c][i] = ctx->mig[4 * i + c];
    return PICA_OK;
}

int pica_field_slab(pica_ctx* ctx, int32_t comp, int32_t x0, int32_t nx, void* dev, int32_t mode) {
    if (!ctx || !dev || comp < 0 || comp > 8 || mode < 0 || mode > 2) return PICA_ERR_INVALID;
    const pica_config& c = ctx->cfg;
    if (x0 < 0 || nx < 0 || x0 + nx > c.n[0]) return fail(ctx, PICA_ERR_INVALID, "x-layers outside the grid");
    const size_t es = ctx->fp64 ? 8 : 4;
    const int64_t layer = (int64_t)c.n[1] * c.n[2];
    char* f = static_cast<char*>(ctx->f[comp]) + (size_t)x0 * (size_t)layer * es;
    const int64_t n = (int64_t)nx * layer;
    if (mode == 0) CK(cudaMemcpyAsync(dev, f, (size_t)n * es, cudaMemcpyDeviceToDevice, ctx->stream));
    else if (mode == 1) CK(cudaMemcpyAsync(f, dev, (size_t)n * es, cudaMemcpyDeviceToDevice, ctx->stream));
    else {
        CKL(launchAddSlab(ctx->fp64, f, dev, n, ctx->stream));
        ctx->launches++;
    }
    return PICA_OK;
}

// Counts and live counts of supercells [b, e) of species q, read back to the host.
static int rangeCounts(pica_ctx* ctx, int q, int b, int e, std::vector<int32_t>& cnt, std::vector<int32_t>& alive) {
    SpeciesState& S = ctx->sp[q];
    cnt.resize(e - b);
    alive.resize(e - b);
    CK(cudaMemcpyAsync(cnt.data(), S.d_count + b, (size_t)(e - b) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(alive.data(), S.d_alive + b, (size_t)(e - b) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return PICA_OK;
}

int64_t pica_take_supercells(pica_ctx* ctx, int32_t species, int32_t sc_begin, int32_t sc_end, void* const* dev,
                             int64_t capacity, int32_t* counts) {
    if (!ctx || species < 0 || species >= ctx->cfg.nspecies || sc_begin < 0 || sc_end < sc_begin ||
        sc_end > ctx->nscTot)
        return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "take while a migration is pending");
    SpeciesState& S = ctx->sp[species];
    const int m = sc_end - sc_begin;
    std::vector<int32_t> cnt, alive;
    int rc = rangeCounts(ctx, species, sc_begin, sc_end, cnt, alive);
    if (rc) return rc;
    std::vector<int64_t> off(m);
    int64_t tot = 0;
    for (int i = 0; i < m; i++) {
        if (cnt[i] != alive[i]) return fail(ctx, PICA_ERR_STATE, "supercells with dead slots: reorder first");
        off[i] = tot;
        tot += cnt[i];
    }
    if (counts) std::copy(cnt.begin(), cnt.end(), counts);
    if (!dev) return tot;   // sizes only
    if (tot > capacity) return fail(ctx, PICA_ERR_LIMIT, "the buffers hold fewer slots than the supercells");
    for (int k = 0; k < ctx->ncomp; k++)
        if (!dev[k]) return PICA_ERR_INVALID;
    // From pageable memory: staged before the call returns, ordered on the stream.
    CK(cudaMemcpyAsync(S.d_outOff + sc_begin, off.data(), (size_t)m * 8, cudaMemcpyHostToDevice, ctx->stream));
    for (int k = 0; k < ctx->ncomp; k++) {
        CKL(launchPackCopy(S.buf[ctx->cur][k], dev[k], S.d_start, S.d_count, S.d_outOff, sc_begin, sc_end,
                           (int)(ctx->compBytes[k] / 4), true, ctx->stream));
        ctx->launches++;
    }
    CK(cudaMemsetAsync(S.d_count + sc_begin, 0, (size_t)m * 4, ctx->stream));
    CK(cudaMemsetAsync(S.d_alive + sc_begin, 0, (size_t)m * 4, ctx->stream));
    ctx->epoch++;
    return tot;
}

int pica_append_to_supercells(pica_ctx* ctx, int32_t species, int32_t sc_begin, int32_t sc_end,
                              const int32_t* counts, const void* const* dev, int32_t dx_cells) {
    if (!ctx || !counts || species < 0 || species >= ctx->cfg.nspecies || sc_begin < 0 || sc_end < sc_begin ||
        sc_end > ctx->nscTot)
        return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "append while a migration is pending");
    SpeciesState& S = ctx->sp[species];
    const int m = sc_end - sc_begin;
    int64_t tot = 0;
    for (int i = 0; i < m; i++) {
        if (counts[i] < 0) return PICA_ERR_INVALID;
        tot += counts[i];
    }
    if (tot == 0) return PICA_OK;
    if (!dev) return PICA_ERR_INVALID;
    for (int k = 0; k < ctx->ncomp; k++)
        if (!dev[k]) return PICA_ERR_INVALID;
    std::vector<int32_t> cnt, alive;
    int rc = rangeCounts(ctx, species, sc_begin, sc_end, cnt, alive);
    if (rc) return rc;
    std::vector<int64_t> off(m), st(m);
    int64_t o = 0;
    for (int i = 0; i < m; i++) {
        if ((int64_t)cnt[i] + counts[i] > S.h_cap[sc_begin + i])
            return fail(ctx, PICA_ERR_OVERFLOW, "arrivals exceed the spare slots of a supercell");
        off[i] = o;
        o += counts[i];
        st[i] = S.h_start[sc_begin + i] + cnt[i];
        cnt[i] += counts[i];
        alive[i] += counts[i];
    }
    CK(cudaMemcpyAsync(S.d_outOff + sc_begin, off.data(), (size_t)m * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(S.d_start2 + sc_begin, st.data(), (size_t)m * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(S.d_cap2 + sc_begin, counts, (size_t)m * 4, cudaMemcpyHostToDevice, ctx->stream));
    CKL(launchAppendPositions(ctx->fp64, dev[0], S.buf[ctx->cur][0], S.d_start2, S.d_cap2, S.d_outOff, sc_begin,
                              sc_end, dx_cells, ctx->cfg.n[0], dx_cells * ctx->cfg.h[0], ctx->stream));
    ctx->launches++;
    for (int k = 1; k < ctx->ncomp; k++) {
        CKL(launchPackCopy(dev[k], S.buf[ctx->cur][k], S.d_start2, S.d_cap2, S.d_outOff, sc_begin, sc_end,
                           (int)(ctx->compBytes[k] / 4), false, ctx->stream));
        ctx->launches++;
    }
    CK(cudaMemcpyAsync(S.d_count + sc_begin, cnt.data(), (size_t)m * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(S.d_alive + sc_begin, alive.data(), (size_t)m * 4, cudaMemcpyHostToDevice, ctx->stream));
    ctx->epoch++;
    return PICA_OK;
}

int pica_reorder(pica_ctx* ctx) {
    if (!ctx) return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "reorder between push_deposit and migrate");
    return ctx->fp64 ? resortNow<PlainPtrs>(ctx) : resortNow<CellPtrs>(ctx);
}

int pica_step(pica_ctx* ctx, int32_t nsteps) {
    if (!ctx || nsteps < 0) return PICA_ERR_INVALID;
    const double dt = ctx->cfg.dt;
    for (int i = 0; i < nsteps; i++) {
        int rc;
        if ((rc = pica_push_deposit(ctx))) return rc;
        if ((rc = pica_update_b(ctx, 0.5 * dt))) return rc;
        if ((rc = pica_update_e(ctx, dt))) return rc;
        if ((rc = pica_update_b(ctx, 0.5 * dt))) return rc;
        if ((rc = pica_migrate(ctx))) return rc;
    }
    return PICA_OK;
}

int pica_field_energy(pica_ctx* ctx, double* out) {
    if (!ctx || !out) return PICA_ERR_INVALID;
    const pica_config& c = ctx->cfg;
    const int64_t nodes = (int64_t)c.n[0] * c.n[1] * c.n[2];
    CKL(launchFieldEnergy(ctx->fp64, ctx->f, nodes, ctx->d_red, ctx->d_out, ctx->stream));
    ctx->launches += 2;
    CK(cudaMemcpyAsync(ctx->h_out, ctx->d_out, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    *out = ctx->h_out[0] * (c.h[0] * c.h[1] * c.h[2]) / (8.0 * kPiRef);
    return PICA_OK;
}

static int buildRho(pica_ctx* ctx) {
    const pica_config& c = ctx->cfg;
    const int64_t nodes = (int64_t)c.n[0] * c.n[1] * c.n[2];
    if (!ctx->d_rho) CK(cudaMalloc(&ctx->d_rho, nodes * 8));
    CK(cudaMemsetAsync(ctx->d_rho, 0, nodes * 8, ctx->stream));
    RhoArgs r{};
    r.fp64 = ctx->fp64; r.shape = c.shape; r.nspecies = c.nspecies; r.nscTot = ctx->nscTot;
    for (int d = 0; d < 3; d++) { r.n[d] = c.n[d]; r.S[d] = c.sc[d]; r.nsc[d] = ctx->nsc[d]; r.invh[d] = 1.0 / c.h[d]; }
    r.norm = 1.0 / (c.h[0] * c.h[1] * c.h[2]);
    for (int q = 0; q < c.nspecies; q++) {
        void* const* b = ctx->sp[q].buf[ctx->cur];
        r.p0[q] = b[0]; r.p1[q] = b[1]; r.p2[q] = b[2]; r.p3[q] = ctx->fp64 ? nullptr : b[3];
        r.w[q] = ctx->fp64 ? b[6] : b[7];
        r.start[q] = ctx->sp[q].d_start; r.count[q] = ctx->sp[q].d_count; r.q[q] = c.charge[q];
    }
    CKL(launchRho(r, ctx->d_rho, ctx->stream));
    ctx->launches++;
    return PICA_OK;
}

int pica_charge_density(pica_ctx* ctx, double* rho) {
    if (!ctx || !rho) return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "charge density while a migration is pending");
    int rc = buildRho(ctx);
    if (rc) return rc;
    const int64_t nodes = (int64_t)ctx->cfg.n[0] * ctx->cfg.n[1] * ctx->cfg.n[2];
    CK(cudaMemcpyAsync(rho, ctx->d_rho, nodes * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return PICA_OK;
}

int pica_diagnostics(pica_ctx* ctx, double bg, pica_diag* out) {
    if (!ctx || !out) return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "diagnostics while a migration is pending");
    const pica_config& c = ctx->cfg;
    std::memset(out, 0, sizeof(*out));
    int rc = pica_field_energy(ctx, &out->field_energy);
    if (rc) return rc;
    ParticleSumArgs a{};
    a.fp64 = ctx->fp64; a.nspecies = c.nspecies; a.nscTot = ctx->nscTot;
    for (int q = 0; q < c.nspecies; q++) {
        void* const* b = ctx->sp[q].buf[ctx->cur];
        const int o = ctx->fp64 ? 3 : 4;
        a.ux[q] = b[o]; a.uy[q] = b[o + 1]; a.uz[q] = b[o + 2]; a.w[q] = b[o + 3];
        a.key[q] = b[0];
        a.start[q] = ctx->sp[q].d_start; a.count[q] = ctx->sp[q].d_count;
        a.mc2[q] = c.mass[q] * kC * kC; a.q[q] = c.charge[q];
    }
    CKL(launchParticleSums(a, ctx->d_red, ctx->d_out, ctx->stream));
    ctx->launches += 2;
    if ((rc = buildRho(ctx))) return rc;
    CKL(launchGauss(ctx->fp64, ctx->f, ctx->d_rho, c.n, c.h, bg, ctx->d_red, ctx->d_out + 2, ctx->stream));
    ctx->launches += 2;
    CK(cudaMemcpyAsync(ctx->h_out, ctx->d_out, 4 * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    out->kinetic_energy = ctx->h_out[0];
    out->total_charge = ctx->h_out[1];
    out->gauss_max = ctx->h_out[2];
    out->rho_max = ctx->h_out[3];
    return PICA_OK;
}

int64_t pica_state_slots(pica_ctx* ctx, int32_t species) {
    if (!ctx || species < 0 || species >= ctx->cfg.nspecies) return PICA_ERR_INVALID;
    return ctx->sp[species].layoutSlots;
}

int pica_state_copy(pica_ctx* ctx, int32_t species, int32_t comp, void* host, int32_t to_device) {
    if (!ctx || !host || species < 0 || species >= ctx->cfg.nspecies || comp < 0 || comp >= ctx->ncomp)
        return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "state copy while a migration is pending");
    SpeciesState& S = ctx->sp[species];
    const size_t bytes = S.layoutSlots * ctx->compBytes[comp];
    if (to_device) CK(cudaMemcpyAsync(S.buf[ctx->cur][comp], host, bytes, cudaMemcpyHostToDevice, ctx->stream));
    else CK(cudaMemcpyAsync(host, S.buf[ctx->cur][comp], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return PICA_OK;
}

int pica_state_copy_range_on(pica_ctx* ctx, int32_t species, int32_t comp, void* host, int32_t to_device,
                             int32_t sc_begin, int32_t sc_end, void* copy_stream) {
    if (!ctx || !host || species < 0 || species >= ctx->cfg.nspecies || comp < 0 || comp >= ctx->ncomp ||
        sc_begin < 0 || sc_end < sc_begin || sc_end > ctx->nscTot)
        return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "state copy while a migration is pending");
    SpeciesState& S = ctx->sp[species];
    const int64_t s0 = sc_begin < ctx->nscTot ? S.h_start[sc_begin] : S.layoutSlots;
    const int64_t s1 = sc_end < ctx->nscTot ? S.h_start[sc_end] : S.layoutSlots;
    const size_t cb = ctx->compBytes[comp];
    const size_t bytes = (size_t)(s1 - s0) * cb;
    if (bytes == 0) return PICA_OK;
    char* hp = static_cast<char*>(host) + (size_t)s0 * cb;
    char* dp = static_cast<char*>(S.buf[ctx->cur][comp]) + (size_t)s0 * cb;
    cudaStream_t cs = copy_stream ? static_cast<cudaStream_t>(copy_stream) : ctx->stream;
    if (cs != ctx->stream && !ctx->copyOrder) CK(cudaEventCreateWithFlags(&ctx->copyOrder, cudaEventDisableTiming));
    if (to_device) {
        CK(cudaMemcpyAsync(dp, hp, bytes, cudaMemcpyHostToDevice, cs));
        if (cs != ctx->stream) {
            CK(cudaEventRecord(ctx->copyOrder, cs));
            CK(cudaStreamWaitEvent(ctx->stream, ctx->copyOrder, 0));
        }
    } else {
        if (cs != ctx->stream) {
            CK(cudaEventRecord(ctx->copyOrder, ctx->stream));
            CK(cudaStreamWaitEvent(cs, ctx->copyOrder, 0));
        }
        CK(cudaMemcpyAsync(hp, dp, bytes, cudaMemcpyDeviceToHost, cs));
    }
    return PICA_OK;
}

int64_t pica_state_packed_slots(pica_ctx* ctx, int32_t species) {
    if (!ctx || species < 0 || species >= ctx->cfg.nspecies) return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "packed state while a migration is pending");
    SpeciesState& S = ctx->sp[species];
    const int n = ctx->nscTot;
    std::vector<int32_t> count(n);
    std::vector<int64_t> off(n);
    CK(cudaMemcpyAsync(count.data(), S.d_count, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    int64_t total = 0;
    for (int s = 0; s < n; s++) { off[s] = total; total += count[s]; }
    S.h_packOff.assign(off.begin(), off.end());
    S.h_packOff.push_back(total);
    if (!S.d_packOff) CK(cudaMalloc(&S.d_packOff, (size_t)n * 8));
    CK(cudaMemcpyAsync(S.d_packOff, off.data(), (size_t)n * 8, cudaMemcpyHostToDevice, ctx->stream));
    if (total > S.packCap) {
        CK(cudaStreamSynchronize(ctx->stream));
        for (auto& p : S.d_pack) {
            if (p) CK(cudaFree(p));
            p = nullptr;
        }
        S.packCap = 0;
        const int64_t cap = withHeadroom(total);
        for (int k = 0; k < ctx->ncomp; k++) CK(cudaMalloc(&S.d_pack[k], cap * ctx->compBytes[k]));
        S.packCap = cap;
    }
    CK(cudaStreamSynchronize(ctx->stream));   // the offsets are in place before the host vector goes
    S.packSlots = total;
    S.packEpoch = ctx->epoch;
    return total;
}

int pica_state_copy_packed(pica_ctx* ctx, int32_t species, int32_t comp, void* host, int32_t to_device) {
    if (!ctx) return PICA_ERR_INVALID;
    return pica_state_copy_packed_range(ctx, species, comp, host, to_device, 0, ctx->nscTot);
}

int pica_state_copy_packed_range(pica_ctx* ctx, int32_t species, int32_t comp, void* host, int32_t to_device,
                                 int32_t sc_begin, int32_t sc_end) {
    return pica_state_copy_packed_range_on(ctx, species, comp, host, to_device, sc_begin, sc_end, nullptr);
}

int pica_state_copy_packed_range_on(pica_ctx* ctx, int32_t species, int32_t comp, void* host, int32_t to_device,
                                    int32_t sc_begin, int32_t sc_end, void* copy_stream) {
    if (!ctx || !host || species < 0 || species >= ctx->cfg.nspecies || comp < 0 || comp >= ctx->ncomp ||
        sc_begin < 0 || sc_end < sc_begin || sc_end > ctx->nscTot)
        return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "state copy while a migration is pending");
    SpeciesState& S = ctx->sp[species];
    if (S.packEpoch != ctx->epoch)
        return fail(ctx, PICA_ERR_STATE, "packed layout out of date: call pica_state_packed_slots after each step");
    // Image slots [off[sc_begin], off[sc_end]) of the host image and of the staging copy.
    const size_t cb = ctx->compBytes[comp];
    const int64_t o0 = S.h_packOff[sc_begin], o1 = S.h_packOff[sc_end];
    const size_t bytes = (size_t)(o1 - o0) * cb;
    const int words = (int)(cb / 4);
    if (bytes == 0) return PICA_OK;
    char* hp = static_cast<char*>(host) + (size_t)o0 * cb;
    char* dp = static_cast<char*>(S.d_pack[comp]) + (size_t)o0 * cb;
    // With a copy stream the host copy goes there, and one event orders it against
    // the gather / scatter kernel on the context stream (a wait takes the event's
    // latest record when it is enqueued, so the one event serves every call).
    cudaStream_t cs = copy_stream ? static_cast<cudaStream_t>(copy_stream) : ctx->stream;
    if (cs != ctx->stream && !ctx->copyOrder) CK(cudaEventCreateWithFlags(&ctx->copyOrder, cudaEventDisableTiming));
    if (to_device) {
        CK(cudaMemcpyAsync(dp, hp, bytes, cudaMemcpyHostToDevice, cs));
        if (cs != ctx->stream) {
            CK(cudaEventRecord(ctx->copyOrder, cs));
            CK(cudaStreamWaitEvent(ctx->stream, ctx->copyOrder, 0));
        }
        CKL(launchPackCopy(S.d_pack[comp], S.buf[ctx->cur][comp], S.d_start, S.d_count, S.d_packOff, sc_begin, sc_end,
                           words, false, ctx->stream));
    } else {
        CKL(launchPackCopy(S.buf[ctx->cur][comp], S.d_pack[comp], S.d_start, S.d_count, S.d_packOff, sc_begin, sc_end,
                           words, true, ctx->stream));
        if (cs != ctx->stream) {
            CK(cudaEventRecord(ctx->copyOrder, ctx->stream));
            CK(cudaStreamWaitEvent(cs, ctx->copyOrder, 0));
        }
        CK(cudaMemcpyAsync(hp, dp, bytes, cudaMemcpyDeviceToHost, cs));
    }
    ctx->launches++;
    return PICA_OK;
}

// ---------------------------------------------------------------------------
// Host-side synthetic plasma.  Counter-based random numbers (SplitMix64 finaliser
// of seed, cell, particle and draw index), so the result does not depend on the
// thread count.  Positions uniform in the cell; u = drift + N(0, sigma) per
// component (Box-Muller).
// ---------------------------------------------------------------------------
int64_t pica_plasma_count(const pica_plasma_spec* s) {
    if (!s || s->n[0] <= 0 || s->n[1] <= 0 || s->n[2] <= 0 || s->ppc < 0) return PICA_ERR_INVALID;
    int64_t total = 0;
    for (int i = 0; i < s->n[0]; i++) total += (int64_t)cellCount(s, i) * s->n[1] * s->n[2];
    return total;
}

int pica_plasma_generate(const pica_plasma_spec* s, int32_t threads, double* x, double* y, double* z, double* ux,
                         double* uy, double* uz, double* w, int32_t* species) {
    if (pica_plasma_count(s) < 0 || !x || !y || !z || !ux || !uy || !uz || !w) return PICA_ERR_INVALID;
    const int nx = s->n[0], ny = s->n[1], nz = s->n[2];
    std::vector<int64_t> planeStart(nx + 1, 0);
    for (int i = 0; i < nx; i++) planeStart[i + 1] = planeStart[i] + (int64_t)cellCount(s, i) * ny * nz;
    const int nthreads = threads > 0 ? threads : std::max(1u, std::thread::hardware_concurrency());
    auto work = [&](int i0, int i1) {
        for (int i = i0; i < i1; i++) {
            const int per = cellCount(s, i);
            int64_t o = planeStart[i];
            for (int j = 0; j < ny; j++)
                for (int k = 0; k < nz; k++) {
                    const int64_t cell = ((int64_t)i * ny + j) * nz + k;
                    for (int p = 0; p < per; p++, o++) {
                        x[o] = ((double)i + uniDraw(s->seed, cell, p, 0)) * s->h[0];
                        y[o] = ((double)j + uniDraw(s->seed, cell, p, 1)) * s->h[1];
                        z[o] = ((double)k + uniDraw(s->seed, cell, p, 2)) * s->h[2];
                        double u3[3] = {s->sigma_u * normalDraw(s->seed, cell, p, 3), s->sigma_u * normalDraw(s->seed, cell, p, 5),
                                        s->sigma_u * normalDraw(s->seed, cell, p, 7)};
                        if (s->nbeams == 2) u3[s->drift_axis] += (p % 2 == 0) ? s->drift_u : -s->drift_u;
                        else u3[s->drift_axis] += s->drift_u;
                        ux[o] = u3[0]; uy[o] = u3[1]; uz[o] = u3[2];
                        w[o] = s->weight;
                        if (species) species[o] = s->species;
                    }
                }
        }
    };
    std::vector<std::thread> th;
    const int chunk = (nx + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        const int a = t * chunk, b = std::min(nx, a + chunk);
        if (a >= b) break;
        th.emplace_back(work, a, b);
    }
    for (auto& t : th) t.join();
    return PICA_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batching form: many independent plasmas advanced together.  The push of every
// member is one persistent launch over all members' supercells (arguments in a
// device table); the rest of the step is enqueued per member.  The device part
// of the step is captured once as a CUDA graph and replayed while the launch
// arguments stay the same (they change at a resort or a capacity rebuild, when
// the graph is captured again).  After each step the host reads every member's
// flags and runs the host part of the migration (errors, rebuilds, resorts).
// ---------------------------------------------------------------------------
struct pica_batch {
    std::vector<pica_ctx*> m;
    cudaStream_t stream = nullptr;
    int shape = PICA_SHAPE_CIC;
    int S[3] = {};
    int variant = 0;
    bool useGraph = true;
    int* d_counter = nullptr;                // one work counter per push launch
    // The members' chains after the push (current conversion, field updates,
    // migration) run on kBatchLanes streams forked from and joined back to `stream`.
    static constexpr int kBatchLanes = 8;
    cudaStream_t lanes[kBatchLanes] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kBatchLanes] = {};
    std::vector<int> order;                  // members in work order
    int nsp = 1;                             // species slots of the push arguments (1 or 2)
    std::vector<BatchPushArgs<1>> args1;     // one persistent push launch per batchMembers<NSP>() members
    std::vector<BatchPushArgs<2>> args2;
    // Instantiated graphs by the launch arguments they were captured with (a resort
    // swaps the buffers, so the arguments alternate between a few states).
    struct Graph {
        std::vector<unsigned char> sig;
        cudaGraphExec_t exec;
        int64_t used;
    };
    std::vector<Graph> graphs;
    cudaGraphExec_t exec = nullptr;          // the graph for the current arguments
    std::vector<unsigned char> sig;          // the current launch arguments
    int64_t captures = 0, graphLaunches = 0, steps = 0;
    int64_t kernelLaunches = 0;              // launches of the device part of the steps
    std::string err;
};

namespace {

int batchFail(pica_batch* b, int code, const std::string& msg) {
    b->err = msg;
    return code;
}

#define BK(call)                                                                               \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return batchFail(b, e_ == cudaErrorMemoryAllocation ? PICA_ERR_OOM : PICA_ERR_CUDA, \
                             std::string(#call) + ": " + cudaGetErrorString(e_));              \
    } while (0)

int memberFail(pica_batch* b, int k, int rc) {
    return batchFail(b, rc, "member " + std::to_string(k) + ": " + (b->m[k]->err.empty() ? "error" : b->m[k]->err));
}

void memberPushArgs(pica_ctx* ctx, PushArgs<CellPtrs>& a) {
    std::memset(&a, 0, sizeof a);
    fillPushArgs(ctx, a);
    for (int q = 0; q < ctx->cfg.nspecies; q++) {
        a.sp[q].buf = cellPtrs(ctx, q, ctx->cur);
        a.sp[q].out = cellPtrs(ctx, q, 1 - ctx->cur);
    }
}

// Everything the captured step depends on: per member in work order, the push and
// migration arguments and the current-conversion scale.
void batchSignature(pica_batch* b, std::vector<unsigned char>& sig) {
    sig.clear();
    auto put = [&](const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        sig.insert(sig.end(), c, c + n);
    };
    for (int k : b->order) {
        pica_ctx* ctx = b->m[k];
        PushArgs<CellPtrs> a;
        memberPushArgs(ctx, a);
        put(&a, sizeof a);
        MigrateArgs<CellPtrs> ma;
        std::memset(&ma, 0, sizeof ma);
        migrateArgs(ctx, ma);
        put(&ma, sizeof ma);
        put(&ctx->jfrac, sizeof ctx->jfrac);
        put(&ctx->kmax, sizeof ctx->kmax);
        put(&ctx->cur, sizeof ctx->cur);
    }
    put(&b->variant, sizeof b->variant);
}

// Arguments of the persistent push launches for the current layouts (members in
// work order, batchMembers<NSP>() per launch).
template <int NSP>
void batchLaunchArgs(pica_batch* b, std::vector<BatchPushArgs<NSP>>& out) {
    constexpr int M = batchMembers<NSP>();
    const int n = (int)b->order.size();
    const int launches = (n + M - 1) / M;
    out.resize(launches);
    for (int c = 0; c < launches; c++) {
        BatchPushArgs<NSP>& ba = out[c];
        std::memset(&ba, 0, sizeof ba);
        ba.count = std::min(M, n - c * M);
        ba.counter = b->d_counter + c;
        ba.base[0] = 0;
        for (int i = 0; i < ba.count; i++) {
            pica_ctx* ctx = b->m[b->order[c * M + i]];
            PushArgs<CellPtrs> a;
            memberPushArgs(ctx, a);
            slimArgs(a, ba.members[i]);
            ba.base[i + 1] = ba.base[i] + ctx->nscTot;
        }
        ba.total = ba.base[ba.count];
    }
}

size_t batchPushLaunches(const pica_batch* b) { return b->nsp == 1 ? b->args1.size() : b->args2.size(); }

// The device part of one step of every member, enqueued on the batch stream.
int batchEnqueue(pica_batch* b) {
    for (int k : b->order) BK(cudaMemsetAsync(b->m[k]->d_flags, 0, 4 * sizeof(int), b->stream));
    BK(cudaMemsetAsync(b->d_counter, 0, batchPushLaunches(b) * sizeof(int), b->stream));
    for (const auto& ba : b->args1)
        if (b->nsp == 1 && launchPushBatch(ba, b->shape, b->S, b->variant, b->stream))
            return batchFail(b, PICA_ERR_CUDA, "batched push launch failed");
    for (const auto& ba : b->args2)
        if (b->nsp == 2 && launchPushBatch(ba, b->shape, b->S, b->variant, b->stream))
            return batchFail(b, PICA_ERR_CUDA, "batched push launch failed");
    // Fork: member i's chain goes to lane i % kBatchLanes, after the push.
    BK(cudaEventRecord(b->fork, b->stream));
    for (int l = 0; l < pica_batch::kBatchLanes; l++) BK(cudaStreamWaitEvent(b->lanes[l], b->fork, 0));
    for (size_t i = 0; i < b->order.size(); i++) {
        const int k = b->order[i];
        pica_ctx* ctx = b->m[k];
        cudaStream_t ls = b->lanes[i % pica_batch::kBatchLanes];
        const pica_config& c = ctx->cfg;
        const int64_t nodes = (int64_t)c.n[0] * c.n[1] * c.n[2];
        const double scale = (ctx->kmax * std::ldexp(1.0, -ctx->jfrac)) * (1.0 / (c.h[0] * c.h[1] * c.h[2]));
        if (launchConvertJ(false, ctx->f + 6, ctx->jacc, nodes, scale, ls))
            return batchFail(b, PICA_ERR_CUDA, "current conversion launch failed");
        double cb[3], ce[3];
        for (int d = 0; d < 3; d++) { cb[d] = (kC * (0.5 * c.dt)) / c.h[d]; ce[d] = (kC * c.dt) / c.h[d]; }
        if (launchUpdateB(false, ctx->f, c.n, cb, ls) || launchUpdateE(false, ctx->f, c.n, -4.0 * kPiRef * c.dt, ce, ls) ||
            launchUpdateB(false, ctx->f, c.n, cb, ls))
            return batchFail(b, PICA_ERR_CUDA, "field update launch failed");
        const int64_t before = ctx->launches;   // counted per executed step by the caller
        ctx->stream = ls;
        const int rc = migrateDevice<CellPtrs>(ctx);
        ctx->stream = b->stream;
        ctx->launches = before;
        if (rc) return memberFail(b, k, rc);
    }
    // Join every lane back into the batch stream.
    for (int l = 0; l < pica_batch::kBatchLanes; l++) {
        BK(cudaEventRecord(b->join[l], b->lanes[l]));
        BK(cudaStreamWaitEvent(b->stream, b->join[l], 0));
    }
    return PICA_OK;
}

// Kernel launches of the device part of one step: the batched push launches, then per
// member the current conversion, three field updates and three migration stages.
int64_t batchStepLaunches(const pica_batch* b) { return (int64_t)batchPushLaunches(b) + 7 * (int64_t)b->m.size(); }

// Work order: most particles per supercell first, for a short tail.
int batchOrder(pica_batch* b) {
    const int n = (int)b->m.size();
    std::vector<double> per(n);
    for (int k = 0; k < n; k++) {
        int64_t np = 0;
        for (int q = 0; q < b->m[k]->cfg.nspecies; q++) np += b->m[k]->sp[q].layoutSlots;
        per[k] = (double)np / b->m[k]->nscTot;
    }
    b->order.resize(n);
    for (int k = 0; k < n; k++) b->order[k] = k;
    std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) { return per[x] > per[y]; });
    return PICA_OK;
}

int batchStepOnce(pica_batch* b) {
    for (size_t k = 0; k < b->m.size(); k++) {
        pica_ctx* ctx = b->m[k];
        if (ctx->pending) return batchFail(b, PICA_ERR_STATE, "member " + std::to_string(k) + ": push pending");
        ctx->stream = b->stream;
    }
    if (b->order.empty()) {
        const int rc = batchOrder(b);
        if (rc) return rc;
    }
    std::vector<unsigned char> sig;
    batchSignature(b, sig);
    if (sig != b->sig) {
        if (b->nsp == 1) batchLaunchArgs(b, b->args1);
        else batchLaunchArgs(b, b->args2);
        b->exec = nullptr;
        if (b->useGraph) {
            for (auto& g : b->graphs)
                if (g.sig == sig) b->exec = g.exec;
            if (!b->exec) {
                cudaGraph_t g = nullptr;
                BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed));
                const int rc = batchEnqueue(b);
                const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
                if (rc) {
                    if (g) cudaGraphDestroy(g);
                    return rc;
                }
                BK(e);
                cudaGraphExec_t x = nullptr;
                const cudaError_t ei = cudaGraphInstantiate(&x, g, 0);
                cudaGraphDestroy(g);
                BK(ei);
                b->captures++;
                if (b->graphs.size() >= 4) {   // drop the least recently used
                    auto lru = std::min_element(b->graphs.begin(), b->graphs.end(),
                                                [](const pica_batch::Graph& u, const pica_batch::Graph& v) { return u.used < v.used; });
                    cudaGraphExecDestroy(lru->exec);
                    b->graphs.erase(lru);
                }
                b->graphs.push_back({sig, x, b->steps});
                b->exec = x;
            }
        }
        b->sig.swap(sig);
    }
    for (auto& g : b->graphs)
        if (g.exec == b->exec) g.used = b->steps;
    if (b->useGraph) {
        BK(cudaGraphLaunch(b->exec, b->stream));
        b->graphLaunches++;
    } else {
        const int rc = batchEnqueue(b);
        if (rc) return rc;
    }
    b->kernelLaunches += batchStepLaunches(b);
    for (pica_ctx* ctx : b->m)
        BK(cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    std::vector<int> due;
    for (size_t k = 0; k < b->m.size(); k++) {
        const int rc = migrateFinish<CellPtrs>(b->m[k]);
        if (rc) return memberFail(b, (int)k, rc);
        if (resortDue(b->m[k])) due.push_back((int)k);
    }
    if (!due.empty()) {
        // Resorts of every member due: counts of all, one wait; layouts and launches on
        // the lanes; one wait; swaps.
        for (int k : due) {
            const int rc = resortFetchCounts(b->m[k]);
            if (rc) return memberFail(b, k, rc);
        }
        BK(cudaStreamSynchronize(b->stream));
        for (size_t i = 0; i < due.size(); i++) {
            pica_ctx* ctx = b->m[due[i]];
            ctx->stream = b->lanes[i % pica_batch::kBatchLanes];
            const int rc = resortLaunch<CellPtrs>(ctx);
            ctx->stream = b->stream;
            if (rc) return memberFail(b, due[i], rc);
        }
        for (int l = 0; l < pica_batch::kBatchLanes; l++) BK(cudaStreamSynchronize(b->lanes[l]));
        for (int k : due) {
            const int rc = resortFinish(b->m[k]);
            if (rc) return memberFail(b, k, rc);
        }
    }
    b->steps++;
    return PICA_OK;
}

}  // namespace

extern "C" {

int pica_batch_create(const pica_config* cfgs, int32_t count, pica_batch** out) {
    if (!cfgs || !out || count < 1) return PICA_ERR_INVALID;
    *out = nullptr;
    for (int k = 0; k < count; k++) {
        const pica_config& c = cfgs[k];
        if (c.form != PICA_FORM_FP32_CELL || c.deposit != PICA_DEPOSIT_ESIRKEPOV || c.shape != cfgs[0].shape ||
            c.nspecies > kBatchSpecies)
            return PICA_ERR_INVALID;
        for (int d = 0; d < 3; d++)
            if (c.sc[d] != cfgs[0].sc[d]) return PICA_ERR_INVALID;
    }
    pica_batch* b = new pica_batch();
    b->shape = cfgs[0].shape;
    for (int k = 0; k < count; k++) b->nsp = std::max(b->nsp, (int)cfgs[k].nspecies);
    for (int d = 0; d < 3; d++) b->S[d] = cfgs[0].sc[d];
    auto bail = [&](int rc) {
        pica_batch_destroy(b);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(PICA_ERR_CUDA);
    if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) return bail(PICA_ERR_CUDA);
    for (int l = 0; l < pica_batch::kBatchLanes; l++)
        if (cudaStreamCreateWithFlags(&b->lanes[l], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->join[l], cudaEventDisableTiming) != cudaSuccess)
            return bail(PICA_ERR_CUDA);
    for (int k = 0; k < count; k++) {
        pica_ctx* ctx = nullptr;
        const int rc = pica_ctx_create(&cfgs[k], &ctx);
        if (rc) return bail(rc);
        ctx->stream = b->stream;
        b->m.push_back(ctx);
    }
    if (cudaMalloc(&b->d_counter, ((count + batchMembers<kBatchSpecies>() - 1) / batchMembers<kBatchSpecies>()) * sizeof(int)) !=
        cudaSuccess)
        return bail(PICA_ERR_OOM);
    *out = b;
    return PICA_OK;
}

int pica_batch_destroy(pica_batch* b) {
    if (!b) return PICA_ERR_INVALID;
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
    for (pica_ctx* ctx : b->m) pica_ctx_destroy(ctx);
    if (b->d_counter) cudaFree(b->d_counter);
    for (int l = 0; l < pica_batch::kBatchLanes; l++) {
        if (b->lanes[l]) cudaStreamDestroy(b->lanes[l]);
        if (b->join[l]) cudaEventDestroy(b->join[l]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return PICA_OK;
}

pica_ctx* pica_batch_member(pica_batch* b, int32_t k) {
    if (!b || k < 0 || k >= (int)b->m.size()) return nullptr;
    b->order.clear();   // particle counts may change: recompute the work order at the next step
    b->sig.clear();
    return b->m[k];
}

int pica_batch_set_options(pica_batch* b, int32_t use_graph, int32_t variant) {
    if (!b || variant < 0 || variant >= kPushVariants) return PICA_ERR_INVALID;
    b->useGraph = use_graph != 0;
    b->variant = variant;   // part of the signature: graphs of other variants stay cached
    b->sig.clear();
    return PICA_OK;
}

int pica_batch_step(pica_batch* b, int32_t nsteps) {
    if (!b || nsteps < 0) return PICA_ERR_INVALID;
    for (int s = 0; s < nsteps; s++) {
        const int rc = batchStepOnce(b);
        if (rc) return rc;
    }
    return PICA_OK;
}

int pica_batch_stats(pica_batch* b, int64_t* out4) {
    if (!b || !out4) return PICA_ERR_INVALID;
    int64_t launches = 0;
    for (pica_ctx* ctx : b->m) launches += ctx->launches;
    out4[0] = b->captures;
    out4[1] = b->graphLaunches;
    out4[2] = b->kernelLaunches + launches;   // device part of the steps + rebuilds and resorts
    out4[3] = b->steps;
    return PICA_OK;
}

const char* pica_batch_last_error(pica_batch* b) { return b ? b->err.c_str() : "null batch"; }

}  // extern "C"

// ---------------------------------------------------------------------------
// Checkpoints: the complete state of a context between steps, so that a context
// loaded from one continues bit for bit like the original.  Layout (native byte
// order): magic, version, the pica_config, the step counter and fixed-point
// parameters, the nine field arrays as stored, then per species the slot layout
// (start, capacity, used and live counts per supercell) and the current particle
// buffer (every component, all slots of the layout).
// ---------------------------------------------------------------------------
namespace {

constexpr uint64_t kCkptMagic = 0x31504B4341434950ull;   // "PICACKP1"
constexpr uint32_t kCkptVersion = 1;

struct CkptHeader {
    uint64_t magic;
    uint32_t version;
    uint32_t fp64;
    pica_config cfg;
    int64_t steps;
    double kmax;
    int32_t jfrac, tileSplit;
};

struct FileCloser {
    FILE* f;
    ~FileCloser() { if (f) std::fclose(f); }
};

bool writeAll(FILE* f, const void* p, size_t n) { return n == 0 || std::fwrite(p, 1, n, f) == n; }
bool readAll(FILE* f, void* p, size_t n) { return n == 0 || std::fread(p, 1, n, f) == n; }

}  // namespace

extern "C" {

int64_t pica_step_count(pica_ctx* ctx) { return ctx ? ctx->steps : (int64_t)PICA_ERR_INVALID; }

int pica_checkpoint_save(pica_ctx* ctx, const char* path) {
    if (!ctx || !path) return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "checkpoint while a migration is pending");
    CK(cudaStreamSynchronize(ctx->stream));
    FileCloser fc{std::fopen(path, "wb")};
    if (!fc.f) return fail(ctx, PICA_ERR_INVALID, std::string("cannot open ") + path);
    CkptHeader h;
    std::memset(&h, 0, sizeof h);
    h.magic = kCkptMagic;
    h.version = kCkptVersion;
    h.fp64 = ctx->fp64 ? 1 : 0;
    h.cfg = ctx->cfg;
    h.steps = ctx->steps;
    h.kmax = ctx->kmax;
    h.jfrac = ctx->jfrac;
    h.tileSplit = ctx->tileSplit;
    if (!writeAll(fc.f, &h, sizeof h)) return fail(ctx, PICA_ERR_INVALID, "checkpoint write failed");
    const pica_config& c = ctx->cfg;
    const int64_t nodes = (int64_t)c.n[0] * c.n[1] * c.n[2];
    const size_t rb = ctx->fp64 ? 8 : 4;
    std::vector<unsigned char> buf(nodes * rb);
    for (int k = 0; k < 9; k++) {
        CK(cudaMemcpy(buf.data(), ctx->f[k], nodes * rb, cudaMemcpyDeviceToHost));
        if (!writeAll(fc.f, buf.data(), buf.size())) return fail(ctx, PICA_ERR_INVALID, "checkpoint write failed");
    }
    const size_t n = ctx->nscTot;
    for (int q = 0; q < c.nspecies; q++) {
        SpeciesState& S = ctx->sp[q];
        std::vector<int32_t> count(n), alive(n);
        CK(cudaMemcpy(count.data(), S.d_count, n * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(alive.data(), S.d_alive, n * 4, cudaMemcpyDeviceToHost));
        const int64_t slots = S.layoutSlots;
        if (!writeAll(fc.f, &slots, 8) || !writeAll(fc.f, S.h_start.data(), n * 8) || !writeAll(fc.f, S.h_cap.data(), n * 4) ||
            !writeAll(fc.f, count.data(), n * 4) || !writeAll(fc.f, alive.data(), n * 4))
            return fail(ctx, PICA_ERR_INVALID, "checkpoint write failed");
        for (int k = 0; k < ctx->ncomp; k++) {
            std::vector<unsigned char> comp(slots * ctx->compBytes[k]);
            CK(cudaMemcpy(comp.data(), S.buf[ctx->cur][k], comp.size(), cudaMemcpyDeviceToHost));
            if (!writeAll(fc.f, comp.data(), comp.size())) return fail(ctx, PICA_ERR_INVALID, "checkpoint write failed");
        }
    }
    return std::fflush(fc.f) == 0 ? PICA_OK : fail(ctx, PICA_ERR_INVALID, "checkpoint write failed");
}

int pica_checkpoint_load(pica_ctx* ctx, const char* path) {
    if (!ctx || !path) return PICA_ERR_INVALID;
    if (ctx->pending) return fail(ctx, PICA_ERR_STATE, "checkpoint load while a migration is pending");
    CK(cudaStreamSynchronize(ctx->stream));
    FileCloser fc{std::fopen(path, "rb")};
    if (!fc.f) return fail(ctx, PICA_ERR_INVALID, std::string("cannot open ") + path);
    CkptHeader h;
    if (!readAll(fc.f, &h, sizeof h) || h.magic != kCkptMagic || h.version != kCkptVersion)
        return fail(ctx, PICA_ERR_INVALID, "not a pica_gb300 checkpoint");
    pica_config a = h.cfg, b = ctx->cfg;
    a.threads = b.threads = 0;   // host threads do not change results
    if (std::memcmp(&a, &b, sizeof(pica_config)) != 0 || h.fp64 != (ctx->fp64 ? 1u : 0u))
        return fail(ctx, PICA_ERR_INVALID, "checkpoint of a different configuration");
    const pica_config& c = ctx->cfg;
    const int64_t nodes = (int64_t)c.n[0] * c.n[1] * c.n[2];
    const size_t rb = ctx->fp64 ? 8 : 4;
    std::vector<unsigned char> buf(nodes * rb);
    for (int k = 0; k < 9; k++) {
        if (!readAll(fc.f, buf.data(), buf.size())) return fail(ctx, PICA_ERR_INVALID, "truncated checkpoint");
        CK(cudaMemcpy(ctx->f[k], buf.data(), buf.size(), cudaMemcpyHostToDevice));
    }
    const size_t n = ctx->nscTot;
    for (int q = 0; q < c.nspecies; q++) {
        SpeciesState& S = ctx->sp[q];
        int64_t slots = 0;
        std::vector<int64_t> start(n);
        std::vector<int32_t> cap(n), count(n), alive(n);
        if (!readAll(fc.f, &slots, 8) || !readAll(fc.f, start.data(), n * 8) || !readAll(fc.f, cap.data(), n * 4) ||
            !readAll(fc.f, count.data(), n * 4) || !readAll(fc.f, alive.data(), n * 4))
            return fail(ctx, PICA_ERR_INVALID, "truncated checkpoint");
        if (slots < 0 || (n && (start[n - 1] + cap[n - 1] != slots))) return fail(ctx, PICA_ERR_INVALID, "corrupt checkpoint layout");
        int rc;
        if ((rc = ensureBuffer(ctx, q, 0, slots)) || (rc = ensureBuffer(ctx, q, 1, slots)) || (rc = ensureSlotArrays(ctx, q, slots)))
            return rc;
        for (int k = 0; k < ctx->ncomp; k++) {
            std::vector<unsigned char> comp(slots * ctx->compBytes[k]);
            if (!readAll(fc.f, comp.data(), comp.size())) return fail(ctx, PICA_ERR_INVALID, "truncated checkpoint");
            CK(cudaMemcpy(S.buf[0][k], comp.data(), comp.size(), cudaMemcpyHostToDevice));
        }
        CK(cudaMemcpy(S.d_start, start.data(), n * 8, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(S.d_cap, cap.data(), n * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(S.d_count, count.data(), n * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(S.d_alive, alive.data(), n * 4, cudaMemcpyHostToDevice));
        S.h_start.swap(start);
        S.h_cap.swap(cap);
        S.layoutSlots = slots;
    }
    ctx->cur = 0;
    ctx->steps = h.steps;
    ctx->epoch++;
    ctx->kmax = h.kmax;
    ctx->jfrac = h.jfrac;
    ctx->tileSplit = h.tileSplit;
    for (auto p : ctx->jacc) CK(cudaMemset(p, 0, nodes * 8));
    return PICA_OK;
}

}  // extern "C"
