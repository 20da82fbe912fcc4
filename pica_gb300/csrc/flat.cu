// Flat particle arrays: the GPU form of pica's EnsembleOrdered / EnsembleUnordered
// (particles/EnsembleOrdered.h, particles/EnsembleUnordered.h), which keep one flat
// array of particles instead of supercells.
//
// * pica_order_by_position: EnsembleOrdered::reorder (EnsembleOrdered.h:61-71)
//   sorts the array lexicographically by position.  Here: a stable least-significant-
//   digit radix sort of an index array, 8 bits per pass, over order-preserving 64-bit
//   images of the coordinates (z first, x last), so that the result is the (x, y, z)
//   lexicographic order with ties in input order.  For each coordinate the images are
//   gathered through the index once and then sorted together with it, so the passes
//   read and write both arrays in order.
// * pica_push_flat: one thread per particle of a flat array, in any order: pica's
//   grid-level FieldInterpolatorCIC<YeeGrid<Three>> (fieldInterpolation/
//   FieldInterpolatorYeeGrid.h:23-38, 137-183) gathers from the periodic device grid,
//   BorisPusher moves the particle (particlePush/BorisPusher.h:33-47), and pica's
//   grid-level CurrentDepositorCIC<YeeGrid<Three>> (currentDeposition/
//   CurrentDepositorYeeGrid.h:23-38, 126-163) adds the current to the grid with FP64
//   global atomics.  The array order never changes (the unordered layout keeps
//   insertion order), so no migration exists; positions wrap periodically.
#include <algorithm>
#include <vector>

#include "push_kernels.cuh"   // wrapi, stag, tscWeights, boris, kC (device helpers of the FP64 push)

namespace pgb {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;   // elements per tile
constexpr int kSortWarps = kSortThreads / 32;

// Order-preserving image of a double: unsigned comparison of the images equals the
// numeric comparison of the values (negatives: all bits flipped; others: sign bit
// set).  -0.0 is taken as +0.0, as pica's comparator (operator<) treats them.
__device__ __forceinline__ unsigned long long orderImage(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v == 0.0 ? 0.0 : v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// img[i] = the order-preserving image of key[idx[i]].
__global__ void k_gatherImages(const double* key, const int64_t* idx, int64_t n, unsigned long long* img) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) img[i] = orderImage(key[idx[i]]);
}

// hist[d * tiles + t]: elements of tile t with digit d.
__global__ void __launch_bounds__(kSortThreads) k_sortHist(const unsigned long long* img, int64_t n, int shift,
                                                           unsigned* hist, int tiles) {
    __shared__ unsigned h[256];
    h[threadIdx.x] = 0u;
    __syncthreads();
    const int64_t t0 = (int64_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; r++) {
        const int64_t i = t0 + (int64_t)r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(unsigned)(img[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// total[d]: elements with digit d (one block per digit).
__global__ void __launch_bounds__(kSortThreads) k_sortTotals(const unsigned* hist, int tiles, unsigned long long* total) {
    __shared__ unsigned long long part[kSortThreads];
    unsigned long long s = 0;
    const unsigned* row = hist + (int64_t)blockIdx.x * tiles;
    for (int t = threadIdx.x; t < tiles; t += kSortThreads) s += row[t];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int w = kSortThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) total[blockIdx.x] = part[0];
}

// offs[d * tiles + t]: first output position of tile t's elements with digit d, the
// exclusive scan of hist in (digit, tile) order (one block per digit scans its row
// on top of the elements of all smaller digits).
__global__ void __launch_bounds__(kSortThreads) k_sortRowScan(unsigned* hist, int tiles, const unsigned long long* total,
                                                              int64_t* offs) {
    __shared__ unsigned long long carry;
    __shared__ unsigned long long ws[kSortWarps];
    const int d = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        unsigned long long base = 0;
        for (int k = 0; k < d; k++) base += total[k];
        carry = base;
    }
    __syncthreads();
    const unsigned* row = hist + (int64_t)d * tiles;
    int64_t* out = offs + (int64_t)d * tiles;
    for (int t0 = 0; t0 < tiles; t0 += kSortThreads) {
        const int t = t0 + threadIdx.x;
        const unsigned long long v = t < tiles ? row[t] : 0ull;
        unsigned long long x = v;   // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        unsigned long long before = carry;
        for (int k = 0; k < warp; k++) before += ws[k];
        if (t < tiles) out[t] = (int64_t)(before + x - v);
        __syncthreads();
        if (threadIdx.x == kSortThreads - 1) carry = before + x;
        __syncthreads();
    }
}

// Stable scatter: the elements of a tile go to their digit's next positions in
// tile order.  Rounds of kSortThreads elements; in a round the warps take
// consecutive runs of 32, and an element's rank among equal digits is (earlier
// rounds) + (earlier warps of this round) + (earlier lanes of its warp).
__global__ void __launch_bounds__(kSortThreads) k_sortScatter(const unsigned long long* img, const int64_t* idx, int64_t n,
                                                              int shift, const int64_t* offs, int tiles,
                                                              unsigned long long* imgOut, int64_t* out) {
    __shared__ unsigned long long base[256];
    __shared__ unsigned short wc[kSortWarps][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    base[threadIdx.x] = (unsigned long long)offs[(int64_t)threadIdx.x * tiles + blockIdx.x];
    for (int w = 0; w < kSortWarps; w++) wc[w][threadIdx.x] = 0;
    __syncthreads();
    const int64_t t0 = (int64_t)blockIdx.x * kSortTile;
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < kSortItems; r++) {
        const int64_t i = t0 + (int64_t)r * kSortThreads + threadIdx.x;
        const bool valid = i < n;
        const int64_t v = valid ? idx[i] : 0;
        const unsigned long long k = valid ? img[i] : 0ull;
        const unsigned dg = valid ? (unsigned)(k >> shift) & 0xFFu : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, dg);
        const int rank = __popc(peers & lt);
        if (valid && rank == 0) wc[warp][dg] = (unsigned short)__popc(peers);
        __syncthreads();
        // thread t: digit t, prefix over warps
        unsigned run = 0;
        for (int w = 0; w < kSortWarps; w++) {
            const unsigned c = wc[w][threadIdx.x];
            wc[w][threadIdx.x] = (unsigned short)run;
            run += c;
        }
        __syncthreads();
        if (valid) {
            const unsigned long long o = base[dg] + wc[warp][dg] + rank;
            out[o] = v;
            imgOut[o] = k;
        }
        __syncthreads();
        base[threadIdx.x] += run;
        for (int w = 0; w < kSortWarps; w++) wc[w][threadIdx.x] = 0;
        __syncthreads();
    }
}

__global__ void k_iota(int64_t* a, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = i;
}

// ---------------------------------------------------------------------------
// Push of a flat array.
// ---------------------------------------------------------------------------
struct FlatArgs {
    int n[3];
    double h[3], invh[3], L[3], dt;
    double no[3], nos[3];   // pica's normalizedOrigin and normalizedOriginStaggered of the grid
    int guard[3];           // pica grid node g is device node g - guard (periodic)
    const double* eb[6];
    double* j[3];
    double norm;            // 1 / (hx hy hz)
    double ec[kMaxSpecies], q[kMaxSpecies];
    int nspecies;
    int* flags;
};

__device__ __forceinline__ int64_t nodeAt(const FlatArgs& a, int gx, int gy, int gz) {
    return ((int64_t)gx * a.n[1] + gy) * a.n[2] + gz;
}

// The 8 wrapped device nodes of a CIC stencil at pica grid node b.
__device__ __forceinline__ void cicNodes(const FlatArgs& a, const int* b, int64_t* o) {
    int lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        lo[d] = wrapi(b[d] - a.guard[d], a.n[d]);
        hi[d] = lo[d] + 1 == a.n[d] ? 0 : lo[d] + 1;
    }
    o[0] = nodeAt(a, lo[0], lo[1], lo[2]); o[1] = nodeAt(a, lo[0], lo[1], hi[2]);
    o[2] = nodeAt(a, lo[0], hi[1], lo[2]); o[3] = nodeAt(a, lo[0], hi[1], hi[2]);
    o[4] = nodeAt(a, hi[0], lo[1], lo[2]); o[5] = nodeAt(a, hi[0], lo[1], hi[2]);
    o[6] = nodeAt(a, hi[0], hi[1], lo[2]); o[7] = nodeAt(a, hi[0], hi[1], hi[2]);
}

// pica's getIndexCoeff (FieldInterpolatorYeeGrid.h:29-38, CurrentDepositorYeeGrid.h:29-38).
__device__ __forceinline__ void indexCoeff(const FlatArgs& a, const double* pos, int* ic, double* cc, int* is, double* cs) {
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double np = pos[d] * a.invh[d];
        double in = np - a.no[d];
        ic[d] = (int)in; cc[d] = in - (double)ic[d];
        in = np - a.nos[d];
        is[d] = (int)in; cs[d] = in - (double)is[d];
    }
}

template <int SHAPE>
__global__ void __launch_bounds__(256) k_push_flat(const __grid_constant__ FlatArgs a, int64_t np_, double* x, double* y,
                                                   double* z, double* ux, double* uy, double* uz, const double* w,
                                                   const int32_t* species) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np_) return;
    const int sp = species ? species[i] : 0;
    if (sp < 0 || sp >= a.nspecies) { atomicExch(a.flags, PICA_ERR_INVALID); return; }
    const double pos[3] = {x[i], y[i], z[i]};
    double u[3] = {ux[i], uy[i], uz[i]};
    const double wgt = w[i];
    double eb6[6];
    if constexpr (SHAPE == PICA_SHAPE_CIC) {
        int ic[3], is[3];
        double cc[3], cs[3];
        indexCoeff(a, pos, ic, cc, is, cs);
#pragma unroll
        for (int comp = 0; comp < 6; comp++) {
            int b[3]; double c[3];
#pragma unroll
            for (int d = 0; d < 3; d++) {
                b[d] = stag(comp, d) ? is[d] : ic[d];
                c[d] = stag(comp, d) ? cs[d] : cc[d];
            }
            int64_t o[8];
            cicNodes(a, b, o);
            const double* f = a.eb[comp];
            // FieldInterpolatorYeeGrid.h:172-181, same term order.
            eb6[comp] = f[o[0]] * (1.0 - c[0]) * (1.0 - c[1]) * (1.0 - c[2]) + f[o[1]] * (1.0 - c[0]) * (1.0 - c[1]) * c[2] +
                        f[o[2]] * (1.0 - c[0]) * c[1] * (1.0 - c[2]) + f[o[3]] * (1.0 - c[0]) * c[1] * c[2] +
                        f[o[4]] * c[0] * (1.0 - c[1]) * (1.0 - c[2]) + f[o[5]] * c[0] * (1.0 - c[1]) * c[2] +
                        f[o[6]] * c[0] * c[1] * (1.0 - c[2]) + f[o[7]] * c[0] * c[1] * c[2];
        }
    } else {
        // TSC (quadratic B-spline; no pica counterpart): nodes nearest to the position.
        int nc[3], ns[3];
        double wc[3][3], ws[3][3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const double xi = pos[d] * a.invh[d];
            nc[d] = (int)floor(xi + 0.5); tscWeights(xi - (double)nc[d], wc[d]);
            const double xs = xi - 0.5;
            ns[d] = (int)floor(xs + 0.5); tscWeights(xs - (double)ns[d], ws[d]);
        }
#pragma unroll
        for (int comp = 0; comp < 6; comp++) {
            const double* f = a.eb[comp];
            int gi[3][3];
#pragma unroll
            for (int d = 0; d < 3; d++)
#pragma unroll
                for (int k = 0; k < 3; k++) gi[d][k] = wrapi((stag(comp, d) ? ns[d] : nc[d]) - 1 + k, a.n[d]);
            const double* wx = stag(comp, 0) ? ws[0] : wc[0];
            const double* wy = stag(comp, 1) ? ws[1] : wc[1];
            const double* wz = stag(comp, 2) ? ws[2] : wc[2];
            double r = 0.0;
#pragma unroll
            for (int p = 0; p < 3; p++) {
                double ry = 0.0;
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    double rz = 0.0;
#pragma unroll
                    for (int k = 0; k < 3; k++) rz += wz[k] * f[nodeAt(a, gi[0][p], gi[1][q], gi[2][k])];
                    ry += wy[q] * rz;
                }
                r += wx[p] * ry;
            }
            eb6[comp] = r;
        }
    }
    const double ig = boris<double>(a.ec[sp], eb6, u);
    double v[3], np[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        v[d] = (u[d] * kC) * ig;          // ParticleArray.h:263
        np[d] = pos[d] + v[d] * a.dt;     // BorisPusher.h:44-46
    }
    // Current at the new position: pica's grid-level deposit of the current
    // v (q w) / (hx hy hz) (CurrentDepositorYeeGrid.h:142-162, same factor order).
    const double qw = a.q[sp] * wgt;
    const double cur[3] = {(v[0] * qw) * a.norm, (v[1] * qw) * a.norm, (v[2] * qw) * a.norm};
    if constexpr (SHAPE == PICA_SHAPE_CIC) {
        int ic[3], is[3];
        double cc[3], cs[3];
        indexCoeff(a, np, ic, cc, is, cs);
#pragma unroll
        for (int comp = 0; comp < 3; comp++) {
            int b[3]; double c[3];
#pragma unroll
            for (int d = 0; d < 3; d++) {
                b[d] = stag(comp, d) ? is[d] : ic[d];
                c[d] = stag(comp, d) ? cs[d] : cc[d];
            }
            int64_t o[8];
            cicNodes(a, b, o);
            double* J = a.j[comp];
            const double vv = cur[comp];
            atomicAdd(J + o[0], (1.0 - c[0]) * (1.0 - c[1]) * (1.0 - c[2]) * vv);
            atomicAdd(J + o[1], (1.0 - c[0]) * (1.0 - c[1]) * c[2] * vv);
            atomicAdd(J + o[2], (1.0 - c[0]) * c[1] * (1.0 - c[2]) * vv);
            atomicAdd(J + o[3], (1.0 - c[0]) * c[1] * c[2] * vv);
            atomicAdd(J + o[4], c[0] * (1.0 - c[1]) * (1.0 - c[2]) * vv);
            atomicAdd(J + o[5], c[0] * (1.0 - c[1]) * c[2] * vv);
            atomicAdd(J + o[6], c[0] * c[1] * (1.0 - c[2]) * vv);
            atomicAdd(J + o[7], c[0] * c[1] * c[2] * vv);
        }
    } else {
        int nc[3], ns[3];
        double wc[3][3], ws[3][3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const double xi = np[d] * a.invh[d];
            nc[d] = (int)floor(xi + 0.5); tscWeights(xi - (double)nc[d], wc[d]);
            const double xs = xi - 0.5;
            ns[d] = (int)floor(xs + 0.5); tscWeights(xs - (double)ns[d], ws[d]);
        }
#pragma unroll
        for (int comp = 0; comp < 3; comp++) {
            double* J = a.j[comp];
            const double* wx = stag(comp, 0) ? ws[0] : wc[0];
            const double* wy = stag(comp, 1) ? ws[1] : wc[1];
            const double* wz = stag(comp, 2) ? ws[2] : wc[2];
#pragma unroll
            for (int p = 0; p < 3; p++) {
                const int gx = wrapi((stag(comp, 0) ? ns[0] : nc[0]) - 1 + p, a.n[0]);
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    const int gy = wrapi((stag(comp, 1) ? ns[1] : nc[1]) - 1 + q, a.n[1]);
                    const double wxy = wx[p] * wy[q];
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        const int gz = wrapi((stag(comp, 2) ? ns[2] : nc[2]) - 1 + k, a.n[2]);
                        atomicAdd(J + nodeAt(a, gx, gy, gz), wxy * wz[k] * cur[comp]);
                    }
                }
            }
        }
    }
    // Periodic wrap, as the supercell layout's migration does.
#pragma unroll
    for (int d = 0; d < 3; d++) {
        if (np[d] < 0.0) np[d] += a.L[d];
        if (np[d] >= a.L[d]) np[d] -= a.L[d];
    }
    x[i] = np[0]; y[i] = np[1]; z[i] = np[2];
    ux[i] = u[0]; uy[i] = u[1]; uz[i] = u[2];
}

}  // namespace

int orderByPosition(int64_t n, int dims, const double* const* key, int64_t* order, cudaStream_t s) {
    if (n <= 0) return 0;
    const int tiles = (int)((n + kSortTile - 1) / kSortTile);
    int64_t* tmp = nullptr;
    unsigned long long* img[2] = {nullptr, nullptr};
    unsigned* hist = nullptr;
    int64_t* offs = nullptr;
    unsigned long long* total = nullptr;
    cudaError_t e = cudaMalloc(&tmp, (size_t)n * 8);
    if (e == cudaSuccess) e = cudaMalloc(&img[0], (size_t)n * 8);
    if (e == cudaSuccess) e = cudaMalloc(&img[1], (size_t)n * 8);
    if (e == cudaSuccess) e = cudaMalloc(&hist, (size_t)256 * tiles * 4);
    if (e == cudaSuccess) e = cudaMalloc(&offs, (size_t)256 * tiles * 8);
    if (e == cudaSuccess) e = cudaMalloc(&total, 256 * 8);
    if (e == cudaSuccess) {
        const unsigned blocks = (unsigned)((n + 255) / 256);
        k_iota<<<blocks, 256, 0, s>>>(order, n);
        // Least significant first: z, then y, then x; 8 passes of 8 bits per coordinate,
        // an even count, so every coordinate's passes end with the index back in `order`.
        for (int d = dims - 1; d >= 0; d--) {
            k_gatherImages<<<blocks, 256, 0, s>>>(key[d], order, n, img[0]);
            int64_t* src = order;
            int64_t* dst = tmp;
            unsigned long long* isrc = img[0];
            unsigned long long* idst = img[1];
            for (int shift = 0; shift < 64; shift += 8) {
                k_sortHist<<<tiles, kSortThreads, 0, s>>>(isrc, n, shift, hist, tiles);
                k_sortTotals<<<256, kSortThreads, 0, s>>>(hist, tiles, total);
                k_sortRowScan<<<256, kSortThreads, 0, s>>>(hist, tiles, total, offs);
                k_sortScatter<<<tiles, kSortThreads, 0, s>>>(isrc, src, n, shift, offs, tiles, idst, dst);
                std::swap(src, dst);
                std::swap(isrc, idst);
            }
        }
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    cudaFree(tmp); cudaFree(img[0]); cudaFree(img[1]); cudaFree(hist); cudaFree(offs); cudaFree(total);
    return (int)e;
}

int launchPushFlat(const pica_config& c, void* const* f, int guard, int64_t n, double* const* xu, const double* w,
                   const int32_t* species, int* flags, cudaStream_t s) {
    FlatArgs a{};
    for (int d = 0; d < 3; d++) {
        a.n[d] = c.n[d];
        a.h[d] = c.h[d];
        a.invh[d] = 1.0 / c.h[d];   // inverse(grid.getStep())
        a.L[d] = (double)c.n[d] * c.h[d];
        a.no[d] = (-(double)guard * c.h[d]) / c.h[d];   // grid.getOrigin() / grid.getStep(), origin = -guard h
        a.nos[d] = a.no[d] + 0.5;
        a.guard[d] = guard;
    }
    a.dt = c.dt;
    for (int k = 0; k < 6; k++) a.eb[k] = static_cast<const double*>(f[k]);
    for (int k = 0; k < 3; k++) a.j[k] = static_cast<double*>(f[6 + k]);
    a.norm = 1.0 / (c.h[0] * c.h[1] * c.h[2]);
    a.nspecies = c.nspecies;
    for (int q = 0; q < c.nspecies; q++) {
        a.ec[q] = c.charge[q] * c.dt / (2.0 * c.mass[q] * kC);   // BorisPusher.h:29
        a.q[q] = c.charge[q];
    }
    a.flags = flags;
    if (n <= 0) return 0;
    if (n > (int64_t)0x7fffffff * 256) return (int)cudaErrorInvalidValue;
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (c.shape == PICA_SHAPE_TSC)
        k_push_flat<PICA_SHAPE_TSC><<<grid, 256, 0, s>>>(a, n, xu[0], xu[1], xu[2], xu[3], xu[4], xu[5], w, species);
    else
        k_push_flat<PICA_SHAPE_CIC><<<grid, 256, 0, s>>>(a, n, xu[0], xu[1], xu[2], xu[3], xu[4], xu[5], w, species);
    return (int)cudaGetLastError();
}

}  // namespace pgb
