// Fused supercell kernel (field gather + Boris push + current deposit + migration
// partition) and the migration kernels.  Included by push_fp64.cu and by
// push_fp32.cu, both built with --fmad=false, so FP64 arithmetic rounds exactly
// as pica's C++ does.
//
// One CTA owns one supercell.  It stages the E/B tile of nodes [m-2, m+S+3)
// per dimension (periodic) into shared memory -- the GPU form of pica's
// FieldInterpolatorCICSupercell / CurrentDepositorCICSupercell pair
// (fieldInterpolation/FieldInterpolatorYeeGrid.h:188-283,
//  currentDeposition/CurrentDepositorYeeGrid.h:168-264).  The FP32 form
// accumulates the supercell's current in a shared-memory tile of the same extent
// (exact fixed point in split 32-bit words, native integer shared-memory
// atomics) and adds it to the global accumulators once at the end; the FP64 form
// adds every contribution to the global current with FP64 atomics, which run in
// L2 (a shared FP64 tile would spend the SM's low FP64 rate on its sums).
#pragma once

#include <cstdint>
#include <type_traits>

#include "pica_internal.h"

namespace pgb {

constexpr double kC = 29979245800.0;  // pica math/Constants.h:11
constexpr double kThird = 1.0 / 3.0;

__device__ __forceinline__ int wrapi(int a, int n) {
    a %= n;
    return a < 0 ? a + n : a;
}

// Yee staggering: bit d set when the component sits at a half-integer node
// along dimension d.  Ex(i,j+1/2,k+1/2) Ey(i+1/2,j,k+1/2) Ez(i+1/2,j+1/2,k)
// Bx(i+1/2,j,k) By(i,j+1/2,k) Bz(i,j,k+1/2)  (grid/YeeGrid.h:11-14,336-344).
__device__ __forceinline__ bool stag(int comp, int d) {
    const int mask[6] = {6, 5, 3, 1, 2, 4};
    return (mask[comp] >> d) & 1;
}

template <typename R>
__device__ __forceinline__ void tscWeights(R d, R* w) {
    const R h = R(0.5);
    w[0] = h * (h - d) * (h - d);
    w[1] = R(0.75) - d * d;
    w[2] = h * (h + d) * (h + d);
}

// Current tiles in shared memory.  FP32 form: each node keeps the exact
// integer (fixed-point) sum split into a low part (the low L bits of every
// contribution, summed as unsigned 32-bit) and a high part (the rest, summed
// as signed 32-bit), both with native 32-bit shared-memory atomics; L and the
// fraction bits are chosen so that neither part can overflow for the largest
// supercell (see the host).  The 64-bit node sum is hi * 2^L + lo.  Integer
// sums are exact, so the result does not depend on the order of the adds.
// FP64 form: plain FP64 adds, so the FP64 result differs from pica's only by
// the order of the sums.
struct FixTile {
    unsigned int* lo;
    int* hi;
    int L;       // low-part bits, 1..23
    float up;    // 2^L
    float down;  // 2^-L
    __device__ __forceinline__ void setSplit(int bits) {
        L = bits;
        up = __int_as_float((127 + bits) << 23);
        down = __int_as_float((127 - bits) << 23);
    }
    // Adds v = round-to-nearest-even(scaled) as hi*2^L + lo, lo in [0, 2^L), with
    // 32-bit operations only (a 64-bit float-to-integer conversion runs on the
    // FP64 pipe, which is narrow on this part).  r = rint(scaled) is an integer
    // m*2^e with |m| < 2^24; h = floor(r 2^-L) is exact, and r - h 2^L is a
    // multiple of 2^e below 2^L <= 2^23, hence exact in FP32 and recovered from
    // the mantissa of (l + 2^23).  A zero adds zeros: no test for it (the branch
    // around the two atomics cost more than the rare zero's atomics: two-stream push
    // 47.2 -> 46.1 ms without it).
    __device__ __forceinline__ void add(int idx, float scaled) const {
        const float r = rintf(scaled);
        const float h = floorf(r * down);
        const float l = fmaf(-h, up, r);
        atomicAdd(lo + idx, __float_as_uint(l + 8388608.0f) - 0x4B000000u);
        atomicAdd(hi + idx, __float2int_rz(h));
    }
    __device__ __forceinline__ long long node(int idx) const { return ((long long)hi[idx] << L) + (long long)lo[idx]; }
};
// Deposit target of the FP64 plain form: the global current itself, added to with
// FP64 atomics (performed in L2; the SM's FP64 rate is low, and a shared tile's
// segmented sums spend it).  Tile coordinates (x, y, z) of component c are grid
// nodes o + (x, y, z), within one period of the grid (wrapped once).
struct GlobalJ {
    double* j[3];
    int o[3], n[3];
    double norm;   // 1 / (hx hy hz), applied to every term
};
// Add v to component c at tile node (x, y, z) (linear index c TT + (x T1 + y) T2 + z
// for the shared tiles).
template <class Tile>
__device__ __forceinline__ void depositAt(const Tile& t, int TT, int T1, int T2, int c, int x, int y, int z,
                                          float v) {
    t.add(c * TT + (x * T1 + y) * T2 + z, v);
}
__device__ __forceinline__ void depositAt(const GlobalJ& g, int, int, int, int c, int x, int y, int z, double v) {
    if (v == 0.0) return;
    auto near = [](int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); };
    const int gx = near(g.o[0] + x, g.n[0]), gy = near(g.o[1] + y, g.n[1]), gz = near(g.o[2] + z, g.n[2]);
    atomicAdd(g.j[c] + ((int64_t)gx * g.n[1] + gy) * g.n[2] + gz, v * g.norm);
}

// Separable W^3-point gather: sum_i wx_i sum_j wy_j (sum_k wz_k F), left to right.
template <typename R, int W>
__device__ __forceinline__ R gatherSep(const R* tile, int T1, int T2, const int* t0, const R* wx, const R* wy,
                                       const R* wz) {
    R r = R(0);
#pragma unroll
    for (int i = 0; i < W; i++) {
        R ry = R(0);
#pragma unroll
        for (int j = 0; j < W; j++) {
            const R* row = tile + ((t0[0] + i) * T1 + (t0[1] + j)) * T2 + t0[2];
            R rz = row[0] * wz[0];
#pragma unroll
            for (int k = 1; k < W; k++) rz = rz + row[k] * wz[k];
            ry = ry + wy[j] * rz;
        }
        r = r + wx[i] * ry;
    }
    return r;
}

template <typename R, int W, typename Tile>
__device__ __forceinline__ void scatterSep(const Tile& tile, int TT, int c, int T1, int T2, const int* t0, const R* wx,
                                           const R* wy, const R* wz, R v) {
#pragma unroll
    for (int i = 0; i < W; i++)
#pragma unroll
        for (int j = 0; j < W; j++) {
            R vij = (v * wx[i]) * wy[j];
#pragma unroll
            for (int k = 0; k < W; k++) depositAt(tile, TT, T1, T2, c, t0[0] + i, t0[1] + j, t0[2] + k, vij * wz[k]);
        }
}

// pica's CIC 8-point interpolation, FieldInterpolatorYeeGrid.h:272-280 (same term order).
__device__ __forceinline__ double cicGatherRef(const double* t, int T1, int T2, const int* b, const double* c) {
    const double* p = t + (b[0] * T1 + b[1]) * T2 + b[2];
    const int sy = T2, sx = T1 * T2;
    const double cx = c[0], cy = c[1], cz = c[2];
    return p[0] * (1.0 - cx) * (1.0 - cy) * (1.0 - cz) + p[1] * (1.0 - cx) * (1.0 - cy) * cz +
           p[sy] * (1.0 - cx) * cy * (1.0 - cz) + p[sy + 1] * (1.0 - cx) * cy * cz +
           p[sx] * cx * (1.0 - cy) * (1.0 - cz) + p[sx + 1] * cx * (1.0 - cy) * cz +
           p[sx + sy] * cx * cy * (1.0 - cz) + p[sx + sy + 1] * cx * cy * cz;
}
// pica's CIC 8-point deposit (CurrentDepositorYeeGrid.h:254-261, same factor order)
// straight into the global current with FP64 atomics (performed in L2): nodes of
// tile index b (tile origin o, periodic grid n), each term multiplied by norm
// (1 / h^3) on its own.
__device__ __forceinline__ void cicScatterGlobal(double* J, const int* o, const int* n, const int* b, const double* c,
                                                 double v, double norm) {
    int lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        lo[d] = wrapi(o[d] + b[d], n[d]);
        hi[d] = lo[d] + 1 == n[d] ? 0 : lo[d] + 1;
    }
    auto at = [&](int x, int y, int z) { return J + ((int64_t)x * n[1] + y) * n[2] + z; };
    const double cx = c[0], cy = c[1], cz = c[2];
    atomicAdd(at(lo[0], lo[1], lo[2]), (1.0 - cx) * (1.0 - cy) * (1.0 - cz) * v * norm);
    atomicAdd(at(lo[0], lo[1], hi[2]), (1.0 - cx) * (1.0 - cy) * cz * v * norm);
    atomicAdd(at(lo[0], hi[1], lo[2]), (1.0 - cx) * cy * (1.0 - cz) * v * norm);
    atomicAdd(at(lo[0], hi[1], hi[2]), (1.0 - cx) * cy * cz * v * norm);
    atomicAdd(at(hi[0], lo[1], lo[2]), cx * (1.0 - cy) * (1.0 - cz) * v * norm);
    atomicAdd(at(hi[0], lo[1], hi[2]), cx * (1.0 - cy) * cz * v * norm);
    atomicAdd(at(hi[0], hi[1], lo[2]), cx * cy * (1.0 - cz) * v * norm);
    atomicAdd(at(hi[0], hi[1], hi[2]), cx * cy * cz * v * norm);
}

// Boris rotation of BorisPusher.h:33-43 on normalised momentum u; returns 1/gamma
// of the new u as ParticleArraySoA::setP does (ParticleArray.h:311-317).
template <typename R>
__device__ __forceinline__ R boris(R ec, const R* eb, R* u) {
    const R em[3] = {eb[0] * ec, eb[1] * ec, eb[2] * ec};
    const R um[3] = {u[0] + em[0], u[1] + em[1], u[2] + em[2]};
    const R tc = ec / sqrt(R(1) + (um[0] * um[0] + um[1] * um[1] + um[2] * um[2]));
    const R t[3] = {eb[3] * tc, eb[4] * tc, eb[5] * tc};
    const R up[3] = {um[0] + (um[1] * t[2] - um[2] * t[1]), um[1] + (um[2] * t[0] - um[0] * t[2]),
                     um[2] + (um[0] * t[1] - um[1] * t[0])};
    const R sc = R(2) / (R(1) + (t[0] * t[0] + t[1] * t[1] + t[2] * t[2]));
    const R s[3] = {t[0] * sc, t[1] * sc, t[2] * sc};
    u[0] = um[0] + (up[1] * s[2] - up[2] * s[1]) + em[0];
    u[1] = um[1] + (up[2] * s[0] - up[0] * s[2]) + em[1];
    u[2] = um[2] + (up[0] * s[1] - up[1] * s[0]) + em[2];
    return R(1) / sqrt(R(1) + (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
}

// Esirkepov (CPC 135 (2001) 144, eqs. 21-23) on pica's dual Yee lattice: rho at
// cell centres, J on faces.  s0/s1: old/new shape in an NW-node window of the
// rho lattice starting at tile index b; k: -(q w) h_d / dt.  Jx of the face
// between window nodes i and i+1 is pica Jx node b_x + i + 1.
template <typename R, int NW, typename Tile>
__device__ __forceinline__ void esirkepov(const Tile& jt, int TT, int T1, int T2, const int* b, const R (*s0)[NW],
                                          const R (*s1)[NW], const R* k) {
    R ds[3][NW];
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
        for (int i = 0; i < NW; i++) ds[d][i] = s1[d][i] - s0[d][i];
    const R hf = R(0.5), th = R(kThird);
#pragma unroll
    for (int j = 0; j < NW; j++)
#pragma unroll
        for (int l = 0; l < NW; l++) {
            const R yz = s0[1][j] * s0[2][l] + hf * (ds[1][j] * s0[2][l] + s0[1][j] * ds[2][l]) + th * (ds[1][j] * ds[2][l]);
            R acc = R(0);
#pragma unroll
            for (int i = 0; i < NW - 1; i++) {
                acc = acc + ds[0][i] * yz;
                depositAt(jt, TT, T1, T2, 0, b[0] + i + 1, b[1] + j, b[2] + l, acc * k[0]);
            }
        }
#pragma unroll
    for (int i = 0; i < NW; i++)
#pragma unroll
        for (int l = 0; l < NW; l++) {
            const R xz = s0[0][i] * s0[2][l] + hf * (ds[0][i] * s0[2][l] + s0[0][i] * ds[2][l]) + th * (ds[0][i] * ds[2][l]);
            R acc = R(0);
#pragma unroll
            for (int j = 0; j < NW - 1; j++) {
                acc = acc + ds[1][j] * xz;
                depositAt(jt, TT, T1, T2, 1, b[0] + i, b[1] + j + 1, b[2] + l, acc * k[1]);
            }
        }
#pragma unroll
    for (int i = 0; i < NW; i++)
#pragma unroll
        for (int j = 0; j < NW; j++) {
            const R xy = s0[0][i] * s0[1][j] + hf * (ds[0][i] * s0[1][j] + s0[0][i] * ds[1][j]) + th * (ds[0][i] * ds[1][j]);
            R acc = R(0);
#pragma unroll
            for (int l = 0; l < NW - 1; l++) {
                acc = acc + ds[2][l] * xy;
                depositAt(jt, TT, T1, T2, 2, b[0] + i, b[1] + j, b[2] + l + 1, acc * k[2]);
            }
        }
}

// s[lo - base + k] = w[k] in an NW window, written with selects so s stays in registers.
template <typename R, int NW, int P>
__device__ __forceinline__ void placeShape(R* s, int lo, int base, const R* w) {
    const int off = lo - base;
#pragma unroll
    for (int i = 0; i < NW; i++) {
        R v = R(0);
#pragma unroll
        for (int k = 0; k < P; k++) v = (i - off == k) ? w[k] : v;
        s[i] = v;
    }
}

// Direction code of a supercell move, (dx+1)*9 + (dy+1)*3 + (dz+1); 13 = stay.
__device__ __forceinline__ int dirCode(const int* o, const int* nw, const int* nsc, bool& bad) {
    int code = 0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        int ds = nw[d] - o[d];
        if (ds > 1) ds -= nsc[d];
        if (ds < -1) ds += nsc[d];
        if (ds < -1 || ds > 1) { bad = true; ds = 0; }
        code = code * 3 + (ds + 1);
    }
    return code;
}

__device__ __forceinline__ bool aliveAt(const PlainPtrs& p, int64_t i) { return aliveX(p.x[i]); }
__device__ __forceinline__ bool aliveAt(const CellPtrs& p, int64_t i) { return p.cell[i] != kDeadCell; }
__device__ __forceinline__ void killAt(const PlainPtrs& p, int64_t i) { p.x[i] = kDeadX; }
__device__ __forceinline__ void killAt(const CellPtrs& p, int64_t i) { p.cell[i] = kDeadCell; }

__device__ __forceinline__ void copyParticle(const PlainPtrs& s, int64_t i, const PlainPtrs& d, int64_t j) {
    d.x[j] = s.x[i]; d.y[j] = s.y[i]; d.z[j] = s.z[i];
    d.ux[j] = s.ux[i]; d.uy[j] = s.uy[i]; d.uz[j] = s.uz[i]; d.w[j] = s.w[i];
}
__device__ __forceinline__ void copyParticle(const CellPtrs& s, int64_t i, const CellPtrs& d, int64_t j) {
    d.cell[j] = s.cell[i]; d.ox[j] = s.ox[i]; d.oy[j] = s.oy[i]; d.oz[j] = s.oz[i];
    d.ux[j] = s.ux[i]; d.uy[j] = s.uy[i]; d.uz[j] = s.uz[i]; d.w[j] = s.w[i];
}

// ---------------------------------------------------------------------------
// Fused push kernel.
// ---------------------------------------------------------------------------
template <bool PLAIN, int SHAPE, int DEP>
__global__ void __launch_bounds__(kPushThreads)
k_push(const __grid_constant__ PushArgs<typename std::conditional<PLAIN, PlainPtrs, CellPtrs>::type> a) {
    using R = typename std::conditional<PLAIN, double, float>::type;
    using P = typename std::conditional<PLAIN, PlainPtrs, CellPtrs>::type;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_nleave;

    const int T1 = a.T[1], T2 = a.T[2], TT = a.T[0] * T1 * T2;
    // FP32: J tile (3 components x TT nodes) then the E/B tile (6 x TT).  FP64: the
    // E/B tile only (the current goes straight to the global arrays, GlobalJ).
    FixTile jt{};
    R* eb;
    if constexpr (PLAIN) {
        eb = reinterpret_cast<R*>(smem_raw);
    } else {
        jt.lo = reinterpret_cast<unsigned int*>(smem_raw);
        jt.hi = reinterpret_cast<int*>(jt.lo + 3 * TT);
        jt.setSplit(a.tileSplit);
        eb = reinterpret_cast<R*>(jt.hi + 3 * TT);
    }
    const int s = blockIdx.x;
    int sc[3];
    sc[2] = s % a.nsc[2];
    sc[1] = (s / a.nsc[2]) % a.nsc[1];
    sc[0] = s / (a.nsc[1] * a.nsc[2]);
    const int m[3] = {sc[0] * a.S[0], sc[1] * a.S[1], sc[2] * a.S[2]};
    // Stage the E/B tile (periodic) and clear the FP32 J tile.
    for (int t = threadIdx.x; t < 6 * TT; t += blockDim.x) {
        const int c = t / TT, r = t - c * TT;
        const int i = r / (T1 * T2), jj = (r / T2) % T1, k = r % T2;
        const int gx = wrapi(m[0] - kG + i, a.n[0]), gy = wrapi(m[1] - kG + jj, a.n[1]), gz = wrapi(m[2] - kG + k, a.n[2]);
        eb[t] = static_cast<const R*>(a.eb[c])[((int64_t)gx * a.n[1] + gy) * a.n[2] + gz];
    }
    if constexpr (!PLAIN)   // the FP64 form deposits straight into the global current (GlobalJ)
        for (int t = threadIdx.x; t < 3 * TT; t += blockDim.x) { jt.lo[t] = 0u; jt.hi[t] = 0; }

    // pica supercell index math (FieldInterpolatorYeeGrid.h:197-205): tile index t of
    // the reference maps to node trunc(minPos/h) - 1 + t, i.e. our tile index t + off.
    double no[3], nos[3];
    int off[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double minPos = (double)m[d] * a.h[d];
        no[d] = (minPos - a.h[d]) / a.h[d];
        nos[d] = no[d] + 0.5;
        off[d] = ((int)(minPos / a.h[d]) - 1) - (m[d] - kG);
    }
    const R invU = (R)a.invUnit;
    // FP64 plain form: the current goes straight to the global arrays (GlobalJ).
    GlobalJ gj{};
    if constexpr (PLAIN) {
        for (int d = 0; d < 3; d++) {
            gj.j[d] = static_cast<double*>(a.j[d]);
            gj.o[d] = m[d] - kG;
            gj.n[d] = a.n[d];
        }
        gj.norm = a.norm;
    }
    bool bad = false;
    __syncthreads();

    for (int spi = 0; spi < a.nspecies; spi++) {
        const SpeciesArgs<P>& sa = a.sp[spi];
        const int64_t start = sa.start[s];
        const int count = sa.count[s];
        const R ec = (R)sa.ec;
        if (threadIdx.x == 0) s_nleave = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < count; i += blockDim.x) {
            const int64_t slot = start + i;
            if (!aliveAt(sa.buf, slot)) continue;
            int code = 13;
            R nu[3];
            double npos[3];
            uint32_t ncell = 0;
            float no3[3];
            {
                R u[3], eb6[6], wgt;
                if constexpr (PLAIN) {
                    const double pos[3] = {sa.buf.x[slot], sa.buf.y[slot], sa.buf.z[slot]};
                    u[0] = sa.buf.ux[slot]; u[1] = sa.buf.uy[slot]; u[2] = sa.buf.uz[slot];
                    wgt = sa.buf.w[slot];
                    if constexpr (SHAPE == PICA_SHAPE_CIC) {
                        int ic[3], is[3];
                        double cc[3], cs[3];
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            const double np = pos[d] * a.invh[d];
                            double in = np - no[d];
                            ic[d] = (int)in; cc[d] = in - (double)ic[d];
                            in = np - nos[d];
                            is[d] = (int)in; cs[d] = in - (double)is[d];
                        }
#pragma unroll
                        for (int comp = 0; comp < 6; comp++) {
                            int b[3]; double w[3];
#pragma unroll
                            for (int d = 0; d < 3; d++) {
                                b[d] = (stag(comp, d) ? is[d] : ic[d]) + off[d];
                                w[d] = stag(comp, d) ? cs[d] : cc[d];
                            }
                            eb6[comp] = cicGatherRef(eb + comp * TT, T1, T2, b, w);
                        }
                    } else {
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
                            int t0[3];
#pragma unroll
                            for (int d = 0; d < 3; d++) t0[d] = (stag(comp, d) ? ns[d] : nc[d]) - 1 - (m[d] - kG);
                            eb6[comp] = gatherSep<double, 3>(eb + comp * TT, T1, T2, t0, stag(comp, 0) ? ws[0] : wc[0],
                                                             stag(comp, 1) ? ws[1] : wc[1], stag(comp, 2) ? ws[2] : wc[2]);
                        }
                    }
                    const R ig = boris<R>(ec, eb6, u);
                    double v[3], np[3];
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        v[d] = (u[d] * kC) * ig;           // ParticleArray.h:263
                        np[d] = pos[d] + v[d] * a.dt;      // BorisPusher.h:44-46
                    }
                    // The deposit stencils stay inside the tile while the new position is
                    // within one cell of the supercell; anything else (a non-finite state or
                    // a time step far above the Courant limit) is reported, not deposited.
                    bool inRange = true;
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        const double rel = np[d] * a.invh[d] - (double)m[d];
                        inRange = inRange && rel >= -1.0 && rel < (double)(a.S[d] + 1) &&
                                  fabs(np[d] - pos[d]) * a.invh[d] < 1.0;
                    }
                    if (!inRange) {
                        bad = true;
                    } else if constexpr (DEP == PICA_DEPOSIT_DIRECT) {
                        const double cur[3] = {v[0] * (sa.q * wgt), v[1] * (sa.q * wgt), v[2] * (sa.q * wgt)};
                        if constexpr (SHAPE == PICA_SHAPE_CIC) {
                            int ic[3], is[3];
                            double cc[3], cs[3];
#pragma unroll
                            for (int d = 0; d < 3; d++) {
                                const double npn = np[d] * a.invh[d];
                                double in = npn - no[d];
                                ic[d] = (int)in; cc[d] = in - (double)ic[d];
                                in = npn - nos[d];
                                is[d] = (int)in; cs[d] = in - (double)is[d];
                            }
#pragma unroll
                            for (int comp = 0; comp < 3; comp++) {
                                int b[3]; double w[3];
#pragma unroll
                                for (int d = 0; d < 3; d++) {
                                    b[d] = (stag(comp, d) ? is[d] : ic[d]) + off[d];
                                    w[d] = stag(comp, d) ? cs[d] : cc[d];
                                }
                                cicScatterGlobal(gj.j[comp], gj.o, gj.n, b, w, cur[comp], gj.norm);
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
                                int t0[3];
#pragma unroll
                                for (int d = 0; d < 3; d++) t0[d] = (stag(comp, d) ? ns[d] : nc[d]) - 1 - (m[d] - kG);
                                scatterSep<double, 3>(gj, TT, comp, T1, T2, t0, stag(comp, 0) ? ws[0] : wc[0],
                                                      stag(comp, 1) ? ws[1] : wc[1], stag(comp, 2) ? ws[2] : wc[2], cur[comp]);
                            }
                        }
                    } else {
                        double kq[3];
#pragma unroll
                        for (int d = 0; d < 3; d++) kq[d] = -(sa.q * wgt) * (a.h[d] / a.dt);
                        int b[3];
                        if constexpr (SHAPE == PICA_SHAPE_CIC) {
                            double s0[3][3], s1[3][3];
#pragma unroll
                            for (int d = 0; d < 3; d++) {
                                const double x0 = pos[d] * a.invh[d] - 0.5, x1 = np[d] * a.invh[d] - 0.5;
                                const int n0 = (int)floor(x0), n1 = (int)floor(x1);
                                const double w0[2] = {1.0 - (x0 - n0), x0 - n0}, w1[2] = {1.0 - (x1 - n1), x1 - n1};
                                const int lo = min(n0, n1);
                                placeShape<double, 3, 2>(s0[d], n0, lo, w0);
                                placeShape<double, 3, 2>(s1[d], n1, lo, w1);
                                b[d] = lo - (m[d] - kG);
                            }
                            esirkepov<double, 3>(gj, TT, T1, T2, b, s0, s1, kq);
                        } else {
                            double s0[3][4], s1[3][4];
#pragma unroll
                            for (int d = 0; d < 3; d++) {
                                const double x0 = pos[d] * a.invh[d] - 0.5, x1 = np[d] * a.invh[d] - 0.5;
                                const int n0 = (int)floor(x0 + 0.5), n1 = (int)floor(x1 + 0.5);
                                double w0[3], w1[3];
                                tscWeights(x0 - (double)n0, w0);
                                tscWeights(x1 - (double)n1, w1);
                                const int lo = min(n0, n1) - 1;
                                placeShape<double, 4, 3>(s0[d], n0 - 1, lo, w0);
                                placeShape<double, 4, 3>(s1[d], n1 - 1, lo, w1);
                                b[d] = lo - (m[d] - kG);
                            }
                            esirkepov<double, 4>(gj, TT, T1, T2, b, s0, s1, kq);
                        }
                    }
                    // Periodic wrap and new supercell (EnsembleSupercells.h:54-57, floor, clamped).
                    int nsc3[3];
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        if (!inRange) np[d] = pos[d];
                        if (np[d] < 0.0) np[d] += a.L[d];
                        if (np[d] >= a.L[d]) np[d] -= a.L[d];
                        nsc3[d] = (int)floor((np[d] - 0.0) * a.scInv[d]);
                        nsc3[d] = min(max(nsc3[d], 0), a.nsc[d] - 1);
                        npos[d] = np[d];
                    }
                    code = dirCode(sc, nsc3, a.nsc, bad);
                } else {
                    // FP32 cell form.
                    int c3[3];
                    unpackCell(sa.buf.cell[slot], c3[0], c3[1], c3[2]);
                    const int lc[3] = {c3[0] - m[0], c3[1] - m[1], c3[2] - m[2]};
                    const float o[3] = {sa.buf.ox[slot], sa.buf.oy[slot], sa.buf.oz[slot]};
                    u[0] = sa.buf.ux[slot]; u[1] = sa.buf.uy[slot]; u[2] = sa.buf.uz[slot];
                    wgt = sa.buf.w[slot];
                    if constexpr (SHAPE == PICA_SHAPE_CIC) {
                        int bc[3], bs[3];
                        float wc[3][2], ws[3][2];
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            bc[d] = lc[d] + kG; wc[d][0] = 1.0f - o[d]; wc[d][1] = o[d];
                            const bool hi = o[d] >= 0.5f;
                            const float dd = hi ? o[d] - 0.5f : o[d] + 0.5f;
                            bs[d] = (hi ? lc[d] : lc[d] - 1) + kG; ws[d][0] = 1.0f - dd; ws[d][1] = dd;
                        }
#pragma unroll
                        for (int comp = 0; comp < 6; comp++) {
                            int t0[3];
#pragma unroll
                            for (int d = 0; d < 3; d++) t0[d] = stag(comp, d) ? bs[d] : bc[d];
                            eb6[comp] = gatherSep<float, 2>(eb + comp * TT, T1, T2, t0, stag(comp, 0) ? ws[0] : wc[0],
                                                            stag(comp, 1) ? ws[1] : wc[1], stag(comp, 2) ? ws[2] : wc[2]);
                        }
                    } else {
                        int bc[3], bs[3];
                        float wc[3][3], ws[3][3];
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            const bool hi = o[d] >= 0.5f;
                            bc[d] = lc[d] + (hi ? 1 : 0) - 1 + kG; tscWeights(hi ? o[d] - 1.0f : o[d], wc[d]);
                            bs[d] = lc[d] - 1 + kG; tscWeights(o[d] - 0.5f, ws[d]);
                        }
#pragma unroll
                        for (int comp = 0; comp < 6; comp++) {
                            int t0[3];
#pragma unroll
                            for (int d = 0; d < 3; d++) t0[d] = stag(comp, d) ? bs[d] : bc[d];
                            eb6[comp] = gatherSep<float, 3>(eb + comp * TT, T1, T2, t0, stag(comp, 0) ? ws[0] : wc[0],
                                                            stag(comp, 1) ? ws[1] : wc[1], stag(comp, 2) ? ws[2] : wc[2]);
                        }
                    }
                    const float ig = boris<float>(ec, eb6, u);
                    int ln[3];
                    float on[3];
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        float onew = o[d] + (u[d] * ig) * (float)a.cdth[d];
                        const float fl = floorf(onew);
                        ln[d] = lc[d] + (int)fl;
                        onew = onew - fl;
                        if (onew >= 1.0f) { onew -= 1.0f; ln[d] += 1; }
                        on[d] = onew;
                    }
                    bool inRange = true;
#pragma unroll
                    for (int d = 0; d < 3; d++)
                        inRange = inRange && ln[d] >= -1 && ln[d] <= a.S[d] && abs(ln[d] - lc[d]) <= 1 &&
                                  on[d] >= 0.0f && on[d] < 1.0f;
                    if (!inRange) {
                        bad = true;
#pragma unroll
                        for (int d = 0; d < 3; d++) { ln[d] = lc[d]; on[d] = o[d]; }
                    } else if constexpr (DEP == PICA_DEPOSIT_DIRECT) {
                        const float qcw = (float)sa.qc * wgt * invU;
                        const float cur[3] = {(u[0] * ig) * qcw, (u[1] * ig) * qcw, (u[2] * ig) * qcw};
                        if constexpr (SHAPE == PICA_SHAPE_CIC) {
                            int bc[3], bs[3];
                            float wc[3][2], ws[3][2];
#pragma unroll
                            for (int d = 0; d < 3; d++) {
                                bc[d] = ln[d] + kG; wc[d][0] = 1.0f - on[d]; wc[d][1] = on[d];
                                const bool hi = on[d] >= 0.5f;
                                const float dd = hi ? on[d] - 0.5f : on[d] + 0.5f;
                                bs[d] = (hi ? ln[d] : ln[d] - 1) + kG; ws[d][0] = 1.0f - dd; ws[d][1] = dd;
                            }
#pragma unroll
                            for (int comp = 0; comp < 3; comp++) {
                                int t0[3];
#pragma unroll
                                for (int d = 0; d < 3; d++) t0[d] = stag(comp, d) ? bs[d] : bc[d];
                                scatterSep<float, 2>(jt, TT, comp, T1, T2, t0, stag(comp, 0) ? ws[0] : wc[0],
                                                     stag(comp, 1) ? ws[1] : wc[1], stag(comp, 2) ? ws[2] : wc[2], cur[comp]);
                            }
                        } else {
                            int bc[3], bs[3];
                            float wc[3][3], ws[3][3];
#pragma unroll
                            for (int d = 0; d < 3; d++) {
                                const bool hi = on[d] >= 0.5f;
                                bc[d] = ln[d] + (hi ? 1 : 0) - 1 + kG; tscWeights(hi ? on[d] - 1.0f : on[d], wc[d]);
                                bs[d] = ln[d] - 1 + kG; tscWeights(on[d] - 0.5f, ws[d]);
                            }
#pragma unroll
                            for (int comp = 0; comp < 3; comp++) {
                                int t0[3];
#pragma unroll
                                for (int d = 0; d < 3; d++) t0[d] = stag(comp, d) ? bs[d] : bc[d];
                                scatterSep<float, 3>(jt, TT, comp, T1, T2, t0, stag(comp, 0) ? ws[0] : wc[0],
                                                     stag(comp, 1) ? ws[1] : wc[1], stag(comp, 2) ? ws[2] : wc[2], cur[comp]);
                            }
                        }
                    } else {
                        const float kq[3] = {(float)sa.kq[0] * wgt * invU, (float)sa.kq[1] * wgt * invU,
                                             (float)sa.kq[2] * wgt * invU};
                        int b[3];
                        if constexpr (SHAPE == PICA_SHAPE_CIC) {
                            float s0[3][3], s1[3][3];
#pragma unroll
                            for (int d = 0; d < 3; d++) {
                                const bool h0 = o[d] >= 0.5f, h1 = on[d] >= 0.5f;
                                const int n0 = h0 ? lc[d] : lc[d] - 1, n1 = h1 ? ln[d] : ln[d] - 1;
                                const float d0 = h0 ? o[d] - 0.5f : o[d] + 0.5f, d1 = h1 ? on[d] - 0.5f : on[d] + 0.5f;
                                const float w0[2] = {1.0f - d0, d0}, w1[2] = {1.0f - d1, d1};
                                const int lo = min(n0, n1);
                                placeShape<float, 3, 2>(s0[d], n0, lo, w0);
                                placeShape<float, 3, 2>(s1[d], n1, lo, w1);
                                b[d] = lo + kG;
                            }
                            esirkepov<float, 3>(jt, TT, T1, T2, b, s0, s1, kq);
                        } else {
                            float s0[3][4], s1[3][4];
#pragma unroll
                            for (int d = 0; d < 3; d++) {
                                float w0[3], w1[3];
                                tscWeights(o[d] - 0.5f, w0);
                                tscWeights(on[d] - 0.5f, w1);
                                const int lo = min(lc[d], ln[d]) - 1;
                                placeShape<float, 4, 3>(s0[d], lc[d] - 1, lo, w0);
                                placeShape<float, 4, 3>(s1[d], ln[d] - 1, lo, w1);
                                b[d] = lo + kG;
                            }
                            esirkepov<float, 4>(jt, TT, T1, T2, b, s0, s1, kq);
                        }
                    }
                    int gc[3], nsc3[3];
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        gc[d] = wrapi(m[d] + ln[d], a.n[d]);
                        nsc3[d] = gc[d] / a.S[d];
                        no3[d] = on[d];
                    }
                    ncell = packCell(gc[0], gc[1], gc[2]);
                    code = dirCode(sc, nsc3, a.nsc, bad);
                }
                nu[0] = u[0]; nu[1] = u[1]; nu[2] = u[2];
            }
            // Stayers are updated in place (the weight does not change); a leaver's record
            // goes to the side buffer, packed at start + k (k: its rank of arrival in the
            // leaver list), its slot dies and joins the leaver list.
            const int k = code == 13 ? 0 : atomicAdd(&s_nleave, 1);
            const int64_t w = code == 13 ? slot : start + k;
            const P& o = code == 13 ? sa.buf : sa.out;
            if constexpr (PLAIN) {
                o.x[w] = npos[0]; o.y[w] = npos[1]; o.z[w] = npos[2];
            } else {
                o.cell[w] = ncell; o.ox[w] = no3[0]; o.oy[w] = no3[1]; o.oz[w] = no3[2];
            }
            o.ux[w] = nu[0]; o.uy[w] = nu[1]; o.uz[w] = nu[2];
            if (code != 13) {
                o.w[w] = sa.buf.w[slot];
                sa.dir[slot] = (uint32_t)code | ((uint32_t)k << 5);
                sa.llist[w] = i;
                killAt(sa.buf, slot);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) sa.nleave[s] = s_nleave;
        __syncthreads();
    }
    if (bad) atomicExch(a.flags, PICA_ERR_MIGRATION);
    __syncthreads();
    // FP32: flush the supercell's tile once (periodic) into the fixed-point
    // accumulators; the 1/h^3 is applied when J is formed from the exact sums.
    if constexpr (!PLAIN)
        for (int t = threadIdx.x; t < 3 * TT; t += blockDim.x) {
            const long long vq = jt.node(t);
            if (vq != 0) {
                const int c = t / TT, r = t - c * TT;
                const int i = r / (T1 * T2), jj = (r / T2) % T1, k = r % T2;
                const int gx = wrapi(m[0] - kG + i, a.n[0]), gy = wrapi(m[1] - kG + jj, a.n[1]), gz = wrapi(m[2] - kG + k, a.n[2]);
                atomicAdd(a.jacc[c] + ((int64_t)gx * a.n[1] + gy) * a.n[2] + gz, (unsigned long long)vq);
            }
        }
}

// ---------------------------------------------------------------------------
// Migration kernels.  A step's leaver lists (slots, in arbitrary order) are
// sorted, then each destination supercell (one warp) takes its arrivals in
// canonical order -- direction code 0..26, then source slot -- into the holes
// its own leavers left (ascending), then appends.  The arrivals are counted
// first so that a capacity overflow is known before anything is written.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int neighbour(const int* nsc, const int* dc, int code) {
    const int ds[3] = {code / 9 - 1, (code / 3) % 3 - 1, code % 3 - 1};
    return (wrapi(dc[0] - ds[0], nsc[0]) * nsc[1] + wrapi(dc[1] - ds[1], nsc[1])) * nsc[2] + wrapi(dc[2] - ds[2], nsc[2]);
}

// Sort each supercell's leaver list ascending with a bitmap over its slots (one CTA per supercell).
template <class P>
__global__ void __launch_bounds__(128) k_sortLeavers(const __grid_constant__ MigrateArgs<P> a) {
    extern __shared__ unsigned int bits[];
    __shared__ int dcnt[kDirBuckets];
    const int s = blockIdx.x;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    for (int spi = 0; spi < a.nspecies; spi++) {
        const MigrateSpecies<P>& sa = a.sp[spi];
        const int n = sa.nleave[s];
        const int64_t start = sa.start[s];
        if (n > 1) {   // uniform across the block
            const int nw = (sa.count[s] + 31) / 32;
            for (int w = threadIdx.x; w < nw; w += blockDim.x) bits[w] = 0u;
            __syncthreads();
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                const int slot = sa.llist[start + k];
                atomicOr(&bits[slot >> 5], 1u << (slot & 31));
            }
            __syncthreads();
            if (threadIdx.x < 32) {
                int base = 0;
                for (int w0 = 0; w0 < nw; w0 += 32) {
                    const int w = w0 + lane;
                    unsigned b = w < nw ? bits[w] : 0u;
                    const int c = __popc(b);
                    int incl = c;
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1) {
                        const int t = __shfl_up_sync(0xffffffffu, incl, d);
                        if (lane >= d) incl += t;
                    }
                    int pos = base + incl - c;
                    while (b) {
                        const int bit = __ffs(b) - 1;
                        sa.llist[start + pos++] = w * 32 + bit;
                        b &= b - 1u;
                    }
                    base += __shfl_sync(0xffffffffu, incl, 31);
                }
            }
            __syncthreads();
        }
        // Buckets by direction code, each in slot order (one warp: counts, scan, scatter).
        if (threadIdx.x < 32) {
            if (lane < kDirBuckets) dcnt[lane] = 0;
            __syncwarp();
            for (int k0 = 0; k0 < n; k0 += 32) {
                const int k = k0 + lane;
                const int code = k < n ? (int)(sa.dir[start + sa.llist[start + k]] & 31u) : -1;
                const unsigned grp = __match_any_sync(0xffffffffu, code);
                if (code >= 0 && lane == __ffs(grp) - 1) dcnt[code] += __popc(grp);
                __syncwarp();
            }
            const int c = lane < 27 ? dcnt[lane] : 0;
            int incl = c;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += t;
            }
            if (lane < kDirBuckets) sa.dirOff[(int64_t)s * kDirBuckets + lane] = incl - c;
            __syncwarp();
            if (lane < 27) dcnt[lane] = incl - c;
            __syncwarp();
            for (int k0 = 0; k0 < n; k0 += 32) {
                const int k = k0 + lane;
                const int slot = k < n ? sa.llist[start + k] : -1;
                const uint32_t dk = k < n ? sa.dir[start + slot] : 0u;
                const int code = k < n ? (int)(dk & 31u) : -1;
                const unsigned grp = __match_any_sync(0xffffffffu, code);
                if (code >= 0) sa.lbydir[start + dcnt[code] + __popc(grp & lt)] = (int32_t)(dk >> 5);
                __syncwarp();
                if (code >= 0 && lane == __ffs(grp) - 1) dcnt[code] += __popc(grp);
                __syncwarp();
            }
        }
        __syncthreads();
    }
}

// The 26 arrival buckets of supercell d, one per lane (lanes 26..31 empty): the
// source supercell, its lbydir start and entry b0 of the bucket, the bucket size,
// and the exclusive prefix of the sizes in canonical order (direction code 0..26
// without 13).  Returns the total.
template <class P>
__device__ __forceinline__ int arrivalBuckets(const MigrateArgs<P>& a, const MigrateSpecies<P>& sa, int d, int& src,
                                              int64_t& sst, int& b0, int& pre) {
    const int lane = threadIdx.x & 31;
    const int dc[3] = {d / (a.nsc[1] * a.nsc[2]), (d / a.nsc[2]) % a.nsc[1], d % a.nsc[2]};
    const int code = lane < 13 ? lane : lane + 1;
    int cnt = 0;
    src = 0; sst = 0; b0 = 0;
    if (lane < 26) {
        src = neighbour(a.nsc, dc, code);
        const int32_t* off = sa.dirOff + (int64_t)src * kDirBuckets;
        b0 = off[code];
        cnt = off[code + 1] - b0;
        sst = sa.start[src];
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    pre = incl - cnt;
    return __shfl_sync(0xffffffffu, incl, 31);
}

// Arrivals at supercell d in canonical order -- by direction code (the move from the
// source), then by source slot -- 32 at a time across the buckets.  fn(k, src, rec, r,
// srcStart): the k-th arrival, whose record is at srcStart + rec in the side buffer
// (srcStart: the first slot of supercell src), entry r of src's lbydir list.
template <class P, class F>
__device__ __forceinline__ int forArrivals(const MigrateArgs<P>& a, const MigrateSpecies<P>& sa, int d, F&& fn, int sub = 0,
                                          int nsub = 1) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int src, b0, pre;
    int64_t sst;
    const int total = arrivalBuckets(a, sa, d, src, sst, b0, pre);
    for (int k0 = 32 * sub; k0 < total; k0 += 32 * nsub) {   // warp `sub` of nsub takes every nsub-th step
        const int k = k0 + lane;
        int c = 0;   // last bucket with pre <= k (buckets 0..25)
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const int cand = c + step;
            const int pc = __shfl_sync(FULL, pre, cand < 26 ? cand : 25);
            if (cand < 26 && pc <= k) c = cand;
        }
        const int ks = __shfl_sync(FULL, src, c);
        const int kb = __shfl_sync(FULL, b0, c);
        const int kp = __shfl_sync(FULL, pre, c);
        const int64_t kst = __shfl_sync(FULL, sst, c);
        if (k < total) {
            const int r = kb + (k - kp);
            fn(k, ks, sa.lbydir[kst + r], r, kst);
        }
    }
    return total;
}

template <class P, int STAGE>
__global__ void __launch_bounds__(256) k_migrate(const __grid_constant__ MigrateArgs<P> a) {
    const int nscTot = a.nsc[0] * a.nsc[1] * a.nsc[2];
    const int d = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (d >= nscTot) return;
    for (int spi = 0; spi < a.nspecies; spi++) {
        const MigrateSpecies<P>& sa = a.sp[spi];
        const int64_t start = sa.start[d];
        const int nh = sa.nleave[d];
        const int cnt = sa.count[d];
        int arrivals;
        if constexpr (STAGE == kCountArrivals) {
            int src, b0, pre;
            int64_t sst;
            arrivals = arrivalBuckets(a, sa, d, src, sst, b0, pre);
            if (lane == 0) {
                const int need = cnt + max(0, arrivals - nh);
                sa.needed[d] = need;
                sa.neededAlive[d] = sa.alive[d] - nh + arrivals;
                if (need > sa.cap[d]) atomicExch(a.flags + 1, 1);
            }
        } else if constexpr (STAGE == kGatherOutbox) {
            const int64_t off = sa.outOff[d];
            for (int k = lane; k < nh; k += 32) copyParticle(sa.b, start + sa.lbydir[start + k], sa.outbox, off + k);
        } else if constexpr (STAGE == kRebuild) {
            const int64_t ns = sa.newStart[d];
            for (int i = lane; i < cnt; i += 32) copyParticle(sa.a, start + i, sa.dst, ns + i);
            __syncwarp();
            arrivals = forArrivals(a, sa, d, [&](int k, int src, int, int r, int64_t) {
                const int target = k < nh ? sa.llist[start + k] : cnt + (k - nh);
                copyParticle(sa.outbox, sa.outOff[src] + r, sa.dst, ns + target);
            });
            if (lane == 0) { sa.count[d] = cnt + max(0, arrivals - nh); sa.alive[d] = sa.alive[d] - nh + arrivals; }
        }
    }
}

// The fill stage with kFillWarps warps per supercell (one CTA), which share its
// arrivals 32 at a time; the used and live counts are updated once all have copied.
constexpr int kFillWarps = 4;
template <class P>
__global__ void __launch_bounds__(kFillWarps * 32) k_fill(const __grid_constant__ MigrateArgs<P> a) {
    if (a.flags[0] != 0 || a.flags[1] != 0) return;   // error, or overflow: the rebuild runs instead
    const int d = blockIdx.x;
    const int warp = threadIdx.x >> 5;
    for (int spi = 0; spi < a.nspecies; spi++) {
        const MigrateSpecies<P>& sa = a.sp[spi];
        const int64_t start = sa.start[d];
        const int nh = sa.nleave[d];
        const int cnt = sa.count[d];
        const int alive = sa.alive[d];
        const int arrivals = forArrivals(
            a, sa, d,
            [&](int k, int, int slot, int, int64_t srcStart) {
                const int target = k < nh ? sa.llist[start + k] : cnt + (k - nh);
                copyParticle(sa.b, srcStart + slot, sa.a, start + target);
            },
            warp, kFillWarps);
        __syncthreads();   // every warp has read count and alive
        if (threadIdx.x == 0) {
            sa.count[d] = cnt + max(0, arrivals - nh);
            sa.alive[d] = alive - nh + arrivals;
        }
    }
}

// One particle's record, for copies that load several particles before storing any.
template <class P>
struct Rec;
template <>
struct Rec<CellPtrs> {
    uint32_t c;
    float f[7];
    __device__ __forceinline__ void load(const CellPtrs& p, int64_t i) {
        c = p.cell[i]; f[0] = p.ox[i]; f[1] = p.oy[i]; f[2] = p.oz[i];
        f[3] = p.ux[i]; f[4] = p.uy[i]; f[5] = p.uz[i]; f[6] = p.w[i];
    }
    __device__ __forceinline__ void store(const CellPtrs& p, int64_t j) const {
        p.cell[j] = c; p.ox[j] = f[0]; p.oy[j] = f[1]; p.oz[j] = f[2];
        p.ux[j] = f[3]; p.uy[j] = f[4]; p.uz[j] = f[5]; p.w[j] = f[6];
    }
    __device__ __forceinline__ int key(const int* m, const int* S, const double*) const {
        if (c == kDeadCell) return -1;
        int x[3];
        unpackCell(c, x[0], x[1], x[2]);
        return ((x[0] - m[0]) * S[1] + (x[1] - m[1])) * S[2] + (x[2] - m[2]);
    }
};
template <>
struct Rec<PlainPtrs> {
    double v[7];
    __device__ __forceinline__ void load(const PlainPtrs& p, int64_t i) {
        v[0] = p.x[i]; v[1] = p.y[i]; v[2] = p.z[i]; v[3] = p.ux[i]; v[4] = p.uy[i]; v[5] = p.uz[i]; v[6] = p.w[i];
    }
    __device__ __forceinline__ void store(const PlainPtrs& p, int64_t j) const {
        p.x[j] = v[0]; p.y[j] = v[1]; p.z[j] = v[2]; p.ux[j] = v[3]; p.uy[j] = v[4]; p.uz[j] = v[5]; p.w[j] = v[6];
    }
    __device__ __forceinline__ int key(const int* m, const int* S, const double* invh) const {
        if (!aliveX(v[0])) return -1;
        int l[3];
#pragma unroll
        for (int d = 0; d < 3; d++) l[d] = min(max((int)floor(v[d] * invh[d]) - m[d], 0), S[d] - 1);
        return (l[0] * S[1] + l[1]) * S[2] + l[2];
    }
};

// Local cell of slot i, or -1 for a dead slot (loads only what the key needs).
__device__ __forceinline__ int slotKey(const CellPtrs& p, int64_t i, const int* m, const int* S, const double* invh) {
    Rec<CellPtrs> r;
    r.c = p.cell[i];
    return r.key(m, S, invh);
}
__device__ __forceinline__ int slotKey(const PlainPtrs& p, int64_t i, const int* m, const int* S, const double* invh) {
    Rec<PlainPtrs> r;
    r.v[0] = p.x[i]; r.v[1] = p.y[i]; r.v[2] = p.z[i];
    return r.key(m, S, invh);
}

// Compact each supercell (drop dead slots) and sort it by cell, stably, into the new
// layout of buffer dst.  One CTA of kResortWarps warps per supercell: warp w owns
// the w-th contiguous eighth of the slots; a first pass counts cells per warp, a
// scan over (cell, warp) gives every warp its start in each cell, and a second
// pass scatters each warp's particles in slot order (rank within a 32-slot step
// from __match_any_sync).  Both passes load kResortUnroll steps of 32 slots before
// using them, to keep several HBM requests in flight per warp.  The result is
// ordered by (cell, old slot).
constexpr int kResortWarps = 8;
constexpr int kResortUnroll = 4;
// Resident CTAs per SM the register budget is set for: four with the FP32 records
// (64 registers), two with the FP64 ones (no spills).
template <class P>
constexpr int resortMinBlocks() { return std::is_same<P, CellPtrs>::value ? 4 : 2; }

template <class P>
__global__ void __launch_bounds__(kResortWarps * 32, resortMinBlocks<P>()) k_resort(const __grid_constant__ MigrateArgs<P> a) {
    constexpr unsigned FULL = 0xffffffffu;
    constexpr int kT = kResortWarps * 32;
    constexpr int U = kResortUnroll;
    constexpr int kBins = 512;  // largest supercell: 8 x 8 x 8 cells
    __shared__ int cnt[kResortWarps][kBins];
    __shared__ int wsum[kResortWarps];
    const int d = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nb = a.S[0] * a.S[1] * a.S[2];
    const int dc[3] = {d / (a.nsc[1] * a.nsc[2]), (d / a.nsc[2]) % a.nsc[1], d % a.nsc[2]};
    const int m[3] = {dc[0] * a.S[0], dc[1] * a.S[1], dc[2] * a.S[2]};
    const unsigned lt = (1u << lane) - 1u;
    for (int spi = 0; spi < a.nspecies; spi++) {
        const MigrateSpecies<P>& sa = a.sp[spi];
        const int64_t start = sa.start[d], ns = sa.newStart[d];
        const int n = sa.count[d];
        const int R = ((n + kT - 1) / kT) * 32;
        const int lo = min(warp * R, n), hi = min(lo + R, n);
        for (int k = threadIdx.x; k < kResortWarps * nb; k += kT) cnt[k / nb][k % nb] = 0;
        __syncthreads();
        for (int i0 = lo; i0 < hi; i0 += 32 * U) {
            int key[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int i = i0 + u * 32 + lane;
                key[u] = i < hi ? slotKey(sa.a, start + i, m, a.S, a.invh) : -1;
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                const unsigned grp = __match_any_sync(FULL, key[u]);
                if (key[u] >= 0 && lane == __ffs(grp) - 1) cnt[warp][key[u]] += __popc(grp);
                __syncwarp();
            }
        }
        __syncthreads();
        // Exclusive scan over (cell, warp), cell-major: 16 consecutive entries per thread.
        {
            const int E = nb * kResortWarps;
            int loc[16], sum = 0;
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const int f = threadIdx.x * 16 + q;
                loc[q] = f < E ? cnt[f % kResortWarps][f / kResortWarps] : 0;
                sum += loc[q];
            }
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += t;
            }
            if (lane == 31) wsum[warp] = incl;
            __syncthreads();
            int run = incl - sum;
            for (int w = 0; w < warp; w++) run += wsum[w];
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const int f = threadIdx.x * 16 + q;
                if (f < E) cnt[f % kResortWarps][f / kResortWarps] = run;
                run += loc[q];
            }
        }
        __syncthreads();
        for (int i0 = lo; i0 < hi; i0 += 32 * U) {
            Rec<P> r[U];
            int key[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int i = i0 + u * 32 + lane;
                if (i < hi) r[u].load(sa.a, start + i);
            }
#pragma unroll
            for (int u = 0; u < U; u++) key[u] = i0 + u * 32 + lane < hi ? r[u].key(m, a.S, a.invh) : -1;
#pragma unroll
            for (int u = 0; u < U; u++) {
                const unsigned grp = __match_any_sync(FULL, key[u]);
                if (key[u] >= 0) r[u].store(sa.dst, ns + cnt[warp][key[u]] + __popc(grp & lt));
                __syncwarp();
                if (key[u] >= 0 && lane == __ffs(grp) - 1) cnt[warp][key[u]] += __popc(grp);
                __syncwarp();
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) sa.count[d] = sa.alive[d];
    }
}


// FP32 cell form resort with each supercell staged through shared memory.  The
// cell array comes in first (cp.async, 16-byte pieces); the ranks of k_resort
// -- (cell, old slot) order, per-warp contiguous slot ranges, __match_any_sync
// groups -- are computed from it once and kept as 16-bit destinations; then
// each array in turn is copied in and scattered from shared memory to its
// sorted position.  Every array is read from HBM once, in large asynchronous
// pieces, where k_resort reads the cells twice and keeps only a few loads in
// flight per warp.  Shared memory: 6 B per slot of the largest source supercell
// plus the per-warp cell counts (stagedResortSmem).
constexpr int kStagedWarps = 8;

__host__ __device__ constexpr int stagedResortWords(int maxCap) { return (maxCap + 3) & ~3; }
__host__ __device__ constexpr size_t stagedResortSmem(int maxCap, int nb) {
    return (size_t)stagedResortWords(maxCap) * 6 + (size_t)kStagedWarps * nb * 4 + 16;
}

__device__ __forceinline__ void cpAsync16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}

__device__ __forceinline__ uint32_t* cellArray(const CellPtrs& p, int k) {
    switch (k) {
        case 0: return p.cell;
        case 1: return reinterpret_cast<uint32_t*>(p.ox);
        case 2: return reinterpret_cast<uint32_t*>(p.oy);
        case 3: return reinterpret_cast<uint32_t*>(p.oz);
        case 4: return reinterpret_cast<uint32_t*>(p.ux);
        case 5: return reinterpret_cast<uint32_t*>(p.uy);
        case 6: return reinterpret_cast<uint32_t*>(p.uz);
        default: return reinterpret_cast<uint32_t*>(p.w);
    }
}

template <class P>
__global__ void __launch_bounds__(kStagedWarps * 32, 4) k_resortStaged(const __grid_constant__ MigrateArgs<P> a) {
    static_assert(std::is_same<P, CellPtrs>::value, "the staged resort moves 4-byte components");
    constexpr unsigned FULL = 0xffffffffu;
    constexpr int kT = kStagedWarps * 32;
    extern __shared__ __align__(16) unsigned char smem[];
    const int W = stagedResortWords(a.srcMaxCap);
    uint32_t* buf = reinterpret_cast<uint32_t*>(smem);                  // W words
    uint16_t* pos = reinterpret_cast<uint16_t*>(smem + (size_t)W * 4);  // W entries: staged index of sorted slot p
    const int nb = a.S[0] * a.S[1] * a.S[2];
    int* cnt = reinterpret_cast<int*>(smem + (size_t)W * 6);            // [warp][cell]
    __shared__ int wsum[kStagedWarps];
    const int d = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int dc[3] = {d / (a.nsc[1] * a.nsc[2]), (d / a.nsc[2]) % a.nsc[1], d % a.nsc[2]};
    const int m[3] = {dc[0] * a.S[0], dc[1] * a.S[1], dc[2] * a.S[2]};
    const unsigned lt = (1u << lane) - 1u;
    for (int spi = 0; spi < a.nspecies; spi++) {
        const MigrateSpecies<P>& sa = a.sp[spi];
        const int64_t start = sa.start[d], ns = sa.newStart[d];
        const int n = sa.count[d];
        const int nw = (n + 3) & ~3;   // <= the supercell's capacity (a multiple of 32), so in bounds
        // Cells in; per-warp counts zeroed meanwhile.
        for (int c = threadIdx.x; c < nw / 4; c += kT) cpAsync16(buf + 4 * c, sa.a.cell + start + 4 * c);
        asm volatile("cp.async.commit_group;" ::: "memory");
        for (int k = threadIdx.x; k < kStagedWarps * nb; k += kT) cnt[k] = 0;
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();
        const int R = ((n + kT - 1) / kT) * 32;
        const int lo = min(warp * R, n), hi = min(lo + R, n);
        for (int i0 = lo; i0 < hi; i0 += 32) {
            const int i = i0 + lane;
            Rec<CellPtrs> r;
            r.c = i < hi ? buf[i] : kDeadCell;
            const int key = r.key(m, a.S, nullptr);
            const unsigned grp = __match_any_sync(FULL, key);
            if (key >= 0 && lane == __ffs(grp) - 1) cnt[warp * nb + key] += __popc(grp);
            __syncwarp();
        }
        __syncthreads();
        // Exclusive scan over (cell, warp), cell-major, as in k_resort.
        {
            const int E = nb * kStagedWarps;
            const int per = (E + kT - 1) / kT;   // <= 16 for nb <= 512
            int loc[16], sum = 0;
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const int f = threadIdx.x * per + q;
                loc[q] = (q < per && f < E) ? cnt[(f % kStagedWarps) * nb + f / kStagedWarps] : 0;
                sum += loc[q];
            }
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += t;
            }
            if (lane == 31) wsum[warp] = incl;
            __syncthreads();
            int run = incl - sum;
            for (int w = 0; w < warp; w++) run += wsum[w];
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const int f = threadIdx.x * per + q;
                if (q < per && f < E) cnt[(f % kStagedWarps) * nb + f / kStagedWarps] = run;
                run += loc[q];
            }
        }
        __syncthreads();
        for (int i0 = lo; i0 < hi; i0 += 32) {
            const int i = i0 + lane;
            Rec<CellPtrs> r;
            r.c = i < hi ? buf[i] : kDeadCell;
            const int key = r.key(m, a.S, nullptr);
            const unsigned grp = __match_any_sync(FULL, key);
            if (i < hi && key >= 0) pos[cnt[warp * nb + key] + __popc(grp & lt)] = (uint16_t)i;   // inverse
            __syncwarp();
            if (key >= 0 && lane == __ffs(grp) - 1) cnt[warp * nb + key] += __popc(grp);
            __syncwarp();
        }
        __syncthreads();
        // Each array: written out in sorted order, output slot p taking staged entry pos[p]
        // (consecutive threads store consecutive slots), then the next array brought in.
        int total = 0;
        for (int w = 0; w < kStagedWarps; w++) total += wsum[w];
        for (int k = 0; k < 8; k++) {
            uint32_t* dst = cellArray(sa.dst, k) + ns;
            for (int p = threadIdx.x; p < total; p += kT) dst[p] = buf[pos[p]];
            __syncthreads();
            if (k == 7) break;
            const uint32_t* src = cellArray(sa.a, k + 1) + start;
            for (int c = threadIdx.x; c < nw / 4; c += kT) cpAsync16(buf + 4 * c, src + 4 * c);
            asm volatile("cp.async.commit_group;" ::: "memory");
            asm volatile("cp.async.wait_group 0;" ::: "memory");
            __syncthreads();
        }
        if (threadIdx.x == 0) sa.count[d] = sa.alive[d];
        __syncthreads();
    }
}

}  // namespace pgb
