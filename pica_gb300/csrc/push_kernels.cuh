// Fused supercell kernel (field gather + Boris push + current deposit + migration
// partition) and the migration kernels.  Included by push_fp64.cu (built with
// --fmad=false so FP64 arithmetic rounds exactly as pica's C++ does) and by
// push_fp32.cu (FMA contraction allowed).
//
// One CTA owns one supercell.  It stages the E/B tile of nodes [m-2, m+S+3)
// per dimension (periodic) into shared memory, accumulates the supercell's
// current in a shared-memory tile of the same extent (64-bit fixed point,
// native integer shared-memory atomics), and adds the tile to the global
// accumulator once (periodic) at the end -- the GPU form of pica's
// FieldInterpolatorCICSupercell / CurrentDepositorCICSupercell pair
// (fieldInterpolation/FieldInterpolatorYeeGrid.h:188-283,
//  currentDeposition/CurrentDepositorYeeGrid.h:168-264).
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

// Add one current contribution to a tile node.  FP32 form: the contribution is
// already scaled to fixed-point units and is added as a 64-bit integer (exact,
// order-independent).  FP64 form: plain FP64 add, so the FP64 result differs
// from pica's only by the order of the sums.
__device__ __forceinline__ void addQ(unsigned long long* p, float scaled) {
    atomicAdd(p, (unsigned long long)__float2ll_rn(scaled));
}
__device__ __forceinline__ void addQ(double* p, double v) { atomicAdd(p, v); }

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

template <typename R, int W, typename A>
__device__ __forceinline__ void scatterSep(A* tile, int T1, int T2, const int* t0, const R* wx, const R* wy,
                                           const R* wz, R v) {
#pragma unroll
    for (int i = 0; i < W; i++)
#pragma unroll
        for (int j = 0; j < W; j++) {
            A* row = tile + ((t0[0] + i) * T1 + (t0[1] + j)) * T2 + t0[2];
            R vij = (v * wx[i]) * wy[j];
#pragma unroll
            for (int k = 0; k < W; k++) addQ(row + k, vij * wz[k]);
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
// pica's CIC 8-point deposit, CurrentDepositorYeeGrid.h:254-261 (same factor order).
__device__ __forceinline__ void cicScatterRef(double* t, int T1, int T2, const int* b, const double* c, double v) {
    double* p = t + (b[0] * T1 + b[1]) * T2 + b[2];
    const int sy = T2, sx = T1 * T2;
    const double cx = c[0], cy = c[1], cz = c[2];
    addQ(p, (1.0 - cx) * (1.0 - cy) * (1.0 - cz) * v);
    addQ(p + 1, (1.0 - cx) * (1.0 - cy) * cz * v);
    addQ(p + sy, (1.0 - cx) * cy * (1.0 - cz) * v);
    addQ(p + sy + 1, (1.0 - cx) * cy * cz * v);
    addQ(p + sx, cx * (1.0 - cy) * (1.0 - cz) * v);
    addQ(p + sx + 1, cx * (1.0 - cy) * cz * v);
    addQ(p + sx + sy, cx * cy * (1.0 - cz) * v);
    addQ(p + sx + sy + 1, cx * cy * cz * v);
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
template <typename R, int NW, typename A>
__device__ __forceinline__ void esirkepov(A* jx, A* jy, A* jz, int T1, int T2, const int* b, const R (*s0)[NW],
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
                addQ(jx + ((b[0] + i + 1) * T1 + (b[1] + j)) * T2 + (b[2] + l), acc * k[0]);
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
                addQ(jy + ((b[0] + i) * T1 + (b[1] + j + 1)) * T2 + (b[2] + l), acc * k[1]);
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
                addQ(jz + ((b[0] + i) * T1 + (b[1] + j)) * T2 + (b[2] + l + 1), acc * k[2]);
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
    using A = typename std::conditional<PLAIN, double, unsigned long long>::type;  // J tile accumulator
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_cnt[2][kPushThreads / 32];
    __shared__ int s_base[2];

    const int T1 = a.T[1], T2 = a.T[2], TT = a.T[0] * T1 * T2;
    A* jt = reinterpret_cast<A*>(smem_raw);
    R* eb = reinterpret_cast<R*>(jt + 3 * TT);
    const int s = blockIdx.x;
    int sc[3];
    sc[2] = s % a.nsc[2];
    sc[1] = (s / a.nsc[2]) % a.nsc[1];
    sc[0] = s / (a.nsc[1] * a.nsc[2]);
    const int m[3] = {sc[0] * a.S[0], sc[1] * a.S[1], sc[2] * a.S[2]};
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;

    // Stage the E/B tile (periodic) and clear the J tile.
    for (int t = threadIdx.x; t < 6 * TT; t += blockDim.x) {
        const int c = t / TT, r = t - c * TT;
        const int i = r / (T1 * T2), jj = (r / T2) % T1, k = r % T2;
        const int gx = wrapi(m[0] - kG + i, a.n[0]), gy = wrapi(m[1] - kG + jj, a.n[1]), gz = wrapi(m[2] - kG + k, a.n[2]);
        eb[t] = static_cast<const R*>(a.eb[c])[((int64_t)gx * a.n[1] + gy) * a.n[2] + gz];
    }
    for (int t = threadIdx.x; t < 3 * TT; t += blockDim.x) jt[t] = A(0);

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
    A* jx = jt;
    A* jy = jt + TT;
    A* jz = jt + 2 * TT;
    const R invU = (R)a.invUnit;
    bool bad = false;
    __syncthreads();

    for (int spi = 0; spi < a.nspecies; spi++) {
        const SpeciesArgs<P>& sa = a.sp[spi];
        const int64_t start = sa.start[s];
        const int cap = sa.cap[s];
        const int count = sa.count[s];
        const R ec = (R)sa.ec;
        if (threadIdx.x == 0) { s_base[0] = 0; s_base[1] = 0; }
        __syncthreads();
        for (int base = 0; base < count; base += blockDim.x) {
            const int i = base + threadIdx.x;
            const bool act = i < count;
            int code = 13;
            const int64_t slot = start + i;
            // New particle state (written after the rank computation).
            R nu[3], nw8 = R(0);
            double npos[3];
            uint32_t ncell = 0;
            float no3[3];
            if (act) {
                R u[3], eb6[6], wgt;
                if constexpr (PLAIN) {
                    const double pos[3] = {sa.in.x[slot], sa.in.y[slot], sa.in.z[slot]};
                    u[0] = sa.in.ux[slot]; u[1] = sa.in.uy[slot]; u[2] = sa.in.uz[slot];
                    wgt = sa.in.w[slot];
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
                                cicScatterRef(jt + comp * TT, T1, T2, b, w, cur[comp]);
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
                                scatterSep<double, 3>(jt + comp * TT, T1, T2, t0, stag(comp, 0) ? ws[0] : wc[0],
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
                            esirkepov<double, 3>(jx, jy, jz, T1, T2, b, s0, s1, kq);
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
                            esirkepov<double, 4>(jx, jy, jz, T1, T2, b, s0, s1, kq);
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
                    unpackCell(sa.in.cell[slot], c3[0], c3[1], c3[2]);
                    const int lc[3] = {c3[0] - m[0], c3[1] - m[1], c3[2] - m[2]};
                    const float o[3] = {sa.in.ox[slot], sa.in.oy[slot], sa.in.oz[slot]};
                    u[0] = sa.in.ux[slot]; u[1] = sa.in.uy[slot]; u[2] = sa.in.uz[slot];
                    wgt = sa.in.w[slot];
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
                                scatterSep<float, 2>(jt + comp * TT, T1, T2, t0, stag(comp, 0) ? ws[0] : wc[0],
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
                                scatterSep<float, 3>(jt + comp * TT, T1, T2, t0, stag(comp, 0) ? ws[0] : wc[0],
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
                            esirkepov<float, 3>(jx, jy, jz, T1, T2, b, s0, s1, kq);
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
                            esirkepov<float, 4>(jx, jy, jz, T1, T2, b, s0, s1, kq);
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
                nw8 = wgt;
            }
            // Stable partition: stayers packed from the front, leavers from the back.
            const bool stay = act && code == 13, leave = act && code != 13;
            const unsigned ms = __ballot_sync(0xffffffffu, stay), ml = __ballot_sync(0xffffffffu, leave);
            if (lane == 0) { s_cnt[0][warp] = __popc(ms); s_cnt[1][warp] = __popc(ml); }
            __syncthreads();
            int rs = s_base[0], rl = s_base[1];
            for (int w = 0; w < warp; w++) { rs += s_cnt[0][w]; rl += s_cnt[1][w]; }
            const unsigned lt = (1u << lane) - 1u;
            if (act) {
                int64_t o;
                if (stay) o = start + rs + __popc(ms & lt);
                else {
                    o = start + cap - 1 - (rl + __popc(ml & lt));
                    sa.dir[o] = (uint8_t)code;
                }
                if constexpr (PLAIN) {
                    sa.out.x[o] = npos[0]; sa.out.y[o] = npos[1]; sa.out.z[o] = npos[2];
                } else {
                    sa.out.cell[o] = ncell; sa.out.ox[o] = no3[0]; sa.out.oy[o] = no3[1]; sa.out.oz[o] = no3[2];
                }
                sa.out.ux[o] = nu[0]; sa.out.uy[o] = nu[1]; sa.out.uz[o] = nu[2]; sa.out.w[o] = nw8;
            }
            __syncthreads();
            if (threadIdx.x == 0)
                for (int w = 0; w < nwarps; w++) { s_base[0] += s_cnt[0][w]; s_base[1] += s_cnt[1][w]; }
            __syncthreads();
        }
        if (threadIdx.x == 0) { sa.nstay[s] = s_base[0]; sa.nleave[s] = s_base[1]; }
        __syncthreads();
    }
    if (bad) atomicExch(a.flags, PICA_ERR_MIGRATION);
    __syncthreads();
    // Flush the supercell's tile once (periodic).  FP64: J += tile / h^3 as
    // CurrentDepositorYeeGrid.h:201-213; FP32: into the fixed-point accumulator,
    // the 1/h^3 is applied when J is formed from the exact sums.
    for (int t = threadIdx.x; t < 3 * TT; t += blockDim.x) {
        const A v = jt[t];
        if (v != A(0)) {
            const int c = t / TT, r = t - c * TT;
            const int i = r / (T1 * T2), jj = (r / T2) % T1, k = r % T2;
            const int gx = wrapi(m[0] - kG + i, a.n[0]), gy = wrapi(m[1] - kG + jj, a.n[1]), gz = wrapi(m[2] - kG + k, a.n[2]);
            const int64_t node = ((int64_t)gx * a.n[1] + gy) * a.n[2] + gz;
            if constexpr (PLAIN) atomicAdd(static_cast<double*>(a.j[c]) + node, v * a.norm);
            else atomicAdd(a.jacc[c] + node, v);
        }
    }
}

// ---------------------------------------------------------------------------
// Migration: one warp per destination supercell.  Arrivals are appended after
// the destination's stayers in canonical order (direction code 0..26, then the
// source's slot order).  REBUILD copies stayers + arrivals into a new layout.
// ---------------------------------------------------------------------------
template <class P, bool REBUILD>
__global__ void __launch_bounds__(256) k_migrate(const __grid_constant__ MigrateArgs<P> a) {
    const int nscTot = a.nsc[0] * a.nsc[1] * a.nsc[2];
    const int d = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (d >= nscTot) return;
    const int dc[3] = {d / (a.nsc[1] * a.nsc[2]), (d / a.nsc[2]) % a.nsc[1], d % a.nsc[2]};
    const unsigned lt = (1u << lane) - 1u;
    for (int spi = 0; spi < a.nspecies; spi++) {
        const MigrateSpecies<P>& sa = a.sp[spi];
        const int64_t start = sa.start[d];
        const int nstay = sa.nstay[d];
        const int limit = sa.cap[d] - sa.nleave[d];
        int64_t dstBase = start;
        if constexpr (REBUILD) {
            dstBase = sa.newStart[d];
            for (int i = lane; i < nstay; i += 32) copyParticle(sa.buf, start + i, sa.dst, dstBase + i);
        }
        int pos = nstay;
        bool over = false;
        for (int code = 0; code < 27; code++) {
            if (code == 13) continue;
            const int ds[3] = {code / 9 - 1, (code / 3) % 3 - 1, code % 3 - 1};
            const int src = (wrapi(dc[0] - ds[0], a.nsc[0]) * a.nsc[1] + wrapi(dc[1] - ds[1], a.nsc[1])) * a.nsc[2] +
                            wrapi(dc[2] - ds[2], a.nsc[2]);
            const int L = sa.nleave[src];
            if (L == 0) continue;
            const int64_t tail = sa.start[src] + sa.cap[src] - 1;
            for (int r0 = 0; r0 < L; r0 += 32) {
                const int r = r0 + lane;
                const bool match = r < L && sa.dir[tail - r] == code;
                const unsigned mk = __ballot_sync(0xffffffffu, match);
                if (match) {
                    const int dst = pos + __popc(mk & lt);
                    if constexpr (REBUILD) copyParticle(sa.buf, tail - r, sa.dst, dstBase + dst);
                    else {
                        if (dst < limit) copyParticle(sa.buf, tail - r, sa.buf, start + dst);
                        else over = true;
                    }
                }
                pos += __popc(mk);
            }
        }
        if (lane == 0) {
            sa.needed[d] = pos;
            if constexpr (REBUILD) sa.count[d] = pos;
            else if (pos <= limit) sa.count[d] = pos;
        }
        over = __any_sync(0xffffffffu, over);
        if (over && lane == 0) atomicExch(a.flags + 1, 1);
    }
}

}  // namespace pgb
