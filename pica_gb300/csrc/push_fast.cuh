// FP32 cell-form push kernel specialised for charge-conserving (Esirkepov)
// deposition, built around the supercell's particles being stored in cell
// order (they are generated that way and kept so by the periodic in-supercell
// sort):
//
//  * A warp owns contiguous segments of 32*K particles of its supercell; lane
//    l handles the K consecutive particles lK .. lK+K-1 (the next one's data is
//    loaded one iteration ahead), so a lane rarely changes cell and the warp's
//    lanes mostly share one or two cells.  The supercell's last segments are cut
//    into 8 shorter ones so that every warp of the CTA gets the same work.
//  * Particles that stay in their cell (about 96% per step for a thermal plasma
//    at half the Courant step) have old and new shapes on the rho-lattice nodes
//    lc-1 .. lc+1 (TSC: all three; CIC: two of them, by the half of the cell),
//    so they deposit on a fixed window of 54 face values.  Each lane sums
//    its particles' window contributions in registers, keyed by the window.
//    When a lane meets a particle of another window it parks its sums in a
//    spare row of the warp's shared-memory reduction area.  At the end of the
//    segment every lane writes its sums to its own row, and the warp adds the
//    rows of each window in a fixed order (lane rows, then park rows in the
//    order they were taken): lane t sums values t and t+32 over the rows and
//    issues one fixed-point shared-memory atomic per value.  The order depends
//    only on the particle data, so the result is reproducible bit for bit.
//  * Particles that change cell, and particles alone in their cell within a
//    lane's run (out of cell order since the last resort, or arrivals from
//    other supercells), are queued in a per-warp shared-memory ring and
//    deposited on the general 4- (TSC) or 3-node (CIC) window, 32 at a time (one
//    per lane), by one out-of-line routine.
//  * Stayers are written back in place; leavers go to the side buffer, packed
//    per supercell (see pica_internal.h), so the kernel needs no block-wide
//    synchronisation between the tile staging and the final tile flush.
//  * The E/B tile holds only the nodes that the gather reads, m-1 .. m+S+1
//    per dimension; the current tile spans m-2 .. m+S+2 (general windows).
#pragma once

#include "push_kernels.cuh"

namespace pgb {

// Tile address of window contribution j for the stay-in-cell Esirkepov window
// starting at tile node b (per dimension).  TSC: NWn = 3 nodes, 2 faces;
// CIC: NWn = 2 nodes, 1 face.  Layout: Jx (faces x NWn x NWn), then Jy, then Jz.
template <int NWn>
__device__ __forceinline__ int windowIdx(int TT, int T1, int T2, const int* b, int j) {
    constexpr int F = NWn - 1;            // faces per dimension
    constexpr int per = F * NWn * NWn;    // contributions per component
    const int c = j / per, r = j - c * per;
    int o[3];
    if (c == 0) { o[0] = r / (NWn * NWn) + 1; o[1] = (r / NWn) % NWn; o[2] = r % NWn; }
    else if (c == 1) { o[0] = r / (F * NWn); o[1] = (r / NWn) % F + 1; o[2] = r % NWn; }
    else { o[0] = r / (NWn * F); o[1] = (r / F) % NWn; o[2] = r % F + 1; }
    return c * TT + ((b[0] + o[0]) * T1 + (b[1] + o[1])) * T2 + (b[2] + o[2]);
}

// Boris rotation of BorisPusher.h:33-43 in FP32 with the hardware reciprocal
// square root and fast division (a few ulp; the FP32 form is checked against
// the FP32 oracle within 1e-4).  Returns 1/gamma of the new u.  This unit is
// compiled without implicit contraction, so every multiply-add below is written
// out (_rn intrinsics and fused multiply-adds): each instantiation of the push --
// launch variants, the batching form -- then rounds alike.
__device__ __forceinline__ float sumsq3(const float* v) {
    return __fmaf_rn(v[2], v[2], __fmaf_rn(v[1], v[1], __fmul_rn(v[0], v[0])));
}
// a*b - c*d as one fused multiply-add on a rounded product.
__device__ __forceinline__ float mulSub(float a, float b, float c, float d) { return __fmaf_rn(a, b, -__fmul_rn(c, d)); }

__device__ __forceinline__ float borisFast(float ec, const float* eb, float* u) {
    const float em[3] = {__fmul_rn(eb[0], ec), __fmul_rn(eb[1], ec), __fmul_rn(eb[2], ec)};
    const float um[3] = {__fadd_rn(u[0], em[0]), __fadd_rn(u[1], em[1]), __fadd_rn(u[2], em[2])};
    const float tc = __fmul_rn(ec, rsqrtf(__fadd_rn(1.0f, sumsq3(um))));
    const float t[3] = {__fmul_rn(eb[3], tc), __fmul_rn(eb[4], tc), __fmul_rn(eb[5], tc)};
    const float up[3] = {__fadd_rn(um[0], mulSub(um[1], t[2], um[2], t[1])),
                         __fadd_rn(um[1], mulSub(um[2], t[0], um[0], t[2])),
                         __fadd_rn(um[2], mulSub(um[0], t[1], um[1], t[0]))};
    const float sc = __fdividef(2.0f, __fadd_rn(1.0f, sumsq3(t)));
    const float s[3] = {__fmul_rn(t[0], sc), __fmul_rn(t[1], sc), __fmul_rn(t[2], sc)};
    u[0] = __fadd_rn(__fadd_rn(um[0], mulSub(up[1], s[2], up[2], s[1])), em[0]);
    u[1] = __fadd_rn(__fadd_rn(um[1], mulSub(up[2], s[0], up[0], s[2])), em[1]);
    u[2] = __fadd_rn(__fadd_rn(um[2], mulSub(up[0], s[1], up[1], s[0])), em[2]);
    return rsqrtf(__fadd_rn(1.0f, sumsq3(u)));
}

// TSC weights of the three nodes around an offset d in [-1/2, 1/2] (FP32, the
// roundings written out): 1/2 (1/2 - d)^2, 3/4 - d^2, 1/2 (1/2 + d)^2.
__device__ __forceinline__ void tscWeightsF(float d, float* w) {
    const float a = __fsub_rn(0.5f, d), b = __fadd_rn(0.5f, d);
    w[0] = __fmul_rn(0.5f, __fmul_rn(a, a));
    w[1] = __fmaf_rn(-d, d, 0.75f);
    w[2] = __fmul_rn(0.5f, __fmul_rn(b, b));
}

// Two field components gathered together with packed FP32x2 arithmetic (each half
// rounds exactly as the scalar gatherSep does): component A from tile tA with base
// ta and weights wxa, wya, wza; component B likewise.
template <int W>
__device__ __forceinline__ float2 gatherPair(const float* tA, const float* tB, int E1, int E2, const int* ta,
                                             const int* tb, const float* wxa, const float* wya, const float* wza,
                                             const float* wxb, const float* wyb, const float* wzb) {
    float2 wz[W];
#pragma unroll
    for (int k = 0; k < W; k++) wz[k] = make_float2(wza[k], wzb[k]);
    float2 r = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int i = 0; i < W; i++) {
        float2 ry = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int j = 0; j < W; j++) {
            const float* ra = tA + ((ta[0] + i) * E1 + (ta[1] + j)) * E2 + ta[2];
            const float* rb = tB + ((tb[0] + i) * E1 + (tb[1] + j)) * E2 + tb[2];
            float2 rz = __fmul2_rn(make_float2(ra[0], rb[0]), wz[0]);
#pragma unroll
            for (int k = 1; k < W; k++) rz = __ffma2_rn(make_float2(ra[k], rb[k]), wz[k], rz);
            ry = __ffma2_rn(make_float2(wya[j], wyb[j]), rz, ry);
        }
        r = __ffma2_rn(make_float2(wxa[i], wxb[i]), ry, r);
    }
    return r;
}

constexpr int kQWords = 11;  // queued window change: o[3], on[3], kq[3], packed lc, packed ln
constexpr int kStayNodes = 3;    // stay-in-cell window: rho-lattice nodes lc-1 .. lc+1 per dimension
constexpr int kStayValues = 54;  // its face values: 3 components x 2 faces x 3 x 3

// Entry i (a runtime index) of an N-entry register array, by selects, so that
// the array stays in registers.
template <int N>
__device__ __forceinline__ float pickN(const float* a, int i) {
    float v = a[0];
#pragma unroll
    for (int k = 1; k < N; k++) v = (i == k) ? a[k] : v;
    return v;
}

// esirkepov() (push_kernels.cuh) in FP32 with the loops over transverse node
// pairs rolled: the same values from the same expressions, in about a tenth of
// the code.  The general window runs once per queue drain, straight through, so
// its unrolled form is fetched from the instruction cache hierarchy at every
// call; the selects of the rolled loops cost less than those fetch stalls.
// len[k] is the number of window nodes the two shapes cover along k (NW, or NW-1
// when the particle stays in its cell along k): nodes and faces beyond it are not
// visited (their transverse factors are zero, and their sum of shape changes is
// zero but for rounding), nor is a node pair whose transverse factor is zero.  The
// transverse nodes are two nested loops, and the first node's factors are picked
// once per row.
// The arrays are in a per-lane frame: frame dimension k is grid dimension p[k],
// with tile stride sp[k], component offset cofs[k] = p[k] * TT and current factor
// k[k].  The caller puts the dimensions whose window widens first, so the 32 lanes
// of a drain, which each deposit one particle and mostly cross one cell face each
// (along different grid dimensions), run the same loop counts: 75 face values per
// lane (27 + 24 + 24) instead of the 144 that the union of their windows in grid
// order takes.  The transverse factor keeps the grid order of its two dimensions
// (the product a d_b is rounded, d_a b is fused), so every value, and with it the
// fixed-point sum, is the same bit for bit in any frame.  s0 is the old shape and
// ds the shape change on the window's nodes, per frame dimension.
template <int NW, typename Tile>
__device__ __forceinline__ void esirkepovRolled(const Tile& jt, const int* cofs, const int* sp, const int* b,
                                                const int* p, const float (*s0)[NW], const float (*ds)[NW],
                                                const float* k, const int* len) {
    const float hf = 0.5f, th = (float)kThird;
    // Component along frame dimension c: transverse frame dimensions t1 < t2, faces
    // along c.  Transverse factor of a node pair, grid-lower dimension (a, da), the
    // other (b, db): a b + (d_a b + a d_b) / 2 + d_a d_b / 3.
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int t1 = c == 0 ? 1 : 0, t2 = c == 2 ? 1 : 2;
        const bool sw = p[t1] > p[t2];
        const int nf = len[c] - 1, nu = len[t1], nv = len[t2];
        const int cb = cofs[c] + b[c] * sp[c] + b[t1] * sp[t1] + b[t2] * sp[t2];
#pragma unroll 1
        for (int u = 0; u < nu; u++) {
            const float a = pickN<NW>(s0[t1], u), da = pickN<NW>(ds[t1], u);
            const int ub = cb + u * sp[t1];
#pragma unroll 1
            for (int v = 0; v < nv; v++) {
                const float bb = pickN<NW>(s0[t2], v), db = pickN<NW>(ds[t2], v);
                const float mid = sw ? __fmaf_rn(a, db, __fmul_rn(bb, da)) : __fmaf_rn(da, bb, __fmul_rn(a, db));
                const float f = __fmaf_rn(th, __fmul_rn(da, db), __fmaf_rn(hf, mid, __fmul_rn(a, bb)));
                if (f != 0.f) {
                    const int idx = ub + v * sp[t2];
                    float acc = 0.f;
#pragma unroll
                    for (int i = 0; i < NW - 1; i++) {
                        if (i < nf) {
                            acc = __fmaf_rn(ds[c][i], f, acc);
                            jt.add(idx + (i + 1) * sp[c], __fmul_rn(acc, k[c]));
                        }
                    }
                }
            }
        }
    }
}

// Frame order for each 3-bit mask of grid dimensions whose window widens: those
// dimensions first, then the others, each group ascending; entry m holds
// p0 | p1 << 2 | p2 << 4 at bit 6 m.
__host__ __device__ constexpr unsigned long long frameOrders() {
    unsigned long long t = 0;
    for (int m = 0; m < 8; m++) {
        int code = 0, k = 0;
        for (int pass = 0; pass < 2; pass++)
            for (int d = 0; d < 3; d++)
                if ((((m >> d) & 1) != 0) == (pass == 0)) code |= d << (2 * k++);
        t |= (unsigned long long)code << (6 * m);
    }
    return t;
}
constexpr unsigned long long kFrameOrders = frameOrders();

__device__ __forceinline__ float pick3f(const float* a, int d) { return d == 0 ? a[0] : (d == 1 ? a[1] : a[2]); }
__device__ __forceinline__ int pick3i(const int* a, int d) { return d == 0 ? a[0] : (d == 1 ? a[1] : a[2]); }

// Esirkepov deposit of a particle whose rho-lattice window changes (old shape on
// nodes lo0.., new on lo1..): general NWn+1-node window with per-lane atomics.
// TSC runs in the frame that puts the widened dimensions first (thermal plasma at
// 128^3 x 100 ppc: push 12.82 -> 12.44 ms).  CIC keeps grid order: its drains are
// short (2- and 3-node windows), and on the two-stream plasma, whose particles
// widen their windows along x alone, the frame's selects made the push 7.6% slower.
template <int SHAPE, typename Tile>
__device__ __forceinline__ void generalWindow(const Tile& jt, int TT, int T1, int T2, const float* o,
                                              const float* on, const int* lc, const int* ln, const float* kq) {
    constexpr int NWn = SHAPE == PICA_SHAPE_TSC ? 3 : 2;
    constexpr int NW4 = NWn + 1;
    int lo0[3], lo1[3];
    int wide = 0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        if constexpr (SHAPE == PICA_SHAPE_TSC) {
            lo0[d] = lc[d] - 1;
            lo1[d] = ln[d] - 1;
        } else {
            lo0[d] = o[d] >= 0.5f ? lc[d] : lc[d] - 1;
            lo1[d] = on[d] >= 0.5f ? ln[d] : ln[d] - 1;
        }
        wide |= (lo0[d] != lo1[d] ? 1 : 0) << d;   // unused by CIC
    }
    int p[3] = {0, 1, 2};
    if constexpr (SHAPE == PICA_SHAPE_TSC) {
        const int code = (int)((kFrameOrders >> (6 * wide)) & 63ull);
        p[0] = code & 3; p[1] = (code >> 2) & 3; p[2] = (code >> 4) & 3;
    }
    const int st[3] = {T1 * T2, T2, 1};
    float s0[3][NW4], ds[3][NW4], kp[3];
    int b[3], len[3], sp[3], cofs[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int d = p[k];
        const float ok = pick3f(o, d), onk = pick3f(on, d);
        const int l0 = pick3i(lo0, d), l1 = pick3i(lo1, d);
        // Along a dimension where both shapes sit on the same nodes, the shape change
        // in the stay window's factored form, from the displacement D: S1 - S0 in FP32
        // keeps only the bits of D above 2^-24 of the weights, a few 1e-6 of the change
        // of a particle that moves 1% of a cell (the charge-conservation residual of
        // the queued particles that stay in their cell).  Elsewhere S1 - S0.
        const int base = min(l0, l1);
        if (l0 == l1) {
            const float D = __fadd_rn(__fsub_rn(onk, ok), (float)(pick3i(ln, d) - pick3i(lc, d)));
            if constexpr (SHAPE == PICA_SHAPE_TSC) {
                const float dl = __fsub_rn(ok, 0.5f);
                tscWeightsF(dl, s0[k]);
                ds[k][0] = __fmul_rn(D, __fadd_rn(__fmaf_rn(0.5f, D, dl), -0.5f));
                ds[k][1] = -__fmul_rn(D, __fmaf_rn(2.0f, dl, D));
                ds[k][2] = __fmul_rn(D, __fmaf_rn(0.5f, D, __fadd_rn(0.5f, dl)));
            } else {
                const float d0 = ok >= 0.5f ? ok - 0.5f : ok + 0.5f;
                s0[k][0] = 1.0f - d0; s0[k][1] = d0;
                ds[k][0] = -D;
                ds[k][1] = D;
            }
            s0[k][NWn] = 0.0f;
            ds[k][NWn] = 0.0f;
        } else {
            float w0[NWn], w1[NWn], s1[NW4];
            if constexpr (SHAPE == PICA_SHAPE_TSC) {
                tscWeightsF(__fsub_rn(ok, 0.5f), w0);
                tscWeightsF(__fsub_rn(onk, 0.5f), w1);
            } else {
                const bool h0 = ok >= 0.5f, h1 = onk >= 0.5f;
                const float d0 = h0 ? ok - 0.5f : ok + 0.5f, d1 = h1 ? onk - 0.5f : onk + 0.5f;
                w0[0] = 1.0f - d0; w0[1] = d0;
                w1[0] = 1.0f - d1; w1[1] = d1;
            }
            placeShape<float, NW4, NWn>(s0[k], l0, base, w0);
            placeShape<float, NW4, NWn>(s1, l1, base, w1);
#pragma unroll
            for (int i = 0; i < NW4; i++) ds[k][i] = __fsub_rn(s1[i], s0[k][i]);
        }
        b[k] = base + kG;
        len[k] = l0 == l1 ? NWn : NW4;   // |lo1 - lo0| <= 1: at most a third of a cell per step
        sp[k] = pick3i(st, d);
        cofs[k] = d * TT;
        kp[k] = pick3f(kq, d);
    }
    esirkepovRolled<NW4>(jt, cofs, sp, b, p, s0, ds, kp, len);
}

// Fixed-point tile addressed by shared-window byte addresses, for code that is
// not inlined into the kernel (the compiler then no longer knows that the tile
// is in shared memory): same arithmetic as FixTile::add.
struct FixTileS {
    unsigned lo, hi;
    float up, down;
    __device__ __forceinline__ void add(int idx, float scaled) const {
        const float r = rintf(scaled);
        const float h = floorf(r * down);
        const float l = fmaf(-h, up, r);
        const unsigned lu = __float_as_uint(l + 8388608.0f) - 0x4B000000u;
        const int hv = __float2int_rz(h);
        asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(lo + 4u * (unsigned)idx), "r"(lu) : "memory");
        asm volatile("red.shared.add.s32 [%0], %1;" ::"r"(hi + 4u * (unsigned)idx), "r"(hv) : "memory");
    }
};

constexpr int kRing = 32;  // queued cell changes per warp (one drain = one per lane)

// Deposit n <= 32 queued window changes of one warp starting at ring entry head,
// one per lane.  Out of line: one copy of the general-window code serves every
// call site.
template <int SHAPE>
__device__ __noinline__ void drainRing(unsigned ring, int head, int n, FixTileS jt, int TT, int T1, int T2) {
    const int k = threadIdx.x & 31;
    if (k >= n) return;
    const unsigned e = ring + 4u * (unsigned)(((head + k) & (kRing - 1)) * kQWords);
    float v[kQWords];
#pragma unroll
    for (int w = 0; w < kQWords; w++) asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v[w]) : "r"(e + 4u * w) : "memory");
    const int k0 = __float_as_int(v[9]), k1 = __float_as_int(v[10]);
    const int lc[3] = {(k0 >> 16) - 4, ((k0 >> 8) & 0xff) - 4, (k0 & 0xff) - 4};
    const int ln[3] = {(k1 >> 16) - 4, ((k1 >> 8) & 0xff) - 4, (k1 & 0xff) - 4};
    generalWindow<SHAPE>(jt, TT, T1, T2, v, v + 3, lc, ln, v + 6);
}

// Wrap a cell index that is at most one period out of range.
__device__ __forceinline__ int wrapNear(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// A warp's reduction area: 32 lane rows and 15 rows for sums parked when a lane
// changes cell, row r at red[r * kRowStride] (odd stride: a lane writing its row
// and lanes reading one value of a row are both free of bank conflicts).  While
// the segment runs the lane-row block is free and stages the segment's particle
// outputs (kStageWords), which are then written back with coalesced stores.
constexpr int kRedRows = 47;
constexpr int kRowStride = 57;
constexpr int kStageWords = 7 * 256;   // cell, ox, oy, oz, ux, uy, uz of 32 * K = 256 particles
static_assert(32 * kRowStride >= kStageWords, "the lane-row block holds a segment's outputs");

// Staging slot of component w of the particle of iteration it of a lane: iteration
// major, so the per-iteration writes of the 32 lanes and a lane's read-back of its
// own K particles are both free of bank conflicts.
__device__ __forceinline__ int stageIdx(int w, int it, int lane) { return w * 256 + it * 32 + lane; }

// Add up, per window key, the rows of a warp's reduction area (value j of row r
// at red[r * kRowStride + j]; keys[r] < 0: empty) and deposit the sums: lane t
// sums values t and t + 32 over the member rows, lane rows first (unless !lanes),
// then the np park rows, in ascending order.
template <int NWn, int NV>
__device__ __forceinline__ void reduceRows(const float* red, const int* keys, int np, bool lanes, const FixTile& jt,
                                           int TT, int T1, int T2, int lane) {
    const int kl = lanes ? keys[lane] : -1;
    const int kp = lane < np ? keys[32 + lane] : -1;
    unsigned pendL = __ballot_sync(0xffffffffu, kl >= 0);
    unsigned pendP = __ballot_sync(0xffffffffu, kp >= 0);
    const float* c0 = red + lane;
    const float* c1 = red + lane + 32;
    while (pendL | pendP) {
        const int ref = pendL ? __shfl_sync(0xffffffffu, kl, __ffs(pendL) - 1)
                              : __shfl_sync(0xffffffffu, kp, __ffs(pendP) - 1);
        const unsigned mL = __ballot_sync(0xffffffffu, kl == ref) & pendL;
        const unsigned mP = __ballot_sync(0xffffffffu, kp == ref) & pendP;
        pendL &= ~mL;
        pendP &= ~mP;
        // The member rows in a fixed order (lane rows ascending, then park rows in the
        // order taken), row k into partial sum k mod 4: four independent chains of
        // loads and adds instead of one, combined as (p0 + p1) + (p2 + p3).
        float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f, q0 = 0.f, q1 = 0.f, q2 = 0.f, q3 = 0.f;
        const bool hasHigh = lane + 32 < NV;
        unsigned mm[2] = {mL, mP};
#pragma unroll
        for (int part = 0; part < 2; part++) {
            unsigned m = mm[part];
            const int base = part == 0 ? 0 : 32;
            while (m) {
                int r[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    r[k] = m ? (base + __ffs(m) - 1) * kRowStride : -1;
                    m &= m - 1;
                }
                float v[4], w[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    v[k] = r[k] >= 0 ? c0[r[k]] : 0.f;
                    w[k] = r[k] >= 0 && hasHigh ? c1[r[k]] : 0.f;
                }
                p0 = __fadd_rn(p0, v[0]); p1 = __fadd_rn(p1, v[1]); p2 = __fadd_rn(p2, v[2]); p3 = __fadd_rn(p3, v[3]);
                q0 = __fadd_rn(q0, w[0]); q1 = __fadd_rn(q1, w[1]); q2 = __fadd_rn(q2, w[2]); q3 = __fadd_rn(q3, w[3]);
            }
        }
        const float s0 = __fadd_rn(__fadd_rn(p0, p1), __fadd_rn(p2, p3));
        const float s1 = __fadd_rn(__fadd_rn(q0, q1), __fadd_rn(q2, q3));
        const int b[3] = {(ref >> 16) - 4 + kG, ((ref >> 8) & 0xff) - 4 + kG, (ref & 0xff) - 4 + kG};
        if (lane < NV) jt.add(windowIdx<NWn>(TT, T1, T2, b, lane), s0);
        if (lane + 32 < NV) jt.add(windowIdx<NWn>(TT, T1, T2, b, lane + 32), s1);
    }
}

// Dynamic shared memory of k_push_cell_esirkepov, in 4-byte words.
__host__ __device__ constexpr int64_t esirkepovSmemWords(int TT, int ETT, int warps) {
    return 6ll * TT + 6ll * ETT + (int64_t)warps * (kRing * kQWords + kRedRows * kRowStride + kRedRows);
}
// The TMA variant's tensor copies land in the warps' reduction rows (free until the
// particle loop starts), 6 boxes of kTmaCompFloats from a 128-byte boundary.
static_assert(2 * kRedRows * kRowStride >= 6 * kTmaCompFloats + 31, "TMA staging fits two warps' reduction rows");

// Bounded wait on an mbarrier phase (parity): true once the phase completed, false
// when `limit` polls passed without it.
__device__ __forceinline__ bool mbarWait(unsigned mbar, unsigned parity, int limit) {
    for (int it = 0; it < limit; it++) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(mbar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}
constexpr int kTmaWaitPolls = 1 << 20;

// One supercell s of the plasma described by a, on the whole CTA (smem_raw: the
// dynamic shared memory, esirkepovSmemWords words).  SC > 0: cubic supercells of
// edge SC known at compile time (tile strides become constants); SC == 0: edges
// read from the arguments.
//
// TMA != 0 (cubic supercells of edge 4 only): interior supercells fetch the E/B
// tile with one tensor-memory-accelerator copy per component (maps: the six tensor
// maps, in kernel parameter space) into the warps' reduction rows, boxes with z
// rows of kTmaBoxZ floats and node m-1 at z index kTmaZOff; one shared-memory pass
// then packs them into the tile.  Supercells whose tile wraps around the periodic
// domain stage with plain loads.  Shared-memory footprint, park rows and so every
// rounding are those of the plain kernel.
template <int SHAPE, int K, int THREADS, int SC, class A, int TMA = 0>
__device__ __forceinline__ void pushSupercell(const A& a, const int s, unsigned char* smem_raw, int& s_nleave,
                                              const TmaFieldMaps* maps = nullptr) {
    static_assert(!TMA || SC == kTmaS, "the TMA variant has cubic supercells of edge 4");
    constexpr int NWn = kStayNodes;                        // stay-in-cell window: nodes lc-1 .. lc+1
    constexpr int NV = kStayValues;                        // 54 face values
    constexpr int kWarps = THREADS / 32;
    constexpr int kPark = kRedRows - 32;
    static_assert(K == 8, "a segment of 32 x 8 particles is staged in the lane-row block");
    constexpr unsigned FULL = 0xffffffffu;

    // Current tile: origin m - kG, edges S + 2kG + 1.  E/B tile: origin m - 1, edges S + 3.
    const int T1 = SC ? SC + 2 * kG + 1 : a.T[1], T2 = SC ? SC + 2 * kG + 1 : a.T[2];
    const int TT = (SC ? SC + 2 * kG + 1 : a.T[0]) * T1 * T2;
    const int Sx = SC ? SC : a.S[0], Sy = SC ? SC : a.S[1], Sz = SC ? SC : a.S[2];
    const int E1 = Sy + 3, E2 = Sz + 3, ETT = (Sx + 3) * E1 * E2;
    const int Sv[3] = {Sx, Sy, Sz};
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    FixTile jt;
    jt.lo = reinterpret_cast<unsigned int*>(smem_raw);
    jt.hi = reinterpret_cast<int*>(jt.lo + 3 * TT);
    jt.setSplit(a.tileSplit);
    float* eb = reinterpret_cast<float*>(jt.hi + 3 * TT);
    float* ring = eb + 6 * ETT + warp * (kRing * kQWords);
    float* red = eb + 6 * ETT + kWarps * (kRing * kQWords) + warp * (kRedRows * kRowStride);
    int* keys = reinterpret_cast<int*>(eb + 6 * ETT + kWarps * (kRing * kQWords + kRedRows * kRowStride)) + warp * kRedRows;
    uint32_t* stage = reinterpret_cast<uint32_t*>(red);   // the lane-row block, while a segment runs
    FixTileS jts;
    jts.lo = (unsigned)__cvta_generic_to_shared(jt.lo);
    jts.hi = (unsigned)__cvta_generic_to_shared(jt.hi);
    jts.up = jt.up;
    jts.down = jt.down;
    const unsigned ringS = (unsigned)__cvta_generic_to_shared(ring);

    int sc[3];
    sc[2] = s % a.nsc[2];
    sc[1] = (s / a.nsc[2]) % a.nsc[1];
    sc[0] = s / (a.nsc[1] * a.nsc[2]);
    const int m[3] = {sc[0] * Sx, sc[1] * Sy, sc[2] * Sz};

    // The TMA variant's interior supercells: tile nodes m-1 .. m+S+1 inside the grid
    // along every dimension (no periodic wrap), one tensor copy per component.
    bool viaTma = false;
    __shared__ __align__(8) unsigned long long s_mbar;
    const unsigned mbar = (unsigned)__cvta_generic_to_shared(&s_mbar);
    float* stg = eb + 6 * ETT + kWarps * (kRing * kQWords);   // the reduction rows, 128-byte aligned below
    if constexpr (TMA != 0) {
        static_assert(kWarps >= 2, "TMA staging uses the reduction rows of two warps");
        stg += ((128u - ((unsigned)__cvta_generic_to_shared(stg) & 127u)) & 127u) / 4u;
        viaTma = m[0] >= 1 && m[0] + Sx + 1 < a.n[0] && m[1] >= 1 && m[1] + Sy + 1 < a.n[1] && m[2] >= 1 &&
                 m[2] + Sz + 1 < a.n[2];
        if (viaTma && threadIdx.x == 0) {
            constexpr unsigned kBytes = 6u * kTmaBoxZ * (kTmaS + 3) * (kTmaS + 3) * 4u;
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(kBytes) : "memory");
            for (int c = 0; c < 6; c++) {
                const unsigned dst = (unsigned)__cvta_generic_to_shared(stg + c * kTmaCompFloats);
                // Box origin (z, y, x) = (m2 - 4, m1 - 1, m0 - 1): z a multiple of 4 floats.
                asm volatile(
                    "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
                    ::"r"(dst), "l"(reinterpret_cast<uint64_t>(&maps->m[c])), "r"(m[2] - 4), "r"(m[1] - 1), "r"(m[0] - 1),
                      "r"(mbar)
                    : "memory");
            }
        }
    }
    // Periodic grid index of tile node k along d (tile origin m - kG; k < 16 covers the
    // largest tile), so that the staging and flush loops need no modulo.
    __shared__ int s_wrap[3][16];
    if (threadIdx.x < 48) {
        const int d = threadIdx.x >> 4, k = threadIdx.x & 15;
        s_wrap[d][k] = wrapi(m[d] - kG + k, a.n[d]);
    }
    __syncthreads();
    if (!viaTma) {
        for (int t = threadIdx.x; t < 6 * ETT; t += THREADS) {
            const int c = t / ETT, r = t - c * ETT;
            const int i = r / (E1 * E2), jj = (r / E2) % E1, k = r % E2;   // E/B tile origin m - 1
            eb[t] = static_cast<const float*>(a.eb[c])[((int64_t)s_wrap[0][i + 1] * a.n[1] + s_wrap[1][jj + 1]) * a.n[2] +
                                                       s_wrap[2][k + 1]];
        }
    }
    for (int t = threadIdx.x; t < 3 * TT; t += THREADS) { jt.lo[t] = 0u; jt.hi[t] = 0; }
    const float invU = (float)a.invUnit;
    const float cdth[3] = {(float)a.cdth[0], (float)a.cdth[1], (float)a.cdth[2]};
    bool bad = false;
    int qN = 0;   // entries in this warp's queue of cell changes (warp-uniform)
    if (viaTma) {
        // Bounded wait for the copies.  If they never complete, report it, wait once
        // more (also bounded) for copies still in flight, and leave this supercell.
        bool ok = mbarWait(mbar, 0, kTmaWaitPolls);
        if (!ok) {
            if (threadIdx.x == 0) atomicExch(a.flags, PICA_ERR_TIMEOUT);
            ok = mbarWait(mbar, 0, kTmaWaitPolls);
        }
        if (__syncthreads_or(!ok)) return;
        for (int t = threadIdx.x; t < 6 * ETT; t += THREADS) {
            const int c = t / ETT, r = t - c * ETT;
            const int i = r / (E1 * E2), jj = (r / E2) % E1, k = r % E2;
            eb[t] = stg[c * kTmaCompFloats + (i * E1 + jj) * kTmaBoxZ + k + kTmaZOff];
        }
    }
    __syncthreads();

    for (int spi = 0; spi < a.nspecies; spi++) {
        const auto& sa = a.sp[spi];
        const int64_t start = sa.start[s];
        const int count = sa.count[s];
        const float ec = (float)sa.ec;
        const float kqs[3] = {(float)sa.kq[0] * invU, (float)sa.kq[1] * invU, (float)sa.kq[2] * invU};
        if (threadIdx.x == 0) s_nleave = 0;
        __syncthreads();
        // Work units: full segments of 32 K particles (lane l takes K consecutive
        // ones), except that the last (full segments mod 8) of them and the remainder
        // are re-cut into 8 equal sub-segments of 32 subK.  The cut depends only on
        // the count, so the particles summed together (and every rounding) are the
        // same for every CTA size, and the warps of a CTA of 2, 4 or 8 warps get the
        // same number of particle iterations.
        const int nmain = (count / (32 * K)) & ~7;
        const int rest = count - nmain * 32 * K;
        const int subK = (rest + 8 * 32 - 1) / (8 * 32);
        const int nunits = nmain + (rest > 0 ? 8 : 0);
        for (int unit = warp; unit < nunits; unit += kWarps) {
            const int kk = unit < nmain ? K : subK;
            const int segStart = unit < nmain ? unit * 32 * K : nmain * 32 * K + (unit - nmain) * 32 * subK;
            const int segEnd = min(count, segStart + 32 * kk);
            if (segStart >= segEnd) continue;
            float acc[NV];
#pragma unroll
            for (int k = 0; k < NV; k++) acc[k] = 0.0f;
            int accKey = -1;
            uint32_t accCell = kDeadCell;   // packed cell of the lane's window (same test as the key)
            int nPark = 0;   // warp-uniform
            const int i0 = segStart + lane * kk;
            // Particle data one iteration ahead.
            uint32_t pc = kDeadCell;
            float po[3] = {0.f, 0.f, 0.f}, pu[3] = {0.f, 0.f, 0.f}, pw = 0.f;
            if (i0 < segEnd) {
                const int64_t sl = start + i0;
                pc = sa.buf.cell[sl];
                po[0] = sa.buf.ox[sl]; po[1] = sa.buf.oy[sl]; po[2] = sa.buf.oz[sl];
                pu[0] = sa.buf.ux[sl]; pu[1] = sa.buf.uy[sl]; pu[2] = sa.buf.uz[sl];
                pw = sa.buf.w[sl];
            }
#pragma unroll 1
            for (int it = 0; it < kk; it++) {
                const int i = i0 + it;
                const int64_t slot = start + i;
                const uint32_t cellv = pc;
                const float o[3] = {po[0], po[1], po[2]};
                float u[3] = {pu[0], pu[1], pu[2]};
                const float wgt = pw;
                if (it + 1 < kk && i + 1 < segEnd) {
                    const int64_t sl = slot + 1;
                    pc = sa.buf.cell[sl];
                    po[0] = sa.buf.ox[sl]; po[1] = sa.buf.oy[sl]; po[2] = sa.buf.oz[sl];
                    pu[0] = sa.buf.ux[sl]; pu[1] = sa.buf.uy[sl]; pu[2] = sa.buf.uz[sl];
                    pw = sa.buf.w[sl];
                }
                const bool act = i < segEnd && cellv != kDeadCell;
                if (!act && i < segEnd) stage[stageIdx(0, it, lane)] = kDeadCell;   // stays dead
                int lc[3] = {0, 0, 0};
                int key = -1;
                if (act) {
                    int c3[3];
                    unpackCell(cellv, c3[0], c3[1], c3[2]);
                    int lw[3];
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        lc[d] = c3[d] - m[d];
                        lw[d] = lc[d] - 1;
                    }
                    key = ((lw[0] + 4) << 16) | ((lw[1] + 4) << 8) | (lw[2] + 4);
                }
                // A lane meeting another window parks its sums in a park row; when the park
                // rows run out the warp deposits them and goes on parking.
                // A lone particle of another window -- the lane has no next particle, or
                // the next one is in yet another cell: a particle out of cell order since
                // the last resort, or one of the arrivals that the migration appends to a
                // supercell, each in its own cell -- goes to the cell-change queue instead
                // of costing the lane a park (two when the lane's window comes back).
                const bool lone = act && key != accKey && accKey >= 0 &&
                                  (it + 1 >= kk || i + 1 >= segEnd || pc != cellv);
                const bool sw = act && key != accKey && !lone;
                const bool park = sw && accKey >= 0;
                unsigned rem = __ballot_sync(FULL, park);
                while (rem) {
                    if (nPark == kPark) {
                        reduceRows<NWn, NV>(red, keys, nPark, false, jt, TT, T1, T2, lane);
                        __syncwarp();
                        nPark = 0;
                    }
                    const int rank = __popc(rem & lt);
                    const bool mine = ((rem >> lane) & 1u) && rank < kPark - nPark;
                    const unsigned now = __ballot_sync(FULL, mine);
                    if (mine) {
                        const int row = 32 + nPark + rank;
#pragma unroll
                        for (int j = 0; j < NV; j++) red[row * kRowStride + j] = acc[j];
                        keys[row] = accKey;
                    }
                    nPark += __popc(now);
                    rem &= ~now;
                    __syncwarp();
                }
                if (sw) {
#pragma unroll
                    for (int j = 0; j < NV; j++) acc[j] = 0.0f;
                    accKey = key;
                    accCell = cellv;
                }
                bool needQ = false;
                float qe[kQWords];
                if (act) {
                    float eb6[6];
                    if constexpr (SHAPE == PICA_SHAPE_CIC) {
                        int bc[3], bs[3];
                        float wc[3][2], ws[3][2];
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            bc[d] = lc[d] + 1; wc[d][0] = 1.0f - o[d]; wc[d][1] = o[d];
                            const bool hi = o[d] >= 0.5f;
                            const float dd = hi ? o[d] - 0.5f : o[d] + 0.5f;
                            bs[d] = hi ? lc[d] + 1 : lc[d]; ws[d][0] = 1.0f - dd; ws[d][1] = dd;
                        }
#pragma unroll
                        for (int cp = 0; cp < 6; cp += 2) {   // (Ex, Ey), (Ez, Bx), (By, Bz)
                            int ta[3], tb[3];
#pragma unroll
                            for (int d = 0; d < 3; d++) {
                                ta[d] = stag(cp, d) ? bs[d] : bc[d];
                                tb[d] = stag(cp + 1, d) ? bs[d] : bc[d];
                            }
                            const float2 g = gatherPair<2>(
                                eb + cp * ETT, eb + (cp + 1) * ETT, E1, E2, ta, tb, stag(cp, 0) ? ws[0] : wc[0],
                                stag(cp, 1) ? ws[1] : wc[1], stag(cp, 2) ? ws[2] : wc[2], stag(cp + 1, 0) ? ws[0] : wc[0],
                                stag(cp + 1, 1) ? ws[1] : wc[1], stag(cp + 1, 2) ? ws[2] : wc[2]);
                            eb6[cp] = g.x;
                            eb6[cp + 1] = g.y;
                        }
                    } else {
                        int bc[3], bs[3];
                        float wc[3][3], ws[3][3];
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            const bool hi = o[d] >= 0.5f;
                            bc[d] = lc[d] + (hi ? 1 : 0); tscWeightsF(hi ? __fsub_rn(o[d], 1.0f) : o[d], wc[d]);
                            bs[d] = lc[d]; tscWeightsF(__fsub_rn(o[d], 0.5f), ws[d]);
                        }
#pragma unroll
                        for (int cp = 0; cp < 6; cp += 2) {   // (Ex, Ey), (Ez, Bx), (By, Bz)
                            int ta[3], tb[3];
#pragma unroll
                            for (int d = 0; d < 3; d++) {
                                ta[d] = stag(cp, d) ? bs[d] : bc[d];
                                tb[d] = stag(cp + 1, d) ? bs[d] : bc[d];
                            }
                            const float2 g = gatherPair<3>(
                                eb + cp * ETT, eb + (cp + 1) * ETT, E1, E2, ta, tb, stag(cp, 0) ? ws[0] : wc[0],
                                stag(cp, 1) ? ws[1] : wc[1], stag(cp, 2) ? ws[2] : wc[2], stag(cp + 1, 0) ? ws[0] : wc[0],
                                stag(cp + 1, 1) ? ws[1] : wc[1], stag(cp + 1, 2) ? ws[2] : wc[2]);
                            eb6[cp] = g.x;
                            eb6[cp + 1] = g.y;
                        }
                    }
                    const float ig = borisFast(ec, eb6, u);
                    int ln[3];
                    float on[3];
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        float onew = __fmaf_rn(__fmul_rn(u[d], ig), cdth[d], o[d]);
                        const float fl = floorf(onew);
                        ln[d] = lc[d] + (int)fl;
                        onew = onew - fl;
                        if (onew >= 1.0f) { onew -= 1.0f; ln[d] += 1; }
                        on[d] = onew;
                    }
                    bool inRange = true;
#pragma unroll
                    for (int d = 0; d < 3; d++)
                        inRange = inRange && ln[d] >= -1 && ln[d] <= Sv[d] && abs(ln[d] - lc[d]) <= 1 &&
                                  on[d] >= 0.0f && on[d] < 1.0f;
                    if (!inRange) {
                        bad = true;
#pragma unroll
                        for (int d = 0; d < 3; d++) { ln[d] = lc[d]; on[d] = o[d]; }
                    }
                    const float kq[3] = {__fmul_rn(kqs[0], wgt), __fmul_rn(kqs[1], wgt), __fmul_rn(kqs[2], wgt)};
                    const bool sameWindow = !lone && inRange && ln[0] == lc[0] && ln[1] == lc[1] && ln[2] == lc[2];
                    if (sameWindow) {
                        // Old shape S0 and its change dd = S1 - S0 on the rho-lattice nodes lc-1 ..
                        // lc+1 of the cell.  TSC: weights of o - 1/2 on all three.  CIC: nodes base,
                        // base+1 with base = lc or lc-1 by o >= 1/2, the third weight 0.  dd is
                        // written in factored form from the displacement D = on - o, not as the
                        // difference of two shapes: a step moves a particle by about 1% of a cell,
                        // and S1 - S0 in FP32 would keep only the bits of D above 2^-24 of the
                        // weights, a few 1e-6 of dd (the charge-conservation residual).
                        // p = a + d/2, q = a/2 + d/3; yz = a_y p_z + d_y q_z.
                        float aa[3][NWn], dd[3][NWn], pp[3][NWn], qq[3][NWn];
#pragma unroll
                        // Every rounding is spelled out (_rn intrinsics, which the compiler does not
                        // contract), so that every instantiation of this code -- launch variants,
                        // the batching form -- rounds the same way.
                        for (int d = 0; d < 3; d++) {
                            const float D = __fsub_rn(on[d], o[d]);
                            if constexpr (SHAPE == PICA_SHAPE_TSC) {
                                const float dl = __fsub_rn(o[d], 0.5f);
                                tscWeightsF(dl, aa[d]);
                                dd[d][0] = __fmul_rn(D, __fadd_rn(__fmaf_rn(0.5f, D, dl), -0.5f));
                                dd[d][1] = -__fmul_rn(D, __fmaf_rn(2.0f, dl, D));
                                dd[d][2] = __fmul_rn(D, __fmaf_rn(0.5f, D, __fadd_rn(0.5f, dl)));
                            } else {
                                const bool h0 = o[d] >= 0.5f, h1 = on[d] >= 0.5f;
                                const float d0 = h0 ? o[d] - 0.5f : o[d] + 0.5f;
                                aa[d][0] = h0 ? 0.0f : 1.0f - d0; aa[d][1] = h0 ? 1.0f - d0 : d0; aa[d][2] = h0 ? d0 : 0.0f;
                                // Same half: the shape slides by D.  Across the centre: a = o - 1/2 and
                                // b = on - 1/2 are both near zero and exact.
                                const float a = __fsub_rn(o[d], 0.5f), b = __fsub_rn(on[d], 0.5f);
                                const float ab = __fadd_rn(a, b);
                                if (h0 == h1) {
                                    dd[d][0] = h0 ? 0.0f : -D; dd[d][1] = h0 ? -D : D; dd[d][2] = h0 ? D : 0.0f;
                                } else {
                                    dd[d][0] = h1 ? a : -b; dd[d][2] = h1 ? b : -a; dd[d][1] = h1 ? -ab : ab;
                                }
                            }
#pragma unroll
                            for (int k = 0; k < NWn; k++) {
                                pp[d][k] = __fmaf_rn(0.5f, dd[d][k], aa[d][k]);
                                qq[d][k] = __fmaf_rn((float)kThird, dd[d][k], __fmul_rn(0.5f, aa[d][k]));
                            }
                        }
                        // e[d][f]: -(q w) h_d/dt times the running sum of dd over faces 0..f, that is
                        // dd[0] and dd[0] + dd[1] = -dd[2] (the sum of dd is zero; no cancellation).
                        float e[3][NWn - 1];
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            e[d][0] = __fmul_rn(kq[d], dd[d][0]);
                            e[d][1] = -__fmul_rn(kq[d], dd[d][2]);
                        }
                        // Jx and Jy share the z factors (pp2, qq2): their terms and sums go in
                        // packed FP32x2 pairs (each half rounds as the scalar form); Jz alone.
                        constexpr int P = (NWn - 1) * NWn * NWn;
                        float2 ad[NWn], dd01[NWn], ef[NWn - 1];
#pragma unroll
                        for (int y = 0; y < NWn; y++) {
                            ad[y] = make_float2(aa[1][y], aa[0][y]);
                            dd01[y] = make_float2(dd[1][y], dd[0][y]);
                        }
#pragma unroll
                        for (int f = 0; f < NWn - 1; f++) ef[f] = make_float2(e[0][f], e[1][f]);
#pragma unroll
                        for (int z = 0; z < NWn; z++) {
                            const float2 p2 = make_float2(pp[2][z], pp[2][z]), q2 = make_float2(qq[2][z], qq[2][z]);
#pragma unroll
                            for (int y = 0; y < NWn; y++) {
                                const float2 t = __ffma2_rn(dd01[y], q2, __fmul2_rn(ad[y], p2));
#pragma unroll
                                for (int f = 0; f < NWn - 1; f++) {
                                    float2 s2 = make_float2(acc[f * NWn * NWn + y * NWn + z], acc[P + y * (NWn - 1) * NWn + f * NWn + z]);
                                    s2 = __ffma2_rn(ef[f], t, s2);
                                    acc[f * NWn * NWn + y * NWn + z] = s2.x;
                                    acc[P + y * (NWn - 1) * NWn + f * NWn + z] = s2.y;
                                }
                            }
                        }
#pragma unroll
                        for (int f = 0; f < NWn - 1; f++)
#pragma unroll
                            for (int y = 0; y < NWn; y++)
#pragma unroll
                                for (int z = 0; z < NWn; z++)
                                    acc[2 * P + y * NWn * (NWn - 1) + z * (NWn - 1) + f] =
                                        __fmaf_rn(e[2][f], __fmaf_rn(dd[0][y], qq[1][z], __fmul_rn(aa[0][y], pp[1][z])),
                                                  acc[2 * P + y * NWn * (NWn - 1) + z * (NWn - 1) + f]);
                    } else if (inRange) {
                        needQ = true;
#pragma unroll
                        for (int d = 0; d < 3; d++) { qe[d] = o[d]; qe[3 + d] = on[d]; qe[6 + d] = kq[d]; }
                        qe[9] = __int_as_float(((lc[0] + 4) << 16) | ((lc[1] + 4) << 8) | (lc[2] + 4));
                        qe[10] = __int_as_float(((ln[0] + 4) << 16) | ((ln[1] + 4) << 8) | (ln[2] + 4));
                    }
                    // New cell (periodic) and the move's direction code, from the wrapped
                    // supercell coordinates (with one or two supercells along a dimension
                    // the periodic +1 and -1 neighbours coincide; dirCode resolves that
                    // the same way the oracle does).
                    // A particle still inside the supercell stays (code 13) and needs no wrap.
                    int gc[3];
                    int code = 13;
                    if (ln[0] >= 0 && ln[0] < Sv[0] && ln[1] >= 0 && ln[1] < Sv[1] && ln[2] >= 0 && ln[2] < Sv[2]) {
#pragma unroll
                        for (int d = 0; d < 3; d++) gc[d] = m[d] + ln[d];
                    } else {
                        int nsc3[3];
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            gc[d] = wrapNear(m[d] + ln[d], a.n[d]);
                            nsc3[d] = gc[d] / Sv[d];
                        }
                        code = dirCode(sc, nsc3, a.nsc, bad);
                    }
                    // Stayers in place (the weight does not change); a leaver goes to the side
                    // buffer, its slot dies and joins the leaver list.
                    const uint32_t pc2 = packCell(gc[0], gc[1], gc[2]);
                    // staged; written back at the end of the segment
                    stage[stageIdx(0, it, lane)] = code == 13 ? pc2 : kDeadCell;
                    stage[stageIdx(1, it, lane)] = __float_as_uint(on[0]);
                    stage[stageIdx(2, it, lane)] = __float_as_uint(on[1]);
                    stage[stageIdx(3, it, lane)] = __float_as_uint(on[2]);
                    stage[stageIdx(4, it, lane)] = __float_as_uint(u[0]);
                    stage[stageIdx(5, it, lane)] = __float_as_uint(u[1]);
                    stage[stageIdx(6, it, lane)] = __float_as_uint(u[2]);
                    if (code != 13) {
                        const int k = atomicAdd(&s_nleave, 1);
                        const int64_t o = start + k;   // leaver records are packed (see pica_internal.h)
                        sa.out.cell[o] = pc2;
                        sa.out.ox[o] = on[0]; sa.out.oy[o] = on[1]; sa.out.oz[o] = on[2];
                        sa.out.ux[o] = u[0]; sa.out.uy[o] = u[1]; sa.out.uz[o] = u[2];
                        sa.out.w[o] = wgt;
                        sa.dir[slot] = (uint32_t)code | ((uint32_t)k << 5);
                        sa.llist[o] = i;
                    }
                }
                // Queue window changes in the ring; deposit 32 at a time (one per lane).
                const unsigned qm = __ballot_sync(FULL, needQ);
                if (qm) {
                    if (qN + __popc(qm) > kRing) {   // no room: deposit what is queued
                        drainRing<SHAPE>(ringS, 0, qN, jts, TT, T1, T2);
                        __syncwarp();
                        qN = 0;
                    }
                    if (needQ) {
                        float* e = ring + (qN + __popc(qm & lt)) * kQWords;
#pragma unroll
                        for (int k = 0; k < kQWords; k++) e[k] = qe[k];
                    }
                    qN += __popc(qm);
                    __syncwarp();
                    if (qN == kRing) {
                        drainRing<SHAPE>(ringS, 0, kRing, jts, TT, T1, T2);
                        __syncwarp();
                        qN = 0;
                    }
                }
            }
            // Write the segment's particles back: cell, offsets, momenta (the weight does
            // not change; leavers went to the side buffer).  A full segment: every lane
            // stores its own K consecutive particles with 16-byte stores (a supercell's
            // slots start on a 128-byte boundary, so do full segments); otherwise one
            // particle per lane and store, consecutive across the lanes.
            __syncwarp();
            {
                const int nValid = segEnd - segStart;
                const int64_t base = start + segStart;
                uint32_t* const dst[7] = {sa.buf.cell, reinterpret_cast<uint32_t*>(sa.buf.ox),
                                          reinterpret_cast<uint32_t*>(sa.buf.oy), reinterpret_cast<uint32_t*>(sa.buf.oz),
                                          reinterpret_cast<uint32_t*>(sa.buf.ux), reinterpret_cast<uint32_t*>(sa.buf.uy),
                                          reinterpret_cast<uint32_t*>(sa.buf.uz)};
                if (kk == K && nValid == 32 * K && (base & 3) == 0) {
                    const int64_t o = base + lane * K;
#pragma unroll
                    for (int w = 0; w < 7; w++) {
                        uint4 v0, v1;
                        v0.x = stage[stageIdx(w, 0, lane)]; v0.y = stage[stageIdx(w, 1, lane)];
                        v0.z = stage[stageIdx(w, 2, lane)]; v0.w = stage[stageIdx(w, 3, lane)];
                        v1.x = stage[stageIdx(w, 4, lane)]; v1.y = stage[stageIdx(w, 5, lane)];
                        v1.z = stage[stageIdx(w, 6, lane)]; v1.w = stage[stageIdx(w, 7, lane)];
                        *reinterpret_cast<uint4*>(dst[w] + o) = v0;
                        *reinterpret_cast<uint4*>(dst[w] + o + 4) = v1;
                    }
                } else {
                    for (int p = lane; p < nValid; p += 32) {
                        const int l = p / kk, it = p - l * kk;
#pragma unroll
                        for (int w = 0; w < 7; w++) dst[w][base + p] = stage[stageIdx(w, it, l)];
                    }
                }
            }
            __syncwarp();
            // Deposit the segment's window sums: lane rows plus parked rows, by window.
#pragma unroll
            for (int j = 0; j < NV; j++) red[lane * kRowStride + j] = acc[j];
            keys[lane] = accKey;
            __syncwarp();
            reduceRows<NWn, NV>(red, keys, nPark, true, jt, TT, T1, T2, lane);
            __syncwarp();
        }
        __syncthreads();
        if (threadIdx.x == 0) sa.nleave[s] = s_nleave;
        __syncthreads();
    }
    if (qN > 0) drainRing<SHAPE>(ringS, 0, qN, jts, TT, T1, T2);
    if (bad) atomicExch(a.flags, PICA_ERR_MIGRATION);
    __syncthreads();
    for (int t = threadIdx.x; t < 3 * TT; t += THREADS) {
        const unsigned long long v = (unsigned long long)jt.node(t);
        if (v != 0ull) {
            const int c = t / TT, r = t - c * TT;
            const int i = r / (T1 * T2), jj = (r / T2) % T1, k = r % T2;
            atomicAdd(a.jacc[c] + ((int64_t)s_wrap[0][i] * a.n[1] + s_wrap[1][jj]) * a.n[2] + s_wrap[2][k], v);
        }
    }
}

template <int SHAPE, int K, int THREADS, int MINB, int SC>
__global__ void __launch_bounds__(THREADS, MINB) k_push_cell_esirkepov(const __grid_constant__ PushArgsSlim<kMaxSpecies> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_nleave;
    pushSupercell<SHAPE, K, THREADS, SC>(a, a.scOffset + (int)blockIdx.x, smem_raw, s_nleave);
}

// The same push with the E/B tile of interior supercells staged by TMA (launch
// variant 4; cubic supercells of edge 4).
template <int SHAPE, int K, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB)
    k_push_cell_esirkepov_tma(const __grid_constant__ PushArgsSlim<kMaxSpecies> a, const __grid_constant__ TmaFieldMaps maps) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ int s_nleave;
    pushSupercell<SHAPE, K, THREADS, kTmaS, PushArgsSlim<kMaxSpecies>, 1>(a, a.scOffset + (int)blockIdx.x, smem_raw,
                                                                        s_nleave, &maps);
}

// Batching form: one persistent launch over the supercells of many independent
// plasmas.  Each CTA takes the next work item from b.counter (zeroed before the
// launch) and finds its plasma by binary search over b.base; the plasma's
// arguments are read from the kernel parameters.
template <int SHAPE, int K, int THREADS, int MINB, int SC, int NSP>
__global__ void __launch_bounds__(THREADS, MINB) k_push_batch(const __grid_constant__ BatchPushArgs<NSP> b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_nleave;
    __shared__ int s_work;
    for (;;) {
        __syncthreads();   // the previous work item is done with the shared memory
        if (threadIdx.x == 0) s_work = atomicAdd(b.counter, 1);
        __syncthreads();
        const int w = s_work;
        if (w >= b.total) return;
        int lo = 0, hi = b.count;   // largest k with base[k] <= w
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (b.base[mid] <= w) lo = mid; else hi = mid;
        }
        pushSupercell<SHAPE, K, THREADS, SC>(b.members[lo], w - b.base[lo], smem_raw, s_nleave);
    }
}

}  // namespace pgb
