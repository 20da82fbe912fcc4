/*
 * pic_oracle.cpp -- CPU restatement of pica's particle-in-cell step.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for pica_gb300 and the timed CPU
 * baseline.  Nothing in the product links or calls this file.
 *
 * What it restates (all paths relative to the pica project root):
 *   - Yee grid layout and staggering         include/pica/grid/YeeGrid.h:11-14,247-255
 *   - Yee E/B update (3D interior stencil)   include/pica/fieldSolver/YeeSolver.h:132-213
 *   - CIC supercell interpolator             include/pica/fieldInterpolation/FieldInterpolatorYeeGrid.h:197-281
 *   - Boris pusher                           include/pica/particlePush/BorisPusher.h:23-47
 *   - SoA velocity / inverse gamma           include/pica/particles/ParticleArray.h:122-149,263,311-317
 *   - CIC supercell direct depositor         include/pica/currentDeposition/CurrentDepositorYeeGrid.h:178-262
 *   - supercell routing (floor)              include/pica/particles/EnsembleSupercells.h:25-57
 *   - flat (unordered) push, grid-level CIC  include/pica/fieldInterpolation/FieldInterpolatorYeeGrid.h:23-38,137-183
 *                                            include/pica/currentDeposition/CurrentDepositorYeeGrid.h:23-38,126-163
 *   - ordered ensemble sort                  include/pica/particles/EnsembleOrdered.h:31-41,61-71
 * The FP64 CIC/direct path reproduces the reference's floating-point
 * expressions term by term (compile with -ffp-contract=off) and is checked
 * bit-exactly against oracle/ref_harness.cpp, which drives pica's own headers.
 *
 * What pica does not have and is written here from the published methods:
 *   - TSC (quadratic B-spline) gather and direct deposit: Hockney & Eastwood,
 *     "Computer Simulation Using Particles", ch. 5.
 *   - Esirkepov charge-conserving deposition: T.Zh. Esirkepov,
 *     Comput. Phys. Commun. 135 (2001) 144, eqs. (21)-(23), on pica's dual
 *     Yee lattice (J on faces, rho at cell centres).
 *   - periodic boundaries (guard fill / guard fold on a grid padded with
 *     origin -2h, as pica's supercell helpers require), the step order,
 *     supercell migration in a canonical order, and FP64 diagnostics.
 *   - the FP32 precision form: integer cell index + FP32 in-cell offset.
 */
#include "pic_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kPi = 3.14159265358;   // pica math/Constants.h:10 (truncated value)
const double kC = 29979245800.0;    // pica math/Constants.h:11
const int kLo = 2;                  // padded grid: origin at -2h
const int kHi = 3;                  // high-side guard nodes (TSC reaches N+2)
const int kG = 2;                   // supercell tile guard: tile base node = m - 2
const double kThird = 1.0 / 3.0;

inline int wrapi(int a, int n) { a %= n; return a < 0 ? a + n : a; }

// ----------------------------------------------------------------------------
// Padded periodic grid (9 components) in precision R.
// ----------------------------------------------------------------------------
template <typename R>
struct Grid {
    int n[3], sz[3];
    std::vector<R> f[9];  // ex ey ez bx by bz jx jy jz
    void init(const int* nn) {
        for (int d = 0; d < 3; d++) { n[d] = nn[d]; sz[d] = nn[d] + kLo + kHi; }
        for (auto& a : f) a.assign((size_t)sz[0] * sz[1] * sz[2], R(0));
    }
    size_t at(int gx, int gy, int gz) const { return ((size_t)gx * sz[1] + gy) * sz[2] + gz; }
    bool guard(int gx, int gy, int gz) const {
        return gx < kLo || gy < kLo || gz < kLo || gx >= n[0] + kLo || gy >= n[1] + kLo || gz >= n[2] + kLo;
    }
    size_t image(int gx, int gy, int gz) const {
        return at(wrapi(gx - kLo, n[0]) + kLo, wrapi(gy - kLo, n[1]) + kLo, wrapi(gz - kLo, n[2]) + kLo);
    }
    // Periodic guard fill: every guard node takes the value of its interior image.
    void fill(int c0, int c1) {
        for (int gx = 0; gx < sz[0]; gx++)
            for (int gy = 0; gy < sz[1]; gy++)
                for (int gz = 0; gz < sz[2]; gz++)
                    if (guard(gx, gy, gz)) {
                        size_t g = at(gx, gy, gz), i = image(gx, gy, gz);
                        for (int c = c0; c < c1; c++) f[c][g] = f[c][i];
                    }
    }
    // Periodic guard fold of J: guard nodes are added to their interior image in linear order.
    void fold() {
        for (int gx = 0; gx < sz[0]; gx++)
            for (int gy = 0; gy < sz[1]; gy++)
                for (int gz = 0; gz < sz[2]; gz++)
                    if (guard(gx, gy, gz)) {
                        size_t g = at(gx, gy, gz), i = image(gx, gy, gz);
                        for (int c = 6; c < 9; c++) { f[c][i] += f[c][g]; f[c][g] = R(0); }
                    }
    }
    // E += -4 pi dt J + c dt curl B on the padded interior range [0, sz-1):
    // YeeSolver.h:140-155 (the outer-plane "edge" loops only touch guard planes).
    void updateE(R cc, R cx, R cy, R cz) {
        std::vector<R>&ex = f[0], &ey = f[1], &ez = f[2], &bx = f[3], &by = f[4], &bz = f[5];
        std::vector<R>&jx = f[6], &jy = f[7], &jz = f[8];
#pragma omp parallel for collapse(2)
        for (int i = 0; i < sz[0] - 1; i++)
            for (int j = 0; j < sz[1] - 1; j++)
                for (int k = 0; k < sz[2] - 1; k++) {
                    size_t o = at(i, j, k), oxp = at(i + 1, j, k), oyp = at(i, j + 1, k), ozp = at(i, j, k + 1);
                    ex[o] += cc * jx[o] + cy * (bz[oyp] - bz[o]) - cz * (by[ozp] - by[o]);
                    ey[o] += cc * jy[o] + cz * (bx[ozp] - bx[o]) - cx * (bz[oxp] - bz[o]);
                    ez[o] += cc * jz[o] + cx * (by[oxp] - by[o]) - cy * (bx[oyp] - bx[o]);
                }
    }
    // B -= c dt curl E on the padded range [1, sz): YeeSolver.h:184-196.
    void updateB(R cx, R cy, R cz) {
        std::vector<R>&ex = f[0], &ey = f[1], &ez = f[2], &bx = f[3], &by = f[4], &bz = f[5];
#pragma omp parallel for collapse(2)
        for (int i = 1; i < sz[0]; i++)
            for (int j = 1; j < sz[1]; j++)
                for (int k = 1; k < sz[2]; k++) {
                    size_t o = at(i, j, k), oxm = at(i - 1, j, k), oym = at(i, j - 1, k), ozm = at(i, j, k - 1);
                    bx[o] += cz * (ey[o] - ey[ozm]) - cy * (ez[o] - ez[oym]);
                    by[o] += cx * (ez[o] - ez[oxm]) - cz * (ex[o] - ex[ozm]);
                    bz[o] += cy * (ex[o] - ex[oym]) - cx * (ey[o] - ey[oxm]);
                }
    }
};

// ----------------------------------------------------------------------------
// Form factors.
// ----------------------------------------------------------------------------
template <typename R>
inline void tscWeights(R d, R* w) {
    const R h = R(0.5);
    w[0] = h * (h - d) * (h - d);
    w[1] = R(0.75) - d * d;
    w[2] = h * (h + d) * (h + d);
}

// Separable gather over an (order)^3 stencil starting at tile index t0:
// r = sum_i wx_i * sum_j wy_j * (sum_k wz_k F[i][j][k]), each sum left to right.
template <typename R, int W>
inline R gatherSep(const R* tile, int T, const int* t0, const R* wx, const R* wy, const R* wz) {
    R r = R(0);
    for (int i = 0; i < W; i++) {
        R ry = R(0);
        for (int j = 0; j < W; j++) {
            const R* row = tile + ((size_t)(t0[0] + i) * T + (t0[1] + j)) * T + t0[2];
            R rz = row[0] * wz[0];
            for (int k = 1; k < W; k++) rz = rz + row[k] * wz[k];
            ry = ry + wy[j] * rz;
        }
        r = r + wx[i] * ry;
    }
    return r;
}

template <typename R, int W>
inline void scatterSep(R* tile, int T, const int* t0, const R* wx, const R* wy, const R* wz, R v) {
    for (int i = 0; i < W; i++)
        for (int j = 0; j < W; j++) {
            R* row = tile + ((size_t)(t0[0] + i) * T + (t0[1] + j)) * T + t0[2];
            R vij = (v * wx[i]) * wy[j];
            for (int k = 0; k < W; k++) row[k] += vij * wz[k];
        }
}

// Esirkepov deposit of one particle on a tile.  s0/s1: old/new shape on the
// rho lattice in a window of NW nodes starting at tile index b (per dim);
// k[d] = -(q w) h_d / dt; contributions are unnormalised (x h^3).
template <typename R, int NW>
inline void esirkepov(R* jx, R* jy, R* jz, int T, const int* b, const R (*s0)[NW], const R (*s1)[NW],
                      const R* k) {
    R ds[3][NW];
    for (int d = 0; d < 3; d++)
        for (int i = 0; i < NW; i++) ds[d][i] = s1[d][i] - s0[d][i];
    const R hf = R(0.5), th = R(kThird);
    // Jx: faces between rho nodes i and i+1 along x (pica Jx node index b_x + i + 1).
    for (int j = 0; j < NW; j++)
        for (int l = 0; l < NW; l++) {
            R yz = s0[1][j] * s0[2][l] + hf * (ds[1][j] * s0[2][l] + s0[1][j] * ds[2][l]) + th * (ds[1][j] * ds[2][l]);
            R acc = R(0);
            for (int i = 0; i < NW - 1; i++) {
                acc = acc + ds[0][i] * yz;
                jx[((size_t)(b[0] + i + 1) * T + (b[1] + j)) * T + (b[2] + l)] += acc * k[0];
            }
        }
    for (int i = 0; i < NW; i++)
        for (int l = 0; l < NW; l++) {
            R xz = s0[0][i] * s0[2][l] + hf * (ds[0][i] * s0[2][l] + s0[0][i] * ds[2][l]) + th * (ds[0][i] * ds[2][l]);
            R acc = R(0);
            for (int j = 0; j < NW - 1; j++) {
                acc = acc + ds[1][j] * xz;
                jy[((size_t)(b[0] + i) * T + (b[1] + j + 1)) * T + (b[2] + l)] += acc * k[1];
            }
        }
    for (int i = 0; i < NW; i++)
        for (int j = 0; j < NW; j++) {
            R xy = s0[0][i] * s0[1][j] + hf * (ds[0][i] * s0[1][j] + s0[0][i] * ds[1][j]) + th * (ds[0][i] * ds[1][j]);
            R acc = R(0);
            for (int l = 0; l < NW - 1; l++) {
                acc = acc + ds[2][l] * xy;
                jz[((size_t)(b[0] + i) * T + (b[1] + j)) * T + (b[2] + l + 1)] += acc * k[2];
            }
        }
}

// Place a 2- or 3-point shape (weights w at lowest node lo) in a window starting at base.
template <typename R, int NW, int P>
inline void placeShape(R* s, int lo, int base, const R* w) {
    for (int i = 0; i < NW; i++) s[i] = R(0);
    for (int i = 0; i < P; i++) s[lo - base + i] = w[i];
}

// ----------------------------------------------------------------------------
// Particle stores.
// ----------------------------------------------------------------------------
// Dead slots (left by particles that moved to another supercell) are marked
// x = -1e300 (FP64 form; positions are never below -L, even before the
// periodic wrap) or cx = -1 (FP32 form).
const double kDeadX = -1.0e300;
struct PlainStore {  // FP64 absolute positions, normalised momentum u = p/(mc)
    std::vector<double> x, y, z, ux, uy, uz, w;
    size_t size() const { return w.size(); }
    void clear() { x.clear(); y.clear(); z.clear(); ux.clear(); uy.clear(); uz.clear(); w.clear(); }
    void append(const PlainStore& s, size_t i) {
        x.push_back(s.x[i]); y.push_back(s.y[i]); z.push_back(s.z[i]);
        ux.push_back(s.ux[i]); uy.push_back(s.uy[i]); uz.push_back(s.uz[i]); w.push_back(s.w[i]);
    }
    void set(size_t k, const PlainStore& s, size_t i) {
        x[k] = s.x[i]; y[k] = s.y[i]; z[k] = s.z[i]; ux[k] = s.ux[i]; uy[k] = s.uy[i]; uz[k] = s.uz[i]; w[k] = s.w[i];
    }
    bool alive(size_t i) const { return x[i] > -1.0e299; }
    void kill(size_t i) { x[i] = kDeadX; }
};
struct CellStore {  // FP32 form: integer cell + FP32 offset in [0,1)
    std::vector<int32_t> cx, cy, cz;
    std::vector<float> ox, oy, oz, ux, uy, uz, w;
    size_t size() const { return w.size(); }
    void clear() { cx.clear(); cy.clear(); cz.clear(); ox.clear(); oy.clear(); oz.clear(); ux.clear(); uy.clear(); uz.clear(); w.clear(); }
    void append(const CellStore& s, size_t i) {
        cx.push_back(s.cx[i]); cy.push_back(s.cy[i]); cz.push_back(s.cz[i]);
        ox.push_back(s.ox[i]); oy.push_back(s.oy[i]); oz.push_back(s.oz[i]);
        ux.push_back(s.ux[i]); uy.push_back(s.uy[i]); uz.push_back(s.uz[i]); w.push_back(s.w[i]);
    }
    void set(size_t k, const CellStore& s, size_t i) {
        cx[k] = s.cx[i]; cy[k] = s.cy[i]; cz[k] = s.cz[i]; ox[k] = s.ox[i]; oy[k] = s.oy[i]; oz[k] = s.oz[i];
        ux[k] = s.ux[i]; uy[k] = s.uy[i]; uz[k] = s.uz[i]; w[k] = s.w[i];
    }
    bool alive(size_t i) const { return cx[i] >= 0; }
    void kill(size_t i) { cx[i] = -1; }
};

struct Migration { int32_t sp, src, slot, dst; };

// ----------------------------------------------------------------------------
// Simulation.
// ----------------------------------------------------------------------------
struct SimBase {
    orc_config cfg;
    int nsc[3], nscTot, T;
    double L[3], scInv[3], invh[3];
    std::vector<int8_t> dirOf;   // per particle of the current step (scratch)
    std::vector<Migration> migrations;
    int err = 0;
    void setup(const orc_config& c) {
        cfg = c;
        nscTot = 1;
        for (int d = 0; d < 3; d++) {
            nsc[d] = c.n[d] / c.sc[d];
            nscTot *= nsc[d];
            L[d] = (double)c.n[d] * c.h[d];
            // EnsembleSupercells.h:31-33: cellSize = (max-min)/numCells; invSize = 1/(S*cellSize)
            double cell = (L[d] - 0.0) / (double)c.n[d];
            scInv[d] = 1.0 / ((double)c.sc[d] * cell);
            invh[d] = 1.0 / c.h[d];
        }
        T = std::max(std::max(c.sc[0], c.sc[1]), c.sc[2]) + 2 * kG + 1;
#ifdef _OPENMP
        if (c.threads > 0) omp_set_num_threads(c.threads);
#endif
    }
    int steps = 0;
    int scLinear(int sx, int sy, int sz) const { return (sx * nsc[1] + sy) * nsc[2] + sz; }
    void scCoords(int s, int* sxyz) const {
        sxyz[2] = s % nsc[2]; sxyz[1] = (s / nsc[2]) % nsc[1]; sxyz[0] = s / (nsc[1] * nsc[2]);
    }
    static void dirDelta(int dir, int* ds) { ds[0] = dir / 9 - 1; ds[1] = (dir / 3) % 3 - 1; ds[2] = dir % 3 - 1; }
    // Direction code from old/new supercell coordinates (periodic, |delta| <= 1).
    int dirCode(const int* o, const int* nw) {
        int code = 0;
        for (int d = 0; d < 3; d++) {
            int ds = nw[d] - o[d];
            if (ds > 1) ds -= nsc[d];
            if (ds < -1) ds += nsc[d];
            if (ds < -1 || ds > 1) { err = -5; ds = 0; }
            code = code * 3 + (ds + 1);
        }
        return code;
    }
};

template <typename R, typename Store>
struct Sim : SimBase {
    Grid<R> grid;
    std::vector<std::vector<Store>> parts;  // [species][supercell]
    std::vector<R> jtiles;                  // per-supercell J tiles of the current step
    R eCoeff[4];                            // q dt / (2 m c) per species (BorisPusher.h:29)
    double qw_c[4];

    void init(const orc_config& c) {
        setup(c);
        grid.init(c.n);
        parts.assign(c.nspecies, std::vector<Store>(nscTot));
        for (int s = 0; s < c.nspecies; s++)
            eCoeff[s] = (R)(c.charge[s] * c.dt / (2.0 * c.mass[s] * kC));
    }

    // -------------------------------------------------------------- loading
    int load(int64_t n, const double* x, const double* y, const double* z, const double* ux,
             const double* uy, const double* uz, const double* w, const int32_t* sp);
    // ------------------------------------------------------------ stepping
    void step();
    void pushSupercell(int s, R* jt);
    void migrate();
    void resort();   // drop dead slots and sort every supercell by cell (stable)
};

// Local cell of particle i of supercell s: (lx*Sy + ly)*Sz + lz, the sort key.
inline int cellKey(const SimBase& S, const PlainStore& st, size_t i, const int* m) {
    const double p[3] = {st.x[i], st.y[i], st.z[i]};
    int l[3];
    for (int d = 0; d < 3; d++) {
        l[d] = (int)std::floor(p[d] * S.invh[d]) - m[d];
        l[d] = std::min(std::max(l[d], 0), S.cfg.sc[d] - 1);
    }
    return (l[0] * S.cfg.sc[1] + l[1]) * S.cfg.sc[2] + l[2];
}
inline int cellKey(const SimBase& S, const CellStore& st, size_t i, const int* m) {
    return ((st.cx[i] - m[0]) * S.cfg.sc[1] + (st.cy[i] - m[1])) * S.cfg.sc[2] + (st.cz[i] - m[2]);
}

// Live particles of st in (cell, slot) order.
template <typename Store>
Store sortedByCell(const SimBase& S, const Store& st, int s) {
    int sxyz[3]; S.scCoords(s, sxyz);
    const int m[3] = {sxyz[0] * S.cfg.sc[0], sxyz[1] * S.cfg.sc[1], sxyz[2] * S.cfg.sc[2]};
    std::vector<std::pair<int, size_t>> key;
    for (size_t i = 0; i < st.size(); i++)
        if (st.alive(i)) key.push_back({cellKey(S, st, i, m), i});
    std::stable_sort(key.begin(), key.end(), [](const std::pair<int, size_t>& a, const std::pair<int, size_t>& b) {
        return a.first < b.first;
    });
    Store out;
    for (auto& k : key) out.append(st, k.second);
    return out;
}

template <typename R, typename Store>
void Sim<R, Store>::resort() {
    for (auto& v : parts) {
#pragma omp parallel for schedule(dynamic, 8)
        for (int s = 0; s < nscTot; s++) v[s] = sortedByCell(*this, v[s], s);
    }
}

// ---- loading ---------------------------------------------------------------
// Routing of one input particle (EnsembleSupercells.h:56 for the supercell).
inline int routePlain(const SimBase& S, double x, double y, double z) {
    const double p[3] = {x, y, z};
    int c[3];
    for (int d = 0; d < 3; d++) {
        c[d] = (int)std::floor((p[d] - 0.0) * S.scInv[d]);  // EnsembleSupercells.h:56
        c[d] = std::min(std::max(c[d], 0), S.nsc[d] - 1);
    }
    return S.scLinear(c[0], c[1], c[2]);
}
// FP32 form: integer cell and FP32 offset of a position (FP64 arithmetic).
inline void toCell(const SimBase& S, double x, double y, double z, int* c, float* o) {
    const double p[3] = {x, y, z};
    for (int d = 0; d < 3; d++) {
        double xi = p[d] * S.invh[d];
        double fl = std::floor(xi);
        c[d] = (int)fl;
        o[d] = (float)(xi - fl);
        if (o[d] >= 1.0f) { o[d] = 0.0f; c[d] += 1; }
        c[d] = wrapi(c[d], S.cfg.n[d]);
    }
}
inline int routeCell(const SimBase& S, double x, double y, double z) {
    int c[3]; float o[3];
    toCell(S, x, y, z, c, o);
    return S.scLinear(c[0] / S.cfg.sc[0], c[1] / S.cfg.sc[1], c[2] / S.cfg.sc[2]);
}
inline int routeOf(const SimBase& S, const PlainStore*, double x, double y, double z) { return routePlain(S, x, y, z); }
inline int routeOf(const SimBase& S, const CellStore*, double x, double y, double z) { return routeCell(S, x, y, z); }
inline void putParticle(const SimBase&, PlainStore& st, size_t k, double x, double y, double z, double ux, double uy,
                        double uz, double w) {
    st.x[k] = x; st.y[k] = y; st.z[k] = z; st.ux[k] = ux; st.uy[k] = uy; st.uz[k] = uz; st.w[k] = w;
}
inline void putParticle(const SimBase& S, CellStore& st, size_t k, double x, double y, double z, double ux, double uy,
                        double uz, double w) {
    int c[3]; float o[3];
    toCell(S, x, y, z, c, o);
    st.cx[k] = c[0]; st.cy[k] = c[1]; st.cz[k] = c[2];
    st.ox[k] = o[0]; st.oy[k] = o[1]; st.oz[k] = o[2];
    st.ux[k] = (float)ux; st.uy[k] = (float)uy; st.uz[k] = (float)uz; st.w[k] = (float)w;
}
inline void resizeStore(PlainStore& st, size_t n) {
    st.x.resize(n); st.y.resize(n); st.z.resize(n); st.ux.resize(n); st.uy.resize(n); st.uz.resize(n); st.w.resize(n);
}
inline void resizeStore(CellStore& st, size_t n) {
    st.cx.resize(n); st.cy.resize(n); st.cz.resize(n); st.ox.resize(n); st.oy.resize(n); st.oz.resize(n);
    st.ux.resize(n); st.uy.resize(n); st.uz.resize(n); st.w.resize(n);
}

// Every particle goes to the supercell its position routes to, in input order
// (a stable counting sort over contiguous chunks of the input, one per thread),
// then each supercell is sorted by cell, stably (resort).
template <typename R, typename Store>
int Sim<R, Store>::load(int64_t n, const double* x, const double* y, const double* z, const double* ux,
                        const double* uy, const double* uz, const double* w, const int32_t* sp) {
    for (int64_t i = 0; i < n; i++)
        if (sp && (sp[i] < 0 || sp[i] >= cfg.nspecies)) return -2;
    const int ns = cfg.nspecies;
    const size_t bins = (size_t)ns * nscTot;
    std::vector<int32_t> route(n);
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    std::vector<std::vector<int64_t>> hist(nt, std::vector<int64_t>(bins, 0));
    auto chunkOf = [&](int t, int64_t& a, int64_t& b) { a = n * t / nt; b = n * (t + 1) / nt; };
    const Store* tag = nullptr;   // selects the form's routing
#pragma omp parallel for schedule(static, 1) num_threads(nt)
    for (int t = 0; t < nt; t++) {
        int64_t a, b;
        chunkOf(t, a, b);
        for (int64_t i = a; i < b; i++) {
            const int q = sp ? sp[i] : 0;
            route[i] = routeOf(*this, tag, x[i], y[i], z[i]);
            hist[t][(size_t)q * nscTot + route[i]]++;
        }
    }
    // Thread t writes bin k from offset sum over t' < t of hist[t'][k].
    for (size_t k = 0; k < bins; k++) {
        int64_t tot = 0;
        for (int t = 0; t < nt; t++) { const int64_t c = hist[t][k]; hist[t][k] = tot; tot += c; }
        Store& st = parts[k / nscTot][k % nscTot];
        st.clear();
        resizeStore(st, (size_t)tot);
    }
#pragma omp parallel for schedule(static, 1) num_threads(nt)
    for (int t = 0; t < nt; t++) {
        int64_t a, b;
        chunkOf(t, a, b);
        for (int64_t i = a; i < b; i++) {
            const int q = sp ? sp[i] : 0;
            const size_t k = (size_t)q * nscTot + route[i];
            putParticle(*this, parts[q][route[i]], (size_t)hist[t][k]++, x[i], y[i], z[i], ux[i], uy[i], uz[i], w[i]);
        }
    }
    resort();
    return 0;
}

// Boris rotation, BorisPusher.h:33-43, in precision R.  Returns the new u and 1/gamma.
template <typename R>
inline void boris(R ec, const R* e, const R* b, R* u, R& invGamma) {
    R em[3] = {e[0] * ec, e[1] * ec, e[2] * ec};
    R um[3] = {u[0] + em[0], u[1] + em[1], u[2] + em[2]};
    R tc = ec / std::sqrt(R(1) + (um[0] * um[0] + um[1] * um[1] + um[2] * um[2]));
    R t[3] = {b[0] * tc, b[1] * tc, b[2] * tc};
    R up[3] = {um[0] + (um[1] * t[2] - um[2] * t[1]), um[1] + (um[2] * t[0] - um[0] * t[2]),
               um[2] + (um[0] * t[1] - um[1] * t[0])};
    R sc = R(2) / (R(1) + (t[0] * t[0] + t[1] * t[1] + t[2] * t[2]));
    R s[3] = {t[0] * sc, t[1] * sc, t[2] * sc};
    u[0] = um[0] + (up[1] * s[2] - up[2] * s[1]) + em[0];
    u[1] = um[1] + (up[2] * s[0] - up[0] * s[2]) + em[1];
    u[2] = um[2] + (up[0] * s[1] - up[1] * s[0]) + em[2];
    invGamma = R(1) / std::sqrt(R(1) + (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
}

// CIC 8-point sum of FieldInterpolatorYeeGrid.h:272-280 on a T^3 tile.
inline double cicGatherRef(const double* t, int T, int bx, int by, int bz, double cx, double cy, double cz) {
    auto A = [&](int i, int j, int k) { return t[((size_t)(bx + i) * T + (by + j)) * T + (bz + k)]; };
    return A(0, 0, 0) * (1.0 - cx) * (1.0 - cy) * (1.0 - cz) + A(0, 0, 1) * (1.0 - cx) * (1.0 - cy) * cz +
           A(0, 1, 0) * (1.0 - cx) * cy * (1.0 - cz) + A(0, 1, 1) * (1.0 - cx) * cy * cz +
           A(1, 0, 0) * cx * (1.0 - cy) * (1.0 - cz) + A(1, 0, 1) * cx * (1.0 - cy) * cz +
           A(1, 1, 0) * cx * cy * (1.0 - cz) + A(1, 1, 1) * cx * cy * cz;
}
// CIC 8-point scatter of CurrentDepositorYeeGrid.h:254-261 on a T^3 tile.
inline void cicScatterRef(double* t, int T, int bx, int by, int bz, double cx, double cy, double cz, double v) {
    auto A = [&](int i, int j, int k) -> double& { return t[((size_t)(bx + i) * T + (by + j)) * T + (bz + k)]; };
    A(0, 0, 0) += (1.0 - cx) * (1.0 - cy) * (1.0 - cz) * v;
    A(0, 0, 1) += (1.0 - cx) * (1.0 - cy) * cz * v;
    A(0, 1, 0) += (1.0 - cx) * cy * (1.0 - cz) * v;
    A(0, 1, 1) += (1.0 - cx) * cy * cz * v;
    A(1, 0, 0) += cx * (1.0 - cy) * (1.0 - cz) * v;
    A(1, 0, 1) += cx * (1.0 - cy) * cz * v;
    A(1, 1, 0) += cx * cy * (1.0 - cz) * v;
    A(1, 1, 1) += cx * cy * cz * v;
}

// Component staggering: 1 = staggered (half-integer node) along that dimension.
// Ex(i, j+1/2, k+1/2) ... YeeGrid.h:11-14, 336-344.
const int kStag[6][3] = {{0, 1, 1}, {1, 0, 1}, {1, 1, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

template <typename R>
inline void stageTile(const Grid<R>& g, const int* m, int T, R* tile /* 6*T^3 */) {
    // tile node t <-> domain node m - kG + t <-> padded index m - kG + t + kLo
    for (int c = 0; c < 6; c++)
        for (int i = 0; i < T; i++)
            for (int j = 0; j < T; j++)
                for (int k = 0; k < T; k++) {
                    int gx = std::min(m[0] - kG + i + kLo, g.sz[0] - 1);
                    int gy = std::min(m[1] - kG + j + kLo, g.sz[1] - 1);
                    int gz = std::min(m[2] - kG + k + kLo, g.sz[2] - 1);
                    tile[(((size_t)c * T + i) * T + j) * T + k] = g.f[c][g.at(gx, gy, gz)];
                }
}

template <>
void Sim<double, PlainStore>::pushSupercell(int s, double* jt) {
    const orc_config& c = cfg;
    int sxyz[3]; scCoords(s, sxyz);
    int m[3] = {sxyz[0] * c.sc[0], sxyz[1] * c.sc[1], sxyz[2] * c.sc[2]};
    const int TT = T * T * T;
    std::vector<double> tile(6 * (size_t)TT);
    stageTile(grid, m, T, tile.data());
    double* jx = jt; double* jy = jt + TT; double* jz = jt + 2 * TT;
    // Reference supercell index math (FieldInterpolatorYeeGrid.h:197-205, 257-267):
    double minPos[3], no[3], nos[3]; int off[3];
    for (int d = 0; d < 3; d++) {
        minPos[d] = (double)m[d] * c.h[d];
        no[d] = (minPos[d] - c.h[d]) / c.h[d];
        nos[d] = no[d] + 0.5;
        // reference tile index t <-> domain node trunc(minPos/h) - 1 + t
        off[d] = ((int)(minPos[d] / c.h[d]) - 1) - (m[d] - kG);
    }
    const bool cic = c.shape == ORC_SHAPE_CIC;
    for (int sp = 0; sp < c.nspecies; sp++) {
        PlainStore& st = parts[sp][s];
        const double ec = eCoeff[sp];
        const double q = c.charge[sp];
        for (size_t p = 0; p < st.size(); p++) {
            if (!st.alive(p)) continue;
            double pos[3] = {st.x[p], st.y[p], st.z[p]};
            double eb[6];
            if (cic) {
                int ic[3], is[3]; double cc[3], cs[3];
                for (int d = 0; d < 3; d++) {
                    double np = pos[d] * invh[d];
                    double in = np - no[d];
                    ic[d] = (int)in; cc[d] = in - (double)ic[d];
                    in = np - nos[d];
                    is[d] = (int)in; cs[d] = in - (double)is[d];
                }
                for (int comp = 0; comp < 6; comp++) {
                    const int* sg = kStag[comp];
                    int b[3]; double w[3];
                    for (int d = 0; d < 3; d++) { b[d] = (sg[d] ? is[d] : ic[d]) + off[d]; w[d] = sg[d] ? cs[d] : cc[d]; }
                    eb[comp] = cicGatherRef(tile.data() + (size_t)comp * TT, T, b[0], b[1], b[2], w[0], w[1], w[2]);
                }
            } else {
                int nc[3], ns[3]; double wc[3][3], ws[3][3];
                for (int d = 0; d < 3; d++) {
                    double xi = pos[d] * invh[d];
                    nc[d] = (int)std::floor(xi + 0.5); tscWeights(xi - (double)nc[d], wc[d]);
                    double xs = xi - 0.5;
                    ns[d] = (int)std::floor(xs + 0.5); tscWeights(xs - (double)ns[d], ws[d]);
                }
                for (int comp = 0; comp < 6; comp++) {
                    const int* sg = kStag[comp];
                    int t0[3]; const double* w[3];
                    for (int d = 0; d < 3; d++) {
                        t0[d] = (sg[d] ? ns[d] : nc[d]) - 1 - (m[d] - kG);
                        w[d] = sg[d] ? ws[d] : wc[d];
                    }
                    eb[comp] = gatherSep<double, 3>(tile.data() + (size_t)comp * TT, T, t0, w[0], w[1], w[2]);
                }
            }
            double u[3] = {st.ux[p], st.uy[p], st.uz[p]}, ig;
            boris<double>(ec, eb, eb + 3, u, ig);
            double v[3], np[3];
            for (int d = 0; d < 3; d++) {
                v[d] = (u[d] * kC) * ig;             // ParticleArray.h:263
                np[d] = pos[d] + v[d] * c.dt;        // BorisPusher.h:44-46
            }
            const double wgt = st.w[p];
            if (c.deposit == ORC_DEPOSIT_DIRECT) {
                double cur[3] = {v[0] * (q * wgt), v[1] * (q * wgt), v[2] * (q * wgt)};
                if (cic) {
                    int ic[3], is[3]; double cc[3], cs[3];
                    for (int d = 0; d < 3; d++) {
                        double npn = np[d] * invh[d];
                        double in = npn - no[d];
                        ic[d] = (int)in; cc[d] = in - (double)ic[d];
                        in = npn - nos[d];
                        is[d] = (int)in; cs[d] = in - (double)is[d];
                    }
                    double* jc[3] = {jx, jy, jz};
                    for (int comp = 0; comp < 3; comp++) {
                        const int* sg = kStag[comp];
                        int b[3]; double w[3];
                        for (int d = 0; d < 3; d++) { b[d] = (sg[d] ? is[d] : ic[d]) + off[d]; w[d] = sg[d] ? cs[d] : cc[d]; }
                        cicScatterRef(jc[comp], T, b[0], b[1], b[2], w[0], w[1], w[2], cur[comp]);
                    }
                } else {
                    int nc[3], ns[3]; double wc[3][3], ws[3][3];
                    for (int d = 0; d < 3; d++) {
                        double xi = np[d] * invh[d];
                        nc[d] = (int)std::floor(xi + 0.5); tscWeights(xi - (double)nc[d], wc[d]);
                        double xs = xi - 0.5;
                        ns[d] = (int)std::floor(xs + 0.5); tscWeights(xs - (double)ns[d], ws[d]);
                    }
                    double* jc[3] = {jx, jy, jz};
                    for (int comp = 0; comp < 3; comp++) {
                        const int* sg = kStag[comp];
                        int t0[3]; const double* w[3];
                        for (int d = 0; d < 3; d++) {
                            t0[d] = (sg[d] ? ns[d] : nc[d]) - 1 - (m[d] - kG);
                            w[d] = sg[d] ? ws[d] : wc[d];
                        }
                        scatterSep<double, 3>(jc[comp], T, t0, w[0], w[1], w[2], cur[comp]);
                    }
                }
            } else {
                // Esirkepov on the rho lattice (xi = x/h - 1/2).
                double kq[3];
                for (int d = 0; d < 3; d++) kq[d] = -(q * wgt) * (c.h[d] / c.dt);
                int b[3];
                if (cic) {
                    double s0[3][3], s1[3][3];
                    for (int d = 0; d < 3; d++) {
                        double x0 = pos[d] * invh[d] - 0.5, x1 = np[d] * invh[d] - 0.5;
                        int n0 = (int)std::floor(x0), n1 = (int)std::floor(x1);
                        double w0[2] = {1.0 - (x0 - n0), x0 - n0}, w1[2] = {1.0 - (x1 - n1), x1 - n1};
                        int base = std::min(n0, n1);
                        placeShape<double, 3, 2>(s0[d], n0, base, w0);
                        placeShape<double, 3, 2>(s1[d], n1, base, w1);
                        b[d] = base - (m[d] - kG);
                    }
                    esirkepov<double, 3>(jx, jy, jz, T, b, s0, s1, kq);
                } else {
                    double s0[3][4], s1[3][4];
                    for (int d = 0; d < 3; d++) {
                        double x0 = pos[d] * invh[d] - 0.5, x1 = np[d] * invh[d] - 0.5;
                        int n0 = (int)std::floor(x0 + 0.5), n1 = (int)std::floor(x1 + 0.5);
                        double w0[3], w1[3];
                        tscWeights(x0 - (double)n0, w0); tscWeights(x1 - (double)n1, w1);
                        int base = std::min(n0, n1) - 1;
                        placeShape<double, 4, 3>(s0[d], n0 - 1, base, w0);
                        placeShape<double, 4, 3>(s1[d], n1 - 1, base, w1);
                        b[d] = base - (m[d] - kG);
                    }
                    esirkepov<double, 4>(jx, jy, jz, T, b, s0, s1, kq);
                }
            }
            st.x[p] = np[0]; st.y[p] = np[1]; st.z[p] = np[2];
            st.ux[p] = u[0]; st.uy[p] = u[1]; st.uz[p] = u[2];
        }
    }
}

template <>
void Sim<float, CellStore>::pushSupercell(int s, float* jt) {
    const orc_config& c = cfg;
    int sxyz[3]; scCoords(s, sxyz);
    int m[3] = {sxyz[0] * c.sc[0], sxyz[1] * c.sc[1], sxyz[2] * c.sc[2]};
    const int TT = T * T * T;
    std::vector<float> tile(6 * (size_t)TT);
    stageTile(grid, m, T, tile.data());
    float* jx = jt; float* jy = jt + TT; float* jz = jt + 2 * TT;
    float cdth[3];
    for (int d = 0; d < 3; d++) cdth[d] = (float)(kC * c.dt / c.h[d]);
    const bool cic = c.shape == ORC_SHAPE_CIC;
    for (int sp = 0; sp < c.nspecies; sp++) {
        CellStore& st = parts[sp][s];
        const float ec = eCoeff[sp];
        float kqs[3];
        for (int d = 0; d < 3; d++) kqs[d] = (float)(-c.charge[sp] * (c.h[d] / c.dt));
        const float qc = (float)(c.charge[sp] * kC);
        for (size_t p = 0; p < st.size(); p++) {
            if (!st.alive(p)) continue;
            int lc[3] = {st.cx[p] - m[0], st.cy[p] - m[1], st.cz[p] - m[2]};
            float o[3] = {st.ox[p], st.oy[p], st.oz[p]};
            float eb[6];
            if (cic) {
                int bc[3], bs[3]; float wc[3][2], ws[3][2];
                for (int d = 0; d < 3; d++) {
                    bc[d] = lc[d]; wc[d][0] = 1.0f - o[d]; wc[d][1] = o[d];
                    bool hi = o[d] >= 0.5f;
                    float dd = hi ? o[d] - 0.5f : o[d] + 0.5f;
                    bs[d] = hi ? lc[d] : lc[d] - 1; ws[d][0] = 1.0f - dd; ws[d][1] = dd;
                }
                for (int comp = 0; comp < 6; comp++) {
                    const int* sg = kStag[comp]; int t0[3]; const float* w[3];
                    for (int d = 0; d < 3; d++) { t0[d] = (sg[d] ? bs[d] : bc[d]) + kG; w[d] = sg[d] ? ws[d] : wc[d]; }
                    eb[comp] = gatherSep<float, 2>(tile.data() + (size_t)comp * TT, T, t0, w[0], w[1], w[2]);
                }
            } else {
                int bc[3], bs[3]; float wc[3][3], ws[3][3];
                for (int d = 0; d < 3; d++) {
                    bool hi = o[d] >= 0.5f;
                    bc[d] = lc[d] + (hi ? 1 : 0) - 1; tscWeights(hi ? o[d] - 1.0f : o[d], wc[d]);
                    bs[d] = lc[d] - 1; tscWeights(o[d] - 0.5f, ws[d]);
                }
                for (int comp = 0; comp < 6; comp++) {
                    const int* sg = kStag[comp]; int t0[3]; const float* w[3];
                    for (int d = 0; d < 3; d++) { t0[d] = (sg[d] ? bs[d] : bc[d]) + kG; w[d] = sg[d] ? ws[d] : wc[d]; }
                    eb[comp] = gatherSep<float, 3>(tile.data() + (size_t)comp * TT, T, t0, w[0], w[1], w[2]);
                }
            }
            float u[3] = {st.ux[p], st.uy[p], st.uz[p]}, ig;
            boris<float>(ec, eb, eb + 3, u, ig);
            int ln[3]; float on[3];
            for (int d = 0; d < 3; d++) {
                float onew = o[d] + (u[d] * ig) * cdth[d];
                float fl = std::floor(onew);
                ln[d] = lc[d] + (int)fl;
                onew = onew - fl;
                if (onew >= 1.0f) { onew -= 1.0f; ln[d] += 1; }
                on[d] = onew;
            }
            const float wgt = st.w[p];
            if (c.deposit == ORC_DEPOSIT_DIRECT) {
                float cur[3];
                for (int d = 0; d < 3; d++) cur[d] = (u[d] * ig) * (qc * wgt);
                float* jc[3] = {jx, jy, jz};
                if (cic) {
                    int bc[3], bs[3]; float wc[3][2], ws[3][2];
                    for (int d = 0; d < 3; d++) {
                        bc[d] = ln[d]; wc[d][0] = 1.0f - on[d]; wc[d][1] = on[d];
                        bool hi = on[d] >= 0.5f;
                        float dd = hi ? on[d] - 0.5f : on[d] + 0.5f;
                        bs[d] = hi ? ln[d] : ln[d] - 1; ws[d][0] = 1.0f - dd; ws[d][1] = dd;
                    }
                    for (int comp = 0; comp < 3; comp++) {
                        const int* sg = kStag[comp]; int t0[3]; const float* w[3];
                        for (int d = 0; d < 3; d++) { t0[d] = (sg[d] ? bs[d] : bc[d]) + kG; w[d] = sg[d] ? ws[d] : wc[d]; }
                        scatterSep<float, 2>(jc[comp], T, t0, w[0], w[1], w[2], cur[comp]);
                    }
                } else {
                    int bc[3], bs[3]; float wc[3][3], ws[3][3];
                    for (int d = 0; d < 3; d++) {
                        bool hi = on[d] >= 0.5f;
                        bc[d] = ln[d] + (hi ? 1 : 0) - 1; tscWeights(hi ? on[d] - 1.0f : on[d], wc[d]);
                        bs[d] = ln[d] - 1; tscWeights(on[d] - 0.5f, ws[d]);
                    }
                    for (int comp = 0; comp < 3; comp++) {
                        const int* sg = kStag[comp]; int t0[3]; const float* w[3];
                        for (int d = 0; d < 3; d++) { t0[d] = (sg[d] ? bs[d] : bc[d]) + kG; w[d] = sg[d] ? ws[d] : wc[d]; }
                        scatterSep<float, 3>(jc[comp], T, t0, w[0], w[1], w[2], cur[comp]);
                    }
                }
            } else {
                float kq[3] = {kqs[0] * wgt, kqs[1] * wgt, kqs[2] * wgt};
                int b[3];
                if (cic) {
                    float s0[3][3], s1[3][3];
                    for (int d = 0; d < 3; d++) {
                        bool h0 = o[d] >= 0.5f, h1 = on[d] >= 0.5f;
                        int n0 = h0 ? lc[d] : lc[d] - 1, n1 = h1 ? ln[d] : ln[d] - 1;
                        float d0 = h0 ? o[d] - 0.5f : o[d] + 0.5f, d1 = h1 ? on[d] - 0.5f : on[d] + 0.5f;
                        float w0[2] = {1.0f - d0, d0}, w1[2] = {1.0f - d1, d1};
                        int base = std::min(n0, n1);
                        placeShape<float, 3, 2>(s0[d], n0, base, w0);
                        placeShape<float, 3, 2>(s1[d], n1, base, w1);
                        b[d] = base + kG;
                    }
                    esirkepov<float, 3>(jx, jy, jz, T, b, s0, s1, kq);
                } else {
                    float s0[3][4], s1[3][4];
                    for (int d = 0; d < 3; d++) {
                        float w0[3], w1[3];
                        tscWeights(o[d] - 0.5f, w0); tscWeights(on[d] - 0.5f, w1);
                        int base = std::min(lc[d], ln[d]) - 1;
                        placeShape<float, 4, 3>(s0[d], lc[d] - 1, base, w0);
                        placeShape<float, 4, 3>(s1[d], ln[d] - 1, base, w1);
                        b[d] = base + kG;
                    }
                    esirkepov<float, 4>(jx, jy, jz, T, b, s0, s1, kq);
                }
            }
            st.cx[p] = wrapi(m[0] + ln[0], c.n[0]); st.cy[p] = wrapi(m[1] + ln[1], c.n[1]); st.cz[p] = wrapi(m[2] + ln[2], c.n[2]);
            st.ox[p] = on[0]; st.oy[p] = on[1]; st.oz[p] = on[2];
            st.ux[p] = u[0]; st.uy[p] = u[1]; st.uz[p] = u[2];
        }
    }
}

// New supercell coordinates of particle p of supercell store st (after the push).
inline void newSupercell(const SimBase& S, const PlainStore& st, size_t p, int* out) {
    double pos[3] = {st.x[p], st.y[p], st.z[p]};
    for (int d = 0; d < 3; d++) {
        out[d] = (int)std::floor((pos[d] - 0.0) * S.scInv[d]);
        out[d] = std::min(std::max(out[d], 0), S.nsc[d] - 1);
    }
}
inline void newSupercell(const SimBase& S, const CellStore& st, size_t p, int* out) {
    out[0] = st.cx[p] / S.cfg.sc[0]; out[1] = st.cy[p] / S.cfg.sc[1]; out[2] = st.cz[p] / S.cfg.sc[2];
}
inline void wrapPositions(const SimBase& S, PlainStore& st) {
    for (size_t p = 0; p < st.size(); p++) {
        if (!st.alive(p)) continue;
        double* v[3] = {&st.x[p], &st.y[p], &st.z[p]};
        for (int d = 0; d < 3; d++) {
            if (*v[d] < 0.0) *v[d] += S.L[d];
            if (*v[d] >= S.L[d]) *v[d] -= S.L[d];
        }
    }
}
inline void wrapPositions(const SimBase&, CellStore&) {}

template <typename R, typename Store>
void Sim<R, Store>::migrate() {
    migrations.clear();
    for (int sp = 0; sp < cfg.nspecies; sp++) {
        std::vector<Store>& sc = parts[sp];
        std::vector<std::vector<int8_t>> dirs(nscTot);   // -1: dead slot
#pragma omp parallel for schedule(dynamic, 8)
        for (int s = 0; s < nscTot; s++) {
            wrapPositions(*this, sc[s]);
            int o[3]; scCoords(s, o);
            dirs[s].assign(sc[s].size(), -1);
            for (size_t p = 0; p < sc[s].size(); p++) {
                if (!sc[s].alive(p)) continue;
                int nw[3]; newSupercell(*this, sc[s], p, nw);
                dirs[s][p] = (int8_t)dirCode(o, nw);
            }
        }
        for (int s = 0; s < nscTot; s++)
            for (size_t p = 0; p < sc[s].size(); p++)
                if (dirs[s][p] >= 0 && dirs[s][p] != 13) {
                    int ds[3], o[3]; dirDelta(dirs[s][p], ds); scCoords(s, o);
                    int dst = scLinear(wrapi(o[0] + ds[0], nsc[0]), wrapi(o[1] + ds[1], nsc[1]), wrapi(o[2] + ds[2], nsc[2]));
                    migrations.push_back({sp, s, (int32_t)p, dst});
                }
        // Each destination: this step's own leavers leave holes (ascending slots); arrivals
        // in canonical order (direction code, then source slot) fill the holes, then append.
        std::vector<Store> next(nscTot);
#pragma omp parallel for schedule(dynamic, 8)
        for (int d = 0; d < nscTot; d++) {
            next[d] = sc[d];
            std::vector<size_t> holes;
            for (size_t p = 0; p < sc[d].size(); p++)
                if (dirs[d][p] >= 0 && dirs[d][p] != 13) { holes.push_back(p); next[d].kill(p); }
            int dc[3]; scCoords(d, dc);
            size_t k = 0;
            for (int dir = 0; dir < 27; dir++) {
                if (dir == 13) continue;
                int ds[3]; dirDelta(dir, ds);
                int src = scLinear(wrapi(dc[0] - ds[0], nsc[0]), wrapi(dc[1] - ds[1], nsc[1]), wrapi(dc[2] - ds[2], nsc[2]));
                for (size_t p = 0; p < sc[src].size(); p++)
                    if (dirs[src][p] == dir) {
                        if (k < holes.size()) next[d].set(holes[k], sc[src], p);
                        else next[d].append(sc[src], p);
                        k++;
                    }
            }
        }
        sc.swap(next);
    }
    steps++;
    if (cfg.resort_every > 0 && steps % cfg.resort_every == 0) resort();
}

template <typename R, typename Store>
void Sim<R, Store>::step() {
    const orc_config& c = cfg;
    const int TT = T * T * T;
    jtiles.assign((size_t)nscTot * 3 * TT, R(0));
#pragma omp parallel for schedule(dynamic, 4)
    for (int s = 0; s < nscTot; s++) pushSupercell(s, jtiles.data() + (size_t)s * 3 * TT);
    // Serial flush in supercell order: J(node) += tile * 1/h^3 (CurrentDepositorYeeGrid.h:201-213).
    for (int c3 = 6; c3 < 9; c3++) std::fill(grid.f[c3].begin(), grid.f[c3].end(), R(0));
    const double normd = 1.0 / (c.h[0] * c.h[1] * c.h[2]);
    const R norm = (R)normd;
    for (int s = 0; s < nscTot; s++) {
        int sxyz[3]; scCoords(s, sxyz);
        int base[3] = {sxyz[0] * c.sc[0] - kG + kLo, sxyz[1] * c.sc[1] - kG + kLo, sxyz[2] * c.sc[2] - kG + kLo};
        const R* jt = jtiles.data() + (size_t)s * 3 * TT;
        for (int i = 0; i < T; i++)
            for (int j = 0; j < T; j++)
                for (int k = 0; k < T; k++) {
                    int gx = base[0] + i, gy = base[1] + j, gz = base[2] + k;
                    size_t t = ((size_t)i * T + j) * T + k;
                    if (gx >= grid.sz[0] || gy >= grid.sz[1] || gz >= grid.sz[2]) {
                        if (jt[t] != R(0) || jt[TT + t] != R(0) || jt[2 * TT + t] != R(0)) err = -6;
                        continue;
                    }
                    size_t g = grid.at(gx, gy, gz);
                    grid.f[6][g] += jt[t] * norm;
                    grid.f[7][g] += jt[TT + t] * norm;
                    grid.f[8][g] += jt[2 * TT + t] * norm;
                }
    }
    grid.fold();
    // updateB(dt/2); updateE(dt); updateB(dt/2) with periodic guard fills.
    const double dth = 0.5 * c.dt;
    R bx = (R)((kC * dth) / c.h[0]), by = (R)((kC * dth) / c.h[1]), bz = (R)((kC * dth) / c.h[2]);
    R ex = (R)((kC * c.dt) / c.h[0]), ey = (R)((kC * c.dt) / c.h[1]), ez = (R)((kC * c.dt) / c.h[2]);
    R cc = (R)(-4.0 * kPi * c.dt);
    grid.updateB(bx, by, bz); grid.fill(3, 6);
    grid.updateE(cc, ex, ey, ez); grid.fill(0, 3);
    grid.updateB(bx, by, bz); grid.fill(3, 6);
    migrate();
}

// ----------------------------------------------------------------------------
// Diagnostics.
// ----------------------------------------------------------------------------
template <typename R>
void depositRho(const SimBase& S, const std::vector<std::vector<PlainStore>>& parts, std::vector<double>& rho) {
    const orc_config& c = S.cfg;
    const double norm = 1.0 / (c.h[0] * c.h[1] * c.h[2]);
    for (int sp = 0; sp < c.nspecies; sp++)
        for (auto& st : parts[sp])
            for (size_t p = 0; p < st.size(); p++) {
                if (!st.alive(p)) continue;
                double pos[3] = {st.x[p], st.y[p], st.z[p]};
                int lo[3]; double w[3][3]; int np = c.shape == ORC_SHAPE_CIC ? 2 : 3;
                for (int d = 0; d < 3; d++) {
                    double xi = pos[d] * S.invh[d] - 0.5;
                    if (np == 2) { int n = (int)std::floor(xi); w[d][0] = 1.0 - (xi - n); w[d][1] = xi - n; lo[d] = n; }
                    else { int n = (int)std::floor(xi + 0.5); tscWeights(xi - n, w[d]); lo[d] = n - 1; }
                }
                double v = c.charge[sp] * st.w[p] * norm;
                for (int i = 0; i < np; i++)
                    for (int j = 0; j < np; j++)
                        for (int k = 0; k < np; k++)
                            rho[((size_t)wrapi(lo[0] + i, c.n[0]) * c.n[1] + wrapi(lo[1] + j, c.n[1])) * c.n[2] + wrapi(lo[2] + k, c.n[2])] +=
                                v * w[0][i] * w[1][j] * w[2][k];
            }
}
template <typename R>
void depositRho(const SimBase& S, const std::vector<std::vector<CellStore>>& parts, std::vector<double>& rho) {
    const orc_config& c = S.cfg;
    const double norm = 1.0 / (c.h[0] * c.h[1] * c.h[2]);
    for (int sp = 0; sp < c.nspecies; sp++)
        for (auto& st : parts[sp])
            for (size_t p = 0; p < st.size(); p++) {
                if (!st.alive(p)) continue;
                int cc[3] = {st.cx[p], st.cy[p], st.cz[p]};
                double o[3] = {st.ox[p], st.oy[p], st.oz[p]};
                int lo[3]; double w[3][3]; int np = c.shape == ORC_SHAPE_CIC ? 2 : 3;
                for (int d = 0; d < 3; d++) {
                    if (np == 2) {
                        bool hi = o[d] >= 0.5; double dd = hi ? o[d] - 0.5 : o[d] + 0.5;
                        lo[d] = hi ? cc[d] : cc[d] - 1; w[d][0] = 1.0 - dd; w[d][1] = dd;
                    } else { tscWeights(o[d] - 0.5, w[d]); lo[d] = cc[d] - 1; }
                }
                double v = c.charge[sp] * (double)st.w[p] * norm;
                for (int i = 0; i < np; i++)
                    for (int j = 0; j < np; j++)
                        for (int k = 0; k < np; k++)
                            rho[((size_t)wrapi(lo[0] + i, c.n[0]) * c.n[1] + wrapi(lo[1] + j, c.n[1])) * c.n[2] + wrapi(lo[2] + k, c.n[2])] +=
                                v * w[0][i] * w[1][j] * w[2][k];
            }
}

inline double kinetic(const SimBase& S, const std::vector<std::vector<PlainStore>>& parts) {
    double e = 0;
    for (int sp = 0; sp < S.cfg.nspecies; sp++)
        for (auto& st : parts[sp])
            for (size_t p = 0; p < st.size(); p++) {
                if (!st.alive(p)) continue;
                double u2 = st.ux[p] * st.ux[p] + st.uy[p] * st.uy[p] + st.uz[p] * st.uz[p];
                e += st.w[p] * S.cfg.mass[sp] * kC * kC * (u2 / (1.0 + std::sqrt(1.0 + u2)));
            }
    return e;
}
inline double kinetic(const SimBase& S, const std::vector<std::vector<CellStore>>& parts) {
    double e = 0;
    for (int sp = 0; sp < S.cfg.nspecies; sp++)
        for (auto& st : parts[sp])
            for (size_t p = 0; p < st.size(); p++) {
                if (!st.alive(p)) continue;
                double ux = st.ux[p], uy = st.uy[p], uz = st.uz[p];
                double u2 = ux * ux + uy * uy + uz * uz;
                e += (double)st.w[p] * S.cfg.mass[sp] * kC * kC * (u2 / (1.0 + std::sqrt(1.0 + u2)));
            }
    return e;
}

struct Handle {
    int form;
    Sim<double, PlainStore>* plain = nullptr;
    Sim<float, CellStore>* cell = nullptr;
    SimBase* base() { return plain ? (SimBase*)plain : (SimBase*)cell; }
};

template <typename S>
int getFields(S* s, double* const* f9) {
    const orc_config& c = s->cfg;
    for (int comp = 0; comp < 9; comp++)
        for (int i = 0; i < c.n[0]; i++)
            for (int j = 0; j < c.n[1]; j++)
                for (int k = 0; k < c.n[2]; k++)
                    f9[comp][((size_t)i * c.n[1] + j) * c.n[2] + k] = (double)s->grid.f[comp][s->grid.at(i + kLo, j + kLo, k + kLo)];
    return 0;
}
template <typename S>
int setFields(S* s, const double* const* f9) {
    const orc_config& c = s->cfg;
    typedef typename std::remove_reference<decltype(s->grid.f[0][0])>::type R;
    for (int comp = 0; comp < 9; comp++)
        for (int i = 0; i < c.n[0]; i++)
            for (int j = 0; j < c.n[1]; j++)
                for (int k = 0; k < c.n[2]; k++)
                    s->grid.f[comp][s->grid.at(i + kLo, j + kLo, k + kLo)] = (R)f9[comp][((size_t)i * c.n[1] + j) * c.n[2] + k];
    s->grid.fill(0, 6);
    return 0;
}
template <typename Store>
int64_t aliveCount(const Store& st) {
    int64_t n = 0;
    for (size_t p = 0; p < st.size(); p++) n += st.alive(p) ? 1 : 0;
    return n;
}
template <typename S>
int getCounts(S* s, int32_t* counts) {
    for (int sp = 0; sp < s->cfg.nspecies; sp++)
        for (int k = 0; k < s->nscTot; k++) counts[(size_t)sp * s->nscTot + k] = (int32_t)aliveCount(s->parts[sp][k]);
    return 0;
}
template <typename S>
double gaussResidual(S* s, const std::vector<double>& rho, double bg, double* rhoMax) {
    const orc_config& c = s->cfg;
    double gmax = 0, rmax = 0;
    auto F = [&](int comp, int i, int j, int k) {
        return (double)s->grid.f[comp][s->grid.at(wrapi(i, c.n[0]) + kLo, wrapi(j, c.n[1]) + kLo, wrapi(k, c.n[2]) + kLo)];
    };
    for (int i = 0; i < c.n[0]; i++)
        for (int j = 0; j < c.n[1]; j++)
            for (int k = 0; k < c.n[2]; k++) {
                double div = (F(0, i + 1, j, k) - F(0, i, j, k)) / c.h[0] + (F(1, i, j + 1, k) - F(1, i, j, k)) / c.h[1] +
                             (F(2, i, j, k + 1) - F(2, i, j, k)) / c.h[2];
                double r = rho[((size_t)i * c.n[1] + j) * c.n[2] + k];
                gmax = std::max(gmax, std::fabs(div - 4.0 * kPi * (r + bg)));
                rmax = std::max(rmax, std::fabs(r));
            }
    *rhoMax = rmax;
    return gmax;
}

// ----------------------------------------------------------------------------
// Synthetic plasma (the draws of the product's host generator, restated so that
// the CPU baseline needs nothing but this file).  Draw d of particle p of cell c
// is the SplitMix64 output function (S. Vigna, "Further scramblings of
// Marsaglia's xorshift generators", 2014) applied to the mixed seed xor a key of
// (c, p, d); normals by Box-Muller (1958) from draws d and d + 1.
// ----------------------------------------------------------------------------
inline uint64_t splitmixOut(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline double uniformDraw(uint64_t seed, int64_t cell, int64_t p, int d) {
    const uint64_t key = ((uint64_t)cell << 24) ^ ((uint64_t)p << 4) ^ (uint64_t)d;
    return (double)(splitmixOut(splitmixOut(seed) ^ key) >> 11) * 0x1.0p-53;   // 53 bits in [0, 1)
}
inline double gaussianDraw(uint64_t seed, int64_t cell, int64_t p, int d) {
    const double u1 = 1.0 - uniformDraw(seed, cell, p, d), u2 = uniformDraw(seed, cell, p, d + 1);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
}
// Particles per cell of x-plane i: round(ppc (1 + a cos(2 pi (i + 1/2) / nx))).
inline int planeCount(const orc_plasma* s, int i) {
    const double f = 1.0 + s->density_mod * std::cos(2.0 * 3.14159265358979323846 * (i + 0.5) / s->n[0]);
    return (int)std::lround(s->ppc * f);
}

}  // namespace

// ============================================================================
// C API
// ============================================================================
extern "C" {

void* orc_create(const orc_config* cfg) {
    if (!cfg || cfg->nspecies < 1 || cfg->nspecies > 4) return nullptr;
    for (int d = 0; d < 3; d++)
        if (cfg->n[d] <= 0 || cfg->sc[d] <= 0 || cfg->n[d] % cfg->sc[d] != 0) return nullptr;
    Handle* h = new Handle();
    h->form = cfg->form;
    if (cfg->form == ORC_FORM_FP64_PLAIN) { h->plain = new Sim<double, PlainStore>(); h->plain->init(*cfg); }
    else if (cfg->form == ORC_FORM_FP32_CELL) { h->cell = new Sim<float, CellStore>(); h->cell->init(*cfg); }
    else { delete h; return nullptr; }
    return h;
}

void orc_destroy(void* sim) {
    Handle* h = (Handle*)sim;
    if (!h) return;
    delete h->plain; delete h->cell; delete h;
}

int orc_load(void* sim, int64_t n, const double* x, const double* y, const double* z, const double* ux,
             const double* uy, const double* uz, const double* w, const int32_t* species) {
    Handle* h = (Handle*)sim;
    if (!h) return -1;
    return h->plain ? h->plain->load(n, x, y, z, ux, uy, uz, w, species) : h->cell->load(n, x, y, z, ux, uy, uz, w, species);
}

int orc_set_fields(void* sim, const double* const* f9) {
    Handle* h = (Handle*)sim;
    if (!h) return -1;
    return h->plain ? setFields(h->plain, f9) : setFields(h->cell, f9);
}

int orc_get_fields(void* sim, double* const* f9) {
    Handle* h = (Handle*)sim;
    if (!h) return -1;
    return h->plain ? getFields(h->plain, f9) : getFields(h->cell, f9);
}

int orc_step(void* sim, int32_t nsteps) {
    Handle* h = (Handle*)sim;
    if (!h) return -1;
    for (int i = 0; i < nsteps; i++) {
        if (h->plain) h->plain->step(); else h->cell->step();
        if (h->base()->err) return h->base()->err;
    }
    return 0;
}

int64_t orc_num_particles(void* sim) {
    Handle* h = (Handle*)sim;
    if (!h) return -1;
    int64_t n = 0;
    if (h->plain) { for (auto& v : h->plain->parts) for (auto& s : v) n += aliveCount(s); }
    else { for (auto& v : h->cell->parts) for (auto& s : v) n += aliveCount(s); }
    return n;
}

int orc_get_particles(void* sim, double* x, double* y, double* z, double* ux, double* uy, double* uz, double* w,
                      int32_t* species, int32_t* supercell) {
    Handle* h = (Handle*)sim;
    if (!h) return -1;
    int64_t o = 0;
    if (h->plain) {
        auto* s = h->plain;
        for (int sp = 0; sp < s->cfg.nspecies; sp++)
            for (int k = 0; k < s->nscTot; k++) {
                const PlainStore& st = s->parts[sp][k];
                for (size_t p = 0; p < st.size(); p++) {
                    if (!st.alive(p)) continue;
                    x[o] = st.x[p]; y[o] = st.y[p]; z[o] = st.z[p];
                    ux[o] = st.ux[p]; uy[o] = st.uy[p]; uz[o] = st.uz[p]; w[o] = st.w[p];
                    if (species) species[o] = sp;
                    if (supercell) supercell[o] = k;
                    o++;
                }
            }
    } else {
        auto* s = h->cell;
        for (int sp = 0; sp < s->cfg.nspecies; sp++)
            for (int k = 0; k < s->nscTot; k++) {
                const CellStore& st = s->parts[sp][k];
                for (size_t p = 0; p < st.size(); p++) {
                    if (!st.alive(p)) continue;
                    x[o] = ((double)st.cx[p] + (double)st.ox[p]) * s->cfg.h[0];
                    y[o] = ((double)st.cy[p] + (double)st.oy[p]) * s->cfg.h[1];
                    z[o] = ((double)st.cz[p] + (double)st.oz[p]) * s->cfg.h[2];
                    ux[o] = st.ux[p]; uy[o] = st.uy[p]; uz[o] = st.uz[p]; w[o] = st.w[p];
                    if (species) species[o] = sp;
                    if (supercell) supercell[o] = k;
                    o++;
                }
            }
    }
    return 0;
}

int orc_get_particles_cell(void* sim, int32_t* cell, float* ox, float* oy, float* oz, float* ux, float* uy,
                           float* uz, float* w) {
    Handle* h = (Handle*)sim;
    if (!h || !h->cell) return -1;
    auto* s = h->cell;
    int64_t o = 0;
    for (int sp = 0; sp < s->cfg.nspecies; sp++)
        for (int k = 0; k < s->nscTot; k++) {
            const CellStore& st = s->parts[sp][k];
            for (size_t p = 0; p < st.size(); p++) {
                if (!st.alive(p)) continue;
                cell[o] = (st.cx[p] * s->cfg.n[1] + st.cy[p]) * s->cfg.n[2] + st.cz[p];
                ox[o] = st.ox[p]; oy[o] = st.oy[p]; oz[o] = st.oz[p];
                ux[o] = st.ux[p]; uy[o] = st.uy[p]; uz[o] = st.uz[p]; w[o] = st.w[p];
                o++;
            }
        }
    return 0;
}

int orc_get_counts(void* sim, int32_t* counts) {
    Handle* h = (Handle*)sim;
    if (!h) return -1;
    return h->plain ? getCounts(h->plain, counts) : getCounts(h->cell, counts);
}

int64_t orc_num_migrations(void* sim) {
    Handle* h = (Handle*)sim;
    return h ? (int64_t)h->base()->migrations.size() : -1;
}

int orc_get_migrations(void* sim, int32_t* species, int32_t* src, int32_t* slot, int32_t* dst) {
    Handle* h = (Handle*)sim;
    if (!h) return -1;
    const auto& m = h->base()->migrations;
    for (size_t i = 0; i < m.size(); i++) { species[i] = m[i].sp; src[i] = m[i].src; slot[i] = m[i].slot; dst[i] = m[i].dst; }
    return 0;
}

int orc_charge_density(void* sim, double* rho) {
    Handle* h = (Handle*)sim;
    if (!h) return -1;
    SimBase* b = h->base();
    std::vector<double> r((size_t)b->cfg.n[0] * b->cfg.n[1] * b->cfg.n[2], 0.0);
    if (h->plain) depositRho<double>(*b, h->plain->parts, r); else depositRho<float>(*b, h->cell->parts, r);
    std::memcpy(rho, r.data(), r.size() * sizeof(double));
    return 0;
}

int orc_diagnostics(void* sim, double bg, orc_diag* out) {
    Handle* h = (Handle*)sim;
    if (!h || !out) return -1;
    SimBase* b = h->base();
    const orc_config& c = b->cfg;
    std::memset(out, 0, sizeof(*out));
    double vol = c.h[0] * c.h[1] * c.h[2];
    double fe = 0;
    std::vector<double> r((size_t)c.n[0] * c.n[1] * c.n[2], 0.0);
    if (h->plain) {
        auto* s = h->plain;
        for (int comp = 0; comp < 6; comp++)
            for (int i = 0; i < c.n[0]; i++) for (int j = 0; j < c.n[1]; j++) for (int k = 0; k < c.n[2]; k++) {
                double v = s->grid.f[comp][s->grid.at(i + kLo, j + kLo, k + kLo)]; fe += v * v; }
        out->kinetic_energy = kinetic(*b, s->parts);
        depositRho<double>(*b, s->parts, r);
        out->gauss_max = gaussResidual(s, r, bg, &out->rho_max);
        for (int sp = 0; sp < c.nspecies; sp++) for (auto& st : s->parts[sp]) for (size_t p = 0; p < st.size(); p++) if (st.alive(p)) out->total_charge += c.charge[sp] * st.w[p];
    } else {
        auto* s = h->cell;
        for (int comp = 0; comp < 6; comp++)
            for (int i = 0; i < c.n[0]; i++) for (int j = 0; j < c.n[1]; j++) for (int k = 0; k < c.n[2]; k++) {
                double v = s->grid.f[comp][s->grid.at(i + kLo, j + kLo, k + kLo)]; fe += v * v; }
        out->kinetic_energy = kinetic(*b, s->parts);
        depositRho<float>(*b, s->parts, r);
        out->gauss_max = gaussResidual(s, r, bg, &out->rho_max);
        for (int sp = 0; sp < c.nspecies; sp++) for (auto& st : s->parts[sp]) for (size_t p = 0; p < st.size(); p++) if (st.alive(p)) out->total_charge += c.charge[sp] * (double)st.w[p];
    }
    out->field_energy = fe * vol / (8.0 * kPi);
    return 0;
}


int64_t orc_plasma_count(const orc_plasma* s) {
    if (!s || s->n[0] <= 0 || s->n[1] <= 0 || s->n[2] <= 0 || !(s->ppc >= 0)) return -1;
    int64_t tot = 0;
    for (int i = 0; i < s->n[0]; i++) {
        const int c = planeCount(s, i);
        if (c < 0) return -1;
        tot += (int64_t)c * s->n[1] * s->n[2];
    }
    return tot;
}

int orc_plasma_generate(const orc_plasma* s, int32_t threads, double* x, double* y, double* z, double* ux,
                        double* uy, double* uz, double* w, int32_t* species) {
    if (orc_plasma_count(s) < 0 || !x || !y || !z || !ux || !uy || !uz || !w) return -1;
    const int nx = s->n[0], ny = s->n[1], nz = s->n[2];
    std::vector<int64_t> first(nx + 1, 0);
    for (int i = 0; i < nx; i++) first[i + 1] = first[i] + (int64_t)planeCount(s, i) * ny * nz;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    // Order: x-plane, then y, z, then particle index within the cell.
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < nx; i++) {
        const int per = planeCount(s, i);
        int64_t o = first[i];
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int64_t cell = ((int64_t)i * ny + j) * nz + k;
                for (int p = 0; p < per; p++, o++) {
                    x[o] = ((double)i + uniformDraw(s->seed, cell, p, 0)) * s->h[0];
                    y[o] = ((double)j + uniformDraw(s->seed, cell, p, 1)) * s->h[1];
                    z[o] = ((double)k + uniformDraw(s->seed, cell, p, 2)) * s->h[2];
                    double u[3] = {s->sigma_u * gaussianDraw(s->seed, cell, p, 3),
                                   s->sigma_u * gaussianDraw(s->seed, cell, p, 5),
                                   s->sigma_u * gaussianDraw(s->seed, cell, p, 7)};
                    // two beams: even particles drift at +drift_u, odd ones at -drift_u
                    const double drift = s->nbeams == 2 ? (p % 2 == 0 ? s->drift_u : -s->drift_u) : s->drift_u;
                    u[s->drift_axis] = u[s->drift_axis] + drift;
                    ux[o] = u[0]; uy[o] = u[1]; uz[o] = u[2];
                    w[o] = s->weight;
                    if (species) species[o] = s->species;
                }
            }
    }
    return 0;
}

/* EnsembleOrdered::reorder (particles/EnsembleOrdered.h:61-71): indexes sorted by
 * pica's comparator (lexicographic position order over `dims` coordinates,
 * EnsembleOrdered.h:31-41), stably, so that ties keep input order. */
int orc_order_by_position(int64_t n, int32_t dims, const double* x, const double* y, const double* z, int64_t* order) {
    if (n < 0 || dims < 1 || dims > 3) return -1;
    const double* key[3] = {x, y, z};
    for (int64_t i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order, order + n, [&](int64_t a, int64_t b) {
        for (int d = 0; d < dims; d++) {
            if (key[d][a] < key[d][b]) return true;
            if (key[d][a] > key[d][b]) return false;
        }
        return false;
    });
    return 0;
}

/* One push of a flat particle array in array order (the unordered layout): pica's
 * grid-level CIC interpolator and depositor (FieldInterpolatorYeeGrid.h:23-38,
 * 137-183; CurrentDepositorYeeGrid.h:23-38, 126-163) on a grid with `guard`
 * layers below the domain (origin -guard h; pica grid node g is domain node
 * g - guard, periodic), the Boris pusher (BorisPusher.h:33-47) and, for TSC, the
 * quadratic B-spline on the nodes nearest to the position.  The current added
 * at the new position is v (q w) / (hx hy hz).  f6: ex ey ez bx by bz, j3: jx jy
 * jz (added to), N^3 arrays, z fastest.  Positions wrap periodically after the
 * deposit. */
int orc_push_flat(const orc_config* c, int32_t guard, int64_t n, double* x, double* y, double* z, double* ux,
                  double* uy, double* uz, const double* w, const int32_t* species, const double* const* f6,
                  double* const* j3) {
    if (!c || c->form != ORC_FORM_FP64_PLAIN || c->deposit != ORC_DEPOSIT_DIRECT || guard < 0) return -1;
    const int N[3] = {c->n[0], c->n[1], c->n[2]};
    double invh[3], no[3], nos[3], L[3];
    for (int d = 0; d < 3; d++) {
        invh[d] = 1.0 / c->h[d];
        no[d] = (-(double)guard * c->h[d]) / c->h[d];
        nos[d] = no[d] + 0.5;
        L[d] = (double)N[d] * c->h[d];
    }
    const double norm = 1.0 / (c->h[0] * c->h[1] * c->h[2]);
    auto at = [&](int i, int j, int k) {
        return ((size_t)wrapi(i, N[0]) * N[1] + wrapi(j, N[1])) * N[2] + wrapi(k, N[2]);
    };
    const bool cic = c->shape == ORC_SHAPE_CIC;
    for (int64_t p = 0; p < n; p++) {
        const int sp = species ? species[p] : 0;
        if (sp < 0 || sp >= c->nspecies) return -2;
        const double pos[3] = {x[p], y[p], z[p]};
        double eb[6];
        auto indexCoeff = [&](const double* q, int* ic, double* cc, int* is, double* cs) {
            for (int d = 0; d < 3; d++) {
                const double np = q[d] * invh[d];
                double in = np - no[d];
                ic[d] = (int)in; cc[d] = in - (double)ic[d];
                in = np - nos[d];
                is[d] = (int)in; cs[d] = in - (double)is[d];
            }
        };
        auto tsc = [&](const double* q, int* nc, double (*wc)[3], int* ns, double (*ws)[3]) {
            for (int d = 0; d < 3; d++) {
                const double xi = q[d] * invh[d];
                nc[d] = (int)std::floor(xi + 0.5); tscWeights(xi - (double)nc[d], wc[d]);
                const double xs = xi - 0.5;
                ns[d] = (int)std::floor(xs + 0.5); tscWeights(xs - (double)ns[d], ws[d]);
            }
        };
        if (cic) {
            int ic[3], is[3]; double cc[3], cs[3];
            indexCoeff(pos, ic, cc, is, cs);
            for (int comp = 0; comp < 6; comp++) {
                const int* sg = kStag[comp];
                int b[3]; double cw[3];
                for (int d = 0; d < 3; d++) { b[d] = (sg[d] ? is[d] : ic[d]) - guard; cw[d] = sg[d] ? cs[d] : cc[d]; }
                const double* f = f6[comp];
                auto A = [&](int i, int j, int k) { return f[at(b[0] + i, b[1] + j, b[2] + k)]; };
                eb[comp] = A(0, 0, 0) * (1.0 - cw[0]) * (1.0 - cw[1]) * (1.0 - cw[2]) +
                           A(0, 0, 1) * (1.0 - cw[0]) * (1.0 - cw[1]) * cw[2] +
                           A(0, 1, 0) * (1.0 - cw[0]) * cw[1] * (1.0 - cw[2]) + A(0, 1, 1) * (1.0 - cw[0]) * cw[1] * cw[2] +
                           A(1, 0, 0) * cw[0] * (1.0 - cw[1]) * (1.0 - cw[2]) + A(1, 0, 1) * cw[0] * (1.0 - cw[1]) * cw[2] +
                           A(1, 1, 0) * cw[0] * cw[1] * (1.0 - cw[2]) + A(1, 1, 1) * cw[0] * cw[1] * cw[2];
            }
        } else {
            int nc[3], ns[3]; double wc[3][3], ws[3][3];
            tsc(pos, nc, wc, ns, ws);
            for (int comp = 0; comp < 6; comp++) {
                const int* sg = kStag[comp];
                const double* f = f6[comp];
                double r = 0.0;
                for (int a = 0; a < 3; a++) {
                    double ry = 0.0;
                    for (int b = 0; b < 3; b++) {
                        double rz = 0.0;
                        for (int k = 0; k < 3; k++)
                            rz += (sg[2] ? ws[2] : wc[2])[k] *
                                  f[at((sg[0] ? ns[0] : nc[0]) - 1 + a, (sg[1] ? ns[1] : nc[1]) - 1 + b,
                                       (sg[2] ? ns[2] : nc[2]) - 1 + k)];
                        ry += (sg[1] ? ws[1] : wc[1])[b] * rz;
                    }
                    r += (sg[0] ? ws[0] : wc[0])[a] * ry;
                }
                eb[comp] = r;
            }
        }
        const double ec = c->charge[sp] * c->dt / (2.0 * c->mass[sp] * kC);   // BorisPusher.h:29
        double u[3] = {ux[p], uy[p], uz[p]}, ig;
        boris<double>(ec, eb, eb + 3, u, ig);
        double v[3], np[3];
        for (int d = 0; d < 3; d++) {
            v[d] = (u[d] * kC) * ig;
            np[d] = pos[d] + v[d] * c->dt;
        }
        const double qw = c->charge[sp] * w[p];
        const double cur[3] = {(v[0] * qw) * norm, (v[1] * qw) * norm, (v[2] * qw) * norm};
        if (cic) {
            int ic[3], is[3]; double cc[3], cs[3];
            indexCoeff(np, ic, cc, is, cs);
            for (int comp = 0; comp < 3; comp++) {
                const int* sg = kStag[comp];
                int b[3]; double cw[3];
                for (int d = 0; d < 3; d++) { b[d] = (sg[d] ? is[d] : ic[d]) - guard; cw[d] = sg[d] ? cs[d] : cc[d]; }
                double* J = j3[comp];
                auto A = [&](int i, int j, int k) -> double& { return J[at(b[0] + i, b[1] + j, b[2] + k)]; };
                const double vv = cur[comp];
                A(0, 0, 0) += (1.0 - cw[0]) * (1.0 - cw[1]) * (1.0 - cw[2]) * vv;
                A(0, 0, 1) += (1.0 - cw[0]) * (1.0 - cw[1]) * cw[2] * vv;
                A(0, 1, 0) += (1.0 - cw[0]) * cw[1] * (1.0 - cw[2]) * vv;
                A(0, 1, 1) += (1.0 - cw[0]) * cw[1] * cw[2] * vv;
                A(1, 0, 0) += cw[0] * (1.0 - cw[1]) * (1.0 - cw[2]) * vv;
                A(1, 0, 1) += cw[0] * (1.0 - cw[1]) * cw[2] * vv;
                A(1, 1, 0) += cw[0] * cw[1] * (1.0 - cw[2]) * vv;
                A(1, 1, 1) += cw[0] * cw[1] * cw[2] * vv;
            }
        } else {
            int nc[3], ns[3]; double wc[3][3], ws[3][3];
            tsc(np, nc, wc, ns, ws);
            for (int comp = 0; comp < 3; comp++) {
                const int* sg = kStag[comp];
                double* J = j3[comp];
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) {
                        const double wxy = (sg[0] ? ws[0] : wc[0])[a] * (sg[1] ? ws[1] : wc[1])[b];
                        for (int k = 0; k < 3; k++)
                            J[at((sg[0] ? ns[0] : nc[0]) - 1 + a, (sg[1] ? ns[1] : nc[1]) - 1 + b,
                                 (sg[2] ? ns[2] : nc[2]) - 1 + k)] += wxy * (sg[2] ? ws[2] : wc[2])[k] * cur[comp];
                    }
            }
        }
        for (int d = 0; d < 3; d++) {
            if (np[d] < 0.0) np[d] += L[d];
            if (np[d] >= L[d]) np[d] -= L[d];
        }
        x[p] = np[0]; y[p] = np[1]; z[p] = np[2];
        ux[p] = u[0]; uy[p] = u[1]; uz[p] = u[2];
    }
    return 0;
}

}  // extern "C"
