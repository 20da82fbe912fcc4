/*
 * ref_harness.cpp -- host loop around pica's own headers (TEST INFRASTRUCTURE).
 *
 * Built by oracle/Makefile against the pica sources where they lie (include
 * path only, nothing copied) into oracle/_ref/libpica_ref.so.  It is the
 * reference implementation of the FP64 CIC / Boris / direct-deposition step
 * and pins the restatement in oracle/pic_oracle.cpp bit for bit.
 *
 * pica has no host loop (its README says it is the kernel core of PICADOR),
 * so this file supplies one:
 *   - a YeeGrid<Three,double> padded by 2 guard nodes below and 2 above, with
 *     origin -2h, which is what FieldInterpolatorCICSupercell and
 *     CurrentDepositorCICSupercell assume (FieldInterpolatorYeeGrid.h:201,205);
 *   - per supercell: FieldInterpolatorCICSupercell -> BorisPusher::push ->
 *     CurrentDepositorCICSupercell::deposit(x', v * q * w); the depositors are
 *     destroyed (flushed) serially in supercell order after the parallel
 *     particle phase, so the J sums have a fixed order;
 *   - periodic J guard fold, YeeSolver::updateB(dt/2), updateE(dt),
 *     updateB(dt/2) with periodic E/B guard fills;
 *   - periodic position wrap and supercell migration in the canonical order
 *     described in pic_oracle.h (dead slots marked x = -1e300; arrivals by
 *     direction code, then source slot, fill this step's holes, then append),
 *     and every resort_every steps a stable re-sort of each supercell by cell.
 */
#include "pica/math/Constants.h"
#include "pica/math/Vectors.h"
#include "pica/particles/Particle.h"
#include "pica/particles/ParticleArray.h"
#include "pica/particles/EnsembleSupercells.h"
#include "pica/particles/EnsembleOrdered.h"
#include "pica/particles/EnsembleUnordered.h"
#include "pica/grid/YeeGrid.h"
#include "pica/fieldSolver/YeeSolver.h"
#include "pica/fieldInterpolation/FieldInterpolator.h"
#include "pica/currentDeposition/CurrentDepositor.h"
#include "pica/particlePush/BorisPusher.h"

#include "pic_oracle.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace pica {
namespace ParticleTypes {
std::vector<ParticleType> typesVector;
const ParticleType* types = nullptr;
int numTypes = 0;
}  // namespace ParticleTypes
}  // namespace pica

using namespace pica;

namespace {

typedef ParticleArray<Particle3d, ParticleRepresentation_SoA>::Type PArray;
typedef EnsembleSupercells<PArray> Ensemble;

inline int wrapi(int a, int n) { a %= n; return a < 0 ? a + n : a; }

struct RefSim {
    orc_config cfg;
    Int3 N, S, nsc;
    FP3 h, L;
    YeeGrid<Three, double>* grid = nullptr;
    std::vector<Ensemble*> ens;
    struct Mig { int32_t sp, src, slot, dst; };
    std::vector<Mig> migrations;
    int err = 0;

    ~RefSim() { delete grid; for (auto e : ens) delete e; }

    int steps = 0;
    int scLinear(Int3 c) const { return (c.x * nsc.y + c.y) * nsc.z + c.z; }
    // Dead slots carry x = -1e300 (positions never go below -L, even before the wrap).
    static bool alive(PArray::ConstParticleRef p) { return p.getPosition().x > -1.0e299; }
    // Local cell of a particle in supercell s: (lx*Sy + ly)*Sz + lz.
    int cellKey(PArray::ConstParticleRef p, Int3 sc) const {
        FP3 x = p.getPosition();
        int l[3];
        for (int d = 0; d < 3; d++) {
            l[d] = (int)std::floor(x[d] * (1.0 / h[d])) - sc[d] * S[d];
            l[d] = std::min(std::max(l[d], 0), S[d] - 1);
        }
        return (l[0] * S.y + l[1]) * S.z + l[2];
    }
    // Drop dead slots and sort each supercell by cell (stable).
    void resort() {
        const int nscTot = nsc.x * nsc.y * nsc.z;
        for (auto e : ens) {
#pragma omp parallel for schedule(dynamic, 8)
            for (int s = 0; s < nscTot; s++) {
                Int3 c = scCoords(s);
                PArray& arr = e->getParticles(c);
                const PArray& carr = arr;
                std::vector<std::pair<int, int>> key;
                for (int p = 0; p < arr.size(); p++)
                    if (alive(carr[p])) key.push_back({cellKey(carr[p], c), p});
                std::stable_sort(key.begin(), key.end(),
                                 [](const std::pair<int, int>& a, const std::pair<int, int>& b) { return a.first < b.first; });
                PArray out;
                for (auto& k : key) out.pushBack(carr[k.second]);
                arr = out;
            }
        }
    }
    Int3 scCoords(int s) const { return Int3(s / (nsc.y * nsc.z), (s / nsc.z) % nsc.y, s % nsc.z); }

    void init(const orc_config& c) {
        cfg = c;
        N = Int3(c.n[0], c.n[1], c.n[2]);
        S = Int3(c.sc[0], c.sc[1], c.sc[2]);
        nsc = Int3(N.x / S.x, N.y / S.y, N.z / S.z);
        h = FP3(c.h[0], c.h[1], c.h[2]);
        L = FP3((double)N.x * h.x, (double)N.y * h.y, (double)N.z * h.z);
        grid = new YeeGrid<Three, double>(FP3(-2.0 * h.x, -2.0 * h.y, -2.0 * h.z), h, N + Int3(4, 4, 4));
        ParticleTypes::typesVector.resize(c.nspecies);
        for (int s = 0; s < c.nspecies; s++) {
            ParticleTypes::typesVector[s].mass = c.mass[s];
            ParticleTypes::typesVector[s].charge = c.charge[s];
        }
        ParticleTypes::types = &ParticleTypes::typesVector[0];
        ParticleTypes::numTypes = c.nspecies;
        for (int s = 0; s < c.nspecies; s++) ens.push_back(new Ensemble(FP3(0, 0, 0), L, N, S));
#ifdef _OPENMP
        if (c.threads > 0) omp_set_num_threads(c.threads);
#endif
    }

    Int3 supercellOf(Ensemble& e, PArray::ConstParticleRef p) {
        Int3 c = e.getSupercellIndex(p);   // EnsembleSupercells.h:54-57
        c.x = std::min(std::max(c.x, 0), nsc.x - 1);
        c.y = std::min(std::max(c.y, 0), nsc.y - 1);
        c.z = std::min(std::max(c.z, 0), nsc.z - 1);
        return c;
    }

    // Periodic guard handling on the padded grid (guard width 2).
    bool guard(int gx, int gy, int gz) const {
        return gx < 2 || gy < 2 || gz < 2 || gx >= N.x + 2 || gy >= N.y + 2 || gz >= N.z + 2;
    }
    Int3 image(int gx, int gy, int gz) const {
        return Int3(wrapi(gx - 2, N.x) + 2, wrapi(gy - 2, N.y) + 2, wrapi(gz - 2, N.z) + 2);
    }
    template <class Get>
    void fillComponent(Get get) {
        Int3 sz = grid->getSize();
        for (int i = 0; i < sz.x; i++)
            for (int j = 0; j < sz.y; j++)
                for (int k = 0; k < sz.z; k++)
                    if (guard(i, j, k)) { Int3 m = image(i, j, k); get(i, j, k) = get(m.x, m.y, m.z); }
    }
    void fillE() {
        fillComponent([&](int i, int j, int k) -> double& { return grid->ex(i, j, k); });
        fillComponent([&](int i, int j, int k) -> double& { return grid->ey(i, j, k); });
        fillComponent([&](int i, int j, int k) -> double& { return grid->ez(i, j, k); });
    }
    void fillB() {
        fillComponent([&](int i, int j, int k) -> double& { return grid->bx(i, j, k); });
        fillComponent([&](int i, int j, int k) -> double& { return grid->by(i, j, k); });
        fillComponent([&](int i, int j, int k) -> double& { return grid->bz(i, j, k); });
    }
    void foldJ() {
        Int3 sz = grid->getSize();
        for (int i = 0; i < sz.x; i++)
            for (int j = 0; j < sz.y; j++)
                for (int k = 0; k < sz.z; k++)
                    if (guard(i, j, k)) {
                        Int3 m = image(i, j, k);
                        grid->jx(m.x, m.y, m.z) += grid->jx(i, j, k); grid->jx(i, j, k) = 0;
                        grid->jy(m.x, m.y, m.z) += grid->jy(i, j, k); grid->jy(i, j, k) = 0;
                        grid->jz(m.x, m.y, m.z) += grid->jz(i, j, k); grid->jz(i, j, k) = 0;
                    }
    }

    void step() {
        const int nscTot = nsc.x * nsc.y * nsc.z;
        Int3 sz = grid->getSize();
        for (int i = 0; i < sz.x; i++) for (int j = 0; j < sz.y; j++) for (int k = 0; k < sz.z; k++)
            grid->jx(i, j, k) = grid->jy(i, j, k) = grid->jz(i, j, k) = 0;
        BorisPusher<Particle3d, double> pusher(cfg.dt);
        std::vector<CurrentDepositorCICSupercell<double>*> deps(nscTot, nullptr);
#pragma omp parallel for schedule(dynamic, 4)
        for (int s = 0; s < nscTot; s++) {
            Int3 c = scCoords(s);
            FP3 minPos((double)(c.x * S.x) * h.x, (double)(c.y * S.y) * h.y, (double)(c.z * S.z) * h.z);
            FieldInterpolatorCICSupercell<double> fi(*grid, minPos, S);
            CurrentDepositorCICSupercell<double>* cd = new CurrentDepositorCICSupercell<double>(*grid, minPos, S);
            for (int sp = 0; sp < cfg.nspecies; sp++) {
                PArray& arr = ens[sp]->getParticles(c);
                const double q = cfg.charge[sp];
                for (int p = 0; p < arr.size(); p++) {
                    PArray::ParticleRef ref = arr[p];
                    if (!alive(ref)) continue;
                    FP3 e, b;
                    fi.get(ref.getPosition(), e, b);
                    pusher.push(&ref, e, b);
                    FP3 v = ref.getVelocity();
                    cd->deposit(ref.getPosition(), v * (q * ref.getFactor()));
                }
            }
            deps[s] = cd;
        }
        for (int s = 0; s < nscTot; s++) delete deps[s];   // flush in supercell order
        foldJ();
        YeeSolver solver;
        solver.updateB(*grid, 0.5 * cfg.dt); fillB();
        solver.updateE(*grid, cfg.dt); fillE();
        solver.updateB(*grid, 0.5 * cfg.dt); fillB();
        migrate();
    }

    void migrate() {
        migrations.clear();
        const int nscTot = nsc.x * nsc.y * nsc.z;
        for (int sp = 0; sp < cfg.nspecies; sp++) {
            Ensemble& e = *ens[sp];
            std::vector<std::vector<int>> dirs(nscTot);   // -1: dead slot
            int localErr = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(min : localErr)
            for (int s = 0; s < nscTot; s++) {
                Int3 o = scCoords(s);
                PArray& arr = e.getParticles(o);
                dirs[s].assign(arr.size(), -1);
                for (int p = 0; p < arr.size(); p++) {
                    PArray::ParticleRef ref = arr[p];
                    if (!alive(ref)) continue;
                    FP3 x = ref.getPosition();
                    for (int d = 0; d < 3; d++) {
                        if (x[d] < 0.0) x[d] += L[d];
                        if (x[d] >= L[d]) x[d] -= L[d];
                    }
                    ref.setPosition(x);
                    Int3 nw = supercellOf(e, ref);
                    int code = 0;
                    for (int d = 0; d < 3; d++) {
                        int ds = nw[d] - o[d];
                        if (ds > 1) ds -= nsc[d];
                        if (ds < -1) ds += nsc[d];
                        if (ds < -1 || ds > 1) { localErr = -5; ds = 0; }
                        code = code * 3 + ds + 1;
                    }
                    dirs[s][p] = code;
                }
            }
            if (localErr) err = localErr;
            for (int s = 0; s < nscTot; s++) {
                Int3 o = scCoords(s);
                for (int p = 0; p < (int)dirs[s].size(); p++) {
                    int code = dirs[s][p];
                    if (code < 0 || code == 13) continue;
                    Int3 ds(code / 9 - 1, (code / 3) % 3 - 1, code % 3 - 1);
                    int dst = scLinear(Int3(wrapi(o.x + ds.x, nsc.x), wrapi(o.y + ds.y, nsc.y), wrapi(o.z + ds.z, nsc.z)));
                    migrations.push_back({sp, s, p, dst});
                }
            }
            std::vector<PArray> next(nscTot);
#pragma omp parallel for schedule(dynamic, 8)
            for (int d = 0; d < nscTot; d++) {
                Int3 dc = scCoords(d);
                next[d] = e.getParticles(dc);
                std::vector<int> holes;
                for (int p = 0; p < (int)dirs[d].size(); p++)
                    if (dirs[d][p] >= 0 && dirs[d][p] != 13) {
                        holes.push_back(p);
                        PArray::ParticleRef r = next[d][p];
                        FP3 x = r.getPosition();
                        x.x = -1.0e300;
                        r.setPosition(x);
                    }
                size_t k = 0;
                for (int code = 0; code < 27; code++) {
                    if (code == 13) continue;
                    Int3 ds(code / 9 - 1, (code / 3) % 3 - 1, code % 3 - 1);
                    int src = scLinear(Int3(wrapi(dc.x - ds.x, nsc.x), wrapi(dc.y - ds.y, nsc.y), wrapi(dc.z - ds.z, nsc.z)));
                    const PArray& arr = e.getParticles(scCoords(src));
                    for (int p = 0; p < arr.size(); p++)
                        if (dirs[src][p] == code) {
                            if (k < holes.size()) {
                                PArray::ParticleRef r = next[d][holes[k]];
                                PArray::ConstParticleRef a = arr[p];
                                r.setPosition(a.getPosition());
                                r.setP(a.getP());
                                r.setFactor(a.getFactor());
                                r.setType(a.getType());
                            } else {
                                next[d].pushBack(arr[p]);
                            }
                            k++;
                        }
                }
            }
            for (int s = 0; s < nscTot; s++) e.getParticles(scCoords(s)) = next[s];
        }
        steps++;
        if (cfg.resort_every > 0 && steps % cfg.resort_every == 0) resort();
    }
};

}  // namespace

extern "C" {

void* ref_create(const orc_config* cfg) {
    if (!cfg || cfg->form != ORC_FORM_FP64_PLAIN || cfg->shape != ORC_SHAPE_CIC || cfg->deposit != ORC_DEPOSIT_DIRECT)
        return nullptr;
    for (int d = 0; d < 3; d++)
        if (cfg->n[d] <= 0 || cfg->sc[d] <= 0 || cfg->n[d] % cfg->sc[d] != 0 || cfg->sc[d] > 4) return nullptr;
    RefSim* s = new RefSim();
    s->init(*cfg);
    return s;
}

void ref_destroy(void* sim) { delete (RefSim*)sim; }

int ref_load(void* sim, int64_t n, const double* x, const double* y, const double* z, const double* ux,
             const double* uy, const double* uz, const double* w, const int32_t* species) {
    RefSim* s = (RefSim*)sim;
    if (!s) return -1;
    for (int64_t i = 0; i < n; i++) {
        int sp = species ? species[i] : 0;
        if (sp < 0 || sp >= s->cfg.nspecies) return -2;
        Particle3d p;
        p.setPosition(FP3(x[i], y[i], z[i]));
        p.setP(FP3(ux[i], uy[i], uz[i]));
        p.setFactor(w[i]);
        p.setType((short)sp);
        PArray tmp; tmp.pushBack(p);
        Int3 c = s->supercellOf(*s->ens[sp], tmp[0]);
        s->ens[sp]->getParticles(c).pushBack(p);
    }
    s->resort();
    return 0;
}

int ref_set_fields(void* sim, const double* const* f9) {
    RefSim* s = (RefSim*)sim;
    if (!s) return -1;
    Int3 N = s->N;
    for (int i = 0; i < N.x; i++)
        for (int j = 0; j < N.y; j++)
            for (int k = 0; k < N.z; k++) {
                size_t o = ((size_t)i * N.y + j) * N.z + k;
                int a = i + 2, b = j + 2, c = k + 2;
                s->grid->ex(a, b, c) = f9[0][o]; s->grid->ey(a, b, c) = f9[1][o]; s->grid->ez(a, b, c) = f9[2][o];
                s->grid->bx(a, b, c) = f9[3][o]; s->grid->by(a, b, c) = f9[4][o]; s->grid->bz(a, b, c) = f9[5][o];
                s->grid->jx(a, b, c) = f9[6][o]; s->grid->jy(a, b, c) = f9[7][o]; s->grid->jz(a, b, c) = f9[8][o];
            }
    s->fillE(); s->fillB();
    return 0;
}

int ref_get_fields(void* sim, double* const* f9) {
    RefSim* s = (RefSim*)sim;
    if (!s) return -1;
    Int3 N = s->N;
    for (int i = 0; i < N.x; i++)
        for (int j = 0; j < N.y; j++)
            for (int k = 0; k < N.z; k++) {
                size_t o = ((size_t)i * N.y + j) * N.z + k;
                int a = i + 2, b = j + 2, c = k + 2;
                f9[0][o] = s->grid->ex(a, b, c); f9[1][o] = s->grid->ey(a, b, c); f9[2][o] = s->grid->ez(a, b, c);
                f9[3][o] = s->grid->bx(a, b, c); f9[4][o] = s->grid->by(a, b, c); f9[5][o] = s->grid->bz(a, b, c);
                f9[6][o] = s->grid->jx(a, b, c); f9[7][o] = s->grid->jy(a, b, c); f9[8][o] = s->grid->jz(a, b, c);
            }
    return 0;
}

int ref_step(void* sim, int32_t nsteps) {
    RefSim* s = (RefSim*)sim;
    if (!s) return -1;
    for (int i = 0; i < nsteps; i++) {
        s->step();
        if (s->err) return s->err;
    }
    return 0;
}

int64_t ref_num_particles(void* sim) {
    RefSim* s = (RefSim*)sim;
    if (!s) return -1;
    int64_t n = 0;
    int nscTot = s->nsc.x * s->nsc.y * s->nsc.z;
    for (auto e : s->ens)
        for (int k = 0; k < nscTot; k++) {
            const PArray& arr = e->getParticles(s->scCoords(k));
            for (int p = 0; p < arr.size(); p++) n += RefSim::alive(arr[p]) ? 1 : 0;
        }
    return n;
}

int ref_get_particles(void* sim, double* x, double* y, double* z, double* ux, double* uy, double* uz, double* w,
                      int32_t* species, int32_t* supercell) {
    RefSim* s = (RefSim*)sim;
    if (!s) return -1;
    int nscTot = s->nsc.x * s->nsc.y * s->nsc.z;
    int64_t o = 0;
    for (int sp = 0; sp < s->cfg.nspecies; sp++)
        for (int k = 0; k < nscTot; k++) {
            PArray& arr = s->ens[sp]->getParticles(s->scCoords(k));
            for (int p = 0; p < arr.size(); p++) {
                PArray::ConstParticleRef r = ((const PArray&)arr)[p];
                if (!RefSim::alive(r)) continue;
                FP3 pos = r.getPosition(), u = r.getP();
                x[o] = pos.x; y[o] = pos.y; z[o] = pos.z;
                ux[o] = u.x; uy[o] = u.y; uz[o] = u.z; w[o] = r.getFactor();
                if (species) species[o] = sp;
                if (supercell) supercell[o] = k;
                o++;
            }
        }
    return 0;
}

int ref_get_counts(void* sim, int32_t* counts) {
    RefSim* s = (RefSim*)sim;
    if (!s) return -1;
    int nscTot = s->nsc.x * s->nsc.y * s->nsc.z;
    for (int sp = 0; sp < s->cfg.nspecies; sp++)
        for (int k = 0; k < nscTot; k++) {
            const PArray& arr = s->ens[sp]->getParticles(s->scCoords(k));
            int32_t n = 0;
            for (int p = 0; p < arr.size(); p++) n += RefSim::alive(arr[p]) ? 1 : 0;
            counts[(size_t)sp * nscTot + k] = n;
        }
    return 0;
}

int64_t ref_num_migrations(void* sim) {
    RefSim* s = (RefSim*)sim;
    return s ? (int64_t)s->migrations.size() : -1;
}

int ref_get_migrations(void* sim, int32_t* species, int32_t* src, int32_t* slot, int32_t* dst) {
    RefSim* s = (RefSim*)sim;
    if (!s) return -1;
    for (size_t i = 0; i < s->migrations.size(); i++) {
        species[i] = s->migrations[i].sp; src[i] = s->migrations[i].src;
        slot[i] = s->migrations[i].slot; dst[i] = s->migrations[i].dst;
    }
    return 0;
}

// EnsembleOrdered::reorder (EnsembleOrdered.h:61-71) on particles whose factor is
// their input index, so that the reordered factors give the permutation.
int ref_order_by_position(int64_t n, int32_t dims, const double* x, const double* y, const double* z, int64_t* order) {
    if (dims != 3) return -1;   // Particle3d: pica compares all three coordinates
    (void)dims;
    if (n > (int64_t)1 << 31) return -1;
    EnsembleOrdered<PArray> e(FP3(-1e300, -1e300, -1e300), FP3(1e300, 1e300, 1e300));
    for (int64_t i = 0; i < n; i++) {
        Particle3d p;
        p.setPosition(FP3(x[i], y[i], z[i]));
        p.setFactor((double)i);
        e.add(p);
    }
    e.reorder();
    const PArray& arr = e.getParticles();
    for (int i = 0; i < arr.size(); i++) order[i] = (int64_t)arr[i].getFactor();
    return 0;
}

// One push of a flat array through pica's grid-level classes: EnsembleUnordered,
// FieldInterpolatorCIC<YeeGrid<Three, double>>, BorisPusher and
// CurrentDepositorCIC<YeeGrid<Three, double>> on a grid with origin -guard h and
// periodic guard layers (filled before the gather, folded after the deposit).
// The current passed to the depositor is v (q w) / (hx hy hz).
int ref_push_flat(const orc_config* c, int32_t guard, int64_t n, double* x, double* y, double* z, double* ux,
                  double* uy, double* uz, const double* w, const int32_t* species, const double* const* f6,
                  double* const* j3) {
    if (!c || c->shape != ORC_SHAPE_CIC || c->deposit != ORC_DEPOSIT_DIRECT || guard < 2) return -1;
    const Int3 N(c->n[0], c->n[1], c->n[2]);
    const FP3 h(c->h[0], c->h[1], c->h[2]);
    const FP3 L((double)N.x * h.x, (double)N.y * h.y, (double)N.z * h.z);
    YeeGrid<Three, double> grid(FP3(-(double)guard * h.x, -(double)guard * h.y, -(double)guard * h.z), h,
                                N + Int3(2 * guard, 2 * guard, 2 * guard));
    const Int3 sz = grid.getSize();
    auto img = [&](int i, int j, int k) {
        return ((size_t)wrapi(i - guard, N.x) * N.y + wrapi(j - guard, N.y)) * N.z + wrapi(k - guard, N.z);
    };
    for (int i = 0; i < sz.x; i++)
        for (int j = 0; j < sz.y; j++)
            for (int k = 0; k < sz.z; k++) {
                const size_t o = img(i, j, k);
                grid.ex(i, j, k) = f6[0][o]; grid.ey(i, j, k) = f6[1][o]; grid.ez(i, j, k) = f6[2][o];
                grid.bx(i, j, k) = f6[3][o]; grid.by(i, j, k) = f6[4][o]; grid.bz(i, j, k) = f6[5][o];
                grid.jx(i, j, k) = 0; grid.jy(i, j, k) = 0; grid.jz(i, j, k) = 0;
            }
    ParticleTypes::typesVector.resize(c->nspecies);
    for (int q = 0; q < c->nspecies; q++) {
        ParticleTypes::typesVector[q].mass = c->mass[q];
        ParticleTypes::typesVector[q].charge = c->charge[q];
    }
    ParticleTypes::types = &ParticleTypes::typesVector[0];
    ParticleTypes::numTypes = c->nspecies;
    EnsembleUnordered<PArray> e(FP3(0, 0, 0), L);
    for (int64_t i = 0; i < n; i++) {
        Particle3d p;
        p.setPosition(FP3(x[i], y[i], z[i]));
        p.setP(FP3(ux[i], uy[i], uz[i]));
        p.setFactor(w[i]);
        p.setType((short)(species ? species[i] : 0));
        e.add(p);
    }
    FieldInterpolatorCIC<YeeGrid<Three, double> > fi(grid);
    CurrentDepositorCIC<YeeGrid<Three, double> > cd(grid);
    BorisPusher<Particle3d, double> pusher(c->dt);
    const double norm = 1.0 / (h.x * h.y * h.z);
    PArray& arr = e.getParticles();
    for (int i = 0; i < arr.size(); i++) {
        PArray::ParticleRef ref = arr[i];
        FP3 ef, bf;
        fi.get(ref.getPosition(), ef, bf);
        pusher.push(&ref, ef, bf);
        const double q = c->charge[ref.getType()];
        cd.deposit(ref.getPosition(), ref.getVelocity() * (q * ref.getFactor()) * norm);
        FP3 r = ref.getPosition();
        for (int d = 0; d < 3; d++) {
            if (r[d] < 0.0) r[d] += L[d];
            if (r[d] >= L[d]) r[d] -= L[d];
        }
        ref.setPosition(r);
        x[i] = r.x; y[i] = r.y; z[i] = r.z;
        const FP3 u = ref.getP();
        ux[i] = u.x; uy[i] = u.y; uz[i] = u.z;
    }
    for (int i = 0; i < sz.x; i++)
        for (int j = 0; j < sz.y; j++)
            for (int k = 0; k < sz.z; k++) {
                const size_t o = img(i, j, k);
                j3[0][o] += grid.jx(i, j, k); j3[1][o] += grid.jy(i, j, k); j3[2][o] += grid.jz(i, j, k);
            }
    return 0;
}

}  // extern "C"
