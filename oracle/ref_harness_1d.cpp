/*
 * ref_harness_1d.cpp -- host loop around pica's own 1D classes (TEST INFRASTRUCTURE).
 *
 * Built by oracle/Makefile against the pica sources where they lie (include
 * path only, nothing copied) into oracle/_ref/libpica_ref1d.so.  It produces
 * the golden vectors that pin the one-cell-thick (1D) use of the 3D kernels to
 * pica's YeeGrid<One> / FieldInterpolatorCIC<YeeGrid<One>> /
 * CurrentDepositorCIC<YeeGrid<One>> / YeeSolver (fieldSolver/YeeSolver.h:42-80)
 * path.  BorisPusher<Particle1d> does not compile (BorisPusher.h:45 adds a 3D
 * velocity to a 1D position), so the particles are pica Particle3d values at
 * (x, 0, 0) pushed by BorisPusher<Particle3d>, of which x is kept.  pica's 2D
 * counterparts do not compile either (FieldInterpolatorYeeGrid.h:107-118 read the
 * z of a 2D position), so there is no 2D harness.
 *
 * The host loop pica lacks, as in ref_harness.cpp:
 *   - a YeeGrid<One,double> of n + 4 nodes with origin -2h (2 guard nodes each
 *     side), filled and folded periodically;
 *   - per particle, in input order: FieldInterpolatorCIC::get -> BorisPusher::push
 *     -> CurrentDepositorCIC::deposit(x', v q w); J is then scaled by
 *     1 / (hx hy hz), the normalisation of the 3D supercell depositor
 *     (CurrentDepositorYeeGrid.h:201-213), with hy hz the cross-section of the
 *     one-cell-thick 3D grid it is compared with;
 *   - J guard fold, updateB(dt/2), updateE(dt), updateB(dt/2) with E/B guard fills;
 *   - periodic position wrap.  Particles keep their input order.
 */
#include "pica/math/Constants.h"
#include "pica/math/Vectors.h"
#include "pica/particles/Particle.h"
#include "pica/particles/ParticleArray.h"
#include "pica/grid/YeeGrid.h"
#include "pica/fieldSolver/YeeSolver.h"
#include "pica/fieldInterpolation/FieldInterpolator.h"
#include "pica/currentDeposition/CurrentDepositor.h"
#include "pica/particlePush/BorisPusher.h"

#include <cstdint>
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

inline int wrapi(int a, int n) { a %= n; return a < 0 ? a + n : a; }

}  // namespace

extern "C" {

/* Runs `steps` steps.  fields: 9 arrays of n doubles (ex ey ez bx by bz jx jy jz),
 * in: initial E and B; out: all nine after the last step.  x, ux, uy, uz: in and out
 * (u = p / (m c), pica's normalisation); w, species: in.  Returns 0. */
int ref1d_run(int32_t n, double h, double hyz, double dt, int32_t nspecies, const double* mass, const double* charge,
              int64_t np, double* x, double* ux, double* uy, double* uz, const double* w, const int32_t* species,
              double* fields, int32_t steps) {
    if (n <= 0 || np < 0 || nspecies < 1 || nspecies > 4) return -1;
    ParticleTypes::typesVector.resize(nspecies);
    for (int s = 0; s < nspecies; s++) {
        ParticleTypes::typesVector[s].mass = mass[s];
        ParticleTypes::typesVector[s].charge = charge[s];
    }
    ParticleTypes::types = &ParticleTypes::typesVector[0];
    ParticleTypes::numTypes = nspecies;

    typedef YeeGrid<One, double> Grid;
    Grid grid(-2.0 * h, h, n + 4);
    const int G = n + 4;
    auto at = [&](int c, int i) -> double& {
        switch (c) {
            case 0: return grid.ex(i);
            case 1: return grid.ey(i);
            case 2: return grid.ez(i);
            case 3: return grid.bx(i);
            case 4: return grid.by(i);
            case 5: return grid.bz(i);
            case 6: return grid.jx(i);
            case 7: return grid.jy(i);
            default: return grid.jz(i);
        }
    };
    for (int c = 0; c < 9; c++)
        for (int i = 0; i < G; i++) at(c, i) = 0.0;
    for (int c = 0; c < 6; c++)
        for (int i = 0; i < n; i++) at(c, i + 2) = fields[(int64_t)c * n + i];
    auto fill = [&](int c0, int c1) {
        for (int c = c0; c < c1; c++)
            for (int i = 0; i < G; i++)
                if (i < 2 || i >= n + 2) at(c, i) = at(c, wrapi(i - 2, n) + 2);
    };
    fill(0, 6);

    PArray particles;
    for (int64_t p = 0; p < np; p++) {
        Particle3d q;
        q.setPosition(FP3(x[p], 0.0, 0.0));
        q.setP(Vector3<double>(ux[p], uy[p], uz[p]));   // u = p / (m c), as pica stores it
        q.setFactor(w[p]);
        q.setType(species ? species[p] : 0);
        particles.pushBack(q);
    }
    const double L = (double)n * h;
    const double norm = 1.0 / (h * hyz);
    BorisPusher<Particle3d, double> pusher(dt);
    YeeSolver solver;
    for (int st = 0; st < steps; st++) {
        for (int c = 6; c < 9; c++)
            for (int i = 0; i < G; i++) at(c, i) = 0.0;
        FieldInterpolatorCIC<Grid> fi(grid);
        CurrentDepositorCIC<Grid> cd(grid);
        for (int p = 0; p < particles.size(); p++) {
            PArray::ParticleRef ref = particles[p];
            Vector3<double> e, b;
            fi.get(Vector1<double>(ref.getPosition().x), e, b);
            pusher.push(&ref, e, b);
            ref.setPosition(FP3(ref.getPosition().x, 0.0, 0.0));
            const Vector3<double> v = ref.getVelocity();
            cd.deposit(Vector1<double>(ref.getPosition().x), v * (charge[ref.getType()] * ref.getFactor()));
        }
        for (int c = 6; c < 9; c++) {
            for (int i = 0; i < G; i++)
                if (i < 2 || i >= n + 2) {
                    at(c, wrapi(i - 2, n) + 2) += at(c, i);
                    at(c, i) = 0.0;
                }
            for (int i = 2; i < n + 2; i++) at(c, i) *= norm;
        }
        solver.updateB(grid, 0.5 * dt); fill(3, 6);
        solver.updateE(grid, dt); fill(0, 3);
        solver.updateB(grid, 0.5 * dt); fill(3, 6);
        for (int p = 0; p < particles.size(); p++) {
            PArray::ParticleRef ref = particles[p];
            double px = ref.getPosition().x;
            if (px < 0.0) px += L;
            if (px >= L) px -= L;
            ref.setPosition(FP3(px, 0.0, 0.0));
        }
    }
    for (int c = 0; c < 9; c++)
        for (int i = 0; i < n; i++) fields[(int64_t)c * n + i] = at(c, i + 2);
    for (int p = 0; p < particles.size(); p++) {
        PArray::ConstParticleRef ref = particles[p];
        x[p] = ref.getPosition().x;
        const Vector3<double> pp = ref.getP();
        ux[p] = pp.x;
        uy[p] = pp.y;
        uz[p] = pp.z;
    }
    return 0;
}

}  // extern "C"
