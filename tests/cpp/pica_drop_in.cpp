// A pica host loop -- the shape of the "before" loop a pica application writes --
// with three changes: the include, the namespace, and the per-particle supercell
// loop (fi.get / pusher.push / cd.deposit) replaced by one pushSupercells call.
// Everything else is pica's API: YeeGrid<Three, Real>, EnsembleSupercells of
// ParticleArraySoA<Particle3d>, the ParticleTypes table, BorisPusher, the
// supercell interpolator and depositor constructors, YeeSolver, element access to
// the fields and getParticles(idx) with particle references.
//
// Usage: pica_drop_in <steps> <fp64|fp32>
//   fp64: double operators, CIC interpolation and direct CIC deposition (pica's own);
//   fp32: float operators, TSC interpolation and Esirkepov deposition.
// After step 2 the loop changes one particle's momentum through its reference
// (the change reaches the device before the next push).  Prints the particles of
// every supercell in supercell order, then three field values.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "pica_gb300.hpp"   // was: the pica headers

using namespace pica_gb300;   // was: using namespace pica;

template <typename Real, template <class> class Interpolator, template <class> class Depositor>
static void run(int steps) {
    const double n0 = 1e18;
    const double wp = std::sqrt(4 * constants::pi * n0 * constants::electronCharge * constants::electronCharge /
                                constants::electronMass);
    const double h = 0.05 * constants::c / wp;
    const double dt = 0.5 * h / (constants::c * std::sqrt(3.0));
    const Int3 numCells(8, 8, 8), perSupercell(2, 2, 2);
    const FP3 step(h, h, h), minPos(-1.5 * h, 0.25 * h, 0.0);
    const FP3 maxPos = minPos + step * FP3(numCells.x, numCells.y, numCells.z);

    ParticleTypes::typesVector = {{constants::electronMass, constants::electronCharge},
                                  {constants::protonMass, -constants::electronCharge}};
    ParticleTypes::numTypes = 2;

    YeeGrid<Three, Real> grid(minPos, step, numCells);
    EnsembleSupercells<ParticleArraySoA<Particle3d>> ensemble(minPos, maxPos, numCells, perSupercell);
    for (int i = 0; i < numCells.x; i++)
        for (int j = 0; j < numCells.y; j++)
            for (int k = 0; k < numCells.z; k++)
                for (int p = 0; p < 3; p++) {
                    Particle3d q;
                    q.position = minPos + FP3((i + 0.2 + 0.3 * p) * h, (j + 0.35) * h, (k + 0.7 - 0.25 * p) * h);
                    q.setType((short)(p == 2));
                    q.setP(FP3(0.02 * ((i + p) % 3 - 1), 0.03 * ((j + k) % 2) - 0.01, -0.015 + 0.01 * p));
                    q.setFactor(n0 * h * h * h / 3);
                    ensemble.add(q);
                }
    grid.ez(3, 4, 5) = 100.0;
    grid.by(1, 2, 3) = -50.0;
    BorisPusher<Particle3d, Real> pusher((Real)dt);
    YeeSolver solver;
    for (int s = 0; s < steps; s++) {
        // was: for each supercell idx { FieldInterpolatorCICSupercell<Real> fi(...);
        //      CurrentDepositorCICSupercell<Real> cd(...); for each particle:
        //      fi.get(...); pusher.push(...); cd.deposit(...); }
        Interpolator<Real> fi(grid, ensemble.getMinPosition(), ensemble.getNumCellsPerSupercell());
        Depositor<Real> cd(grid, ensemble.getMinPosition(), ensemble.getNumCellsPerSupercell());
        pushSupercells(ensemble, fi, pusher, cd);
        solver.updateB(grid, (Real)(0.5 * dt));
        solver.updateE(grid, (Real)dt);
        solver.updateB(grid, (Real)(0.5 * dt));
        if (s == 1) {
            auto& arr = ensemble.getParticles(Int3(1, 2, 3));
            arr[0].setP(arr[0].getP() + FP3(0.05, 0.0, -0.02));
        }
    }
    const Int3 nsc = ensemble.getNumSupercells();
    for (int a = 0; a < nsc.x; a++)
        for (int b = 0; b < nsc.y; b++)
            for (int c = 0; c < nsc.z; c++) {
                const auto& arr = ensemble.getParticles(Int3(a, b, c));
                for (int i = 0; i < arr.size(); i++) {
                    const FP3 r = arr[i].getPosition(), p = arr[i].getP();
                    std::printf("%d %d %.17g %.17g %.17g %.17g %.17g %.17g\n", (a * nsc.y + b) * nsc.z + c, arr[i].getType(),
                                r.x, r.y, r.z, p.x, p.y, p.z);
                }
            }
    std::printf("fields %.17g %.17g %.17g\n", (double)grid.ex(3, 4, 5), (double)grid.jx(2, 2, 2),
                (double)grid.bz(4, 4, 4));
}

int main(int argc, char** argv) {
    const int steps = argc > 1 ? std::atoi(argv[1]) : 4;
    const bool fp32 = argc > 2 && std::strcmp(argv[2], "fp32") == 0;
    try {
        if (fp32) run<float, FieldInterpolatorTSCSupercell, CurrentDepositorEsirkepovSupercell>(steps);
        else run<double, FieldInterpolatorCICSupercell, CurrentDepositorCICSupercell>(steps);
    } catch (const Error& e) {
        std::printf("error %d: %s\n", e.status, e.what());
        return 1;
    }
    return 0;
}
