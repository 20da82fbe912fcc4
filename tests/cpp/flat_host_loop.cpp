// A pica host loop over a flat ensemble on the C++ mirror: EnsembleUnordered (or,
// with "ordered", EnsembleOrdered and one reorder()) of ParticleArraySoA<Particle3d>,
// pica's grid-level FieldInterpolatorCIC / CurrentDepositorCIC on YeeGrid<Three,
// double>, BorisPusher and YeeSolver; the per-particle loop is one pushParticles call.
// Prints the particles in array order, then three field values.
//
// Usage: flat_host_loop <steps> <unordered|ordered>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "pica_gb300.hpp"

using namespace pica_gb300;

template <class Ens>
static void run(int steps, bool reorder) {
    const double n0 = 1e18;
    const double wp = std::sqrt(4 * constants::pi * n0 * constants::electronCharge * constants::electronCharge /
                                constants::electronMass);
    const double h = 0.05 * constants::c / wp;
    const double dt = 0.5 * h / (constants::c * std::sqrt(3.0));
    const Int3 numCells(8, 6, 10);
    const FP3 step(h, h, h), minPos(0, 0, 0);
    const FP3 maxPos = minPos + step * FP3(numCells.x, numCells.y, numCells.z);
    ParticleTypes::typesVector = {{constants::electronMass, constants::electronCharge},
                                  {constants::protonMass, -constants::electronCharge}};
    ParticleTypes::numTypes = 2;
    YeeGrid<Three, double> grid(minPos, step, numCells);
    Ens ensemble(minPos, maxPos);
    for (int i = 0; i < numCells.x; i++)
        for (int j = 0; j < numCells.y; j++)
            for (int k = 0; k < numCells.z; k++)
                for (int p = 0; p < 2; p++) {
                    Particle3d q;
                    // fill the array in reverse cell order, so that reorder() has work to do
                    const int ii = numCells.x - 1 - i;
                    q.position = FP3((ii + 0.2 + 0.5 * p) * h, (j + 0.35) * h, (k + 0.7 - 0.4 * p) * h);
                    q.setType((short)p);
                    q.setP(FP3(0.02 * ((ii + p) % 3 - 1), 0.03 * ((j + k) % 2) - 0.01, -0.015 + 0.01 * p));
                    q.setFactor(n0 * h * h * h / 2);
                    ensemble.add(q);
                }
    grid.ez(3, 4, 5) = 100.0;
    grid.by(1, 2, 3) = -50.0;
    grid.ex(7, 5, 9) = 30.0;
    if constexpr (std::is_same<Ens, EnsembleOrdered<ParticleArraySoA<Particle3d>>>::value)
        if (reorder) ensemble.reorder();
    BorisPusher<Particle3d, double> pusher(dt);
    YeeSolver solver;
    FieldInterpolatorCIC<YeeGrid<Three, double>> fi(grid);
    CurrentDepositorCIC<YeeGrid<Three, double>> cd(grid);
    for (int s = 0; s < steps; s++) {
        // was: for each particle: fi.get(...); pusher.push(...); cd.deposit(...);
        pushParticles(ensemble, fi, pusher, cd);
        solver.updateB(grid, 0.5 * dt);
        solver.updateE(grid, dt);
        solver.updateB(grid, 0.5 * dt);
    }
    const auto& arr = ensemble.getParticles();
    std::printf("%d\n", arr.size());
    for (int i = 0; i < arr.size(); i++) {
        const FP3 r = arr[i].getPosition(), p = arr[i].getP();
        std::printf("%d %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", arr[i].getType(), r.x, r.y, r.z, p.x, p.y, p.z,
                    arr[i].getFactor());
    }
    std::printf("fields %.17g %.17g %.17g\n", grid.ex(3, 4, 5), grid.jx(2, 2, 2), grid.bz(4, 4, 4));
}

int main(int argc, char** argv) {
    const int steps = argc > 1 ? std::atoi(argv[1]) : 3;
    const bool ordered = argc > 2 && std::strcmp(argv[2], "ordered") == 0;
    try {
        if (ordered) run<Ensemble<ParticleArraySoA<Particle3d>, EnsembleRepresentation_Ordered>::Type>(steps, true);
        else run<Ensemble<ParticleArraySoA<Particle3d>, EnsembleRepresentation_Unordered>::Type>(steps, false);
    } catch (const Error& e) {
        std::printf("error %d: %s\n", e.status, e.what());
        return 1;
    }
    return 0;
}
