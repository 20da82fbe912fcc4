// A pica-style host loop written against include/pica_gb300.hpp: build the
// grid and the supercell ensemble, then per step push every supercell,
// update B(dt/2), E(dt), B(dt/2) and migrate -- the same sequence a loop over
// pica's YeeSolver / FieldInterpolatorCICSupercell / BorisPusher /
// CurrentDepositorCICSupercell objects performs.  Prints the particles and
// fields so the test can compare with the Python binding of the same ABI.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "pica_gb300.hpp"

using namespace pica_gb300;

int main(int argc, char** argv) {
    const int steps = argc > 1 ? std::atoi(argv[1]) : 3;
    const double n0 = 1e18;
    const double wp = std::sqrt(4 * constants::pi * n0 * constants::electronCharge * constants::electronCharge /
                                constants::electronMass);
    const double h = 0.05 * constants::c / wp;
    Config cfg;
    cfg.numCells = Int3(8, 8, 8);
    cfg.numCellsPerSupercell = Int3(2, 2, 2);
    cfg.step = FP3(h, h, h);
    cfg.dt = 0.5 * h / (constants::c * std::sqrt(3.0));
    Simulation sim(cfg);
    auto& ens = sim.ensemble();
    // deterministic particles: 2 per cell, a small drift
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++)
            for (int k = 0; k < 8; k++)
                for (int p = 0; p < 2; p++) {
                    Particle3d q;
                    q.position = FP3((i + 0.25 + 0.5 * p) * h, (j + 0.3) * h, (k + 0.6 - 0.2 * p) * h);
                    q.p = FP3(0.01 * ((i + p) % 3 - 1), 0.02 * ((j + k) % 2), -0.01);
                    q.factor = n0 * h * h * h / 2;
                    ens.add(q);
                }
    ens.upload();
    auto& grid = sim.grid();
    grid.ez(3, 4, 5) = 100.0;
    grid.by(1, 2, 3) = -50.0;
    grid.upload();
    YeeSolver solver;
    for (int s = 0; s < steps; s++) {
        pushSupercells(sim);
        solver.updateB(grid, 0.5 * cfg.dt);
        solver.updateE(grid, cfg.dt);
        solver.updateB(grid, 0.5 * cfg.dt);
        ens.migrate();
    }
    auto parts = ens.particles();
    grid.download();
    std::printf("%zu\n", parts.size());
    for (auto& q : parts)
        std::printf("%.17g %.17g %.17g %.17g %.17g %.17g\n", q.position.x, q.position.y, q.position.z, q.p.x, q.p.y, q.p.z);
    std::printf("%.17g %.17g %.17g\n", grid.ex(3, 4, 5), grid.jx(2, 2, 2), grid.bz(4, 4, 4));
    return 0;
}
