// The C++ Driver over pica_gb300.hpp: diagnostics and checkpoint cadence, and a
// second Simulation that loads the last checkpoint and continues.  Prints the
// diagnostics steps, then "same" if the two final states agree bit for bit.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "pica_gb300.hpp"

using namespace pica_gb300;

static Config config(double h) {
    Config cfg;
    cfg.numCells = Int3(8, 8, 8);
    cfg.numCellsPerSupercell = Int3(4, 4, 4);
    cfg.step = FP3(h, h, h);
    cfg.dt = 0.5 * h / (constants::c * std::sqrt(3.0));
    cfg.form = Form::FP32Cell;
    cfg.shape = Shape::TSC;
    cfg.depositor = Depositor::Esirkepov;
    cfg.resortEvery = 2;
    return cfg;
}

int main(int argc, char** argv) {
    const std::string dir = argc > 1 ? argv[1] : ".";
    const double n0 = 1e18;
    const double wp = std::sqrt(4 * constants::pi * n0 * constants::electronCharge * constants::electronCharge /
                                constants::electronMass);
    const double h = 0.05 * constants::c / wp;
    Simulation sim(config(h));
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++)
            for (int k = 0; k < 8; k++)
                for (int p = 0; p < 3; p++) {
                    Particle3d q;
                    q.position = FP3((i + 0.2 + 0.3 * p) * h, (j + 0.35 + 0.1 * p) * h, (k + 0.7 - 0.25 * p) * h);
                    q.p = FP3(0.05 * ((i + p) % 3 - 1), 0.04 * ((j + k) % 2) - 0.02, 0.03 * (p - 1));
                    q.factor = n0 * h * h * h / 3;
                    sim.ensemble().add(q);
                }
    sim.ensemble().upload();
    sim.grid().upload();
    Driver drv(sim);
    drv.diagEvery = 2;
    drv.checkpointEvery = 3;
    drv.checkpointPath = dir + "/ckpt_";
    drv.onDiagnostics = [](int64_t step, const pica_diag& d) { std::printf("diag %lld %d\n", (long long)step, d.kinetic_energy > 0); };
    drv.run(7);
    Simulation again(config(h));
    again.loadCheckpoint(dir + "/ckpt_6");
    again.step(1);
    const auto a = sim.ensemble().particles(), b = again.ensemble().particles();
    bool same = a.size() == b.size() && sim.stepCount() == again.stepCount();
    for (size_t i = 0; same && i < a.size(); i++)
        same = a[i].position.x == b[i].position.x && a[i].position.y == b[i].position.y &&
               a[i].position.z == b[i].position.z && a[i].p.x == b[i].p.x && a[i].p.y == b[i].p.y && a[i].p.z == b[i].p.z;
    std::printf("%s\n", same ? "same" : "different");
    return 0;
}
