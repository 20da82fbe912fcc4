// The C++ mirror's host plumbing against tests/cpp/fake_abi.cpp (no GPU): a YeeGrid's
// arrays reach the ABI in z-fastest order and come back unchanged by every accessor;
// particles added through ParticleArraySoA references and Particle3d values reach the
// ABI as pica stores them (normalised momentum) and come back through particles(),
// size() and getParticles(idx), each supercell's particles species by species in
// upload order.  Prints "ok", or each failing check and "failed".
#include <cmath>
#include <cstdio>
#include <vector>

#include "pica_gb300.hpp"

using namespace pica_gb300;

int main() {
    int fails = 0;
    Config cfg;
    cfg.numCells = Int3(8, 6, 4);
    cfg.numCellsPerSupercell = Int3(2, 2, 2);
    cfg.step = FP3(0.1, 0.2, 0.3);
    cfg.dt = 1e-12;
    cfg.types = {{constants::electronMass, constants::electronCharge}, {constants::protonMass, -constants::electronCharge}};
    Simulation sim(cfg);
    if (ParticleTypes::numTypes != 2 || ParticleTypes::at(1).mass != constants::protonMass) {
        std::printf("Simulation did not install the type table\n");
        fails++;
    }

    // fields
    auto& g = sim.grid();
    const Int3 n = g.getSize();
    auto val = [](int c, int i, int j, int k) { return 1000.0 * c + 100.0 * i + 10.0 * j + k; };
    for (int i = 0; i < n.x; i++)
        for (int j = 0; j < n.y; j++)
            for (int k = 0; k < n.z; k++) {
                g.ex(i, j, k) = val(0, i, j, k);
                g.by(Int3(i, j, k)) = val(4, i, j, k);
                g.jz()(i, j, k) = val(8, i, j, k);
            }
    if (g.ex().data()[(2 * n.y + 3) * n.z + 1] != val(0, 2, 3, 1)) {
        std::printf("field storage is not z fastest\n");
        fails++;
    }
    g.upload();
    for (int i = 0; i < n.x; i++)
        for (int j = 0; j < n.y; j++)
            for (int k = 0; k < n.z; k++) g.ex(i, j, k) = g.by(i, j, k) = g.jz(i, j, k) = -1.0;
    g.download();
    for (int i = 0; i < n.x; i++)
        for (int j = 0; j < n.y; j++)
            for (int k = 0; k < n.z; k++)
                if (g.ex(i, j, k) != val(0, i, j, k) || g.by(i, j, k) != val(4, i, j, k) ||
                    g.jz(Int3(i, j, k)) != val(8, i, j, k) || g.ey(i, j, k) != 0.0) {
                    std::printf("field round trip at %d %d %d\n", i, j, k);
                    fails++;
                }

    // particles: half through a ParticleArraySoA, half as values
    auto& ens = sim.ensemble();
    ParticleArraySoA<Particle3d> arr;
    std::vector<Particle3d> all;
    for (int q = 0; q < 60; q++) {
        Particle3d p;
        p.position = FP3(0.0131 * ((q * 61) % 61), 0.0197 * ((q * 37) % 61), 0.0193 * ((q * 13) % 62));
        p.typeIndex = (short)(q % 3 == 0);
        p.setMomentum(FP3(1e-19 * (q - 30), 2e-19, -3e-19 * (q % 5)));
        p.factor = 1.0 + q;
        all.push_back(p);
        if (q % 2) arr.pushBack(p);
        else ens.add(p);
    }
    for (int i = 0; i < arr.size(); i++) ens.add(arr[i]);
    ens.upload();
    // the order the mirror uploaded in: the even particles, then the odd ones
    std::vector<Particle3d> uploaded;
    for (int q = 0; q < 60; q += 2) uploaded.push_back(all[q]);
    for (int q = 1; q < 60; q += 2) uploaded.push_back(all[q]);

    auto same = [](const Particle3d& a, const Particle3d& b) {
        return a.position == b.position && a.p == b.p && a.factor == b.factor && a.typeIndex == b.typeIndex;
    };
    if (ens.size() != 60 || ens.particles().size() != 60) {
        std::printf("particle count\n");
        fails++;
    }
    const Int3 nsc = ens.getNumSupercells();
    size_t seen = 0;
    for (int a = 0; a < nsc.x; a++)
        for (int b = 0; b < nsc.y; b++)
            for (int c = 0; c < nsc.z; c++) {
                std::vector<Particle3d> want;
                for (int t = 0; t < 2; t++)
                    for (const auto& p : uploaded)
                        if (p.typeIndex == t && ens.getSupercellIndex(p) == Int3(a, b, c)) want.push_back(p);
                const auto& arrOf = ens.getParticles(Int3(a, b, c));
                std::vector<Particle3d> got;
                for (int i = 0; i < arrOf.size(); i++) got.push_back(arrOf[i]);
                seen += got.size();
                bool ok = got.size() == want.size();
                for (size_t i = 0; ok && i < got.size(); i++) ok = same(got[i], want[i]);
                if (!ok) {
                    std::printf("supercell %d %d %d: %zu particles, want %zu\n", a, b, c, got.size(), want.size());
                    fails++;
                }
            }
    if (seen != 60) {
        std::printf("supercells hold %zu particles\n", seen);
        fails++;
    }

    // flat ensembles: pica's Ensemble traits, EnsembleUnordered keeps insertion order,
    // EnsembleOrdered::reorder applies the position order to every component
    typedef ParticleArray<Particle3d, ParticleRepresentation_SoA>::Type PA;
    Ensemble<PA, EnsembleRepresentation_Unordered>::Type flat(FP3(0, 0, 0), FP3(1, 1, 1));
    Ensemble<PA, EnsembleRepresentation_Ordered>::Type ordered(FP3(0, 0, 0), FP3(1, 1, 1));
    for (int i = 0; i < 40; i++) {
        Particle3d q;
        q.position = FP3(0.1 * ((i * 7) % 5), 0.05 * ((i * 3) % 4), 0.01 * i);
        q.p = FP3(i, -i, 0.5 * i);
        q.factor = 100.0 + i;
        q.typeIndex = (short)(i % 2);
        flat.add(q);
        ordered.add(q);
    }
    if (flat.size() != 40 || flat.getParticles()[7].getFactor() != 107.0) {
        std::printf("EnsembleUnordered does not keep insertion order\n");
        fails++;
    }
    ordered.reorder();
    const PA& o = ordered.getParticles();
    for (int i = 1; i < o.size(); i++) {
        const FP3 a = o[i - 1].getPosition(), b = o[i].getPosition();
        const bool le = a.x < b.x || (a.x == b.x && (a.y < b.y || (a.y == b.y && a.z <= b.z)));
        const int k = (int)o[i].getFactor() - 100;
        const bool same = o[i].getP().x == (double)k && o[i].getType() == (short)(k % 2) &&
                          o[i].getPosition().z == 0.01 * k;
        if (!le || !same) {
            std::printf("EnsembleOrdered::reorder: element %d out of order or torn\n", i);
            fails++;
            break;
        }
    }
    std::printf(fails ? "failed\n" : "ok\n");
    return fails ? 1 : 0;
}
