// pica's particle, constants and grid known-answer checks (test/src/particles/ParticleTests.cpp:37-164,
// test/src/math/ConstantsTests.cpp:15-28, test/src/grid/YeeGridTests.cpp:115-134,
// test/src/particles/ParticleArrayTests.cpp:38-136) restated
// against the C++ mirror: Constants<T> equals the cast namespace value for float and double;
// a particle built from a momentum returns it, with gamma = sqrt(1 + |P|^2 / (m c)^2) to
// 1e-12; momentum and velocity round-trip to 1e-12; mass and charge come from the type
// table; a YeeGrid returns its step and size, the cell of every cell centre, its values by
// every accessor in z-fastest order, and pica's staggering shifts; an EnsembleSupercells
// routes every supercell centre to its supercell (floor rule); a ParticleArraySoA keeps
// every particle as pushed through index access, back, copies and popBack, and its
// references set momentum and velocity like a particle.  Host-only, no GPU.
// Prints "ok", or each failing check and "failed".
#include <cmath>
#include <cstdio>
#include <vector>

#include "pica_gb300.hpp"

using namespace pica_gb300;

static int fails = 0;

static void near(const char* what, double want, double got, double rel = 1e-12) {
    const double err = std::fabs(want - got), scale = std::fmax(std::fabs(want), 1e-300);
    if (!(err <= rel * scale)) {
        std::printf("%s: want %.17g got %.17g\n", what, want, got);
        fails++;
    }
}

static void nearVec(const char* what, const FP3& want, const FP3& got) {
    // relative to the vector's norm, as pica's ASSERT_NEAR_VECTOR
    const double err = (want - got).norm(), scale = std::fmax(want.norm(), 1e-300);
    if (!(err <= 1e-12 * scale)) {
        std::printf("%s: error %.3g of %.3g\n", what, err, scale);
        fails++;
    }
}

template <typename T>
static void constantsOf(const char* name) {
    const bool ok = Constants<T>::pi() == static_cast<T>(constants::pi) && Constants<T>::c() == static_cast<T>(constants::c) &&
                    Constants<T>::lightVelocity() == static_cast<T>(constants::lightVelocity) &&
                    Constants<T>::electronCharge() == static_cast<T>(constants::electronCharge) &&
                    Constants<T>::electronMass() == static_cast<T>(constants::electronMass) &&
                    Constants<T>::protonMass() == static_cast<T>(constants::protonMass) &&
                    Constants<T>::planck() == static_cast<T>(constants::planck) &&
                    Constants<T>::eV() == static_cast<T>(constants::eV) && Constants<T>::meV() == static_cast<T>(constants::meV);
    if (!ok) {
        std::printf("Constants<%s> differ from the namespace values\n", name);
        fails++;
    }
}

int main() {
    constantsOf<float>("float");
    constantsOf<double>("double");

    ParticleTypes::typesVector = {{constants::electronMass, constants::electronCharge},
                                  {constants::protonMass, -constants::electronCharge}};
    ParticleTypes::types = nullptr;
    ParticleTypes::numTypes = 2;

    Particle3d def;
    if (def.getGamma() != 1.0 || def.getFactor() != 1.0 || def.getVelocity().norm2() != 0.0) {
        std::printf("default particle\n");
        fails++;
    }

    const FP3 pos(3.1, -32.1, 4.3e-5), mom(-231.3e9, 0.0, 1.23e-5);
    Particle3d q(pos, mom, 1.4e2, 0);
    if (q.getPosition().x != pos.x || q.getPosition().y != pos.y || q.getPosition().z != pos.z) {
        std::printf("position\n");
        fails++;
    }
    nearVec("momentum from the constructor", mom, q.getMomentum());
    near("mass", constants::electronMass, q.getMass(), 0);
    near("charge", constants::electronCharge, q.getCharge(), 0);
    near("factor", 1.4e2, q.getFactor(), 0);
    const double mc = q.getMass() * Constants<double>::c();
    near("gamma", std::sqrt(1.0 + mom.norm2() / (mc * mc)), q.getGamma());

    const FP3 m2(54.12e+4, -543.63e-2, 643.165e5);
    q.setMomentum(m2);
    nearVec("set / get momentum", m2, q.getMomentum());
    near("gamma after setMomentum", std::sqrt(1.0 + m2.norm2() / (mc * mc)), q.getGamma());

    const FP3 v(5243.1654, -56.23e5, -65.237e-4);
    q.setVelocity(v);
    nearVec("set / get velocity", v, q.getVelocity());

    Particle3d ion(pos, mom, 2.0, 1);
    near("ion mass", constants::protonMass, ion.getMass(), 0);
    near("ion charge", -constants::electronCharge, ion.getCharge(), 0);
    const double mci = constants::protonMass * constants::c;
    near("ion gamma", std::sqrt(1.0 + mom.norm2() / (mci * mci)), ion.getGamma());
    ion.setType(0);
    near("mass after setType", constants::electronMass, ion.getMass(), 0);

    // p is pica's normalised momentum: setP / getP, and P = p m c
    Particle3d r;
    r.setP(FP3(0.3, -0.4, 1.2));
    nearVec("momentum from p", FP3(0.3, -0.4, 1.2) * mc, r.getMomentum());
    near("gamma from p", std::sqrt(1.0 + 0.09 + 0.16 + 1.44), r.getGamma());

    // YeeGrid<Three> (grid/Grid.h:13-83, grid/YeeGrid.h:193-256) as a host container
    const FP3 origin(1.25, -4.5, 0.75), step(0.1, 0.2, 0.05);
    const Int3 size(5, 6, 7);
    YeeGrid<Three, double> g(origin, step, size);
    if (!(g.getStep() == step) || !(g.getSize() == size) || !(g.getOrigin() == origin)) {
        std::printf("grid step / size / origin\n");
        fails++;
    }
    for (int i = 0; i < size.x; i++)
        for (int j = 0; j < size.y; j++)
            for (int k = 0; k < size.z; k++) {
                const FP3 centre = origin + step * FP3(i + 0.5, j + 0.5, k + 0.5);
                if (!(g.getCellIndex(centre) == Int3(i, j, k))) {
                    std::printf("cell index of centre %d %d %d\n", i, j, k);
                    fails++;
                }
                g.ey(i, j, k) = 100.0 * i + 10.0 * j + k;
            }
    const YeeGrid<Three, double>& cg = g;
    const Int3 n(3, 2, 5);
    const double want = 100.0 * 3 + 10.0 * 2 + 5;
    if (cg.ey(3, 2, 5) != want || cg.ey(n) != want || g.ey()(3, 2, 5) != want || g.ey()(n) != want ||
        cg.ey().data()[(3 * size.y + 2) * size.z + 5] != want || g.ex(n) != 0.0) {
        std::printf("grid accessors\n");
        fails++;
    }
    if (!(g.getShiftEx() == FP3(0, 0.1, 0.025)) || !(g.getShiftBz() == FP3(0, 0, 0.025)) ||
        !(g.getShiftJy() == FP3(0.05, 0, 0.025)) || !(g.getShiftBx() == FP3(0.05, 0, 0))) {
        std::printf("staggering shifts\n");
        fails++;
    }
    try {
        g.upload();
        std::printf("upload of a grid without a Simulation did not throw\n");
        fails++;
    } catch (const Error& e) {
        if (e.status != PICA_ERR_INVALID) {
            std::printf("upload of a grid without a Simulation: status %d\n", e.status);
            fails++;
        }
    }

    // ParticleArraySoA (particles/ParticleArray.h:46-203; ParticleArrayTests.cpp:38-136):
    // size, index access, back, copies and popBack keep every particle as pushed
    {
        auto same = [](const Particle3d& a, const Particle3d& b) {
            return a.position == b.position && a.p == b.p && a.factor == b.factor && a.typeIndex == b.typeIndex;
        };
        auto particle = [](int i) {
            Particle3d q;
            q.position = FP3(0.1 * i, -2.5 + i, 3.0 / (i + 1));
            q.p = FP3(0.01 * (i % 7) - 0.03, 0.5 * std::sin(i), -0.2 + 0.05 * i);
            q.factor = 10.0 + i;
            q.typeIndex = (short)(i % 2);
            return q;
        };
        ParticleArraySoA<Particle3d> arr;
        if (arr.size() != 0) { std::printf("empty array size\n"); fails++; }
        std::vector<Particle3d> pushed;
        for (int i = 0; i < 33; i++) {
            pushed.push_back(particle(i));
            arr.pushBack(pushed.back());
            if (!same(pushed.back(), arr.back())) { std::printf("back after push %d\n", i); fails++; }
        }
        const ParticleArraySoA<Particle3d> copy = arr;
        if (arr.size() != 33 || copy.size() != 33) { std::printf("array size\n"); fails++; }
        for (int i = 0; i < 33; i++) {
            if (!same(pushed[i], arr[i]) || !same(pushed[i], copy[i])) { std::printf("element %d\n", i); fails++; }
            near("element gamma", pushed[i].getGamma(), arr[i].getGamma());
            nearVec("element velocity", pushed[i].getVelocity(), arr[i].getVelocity());
        }
        for (int n = 33; n > 0; n--) {
            arr.popBack();
            if (arr.size() != n - 1 || (n > 1 && !same(pushed[n - 2], arr.back()))) { std::printf("popBack %d\n", n); fails++; }
        }
        ParticleArraySoA<Particle3d> one;
        one.pushBack(copy[5]);   // from a reference
        auto r = one[0];
        r.setMomentum(m2);
        nearVec("reference set / get momentum", m2, r.getMomentum());
        r.setVelocity(v);
        nearVec("reference set / get velocity", v, r.getVelocity());
        r.setPosition(FP3(1, 2, 3));
        r.setFactor(7.5);
        r.setType(1);
        if (!(one[0].getPosition() == FP3(1, 2, 3)) || one[0].getFactor() != 7.5 || one[0].getMass() != constants::protonMass) {
            std::printf("reference setters\n");
            fails++;
        }
    }

    // EnsembleSupercells routing (particles/EnsembleSupercells.h:25-57): the supercell of
    // every supercell centre, for an offset domain with uneven cell sizes
    const FP3 lo(-1.0, 2.0, 0.5), hi(0.6, 2.8, 1.3);
    const Int3 cells(16, 8, 8), per(4, 2, 4);
    EnsembleSupercells<ParticleArraySoA<Particle3d>> ens(lo, hi, cells, per);
    if (!(ens.getNumSupercells() == Int3(4, 4, 2)) || !(ens.getNumCells() == cells) ||
        !(ens.getMinPosition() == lo) || !(ens.getMaxPosition() == hi)) {
        std::printf("ensemble geometry\n");
        fails++;
    }
    const FP3 scSize = FP3(per.x, per.y, per.z) * ((hi - lo) / FP3(cells.x, cells.y, cells.z));
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            for (int k = 0; k < 2; k++) {
                Particle3d q;
                q.position = lo + scSize * FP3(i + 0.5, j + 0.5, k + 0.5);
                if (!(ens.getSupercellIndex(q) == Int3(i, j, k))) {
                    std::printf("supercell of centre %d %d %d\n", i, j, k);
                    fails++;
                }
            }
    Particle3d below;
    below.position = lo - FP3(1e-9, 0, 0);   // floor, not truncation: one supercell down
    if (ens.getSupercellIndex(below).x != -1) {
        std::printf("supercell below the minimum\n");
        fails++;
    }
    ens.add(below);
    ParticleArraySoA<Particle3d> some;
    some.pushBack(below);
    ens.add(some[0]);   // from a reference, as pica's templated add
    try {
        ens.upload();
        std::printf("upload of an ensemble without a Simulation did not throw\n");
        fails++;
    } catch (const Error& e) {
        if (e.status != PICA_ERR_INVALID) {
            std::printf("upload of an ensemble without a Simulation: status %d\n", e.status);
            fails++;
        }
    }

    std::printf(fails ? "failed\n" : "ok\n");
    return fails ? 1 : 0;
}
