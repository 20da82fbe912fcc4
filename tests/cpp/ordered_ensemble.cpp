// pica's EnsembleOrdered host code on the C++ mirror: particles added to an
// EnsembleOrdered<ParticleArraySoA<Particle3d>> (through pica's Ensemble traits),
// then reorder() -- sorted on the device.  The factor of particle i is i, so the
// printed factors are the permutation.  Positions are drawn on a coarse lattice
// so that many coincide in x or in (x, y) (ties), some are -0.0 and +0.0.
//
// Usage: ordered_ensemble <n> <seed>
#include <cstdio>
#include <cstdlib>

#include "pica_gb300.hpp"

using namespace pica_gb300;

int main(int argc, char** argv) {
    const int n = argc > 1 ? std::atoi(argv[1]) : 1000;
    unsigned long long s = argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1;
    auto draw = [&s]() {   // splitmix64 onto a lattice of 0.25 in [-2, 2)
        s += 0x9E3779B97F4A7C15ull;
        unsigned long long z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return 0.25 * (double)(int)(z % 16) - 2.0;
    };
    typedef ParticleArray<Particle3d, ParticleRepresentation_SoA>::Type PA;
    Ensemble<PA, EnsembleRepresentation_Ordered>::Type e(FP3(-2, -2, -2), FP3(2, 2, 2));
    for (int i = 0; i < n; i++) {
        Particle3d q;
        q.position = FP3(draw(), draw(), draw());
        if (i % 97 == 0) q.position.x = (i % 2) ? -0.0 : 0.0;
        q.factor = (double)i;
        e.add(q);
    }
    try {
        e.reorder();
    } catch (const Error& err) {
        std::printf("error %d: %s\n", err.status, err.what());
        return 1;
    }
    const PA& a = e.getParticles();
    for (int i = 0; i < a.size(); i++) {
        const FP3 r = a[i].getPosition();
        std::printf("%d %.17g %.17g %.17g\n", (int)a[i].getFactor(), r.x, r.y, r.z);
    }
    return 0;
}
