// Synthetic plasma generated on the device, straight into the FP32 cell form's
// supercell layout (pica_generate_plasma).
//
// The particles are those of the host generator (pica_plasma_generate) for the
// same populations: particle p of cell (i, j, k) takes the same counter-based
// draws, so no host memory holds the ensemble (2e9 particles would need about
// 130 GB there).  The in-cell offset is the uniform draw itself, rounded to
// FP32 (the host path rounds x / h - i, computed in FP64 from x = (i + draw) h),
// and the momenta use the device's log and cos; both agree with the host path
// to the last FP32 bit except in rare roundings.
//
// Layout: supercell s owns slots [start[s], ...); inside it the particles are
// ordered by local cell (x slowest, z fastest), then population in the
// caller's order, then particle index p -- the order pica_upload_particles
// gives the host generator's output.  The number of particles of every cell is
// known from the per-plane table, so each CTA writes its supercell with no
// counting pass.
//
// Built with --fmad=false: the drift is added to sigma times the normal draw
// in two roundings, as the host generator does.
#include <cstdint>

#include "pica_internal.h"

namespace pgb {

namespace {

constexpr int kGenThreads = 128;

__global__ void __launch_bounds__(kGenThreads) k_generate(const __grid_constant__ GenArgs a) {
    const int s = blockIdx.x;
    const int sz = s % a.nsc[2], sy = (s / a.nsc[2]) % a.nsc[1], sx = s / (a.nsc[1] * a.nsc[2]);
    const int m0 = sx * a.S[0], m1 = sy * a.S[1], m2 = sz * a.S[2];
    int64_t slot = a.start[s];
    for (int lx = 0; lx < a.S[0]; lx++) {
        const int i = m0 + lx;
        int tot = 0;
        for (int k = 0; k < a.nspecs; k++) tot += a.per[k * a.n[0] + i];
        for (int ly = 0; ly < a.S[1]; ly++)
            for (int lz = 0; lz < a.S[2]; lz++) {
                const int j = m1 + ly, kk = m2 + lz;
                const int64_t cell = ((int64_t)i * a.n[1] + j) * a.n[2] + kk;
                const uint32_t pc = packCell(i, j, kk);
                for (int t = threadIdx.x; t < tot; t += kGenThreads) {
                    // Population of the t-th particle of the cell (t < tot keeps q < nspecs).
                    int q = 0, p = t;
                    while (p >= a.per[q * a.n[0] + i]) { p -= a.per[q * a.n[0] + i]; q++; }
                    const GenSpec& g = a.sp[q];
                    float o3[3];
                    for (int d = 0; d < 3; d++) {
                        const float v = (float)uniDraw(g.seed, cell, p, d);
                        o3[d] = v < 1.0f ? v : 0x1.fffffep-1f;   // the largest offset below one
                    }
                    double u3[3] = {g.sigma * normalDraw(g.seed, cell, p, 3), g.sigma * normalDraw(g.seed, cell, p, 5),
                                    g.sigma * normalDraw(g.seed, cell, p, 7)};
                    if (g.nbeams == 2) u3[g.axis] += (p % 2 == 0) ? g.drift : -g.drift;
                    else u3[g.axis] += g.drift;
                    const int64_t o = slot + t;
                    a.buf.cell[o] = pc;
                    a.buf.ox[o] = o3[0];
                    a.buf.oy[o] = o3[1];
                    a.buf.oz[o] = o3[2];
                    a.buf.ux[o] = (float)u3[0];
                    a.buf.uy[o] = (float)u3[1];
                    a.buf.uz[o] = (float)u3[2];
                    a.buf.w[o] = (float)g.weight;
                }
                slot += tot;
            }
    }
}

}  // namespace

int launchGenerate(const GenArgs& a, int nscTot, cudaStream_t s) {
    if (nscTot <= 0) return 0;
    k_generate<<<nscTot, kGenThreads, 0, s>>>(a);
    return (int)cudaGetLastError();
}

}  // namespace pgb
