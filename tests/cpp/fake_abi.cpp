// A host-only stand-in for the few C ABI entry points that the C++ mirror's
// plumbing calls (context, field and particle upload / download, migration), so that the
// mirror's host code -- field index order, particle conversion, per-supercell
// selection -- is tested without a GPU.  The fake keeps what is uploaded and
// returns it in the ABI's documented ensemble order (species, then linear
// supercell (sx * nsy + sy) * nsz + sz, then upload order); it does no physics.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <vector>

#include "pica_gb300.h"

struct pica_ctx {
    pica_config cfg;
    std::vector<double> f[9];
    std::vector<double> p[7];
    std::vector<int32_t> species;
};

static int64_t nodes(const pica_ctx* c) { return (int64_t)c->cfg.n[0] * c->cfg.n[1] * c->cfg.n[2]; }

static int32_t supercellOf(const pica_ctx* c, int64_t i) {
    int s[3];
    for (int d = 0; d < 3; d++) {
        const int nsc = c->cfg.n[d] / c->cfg.sc[d];
        s[d] = std::min(nsc - 1, std::max(0, (int)std::floor(c->p[d][i] / (c->cfg.sc[d] * c->cfg.h[d]))));
    }
    return (s[0] * (c->cfg.n[1] / c->cfg.sc[1]) + s[1]) * (c->cfg.n[2] / c->cfg.sc[2]) + s[2];
}

extern "C" {

int pica_ctx_create(const pica_config* cfg, pica_ctx** out) {
    if (!cfg || !out) return PICA_ERR_INVALID;
    pica_ctx* c = new pica_ctx();
    c->cfg = *cfg;
    for (auto& a : c->f) a.assign(nodes(c), 0.0);
    *out = c;
    return PICA_OK;
}

int pica_ctx_destroy(pica_ctx* ctx) {
    delete ctx;
    return PICA_OK;
}

const char* pica_status_string(int) { return "fake"; }
const char* pica_last_error(pica_ctx*) { return ""; }

int pica_upload_fields(pica_ctx* ctx, const double* const* f9) {
    for (int c = 0; c < 9; c++) std::copy(f9[c], f9[c] + nodes(ctx), ctx->f[c].begin());
    return PICA_OK;
}

int pica_download_fields(pica_ctx* ctx, double* const* f9) {
    for (int c = 0; c < 9; c++) std::copy(ctx->f[c].begin(), ctx->f[c].end(), f9[c]);
    return PICA_OK;
}

int pica_upload_particles(pica_ctx* ctx, int64_t n, const double* x, const double* y, const double* z,
                          const double* ux, const double* uy, const double* uz, const double* w,
                          const int32_t* species) {
    const double* src[7] = {x, y, z, ux, uy, uz, w};
    for (int k = 0; k < 7; k++) ctx->p[k].insert(ctx->p[k].end(), src[k], src[k] + n);
    for (int64_t i = 0; i < n; i++) ctx->species.push_back(species ? species[i] : 0);
    return PICA_OK;
}

int64_t pica_num_particles(pica_ctx* ctx) { return (int64_t)ctx->species.size(); }

// The fake moves no particles, so a migration has nothing to do.
int pica_migrate(pica_ctx*) { return PICA_OK; }

int pica_download_particles(pica_ctx* ctx, double* x, double* y, double* z, double* ux, double* uy, double* uz,
                            double* w, int32_t* species, int32_t* supercell) {
    const int64_t n = (int64_t)ctx->species.size();
    std::vector<int64_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        if (ctx->species[a] != ctx->species[b]) return ctx->species[a] < ctx->species[b];
        return supercellOf(ctx, a) < supercellOf(ctx, b);
    });
    double* dst[7] = {x, y, z, ux, uy, uz, w};
    for (int64_t j = 0; j < n; j++) {
        const int64_t i = order[j];
        for (int k = 0; k < 7; k++)
            if (dst[k]) dst[k][j] = ctx->p[k][i];
        if (species) species[j] = ctx->species[i];
        if (supercell) supercell[j] = supercellOf(ctx, i);
    }
    return PICA_OK;
}

}  // extern "C"

// Stand-in for the device sort: a host stable sort with pica's comparator.
int pica_order_by_position_host(int64_t n, int32_t dims, const double* x, const double* y, const double* z,
                                int64_t* order) {
    const double* key[3] = {x, y, z};
    for (int64_t i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order, order + n, [&](int64_t a, int64_t b) {
        for (int d = 0; d < dims; d++) {
            if (key[d][a] < key[d][b]) return true;
            if (key[d][a] > key[d][b]) return false;
        }
        return false;
    });
    return PICA_OK;
}
