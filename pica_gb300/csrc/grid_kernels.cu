// Yee field update and FP64 diagnostics on the periodic grid.
//
// Built with --fmad=false: the FP64 Yee update must round exactly as pica's
// YeeSolver does (fieldSolver/YeeSolver.h:146-154, 190-195), term for term.
// Every node is updated from its periodic neighbours, which replaces pica's
// guard planes and "edge" loops (YeeSolver.h:156-174, 197-212).
#include <cstdint>

#include "pica_internal.h"

namespace pgb {

namespace {

constexpr double kPiRef = 3.14159265358;  // pica math/Constants.h:10

struct Idx {
    int64_t o, xm, ym, zm, xp, yp, zp;
};

__device__ __forceinline__ Idx neighbours(int64_t idx, int nx, int ny, int nz) {
    const int k = (int)(idx % nz);
    const int j = (int)((idx / nz) % ny);
    const int i = (int)(idx / ((int64_t)nz * ny));
    const int64_t sx = (int64_t)ny * nz, sy = nz;
    Idx r;
    r.o = idx;
    r.xm = idx + (i == 0 ? (int64_t)(nx - 1) * sx : -sx);
    r.xp = idx + (i == nx - 1 ? -(int64_t)(nx - 1) * sx : sx);
    r.ym = idx + (j == 0 ? (int64_t)(ny - 1) * sy : -sy);
    r.yp = idx + (j == ny - 1 ? -(int64_t)(ny - 1) * sy : sy);
    r.zm = idx + (k == 0 ? nz - 1 : -1);
    r.zp = idx + (k == nz - 1 ? -(nz - 1) : 1);
    return r;
}

// B += c dt curl E terms of YeeSolver.h:190-195 (updateB) with periodic neighbours.
template <typename R>
__global__ void __launch_bounds__(256) k_updateB(R* __restrict__ bx, R* __restrict__ by, R* __restrict__ bz,
                                                 const R* __restrict__ ex, const R* __restrict__ ey,
                                                 const R* __restrict__ ez, int nx, int ny, int nz, R cx, R cy, R cz) {
    const int64_t total = (int64_t)nx * ny * nz;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const Idx q = neighbours(idx, nx, ny, nz);
        const int64_t o = q.o;
        bx[o] += cz * (ey[o] - ey[q.zm]) - cy * (ez[o] - ez[q.ym]);
        by[o] += cx * (ez[o] - ez[q.xm]) - cz * (ex[o] - ex[q.zm]);
        bz[o] += cy * (ex[o] - ex[q.ym]) - cx * (ey[o] - ey[q.xm]);
    }
}

// E += -4 pi dt J + c dt curl B, YeeSolver.h:146-154 (updateE) with periodic neighbours.
template <typename R>
__global__ void __launch_bounds__(256) k_updateE(R* __restrict__ ex, R* __restrict__ ey, R* __restrict__ ez,
                                                 const R* __restrict__ bx, const R* __restrict__ by,
                                                 const R* __restrict__ bz, const R* __restrict__ jx,
                                                 const R* __restrict__ jy, const R* __restrict__ jz, int nx, int ny,
                                                 int nz, R cc, R cx, R cy, R cz) {
    const int64_t total = (int64_t)nx * ny * nz;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const Idx q = neighbours(idx, nx, ny, nz);
        const int64_t o = q.o;
        ex[o] += cc * jx[o] + cy * (bz[q.yp] - bz[o]) - cz * (by[q.zp] - by[o]);
        ey[o] += cc * jy[o] + cz * (bx[q.zp] - bx[o]) - cx * (bz[q.xp] - bz[o]);
        ez[o] += cc * jz[o] + cx * (by[q.xp] - by[o]) - cy * (bx[q.yp] - bx[o]);
    }
}

// FP32 forms of the two stencils with float4 accesses along z (nz a multiple of 4):
// one thread updates four consecutive cells of a row.  The x and y neighbours are
// whole float4 rows of the neighbouring planes; the z neighbour of the first (B) or
// last (E) cell comes from one more scalar load, wrapped within the row.  Each
// element is the scalar kernel's expression, so results are the same.
struct Row4 {
    int64_t o, xm, ym, xp, yp, zm1, zp4;   // row starts of the neighbours; the z neighbours' scalars
};
__device__ __forceinline__ Row4 row4(int64_t g, int nx, int ny, int nz) {
    const int nz4 = nz >> 2;
    const int k0 = (int)(g % nz4) * 4;
    const int j = (int)((g / nz4) % ny);
    const int i = (int)(g / ((int64_t)nz4 * ny));
    const int64_t sx = (int64_t)ny * nz, sy = nz;
    Row4 r;
    r.o = ((int64_t)i * ny + j) * nz + k0;
    r.xm = r.o + (i == 0 ? (int64_t)(nx - 1) * sx : -sx);
    r.xp = r.o + (i == nx - 1 ? -(int64_t)(nx - 1) * sx : sx);
    r.ym = r.o + (j == 0 ? (int64_t)(ny - 1) * sy : -sy);
    r.yp = r.o + (j == ny - 1 ? -(int64_t)(ny - 1) * sy : sy);
    r.zm1 = k0 == 0 ? r.o + nz - 1 : r.o - 1;
    r.zp4 = k0 + 4 == nz ? r.o - (nz - 4) : r.o + 4;
    return r;
}
__device__ __forceinline__ float4 ld4(const float* p, int64_t i) { return *reinterpret_cast<const float4*>(p + i); }
__device__ __forceinline__ float el(const float4& v, int e) { return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w; }
__device__ __forceinline__ void setEl(float4& v, int e, float x) {
    if (e == 0) v.x = x; else if (e == 1) v.y = x; else if (e == 2) v.z = x; else v.w = x;
}

__global__ void __launch_bounds__(256) k_updateB4(float* __restrict__ bx, float* __restrict__ by, float* __restrict__ bz,
                                                  const float* __restrict__ ex, const float* __restrict__ ey,
                                                  const float* __restrict__ ez, int nx, int ny, int nz, float cx,
                                                  float cy, float cz) {
    const int64_t total = (int64_t)nx * ny * (nz >> 2);
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        const Row4 r = row4(g, nx, ny, nz);
        const float4 exo = ld4(ex, r.o), eyo = ld4(ey, r.o), ezo = ld4(ez, r.o);
        const float4 exym = ld4(ex, r.ym), eyxm = ld4(ey, r.xm), ezxm = ld4(ez, r.xm), ezym = ld4(ez, r.ym);
        const float exzm0 = ex[r.zm1], eyzm0 = ey[r.zm1];
        float4 b0 = ld4(bx, r.o), b1 = ld4(by, r.o), b2 = ld4(bz, r.o);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const float eyzm = e == 0 ? eyzm0 : el(eyo, e - 1), exzm = e == 0 ? exzm0 : el(exo, e - 1);
            setEl(b0, e, el(b0, e) + (cz * (el(eyo, e) - eyzm) - cy * (el(ezo, e) - el(ezym, e))));
            setEl(b1, e, el(b1, e) + (cx * (el(ezo, e) - el(ezxm, e)) - cz * (el(exo, e) - exzm)));
            setEl(b2, e, el(b2, e) + (cy * (el(exo, e) - el(exym, e)) - cx * (el(eyo, e) - el(eyxm, e))));
        }
        *reinterpret_cast<float4*>(bx + r.o) = b0;
        *reinterpret_cast<float4*>(by + r.o) = b1;
        *reinterpret_cast<float4*>(bz + r.o) = b2;
    }
}

__global__ void __launch_bounds__(256) k_updateE4(float* __restrict__ ex, float* __restrict__ ey, float* __restrict__ ez,
                                                  const float* __restrict__ bx, const float* __restrict__ by,
                                                  const float* __restrict__ bz, const float* __restrict__ jx,
                                                  const float* __restrict__ jy, const float* __restrict__ jz, int nx,
                                                  int ny, int nz, float cc, float cx, float cy, float cz) {
    const int64_t total = (int64_t)nx * ny * (nz >> 2);
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        const Row4 r = row4(g, nx, ny, nz);
        const float4 bxo = ld4(bx, r.o), byo = ld4(by, r.o), bzo = ld4(bz, r.o);
        const float4 bzyp = ld4(bz, r.yp), bzxp = ld4(bz, r.xp), byxp = ld4(by, r.xp), bxyp = ld4(bx, r.yp);
        const float byzp3 = by[r.zp4], bxzp3 = bx[r.zp4];
        const float4 j0 = ld4(jx, r.o), j1 = ld4(jy, r.o), j2 = ld4(jz, r.o);
        float4 e0 = ld4(ex, r.o), e1 = ld4(ey, r.o), e2 = ld4(ez, r.o);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const float byzp = e == 3 ? byzp3 : el(byo, e + 1), bxzp = e == 3 ? bxzp3 : el(bxo, e + 1);
            setEl(e0, e, el(e0, e) + (cc * el(j0, e) + cy * (el(bzyp, e) - el(bzo, e)) - cz * (byzp - el(byo, e))));
            setEl(e1, e, el(e1, e) + (cc * el(j1, e) + cz * (bxzp - el(bxo, e)) - cx * (el(bzxp, e) - el(bzo, e))));
            setEl(e2, e, el(e2, e) + (cc * el(j2, e) + cx * (el(byxp, e) - el(byo, e)) - cy * (el(bxyp, e) - el(bxo, e))));
        }
        *reinterpret_cast<float4*>(ex + r.o) = e0;
        *reinterpret_cast<float4*>(ey + r.o) = e1;
        *reinterpret_cast<float4*>(ez + r.o) = e2;
    }
}

// J = Jacc * scale (one rounding from the exact integer sum), and clear Jacc for the next deposit.
template <typename R>
__global__ void __launch_bounds__(256) k_convertJ(R* __restrict__ jx, R* __restrict__ jy, R* __restrict__ jz,
                                                  unsigned long long* __restrict__ ax, unsigned long long* __restrict__ ay,
                                                  unsigned long long* __restrict__ az, int64_t n, double scale) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        jx[i] = (R)((double)(long long)ax[i] * scale);
        jy[i] = (R)((double)(long long)ay[i] * scale);
        jz[i] = (R)((double)(long long)az[i] * scale);
        ax[i] = 0ull; ay[i] = 0ull; az[i] = 0ull;
    }
}

// Fixed-order block reduction (sum or max) of one double per thread.
template <bool MAX>
__device__ __forceinline__ double blockReduce(double v, double* sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] = MAX ? fmax(sh[threadIdx.x], sh[threadIdx.x + w]) : sh[threadIdx.x] + sh[threadIdx.x + w];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

template <typename R>
__global__ void __launch_bounds__(256) k_sumsq(const R* f0, const R* f1, const R* f2, const R* f3, const R* f4,
                                               const R* f5, int64_t n, double* partial) {
    __shared__ double sh[256];
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double a0 = f0[i], a1 = f1[i], a2 = f2[i], a3 = f3[i], a4 = f4[i], a5 = f5[i];
        acc += a0 * a0 + a1 * a1 + a2 * a2 + a3 * a3 + a4 * a4 + a5 * a5;
    }
    const double r = blockReduce<false>(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

// Single-block final reduction over `np` partials in a fixed order.
template <bool MAX>
__global__ void __launch_bounds__(256) k_final(const double* partial, int np, int stride, int nvals, double* out) {
    __shared__ double sh[256];
    for (int v = 0; v < nvals; v++) {
        double acc = 0.0;
        for (int i = threadIdx.x; i < np; i += blockDim.x) {
            const double x = partial[(int64_t)v * stride + i];
            acc = MAX ? fmax(acc, x) : acc + x;
        }
        const double r = blockReduce<MAX>(acc, sh);
        if (threadIdx.x == 0) out[v] = r;
    }
}

template <typename T>
__device__ __forceinline__ double asDouble(const void* p, int64_t i) {
    return (double)static_cast<const T*>(p)[i];
}

// Per-supercell kinetic energy and charge (FP64), one block per supercell.
__global__ void __launch_bounds__(256) k_particleSums(const ParticleSumArgs a, double* partial) {
    __shared__ double sh[256];
    const int s = blockIdx.x;
    double ek = 0.0, q = 0.0;
    for (int sp = 0; sp < a.nspecies; sp++) {
        const int64_t start = a.start[sp][s];
        const int cnt = a.count[sp][s];
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
            const int64_t o = start + i;
            if (a.fp64 ? !aliveX(static_cast<const double*>(a.key[sp])[o])
                       : static_cast<const uint32_t*>(a.key[sp])[o] == kDeadCell)
                continue;
            double ux, uy, uz, w;
            if (a.fp64) { ux = asDouble<double>(a.ux[sp], o); uy = asDouble<double>(a.uy[sp], o); uz = asDouble<double>(a.uz[sp], o); w = asDouble<double>(a.w[sp], o); }
            else { ux = asDouble<float>(a.ux[sp], o); uy = asDouble<float>(a.uy[sp], o); uz = asDouble<float>(a.uz[sp], o); w = asDouble<float>(a.w[sp], o); }
            const double u2 = ux * ux + uy * uy + uz * uz;
            ek += w * a.mc2[sp] * (u2 / (1.0 + sqrt(1.0 + u2)));
            q += a.q[sp] * w;
        }
    }
    const double r0 = blockReduce<false>(ek, sh);
    const double r1 = blockReduce<false>(q, sh);
    if (threadIdx.x == 0) { partial[s] = r0; partial[a.nscTot + s] = r1; }
}

__device__ __forceinline__ void tsc3(double d, double* w) {
    w[0] = 0.5 * (0.5 - d) * (0.5 - d);
    w[1] = 0.75 - d * d;
    w[2] = 0.5 * (0.5 + d) * (0.5 + d);
}

// Charge density at cell centres (the rho lattice, node m at (m+1/2) h), FP64 atomics.
__global__ void __launch_bounds__(256) k_rho(const RhoArgs a, double* rho) {
    const int s = blockIdx.x;
    const int np = a.shape == PICA_SHAPE_CIC ? 2 : 3;
    for (int sp = 0; sp < a.nspecies; sp++) {
        const int64_t start = a.start[sp][s];
        const int cnt = a.count[sp][s];
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
            const int64_t o = start + i;
            if (a.fp64 ? !aliveX(static_cast<const double*>(a.p0[sp])[o])
                       : static_cast<const uint32_t*>(a.p0[sp])[o] == kDeadCell)
                continue;
            int lo[3];
            double w[3][3];
            double wt;
            if (a.fp64) {
                const double pos[3] = {asDouble<double>(a.p0[sp], o), asDouble<double>(a.p1[sp], o), asDouble<double>(a.p2[sp], o)};
                wt = asDouble<double>(a.w[sp], o);
                for (int d = 0; d < 3; d++) {
                    const double xi = pos[d] * a.invh[d] - 0.5;
                    if (np == 2) { const int n = (int)floor(xi); w[d][0] = 1.0 - (xi - n); w[d][1] = xi - n; lo[d] = n; }
                    else { const int n = (int)floor(xi + 0.5); tsc3(xi - n, w[d]); lo[d] = n - 1; }
                }
            } else {
                int c3[3];
                unpackCell(static_cast<const uint32_t*>(a.p0[sp])[o], c3[0], c3[1], c3[2]);
                const double off[3] = {asDouble<float>(a.p1[sp], o), asDouble<float>(a.p2[sp], o), asDouble<float>(a.p3[sp], o)};
                wt = asDouble<float>(a.w[sp], o);
                for (int d = 0; d < 3; d++) {
                    if (np == 2) {
                        const bool hi = off[d] >= 0.5;
                        const double dd = hi ? off[d] - 0.5 : off[d] + 0.5;
                        lo[d] = hi ? c3[d] : c3[d] - 1; w[d][0] = 1.0 - dd; w[d][1] = dd;
                    } else { tsc3(off[d] - 0.5, w[d]); lo[d] = c3[d] - 1; }
                }
            }
            const double v = a.q[sp] * wt * a.norm;
            for (int ii = 0; ii < np; ii++)
                for (int jj = 0; jj < np; jj++)
                    for (int kk = 0; kk < np; kk++) {
                        int gx = (lo[0] + ii) % a.n[0]; if (gx < 0) gx += a.n[0];
                        int gy = (lo[1] + jj) % a.n[1]; if (gy < 0) gy += a.n[1];
                        int gz = (lo[2] + kk) % a.n[2]; if (gz < 0) gz += a.n[2];
                        atomicAdd(rho + ((int64_t)gx * a.n[1] + gy) * a.n[2] + gz, v * w[0][ii] * w[1][jj] * w[2][kk]);
                    }
        }
    }
}

// max |div E - 4 pi (rho + bg)| and max |rho|; div E at the cell centre from the
// face-centred E of pica's lattice (Ex at (i, j+1/2, k+1/2) is the x face of cell (i,j,k)).
template <typename R>
__global__ void __launch_bounds__(256) k_gauss(const R* ex, const R* ey, const R* ez, const double* rho, int nx,
                                               int ny, int nz, double hx, double hy, double hz, double bg,
                                               double* partial) {
    __shared__ double sh[256];
    const int64_t total = (int64_t)nx * ny * nz;
    double g = 0.0, r = 0.0;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const Idx q = neighbours(idx, nx, ny, nz);
        const double div = ((double)ex[q.xp] - (double)ex[idx]) / hx + ((double)ey[q.yp] - (double)ey[idx]) / hy +
                           ((double)ez[q.zp] - (double)ez[idx]) / hz;
        const double rv = rho[idx];
        g = fmax(g, fabs(div - 4.0 * kPiRef * (rv + bg)));
        r = fmax(r, fabs(rv));
    }
    const double g0 = blockReduce<true>(g, sh);
    const double r0 = blockReduce<true>(r, sh);
    if (threadIdx.x == 0) { partial[blockIdx.x] = g0; partial[kReduceBlocks + blockIdx.x] = r0; }
}

inline int gridFor(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (int)(b < 152 * 16 ? b : 152 * 16);
}

}  // namespace

int launchConvertJ(bool fp64, void* const* j, unsigned long long* const* a, int64_t nodes, double scale,
                   cudaStream_t s) {
    if (fp64)
        k_convertJ<double><<<gridFor(nodes), 256, 0, s>>>((double*)j[0], (double*)j[1], (double*)j[2], a[0], a[1], a[2],
                                                          nodes, scale);
    else
        k_convertJ<float><<<gridFor(nodes), 256, 0, s>>>((float*)j[0], (float*)j[1], (float*)j[2], a[0], a[1], a[2],
                                                         nodes, scale);
    return (int)cudaGetLastError();
}

int launchUpdateB(bool fp64, void* const* f, const int* n, const double* c, cudaStream_t s) {
    const int64_t total = (int64_t)n[0] * n[1] * n[2];
    if (fp64)
        k_updateB<double><<<gridFor(total), 256, 0, s>>>((double*)f[3], (double*)f[4], (double*)f[5], (const double*)f[0],
                                                         (const double*)f[1], (const double*)f[2], n[0], n[1], n[2], c[0], c[1], c[2]);
    else if (n[2] % 4 == 0)
        k_updateB4<<<gridFor(total / 4), 256, 0, s>>>((float*)f[3], (float*)f[4], (float*)f[5], (const float*)f[0],
                                                       (const float*)f[1], (const float*)f[2], n[0], n[1], n[2],
                                                       (float)c[0], (float)c[1], (float)c[2]);
    else
        k_updateB<float><<<gridFor(total), 256, 0, s>>>((float*)f[3], (float*)f[4], (float*)f[5], (const float*)f[0],
                                                        (const float*)f[1], (const float*)f[2], n[0], n[1], n[2], (float)c[0],
                                                        (float)c[1], (float)c[2]);
    return (int)cudaGetLastError();
}

int launchUpdateE(bool fp64, void* const* f, const int* n, double cc, const double* c, cudaStream_t s) {
    const int64_t total = (int64_t)n[0] * n[1] * n[2];
    if (fp64)
        k_updateE<double><<<gridFor(total), 256, 0, s>>>((double*)f[0], (double*)f[1], (double*)f[2], (const double*)f[3],
                                                         (const double*)f[4], (const double*)f[5], (const double*)f[6],
                                                         (const double*)f[7], (const double*)f[8], n[0], n[1], n[2], cc,
                                                         c[0], c[1], c[2]);
    else if (n[2] % 4 == 0)
        k_updateE4<<<gridFor(total / 4), 256, 0, s>>>((float*)f[0], (float*)f[1], (float*)f[2], (const float*)f[3],
                                                       (const float*)f[4], (const float*)f[5], (const float*)f[6],
                                                       (const float*)f[7], (const float*)f[8], n[0], n[1], n[2],
                                                       (float)cc, (float)c[0], (float)c[1], (float)c[2]);
    else
        k_updateE<float><<<gridFor(total), 256, 0, s>>>((float*)f[0], (float*)f[1], (float*)f[2], (const float*)f[3],
                                                        (const float*)f[4], (const float*)f[5], (const float*)f[6],
                                                        (const float*)f[7], (const float*)f[8], n[0], n[1], n[2], (float)cc,
                                                        (float)c[0], (float)c[1], (float)c[2]);
    return (int)cudaGetLastError();
}

int launchFieldEnergy(bool fp64, void* const* f, int64_t nodes, double* partial, double* out, cudaStream_t s) {
    if (fp64)
        k_sumsq<double><<<kReduceBlocks, 256, 0, s>>>((const double*)f[0], (const double*)f[1], (const double*)f[2],
                                                      (const double*)f[3], (const double*)f[4], (const double*)f[5], nodes, partial);
    else
        k_sumsq<float><<<kReduceBlocks, 256, 0, s>>>((const float*)f[0], (const float*)f[1], (const float*)f[2],
                                                     (const float*)f[3], (const float*)f[4], (const float*)f[5], nodes, partial);
    k_final<false><<<1, 256, 0, s>>>(partial, kReduceBlocks, 0, 1, out);
    return (int)cudaGetLastError();
}

int launchParticleSums(const ParticleSumArgs& a, double* partial, double* out2, cudaStream_t s) {
    k_particleSums<<<a.nscTot, 256, 0, s>>>(a, partial);
    k_final<false><<<1, 256, 0, s>>>(partial, a.nscTot, a.nscTot, 2, out2);
    return (int)cudaGetLastError();
}

int launchRho(const RhoArgs& a, double* rho, cudaStream_t s) {
    k_rho<<<a.nscTot, 256, 0, s>>>(a, rho);
    return (int)cudaGetLastError();
}

int launchGauss(bool fp64, void* const* f, const double* rho, const int* n, const double* h, double bg,
                double* partial, double* out2, cudaStream_t s) {
    if (fp64)
        k_gauss<double><<<kReduceBlocks, 256, 0, s>>>((const double*)f[0], (const double*)f[1], (const double*)f[2], rho,
                                                      n[0], n[1], n[2], h[0], h[1], h[2], bg, partial);
    else
        k_gauss<float><<<kReduceBlocks, 256, 0, s>>>((const float*)f[0], (const float*)f[1], (const float*)f[2], rho,
                                                     n[0], n[1], n[2], h[0], h[1], h[2], bg, partial);
    k_final<true><<<1, 256, 0, s>>>(partial, kReduceBlocks, kReduceBlocks, 2, out2);
    return (int)cudaGetLastError();
}

namespace {
__global__ void __launch_bounds__(256) k_packCopy(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst,
                                                  const int64_t* start, const int32_t* count, const int64_t* off,
                                                  int scBegin, int words, bool gather) {
    const int s = scBegin + blockIdx.x;
    const int64_t a = start[s] * words, b = off[s] * words;
    const int n = count[s] * words;
    if (gather) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) dst[b + i] = src[a + i];
    } else {
        for (int i = threadIdx.x; i < n; i += blockDim.x) dst[a + i] = src[b + i];
    }
}
}  // namespace

int launchPackCopy(const void* src, void* dst, const int64_t* start, const int32_t* count, const int64_t* off,
                   int scBegin, int scEnd, int words, bool gather, cudaStream_t s) {
    if (scEnd <= scBegin) return 0;
    k_packCopy<<<scEnd - scBegin, 256, 0, s>>>(static_cast<const uint32_t*>(src), static_cast<uint32_t*>(dst), start,
                                               count, off, scBegin, words, gather);
    return (int)cudaGetLastError();
}

}  // namespace pgb
