// Kernels of the domain decomposition of one plasma into slabs along x
// (pica_field_slab, pica_take_supercells, pica_append_to_supercells).
//
// A slab's context holds its own cells plus guard layers on both x faces.  Per
// step the guard fields are filled from the neighbours' cells, the current that
// the slab's particles deposit into its guards is added to the neighbours' cells,
// and the particles that migrated into guard supercells move to the neighbour
// that owns those cells.  Fields are z-fastest arrays, so a run of x-layers is one
// contiguous block; particles move supercell by supercell as packed blocks.
#include <cstdint>

#include "pica_internal.h"

namespace pgb {

namespace {

template <typename R>
__global__ void __launch_bounds__(256) k_addSlab(R* __restrict__ dst, const R* __restrict__ src, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] += src[i];
}

// Scatter of the position component (FP32 form: packed cell; FP64 form: x) of packed
// arrivals into supercells [scBegin, ...): supercell s takes count[s] of them from
// image offset off[s] into slots from start[s], the x cell shifted by dx cells.
__global__ void __launch_bounds__(256) k_appendCells(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst,
                                                     const int64_t* start, const int32_t* count, const int64_t* off,
                                                     int scBegin, int dx, int nx) {
    const int s = scBegin + blockIdx.x;
    const int64_t a = start[s], b = off[s];
    for (int i = threadIdx.x; i < count[s]; i += blockDim.x) {
        const uint32_t c = src[b + i];
        int x, y, z;
        unpackCell(c, x, y, z);
        x += dx;
        x = x < 0 ? x + nx : (x >= nx ? x - nx : x);
        dst[a + i] = packCell(x, y, z);
    }
}

__global__ void __launch_bounds__(256) k_appendX(const double* __restrict__ src, double* __restrict__ dst,
                                                 const int64_t* start, const int32_t* count, const int64_t* off,
                                                 int scBegin, double dx) {
    const int s = scBegin + blockIdx.x;
    const int64_t a = start[s], b = off[s];
    for (int i = threadIdx.x; i < count[s]; i += blockDim.x) dst[a + i] = src[b + i] + dx;
}

}  // namespace

int launchAddSlab(bool fp64, void* dst, const void* src, int64_t n, cudaStream_t s) {
    if (n <= 0) return 0;
    const int blocks = (int)((n + 255) / 256 < 4 * 152 * 8 ? (n + 255) / 256 : 4 * 152 * 8);
    if (fp64) k_addSlab<double><<<blocks, 256, 0, s>>>(static_cast<double*>(dst), static_cast<const double*>(src), n);
    else k_addSlab<float><<<blocks, 256, 0, s>>>(static_cast<float*>(dst), static_cast<const float*>(src), n);
    return (int)cudaGetLastError();
}

int launchAppendPositions(bool fp64, const void* src, void* dst, const int64_t* start, const int32_t* count,
                          const int64_t* off, int scBegin, int scEnd, int dxCells, int nx, double dxLength,
                          cudaStream_t s) {
    if (scEnd <= scBegin) return 0;
    if (fp64)
        k_appendX<<<scEnd - scBegin, 256, 0, s>>>(static_cast<const double*>(src), static_cast<double*>(dst), start,
                                                  count, off, scBegin, dxLength);
    else
        k_appendCells<<<scEnd - scBegin, 256, 0, s>>>(static_cast<const uint32_t*>(src), static_cast<uint32_t*>(dst),
                                                      start, count, off, scBegin, dxCells, nx);
    return (int)cudaGetLastError();
}

}  // namespace pgb
