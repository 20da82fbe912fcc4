// Field energy without a context and without allocation.
//
// pica_field_energy reduces through scratch that its context allocated at
// creation.  This entry point does the same reduction on six caller-owned device
// arrays with its scratch in one fixed static device array, so that callers that
// must not allocate (a diagnostics hook beside a live step: cudaMalloc/cudaFree
// synchronise the device; an application whose memory pool has reserved the
// device; a component that owns its fields but has no pica context) can still
// take the field energy.
//
// Reduction: block b sums the squares of nodes [b*kChunk, (b+1)*kChunk) (fixed
// thread stride, fixed tree), a single block then sums the block partials in a
// fixed order.  The order depends only on the node count, so repeated calls
// return the same bits.  Every partial slot that the final pass reads is written
// by the same call, so nothing has to start at zero.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "pica_gb300.h"

namespace {

constexpr int kThreads = 256;
constexpr int64_t kChunk = 8192;                       // nodes per block
constexpr int kMaxBlocks = 16384;                      // partial slots in the scratch
constexpr int64_t kMaxNodes = kChunk * kMaxBlocks;     // 134,217,728 = 512^3
constexpr int kOutSlot = kMaxBlocks;                   // result slot, after the partials
constexpr int kMaxDevices = 64;
constexpr double kPiRef = 3.14159265358;               // pica math/Constants.h:10

// 128 KB of partials plus the result, on its own 256-byte line.
static __device__ __align__(256) double g_scratch[kMaxBlocks + 32];

std::mutex g_mutex;
double* g_scratchAddr[kMaxDevices] = {};

__device__ __forceinline__ double blockSum(double v, double* sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    return sh[0];
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_chunkSumsq(const R* f0, const R* f1, const R* f2, const R* f3,
                                                        const R* f4, const R* f5, int64_t n, double* partial) {
    __shared__ double sh[kThreads];
    const int64_t lo = (int64_t)blockIdx.x * kChunk;
    const int64_t hi = lo + kChunk < n ? lo + kChunk : n;
    double acc = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += kThreads) {
        const double a0 = f0[i], a1 = f1[i], a2 = f2[i], a3 = f3[i], a4 = f4[i], a5 = f5[i];
        acc += a0 * a0 + a1 * a1 + a2 * a2 + a3 * a3 + a4 * a4 + a5 * a5;
    }
    const double r = blockSum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

__global__ void __launch_bounds__(kThreads) k_chunkFinal(const double* partial, int nb, double* out) {
    __shared__ double sh[kThreads];
    double acc = 0.0;
    for (int i = threadIdx.x; i < nb; i += kThreads) acc += partial[i];
    const double r = blockSum(acc, sh);
    if (threadIdx.x == 0) *out = r;
}

// Address of g_scratch on the current device, looked up once per device.
int scratchAddress(double** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return PICA_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return PICA_ERR_LIMIT;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratchAddr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return PICA_ERR_CUDA;
        g_scratchAddr[dev] = static_cast<double*>(p);
    }
    *out = g_scratchAddr[dev];
    return PICA_OK;
}

}  // namespace

extern "C" int pica_field_energy_noalloc(const void* const* fields, int32_t fp64, const int32_t* n, const double* h,
                                         void* stream, double* out) {
    if (!fields || !n || !h || !out || (fp64 != 0 && fp64 != 1)) return PICA_ERR_INVALID;
    const uintptr_t align = fp64 ? 8 : 4;
    for (int c = 0; c < 6; c++)
        if (!fields[c] || reinterpret_cast<uintptr_t>(fields[c]) % align) return PICA_ERR_INVALID;
    int64_t nodes = 1;
    for (int d = 0; d < 3; d++) {
        if (n[d] < 1 || !(h[d] > 0.0)) return PICA_ERR_INVALID;
        nodes *= n[d];
        if (nodes > kMaxNodes) return PICA_ERR_LIMIT;  // grids above 512^3 nodes: use pica_field_energy
    }
    double* scratch = nullptr;
    int rc = scratchAddress(&scratch);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nb = (int)((nodes + kChunk - 1) / kChunk);
    if (fp64)
        k_chunkSumsq<double><<<nb, kThreads, 0, s>>>(
            static_cast<const double*>(fields[0]), static_cast<const double*>(fields[1]),
            static_cast<const double*>(fields[2]), static_cast<const double*>(fields[3]),
            static_cast<const double*>(fields[4]), static_cast<const double*>(fields[5]), nodes, scratch);
    else
        k_chunkSumsq<float><<<nb, kThreads, 0, s>>>(
            static_cast<const float*>(fields[0]), static_cast<const float*>(fields[1]),
            static_cast<const float*>(fields[2]), static_cast<const float*>(fields[3]),
            static_cast<const float*>(fields[4]), static_cast<const float*>(fields[5]), nodes, scratch);
    k_chunkFinal<<<1, kThreads, 0, s>>>(scratch, nb, scratch + kOutSlot);
    if (cudaGetLastError() != cudaSuccess) return PICA_ERR_CUDA;
    double sum = 0.0;
    if (cudaMemcpyAsync(&sum, scratch + kOutSlot, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return PICA_ERR_CUDA;
    *out = sum * (h[0] * h[1] * h[2]) / (8.0 * kPiRef);
    return PICA_OK;
}
