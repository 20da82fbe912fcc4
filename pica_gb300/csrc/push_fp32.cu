// FP32 cell form: push and migration kernels.  Compiled without implicit FMA
// contraction: every fused multiply-add is written out, so that each template
// instantiation (launch variant, batch member) rounds the same way.
#include <algorithm>

#include "push_fast.cuh"

namespace pgb {

namespace {
template <int SHAPE, int DEP>
int launchOne(const PushArgs<CellPtrs>& a, cudaStream_t s) {
    const int TT = a.T[0] * a.T[1] * a.T[2];
    const size_t smem = (size_t)6 * TT * sizeof(float) + (size_t)3 * TT * sizeof(unsigned long long);
    auto k = k_push<false, SHAPE, DEP>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return (int)e;
    const int nscTot = a.nsc[0] * a.nsc[1] * a.nsc[2];
    k<<<nscTot, kPushThreads, smem, s>>>(a);
    return (int)cudaGetLastError();
}
}  // namespace

template <int SHAPE, int SC, int K, int THREADS, int MINB>
int launchEsirkepovV(const PushArgs<CellPtrs>& a, cudaStream_t s) {
    const int TT = a.T[0] * a.T[1] * a.T[2];
    const int ETT = (a.S[0] + 3) * (a.S[1] + 3) * (a.S[2] + 3);
    const size_t smem = (size_t)esirkepovSmemWords(TT, ETT, THREADS / 32) * 4;
    auto k = k_push_cell_esirkepov<SHAPE, K, THREADS, MINB, SC>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return (int)e;
    const int nscTot = a.nsc[0] * a.nsc[1] * a.nsc[2];
    const int n = a.scEnd > a.scBegin ? a.scEnd - a.scBegin : nscTot;
    PushArgsSlim<kMaxSpecies> sl;
    slimArgs(a, sl);
    k<<<n, THREADS, smem, s>>>(sl);
    return (int)cudaGetLastError();
}

// Variant 4: 128 threads, >= 3 CTAs/SM, the E/B tile of interior supercells staged
// by TMA (cubic supercells of edge 4 with tensor maps; variant 0 otherwise).
template <int SHAPE, int K, int THREADS, int MINB>
int launchEsirkepovTma(const PushArgs<CellPtrs>& a, cudaStream_t s) {
    const int TT = a.T[0] * a.T[1] * a.T[2];
    const size_t smem = (size_t)esirkepovSmemWords(TT, (kTmaS + 3) * (kTmaS + 3) * (kTmaS + 3), THREADS / 32) * 4;
    auto k = k_push_cell_esirkepov_tma<SHAPE, K, THREADS, MINB>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return (int)e;
    const int nscTot = a.nsc[0] * a.nsc[1] * a.nsc[2];
    const int n = a.scEnd > a.scBegin ? a.scEnd - a.scBegin : nscTot;
    PushArgsSlim<kMaxSpecies> sl;
    slimArgs(a, sl);
    k<<<n, THREADS, smem, s>>>(sl, *a.tmaps);
    return (int)cudaGetLastError();
}

// Launch variants of the Esirkepov kernel.  All keep K = 8 particles per lane, so the
// particles summed together in registers (and hence every rounding) are the same and
// the variants give bit-identical results; they differ in CTA size and occupancy:
// 0: 128 threads, >= 3 CTAs/SM   1: 128 threads, >= 2 CTAs/SM
// 2: 64 threads, >= 6 CTAs/SM    3: 256 threads, >= 1 CTA/SM
// 4: as 0, E/B tile by TMA.
template <int SHAPE, int SC>
int launchEsirkepovS(const PushArgs<CellPtrs>& a, int variant, cudaStream_t s) {
    if constexpr (SC == kTmaS) {
        if (variant == 4 && a.tmaps) return launchEsirkepovTma<SHAPE, 8, 128, 3>(a, s);
    }
    switch (variant) {
        case 1: return launchEsirkepovV<SHAPE, SC, 8, 128, 2>(a, s);
        case 2: return launchEsirkepovV<SHAPE, SC, 8, 64, 6>(a, s);
        case 3: return launchEsirkepovV<SHAPE, SC, 8, 256, 1>(a, s);
        default: return launchEsirkepovV<SHAPE, SC, 8, 128, 3>(a, s);
    }
}

template <int SHAPE>
int launchEsirkepov(const PushArgs<CellPtrs>& a, int variant, cudaStream_t s) {
    const bool cubic = a.S[0] == a.S[1] && a.S[1] == a.S[2];
    if (cubic && a.S[0] == 4) return launchEsirkepovS<SHAPE, 4>(a, variant, s);
    return launchEsirkepovS<SHAPE, 0>(a, variant, s);
}

template <int SHAPE, int SC, int K, int THREADS, int MINB, int NSP>
int launchBatchV(const BatchPushArgs<NSP>& b, const int* S, cudaStream_t s) {
    const int TT = (S[0] + 2 * kG + 1) * (S[1] + 2 * kG + 1) * (S[2] + 2 * kG + 1);
    const int ETT = (S[0] + 3) * (S[1] + 3) * (S[2] + 3);
    const size_t smem = (size_t)esirkepovSmemWords(TT, ETT, THREADS / 32) * 4;
    auto k = k_push_batch<SHAPE, K, THREADS, MINB, SC, NSP>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return (int)e;
    int dev = 0, sms = 0, per = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return (int)e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return (int)e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, THREADS, smem)) != cudaSuccess) return (int)e;
    const int grid = std::max(1, std::min(b.total, sms * std::max(per, 1)));
    k<<<grid, THREADS, smem, s>>>(b);
    return (int)cudaGetLastError();
}

template <int SHAPE, int SC, int NSP>
int launchBatchS(const BatchPushArgs<NSP>& b, const int* S, int variant, cudaStream_t s) {
    switch (variant) {
        case 1: return launchBatchV<SHAPE, SC, 8, 128, 2>(b, S, s);
        case 2: return launchBatchV<SHAPE, SC, 8, 64, 6>(b, S, s);
        case 3: return launchBatchV<SHAPE, SC, 8, 256, 1>(b, S, s);
        default: return launchBatchV<SHAPE, SC, 8, 128, 3>(b, S, s);
    }
}

template <int NSP>
int launchPushBatch(const BatchPushArgs<NSP>& b, int shape, const int* S, int variant, cudaStream_t s) {
    const bool sc4 = S[0] == 4 && S[1] == 4 && S[2] == 4;
    if (shape == PICA_SHAPE_TSC) return sc4 ? launchBatchS<PICA_SHAPE_TSC, 4>(b, S, variant, s) : launchBatchS<PICA_SHAPE_TSC, 0>(b, S, variant, s);
    if (shape == PICA_SHAPE_CIC) return sc4 ? launchBatchS<PICA_SHAPE_CIC, 4>(b, S, variant, s) : launchBatchS<PICA_SHAPE_CIC, 0>(b, S, variant, s);
    return (int)cudaErrorInvalidValue;
}
template int launchPushBatch<1>(const BatchPushArgs<1>&, int, const int*, int, cudaStream_t);
template int launchPushBatch<2>(const BatchPushArgs<2>&, int, const int*, int, cudaStream_t);

int launchPushCell(const PushArgs<CellPtrs>& a, int shape, int dep, int variant, cudaStream_t s) {
    if (shape == PICA_SHAPE_TSC && dep == PICA_DEPOSIT_ESIRKEPOV) return launchEsirkepov<PICA_SHAPE_TSC>(a, variant, s);
    if (shape == PICA_SHAPE_CIC && dep == PICA_DEPOSIT_ESIRKEPOV) return launchEsirkepov<PICA_SHAPE_CIC>(a, variant, s);
    if (shape == PICA_SHAPE_CIC && dep == PICA_DEPOSIT_DIRECT) return launchOne<PICA_SHAPE_CIC, PICA_DEPOSIT_DIRECT>(a, s);
    if (shape == PICA_SHAPE_CIC && dep == PICA_DEPOSIT_ESIRKEPOV) return launchOne<PICA_SHAPE_CIC, PICA_DEPOSIT_ESIRKEPOV>(a, s);
    if (shape == PICA_SHAPE_TSC && dep == PICA_DEPOSIT_DIRECT) return launchOne<PICA_SHAPE_TSC, PICA_DEPOSIT_DIRECT>(a, s);
    if (shape == PICA_SHAPE_TSC && dep == PICA_DEPOSIT_ESIRKEPOV) return launchOne<PICA_SHAPE_TSC, PICA_DEPOSIT_ESIRKEPOV>(a, s);
    return -1;
}

int launchMigrateCell(const MigrateArgs<CellPtrs>& a, int stage, cudaStream_t s) {
    const int64_t nscTot = (int64_t)a.nsc[0] * a.nsc[1] * a.nsc[2];
    const int warpBlocks = (int)((nscTot * 32 + 255) / 256);
    switch (stage) {
        case kSortLeavers: {
            const size_t smem = (size_t)a.bitmapWords * sizeof(unsigned int);
            if (smem > 48 * 1024) {
                const cudaError_t e = cudaFuncSetAttribute(k_sortLeavers<CellPtrs>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                if (e != cudaSuccess) return (int)e;
            }
            k_sortLeavers<CellPtrs><<<(int)nscTot, 128, smem, s>>>(a);
            break;
        }
        case kCountArrivals: k_migrate<CellPtrs, kCountArrivals><<<warpBlocks, 256, 0, s>>>(a); break;
        case kFill: k_fill<CellPtrs><<<(int)nscTot, kFillWarps * 32, 0, s>>>(a); break;
        case kGatherOutbox: k_migrate<CellPtrs, kGatherOutbox><<<warpBlocks, 256, 0, s>>>(a); break;
        case kRebuild: k_migrate<CellPtrs, kRebuild><<<warpBlocks, 256, 0, s>>>(a); break;
        case kResort: {
            // Staged through shared memory while at least two CTAs fit on an SM (16-bit
            // destinations need supercells below 65535 slots); else the two-pass kernel.
            const int nb = a.S[0] * a.S[1] * a.S[2];
            const size_t smem = stagedResortSmem(a.srcMaxCap, nb);
            if (a.srcMaxCap > 0 && a.srcMaxCap < 65535 && smem <= 110 * 1024) {
                const cudaError_t e = cudaFuncSetAttribute(k_resortStaged<CellPtrs>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                if (e != cudaSuccess) return (int)e;
                k_resortStaged<CellPtrs><<<(int)nscTot, kStagedWarps * 32, smem, s>>>(a);
            } else {
                k_resort<CellPtrs><<<(int)nscTot, kResortWarps * 32, 0, s>>>(a);
            }
            break;
        }
        default: return (int)cudaErrorInvalidValue;
    }
    return (int)cudaGetLastError();
}

}  // namespace pgb
