// FP32 cell form: push and migration kernels (FMA contraction allowed).
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

template <int SHAPE, int SC>
int launchEsirkepovS(const PushArgs<CellPtrs>& a, cudaStream_t s) {
    const int TT = a.T[0] * a.T[1] * a.T[2];
    constexpr int K = 8, THREADS = 128, MINB = 3;
    const size_t smem = (size_t)6 * TT * sizeof(float) + (size_t)3 * TT * 2 * sizeof(uint32_t);
    auto k = k_push_cell_esirkepov<SHAPE, K, THREADS, MINB, SC>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return (int)e;
    const int nscTot = a.nsc[0] * a.nsc[1] * a.nsc[2];
    k<<<nscTot, THREADS, smem, s>>>(a);
    return (int)cudaGetLastError();
}

template <int SHAPE>
int launchEsirkepov(const PushArgs<CellPtrs>& a, cudaStream_t s) {
    const bool cubic = a.S[0] == a.S[1] && a.S[1] == a.S[2];
    if (cubic && a.S[0] == 4) return launchEsirkepovS<SHAPE, 4>(a, s);
    if (cubic && a.S[0] == 2) return launchEsirkepovS<SHAPE, 2>(a, s);
    return launchEsirkepovS<SHAPE, 0>(a, s);
}

int launchPushCell(const PushArgs<CellPtrs>& a, int shape, int dep, cudaStream_t s) {
    if (shape == PICA_SHAPE_TSC && dep == PICA_DEPOSIT_ESIRKEPOV) return launchEsirkepov<PICA_SHAPE_TSC>(a, s);
    if (shape == PICA_SHAPE_CIC && dep == PICA_DEPOSIT_ESIRKEPOV) return launchEsirkepov<PICA_SHAPE_CIC>(a, s);
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
        case kFill: k_migrate<CellPtrs, kFill><<<warpBlocks, 256, 0, s>>>(a); break;
        case kGatherOutbox: k_migrate<CellPtrs, kGatherOutbox><<<warpBlocks, 256, 0, s>>>(a); break;
        case kRebuild: k_migrate<CellPtrs, kRebuild><<<warpBlocks, 256, 0, s>>>(a); break;
        case kResort: k_resort<CellPtrs><<<(int)((nscTot + 3) / 4), 128, 0, s>>>(a); break;
        default: return (int)cudaErrorInvalidValue;
    }
    return (int)cudaGetLastError();
}

}  // namespace pgb
