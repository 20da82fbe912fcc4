// FP64 plain form: push and migration kernels.  Compiled with --fmad=false so
// every double expression rounds as pica's C++ does (no contraction).
#include "push_kernels.cuh"

namespace pgb {

namespace {
template <int SHAPE, int DEP>
int launchOne(const PushArgs<PlainPtrs>& a, cudaStream_t s) {
    const int TT = a.T[0] * a.T[1] * a.T[2];
    const size_t smem = (size_t)6 * TT * sizeof(double);   // the E/B tile
    auto k = k_push<true, SHAPE, DEP>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return (int)e;
    const int nscTot = a.nsc[0] * a.nsc[1] * a.nsc[2];
    k<<<nscTot, kPushThreads, smem, s>>>(a);
    return (int)cudaGetLastError();
}
}  // namespace

int launchPushPlain(const PushArgs<PlainPtrs>& a, int shape, int dep, cudaStream_t s) {
    if (shape == PICA_SHAPE_CIC && dep == PICA_DEPOSIT_DIRECT) return launchOne<PICA_SHAPE_CIC, PICA_DEPOSIT_DIRECT>(a, s);
    if (shape == PICA_SHAPE_CIC && dep == PICA_DEPOSIT_ESIRKEPOV) return launchOne<PICA_SHAPE_CIC, PICA_DEPOSIT_ESIRKEPOV>(a, s);
    if (shape == PICA_SHAPE_TSC && dep == PICA_DEPOSIT_DIRECT) return launchOne<PICA_SHAPE_TSC, PICA_DEPOSIT_DIRECT>(a, s);
    if (shape == PICA_SHAPE_TSC && dep == PICA_DEPOSIT_ESIRKEPOV) return launchOne<PICA_SHAPE_TSC, PICA_DEPOSIT_ESIRKEPOV>(a, s);
    return -1;
}

int launchMigratePlain(const MigrateArgs<PlainPtrs>& a, int stage, cudaStream_t s) {
    const int64_t nscTot = (int64_t)a.nsc[0] * a.nsc[1] * a.nsc[2];
    const int warpBlocks = (int)((nscTot * 32 + 255) / 256);
    switch (stage) {
        case kSortLeavers: {
            const size_t smem = (size_t)a.bitmapWords * sizeof(unsigned int);
            if (smem > 48 * 1024) {
                const cudaError_t e = cudaFuncSetAttribute(k_sortLeavers<PlainPtrs>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                if (e != cudaSuccess) return (int)e;
            }
            k_sortLeavers<PlainPtrs><<<(int)nscTot, 128, smem, s>>>(a);
            break;
        }
        case kCountArrivals: k_migrate<PlainPtrs, kCountArrivals><<<warpBlocks, 256, 0, s>>>(a); break;
        case kFill: k_fill<PlainPtrs><<<(int)nscTot, kFillWarps * 32, 0, s>>>(a); break;
        case kGatherOutbox: k_migrate<PlainPtrs, kGatherOutbox><<<warpBlocks, 256, 0, s>>>(a); break;
        case kRebuild: k_migrate<PlainPtrs, kRebuild><<<warpBlocks, 256, 0, s>>>(a); break;
        case kResort: k_resort<PlainPtrs><<<(int)nscTot, kResortWarps * 32, 0, s>>>(a); break;
        default: return (int)cudaErrorInvalidValue;
    }
    return (int)cudaGetLastError();
}

}  // namespace pgb
