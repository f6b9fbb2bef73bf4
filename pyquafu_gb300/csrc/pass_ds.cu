// Fused tile-pass kernel, complex128 storage with double-single (FP32 pair)
// arithmetic: 4 float registers per amplitude, as for FP64.
#include "device.cuh"
#include "kernels.h"

namespace qsv {
namespace {

template <class P, int T, int R>
cudaError_t launch_pass_t(void* state, const PassDesc* dpass, const StepDesc* dsteps, const KOp* dops,
                          const void* dcoef, int n, int H, cudaStream_t st) {
    const size_t smem = (sizeof(typename P::S) << T) + (sizeof(uint64_t) << H);
    static bool attr_set = false;  // per instantiation
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_pass<P, T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem + 4096));
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const uint64_t tiles = 1ULL << (n - T);
    k_pass<P, T, R><<<static_cast<unsigned>(tiles), 1 << (T - R), smem, st>>>(
        static_cast<typename P::G*>(state), dpass, dsteps, dops, static_cast<const typename P::C*>(dcoef));
    return cudaGetLastError();
}

}  // namespace

#define QSV_SHAPE(TT, RR) \
    if (T == TT && R == RR) return launch_pass_t<P, TT, RR>(state, dpass, dsteps, dops, dcoef, n, H, st);

cudaError_t launch_pass_ds(int T, int R, void* state, const PassDesc* dpass, const StepDesc* dsteps,
                             const KOp* dops, const void* dcoef, int n, int H, cudaStream_t st) {
    using P = PDS;
    QSV_SHAPE(11, 4)
    QSV_SHAPE(12, 4)
    QSV_SHAPE(12, 5)
    QSV_SHAPE(13, 5)
    return cudaErrorInvalidValue;
}

bool pass_shape_ds(int T, int R) { return (T == 11 && R == 4) || (T == 12 && (R == 4 || R == 5)) || (T == 13 && R == 5); }

}  // namespace qsv
