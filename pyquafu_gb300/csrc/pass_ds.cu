// Fused tile-pass kernel, complex128 storage with double-single (FP32 pair)
// arithmetic: 4 float registers per amplitude, as for FP64.
#include "device.cuh"
#include "kernels.h"

namespace qsv {
namespace {

template <class P, int T, int R>
cudaError_t launch_pass_t(void* state, const PassDesc* dpass, const StepDesc* dsteps, const KOp* dops,
                          const void* dcoef, int n, int H, int items, uint64_t cstride, cudaStream_t st) {
    // two tile buffers + the chunk-offset table
    const size_t smem = 2 * (sizeof(typename P::S) << T) + (sizeof(uint64_t) << H);
    static int grid_cap = 0;  // per instantiation: SMs x resident CTAs per SM
    if (grid_cap == 0) {
        cudaError_t e = cudaFuncSetAttribute(k_pass<P, T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(2 * (sizeof(typename P::S) << T) + (8 << 12)));
        if (e != cudaSuccess) return e;
        int dev = 0, nsm = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pass<P, T, R>, 1 << (T - R), smem);
        if (e != cudaSuccess) return e;
        grid_cap = (nsm > 0 ? nsm : 1) * (per_sm > 0 ? per_sm : 1);
    }
    const uint64_t tiles = static_cast<uint64_t>(items) << (n - T);
    const unsigned grid = static_cast<unsigned>(tiles < static_cast<uint64_t>(grid_cap) ? tiles : grid_cap);
    k_pass<P, T, R><<<grid, 1 << (T - R), smem, st>>>(static_cast<typename P::G*>(state), tiles, dpass, dsteps,
                                                       dops, static_cast<const typename P::C*>(dcoef), cstride, n - T);
    return cudaGetLastError();
}

}  // namespace

#define QSV_SHAPE(TT, RR) \
    if (T == TT && R == RR) return launch_pass_t<P, TT, RR>(state, dpass, dsteps, dops, dcoef, n, H, items, cstride, st);

cudaError_t launch_pass_ds(int T, int R, void* state, const PassDesc* dpass, const StepDesc* dsteps,
                             const KOp* dops, const void* dcoef, int n, int H, int items,
                            uint64_t cstride, cudaStream_t st) {
    using P = PDS;
    QSV_SHAPE(11, 4)
    QSV_SHAPE(12, 4)
    QSV_SHAPE(12, 5)
    return cudaErrorInvalidValue;
}

bool pass_shape_ds(int T, int R) { return (T == 11 && R == 4) || (T == 12 && (R == 4 || R == 5)); }

}  // namespace qsv
