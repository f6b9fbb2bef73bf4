// Launcher of the fused tile pass, shared by the per-precision translation
// units (pass_c128.cu, pass_c64.cu, pass_ds.cu).  Each unit lists its shapes
// as X(T, R, NB, MINB): tile qubits, register qubits, tile buffers, minimum
// resident CTAs per SM for the register budget.
#pragma once
#include "device.cuh"
#include "kernels.h"

namespace qsv {

template <class P, int T, int R, int NB, int MINB>
cudaError_t launch_pass_t(void* state, const PassDesc* dpass, const StepDesc* dsteps, const KOp* dops,
                          const void* dcoef, int n, int H, int items, uint64_t cstride, const uint8_t* active,
                          cudaStream_t st) {
    // NB tile buffers + the chunk-offset table
    const size_t tiles_b = NB * sizeof(typename P::S) * tile_elems(T, sizeof(typename P::S));
    const size_t smem = tiles_b + (sizeof(uint64_t) << H);
    static int grid_cap = 0;  // per instantiation: SMs x resident CTAs per SM
    if (grid_cap == 0) {
        cudaError_t e = cudaFuncSetAttribute(k_pass<P, T, R, NB, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(tiles_b + (8 << 12)));
        if (e != cudaSuccess) return e;
        int dev = 0, nsm = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pass<P, T, R, NB, MINB>, 1 << (T - R), smem);
        if (e != cudaSuccess) return e;
        grid_cap = (nsm > 0 ? nsm : 1) * (per_sm > 0 ? per_sm : 1);
    }
    const uint64_t tiles = static_cast<uint64_t>(items) << (n - T);
    const unsigned grid = static_cast<unsigned>(tiles < static_cast<uint64_t>(grid_cap) ? tiles : grid_cap);
    k_pass<P, T, R, NB, MINB><<<grid, 1 << (T - R), smem, st>>>(static_cast<typename P::G*>(state), tiles, dpass,
                                                                 dsteps, dops,
                                                                 static_cast<const typename P::C*>(dcoef), cstride,
                                                                 n - T, active);
    return cudaGetLastError();
}

}  // namespace qsv

#define QSV_LAUNCH_SHAPE(TT, RR, NBB, MB)                                                                  \
    if (T == TT && R == RR)                                                                                \
        return launch_pass_t<P, TT, RR, NBB, MB>(state, dpass, dsteps, dops, dcoef, n, H, items, cstride, active, \
                                                 st);
#define QSV_HAS_SHAPE(TT, RR, NBB, MB) \
    if (T == TT && R == RR) return true;
