// Launcher of the fused two-state pass (adjoint reverse sweep), shared by the
// per-precision translation units (adjoint_c128.cu, adjoint_c64.cu,
// adjoint_ds.cu).  Each unit lists its shapes as X(T, R, NB, MINB): tile
// qubits, register qubits, tile buffers per state, minimum resident CTAs per
// SM for the register budget.
#pragma once
#include "adjoint.cuh"
#include "kernels.h"

namespace qsv {

template <class P, int T, int R, int NB, int MINB>
cudaError_t launch_pass2_t(void* psi, void* lam, const PassDesc* dpass, const StepDesc* dsteps, const KOp* dops,
                           const void* dcoef, int n, int H, int items, uint64_t cstride, int per_tile,
                           double* partial, int* grid_out, cudaStream_t st) {
    constexpr int NT = 1 << (T - R);
    const size_t tiles_b = 2 * NB * sizeof(typename P::S) * tile_elems(T, sizeof(typename P::S));
    const size_t smem = tiles_b + (sizeof(uint64_t) << H) + sizeof(double) * (NT / 32) * MAX_PASS_PROBES;
    static int grid_cap = 0;  // per instantiation: SMs x resident CTAs per SM
    if (grid_cap == 0) {
        const size_t most = tiles_b + (8 << 12) + sizeof(double) * (NT / 32) * MAX_PASS_PROBES;
        cudaError_t e = cudaFuncSetAttribute(k_pass2<P, T, R, NB, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(most));
        if (e != cudaSuccess) return e;
        int dev = 0, nsm = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pass2<P, T, R, NB, MINB>, NT, smem);
        if (e != cudaSuccess) return e;
        grid_cap = (nsm > 0 ? nsm : 1) * (per_sm > 0 ? per_sm : 1);
        if (grid_cap > pass2_grid_cap()) grid_cap = pass2_grid_cap();  // partial[] is sized for this many CTAs
    }
    const uint64_t tiles = static_cast<uint64_t>(items) << (n - T);
    const unsigned grid = static_cast<unsigned>(tiles < static_cast<uint64_t>(grid_cap) ? tiles : grid_cap);
    *grid_out = static_cast<int>(grid);
    k_pass2<P, T, R, NB, MINB><<<grid, NT, smem, st>>>(
        static_cast<typename P::G*>(psi), static_cast<typename P::G*>(lam), tiles, dpass, dsteps, dops,
        static_cast<const typename P::C*>(dcoef), cstride, n - T, per_tile, partial);
    return cudaGetLastError();
}

}  // namespace qsv

#define QSV_LAUNCH2_SHAPE(TT, RR, NBB, MB)                                                                  \
    if (T == TT && R == RR)                                                                                 \
        return launch_pass2_t<P, TT, RR, NBB, MB>(psi, lam, dpass, dsteps, dops, dcoef, n, H, items, cstride, \
                                                  per_tile, partial, grid_out, st);
#define QSV_HAS2_SHAPE(TT, RR, NBB, MB) \
    if (T == TT && R == RR) return true;
