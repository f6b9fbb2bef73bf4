// Fused two-state pass of the adjoint reverse sweep, complex128 storage with
// double-single (FP32 pair) arithmetic.
#include "pass2_launch.cuh"

// shapes: (tile qubits, register qubits, tile buffers per state, min CTAs per SM)
// (the four-register shape is in adjoint_ds_r4.cu: its unrolled rounds compile as
// long as the rest of this unit)
#define QSV_SHAPES2(X) X(12, 3, 1, 1) X(11, 3, 1, 2)

namespace qsv {

cudaError_t launch_pass2_ds(int T, int R, void* psi, void* lam, const PassDesc* dpass, const StepDesc* dsteps,
                            const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                            int per_tile, double* partial, int* grid_out, cudaStream_t st) {
    using P = PDS;
    QSV_SHAPES2(QSV_LAUNCH2_SHAPE)
    return launch_pass2_ds_r4(T, R, psi, lam, dpass, dsteps, dops, dcoef, n, H, items, cstride, per_tile, partial,
                              grid_out, st);
}

bool pass2_shape_ds(int T, int R) {
    QSV_SHAPES2(QSV_HAS2_SHAPE)
    return pass2_shape_ds_r4(T, R);
}

}  // namespace qsv
