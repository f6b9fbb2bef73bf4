// Fused tile-pass kernel, complex128 storage with double-single (FP32 pair)
// arithmetic: 4 float registers per amplitude, as for FP64.
#include "pass_launch.cuh"

// shapes: (tile qubits, register qubits, tile buffers, min CTAs per SM)
// (the five-register shape is in pass_ds_r5.cu: its unrolled rounds compile as long
// as the rest of this unit)
#define QSV_SHAPES(X) X(11, 4, 2, 1) X(12, 4, 2, 1) X(12, 3, 1, 1)

namespace qsv {

cudaError_t launch_pass_ds(int T, int R, void* state, const PassDesc* dpass, const StepDesc* dsteps,
                            const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                            const uint8_t* active, cudaStream_t st) {
    using P = PDS;
    QSV_SHAPES(QSV_LAUNCH_SHAPE)
    return launch_pass_ds_r5(T, R, state, dpass, dsteps, dops, dcoef, n, H, items, cstride, active, st);
}

bool pass_shape_ds(int T, int R) {
    QSV_SHAPES(QSV_HAS_SHAPE)
    return pass_shape_ds_r5(T, R);
}

}  // namespace qsv
