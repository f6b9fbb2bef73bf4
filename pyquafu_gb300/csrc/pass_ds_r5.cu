// Fused tile-pass kernel, complex128 storage with double-single (FP32 pair)
// arithmetic: the five-register shape.
#include "pass_launch.cuh"

// shapes: (tile qubits, register qubits, tile buffers, min CTAs per SM)
#define QSV_SHAPES(X) X(12, 5, 2, 1)

namespace qsv {

cudaError_t launch_pass_ds_r5(int T, int R, void* state, const PassDesc* dpass, const StepDesc* dsteps,
                              const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                              const uint8_t* active, cudaStream_t st) {
    using P = PDS;
    QSV_SHAPES(QSV_LAUNCH_SHAPE)
    return cudaErrorInvalidValue;
}

bool pass_shape_ds_r5(int T, int R) {
    QSV_SHAPES(QSV_HAS_SHAPE)
    return false;
}

}  // namespace qsv
