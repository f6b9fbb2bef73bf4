// Fused tile-pass kernel, complex64 storage with FP32 arithmetic.
#include "pass_launch.cuh"

// shapes: (tile qubits, register qubits, tile buffers, min CTAs per SM)
#define QSV_SHAPES(X) X(12, 5, 2, 1) X(13, 5, 2, 1) X(12, 4, 1, 2) X(13, 4, 1, 1)

namespace qsv {

cudaError_t launch_pass_c64(int T, int R, void* state, const PassDesc* dpass, const StepDesc* dsteps,
                            const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                            const uint8_t* active, cudaStream_t st) {
    using P = P32;
    QSV_SHAPES(QSV_LAUNCH_SHAPE)
    return cudaErrorInvalidValue;
}

bool pass_shape_c64(int T, int R) {
    QSV_SHAPES(QSV_HAS_SHAPE)
    return false;
}

}  // namespace qsv
