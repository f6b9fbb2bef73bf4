// Fused two-state pass of the adjoint reverse sweep, complex128 storage with FP64 arithmetic.
#include "pass2_launch.cuh"

// shapes: (tile qubits, register qubits, tile buffers per state, min CTAs per SM)
#define QSV_SHAPES2(X) X(11, 4, 2, 1) X(11, 3, 1, 2)

namespace qsv {

cudaError_t launch_pass2_c128(int T, int R, void* psi, void* lam, const PassDesc* dpass, const StepDesc* dsteps,
                              const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                              int per_tile, double* partial, int* grid_out, cudaStream_t st) {
    using P = P64;
    QSV_SHAPES2(QSV_LAUNCH2_SHAPE)
    return cudaErrorInvalidValue;
}

bool pass2_shape_c128(int T, int R) {
    QSV_SHAPES2(QSV_HAS2_SHAPE)
    return false;
}

}  // namespace qsv
