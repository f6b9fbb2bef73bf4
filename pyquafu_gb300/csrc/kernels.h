// Host-side launchers of the statevector kernels (kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"

namespace qsv {

constexpr int EXPECT_BATCH = 8;   // Pauli terms reduced per kernel launch
constexpr int REDUCE_BLOCKS = 152 * 4;

bool pass_shape_supported(int precision, int T, int R);
// Shape of a pass kind (0 one-state, 1 two-state reverse sweep) for n qubits:
// the autotuned one if set, else the built-in default.
void resolve_shape(int arith, int kind, int n, int* T, int* R);
bool set_tuned_shape(int arith, int kind, int n, int T, int R);
bool pass_shape_c128(int T, int R);
bool pass_shape_c64(int T, int R);
bool pass_shape_ds(int T, int R);
bool pass_shape_ds_r5(int T, int R);  // pass_ds_r5.cu
cudaError_t launch_pass_ds(int T, int R, void* state, const PassDesc* dpass, const StepDesc* dsteps,
                           const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                            const uint8_t* active, cudaStream_t st);
cudaError_t launch_pass_ds_r5(int T, int R, void* state, const PassDesc* dpass, const StepDesc* dsteps,
                              const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                              const uint8_t* active, cudaStream_t st);
cudaError_t launch_pass_c128(int T, int R, void* state, const PassDesc* dpass, const StepDesc* dsteps,
                             const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                            const uint8_t* active, cudaStream_t st);
cudaError_t launch_pass_c64(int T, int R, void* state, const PassDesc* dpass, const StepDesc* dsteps,
                            const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                            const uint8_t* active, cudaStream_t st);

cudaError_t launch_tile_pass(int precision, int T, int R, void* state, const PassDesc* dpass,
                             const StepDesc* dsteps, const KOp* dops, const void* dcoef, int n, int H,
                             int items, uint64_t cstride, const uint8_t* active, cudaStream_t st);
cudaError_t launch_small(int precision, void* state, uint64_t stride, int batch, int n, const KOp* dops, int nops,
                         const void* dcoef, uint64_t cstride, const uint8_t* active, cudaStream_t st);
// k: the op's dense target count (host copy of dop->k; selects the wide kernel)
cudaError_t launch_globalop(int precision, void* state, int n, int k, const KOp* dop, const void* dcoef, int items,
                            uint64_t cstride, const uint8_t* active, cudaStream_t st);
cudaError_t launch_set_basis(int precision, void* state, uint64_t N, uint64_t index, cudaStream_t st);
cudaError_t launch_convert(bool to64, const void* in, void* out, uint64_t n, cudaStream_t st);
cudaError_t launch_expect_z(int precision, const void* state, uint64_t N, const uint64_t* dzm, int nterms,
                            double* dpartial, int nblocks, cudaStream_t st);
cudaError_t launch_expect_x(int precision, const void* state, uint64_t N, uint64_t xmask, int flip_q,
                            const uint64_t* dzm, const int32_t* dny, int nterms, double* dpartial, int nblocks,
                            cudaStream_t st);
cudaError_t launch_reduce_partials(const double* dpartial, int nblocks, int nterms, double* dout, cudaStream_t st);
// Exact parallel sampling (sample.cu): blocks of SAMPLE_BS amplitudes, grid
// counts for SAMPLE_BINADES binades below 2^e_top.  cnt: SAMPLE_BINADES * nb
// uint64, ties: SAMPLE_BINADES * nb bytes, start: nb + 1 doubles (the exact
// running sum at every block start), seq: blocks summed element by element.
constexpr int SAMPLE_BS = 4096;
constexpr int SAMPLE_BINADES = 16;
cudaError_t launch_sample_binade(int precision, const void* state, uint64_t N, int e_top, uint64_t* cnt,
                                 uint8_t* ties, double* start, int64_t* seq, const double* uni, int64_t shots,
                                 uint64_t* out, cudaStream_t st);
// FP64 sums of |a|^2 over blocks of bs amplitudes and their exclusive prefix
// (dpre[N / bs] = the parallel total)
cudaError_t launch_block_prefix(int precision, const void* state, uint64_t N, uint64_t bs, double* dbsum,
                                double* dpre, cudaStream_t st);

}  // namespace qsv

namespace qsv {
// adjoint.cu
void adjoint_shape(int arith, int* T, int* R);
int adjoint_small_max(int arith);
bool pass2_shape_supported(int arith, int T, int R);
cudaError_t launch_pass2(int arith, int T, int R, void* psi, void* lam, const PassDesc* dpass, const StepDesc* dsteps,
                         const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride, int per_tile,
                         double* partial, int* grid_out, cudaStream_t st);
int pass2_grid_cap();
// adjoint_c128.cu, adjoint_ds.cu (+ adjoint_ds_r4.cu), adjoint_c64.cu: the tiled two-state
// pass per arithmetic
bool pass2_shape_c128(int T, int R);
bool pass2_shape_ds(int T, int R);
bool pass2_shape_ds_r4(int T, int R);  // adjoint_ds_r4.cu
bool pass2_shape_c64(int T, int R);
cudaError_t launch_pass2_c128(int T, int R, void* psi, void* lam, const PassDesc* dpass, const StepDesc* dsteps,
                              const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                              int per_tile, double* partial, int* grid_out, cudaStream_t st);
cudaError_t launch_pass2_ds(int T, int R, void* psi, void* lam, const PassDesc* dpass, const StepDesc* dsteps,
                            const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                            int per_tile, double* partial, int* grid_out, cudaStream_t st);
cudaError_t launch_pass2_ds_r4(int T, int R, void* psi, void* lam, const PassDesc* dpass, const StepDesc* dsteps,
                               const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                               int per_tile, double* partial, int* grid_out, cudaStream_t st);
cudaError_t launch_pass2_c64(int T, int R, void* psi, void* lam, const PassDesc* dpass, const StepDesc* dsteps,
                             const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride,
                             int per_tile, double* partial, int* grid_out, cudaStream_t st);
cudaError_t launch_small2(int arith, void* psi, void* lam, int n, const KOp* dops, int nops, const void* dcoef,
                          int items, uint64_t cstride, double* probe_out, uint64_t pstride, cudaStream_t st);
cudaError_t launch_hamiltonian(int storage, const void* psi, void* lam, uint64_t N, const uint64_t* dx,
                               const uint64_t* dz, const int32_t* dny, const double* dc, int nterms, cudaStream_t st);
cudaError_t launch_probe_reduce(const double* partial, int grid, int np, double* out, cudaStream_t st);
}  // namespace qsv

namespace qsv {
// batch.cu
cudaError_t launch_bind(int arith, void* pool, uint64_t cstride, const Bind* dbinds, int nb, const double* dvals,
                        int nslots, int items, cudaStream_t st);
cudaError_t launch_replicate(int arith, void* pool, uint64_t cstride, uint64_t len, int items, cudaStream_t st);
cudaError_t launch_zero_items(int storage, void* state, int n, int items, cudaStream_t st);
uint64_t hamiltonian_chunk(int n);
cudaError_t launch_expect_seg(int storage, const void* psi, int n, int items, const uint64_t* dx, const uint64_t* dz,
                              const int32_t* dny, const double* dc, const int32_t* doptr, int nobs, double* epart,
                              double* out, cudaStream_t st);
cudaError_t launch_lambda_seg(int storage, const void* psi, void* lam, int n, int items, const uint64_t* dx,
                              const uint64_t* dz, const int32_t* dny, const double* dc, const int32_t* dtobs,
                              int nterms, int nobs, const double* dw, cudaStream_t st);
cudaError_t launch_probe_reduce_seg(const double* partial, uint64_t ntiles, int tpi, int items, int np, double* out,
                                    int ostride, int ooff, cudaStream_t st);
cudaError_t launch_slot_gather(const double* vals, int nprobe, int items, const int32_t* sptr, const int32_t* sidx,
                               int nslots, double* grads, cudaStream_t st);
}  // namespace qsv

namespace qsv {
// shots.cu: per-shot trajectories (mid-circuit measure / reset / cif)
struct MeasureSpec {
    uint8_t q[8];    // measured qubits, outcome bit order
    uint8_t srt[8];  // the same, ascending
    uint8_t cb[8];   // classical bits written (measure)
    int32_t k;       // qubits measured
    int32_t reset;   // 1: reset (final block 0), 0: measure
};
struct CifSpec {
    uint8_t cb[16];
    int32_t nc;
    uint64_t condition;
};
int outcome_blocks_per_item(int n, int k);
cudaError_t launch_measure(void* state, int n, const MeasureSpec& ms, int items, const double* duni, int draw,
                           int ndraws, uint8_t* dcreg, int ncb, double* dpart, int32_t* doutcome, double* dscale,
                           cudaStream_t st);
cudaError_t launch_cif_mask(const uint8_t* dcreg, int ncb, int items, const CifSpec& cs, uint8_t* dactive,
                            cudaStream_t st);
cudaError_t launch_items_copy(void* state, int n, int items, const void* psi0, cudaStream_t st);
}  // namespace qsv

namespace qsv {
// noise.cu: per-shot noise channels on one qubit, per-item final sample
constexpr int MAX_CHANNEL_OPS = 8;
int channel_blocks_per_item(int n);  // CTAs per item of the Kraus-norm reduction
// cross: some Kraus operator's Gram matrix K^dagger K has a nonzero
// off-diagonal entry (the norms then need sum conj(a) c as well)
cudaError_t launch_channel(void* state, int n, int q, int m, int kraus, int cross, const double* dmats,
                           const double* dprobs, int items, const double* duni, int draw, int ndraws, double* dpart,
                           double* dimat, cudaStream_t st);
cudaError_t launch_item_sample(const void* state, int n, int items, const double* duni, int draw, int ndraws,
                               uint64_t* dout, cudaStream_t st);
}  // namespace qsv
