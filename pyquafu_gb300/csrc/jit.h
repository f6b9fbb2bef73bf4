// Circuit-specialised tile passes: each register round of a pass is emitted
// as straight-line PTX for sm_103a (targets, controls, coefficient offsets
// and shared-memory offsets in the tile layout become constants; X/SWAP/Y become
// register renames), two-target dense gates as shared-memory steps; the PTX
// is compiled once per distinct pass and launched instead of the
// interpreting kernels k_pass / k_pass2.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "engine.h"

struct qfvm_plan;

namespace qsv {

struct JitShape {
    int nstates = 1;  // 1: one-state pass (k_pass), 2: psi + lam with probes (k_pass2)
    int nb = 1;       // tile buffers (2 = prefetch the next tile during this one)
    int minb = 1;     // .minnctapersm (register budget = 64K / (threads * minb))
    int pcoef = 0;    // 1: coefficients travel in the kernel parameters (plans whose pool is never rebound)
    int bounds = 0;   // 1: every shared / global / bulk access checked against its buffer (QFVM_BOUNDS_CHECK=1)
    int chain = 0;    // 1: double-single passes hand the states on as float pairs (first reads FP64, last writes it)
};

// 1 when the passes of `hp` run with shape `sh` hand the states on as float
// pairs (double-single, every pass a specialised tile pass).
int chain_for(const HostPlan& hp, const JitShape& sh);

// QFVM_BOUNDS_CHECK=1 in the environment (read when a plan's passes are
// compiled): the specialised passes check each shared-memory access, each
// global store and each bulk copy against its buffer; an access outside is
// skipped and the pass writes QFVM_ERR_BOUNDS to the status word.
int bounds_check_env();

// PTX of tile pass `pi` of plan `hp` as kernel `entry`; false (with a reason)
// when the pass has a step the generator does not handle.
bool jit_pass_ptx(const HostPlan& hp, int pi, const JitShape& sh, const std::string& entry, std::string* ptx,
                  std::string* why);

// Parameter-block coefficients of pass `pi` (sh.pcoef): true with the pool
// range [cmin, cmax) the kernel takes as its last parameter p_cblob (in the
// arithmetic's format: float, float pair or double per pool entry); false
// when the pass reads them from the pool in global memory.
bool jit_pass_coef_block(const HostPlan& hp, int pi, const JitShape& sh, uint32_t* cmin, uint32_t* cmax);

// Dynamic shared memory of a specialised pass: nb tile slots of nstates
// tiles in the padded tile layout, the per-warp probe sums, one mbarrier per
// slot.
size_t jit_smem_bytes(const HostPlan& hp, const JitShape& sh, int nprobe);

// Device status word of the specialised passes (per device, zeroed): a
// kernel whose bounded wait for its tile copies gave up writes
// QFVM_ERR_TIMEOUT.  jit_status_take reads it after the stream's work
// (synchronising `st`), clears it and returns 0 or QFVM_ERR_TIMEOUT.
int jit_status_take(cudaStream_t st);
// Test hook: the next launches expect `extra` more bytes per tile than the
// copies bring (their waits run out after `wait_ns`); 0, 0 restores the
// defaults.
void jit_set_wait_test(uint32_t extra, uint64_t wait_ns);

// Kernel name of a specialised pass: qsv_tile_pass_<c128|ds|c64> (one
// state) or qsv_tile_sweep_<c128|c64> (reverse sweep with probes).
std::string jit_entry_name(int arith, int nstates);

// Everything the generator reads for pass `pi` (the module cache key);
// false when the pass is not handled.
bool jit_pass_key(const HostPlan& hp, int pi, const JitShape& sh, std::string* key, std::string* why);

// Global switch (default on) and launch shape knobs.
struct JitConfig {
    int enabled = 1;
    int nb1 = 2, minb1 = 0;  // one-state passes (minb 0 = automatic)
    int nb2 = 1, minb2 = 0;  // two-state passes
};
JitConfig jit_config();
void jit_set_config(const JitConfig& c);

// Compiles every eligible tile pass of `p` for `nstates` (no-op when the
// plan's arithmetic or the switch rules it out).  Call outside stream
// capture.  A failed compile leaves the plan on the interpreting kernels
// (reported once on stderr, message in *err); the return value is 0.
int jit_prepare(qfvm_plan* p, int nstates, std::string* err);
void jit_release(qfvm_plan* p);

// Launches pass `pi` of `p` through its compiled kernel; *launched = false
// (nothing issued) when the pass has none.
cudaError_t jit_launch_pass(qfvm_plan* p, int pi, void* psi, void* lam, const void* dcoef, int items,
                            uint64_t cstride, const uint8_t* active, int per_tile, double* partial, int* grid_out,
                            cudaStream_t st, bool* launched);

// Number of compiled passes of `p` for nstates (diagnostics).
int jit_compiled_passes(const qfvm_plan* p, int nstates);

}  // namespace qsv
