// Internals of the C ABI shared by its translation units (capi.cu, batch_capi.cu).
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"
#include "qfvm_gb300.h"

namespace qsv_capi {

extern std::atomic<uint64_t> g_launches;
extern std::mutex g_boundary_mu;  // serialises the host-buffer entry points (shared cached state)

int fail(int code, const std::string& msg);
// After `st` is synchronised: QFVM_ERR_TIMEOUT (with the message set) when a
// specialised pass's bounded wait for its tile copies gave up since the last
// check, else QFVM_OK.
int check_status(cudaStream_t st);
int check_device();

// NVTX range over a scope (a pass launch, a sampling call, a batched run):
// profilers group the kernels launched inside it; free when no tool is
// attached.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

#define QSV_CUDA(call, what)                                                                        \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            return ::qsv_capi::fail(e_ == cudaErrorMemoryAllocation ? QFVM_ERR_NOMEM : QFVM_ERR_CUDA, \
                                    std::string(what) + ": " + cudaGetErrorString(e_));            \
        }                                                                                          \
    } while (0)

#define QSV_TRY(expr)                   \
    do {                                \
        int rc_ = (expr);               \
        if (rc_ != QFVM_OK) return rc_; \
    } while (0)

// Arithmetic of complex128 work issued by the host-buffer entry points
// (simulate_circuit, applyop_statevec, per-shot and noisy trajectories):
// QFVM_C128_DS (float pairs, the default) or QFVM_C128 (IEEE FP64).
int c128_arith();

// Host-side fault injection (qfvm_test_fault): once armed, the countdown-th
// device allocation or kernel stage from then on fails on the host without
// calling CUDA, so failure paths are exercised with no GPU fault.
enum { FAULT_NONE = 0, FAULT_ALLOC = 1, FAULT_STAGE = 2 };
bool fault_hit(int kind);
// cudaMalloc, unless an armed allocation fault fires (then
// cudaErrorMemoryAllocation with *p = nullptr)
cudaError_t dev_malloc(void** p, size_t bytes);

// Growable device scratch buffer.
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes) {
        if (bytes <= cap) return QFVM_OK;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(bytes, 256);
        QSV_CUDA(dev_malloc(&p, want), "scratch allocation");
        cap = want;
        return QFVM_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T>
    T* as() {
        return static_cast<T*>(p);
    }
};

inline int store_precision(int precision) { return precision == QFVM_C64 ? QFVM_C64 : QFVM_C128; }
inline size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

}  // namespace qsv_capi

struct qfvm_sv {
    int n = 0, precision = QFVM_C128;  // storage: QFVM_C128 or QFVM_C64
    int arith = QFVM_C128;             // arithmetic of qfvm_sv_apply: QFVM_C128, QFVM_C128_DS or QFVM_C64
    int64_t last_seq_blocks = 0;       // blocks the last qfvm_sv_sample summed element by element
    uint64_t N = 0;
    void* d = nullptr;
    cudaStream_t stream = nullptr;
    qsv_capi::DevBuf red, masks, sample_blk, sample_shots, staging;
};

struct qfvm_plan {
    qsv::HostPlan hp;
    std::vector<cudaEvent_t> events;  // for timed runs
    void* dbuf = nullptr;
    qsv::PassDesc* dpass = nullptr;
    qsv::StepDesc* dsteps = nullptr;
    qsv::KOp* dops = nullptr;
    void* dcoef = nullptr;
    // circuit-specialised kernels of the tile passes (jit.cu), per state
    // count (index 0: one state, 1: psi + lam); null entries run interpreted
    std::vector<const void*> jit[2];
    bool jit_ready[2] = {false, false};
    // per pass: the coefficient parameter block of its kernel (empty: the
    // kernel reads the pool in global memory)
    std::vector<std::vector<unsigned char>> jit_cblob[2];
    // double-single plans whose passes are all specialised hand the states
    // from pass to pass as float pairs (jit_chain, per state count); runs
    // that write back only some items (active masks) clear chain_ok before
    // the first run
    bool chain_ok = true;
    bool jit_chain[2] = {false, false};
};

namespace qsv_capi {
int make_plan(int n, int precision, const qfvm_op* ops, int64_t n_ops, const double* matpool, int64_t matpool_len,
              int T, int R, qfvm_plan** out);
// merge_diagonals: plain simulation plans only (merge_round_diagonals)
int make_plan_gops(int n, int precision, const std::vector<qsv::GOp>& gops, int T, int R, qfvm_plan** out,
                   bool merge_diagonals = false);
void free_plan(qfvm_plan* p);
// Every pass of a plan over `items` states back to back (shared coefficients;
// active = optional per-item write-back mask).
int run_plan_items(qfvm_plan* p, void* state, int items, const uint8_t* active, cudaStream_t st);
}  // namespace qsv_capi
