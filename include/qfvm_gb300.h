/*
 * qfvm_gb300 — GB300 (sm_103a) statevector engine, C ABI.
 *
 * This header is the drop-in boundary for pyquafu's statevector hot path.  The
 * reference binds its C++ engine to Python through the pybind11 module `qfvm`
 * (src/qfvm/qfvm.cpp:263-288); the entry points below carry the same
 * operations over plain pointers and sizes, so any FFI (ctypes, cffi, a
 * pybind11 shim) can bind them.  All functions return a qfvm_status; on
 * failure qfvm_last_error() holds a message for the calling thread.  Nothing
 * here exits the process or traps the device.
 *
 * Conventions (identical to the reference):
 *   - amplitude index bit q is qubit q (little-endian), statevector.hpp:1388-1401;
 *   - host states are interleaved complex128 (re, im) arrays of 2^n entries;
 *   - a gate's qubits list holds its controls first, then its targets
 *     (ControlledGate.pos = ctrls + targs); matrix row/column bit j refers to
 *     target j (statevector.hpp:954-963).
 */
#ifndef QFVM_GB300_H
#define QFVM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QFVM_ABI_VERSION 1
#define QFVM_MAX_OP_QUBITS 16
#define QFVM_MAX_QUBITS 34

/* Status codes. */
typedef enum {
    QFVM_OK = 0,
    QFVM_ERR_INVALID = 1,     /* bad argument (qubit index, size, matrix shape ...) */
    QFVM_ERR_CUDA = 2,        /* a CUDA call failed */
    QFVM_ERR_NOMEM = 3,       /* device allocation failed */
    QFVM_ERR_UNSUPPORTED = 4, /* valid input the engine does not handle */
    QFVM_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
    QFVM_ERR_NODEVICE = 6,    /* no CUDA device */
    QFVM_ERR_BOUNDS = 7       /* bounds-checked kernels (QFVM_BOUNDS_CHECK=1): an index out of range, access skipped */
} qfvm_status;

/* Operation kinds.  1..17 are the named gates of the reference's OPMAP table
 * (src/qfvm/qasm.hpp:43-46, dispatched in simulator.hpp:30-113); everything
 * else is a matrix gate (simulator.hpp:12-28). */
enum {
    QFVM_OP_X = 1, QFVM_OP_Y, QFVM_OP_Z, QFVM_OP_H, QFVM_OP_S, QFVM_OP_SDG, QFVM_OP_T,
    QFVM_OP_TDG, QFVM_OP_P, QFVM_OP_RX, QFVM_OP_RY, QFVM_OP_RZ, QFVM_OP_CX, QFVM_OP_CZ,
    QFVM_OP_CP, QFVM_OP_CCX, QFVM_OP_RZZ,
    QFVM_OP_MATRIX = 32,  /* targ matrix in the pool: mat_dim x mat_dim, row-major complex128 */
    QFVM_OP_MEASURE = 40, /* qfvm_simulate_shots only (not a gate) */
    QFVM_OP_RESET = 41,   /* qfvm_simulate_shots only */
    QFVM_OP_CIF = 42,     /* qfvm_simulate_shots only */
    QFVM_OP_UCHANNEL = 44, /* qfvm_simulate_noise only: unitary channel */
    QFVM_OP_KRAUS = 45     /* qfvm_simulate_noise only: Kraus channel */
};

/* Precision of a device state. */
enum {
    QFVM_C128 = 0, /* complex128 storage, IEEE FP64 arithmetic */
    QFVM_C64 = 1,  /* complex64 storage, FP32 arithmetic, FP64 reductions */
    QFVM_C128_DS = 2 /* complex128 storage, double-single (FP32 pair) arithmetic */
};

/* Generators of parameterised matrix gates (dG/dtheta = -i/2 Q G): Q is the
 * Pauli X, Y or Z string on the targets with the controls as a projector, or
 * (QFVM_GEN_PHASE) -2 times the projector onto targets and controls all 1. */
enum { QFVM_GEN_NONE = 0, QFVM_GEN_X = 1, QFVM_GEN_Y = 2, QFVM_GEN_Z = 3, QFVM_GEN_PHASE = 4 };

/* One gate of a packed circuit (128 bytes). */
typedef struct qfvm_op {
    int32_t kind;      /* QFVM_OP_* */
    int32_t ncontrols; /* leading entries of qubits[] that are controls */
    int32_t nqubits;   /* controls + targets */
    int32_t mat_dim;   /* QFVM_OP_MATRIX: 2^targets; else 0 */
    int32_t qubits[QFVM_MAX_OP_QUBITS];
    int32_t slot;      /* parameter slot for batched/adjoint runs, -1 if none */
    int32_t gen;       /* QFVM_OP_MATRIX with a slot: generator, QFVM_GEN_* (0 for named gates) */
    double params[4];  /* gate angles (params[0] is the rotation angle) */
    int64_t mat_offset; /* complex index of the matrix in the pool, -1 if none */
} qfvm_op;

/* ------------------------------------------------------------------ */
/* Library state                                                       */
/* ------------------------------------------------------------------ */

/* Message for the last failed call on this thread ("" if none). */
const char* qfvm_last_error(void);
int32_t qfvm_abi_version(void);
/* Number of kernel launches issued by this library since load (all threads). */
uint64_t qfvm_launch_count(void);

/* ------------------------------------------------------------------ */
/* Reference-shaped entry points (host buffers), src/qfvm/qfvm.cpp      */
/* ------------------------------------------------------------------ */

/* simulate_circuit (qfvm.cpp:68-134, final-measure branch :90-103).
 * Runs the gates of a circuit on the GPU.  `state` holds 2^n complex128
 * amplitudes: if `state_given` is nonzero it is the input state (the
 * reference adopts a non-empty inputstate in place, qfvm.cpp:86-89),
 * otherwise the run starts from |0..0>.  On return `state` holds the final
 * state.  If shots > 0, `uniforms[shots]` (host draws in [0,1)) select one
 * basis index per shot by the sequential FP64 CDF scan of
 * measure_samples (statevector.hpp:1387-1397), written to out_indices; an
 * index of 2^n means the uniform was not below the total probability. */
int qfvm_simulate_circuit(int32_t num_qubits, const qfvm_op* ops, int64_t n_ops, const double* matpool,
                          int64_t matpool_len, double* state, int32_t state_given, const double* uniforms,
                          int64_t shots, uint64_t* out_indices);

/* applyop_statevec (qfvm.cpp:36-50): one gate applied in place to a host state
 * of state_len amplitudes (a power of two). */
int qfvm_applyop_statevec(const qfvm_op* op, const double* matpool, int64_t matpool_len, double* state,
                          uint64_t state_len);

/* sampling_statevec (qfvm.cpp:52-66): one basis index per host uniform. */
int qfvm_sampling_statevec(const double* state, uint64_t state_len, const double* uniforms, int64_t shots,
                           uint64_t* out_indices);

/* expect_statevec (qfvm.cpp:246-261, statevector.hpp:1250-1305): unweighted
 * <P_k> for Pauli strings given as flip mask (X and Y), Z mask (Z and Y) and
 * the number of Y factors. */
int qfvm_expect_statevec(const double* state, uint64_t state_len, const uint64_t* x_masks,
                         const uint64_t* z_masks, const int32_t* y_counts, int64_t n_terms, double* out);

/* Adjoint gradient: grad_adjoint of quafu/algorithms/gradients/gradiant.py:144-173.
 * Runs the gates from |0..0> (or from psi_in, 2^n host complex128 amplitudes
 * when not NULL), evaluates E = sum_t coeffs[t] <P_t> (Pauli terms as for
 * qfvm_expect_statevec), forms lam = H psi and sweeps the gates backwards
 * through their inverses, un-applying each to psi and lam together.  For
 * every gate with slot >= 0 it adds dE/dtheta = Im<lam| Q |psi> (Q the gate's
 * generator: RX/RY/RZ/RZZ, P/CP, or QFVM_GEN_* for matrix gates) into
 * grads[slot]; grads has n_slots entries and is overwritten.  precision:
 * QFVM_C128 (FP64), QFVM_C128_DS or QFVM_C64 (FP32 gates, FP64 reductions). */
int qfvm_adjoint(int32_t num_qubits, int32_t precision, const qfvm_op* ops, int64_t n_ops, const double* matpool,
                 int64_t matpool_len, const uint64_t* x_masks, const uint64_t* z_masks, const int32_t* y_counts,
                 const double* coeffs, int64_t n_terms, const double* psi_in, double* energy, double* grads,
                 int64_t n_slots);

/* Allocation-free expectation (no counterpart in the reference).
 * For callers that cannot allocate GPU memory while they run -- processes
 * that reserve all of HBM for their own pool at start-up, or hot loops where
 * cudaMalloc/cudaFree would synchronise the device -- this computes the same
 * unweighted <P_k> as qfvm_expect_statevec on a state that already lives in
 * device memory the caller owns (`dev_state`, state_len amplitudes of
 * complex128 or complex64 per `precision`), issuing its work on `stream`
 * (NULL = default stream) and waiting for it.  It allocates nothing: its
 * scratch is a fixed 64 KiB __device__ array in the library, which every GPU
 * that loads the library holds until exit.  At most QFVM_NOALLOC_MAX_TERMS
 * terms per call (larger requests are rejected).  All calls on a device share
 * that scratch, so calls that overlap on the GPU race and must be serialised
 * by the caller.  The first call on each device resolves the scratch address
 * (with that device current).  A call synchronises its stream and copies
 * through pageable host memory, so it cannot be used inside a stream capture:
 * on a capturing stream it returns QFVM_ERR_UNSUPPORTED.  `dev_state` must be
 * device (or managed) memory of the current device, else QFVM_ERR_INVALID.
 * On failure the message is in qfvm_noalloc_last_error() (kept per calling
 * thread). */
#define QFVM_NOALLOC_MAX_TERMS 1024
int qfvm_expect_device_noalloc(const void* dev_state, uint64_t state_len, int32_t precision,
                               const uint64_t* x_masks, const uint64_t* z_masks, const int32_t* y_counts,
                               int64_t n_terms, double* out, void* stream);
const char* qfvm_noalloc_last_error(void);

/* Arithmetic of the complex128 work the host-buffer entry points issue
 * (qfvm_simulate_circuit, qfvm_applyop_statevec, qfvm_simulate_shots,
 * qfvm_simulate_noise): QFVM_C128_DS (the default; float-pair arithmetic on
 * the FP32 pipes, per-amplitude error below 1e-12 against FP64) or QFVM_C128
 * (IEEE FP64).  Storage is complex128 either way.  No counterpart in the
 * reference, whose CPU path is FP64. */
int qfvm_set_c128_arithmetic(int32_t arith);
int32_t qfvm_get_c128_arithmetic(void);

/* Failure-path test hook (no counterpart in the reference).  kind 1: the
 * countdown-th device allocation from now on fails (QFVM_ERR_NOMEM) without
 * calling cudaMalloc; kind 2: the countdown-th pass of a plan run fails
 * (QFVM_ERR_CUDA, "injected kernel-stage failure") before its launch; kind
 * 0 disarms.  One fault fires, then the hook disarms itself.  Nothing
 * touches the GPU, so the context stays usable.
 * kind 3 (stays armed until kind 0): every specialised tile pass expects 16
 * bytes more per tile than its bulk copies bring, so its bounded wait for the
 * tile (limit: countdown milliseconds) runs out; the kernel records
 * QFVM_ERR_TIMEOUT in its status word and returns, and the next
 * synchronising call reports QFVM_ERR_TIMEOUT.  No fault, no hang: the copies
 * themselves complete and the context stays usable. */
#define QFVM_FAULT_NONE 0
#define QFVM_FAULT_ALLOC 1
#define QFVM_FAULT_STAGE 2
#define QFVM_FAULT_WAIT 3
int qfvm_test_fault(int32_t kind, int64_t countdown);

/* ------------------------------------------------------------------ */
/* Device-resident statevector (engine-owned HBM buffer)               */
/* ------------------------------------------------------------------ */

typedef struct qfvm_sv qfvm_sv;

int qfvm_sv_create(int32_t num_qubits, int32_t precision, qfvm_sv** out);
int qfvm_sv_destroy(qfvm_sv* sv);
int qfvm_sv_set_zero(qfvm_sv* sv);                                     /* |0..0> */
int qfvm_sv_upload(qfvm_sv* sv, const double* host_c128, uint64_t n_amps);   /* host complex128 -> device */
int qfvm_sv_download(qfvm_sv* sv, double* host_c128, uint64_t n_amps); /* device -> host complex128 */
int qfvm_sv_apply(qfvm_sv* sv, const qfvm_op* ops, int64_t n_ops, const double* matpool, int64_t matpool_len);
int qfvm_sv_expect(qfvm_sv* sv, const uint64_t* x_masks, const uint64_t* z_masks, const int32_t* y_counts,
                   int64_t n_terms, double* out);
int qfvm_sv_sample(qfvm_sv* sv, const double* uniforms, int64_t shots, uint64_t* out_indices);
int qfvm_sv_norm2(qfvm_sv* sv, double* out);                           /* FP64 sum |a|^2 */
/* Blocks of 4096 amplitudes that the last qfvm_sv_sample on this state summed
 * element by element (the exact running sum crossed a binade or met a
 * rounding tie there); every other block advanced the sum by one integer
 * addition.  Sampling is exact either way. */
int qfvm_sv_sample_stats(qfvm_sv* sv, int64_t* sequential_blocks);
/* Raw device pointer and byte size of the state (for host-side interop). */
int qfvm_sv_device_ptr(qfvm_sv* sv, void** dev_ptr, uint64_t* nbytes);
/* Stream the engine issues this state's work on (cudaStream_t as void*). */
int qfvm_sv_stream(qfvm_sv* sv, void** stream);

/* ------------------------------------------------------------------ */
/* Compiled circuits: plan once, run many times on device states        */
/* ------------------------------------------------------------------ */

typedef struct qfvm_plan qfvm_plan;

/* Classify and fuse a gate list for states of `num_qubits` at `precision`.
 * tile_qubits / reg_qubits select the fused-pass shape (0 = engine default). */
int qfvm_plan_create(int32_t num_qubits, int32_t precision, const qfvm_op* ops, int64_t n_ops,
                     const double* matpool, int64_t matpool_len, int32_t tile_qubits, int32_t reg_qubits,
                     qfvm_plan** out);
int qfvm_plan_destroy(qfvm_plan* plan);
/* Plan statistics: fused passes, register rounds, gates, algorithmic bytes of
 * one run (2 * bytes per amplitude * 2^n per pass) and gate-equivalent bytes. */
int qfvm_plan_stats(const qfvm_plan* plan, int64_t* passes, int64_t* rounds, int64_t* gates,
                    double* pass_bytes, double* gate_bytes);
int qfvm_plan_run(qfvm_plan* plan, qfvm_sv* sv);
/* Run the plan with a CUDA event recorded on the state's stream around every
 * pass launch; waits for completion and writes each pass's device time (ms)
 * to pass_ms[0..passes-1] and its type (0 tile, 1 whole-state, 2 k-target)
 * to pass_type. */
int qfvm_plan_run_timed(qfvm_plan* plan, qfvm_sv* sv, float* pass_ms, int32_t* pass_type);

/* ---------------------------------------------------------------------------
 * Per-shot trajectories: the branch of simulate_circuit for circuits with
 * operations after a measurement (qfvm.cpp:104-133, dispatch of measure /
 * reset / cif in simulator.hpp:95-111).  Every shot runs the whole circuit on
 * its own copy of psi_in (|0...0> when NULL); shots run side by side on the
 * device.  Besides gates, `ops` holds:
 *   QFVM_OP_MEASURE  nqubits = k (1..8) qubits in qubits[0..k), the classical
 *                    bits they write in qubits[8..8+k)
 *   QFVM_OP_RESET    nqubits = k (1..8) qubits in qubits[0..k)
 *   QFVM_OP_CIF      classical bits in qubits[0..nqubits), condition in
 *                    params[0]; the next mat_dim ops (gates only) are its body,
 *                    applied when the bits, first most significant, equal it
 * Every measure and reset draws one uniform: uniforms[s * n_draws + d] is
 * shot s's d-th draw (n_draws = measures + resets), and the outcome is the
 * first joint outcome m with u * total < cumulative probability (FP64, in
 * outcome order; bit j of m is qubits[j]).  outcomes[s] = the measured
 * classical bits of shot s in ascending order, the first most significant
 * (the reference's count key); final_state (optional, 2^n complex128)
 * receives the last shot's state. */
int qfvm_simulate_shots(int32_t num_qubits, int32_t num_cbits, const qfvm_op* ops, int64_t n_ops,
                        const double* matpool, int64_t matpool_len, const double* psi_in, int64_t shots,
                        const double* uniforms, int64_t n_draws, uint64_t* outcomes, double* final_state);

/* ---------------------------------------------------------------------------
 * Noisy trajectories: NoiseSVSimulator.run (quafu/simulators/simulator.py:
 * 148-225), the shots side by side on the device.  Besides gates, `ops` holds
 * one-qubit channels on qubits[0] (nqubits = 1, mat_dim = 2) with m =
 * params[0] operators (1..8) as m consecutive row-major 2x2 matrices at
 * mat_offset in the pool:
 *   QFVM_OP_UCHANNEL  unitary channel; the m pool entries after the matrices
 *                     hold the probabilities (real parts); operator i is
 *                     picked as np.random.choice does (first i with
 *                     cumsum(p)[i] / sum(p) > u), noise.py:86-91
 *   QFVM_OP_KRAUS     Kraus channel, the reference's rule (simulator.py:61-76):
 *                     s += ||K_i psi|| / ||psi|| in order, the first i with
 *                     u < s is applied as K_i psi / ||K_i psi||; none: no change
 * Draws per shot (uniforms[s * n_draws + d]), in the reference's order: one per
 * unitary channel (op order), one per Kraus channel (op order), one for the
 * final sample; n_draws = unitary + Kraus channels + 1.  samples[s] is the
 * basis index measure_samples' scan picks (first index whose running |a|^2
 * sum exceeds u; 2^n when none); with n_terms > 0, expvals[s * n_terms + t] =
 * coeffs[t] <P_t> of shot s's final state (FP64).  psi_in NULL: |0...0>. */
int qfvm_simulate_noise(int32_t num_qubits, const qfvm_op* ops, int64_t n_ops, const double* matpool,
                        int64_t matpool_len, const double* psi_in, int64_t shots, const double* uniforms,
                        int64_t n_draws, uint64_t* samples, const uint64_t* x_masks, const uint64_t* z_masks,
                        const int32_t* y_counts, const double* coeffs, int64_t n_terms, double* expvals);

/* ---------------------------------------------------------------------------
 * Batched runs.  Replaces the reference's per-sample Python loops over
 * Estimator.run: quafu/algorithms/interface/torch.py:76-78 (ExecuteCircuits
 * forward), quafu/algorithms/gradients/vjp.py:93-103 (jacobian via
 * ParamShift per sample and observable) and quafu/algorithms/estimator.py:186-229.
 *
 * A batch holds groups.  A group is n_items circuits on num_qubits qubits
 * that share one gate list `ops` and one set of n_obs observables; they
 * differ only in the angles of their slotted rx/ry/rz/p/cp/rzz gates, which a
 * run reads from values[item * n_slots + slot] (ops[k].params give the
 * structure only).  Every item starts in |0...0>.  Observable o is the sum of
 * the terms t with obs_index[t] == o (obs_index NULL: one observable), term t
 * being coeffs[t] * P_t with P_t given by x/z masks and y count as in
 * qfvm_expect_statevec.
 *
 * A run takes the slot values of all groups back to back (group order, then
 * item-major) and writes expvals[item * n_obs + o] = <O_o> (FP64 sums) for all
 * groups back to back.  Mode 1 (batch created with QFVM_BATCH_GRADS) also
 * writes grads[item * n_slots + s] = d(sum_o w[item, o] <O_o>)/d value[s], by
 * the adjoint method, with weights w laid out like expvals (NULL: all 1).
 * Groups run concurrently on their own streams; the first run of a mode is
 * issued directly, the second is captured into a CUDA graph and every later
 * run of that mode replays it as a single graph launch.  A batch is used by
 * one thread at a time.
 * ------------------------------------------------------------------------- */
typedef struct qfvm_batch qfvm_batch;
#define QFVM_BATCH_GRADS 1    /* prepare gradient (mode 1) runs */
#define QFVM_BATCH_NO_GRAPH 2 /* always issue runs directly (no CUDA graph) */
/* shapes: NULL (defaults) or {tile qubits, register qubits} of the forward
 * passes then of the reverse-sweep passes, 0 for a default entry; an
 * uncompiled shape is QFVM_ERR_INVALID (qfvm_shape_supported lists them). */
int qfvm_batch_create(int32_t precision, int32_t flags, const int32_t* shapes, qfvm_batch** out);
/* Whether a fused-pass shape is compiled in: kind 0 = one-state passes
 * (qfvm_plan_create, batch forward), 1 = two-state reverse-sweep passes. */
int32_t qfvm_shape_supported(int32_t precision, int32_t kind, int32_t tile_qubits, int32_t reg_qubits);
/* Process-wide shape for plans of `num_qubits` qubits that do not name one
 * (every entry point above and batch groups without explicit shapes), set by
 * the autotuner (pyquafu_gb300.autotune); tile_qubits 0 restores the
 * built-in default. */
int qfvm_set_tuned_shape(int32_t precision, int32_t kind, int32_t num_qubits, int32_t tile_qubits,
                         int32_t reg_qubits);
int qfvm_get_shape(int32_t precision, int32_t kind, int32_t num_qubits, int32_t* tile_qubits, int32_t* reg_qubits);
int qfvm_batch_add_group(qfvm_batch* batch, int32_t num_qubits, const qfvm_op* ops, int64_t n_ops,
                         const double* matpool, int64_t matpool_len, const uint64_t* x_masks, const uint64_t* z_masks,
                         const int32_t* y_counts, const double* coeffs, const int32_t* obs_index, int64_t n_terms,
                         int64_t n_obs, int64_t n_items, int64_t n_slots);
int qfvm_batch_run(qfvm_batch* batch, int32_t mode, const double* values, const double* weights, double* expvals,
                   double* grads);
/* As qfvm_batch_run, plus the device time of the run (uploads, kernels and
 * downloads) from CUDA events on the batch's stream. */
int qfvm_batch_run_timed(qfvm_batch* batch, int32_t mode, const double* values, const double* weights,
                         double* expvals, double* grads, float* device_ms);
/* Sizes of the value / result arrays; per mode: kernels one run launches and
 * whether its graph has been captured. */
int qfvm_batch_info(const qfvm_batch* batch, int64_t* n_groups, int64_t* n_values, int64_t* n_expvals,
                    int64_t* n_grads, int64_t kernels_per_run[2], int32_t graph_ready[2]);
int qfvm_batch_destroy(qfvm_batch* batch);

/* Host-only planning (no device needed): build the fused schedule and copy
 * its records out, for inspection and for testing the fuser.  Records are the
 * engine's internal layouts: 56-byte pass, 100-byte step and 48-byte op
 * records; counts[] receives passes, steps, ops, coefficients. */
int qfvm_plan_host_build(int32_t num_qubits, int32_t precision, const qfvm_op* ops, int64_t n_ops,
                         const double* matpool, int64_t matpool_len, int32_t tile_qubits, int32_t reg_qubits,
                         qfvm_plan** out);
/* The reverse sweep qfvm_adjoint runs (probes and inverse gates), host only. */
int qfvm_plan_host_build_adjoint(int32_t num_qubits, int32_t precision, const qfvm_op* ops, int64_t n_ops,
                                 const double* matpool, int64_t matpool_len, qfvm_plan** out);
/* The forward plan (adjoint == 0) or reverse sweep (adjoint != 0) that a
 * batch group runs, host only: value-dependent fast paths of slotted gates are
 * dropped and the pool blocks a run rewrites per item are recorded. */
int qfvm_plan_host_build_batched(int32_t num_qubits, int32_t precision, const qfvm_op* ops, int64_t n_ops,
                                 const double* matpool, int64_t matpool_len, int32_t adjoint, qfvm_plan** out);
/* Bind records of a plan: 4 int32 each (pool offset, gate kind, angle sign,
 * slot); records may be NULL to query the count. */
int qfvm_plan_host_binds(const qfvm_plan* plan, int64_t* count, int32_t* records);
/* Parameter slot of each probe of an adjoint plan, in probe-id order. */
int qfvm_plan_host_probe_slots(const qfvm_plan* plan, int32_t* slots);
int qfvm_plan_host_counts(const qfvm_plan* plan, int64_t counts[4], int32_t shape[3]);
int qfvm_plan_host_copy(const qfvm_plan* plan, void* passes, void* steps, void* kops, double* coef);

/* ---------------------------------------------------------------------------
 * Circuit-specialised tile passes.  Tile passes of complex128 (FP64 and
 * double-single) and complex64 plans are, by default, emitted as
 * straight-line PTX for sm_103a (every register round unrolled with its
 * targets, controls and coefficient offsets as constants) and compiled once
 * per distinct pass (two-target dense gates as shared-memory steps of the
 * pass); whole-state passes and k-target gates run the hand-written kernels.
 * The environment variable QFVM_JIT=0 turns specialisation off at start-up.
 * ------------------------------------------------------------------------- */
/* enabled: 0/1; nb_*: tile buffers (1 or 2) of one-state / two-state passes;
 * minb_*: minimum resident CTAs per SM the register budget is set for
 * (0 = automatic).  Applies to plans prepared afterwards. */
int qfvm_jit_configure(int32_t enabled, int32_t nb_one, int32_t minb_one, int32_t nb_two, int32_t minb_two);
int qfvm_jit_get_config(int32_t config[5]);
/* PTX the generator emits for pass `pass` of a plan (host only; nstates 1 =
 * forward pass, 2 = reverse-sweep pass with probes).  *len receives the text
 * length (without the terminating zero); text may be NULL to query it.
 * QFVM_ERR_UNSUPPORTED when the pass runs interpreted. */
int qfvm_jit_pass_ptx(const qfvm_plan* plan, int32_t pass, int32_t nstates, char* text, int64_t capacity,
                      int64_t* len);
/* Compiles that PTX for sm_103a on the host (no device needed) and writes the
 * compiler's info log (registers, spills) or error to info. */
int qfvm_jit_pass_compile(const qfvm_plan* plan, int32_t pass, int32_t nstates, char* info, int64_t capacity);
/* Passes of a device plan that run specialised (after its first run). */
int qfvm_jit_plan_passes(const qfvm_plan* plan, int32_t nstates, int64_t* count);

#ifdef __cplusplus
}
#endif
#endif /* QFVM_GB300_H */
