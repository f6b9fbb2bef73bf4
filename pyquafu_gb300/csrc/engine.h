// Internal declarations of the GB300 statevector engine (host planner + kernels).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "qfvm_gb300.h"

namespace qsv {

// ---------------------------------------------------------------------------
// Classified gates ("gops"): every circuit gate becomes one of these kinds,
// expressed on global qubit indices.  Coefficients are FP64, computed on the
// host exactly as the reference builds its matrices (statevector.hpp:340-437).
// ---------------------------------------------------------------------------
enum GKind : uint8_t {
    K_DENSE = 1,  // 2x2 complex on t0 (8 coefs: m00 re,im, m01, m10, m11)
    K_REAL = 2,   // 2x2 real on t0 (4 coefs)
    K_RX = 3,     // [[c, -i s], [-i s, c]] on t0 (coefs c, s)
    K_DIAG = 4,   // amp *= d[parity(idx & pmask)] (coefs d0 re,im, d1 re,im)
    K_X = 5,      // swap the t0 pair
    K_Y = 6,      // [[0,-i],[i,0]] on t0
    K_SWAP = 7,   // exchange qubits t0 and t1
    K_DENSE2 = 8, // 4x4 complex on (t0 = bit 0, t1 = bit 1), 32 coefs
    K_DENSEK = 9, // 2^k x 2^k complex on tk[0..k-1] (bit j = tk[j]), 2*4^k coefs
    K_PROBE = 10, // adjoint sweep: accumulate Im<lam| Q |psi> (reads both states, changes neither)
    K_HAD = 11,   // sqrt(2) H = [[1, 1], [1, -1]] on t0, no coefficients (see unnormalize_hadamards)
    K_DIAGR = 12  // register round only: amp j of the thread's 2^k registers *= d[j] (2 * 2^k coefs);
                  // a 3-bit code per entry (DIAGR_* below) in cthr / pthr (diagr_code), k <= 5
};
enum : uint8_t { DIAGR_GENERAL = 0, DIAGR_ONE = 1, DIAGR_NEG1 = 2, DIAGR_I = 3, DIAGR_NEGI = 4 };
#if defined(__CUDACC__)
#define QSV_HD __host__ __device__
#else
#define QSV_HD
#endif

// DIAG flags
enum : uint8_t {
    F_D0_ONE = 1,  // d0 == 1 exactly: parity-0 amplitudes are untouched
    F_D1_SPEC = 2,  // d1 is exactly -1, i or -i (see SP_*), applied without arithmetic
    F_UNIFORM = 4,  // register round: no parity / control bit in the registers
    F_ONEBIT = 8,   // register round: one parity bit in the registers (t0), no register control
    F_TCTRL = 16,   // register round: cthr != 0 (a control on a thread bit)
    F_TPAR = 32     // register round: pthr != 0 (a parity or Z bit on a thread bit)
};
enum : uint8_t { SP_NEG1 = 1, SP_I = 2, SP_NEGI = 3 };

constexpr int MAXK = 6;  // largest dense target count held in a thread's registers (k_globalop, k_small)
// Dense gates on MAXK+1 .. MAX_DENSE_TARGETS targets run one CTA per group of
// 2^k amplitudes in shared memory (k_globalop_wide); their targets are
// ascending (the matrix is relabelled on the host) and travel as the mask
// KOp::pthr.
constexpr int MAX_DENSE_TARGETS = 12;

struct GOp {
    GKind kind;
    uint8_t flags = 0, special = 0;
    int t0 = -1, t1 = -1;
    int k = 0;
    int tk[MAX_DENSE_TARGETS] = {0};
    uint64_t cmask = 0;  // control qubits (all must be 1)
    uint64_t pmask = 0;  // DIAG parity qubits
    std::vector<double> coef;
    int src = -1;   // index of the circuit op it came from
    int slot = -1;  // parameter slot (batched / adjoint runs)
    // Generator of a parameterised gate: dG/dtheta = -i/2 Q G with
    // Q = scale * proj(gcmask) * (Pauli with flip mask gx, phase mask gz, gny Y factors).
    bool has_gen = false;
    uint64_t gx = 0, gz = 0, gcmask = 0;
    int gny = 0;
    double gscale = 1.0;
    // K_PROBE: xmask = flip bits, pmask = Z bits, cmask = projector bits,
    // special = number of Y factors, coef = {scale}
    uint64_t xmask = 0;
    // Batched runs: a slotted RX/RY/RZ/P/CP/RZZ is re-bound per item from its
    // slot value; bkind is the circuit op kind (QFVM_OP_*), bsign = -1 for the
    // inverse gate of a reverse sweep (angle -theta).
    uint8_t bkind = 0;
    int8_t bsign = 1;
};

// One coefficient block of the pool that a batched run rewrites per item:
// coef[off ..] = coefficients of gate kind `kind` at angle sign * value[slot].
struct Bind {
    uint32_t off;
    uint8_t kind;
    int8_t sign;
    uint16_t pad;
    int32_t slot;
};
static_assert(sizeof(Bind) == 12, "Bind layout");

// ---------------------------------------------------------------------------
// Device-side plan records (POD, uploaded once per plan)
// ---------------------------------------------------------------------------
// One operation as executed by a kernel.  For register rounds the target
// fields are register-bit indices and creg/preg are masks over register-index
// bits; cthr/pthr are masks over global index bits evaluated against the
// thread's base index.  For whole-state kernels all masks are global.
struct KOp {
    uint8_t kind, flags, special, k;
    uint8_t t0, t1;
    uint16_t probe;  // K_PROBE: index of the probe within its pass
    uint32_t creg, preg;
    uint64_t cthr, pthr;
    uint32_t coef;  // offset into the coefficient pool (in reals)
    uint8_t tk[MAXK];
    uint8_t pad2[2];
    uint32_t xreg;  // K_PROBE: flip mask over register bits (or over global bits in whole-state passes)
};
static_assert(sizeof(KOp) == 48, "KOp layout");

// Code of register entry j of a K_DIAGR op: entries 0..20 in cthr, 21..31
// in pthr, 3 bits each (a K_DIAGR op has no controls or parities).
constexpr int DIAGR_LOW = 21;
QSV_HD inline int diagr_code(const KOp& o, int j) {
    return j < DIAGR_LOW ? static_cast<int>((o.cthr >> (3 * j)) & 7)
                         : static_cast<int>((o.pthr >> (3 * (j - DIAGR_LOW))) & 7);
}

constexpr int MAX_TILE = 14;

// ---------------------------------------------------------------------------
// Shared-memory layout of a tile pass.  Element s of a tile (bit k of s is
// tile-local position k) sits at element offset
//     tile_off(s) = s + u * ((s >> 5) + (s >> 8) + (s >> 11)),
// u = 16 bytes / element size.  The tile's low TILE_RUN_BITS positions are the
// contiguous qubits 0..4, so each run of 32 amplitudes is one contiguous
// piece of global memory and stays contiguous here, starting 16-byte aligned:
// a run moves with one bulk copy.  Run r starts u * (r + r/8 + r/64) elements
// after its unpadded place.  The shifted terms of disjoint bit sets do not
// overlap, so tile_off(a | b) = tile_off(a) + tile_off(b) for a & b == 0: an
// address is a thread's base plus per-bit constants tile_weight(p).
// Within a 128-byte wavefront, position p < 3 (16-byte elements; p < 4 for
// 8-byte ones) lands on slot bit p, positions 3..4 (4) on none, and position
// 5 + j on slot bit j mod 3 (plus 1 for 8-byte elements): lanes whose
// positions land on distinct slot bits hit distinct bank groups
// (tile_slot_bit).
// ---------------------------------------------------------------------------
constexpr int TILE_RUN_BITS = 5;
QSV_HD constexpr uint32_t tile_off(uint32_t s, uint32_t u) { return s + u * ((s >> 5) + (s >> 8) + (s >> 11)); }
QSV_HD constexpr uint32_t tile_weight(int p, uint32_t u) { return tile_off(1u << p, u); }
// elements of one tile buffer (a multiple of 128 bytes)
QSV_HD constexpr uint32_t tile_elems(int T, int elem_bytes) {
    const uint32_t u = 16u / static_cast<uint32_t>(elem_bytes);
    const uint32_t per128 = 128u / static_cast<uint32_t>(elem_bytes);
    const uint32_t e = tile_off((1u << T) - 1, u) + 1;
    return (e + per128 - 1) / per128 * per128;
}
// Slot bit that tile position p selects for accesses of `access` bytes to
// elements of `elem_bytes` (-1: none): bit k of (byte offset / access) mod
// (128 / access).  p = 0 with 16-byte accesses to 8-byte elements (pairs)
// is not an access position and gives -1.
inline int tile_slot_bit(int p, int elem_bytes, int access) {
    const uint32_t u = 16u / static_cast<uint32_t>(elem_bytes);
    const uint32_t b = tile_weight(p, u) * static_cast<uint32_t>(elem_bytes);
    if (b % static_cast<uint32_t>(access)) return -1;
    const uint32_t c = (b / static_cast<uint32_t>(access)) % (128u / static_cast<uint32_t>(access));
    if (c == 0 || (c & (c - 1))) return -1;
    int k = 0;
    while ((1u << k) != c) ++k;
    return k;
}

// A fused pass over the state: tiles of T qubits, the low L of which are the
// contiguous qubits 0..L-1; tq[] lists the tile's global qubits ascending.
struct PassDesc {
    int32_t type;  // PASS_*
    int32_t T, L, H;
    int32_t step_begin, step_count;
    int32_t op_begin, op_count;  // PASS_SMALL / PASS_GLOBALOP: ops applied
    int32_t probe_base, nprobe;  // adjoint sweeps: probes evaluated in this pass
    uint8_t tq[16];
};
enum : int32_t { PASS_TILE = 0, PASS_SMALL = 1, PASS_GLOBALOP = 2 };
static_assert(sizeof(PassDesc) == 56, "PassDesc layout");
constexpr int MAX_PASS_PROBES = 64;

// One register round inside a tile pass: register bit k holds tile-local
// position rpos[k]; thread-index bit k selects tile-local position tpos[k].
// rsw / tsw are the element offsets those positions add in the tile layout
// (tile_weight): a thread's base offset is the sum of the tsw of its set
// index bits, register j adds the rsw of j's set bits.
struct StepDesc {
    int32_t type;  // STEP_*
    int32_t op_begin, op_count;
    uint8_t rpos[8];
    uint8_t tpos[16];
    uint8_t tglob[16];  // global qubit of thread bit k (= tq[tpos[k]])
    uint16_t rsw[8];
    uint16_t tsw[16];
};
enum : int32_t { STEP_ROUND = 0, STEP_SMEM = 1 };
static_assert(sizeof(StepDesc) == 100, "StepDesc layout");

struct PlanStats {
    int64_t passes = 0, rounds = 0, gates = 0;
    double pass_bytes = 0, gate_bytes = 0;
};

// Host-side plan (built by plan.cpp, executed by kernels.cu).
struct HostPlan {
    int n = 0, precision = QFVM_C128, T = 0, R = 0, L = 0;
    std::vector<int> probe_slot;  // adjoint sweeps: parameter slot of every probe, by probe id
    int arith = QFVM_C128;  // kernel arithmetic: QFVM_C128 (FP64), QFVM_C64 (FP32), QFVM_C128_DS
    std::vector<PassDesc> passes;
    std::vector<StepDesc> steps;
    std::vector<KOp> ops;
    std::vector<double> coef;  // FP64 coefficient pool
    std::vector<Bind> binds;   // pool blocks that depend on a slot value
    PlanStats stats;
};

int amp_bytes(int precision);
int small_max_qubits(int precision);
void default_shape(int n, int precision, int* T, int* R);

// plan.cpp
// Classify circuit ops into gops; returns a message on invalid input.
bool classify(int n, const qfvm_op* ops, int64_t n_ops, const double* matpool, int64_t matpool_len,
              std::vector<GOp>* out, std::string* err);
bool build_plan(int n, int precision, const std::vector<GOp>& gops, int T, int R, HostPlan* plan,
                std::string* err);
// Reverse sweep of the adjoint method: for each gate from last to first, a
// probe of its generator (if it carries a parameter slot) and its inverse.
bool build_adjoint_sweep(const std::vector<GOp>& gops, std::vector<GOp>* out, std::string* err);
GOp gop_dagger(const GOp& g);
// Batched runs: drop the fast paths that depend on a bindable gate's value
// (special phases, unit first diagonal entry of RZ/RZZ) so one plan serves
// every value.  Returns false (with a message) for a slotted gate that
// cannot be re-bound on the device.
bool unfix_bound(std::vector<GOp>* gops, std::string* err);
// Plain simulation plans: uncontrolled Hadamards become K_HAD (additions only)
// and their 1/sqrt(2) factors, a global scalar, are folded into the
// coefficients of other uncontrolled dense or diagonal gates of the list.
// Hadamards whose factor finds no such gate stay as they are.
void unnormalize_hadamards(std::vector<GOp>* gops);
// Plain simulation plans: an uncontrolled one-qubit diagonal, RX or X gate
// is merged into the previous gate of the same class on its qubit when every
// gate between commutes with it (diagonals pass diagonals and gates that use
// the qubit only as a control; X-type gates pass X / RX on the same target):
// d.d' -> one diagonal, rx(a) rx(b) -> rx(a + b), X X -> nothing.
void fuse_single_qubit(std::vector<GOp>* gops);
// Plain simulation plans: inside every register round of at most 4 register
// qubits, diagonal ops whose parity and controls are all register bits are
// multiplied into one per-register-entry phase table (K_DIAGR), applied
// where the first op that acts non-diagonally on one of the table's bits
// comes (or at the round's end).  The merged ops commute with everything
// between their places and that point.  Entries that come out exactly 1,
// -1, i or -i are coded so the kernels apply them without arithmetic.
void merge_round_diagonals(HostPlan* plan);
// Coefficients of a bindable gate kind at angle th (2 or 4 doubles).
int bind_coef(int kind, double th, double* c);
// Gate-equivalent bytes of one gop: 2 * bytes per amplitude * amplitudes it
// must touch.
double gop_bytes(const GOp& g, int n, int precision);

}  // namespace qsv
