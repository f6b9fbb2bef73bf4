// Host planner: classify circuit gates and fuse them into tile passes.
//
// Classification follows the reference's dispatch (src/qfvm/simulator.hpp:
// 12-113) and matrix construction (src/qfvm/statevector.hpp:340-437); the
// fuser is this engine's own: gates are grouped into passes over tiles of T
// qubits (the low L qubits are always in the tile so that HBM accesses are
// contiguous runs), and inside a pass into register rounds of R qubits.
// Diagonal gates and controls need no tile membership: they are evaluated
// from each amplitude's global index, so only the targets of non-diagonal
// gates constrain the schedule.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <set>

#include "engine.h"

namespace qsv {

int amp_bytes(int precision) { return precision == QFVM_C64 ? 8 : 16; }

// Largest state handled by the whole-state (single CTA, shared memory) kernel.
int small_max_qubits(int precision) { return precision == QFVM_C64 ? 14 : 13; }

// Built-in shapes (the autotuner's choices on GB300 for the random-layer and
// hardware-efficient workloads; a tuned table entry overrides them).
void default_shape(int n, int precision, int* T, int* R) {
    if (precision == QFVM_C64) {
        *T = 13;
        *R = 5;
    } else if (precision == QFVM_C128_DS) {
        *T = 12;
        *R = 3;
    } else {
        *T = 11;
        *R = 4;
    }
    (void)n;
}

namespace {

using cd = std::complex<double>;

void set_diag(GOp& g, cd d0, cd d1) {
    g.kind = K_DIAG;
    g.coef = {d0.real(), d0.imag(), d1.real(), d1.imag()};
    if (d0 == cd(1.0, 0.0)) {
        g.flags |= F_D0_ONE;
        if (d1 == cd(-1.0, 0.0)) {
            g.flags |= F_D1_SPEC;
            g.special = SP_NEG1;
        } else if (d1 == cd(0.0, 1.0)) {
            g.flags |= F_D1_SPEC;
            g.special = SP_I;
        } else if (d1 == cd(0.0, -1.0)) {
            g.flags |= F_D1_SPEC;
            g.special = SP_NEGI;
        }
    }
}

bool is_zero(cd z) { return z.real() == 0.0 && z.imag() == 0.0; }

}  // namespace

bool classify(int n, const qfvm_op* ops, int64_t n_ops, const double* matpool, int64_t matpool_len,
              std::vector<GOp>* out, std::string* err) {
    out->clear();
    out->reserve(static_cast<size_t>(n_ops));
    const double PI_ = 3.14159265358979323846;
    for (int64_t i = 0; i < n_ops; ++i) {
        const qfvm_op& o = ops[i];
        const int nq = o.nqubits;
        if (nq < 1 || nq > QFVM_MAX_OP_QUBITS) {
            *err = "op " + std::to_string(i) + ": bad qubit count " + std::to_string(nq);
            return false;
        }
        uint64_t seen = 0;
        for (int j = 0; j < nq; ++j) {
            int q = o.qubits[j];
            if (q < 0 || q >= n) {
                *err = "op " + std::to_string(i) + ": qubit " + std::to_string(q) + " outside a " +
                       std::to_string(n) + "-qubit state";
                return false;
            }
            if (seen & (1ULL << q)) {
                *err = "op " + std::to_string(i) + ": repeated qubit " + std::to_string(q);
                return false;
            }
            seen |= 1ULL << q;
        }
        for (int j = 0; j < 4; ++j) {
            if (!std::isfinite(o.params[j])) {
                *err = "op " + std::to_string(i) + ": non-finite parameter";
                return false;
            }
        }
        GOp g;
        g.src = static_cast<int>(i);
        g.slot = o.slot;
        if (o.slot >= 0 && (o.kind == QFVM_OP_RX || o.kind == QFVM_OP_RY || o.kind == QFVM_OP_RZ ||
                            o.kind == QFVM_OP_P || o.kind == QFVM_OP_CP || o.kind == QFVM_OP_RZZ))
            g.bkind = static_cast<uint8_t>(o.kind);
        const int* q = o.qubits;
        auto need = [&](int k) {
            if (nq < k) {
                *err = "op " + std::to_string(i) + ": gate kind " + std::to_string(o.kind) + " needs " +
                       std::to_string(k) + " qubits";
                return false;
            }
            return true;
        };
        const double th = o.params[0];
        switch (o.kind) {
            case QFVM_OP_X:
                g.kind = K_X;
                g.t0 = q[0];
                break;
            case QFVM_OP_Y:
                g.kind = K_Y;
                g.t0 = q[0];
                break;
            case QFVM_OP_Z:
                g.pmask = 1ULL << q[0];
                set_diag(g, 1.0, -1.0);
                break;
            case QFVM_OP_H: {
                const double s = 1. / std::sqrt(2.);
                g.kind = K_REAL;
                g.t0 = q[0];
                g.coef = {s, s, s, -s};
                break;
            }
            case QFVM_OP_S:
                g.pmask = 1ULL << q[0];
                set_diag(g, 1.0, cd(0, 1));
                break;
            case QFVM_OP_SDG:
                g.pmask = 1ULL << q[0];
                set_diag(g, 1.0, cd(0, -1));
                break;
            case QFVM_OP_T:
            case QFVM_OP_TDG: {
                const double a = (o.kind == QFVM_OP_T ? 1.0 : -1.0) * PI_ / 4.;
                g.pmask = 1ULL << q[0];
                set_diag(g, 1.0, cd(std::cos(a), std::sin(a)));
                break;
            }
            case QFVM_OP_P:
                g.pmask = 1ULL << q[0];
                set_diag(g, 1.0, cd(std::cos(th), std::sin(th)));
                break;
            case QFVM_OP_RX:
                g.kind = K_RX;
                g.t0 = q[0];
                g.coef = {std::cos(th / 2), std::sin(th / 2)};
                break;
            case QFVM_OP_RY: {
                const double c = std::cos(th / 2), s = std::sin(th / 2);
                g.kind = K_REAL;
                g.t0 = q[0];
                g.coef = {c, -s, s, c};
                break;
            }
            case QFVM_OP_RZ: {
                const double h = th / 2.;
                g.pmask = 1ULL << q[0];
                set_diag(g, cd(std::cos(-h), std::sin(-h)), cd(std::cos(h), std::sin(h)));
                break;
            }
            case QFVM_OP_CX:
                if (!need(2)) return false;
                g.kind = K_X;
                g.cmask = 1ULL << q[0];
                g.t0 = q[1];
                break;
            case QFVM_OP_CZ:
                if (!need(2)) return false;
                g.cmask = 1ULL << q[0];
                g.pmask = 1ULL << q[1];
                set_diag(g, 1.0, -1.0);
                break;
            case QFVM_OP_CP:
                if (!need(2)) return false;
                g.cmask = 1ULL << q[0];
                g.pmask = 1ULL << q[1];
                set_diag(g, 1.0, cd(std::cos(th), std::sin(th)));
                break;
            case QFVM_OP_CCX:
                if (!need(3)) return false;
                g.kind = K_X;
                g.cmask = (1ULL << q[0]) | (1ULL << q[1]);
                g.t0 = q[2];
                break;
            case QFVM_OP_RZZ: {
                // simulator.hpp:90-94 applies cx . rz . cx: a phase by the parity of the two qubits.
                if (!need(2)) return false;
                const double h = th / 2.;
                g.pmask = (1ULL << q[0]) | (1ULL << q[1]);
                set_diag(g, cd(std::cos(-h), std::sin(-h)), cd(std::cos(h), std::sin(h)));
                break;
            }
            case QFVM_OP_MATRIX: {
                const int nc = o.ncontrols;
                const int k = nq - nc;
                if (nc < 0 || k < 1) {
                    *err = "op " + std::to_string(i) + ": matrix gate without a target";
                    return false;
                }
                if (k > MAX_DENSE_TARGETS) {
                    *err = "op " + std::to_string(i) + ": " + std::to_string(k) +
                           "-target matrix gates are not supported (at most " + std::to_string(MAX_DENSE_TARGETS) +
                           " targets)";
                    return false;
                }
                const int64_t dim = 1LL << k;
                if (o.mat_dim != dim || o.mat_offset < 0 || o.mat_offset + dim * dim > matpool_len) {
                    *err = "op " + std::to_string(i) + ": matrix does not match its target count";
                    return false;
                }
                const cd* m = reinterpret_cast<const cd*>(matpool) + o.mat_offset;
                for (int j = 0; j < nc; ++j) g.cmask |= 1ULL << q[j];
                for (int64_t j = 0; j < dim * dim; ++j) {
                    if (!std::isfinite(m[j].real()) || !std::isfinite(m[j].imag())) {
                        *err = "op " + std::to_string(i) + ": non-finite matrix entry";
                        return false;
                    }
                }
                if (k == 1) {
                    const int t = q[nc];
                    g.t0 = t;
                    if (is_zero(m[1]) && is_zero(m[2])) {
                        g.pmask = 1ULL << t;
                        set_diag(g, m[0], m[3]);
                    } else if (is_zero(m[0]) && is_zero(m[3]) && m[1] == cd(1, 0) && m[2] == cd(1, 0)) {
                        g.kind = K_X;
                    } else if (m[0].imag() == 0 && m[1].imag() == 0 && m[2].imag() == 0 && m[3].imag() == 0) {
                        g.kind = K_REAL;
                        g.coef = {m[0].real(), m[1].real(), m[2].real(), m[3].real()};
                    } else {
                        g.kind = K_DENSE;
                        g.coef.resize(8);
                        for (int j = 0; j < 4; ++j) {
                            g.coef[2 * j] = m[j].real();
                            g.coef[2 * j + 1] = m[j].imag();
                        }
                    }
                } else if (k == 2) {
                    g.t0 = q[nc];
                    g.t1 = q[nc + 1];
                    bool swap = true;
                    for (int r = 0; r < 4 && swap; ++r)
                        for (int c = 0; c < 4; ++c) {
                            int want = (r == 0 && c == 0) || (r == 3 && c == 3) || (r == 1 && c == 2) ||
                                       (r == 2 && c == 1);
                            if (m[r * 4 + c] != cd(want ? 1.0 : 0.0, 0.0)) {
                                swap = false;
                                break;
                            }
                        }
                    if (swap) {
                        g.kind = K_SWAP;
                    } else {
                        g.kind = K_DENSE2;
                        g.coef.resize(32);
                        for (int j = 0; j < 16; ++j) {
                            g.coef[2 * j] = m[j].real();
                            g.coef[2 * j + 1] = m[j].imag();
                        }
                    }
                } else if (k <= MAXK) {
                    g.kind = K_DENSEK;
                    g.k = k;
                    for (int j = 0; j < k; ++j) g.tk[j] = q[nc + j];
                    g.coef.resize(static_cast<size_t>(2 * dim * dim));
                    for (int64_t j = 0; j < dim * dim; ++j) {
                        g.coef[2 * j] = m[j].real();
                        g.coef[2 * j + 1] = m[j].imag();
                    }
                } else {
                    // wide gate: targets in ascending order, the matrix's index
                    // bits relabelled to match (a permutation of entries, exact)
                    g.kind = K_DENSEK;
                    g.k = k;
                    int ord[MAX_DENSE_TARGETS];
                    for (int j = 0; j < k; ++j) ord[j] = j;
                    std::sort(ord, ord + k, [&](int a, int b) { return q[nc + a] < q[nc + b]; });
                    for (int j = 0; j < k; ++j) g.tk[j] = q[nc + ord[j]];
                    std::vector<int64_t> old_of(static_cast<size_t>(dim));
                    for (int64_t v = 0; v < dim; ++v) {
                        int64_t o2 = 0;
                        for (int j = 0; j < k; ++j)
                            if ((v >> j) & 1) o2 |= int64_t{1} << ord[j];
                        old_of[static_cast<size_t>(v)] = o2;
                    }
                    g.coef.resize(static_cast<size_t>(2 * dim * dim));
                    for (int64_t r = 0; r < dim; ++r)
                        for (int64_t c = 0; c < dim; ++c) {
                            const cd e = m[old_of[static_cast<size_t>(r)] * dim + old_of[static_cast<size_t>(c)]];
                            g.coef[static_cast<size_t>(2 * (r * dim + c))] = e.real();
                            g.coef[static_cast<size_t>(2 * (r * dim + c) + 1)] = e.imag();
                        }
                }
                break;
            }
            default:
                *err = "op " + std::to_string(i) + ": kind " + std::to_string(o.kind) +
                       " is not a gate this entry point applies";
                return false;
        }
        if (g.kind == K_X || g.kind == K_Y || g.kind == K_REAL || g.kind == K_RX || g.kind == K_DENSE) {
            if (g.cmask & (1ULL << g.t0)) {
                *err = "op " + std::to_string(i) + ": target is also a control";
                return false;
            }
        }
        // generator of a parameterised gate: dG/dtheta = -i/2 Q G
        // (rotations exp(-i theta Q / 2); phase gates diag(1, e^{i l}) give Q = -2 proj)
        {
            const uint64_t b0 = 1ULL << q[0];
            switch (o.kind) {
                case QFVM_OP_RX: g.has_gen = true; g.gx = b0; break;
                case QFVM_OP_RY: g.has_gen = true; g.gx = b0; g.gz = b0; g.gny = 1; break;
                case QFVM_OP_RZ: g.has_gen = true; g.gz = b0; break;
                case QFVM_OP_RZZ: g.has_gen = true; g.gz = b0 | (1ULL << q[1]); break;
                case QFVM_OP_P: g.has_gen = true; g.gcmask = b0; g.gscale = -2.0; break;
                case QFVM_OP_CP: g.has_gen = true; g.gcmask = b0 | (1ULL << q[1]); g.gscale = -2.0; break;
                case QFVM_OP_MATRIX: {
                    uint64_t tm = 0, cm = 0;
                    for (int j = 0; j < o.ncontrols; ++j) cm |= 1ULL << q[j];
                    for (int j = o.ncontrols; j < nq; ++j) tm |= 1ULL << q[j];
                    const int nt = nq - o.ncontrols;
                    switch (o.gen) {
                        case QFVM_GEN_X: g.has_gen = true; g.gx = tm; g.gcmask = cm; break;
                        case QFVM_GEN_Y: g.has_gen = true; g.gx = tm; g.gz = tm; g.gny = nt; g.gcmask = cm; break;
                        case QFVM_GEN_Z: g.has_gen = true; g.gz = tm; g.gcmask = cm; break;
                        case QFVM_GEN_PHASE: g.has_gen = true; g.gcmask = tm | cm; g.gscale = -2.0; break;
                        default: break;
                    }
                    break;
                }
                default: break;
            }
        }
        out->push_back(std::move(g));
    }
    return true;
}

double gop_bytes(const GOp& g, int n, int precision) {
    const double N = std::ldexp(1.0, n);
    const int nc = __builtin_popcountll(g.cmask);
    double amps = N / std::ldexp(1.0, nc);
    switch (g.kind) {
        case K_DIAG:
            if (g.flags & F_D0_ONE) amps *= 0.5;
            break;
        case K_SWAP:
            amps *= 0.5;
            break;
        default:
            break;
    }
    return 2.0 * amp_bytes(precision) * amps;
}

namespace {

// Qubit actions for commutation: two gates commute if on every shared qubit
// both act diagonally (controls, phases) or both act as X (targets of X/CX).
enum Act : uint8_t { A_Z = 1, A_X = 2, A_G = 4 };

void gop_actions(const GOp& g, std::vector<std::pair<int, uint8_t>>* acts) {
    acts->clear();
    for (int q = 0; q < 64; ++q) {
        if (g.cmask & (1ULL << q)) acts->push_back({q, A_Z});
        if (g.pmask & (1ULL << q)) acts->push_back({q, A_Z});
    }
    switch (g.kind) {
        case K_X: acts->push_back({g.t0, A_X}); break;
        case K_DIAG: break;
        case K_SWAP:
        case K_DENSE2:
            acts->push_back({g.t0, A_G});
            acts->push_back({g.t1, A_G});
            break;
        case K_DENSEK:
            for (int j = 0; j < g.k; ++j) acts->push_back({g.tk[j], A_G});
            break;
        case K_PROBE:
            // a probe of Q commutes with a gate that commutes with Q: Z bits and
            // the projector act diagonally, pure flip bits as X, Y bits as both
            for (int q = 0; q < 64; ++q) {
                const uint64_t b = 1ULL << q;
                if (g.xmask & b) acts->push_back({q, (g.pmask & b) ? A_G : A_X});
            }
            break;
        default: acts->push_back({g.t0, A_G}); break;
    }
}

bool act_conflict(uint8_t blocked, uint8_t a) {
    if (!blocked) return false;
    if (a == A_Z) return (blocked & (A_X | A_G)) != 0;
    if (a == A_X) return (blocked & (A_Z | A_G)) != 0;
    return true;
}

void gop_targets(const GOp& g, std::vector<int>* t) {
    t->clear();
    switch (g.kind) {
        case K_DIAG: break;
        case K_SWAP:
        case K_DENSE2:
            t->push_back(g.t0);
            t->push_back(g.t1);
            break;
        case K_DENSEK:
            for (int j = 0; j < g.k; ++j) t->push_back(g.tk[j]);
            break;
        case K_PROBE:  // flipped qubits pair amplitudes: they must be register bits
            for (int q = 0; q < 64; ++q)
                if (g.xmask & (1ULL << q)) t->push_back(q);
            break;
        default: t->push_back(g.t0); break;
    }
}

// Copy a gop's coefficients into the pool and return the offset.
uint32_t push_coef(HostPlan* p, const GOp& g) {
    // every block starts 4-aligned (the kernels read coefficients four at a
    // time with 16-byte loads); the padding stays zero
    while (p->coef.size() % 4) p->coef.push_back(0.0);
    uint32_t off = static_cast<uint32_t>(p->coef.size());
    p->coef.insert(p->coef.end(), g.coef.begin(), g.coef.end());
    if (g.bkind != 0 && g.slot >= 0 && g.kind != K_PROBE)
        p->binds.push_back(Bind{off, g.bkind, g.bsign, 0, g.slot});
    return off;
}

// Whole-state op record: all masks over global index bits.
KOp global_kop(HostPlan* p, const GOp& g) {
    KOp k;
    std::memset(&k, 0, sizeof(k));
    k.kind = g.kind;
    k.flags = g.flags;
    k.special = g.special;
    k.t0 = static_cast<uint8_t>(g.t0 < 0 ? 0 : g.t0);
    k.t1 = static_cast<uint8_t>(g.t1 < 0 ? 0 : g.t1);
    k.k = static_cast<uint8_t>(g.k);
    for (int j = 0; j < g.k && j < MAXK; ++j) k.tk[j] = static_cast<uint8_t>(g.tk[j]);
    k.cthr = g.cmask;
    k.pthr = g.pmask;
    if (g.kind == K_DENSEK && g.k > MAXK) {
        k.pthr = 0;
        for (int j = 0; j < g.k; ++j) k.pthr |= 1ULL << g.tk[j];  // ascending targets as a mask
    }
    if (g.kind == K_PROBE) {
        k.xreg = static_cast<uint32_t>(g.xmask);  // whole-state kernels: global flip bits (n <= 14)
        k.probe = static_cast<uint16_t>(p->probe_slot.size());
        p->probe_slot.push_back(g.slot);
    }
    k.coef = push_coef(p, g);
    return k;
}

// Thread-bit order for a register round: the first lanes get positions that
// land on distinct slot bits of the tile layout (tile_slot_bit), so each
// wavefront of the round's shared-memory accesses (`access` bytes per lane)
// covers distinct bank groups.
void order_thread_bits(std::vector<int>& free_pos, int elem_bytes, int access) {
    const int nslot = access == 16 ? 3 : 4;  // 128 / access = 2^nslot slots per wavefront
    std::vector<int> head, rest;
    std::vector<bool> used(free_pos.size(), false);
    for (int r = 0; r < nslot; ++r) {
        for (size_t i = 0; i < free_pos.size(); ++i) {
            if (!used[i] && tile_slot_bit(free_pos[i], elem_bytes, access) == r) {
                head.push_back(free_pos[i]);
                used[i] = true;
                break;
            }
        }
    }
    for (size_t i = 0; i < free_pos.size(); ++i)
        if (!used[i]) rest.push_back(free_pos[i]);
    free_pos = head;
    free_pos.insert(free_pos.end(), rest.begin(), rest.end());
}

// Order in which free tile positions pad a round's register set: positions
// that select no slot bit first, then ascending, position 0 last (for 8-byte
// elements it is the only position on slot bit 0).
std::vector<int> register_pad_order(int T, int elem_bytes) {
    std::vector<int> o;
    for (int p = 1; p < T; ++p)
        if (tile_slot_bit(p, elem_bytes, elem_bytes) < 0) o.push_back(p);
    for (int p = 1; p < T; ++p)
        if (tile_slot_bit(p, elem_bytes, elem_bytes) >= 0) o.push_back(p);
    o.push_back(0);
    return o;
}

}  // namespace

bool build_plan(int n, int precision, const std::vector<GOp>& gops, int T, int R, HostPlan* plan,
                std::string* err) {
    *plan = HostPlan();
    plan->n = n;
    plan->precision = precision;
    if (n < 1 || n > QFVM_MAX_QUBITS) {
        *err = "qubit count " + std::to_string(n) + " outside 1.." + std::to_string(QFVM_MAX_QUBITS);
        return false;
    }
    int dT, dR;
    default_shape(n, precision, &dT, &dR);
    if (T <= 0) T = dT;
    if (R <= 0) R = dR;
    if (T < 6 || T > MAX_TILE || R < 2 || R > 6 || R >= T) {
        *err = "invalid tile shape";
        return false;
    }
    const double Sb = amp_bytes(precision);
    const double N = std::ldexp(1.0, n);
    PlanStats& st = plan->stats;
    st.gates = static_cast<int64_t>(gops.size());
    for (const auto& g : gops) st.gate_bytes += gop_bytes(g, n, precision);

    // Small states: one whole-state pass with every gate in order.
    if (n < T) {
        if (n > small_max_qubits(precision)) {
            *err = "state too large for the whole-state kernel";
            return false;
        }
        // runs of gates become whole-state passes; a dense gate on more than
        // MAXK targets (beyond the whole-state kernel's registers) runs as its
        // own global pass between them
        size_t gi = 0;
        while (gi < gops.size()) {
            PassDesc pd;
            std::memset(&pd, 0, sizeof(pd));
            pd.T = n;
            pd.op_begin = static_cast<int32_t>(plan->ops.size());
            pd.probe_base = static_cast<int32_t>(plan->probe_slot.size());
            if (gops[gi].kind == K_DENSEK && gops[gi].k > MAXK) {
                pd.type = PASS_GLOBALOP;
                plan->ops.push_back(global_kop(plan, gops[gi]));
                ++gi;
            } else {
                pd.type = PASS_SMALL;
                while (gi < gops.size() && !(gops[gi].kind == K_DENSEK && gops[gi].k > MAXK))
                    plan->ops.push_back(global_kop(plan, gops[gi++]));
            }
            pd.op_count = static_cast<int32_t>(plan->ops.size()) - pd.op_begin;
            pd.nprobe = static_cast<int32_t>(plan->probe_slot.size()) - pd.probe_base;
            plan->passes.push_back(pd);
            st.passes += 1;
            st.pass_bytes += 2.0 * Sb * N;
        }
        st.rounds = 0;
        plan->T = n;
        plan->R = 0;
        plan->L = n;
        while (plan->coef.size() % 4) plan->coef.push_back(0.0);  // 4-wide reads of the last block
        return true;
    }

    const int L = std::min(5, T - 1);
    const int H = T - L;
    plan->T = T;
    plan->R = R;
    plan->L = L;
    const int eb = amp_bytes(precision);  // element bytes of the shared-memory tile
    const std::vector<int> pad_order = register_pad_order(T, eb);

    std::vector<int> pending(gops.size());
    for (size_t i = 0; i < gops.size(); ++i) pending[i] = static_cast<int>(i);
    std::vector<std::pair<int, uint8_t>> acts;
    std::vector<int> targ;

    while (!pending.empty()) {
        // ---- choose the tile's high qubits and the gates of this pass ----
        uint8_t blocked[64] = {0};
        std::vector<int> high;  // global qubits >= L in the tile
        std::vector<int> sched, rest;
        int probes = 0;
        for (int gi : pending) {
            const GOp& g = gops[gi];
            gop_actions(g, &acts);
            bool conflict = false;
            for (auto& a : acts) conflict |= act_conflict(blocked[a.first], a.second);
            bool ok = !conflict && g.kind != K_DENSEK;
            if (ok && g.kind == K_PROBE && probes >= MAX_PASS_PROBES) ok = false;
            if (ok) {
                gop_targets(g, &targ);
                std::vector<int> add;
                for (int t : targ)
                    if (t >= L && std::find(high.begin(), high.end(), t) == high.end() &&
                        std::find(add.begin(), add.end(), t) == add.end())
                        add.push_back(t);
                if (static_cast<int>(high.size() + add.size()) <= H) {
                    high.insert(high.end(), add.begin(), add.end());
                } else {
                    ok = false;
                }
            }
            if (ok) {
                sched.push_back(gi);
                if (g.kind == K_PROBE) ++probes;
            } else {
                for (auto& a : acts) blocked[a.first] |= a.second;
                rest.push_back(gi);
            }
        }
        if (sched.empty()) {
            // The first pending gate cannot join a tile pass (a dense gate on
            // more than two targets): apply it on its own.
            const int gi = pending.front();
            PassDesc pd;
            std::memset(&pd, 0, sizeof(pd));
            pd.type = PASS_GLOBALOP;
            pd.op_begin = static_cast<int32_t>(plan->ops.size());
            pd.op_count = 1;
            plan->ops.push_back(global_kop(plan, gops[gi]));
            plan->passes.push_back(pd);
            st.passes += 1;
            st.pass_bytes += 2.0 * Sb * N;
            pending.erase(pending.begin());
            continue;
        }
        // fill the tile to exactly T qubits
        for (int q = L; q < n && static_cast<int>(high.size()) < H; ++q)
            if (std::find(high.begin(), high.end(), q) == high.end()) high.push_back(q);
        std::sort(high.begin(), high.end());
        PassDesc pd;
        std::memset(&pd, 0, sizeof(pd));
        pd.type = PASS_TILE;
        pd.T = T;
        pd.L = L;
        pd.H = H;
        int local_of[64];
        for (int q = 0; q < 64; ++q) local_of[q] = -1;
        for (int k = 0; k < L; ++k) {
            pd.tq[k] = static_cast<uint8_t>(k);
            local_of[k] = k;
        }
        for (int k = 0; k < H; ++k) {
            pd.tq[L + k] = static_cast<uint8_t>(high[k]);
            local_of[high[k]] = L + k;
        }
        pd.step_begin = static_cast<int32_t>(plan->steps.size());
        pd.probe_base = static_cast<int32_t>(plan->probe_slot.size());

        // ---- split the pass's gates into register rounds ----
        // Two-target dense gates run as shared-memory steps of the tile (in
        // order); everything else runs in register rounds.
        std::vector<int> todo = sched;
        while (!todo.empty()) {
            if (gops[todo.front()].kind == K_DENSE2) {
                const GOp& g = gops[todo.front()];
                StepDesc sd;
                std::memset(&sd, 0, sizeof(sd));
                sd.type = STEP_SMEM;
                sd.op_begin = static_cast<int32_t>(plan->ops.size());
                sd.op_count = 1;
                KOp ko;
                std::memset(&ko, 0, sizeof(ko));
                ko.kind = g.kind;
                ko.t0 = static_cast<uint8_t>(local_of[g.t0]);
                ko.t1 = static_cast<uint8_t>(local_of[g.t1]);
                for (int q = 0; q < n; ++q) {
                    const uint64_t b = 1ULL << q;
                    if (g.cmask & b) {
                        if (local_of[q] >= 0) ko.creg |= 1u << local_of[q];
                        else ko.cthr |= b;
                    }
                }
                ko.coef = push_coef(plan, g);
                plan->ops.push_back(ko);
                plan->steps.push_back(sd);
                st.rounds += 1;
                todo.erase(todo.begin());
                continue;
            }
            uint8_t rblocked[64] = {0};
            std::vector<int> regs;  // tile-local positions
            std::vector<int> round_ops, left;
            for (int gi : todo) {
                const GOp& g = gops[gi];
                gop_actions(g, &acts);
                bool conflict = false;
                for (auto& a : acts) conflict |= act_conflict(rblocked[a.first], a.second);
                bool ok = !conflict && g.kind != K_DENSE2;
                if (ok) {
                    gop_targets(g, &targ);
                    std::vector<int> add;
                    for (int t : targ) {
                        int lp = local_of[t];
                        if (std::find(regs.begin(), regs.end(), lp) == regs.end() &&
                            std::find(add.begin(), add.end(), lp) == add.end())
                            add.push_back(lp);
                    }
                    if (static_cast<int>(regs.size() + add.size()) <= R)
                        regs.insert(regs.end(), add.begin(), add.end());
                    else
                        ok = false;
                }
                if (ok) {
                    round_ops.push_back(gi);
                } else {
                    for (auto& a : acts) rblocked[a.first] |= a.second;
                    left.push_back(gi);
                }
            }
            // pad the register set (register_pad_order)
            for (size_t x = 0; x < pad_order.size() && static_cast<int>(regs.size()) < R; ++x)
                if (std::find(regs.begin(), regs.end(), pad_order[x]) == regs.end()) regs.push_back(pad_order[x]);
            StepDesc sd;
            std::memset(&sd, 0, sizeof(sd));
            sd.type = STEP_ROUND;
            for (int k = 0; k < R; ++k) sd.rpos[k] = static_cast<uint8_t>(regs[k]);
            std::vector<int> freep;
            for (int p = 0; p < T; ++p)
                if (std::find(regs.begin(), regs.end(), p) == regs.end()) freep.push_back(p);
            // 8-byte elements with position 0 in the registers: the specialised
            // passes access the register pairs (j, j | bit of position 0) 16 bytes at a time
            const bool pairs = eb == 8 && std::find(regs.begin(), regs.end(), 0) != regs.end();
            order_thread_bits(freep, eb, pairs ? 16 : eb);
            const uint32_t u = 16u / static_cast<uint32_t>(eb);
            for (size_t k = 0; k < freep.size(); ++k) {
                sd.tpos[k] = static_cast<uint8_t>(freep[k]);
                sd.tglob[k] = pd.tq[freep[k]];
                sd.tsw[k] = static_cast<uint16_t>(tile_weight(freep[k], u));
            }
            for (int k = 0; k < R; ++k) sd.rsw[k] = static_cast<uint16_t>(tile_weight(regs[k], u));
            int reg_of_local[MAX_TILE];
            for (int p = 0; p < MAX_TILE; ++p) reg_of_local[p] = -1;
            for (int k = 0; k < R; ++k) reg_of_local[regs[k]] = k;
            sd.op_begin = static_cast<int32_t>(plan->ops.size());
            for (int gi : round_ops) {
                const GOp& g = gops[gi];
                KOp ko;
                std::memset(&ko, 0, sizeof(ko));
                ko.kind = g.kind;
                ko.flags = g.flags;
                ko.special = g.special;
                if (g.t0 >= 0) ko.t0 = static_cast<uint8_t>(reg_of_local[local_of[g.t0]]);
                if (g.t1 >= 0) ko.t1 = static_cast<uint8_t>(reg_of_local[local_of[g.t1]]);
                for (int q = 0; q < n; ++q) {
                    const uint64_t b = 1ULL << q;
                    const int lp = local_of[q];
                    const int rb = (lp >= 0) ? reg_of_local[lp] : -1;
                    if (g.cmask & b) {
                        if (rb >= 0) ko.creg |= 1u << rb;
                        else ko.cthr |= b;
                    }
                    if (g.pmask & b) {
                        if (rb >= 0) ko.preg |= 1u << rb;
                        else ko.pthr |= b;
                    }
                }
                if (ko.cthr) ko.flags |= F_TCTRL;
                if (ko.pthr) ko.flags |= F_TPAR;
                if (g.kind == K_PROBE) {
                    for (int q = 0; q < n; ++q)
                        if (g.xmask & (1ULL << q)) ko.xreg |= 1u << reg_of_local[local_of[q]];
                    ko.probe = static_cast<uint16_t>(plan->probe_slot.size() - pd.probe_base);
                    plan->probe_slot.push_back(g.slot);
                }
                if (g.kind == K_DIAG && ko.creg == 0) {
                    if (ko.preg == 0) {
                        ko.flags |= F_UNIFORM;  // one factor per thread, folded into the round phase
                    } else if (__builtin_popcount(ko.preg) == 1) {
                        ko.flags |= F_ONEBIT;
                        ko.t0 = static_cast<uint8_t>(__builtin_ctz(ko.preg));
                    }
                }
                ko.coef = push_coef(plan, g);
                plan->ops.push_back(ko);
            }
            sd.op_count = static_cast<int32_t>(round_ops.size());
            plan->steps.push_back(sd);
            st.rounds += 1;
            todo = left;
        }
        pd.step_count = static_cast<int32_t>(plan->steps.size()) - pd.step_begin;
        pd.nprobe = static_cast<int32_t>(plan->probe_slot.size()) - pd.probe_base;
        plan->passes.push_back(pd);
        st.passes += 1;
        st.pass_bytes += 2.0 * Sb * N;
        pending = rest;
    }
    while (plan->coef.size() % 4) plan->coef.push_back(0.0);  // 4-wide reads of the last block
    return true;
}

GOp gop_dagger(const GOp& g) {
    GOp d = g;
    d.bsign = static_cast<int8_t>(-g.bsign);
    auto conj_transpose = [&](int dim) {
        std::vector<double> c(g.coef.size());
        for (int r = 0; r < dim; ++r)
            for (int k = 0; k < dim; ++k) {
                c[2 * (r * dim + k)] = g.coef[2 * (k * dim + r)];
                c[2 * (r * dim + k) + 1] = -g.coef[2 * (k * dim + r) + 1];
            }
        d.coef = c;
    };
    switch (g.kind) {
        case K_REAL: d.coef = {g.coef[0], g.coef[2], g.coef[1], g.coef[3]}; break;  // real unitary: transpose
        case K_RX: d.coef = {g.coef[0], -g.coef[1]}; break;
        case K_DENSE: conj_transpose(2); break;
        case K_DENSE2: conj_transpose(4); break;
        case K_DENSEK: conj_transpose(1 << g.k); break;
        case K_DIAG:
            d.coef = {g.coef[0], -g.coef[1], g.coef[2], -g.coef[3]};
            if (g.flags & F_D1_SPEC) {
                if (g.special == SP_I) d.special = SP_NEGI;
                else if (g.special == SP_NEGI) d.special = SP_I;
            }
            break;
        default: break;  // X, Y, SWAP are self-inverse
    }
    return d;
}

bool build_adjoint_sweep(const std::vector<GOp>& gops, std::vector<GOp>* out, std::string* err) {
    out->clear();
    out->reserve(gops.size() * 2);
    for (size_t r = gops.size(); r-- > 0;) {
        const GOp& g = gops[r];
        if (g.slot >= 0) {
            if (!g.has_gen) {
                *err = "op " + std::to_string(g.src) + " carries a parameter slot but has no generator";
                return false;
            }
            GOp pr;
            pr.kind = K_PROBE;
            pr.xmask = g.gx;
            pr.pmask = g.gz;
            pr.cmask = g.gcmask;
            pr.special = static_cast<uint8_t>(g.gny & 3);
            pr.coef = {g.gscale};
            pr.slot = g.slot;
            pr.src = g.src;
            out->push_back(pr);
        }
        out->push_back(gop_dagger(g));
    }
    return true;
}

int bind_coef(int kind, double th, double* c) {
    switch (kind) {
        case QFVM_OP_RX:
            c[0] = std::cos(th / 2);
            c[1] = std::sin(th / 2);
            return 2;
        case QFVM_OP_RY:
            c[0] = std::cos(th / 2);
            c[1] = -std::sin(th / 2);
            c[2] = std::sin(th / 2);
            c[3] = std::cos(th / 2);
            return 4;
        case QFVM_OP_RZ:
        case QFVM_OP_RZZ:
            c[0] = std::cos(-th / 2);
            c[1] = std::sin(-th / 2);
            c[2] = std::cos(th / 2);
            c[3] = std::sin(th / 2);
            return 4;
        case QFVM_OP_P:
        case QFVM_OP_CP:
            c[0] = 1.0;
            c[1] = 0.0;
            c[2] = std::cos(th);
            c[3] = std::sin(th);
            return 4;
        default: return 0;
    }
}

bool unfix_bound(std::vector<GOp>* gops, std::string* err) {
    for (GOp& g : *gops) {
        if (g.slot < 0) continue;
        if (g.bkind == 0) {
            *err = "op " + std::to_string(g.src) +
                   ": only rx/ry/rz/p/cp/rzz gates can carry a per-item parameter in a batched run";
            return false;
        }
        if (g.kind == K_DIAG) {
            g.flags &= static_cast<uint8_t>(~F_D1_SPEC);
            g.special = 0;
            if (g.bkind == QFVM_OP_RZ || g.bkind == QFVM_OP_RZZ) g.flags &= static_cast<uint8_t>(~F_D0_ONE);
        }
    }
    return true;
}

namespace {

bool is_plain_hadamard(const GOp& g) {
    const double h = 1. / std::sqrt(2.);
    return g.kind == K_REAL && g.cmask == 0 && g.slot < 0 && g.bkind == 0 && g.coef.size() == 4 &&
           g.coef[0] == h && g.coef[1] == h && g.coef[2] == h && g.coef[3] == -h;
}

// a gate that touches every amplitude through its coefficients alone, so a
// scalar multiplies into them exactly where it would multiply the state
bool can_absorb_scalar(const GOp& g) {
    if (g.cmask != 0 || g.slot >= 0 || g.bkind != 0) return false;
    if (g.kind == K_REAL || g.kind == K_RX || g.kind == K_DENSE) return !is_plain_hadamard(g);
    if (g.kind == K_DIAG) return (g.flags & (F_D0_ONE | F_D1_SPEC)) == 0;
    return false;
}

void scale_coefs(GOp& g, int halves) {
    // (1/sqrt(2))^halves = 2^(-halves/2), one rounding when halves is odd
    double f = std::ldexp(1.0, -(halves / 2));
    if (halves & 1) f *= 1. / std::sqrt(2.);
    for (double& c : g.coef) c *= f;
}

}  // namespace

namespace {

uint64_t targets_of(const GOp& g) {
    uint64_t m = 0;
    if (g.t0 >= 0) m |= 1ULL << g.t0;
    if (g.t1 >= 0) m |= 1ULL << g.t1;
    if (g.kind == K_DENSEK)
        for (int j = 0; j < g.k; ++j) m |= 1ULL << g.tk[j];
    return m;
}
uint64_t touches(const GOp& g) { return g.cmask | g.pmask | targets_of(g); }

enum MergeClass { M_NONE, M_DIAG, M_RX, M_X };
MergeClass merge_class(const GOp& g) {
    if (g.cmask != 0 || g.slot >= 0 || g.bkind != 0) return M_NONE;
    if (g.kind == K_DIAG && g.pmask != 0 && (g.pmask & (g.pmask - 1)) == 0 && g.coef.size() == 4) return M_DIAG;
    if (g.kind == K_RX && g.coef.size() == 2) return M_RX;
    if (g.kind == K_X) return M_X;
    return M_NONE;
}

// whether a one-qubit gate of class c on qubit bit qb commutes with p (which
// touches qb): diagonals commute with diagonals and with gates that use qb
// only as a control; X-type gates commute with X / RX on the same target
bool commutes(MergeClass c, uint64_t qb, const GOp& p) {
    if (c == M_DIAG) return p.kind == K_DIAG || ((p.cmask & qb) && !(p.pmask & qb) && !(targets_of(p) & qb));
    return (p.kind == K_X || p.kind == K_RX) && p.t0 >= 0 && (1ULL << p.t0) == qb && !(p.cmask & qb);
}

}  // namespace

void fuse_single_qubit(std::vector<GOp>* gops) {
    constexpr int MAX_SCAN = 512;
    std::vector<GOp>& g = *gops;
    std::vector<char> dead(g.size(), 0);
    for (size_t j = 0; j < g.size(); ++j) {
        const MergeClass c = merge_class(g[j]);
        if (c == M_NONE) continue;
        const uint64_t qb = c == M_DIAG ? g[j].pmask : (1ULL << g[j].t0);
        int scanned = 0;
        for (size_t i = j; i-- > 0 && scanned < MAX_SCAN; ++scanned) {
            if (dead[i] || !(touches(g[i]) & qb)) continue;
            GOp& a = g[i];
            if (merge_class(a) == c && (c == M_DIAG ? a.pmask == qb : (1ULL << a.t0) == qb)) {
                if (c == M_DIAG) {
                    const cd d0 = cd(a.coef[0], a.coef[1]) * cd(g[j].coef[0], g[j].coef[1]);
                    const cd d1 = cd(a.coef[2], a.coef[3]) * cd(g[j].coef[2], g[j].coef[3]);
                    a.flags &= static_cast<uint8_t>(~(F_D0_ONE | F_D1_SPEC));
                    a.special = 0;
                    set_diag(a, d0, d1);
                } else if (c == M_RX) {
                    // rx(a) rx(b) = rx(a + b): [[c, -is], [-is, c]]
                    const double c1 = a.coef[0], s1 = a.coef[1], c2 = g[j].coef[0], s2 = g[j].coef[1];
                    a.coef = {c1 * c2 - s1 * s2, s1 * c2 + c1 * s2};
                } else {
                    dead[i] = 1;  // X X = I
                }
                dead[j] = 1;
                break;
            }
            if (!commutes(c, qb, a)) break;
        }
    }
    size_t w = 0;
    for (size_t i = 0; i < g.size(); ++i)
        if (!dead[i]) g[w++] = g[i];
    g.resize(w);
}

void unnormalize_hadamards(std::vector<GOp>* gops) {
    constexpr int MAX_PENDING = 256;  // keeps |amplitudes| below 2^128 between absorptions
    std::vector<size_t> pending;
    int last = -1;
    for (size_t i = 0; i < gops->size(); ++i) {
        GOp& g = (*gops)[i];
        if (is_plain_hadamard(g) && static_cast<int>(pending.size()) < MAX_PENDING) {
            pending.push_back(i);
        } else if (can_absorb_scalar(g)) {
            if (!pending.empty()) {
                scale_coefs(g, static_cast<int>(pending.size()));
                for (size_t k : pending) {
                    (*gops)[k].kind = K_HAD;
                    (*gops)[k].coef.clear();
                }
                pending.clear();
            }
            last = static_cast<int>(i);
        }
    }
    if (!pending.empty() && last >= 0) {
        // a global scalar commutes with every gate: an earlier gate takes it
        scale_coefs((*gops)[static_cast<size_t>(last)], static_cast<int>(pending.size()));
        for (size_t k : pending) {
            (*gops)[k].kind = K_HAD;
            (*gops)[k].coef.clear();
        }
    }
}

namespace {

// bits of the register index an op of a round acts on non-diagonally
uint32_t nondiag_reg_bits(const KOp& o) {
    switch (o.kind) {
        case K_X: case K_Y: case K_REAL: case K_RX: case K_DENSE: case K_HAD:
            return 1u << o.t0;
        case K_SWAP:
            return (1u << o.t0) | (1u << o.t1);
        case K_DIAG: case K_DIAGR:
            return 0;
        default:
            return ~0u;  // anything else: flush
    }
}

bool mergeable_diag(const KOp& o) {
    return o.kind == K_DIAG && !(o.flags & (F_TCTRL | F_TPAR | F_UNIFORM));
}

int entry_code(cd z) {
    if (z == cd(1.0, 0.0)) return DIAGR_ONE;
    if (z == cd(-1.0, 0.0)) return DIAGR_NEG1;
    if (z == cd(0.0, 1.0)) return DIAGR_I;
    if (z == cd(0.0, -1.0)) return DIAGR_NEGI;
    return DIAGR_GENERAL;
}

}  // namespace

void merge_round_diagonals(HostPlan* plan) {
    // rounds of five register qubits are left alone: their 32-entry tables,
    // and the flips they resolve, measured slower at the complex64 register
    // budget (spills)
    if (plan->R < 1 || plan->R > 4 || !plan->binds.empty() || !plan->probe_slot.empty()) return;
    const int R = plan->R;
    const int NA = 1 << R;
    std::vector<KOp> out;
    out.reserve(plan->ops.size());
    // whole-state passes keep their ops (re-indexed); rounds are rewritten
    std::vector<int32_t> step_begin(plan->steps.size()), step_count(plan->steps.size());
    std::vector<int32_t> pass_begin(plan->passes.size());
    std::vector<bool> step_done(plan->steps.size(), false);
    for (size_t pi = 0; pi < plan->passes.size(); ++pi) {
        PassDesc& pd = plan->passes[pi];
        if (pd.type != PASS_TILE) {
            pass_begin[pi] = static_cast<int32_t>(out.size());
            out.insert(out.end(), plan->ops.begin() + pd.op_begin, plan->ops.begin() + pd.op_begin + pd.op_count);
            continue;
        }
        for (int si = pd.step_begin; si < pd.step_begin + pd.step_count; ++si) {
            const StepDesc& sd = plan->steps[si];
            step_begin[si] = static_cast<int32_t>(out.size());
            step_done[si] = true;
            if (sd.type != STEP_ROUND) {
                out.insert(out.end(), plan->ops.begin() + sd.op_begin, plan->ops.begin() + sd.op_begin + sd.op_count);
                step_count[si] = static_cast<int32_t>(out.size()) - step_begin[si];
                continue;
            }
            std::vector<cd> table(NA, cd(1.0, 0.0));
            std::vector<KOp> merged;
            uint32_t support = 0;
            auto flush = [&]() {
                if (merged.empty()) return;
                if (merged.size() == 1) {
                    out.push_back(merged[0]);
                } else {
                    while (plan->coef.size() % 4) plan->coef.push_back(0.0);
                    KOp k;
                    std::memset(&k, 0, sizeof(k));
                    k.kind = K_DIAGR;
                    k.k = static_cast<uint8_t>(R);
                    k.coef = static_cast<uint32_t>(plan->coef.size());
                    for (int j = 0; j < NA; ++j) {
                        plan->coef.push_back(table[j].real());
                        plan->coef.push_back(table[j].imag());
                        const uint64_t c = static_cast<uint64_t>(entry_code(table[j]));
                        if (j < DIAGR_LOW) k.cthr |= c << (3 * j);
                        else k.pthr |= c << (3 * (j - DIAGR_LOW));
                    }
                    out.push_back(k);
                }
                merged.clear();
                std::fill(table.begin(), table.end(), cd(1.0, 0.0));
                support = 0;
            };
            for (int oi = sd.op_begin; oi < sd.op_begin + sd.op_count; ++oi) {
                const KOp& o = plan->ops[oi];
                if (mergeable_diag(o)) {
                    const double* c = plan->coef.data() + o.coef;
                    const cd d0(c[0], c[1]), d1(c[2], c[3]);
                    for (int j = 0; j < NA; ++j) {
                        if ((static_cast<uint32_t>(j) & o.creg) != o.creg) continue;
                        table[j] *= (__builtin_popcount(static_cast<uint32_t>(j) & o.preg) & 1) ? d1 : d0;
                    }
                    support |= o.creg | o.preg;
                    merged.push_back(o);
                    continue;
                }
                if (nondiag_reg_bits(o) & support) flush();
                out.push_back(o);
            }
            flush();
            step_count[si] = static_cast<int32_t>(out.size()) - step_begin[si];
        }
    }
    for (size_t si = 0; si < plan->steps.size(); ++si) {
        if (!step_done[si]) continue;
        plan->steps[si].op_begin = step_begin[si];
        plan->steps[si].op_count = step_count[si];
    }
    for (size_t pi = 0; pi < plan->passes.size(); ++pi)
        if (plan->passes[pi].type != PASS_TILE) plan->passes[pi].op_begin = pass_begin[pi];
    plan->ops.swap(out);
    while (plan->coef.size() % 4) plan->coef.push_back(0.0);
}

}  // namespace qsv
