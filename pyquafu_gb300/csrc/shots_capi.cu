// qfvm_simulate_shots: circuits with mid-circuit measurement, reset and
// classically controlled blocks, one trajectory per shot (the per-shot branch
// of simulate_circuit, qfvm.cpp:104-133; simulator.hpp:95-111 dispatches
// measure / reset / cif).  The op list is cut into segments at every
// measure, reset and cif; gate segments are fused plans that run over all
// shots of a chunk at once (shots are batch items sharing one coefficient
// pool), a cif body runs only on the items whose classical bits match.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <set>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "jit.h"
#include "kernels.h"

using namespace qsv;
using namespace qsv_capi;

namespace {

struct Segment {
    int type = 0;  // 0 gates, 1 measure / reset, 2 cif body
    qfvm_plan* plan = nullptr;
    MeasureSpec ms{};
    CifSpec cs{};
    int draw = -1;
};

void free_segments(std::vector<Segment>& segs) {
    for (auto& s : segs) free_plan(s.plan);
    segs.clear();
}

bool is_gate_kind(int k) { return (k >= QFVM_OP_X && k <= QFVM_OP_RZZ) || k == QFVM_OP_MATRIX; }

int parse_program(int n, int ncb, const qfvm_op* ops, int64_t n_ops, const double* matpool, int64_t matpool_len,
                  std::vector<Segment>* segs, int* ndraws) {
    std::vector<qfvm_op> pending;
    auto flush = [&]() -> int {
        if (pending.empty()) return QFVM_OK;
        Segment s;
        s.type = 0;
        QSV_TRY(make_plan(n, c128_arith(), pending.data(), static_cast<int64_t>(pending.size()), matpool, matpool_len, 0,
                          0, &s.plan));
        segs->push_back(s);
        pending.clear();
        return QFVM_OK;
    };
    *ndraws = 0;
    for (int64_t i = 0; i < n_ops; ++i) {
        const qfvm_op& o = ops[i];
        if (o.kind == QFVM_OP_MEASURE || o.kind == QFVM_OP_RESET) {
            QSV_TRY(flush());
            const int k = o.nqubits;
            if (k < 1 || k > 8) return fail(QFVM_ERR_UNSUPPORTED, "measure/reset of more than 8 qubits at once");
            Segment s;
            s.type = 1;
            s.ms.k = k;
            s.ms.reset = o.kind == QFVM_OP_RESET ? 1 : 0;
            uint64_t seen = 0;
            for (int j = 0; j < k; ++j) {
                const int q = o.qubits[j];
                if (q < 0 || q >= n || ((seen >> q) & 1)) return fail(QFVM_ERR_INVALID, "bad measured qubit");
                seen |= 1ULL << q;
                s.ms.q[j] = static_cast<uint8_t>(q);
                s.ms.srt[j] = static_cast<uint8_t>(q);
                if (!s.ms.reset) {
                    const int c = o.qubits[8 + j];
                    if (c < 0 || c >= ncb) return fail(QFVM_ERR_INVALID, "classical bit out of range");
                    s.ms.cb[j] = static_cast<uint8_t>(c);
                }
            }
            for (int x = 1; x < k; ++x)
                for (int y = x; y > 0 && s.ms.srt[y - 1] > s.ms.srt[y]; --y) std::swap(s.ms.srt[y], s.ms.srt[y - 1]);
            s.draw = (*ndraws)++;
            segs->push_back(s);
        } else if (o.kind == QFVM_OP_CIF) {
            QSV_TRY(flush());
            const int nc = o.nqubits;
            const int64_t nb = o.mat_dim;
            if (nc < 1 || nc > 16) return fail(QFVM_ERR_INVALID, "cif needs 1..16 classical bits");
            if (nb < 0 || i + nb >= n_ops) return fail(QFVM_ERR_INVALID, "cif body runs past the op list");
            const double cond = o.params[0];
            if (!(cond >= 0.0) || cond != std::floor(cond) || cond > 9.0e15)
                return fail(QFVM_ERR_INVALID, "cif condition must be a non-negative integer");
            Segment s;
            s.type = 2;
            s.cs.nc = nc;
            s.cs.condition = static_cast<uint64_t>(cond);
            for (int j = 0; j < nc; ++j) {
                const int c = o.qubits[j];
                if (c < 0 || c >= ncb) return fail(QFVM_ERR_INVALID, "classical bit out of range");
                s.cs.cb[j] = static_cast<uint8_t>(c);
            }
            for (int64_t b = 1; b <= nb; ++b)
                if (!is_gate_kind(ops[i + b].kind))
                    return fail(QFVM_ERR_UNSUPPORTED, "a cif body holds gates only");
            if (nb > 0) {
                QSV_TRY(make_plan(n, c128_arith(), ops + i + 1, nb, matpool, matpool_len, 0, 0, &s.plan));
                segs->push_back(s);
            }
            i += nb;
        } else if (is_gate_kind(o.kind)) {
            pending.push_back(o);
        } else {
            return fail(QFVM_ERR_INVALID, "unknown op kind " + std::to_string(o.kind));
        }
    }
    return flush();
}

}  // namespace

namespace qsv_capi {

// Every pass of a plan over `items` states (shared coefficient pool).
int run_plan_items(qfvm_plan* p, void* state, int items, const uint8_t* active, cudaStream_t st) {
    p->chain_ok = false;  // inactive items keep their FP64 state: no float pairs between passes
    const HostPlan& hp = p->hp;
    for (size_t i = 0; i < hp.passes.size(); ++i) {
        const PassDesc& pd = hp.passes[i];
        cudaError_t e;
        if (pd.type == PASS_TILE) {
            bool done = false;
            e = qsv::jit_launch_pass(p, static_cast<int>(i), state, nullptr, p->dcoef, items, 0, active, 0, nullptr,
                                     nullptr, st, &done);
            if (e == cudaSuccess && !done)
                e = launch_tile_pass(hp.arith, hp.T, hp.R, state, p->dpass + i, p->dsteps, p->dops, p->dcoef, hp.n,
                                     pd.H, items, 0, active, st);
        } else if (pd.type == PASS_SMALL)
            e = launch_small(hp.arith, state, 1ULL << hp.n, items, hp.n, p->dops + pd.op_begin, pd.op_count, p->dcoef,
                             0, active, st);
        else
            e = launch_globalop(hp.arith, state, hp.n, hp.ops[pd.op_begin].k, p->dops + pd.op_begin, p->dcoef, items, 0, active, st);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        if (e != cudaSuccess) return fail(QFVM_ERR_CUDA, std::string("pass launch: ") + cudaGetErrorString(e));
    }
    return QFVM_OK;
}

}  // namespace qsv_capi

extern "C" {

int qfvm_simulate_shots(int32_t num_qubits, int32_t num_cbits, const qfvm_op* ops, int64_t n_ops,
                        const double* matpool, int64_t matpool_len, const double* psi_in, int64_t shots,
                        const double* uniforms, int64_t n_draws, uint64_t* outcomes, double* final_state) {
    qsv_capi::NvtxRange range("qfvm trajectories");
    const int n = num_qubits;
    if (n < 1 || n > 30) return fail(QFVM_ERR_INVALID, "per-shot trajectories take 1..30 qubits");
    if (num_cbits < 0 || num_cbits > 64) return fail(QFVM_ERR_INVALID, "classical register of 0..64 bits");
    if (shots < 1) return fail(QFVM_ERR_INVALID, "per-shot trajectories need at least one shot");
    if (n_ops < 0 || (n_ops > 0 && !ops)) return fail(QFVM_ERR_INVALID, "bad op list");
    if (!outcomes) return fail(QFVM_ERR_INVALID, "missing outcome buffer");
    QSV_TRY(check_device());
    std::lock_guard<std::mutex> lk(g_boundary_mu);
    std::vector<Segment> segs;
    int ndraws = 0;
    const int ncb = num_cbits > 0 ? num_cbits : 1;
    int rc = parse_program(n, ncb, ops, n_ops, matpool, matpool_len, &segs, &ndraws);
    if (rc != QFVM_OK) {
        free_segments(segs);
        return rc;
    }
    if (ndraws != n_draws || (ndraws > 0 && !uniforms)) {
        free_segments(segs);
        return fail(QFVM_ERR_INVALID, "expected " + std::to_string(ndraws) + " uniforms per shot");
    }
    std::set<int> measured;
    int kmax = 1;
    for (const auto& sg : segs)
        if (sg.type == 1) {
            kmax = std::max(kmax, sg.ms.k);
            if (!sg.ms.reset)
                for (int j = 0; j < sg.ms.k; ++j) measured.insert(sg.ms.cb[j]);
        }

    // chunk of shots resident at once: at most about half of the free memory
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t per_item = (sizeof(double2) << n) + static_cast<size_t>(ncb) + 64 +
                            static_cast<size_t>(outcome_blocks_per_item(n, 1)) * (8u << kmax) + 8u * ndraws;
    int64_t chunk = static_cast<int64_t>((free_b / 2) / per_item);
    if (chunk < 1) chunk = 1;
    if (chunk > shots) chunk = shots;
    if (chunk > (1 << 20)) chunk = 1 << 20;

    cudaStream_t st = nullptr;
    DevBuf dstate, dpsi0, duni, dcreg, dscratch;
    auto done = [&](int code) {
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
        dstate.release();
        dpsi0.release();
        duni.release();
        dcreg.release();
        dscratch.release();
        free_segments(segs);
        return code;
    };
#define SHOT_CUDA(call, what)                                                                                  \
    do {                                                                                                       \
        cudaError_t e_ = (call);                                                                               \
        if (e_ != cudaSuccess)                                                                                 \
            return done(fail(e_ == cudaErrorMemoryAllocation ? QFVM_ERR_NOMEM : QFVM_ERR_CUDA,                  \
                             std::string(what) + ": " + cudaGetErrorString(e_)));                              \
    } while (0)
#define SHOT_TRY(expr)                  \
    do {                                \
        int rc_ = (expr);               \
        if (rc_ != QFVM_OK) return done(rc_); \
    } while (0)
    SHOT_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
    const size_t N = 1ULL << n;
    SHOT_TRY(dstate.ensure(static_cast<size_t>(chunk) * N * sizeof(double2)));
    if (psi_in) {
        SHOT_TRY(dpsi0.ensure(N * sizeof(double2)));
        SHOT_CUDA(cudaMemcpyAsync(dpsi0.p, psi_in, N * sizeof(double2), cudaMemcpyHostToDevice, st), "input upload");
    }
    SHOT_TRY(duni.ensure(static_cast<size_t>(chunk) * std::max(ndraws, 1) * 8));
    SHOT_TRY(dcreg.ensure(static_cast<size_t>(chunk) * ncb));
    const size_t b_part = align256(static_cast<size_t>(chunk) * outcome_blocks_per_item(n, 1) * (8u << kmax));
    const size_t b_out = align256(static_cast<size_t>(chunk) * 4), b_scale = align256(static_cast<size_t>(chunk) * 8);
    SHOT_TRY(dscratch.ensure(b_part + b_out + b_scale + align256(static_cast<size_t>(chunk))));
    char* sp = static_cast<char*>(dscratch.p);
    double* dpart = reinterpret_cast<double*>(sp);
    int32_t* doutcome = reinterpret_cast<int32_t*>(sp + b_part);
    double* dscale = reinterpret_cast<double*>(sp + b_part + b_out);
    uint8_t* dactive = reinterpret_cast<uint8_t*>(sp + b_part + b_out + b_scale);
    std::vector<uint8_t> hcreg(static_cast<size_t>(chunk) * ncb);

    for (int64_t c0 = 0; c0 < shots; c0 += chunk) {
        const int items = static_cast<int>(std::min<int64_t>(chunk, shots - c0));
        if (ndraws > 0)
            SHOT_CUDA(cudaMemcpyAsync(duni.p, uniforms + c0 * ndraws, static_cast<size_t>(items) * ndraws * 8,
                                      cudaMemcpyHostToDevice, st),
                      "uniform upload");
        SHOT_CUDA(cudaMemsetAsync(dcreg.p, 0, static_cast<size_t>(items) * ncb, st), "classical bits");
        if (psi_in) SHOT_CUDA(launch_items_copy(dstate.p, n, items, dpsi0.p, st), "initial states");
        else SHOT_CUDA(launch_zero_items(QFVM_C128, dstate.p, n, items, st), "initial states");
        g_launches.fetch_add(1, std::memory_order_relaxed);
        for (const auto& sg : segs) {
            if (sg.type == 0) {
                SHOT_TRY(run_plan_items(sg.plan, dstate.p, items, nullptr, st));
            } else if (sg.type == 1) {
                SHOT_CUDA(launch_measure(dstate.p, n, sg.ms, items, duni.as<double>(), sg.draw, ndraws,
                                         dcreg.as<uint8_t>(), ncb, dpart, doutcome, dscale, st),
                          "measure");
                g_launches.fetch_add(3, std::memory_order_relaxed);
            } else {
                SHOT_CUDA(launch_cif_mask(dcreg.as<uint8_t>(), ncb, items, sg.cs, dactive, st), "cif");
                g_launches.fetch_add(1, std::memory_order_relaxed);
                SHOT_TRY(run_plan_items(sg.plan, dstate.p, items, dactive, st));
            }
        }
        SHOT_CUDA(cudaMemcpyAsync(hcreg.data(), dcreg.p, static_cast<size_t>(items) * ncb, cudaMemcpyDeviceToHost, st),
                  "classical bits download");
        const bool last = c0 + items >= shots;
        if (last && final_state)
            SHOT_CUDA(cudaMemcpyAsync(final_state, dstate.as<double2>() + static_cast<size_t>(items - 1) * N,
                                      N * sizeof(double2), cudaMemcpyDeviceToHost, st),
                      "state download");
        SHOT_CUDA(cudaStreamSynchronize(st), "trajectories");
        if (const int src = check_status(st)) return done(src);
        for (int it = 0; it < items; ++it) {
            uint64_t v = 0;
            for (int c : measured) v = v * 2 + hcreg[static_cast<size_t>(it) * ncb + c];
            outcomes[c0 + it] = v;
        }
    }
    return done(QFVM_OK);
#undef SHOT_CUDA
#undef SHOT_TRY
}

}  // extern "C"
