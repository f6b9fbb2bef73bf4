// qfvm_simulate_noise: NoiseSVSimulator.run (quafu/simulators/simulator.py:
// 148-225) with the shots side by side on the device.  Per shot the reference
// draws, in order, one number per unitary channel (gen_circuit, :196-218,
// np.random.choice), one per Kraus channel while running (:61-76,
// np.random.rand), then samples one outcome (sampling_statevec) and, with a
// Hamiltonian, evaluates every term (expect_statevec).  Here every draw is a
// given uniform in that order, gate segments are fused plans over all shots
// of a chunk, and channels are per-item 2x2 matrices (noise.cu).
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "kernels.h"

using namespace qsv;
using namespace qsv_capi;

namespace {

struct NoiseSegment {
    int type = 0;  // 0 gates, 1 channel
    qfvm_plan* plan = nullptr;
    int q = 0, m = 0, kraus = 0, draw = -1;
    int cross = 0;  // Kraus: some K^dagger K has a nonzero off-diagonal entry
    size_t mat_off = 0, prob_off = 0;  // into the channel data (doubles)
};

void free_noise(std::vector<NoiseSegment>& segs) {
    for (auto& s : segs) free_plan(s.plan);
    segs.clear();
}

bool gate_kind(int k) { return (k >= QFVM_OP_X && k <= QFVM_OP_RZZ) || k == QFVM_OP_MATRIX; }

int parse_noise(int n, const qfvm_op* ops, int64_t n_ops, const double* matpool, int64_t matpool_len,
                std::vector<NoiseSegment>* segs, std::vector<double>* data, int* ndraws) {
    std::vector<qfvm_op> pending;
    auto flush = [&]() -> int {
        if (pending.empty()) return QFVM_OK;
        NoiseSegment s;
        QSV_TRY(make_plan(n, c128_arith(), pending.data(), static_cast<int64_t>(pending.size()), matpool, matpool_len, 0,
                          0, &s.plan));
        segs->push_back(s);
        pending.clear();
        return QFVM_OK;
    };
    int nu = 0, nk = 0;
    for (int64_t i = 0; i < n_ops; ++i) {
        const qfvm_op& o = ops[i];
        if (o.kind == QFVM_OP_UCHANNEL || o.kind == QFVM_OP_KRAUS) {
            QSV_TRY(flush());
            const int m = static_cast<int>(o.params[0]);
            const int q = o.qubits[0];
            if (o.nqubits != 1 || q < 0 || q >= n) return fail(QFVM_ERR_INVALID, "a channel acts on one qubit");
            if (m < 1 || m > MAX_CHANNEL_OPS || o.params[0] != m)
                return fail(QFVM_ERR_UNSUPPORTED, "a channel has 1.." + std::to_string(MAX_CHANNEL_OPS) + " operators");
            const bool kraus = o.kind == QFVM_OP_KRAUS;
            const int64_t need = 4LL * m + (kraus ? 0 : m);
            if (o.mat_dim != 2 || o.mat_offset < 0 || o.mat_offset + need > matpool_len)
                return fail(QFVM_ERR_INVALID, "channel operators outside the matrix pool");
            NoiseSegment s;
            s.type = 1;
            s.q = q;
            s.m = m;
            s.kraus = kraus ? 1 : 0;
            s.draw = kraus ? nk++ : nu++;  // rebased below: unitary draws first
            s.mat_off = data->size();
            const double* src = matpool + 2 * o.mat_offset;  // complex128 pool
            data->insert(data->end(), src, src + 8 * m);
            for (int j = 0; kraus && j < m; ++j) {
                const double* k = src + 8 * j;  // row-major 2x2, (re, im) pairs
                const double m01r = k[0] * k[2] + k[1] * k[3] + k[4] * k[6] + k[5] * k[7];
                const double m01i = k[0] * k[3] - k[1] * k[2] + k[4] * k[7] - k[5] * k[6];
                if (m01r != 0.0 || m01i != 0.0) s.cross = 1;
            }
            s.prob_off = data->size();
            double tot = 0.0;
            for (int j = 0; j < m; ++j) {
                const double p = kraus ? 0.0 : src[8 * m + 2 * j];
                if (!kraus && !(p >= 0.0)) return fail(QFVM_ERR_INVALID, "channel probabilities must be >= 0");
                tot += p;
                data->push_back(p);
            }
            if (!kraus && !(tot > 0.0)) return fail(QFVM_ERR_INVALID, "channel probabilities sum to zero");
            segs->push_back(s);
        } else if (gate_kind(o.kind)) {
            pending.push_back(o);
        } else {
            return fail(QFVM_ERR_INVALID, "noisy circuits take gates and channels only (op kind " +
                                              std::to_string(o.kind) + ")");
        }
    }
    QSV_TRY(flush());
    for (auto& s : *segs)
        if (s.type == 1 && s.kraus) s.draw += nu;
    *ndraws = nu + nk + 1;  // + the final sample
    return QFVM_OK;
}

}  // namespace

extern "C" {

int qfvm_simulate_noise(int32_t num_qubits, const qfvm_op* ops, int64_t n_ops, const double* matpool,
                        int64_t matpool_len, const double* psi_in, int64_t shots, const double* uniforms,
                        int64_t n_draws, uint64_t* samples, const uint64_t* x_masks, const uint64_t* z_masks,
                        const int32_t* y_counts, const double* coeffs, int64_t n_terms, double* expvals) {
    qsv_capi::NvtxRange range("qfvm noisy trajectories");
    const int n = num_qubits;
    if (n < 1 || n > 30) return fail(QFVM_ERR_INVALID, "noisy trajectories take 1..30 qubits");
    if (shots < 1) return fail(QFVM_ERR_INVALID, "noisy trajectories need at least one shot");
    if (n_ops < 0 || (n_ops > 0 && !ops)) return fail(QFVM_ERR_INVALID, "bad op list");
    if (!samples || !uniforms) return fail(QFVM_ERR_INVALID, "missing sample or uniform buffer");
    if (n_terms < 0 || n_terms > 4096 || (n_terms > 0 && (!x_masks || !z_masks || !y_counts || !coeffs || !expvals)))
        return fail(QFVM_ERR_INVALID, "bad Hamiltonian terms");
    const uint64_t lim = (1ULL << n) - 1;
    for (int64_t t = 0; t < n_terms; ++t)
        if ((x_masks[t] | z_masks[t]) & ~lim) return fail(QFVM_ERR_INVALID, "Pauli term acts outside the state");
    QSV_TRY(check_device());
    std::lock_guard<std::mutex> lk(g_boundary_mu);
    std::vector<NoiseSegment> segs;
    std::vector<double> cdata;
    int ndraws = 0;
    int rc = parse_noise(n, ops, n_ops, matpool, matpool_len, &segs, &cdata, &ndraws);
    if (rc != QFVM_OK) {
        free_noise(segs);
        return rc;
    }
    if (ndraws != n_draws) {
        free_noise(segs);
        return fail(QFVM_ERR_INVALID, "expected " + std::to_string(ndraws) + " uniforms per shot");
    }
    const size_t N = 1ULL << n;
    const int bpi = channel_blocks_per_item(n);
    const uint64_t chunk_amps = hamiltonian_chunk(n);
    const uint64_t epi = N / chunk_amps;  // expectation chunks per item
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t per_item = (sizeof(double2) << n) + 8u * ndraws + 8u * bpi * (MAX_CHANNEL_OPS + 1) + 64 + 8 +
                            8u * static_cast<size_t>(n_terms) * (epi + 1);
    int64_t chunk = static_cast<int64_t>((free_b / 2) / per_item);
    if (chunk < 1) chunk = 1;
    if (chunk > shots) chunk = shots;
    if (chunk > (1 << 20)) chunk = 1 << 20;

    cudaStream_t st = nullptr;
    DevBuf dstate, dpsi0, duni, dscratch, dterms;
    auto done = [&](int code) {
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
        dstate.release();
        dpsi0.release();
        duni.release();
        dscratch.release();
        dterms.release();
        free_noise(segs);
        return code;
    };
#define NZ_CUDA(call, what)                                                                                    \
    do {                                                                                                       \
        cudaError_t e_ = (call);                                                                               \
        if (e_ != cudaSuccess)                                                                                 \
            return done(fail(e_ == cudaErrorMemoryAllocation ? QFVM_ERR_NOMEM : QFVM_ERR_CUDA,                  \
                             std::string(what) + ": " + cudaGetErrorString(e_)));                              \
    } while (0)
#define NZ_TRY(expr)                          \
    do {                                      \
        int rc_ = (expr);                     \
        if (rc_ != QFVM_OK) return done(rc_); \
    } while (0)
    NZ_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
    NZ_TRY(dstate.ensure(static_cast<size_t>(chunk) * N * sizeof(double2)));
    if (psi_in) {
        NZ_TRY(dpsi0.ensure(N * sizeof(double2)));
        NZ_CUDA(cudaMemcpyAsync(dpsi0.p, psi_in, N * sizeof(double2), cudaMemcpyHostToDevice, st), "input upload");
    }
    NZ_TRY(duni.ensure(static_cast<size_t>(chunk) * ndraws * 8));
    // scratch: channel data, channel norms, per-item matrices, samples, expectation chunks and values
    const size_t b_cd = align256(std::max<size_t>(cdata.size(), 1) * 8);
    const size_t b_part = align256(static_cast<size_t>(chunk) * bpi * (MAX_CHANNEL_OPS + 1) * 8);
    const size_t b_imat = align256(static_cast<size_t>(chunk) * 8 * 8);
    const size_t b_smp = align256(static_cast<size_t>(chunk) * 8);
    const size_t b_ep = align256(static_cast<size_t>(chunk) * epi * std::max<int64_t>(n_terms, 1) * 8);
    const size_t b_ev = align256(static_cast<size_t>(chunk) * std::max<int64_t>(n_terms, 1) * 8);
    NZ_TRY(dscratch.ensure(b_cd + b_part + b_imat + b_smp + b_ep + b_ev));
    char* sp = static_cast<char*>(dscratch.p);
    double* dcd = reinterpret_cast<double*>(sp);
    double* dpart = reinterpret_cast<double*>(sp + b_cd);
    double* dimat = reinterpret_cast<double*>(sp + b_cd + b_part);
    uint64_t* dsmp = reinterpret_cast<uint64_t*>(sp + b_cd + b_part + b_imat);
    double* depart = reinterpret_cast<double*>(sp + b_cd + b_part + b_imat + b_smp);
    double* dev = reinterpret_cast<double*>(sp + b_cd + b_part + b_imat + b_smp + b_ep);
    if (!cdata.empty())
        NZ_CUDA(cudaMemcpyAsync(dcd, cdata.data(), cdata.size() * 8, cudaMemcpyHostToDevice, st), "channel upload");
    uint64_t* dx = nullptr;
    uint64_t* dz = nullptr;
    double* dc = nullptr;
    int32_t* dy = nullptr;
    int32_t* doptr = nullptr;
    if (n_terms > 0) {
        // every term its own observable: terms t..t+1
        const size_t nt = static_cast<size_t>(n_terms);
        const size_t b8 = align256(nt * 8), b4 = align256(nt * 4), bo = align256((nt + 1) * 4);
        NZ_TRY(dterms.ensure(3 * b8 + b4 + bo));
        char* tb = static_cast<char*>(dterms.p);
        dx = reinterpret_cast<uint64_t*>(tb);
        dz = reinterpret_cast<uint64_t*>(tb + b8);
        dc = reinterpret_cast<double*>(tb + 2 * b8);
        dy = reinterpret_cast<int32_t*>(tb + 3 * b8);
        doptr = reinterpret_cast<int32_t*>(tb + 3 * b8 + b4);
        std::vector<int32_t> optr(nt + 1);
        for (size_t t = 0; t <= nt; ++t) optr[t] = static_cast<int32_t>(t);
        NZ_CUDA(cudaMemcpyAsync(dx, x_masks, nt * 8, cudaMemcpyHostToDevice, st), "term upload");
        NZ_CUDA(cudaMemcpyAsync(dz, z_masks, nt * 8, cudaMemcpyHostToDevice, st), "term upload");
        NZ_CUDA(cudaMemcpyAsync(dc, coeffs, nt * 8, cudaMemcpyHostToDevice, st), "term upload");
        NZ_CUDA(cudaMemcpyAsync(dy, y_counts, nt * 4, cudaMemcpyHostToDevice, st), "term upload");
        NZ_CUDA(cudaMemcpyAsync(doptr, optr.data(), (nt + 1) * 4, cudaMemcpyHostToDevice, st), "term upload");
        NZ_CUDA(cudaStreamSynchronize(st), "term upload");
    }

    for (int64_t c0 = 0; c0 < shots; c0 += chunk) {
        const int items = static_cast<int>(std::min<int64_t>(chunk, shots - c0));
        NZ_CUDA(cudaMemcpyAsync(duni.p, uniforms + c0 * ndraws, static_cast<size_t>(items) * ndraws * 8,
                                cudaMemcpyHostToDevice, st),
                "uniform upload");
        if (psi_in) NZ_CUDA(launch_items_copy(dstate.p, n, items, dpsi0.p, st), "initial states");
        else NZ_CUDA(launch_zero_items(QFVM_C128, dstate.p, n, items, st), "initial states");
        g_launches.fetch_add(1, std::memory_order_relaxed);
        for (const auto& sg : segs) {
            if (sg.type == 0) {
                NZ_TRY(run_plan_items(sg.plan, dstate.p, items, nullptr, st));
            } else {
                NZ_CUDA(launch_channel(dstate.p, n, sg.q, sg.m, sg.kraus, sg.cross, dcd + sg.mat_off, dcd + sg.prob_off,
                                       items,
                                       duni.as<double>(), sg.draw, ndraws, dpart, dimat, st),
                        "channel");
                g_launches.fetch_add(sg.kraus ? 3 : 2, std::memory_order_relaxed);
            }
        }
        NZ_CUDA(launch_item_sample(dstate.p, n, items, duni.as<double>(), ndraws - 1, ndraws, dsmp, st), "sample");
        g_launches.fetch_add(1, std::memory_order_relaxed);
        NZ_CUDA(cudaMemcpyAsync(samples + c0, dsmp, static_cast<size_t>(items) * 8, cudaMemcpyDeviceToHost, st),
                "sample download");
        if (n_terms > 0) {
            NZ_CUDA(launch_expect_seg(QFVM_C128, dstate.p, n, items, dx, dz, dy, dc, doptr, static_cast<int>(n_terms),
                                      depart, dev, st),
                    "expectation");
            g_launches.fetch_add(2, std::memory_order_relaxed);
            NZ_CUDA(cudaMemcpyAsync(expvals + c0 * n_terms, dev, static_cast<size_t>(items) * n_terms * 8,
                                    cudaMemcpyDeviceToHost, st),
                    "expectation download");
        }
        NZ_CUDA(cudaStreamSynchronize(st), "noisy trajectories");
        if (const int src = check_status(st)) return done(src);
    }
    return done(QFVM_OK);
#undef NZ_CUDA
#undef NZ_TRY
}

}  // extern "C"
