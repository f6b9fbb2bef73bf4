// C ABI of the GB300 statevector engine (declared in include/qfvm_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"
#include "kernels.h"
#include "qfvm_gb300.h"
#include "capi_internal.h"
#include "jit.h"

using namespace qsv;

namespace qsv_capi {

thread_local std::string g_err;
std::atomic<uint64_t> g_launches{0};

namespace {
std::atomic<int> g_c128_arith{QFVM_C128_DS};
std::atomic<int> g_fault_kind{FAULT_NONE};
std::atomic<int64_t> g_fault_count{0};
}  // namespace

int c128_arith() { return g_c128_arith.load(std::memory_order_relaxed); }

bool fault_hit(int kind) {
    if (g_fault_kind.load(std::memory_order_relaxed) != kind) return false;
    if (g_fault_count.fetch_sub(1) != 1) return false;
    g_fault_kind.store(FAULT_NONE);
    return true;
}

cudaError_t dev_malloc(void** p, size_t bytes) {
    if (fault_hit(FAULT_ALLOC)) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}
std::mutex g_boundary_mu;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int check_status(cudaStream_t st) {
    const int rc = jit_status_take(st);
    if (rc == QFVM_ERR_TIMEOUT) return fail(rc, "a specialised pass gave up waiting for its tile copies");
    if (rc == QFVM_ERR_BOUNDS) return fail(rc, "a bounds-checked specialised pass found an index out of range");
    if (rc != QFVM_OK) return fail(rc, "reading the device status word");
    return QFVM_OK;
}

int check_device() {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return fail(QFVM_ERR_NODEVICE, "no CUDA device available");
    return QFVM_OK;
}

}  // namespace qsv_capi

using namespace qsv_capi;


namespace qsv_capi {

int upload_plan(qfvm_plan* p) {
    const HostPlan& hp = p->hp;
    const bool f32 = hp.arith == QFVM_C64;
    const bool dsp = hp.arith == QFVM_C128_DS;
    const size_t b_pass = align256(hp.passes.size() * sizeof(PassDesc));
    const size_t b_steps = align256(std::max<size_t>(hp.steps.size(), 1) * sizeof(StepDesc));
    const size_t b_ops = align256(std::max<size_t>(hp.ops.size(), 1) * sizeof(KOp));
    const size_t b_coef = align256(std::max<size_t>(hp.coef.size(), 1) * (f32 ? sizeof(float) : sizeof(double)));
    // (a double-single coefficient is a float pair: same 8 bytes as a double)
    const size_t total = b_pass + b_steps + b_ops + b_coef;
    std::vector<unsigned char> host(total, 0);
    std::memcpy(host.data(), hp.passes.data(), hp.passes.size() * sizeof(PassDesc));
    if (!hp.steps.empty()) std::memcpy(host.data() + b_pass, hp.steps.data(), hp.steps.size() * sizeof(StepDesc));
    if (!hp.ops.empty()) std::memcpy(host.data() + b_pass + b_steps, hp.ops.data(), hp.ops.size() * sizeof(KOp));
    unsigned char* cdst = host.data() + b_pass + b_steps + b_ops;
    if (f32) {
        float* f = reinterpret_cast<float*>(cdst);
        for (size_t i = 0; i < hp.coef.size(); ++i) f[i] = static_cast<float>(hp.coef[i]);
    } else if (dsp) {
        float* f = reinterpret_cast<float*>(cdst);
        for (size_t i = 0; i < hp.coef.size(); ++i) {
            const float h = static_cast<float>(hp.coef[i]);
            f[2 * i] = h;
            f[2 * i + 1] = static_cast<float>(hp.coef[i] - static_cast<double>(h));
        }
    } else if (!hp.coef.empty()) {
        std::memcpy(cdst, hp.coef.data(), hp.coef.size() * sizeof(double));
    }
    QSV_CUDA(dev_malloc(&p->dbuf, total), "plan allocation");
    QSV_CUDA(cudaMemcpy(p->dbuf, host.data(), total, cudaMemcpyHostToDevice), "plan upload");
    unsigned char* b = static_cast<unsigned char*>(p->dbuf);
    p->dpass = reinterpret_cast<PassDesc*>(b);
    p->dsteps = reinterpret_cast<StepDesc*>(b + b_pass);
    p->dops = reinterpret_cast<KOp*>(b + b_pass + b_steps);
    p->dcoef = b + b_pass + b_steps + b_ops;
    return QFVM_OK;
}

int make_plan(int n, int precision, const qfvm_op* ops, int64_t n_ops, const double* matpool, int64_t matpool_len,
              int T, int R, qfvm_plan** out) {
    if (n < 1 || n > QFVM_MAX_QUBITS) return fail(QFVM_ERR_INVALID, "qubit count out of range");
    if (n_ops < 0 || (n_ops > 0 && ops == nullptr)) return fail(QFVM_ERR_INVALID, "bad op list");
    std::vector<GOp> gops;
    std::string err;
    if (!classify(n, ops, n_ops, matpool, matpool_len, &gops, &err)) return fail(QFVM_ERR_INVALID, err);
    fuse_single_qubit(&gops);
    unnormalize_hadamards(&gops);
    const int sp = store_precision(precision);
    if (T > 0 || R > 0) {
        int dT, dR;
        default_shape(n, sp, &dT, &dR);
        const int tt = T > 0 ? T : dT, rr = R > 0 ? R : dR;
        if (!pass_shape_supported(precision == QFVM_C128_DS ? QFVM_C128_DS : sp, tt, rr))
            return fail(QFVM_ERR_INVALID, "tile shape not compiled in");
    }
    return make_plan_gops(n, precision, gops, T, R, out, true);
}

int make_plan_gops(int n, int precision, const std::vector<GOp>& gops, int T, int R, qfvm_plan** out,
                   bool merge_diagonals) {
    std::string err;
    const int sp = store_precision(precision);
    if (T <= 0 && R <= 0) resolve_shape(precision, 0, n, &T, &R);
    qfvm_plan* p = new qfvm_plan();
    if (!build_plan(n, sp, gops, T, R, &p->hp, &err)) {
        delete p;
        return fail(QFVM_ERR_INVALID, err);
    }
    if (merge_diagonals) merge_round_diagonals(&p->hp);
    p->hp.arith = (precision == QFVM_C128_DS) ? QFVM_C128_DS : sp;
    int rc = upload_plan(p);
    if (rc != QFVM_OK) {
        if (p->dbuf) cudaFree(p->dbuf);
        delete p;
        return rc;
    }
    *out = p;
    return QFVM_OK;
}

void free_plan(qfvm_plan* p) {
    if (!p) return;
    jit_release(p);
    for (cudaEvent_t e : p->events) cudaEventDestroy(e);
    if (p->dbuf) cudaFree(p->dbuf);
    delete p;
}

int run_plan(qfvm_plan* p, qfvm_sv* sv, bool timed = false) {
    const HostPlan& hp = p->hp;
    if (hp.n != sv->n || hp.precision != sv->precision) return fail(QFVM_ERR_INVALID, "plan/state mismatch");
    if (timed && p->events.size() != hp.passes.size() + 1) {
        for (cudaEvent_t e : p->events) cudaEventDestroy(e);
        p->events.assign(hp.passes.size() + 1, nullptr);
        for (auto& e : p->events) QSV_CUDA(cudaEventCreate(&e), "event");
    }
    if (timed) QSV_CUDA(cudaEventRecord(p->events[0], sv->stream), "event record");
    for (size_t i = 0; i < hp.passes.size(); ++i) {
        const PassDesc& pd = hp.passes[i];
        if (fault_hit(FAULT_STAGE)) return fail(QFVM_ERR_CUDA, "pass launch: injected kernel-stage failure");
        NvtxRange range(pd.type == PASS_TILE ? "qfvm tile pass" : (pd.type == PASS_SMALL ? "qfvm whole-state pass"
                                                                                        : "qfvm global op"));
        cudaError_t e = cudaSuccess;
        if (pd.type == PASS_TILE) {
            bool done = false;
            e = jit_launch_pass(p, static_cast<int>(i), sv->d, nullptr, p->dcoef, 1, 0, nullptr, 0, nullptr, nullptr,
                                sv->stream, &done);
            if (e == cudaSuccess && !done)
                e = launch_tile_pass(hp.arith, hp.T, hp.R, sv->d, p->dpass + i, p->dsteps, p->dops, p->dcoef, hp.n,
                                     pd.H, 1, 0, nullptr, sv->stream);
        } else if (pd.type == PASS_SMALL) {
            e = launch_small(hp.arith, sv->d, 0, 1, hp.n, p->dops + pd.op_begin, pd.op_count, p->dcoef, 0, nullptr, sv->stream);
        } else {
            e = launch_globalop(hp.arith, sv->d, hp.n, hp.ops[pd.op_begin].k, p->dops + pd.op_begin, p->dcoef, 1, 0, nullptr, sv->stream);
        }
        g_launches.fetch_add(1, std::memory_order_relaxed);
        if (e != cudaSuccess) return fail(QFVM_ERR_CUDA, std::string("pass launch: ") + cudaGetErrorString(e));
        if (timed) QSV_CUDA(cudaEventRecord(p->events[i + 1], sv->stream), "event record");
    }
    return QFVM_OK;
}

int sv_create(int n, int precision, qfvm_sv** out) {
    QSV_TRY(check_device());
    if (n < 1 || n > QFVM_MAX_QUBITS) return fail(QFVM_ERR_INVALID, "qubit count out of range");
    if (precision != QFVM_C128 && precision != QFVM_C64 && precision != QFVM_C128_DS)
        return fail(QFVM_ERR_INVALID, "unknown precision");
    qfvm_sv* sv = new qfvm_sv();
    sv->n = n;
    sv->precision = store_precision(precision);
    sv->arith = precision;
    sv->N = 1ULL << n;
    cudaError_t e = cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete sv;
        return fail(QFVM_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(e));
    }
    e = dev_malloc(&sv->d, sv->N * amp_bytes(sv->precision));
    if (e != cudaSuccess) {
        cudaStreamDestroy(sv->stream);
        delete sv;
        return fail(e == cudaErrorMemoryAllocation ? QFVM_ERR_NOMEM : QFVM_ERR_CUDA,
                    std::string("state allocation: ") + cudaGetErrorString(e));
    }
    *out = sv;
    return QFVM_OK;
}

void sv_free(qfvm_sv* sv) {
    if (!sv) return;
    if (sv->stream) cudaStreamSynchronize(sv->stream);
    if (sv->d) cudaFree(sv->d);
    sv->red.release();
    sv->masks.release();
    sv->sample_blk.release();
    sv->sample_shots.release();
    sv->staging.release();
    if (sv->stream) cudaStreamDestroy(sv->stream);
    delete sv;
}

int sv_set_zero(qfvm_sv* sv) {
    cudaError_t e = launch_set_basis(sv->precision, sv->d, sv->N, 0, sv->stream);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    QSV_CUDA(e, "set_zero");
    return QFVM_OK;
}

constexpr uint64_t STAGE_AMPS = 1ULL << 24;

int sv_upload(qfvm_sv* sv, const double* host, uint64_t n_amps) {
    if (n_amps != sv->N) return fail(QFVM_ERR_INVALID, "state length does not match the device state");
    if (!host) return fail(QFVM_ERR_INVALID, "null host buffer");
    if (sv->precision == QFVM_C128) {
        QSV_CUDA(cudaMemcpyAsync(sv->d, host, sv->N * 16, cudaMemcpyHostToDevice, sv->stream), "upload");
        QSV_CUDA(cudaStreamSynchronize(sv->stream), "upload sync");
        return QFVM_OK;
    }
    const uint64_t chunk = std::min<uint64_t>(STAGE_AMPS, sv->N);
    QSV_TRY(sv->staging.ensure(chunk * 16));
    for (uint64_t off = 0; off < sv->N; off += chunk) {
        const uint64_t m = std::min(chunk, sv->N - off);
        QSV_CUDA(cudaMemcpyAsync(sv->staging.p, host + 2 * off, m * 16, cudaMemcpyHostToDevice, sv->stream),
                 "upload");
        QSV_CUDA(launch_convert(true, sv->staging.p, static_cast<float2*>(sv->d) + off, m, sv->stream), "convert");
        g_launches.fetch_add(1, std::memory_order_relaxed);
        QSV_CUDA(cudaStreamSynchronize(sv->stream), "upload sync");
    }
    return QFVM_OK;
}

int sv_download(qfvm_sv* sv, double* host, uint64_t n_amps) {
    if (n_amps != sv->N) return fail(QFVM_ERR_INVALID, "state length does not match the device state");
    if (!host) return fail(QFVM_ERR_INVALID, "null host buffer");
    if (sv->precision == QFVM_C128) {
        QSV_CUDA(cudaMemcpyAsync(host, sv->d, sv->N * 16, cudaMemcpyDeviceToHost, sv->stream), "download");
        QSV_CUDA(cudaStreamSynchronize(sv->stream), "download sync");
        return check_status(sv->stream);
    }
    const uint64_t chunk = std::min<uint64_t>(STAGE_AMPS, sv->N);
    QSV_TRY(sv->staging.ensure(chunk * 16));
    for (uint64_t off = 0; off < sv->N; off += chunk) {
        const uint64_t m = std::min(chunk, sv->N - off);
        QSV_CUDA(launch_convert(false, static_cast<float2*>(sv->d) + off, sv->staging.p, m, sv->stream), "convert");
        g_launches.fetch_add(1, std::memory_order_relaxed);
        QSV_CUDA(cudaMemcpyAsync(host + 2 * off, sv->staging.p, m * 16, cudaMemcpyDeviceToHost, sv->stream),
                 "download");
        QSV_CUDA(cudaStreamSynchronize(sv->stream), "download sync");
    }
    return check_status(sv->stream);
}

int sv_expect(qfvm_sv* sv, const uint64_t* xm, const uint64_t* zm, const int32_t* ny, int64_t nterms, double* out) {
    NvtxRange range("qfvm expectation");
    if (nterms < 0) return fail(QFVM_ERR_INVALID, "negative term count");
    if (nterms == 0) return QFVM_OK;
    if (!xm || !zm || !ny || !out) return fail(QFVM_ERR_INVALID, "null term buffer");
    const uint64_t lim = sv->n >= 64 ? ~0ULL : ((1ULL << sv->n) - 1);
    for (int64_t t = 0; t < nterms; ++t)
        if ((xm[t] | zm[t]) & ~lim) return fail(QFVM_ERR_INVALID, "Pauli term acts outside the state");
    // group terms by flip mask, in first-seen order
    std::vector<uint64_t> keys;
    std::vector<std::vector<int64_t>> groups;
    for (int64_t t = 0; t < nterms; ++t) {
        auto it = std::find(keys.begin(), keys.end(), xm[t]);
        if (it == keys.end()) {
            keys.push_back(xm[t]);
            groups.push_back({t});
        } else {
            groups[it - keys.begin()].push_back(t);
        }
    }
    // launch batches of up to EXPECT_BATCH terms
    std::vector<uint64_t> hz;
    std::vector<int32_t> hy;
    std::vector<std::pair<int64_t, int>> where;  // (term, batch slot)
    struct Batch {
        uint64_t x;
        size_t first;
        int count;
    };
    std::vector<Batch> batches;
    for (size_t g = 0; g < groups.size(); ++g) {
        for (size_t s = 0; s < groups[g].size(); s += EXPECT_BATCH) {
            Batch b{keys[g], hz.size(), 0};
            for (size_t k = s; k < groups[g].size() && k < s + EXPECT_BATCH; ++k) {
                hz.push_back(zm[groups[g][k]]);
                hy.push_back(ny[groups[g][k]]);
                ++b.count;
            }
            batches.push_back(b);
        }
    }
    // order of terms as laid out in hz
    std::vector<int64_t> order;
    for (auto& g : groups)
        for (int64_t t : g) order.push_back(t);
    const size_t nt = hz.size();
    QSV_TRY(sv->masks.ensure(align256(nt * 8) + align256(nt * 4) + align256(nt * 8)));
    uint64_t* dz = sv->masks.as<uint64_t>();
    int32_t* dy = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(sv->masks.p) + align256(nt * 8));
    double* dout = reinterpret_cast<double*>(reinterpret_cast<char*>(sv->masks.p) + align256(nt * 8) + align256(nt * 4));
    QSV_TRY(sv->red.ensure(static_cast<size_t>(REDUCE_BLOCKS) * EXPECT_BATCH * sizeof(double)));
    QSV_CUDA(cudaMemcpyAsync(dz, hz.data(), nt * 8, cudaMemcpyHostToDevice, sv->stream), "term upload");
    QSV_CUDA(cudaMemcpyAsync(dy, hy.data(), nt * 4, cudaMemcpyHostToDevice, sv->stream), "term upload");
    const int nblocks = static_cast<int>(std::min<uint64_t>(REDUCE_BLOCKS, std::max<uint64_t>(1, sv->N / 2048)));
    for (const Batch& b : batches) {
        cudaError_t e;
        if (b.x == 0) {
            e = launch_expect_z(sv->precision, sv->d, sv->N, dz + b.first, b.count, sv->red.as<double>(), nblocks,
                                sv->stream);
        } else {
            const int flip_q = 63 - __builtin_clzll(b.x);
            e = launch_expect_x(sv->precision, sv->d, sv->N, b.x, flip_q, dz + b.first, dy + b.first, b.count,
                                sv->red.as<double>(), nblocks, sv->stream);
        }
        QSV_CUDA(e, "expectation");
        QSV_CUDA(launch_reduce_partials(sv->red.as<double>(), nblocks, b.count, dout + b.first, sv->stream),
                 "expectation reduce");
        g_launches.fetch_add(2, std::memory_order_relaxed);
    }
    std::vector<double> res(nt);
    QSV_CUDA(cudaMemcpyAsync(res.data(), dout, nt * 8, cudaMemcpyDeviceToHost, sv->stream), "result download");
    QSV_CUDA(cudaStreamSynchronize(sv->stream), "expectation sync");
    QSV_TRY(check_status(sv->stream));
    for (size_t i = 0; i < nt; ++i) out[order[i]] = res[i];
    return QFVM_OK;
}

int sv_sample(qfvm_sv* sv, const double* uni, int64_t shots, uint64_t* out) {
    NvtxRange range("qfvm sampling");
    if (shots < 0) return fail(QFVM_ERR_INVALID, "negative shot count");
    if (shots == 0) return QFVM_OK;
    if (!uni || !out) return fail(QFVM_ERR_INVALID, "null sample buffer");
    // the approximate total (parallel FP64 block sums) fixes the candidate binades
    const uint64_t bs = std::min<uint64_t>(4096, sv->N);
    const uint64_t nbs = sv->N / bs;
    const uint64_t nb = (sv->N + SAMPLE_BS - 1) / SAMPLE_BS;
    const size_t b_bsum = align256(nbs * 8), b_pre = align256((nbs + 1) * 8);
    const size_t b_cnt = align256(static_cast<size_t>(SAMPLE_BINADES) * nb * 8);
    const size_t b_ties = align256(static_cast<size_t>(SAMPLE_BINADES) * nb);
    const size_t b_start = align256((nb + 1) * 8);
    QSV_TRY(sv->sample_blk.ensure(b_bsum + b_pre + b_cnt + b_ties + b_start + 256));
    char* blk = static_cast<char*>(sv->sample_blk.p);
    double* dbsum = reinterpret_cast<double*>(blk);
    double* dpre = reinterpret_cast<double*>(blk + b_bsum);
    uint64_t* dcnt = reinterpret_cast<uint64_t*>(blk + b_bsum + b_pre);
    uint8_t* dties = reinterpret_cast<uint8_t*>(blk + b_bsum + b_pre + b_cnt);
    double* dstart = reinterpret_cast<double*>(blk + b_bsum + b_pre + b_cnt + b_ties);
    int64_t* dseq = reinterpret_cast<int64_t*>(blk + b_bsum + b_pre + b_cnt + b_ties + b_start);
    const size_t sz = static_cast<size_t>(shots);
    QSV_TRY(sv->sample_shots.ensure(align256(sz * 8) * 2));
    char* sb = static_cast<char*>(sv->sample_shots.p);
    double* duni = reinterpret_cast<double*>(sb);
    uint64_t* didx = reinterpret_cast<uint64_t*>(sb + align256(sz * 8));
    QSV_CUDA(cudaMemcpyAsync(duni, uni, sz * 8, cudaMemcpyHostToDevice, sv->stream), "uniform upload");
    QSV_CUDA(launch_block_prefix(sv->precision, sv->d, sv->N, bs, dbsum, dpre, sv->stream), "block sums");
    double total = 0.0;
    QSV_CUDA(cudaMemcpyAsync(&total, dpre + nbs, 8, cudaMemcpyDeviceToHost, sv->stream), "total download");
    QSV_CUDA(cudaStreamSynchronize(sv->stream), "sampling sync");
    // binade of a value a little above the total (so a sequential total just
    // past a power of two is still covered)
    int e_top = 0;
    const double tb = total * (1.0 + 1.0 / (1 << 20));
    if (tb > 0.0 && std::isfinite(tb)) {
        std::frexp(tb, &e_top);  // tb = f * 2^e_top, f in [0.5, 1)
        e_top -= 1;
    }
    QSV_CUDA(launch_sample_binade(sv->precision, sv->d, sv->N, e_top, dcnt, dties, dstart, dseq, duni, shots, didx,
                                  sv->stream),
             "exact sampling");
    g_launches.fetch_add(5, std::memory_order_relaxed);
    int64_t seq = 0;
    QSV_CUDA(cudaMemcpyAsync(out, didx, sz * 8, cudaMemcpyDeviceToHost, sv->stream), "sample download");
    QSV_CUDA(cudaMemcpyAsync(&seq, dseq, 8, cudaMemcpyDeviceToHost, sv->stream), "sample download");
    QSV_CUDA(cudaStreamSynchronize(sv->stream), "sampling sync");
    sv->last_seq_blocks = seq;
    return check_status(sv->stream);
}

// Process-wide cached state for the host-buffer entry points (one per
// storage precision), so repeated calls do not re-allocate HBM.
qfvm_sv* g_cached[2] = {nullptr, nullptr};

int cached_state(int n, int precision, qfvm_sv** out) {
    const int k = store_precision(precision) == QFVM_C64 ? 1 : 0;
    if (g_cached[k] && g_cached[k]->n == n) {
        g_cached[k]->arith = precision;
        *out = g_cached[k];
        return QFVM_OK;
    }
    if (g_cached[k]) {
        sv_free(g_cached[k]);
        g_cached[k] = nullptr;
    }
    QSV_TRY(sv_create(n, precision, &g_cached[k]));
    *out = g_cached[k];
    return QFVM_OK;
}

// Plans of the last few circuits simulate_circuit saw, keyed by the raw op
// records and matrix pool (callers that re-run one circuit, as a sampling or
// parameter loop does, skip classification, fusion, the plan upload and the
// specialised-kernel lookup).  Guarded by g_boundary_mu.
struct CachedPlan {
    int n = 0, arith = 0;
    std::vector<unsigned char> key;
    qfvm_plan* plan = nullptr;
};
std::vector<CachedPlan> g_plan_cache;
constexpr size_t PLAN_CACHE_SIZE = 4;

int cached_plan(int n, int arith, const qfvm_op* ops, int64_t n_ops, const double* matpool, int64_t matpool_len,
                qfvm_plan** out) {
    if (n_ops < 0 || (n_ops > 0 && !ops) || matpool_len < 0 || (matpool_len > 0 && !matpool))
        return fail(QFVM_ERR_INVALID, "bad op list");
    std::vector<unsigned char> key(static_cast<size_t>(n_ops) * sizeof(qfvm_op) +
                                   static_cast<size_t>(matpool_len) * sizeof(double));
    if (n_ops) std::memcpy(key.data(), ops, static_cast<size_t>(n_ops) * sizeof(qfvm_op));
    if (matpool_len)
        std::memcpy(key.data() + static_cast<size_t>(n_ops) * sizeof(qfvm_op), matpool,
                    static_cast<size_t>(matpool_len) * sizeof(double));
    for (size_t i = 0; i < g_plan_cache.size(); ++i) {
        CachedPlan& c = g_plan_cache[i];
        if (c.n == n && c.arith == arith && c.key == key) {
            std::rotate(g_plan_cache.begin(), g_plan_cache.begin() + static_cast<std::ptrdiff_t>(i),
                        g_plan_cache.begin() + static_cast<std::ptrdiff_t>(i) + 1);
            *out = g_plan_cache.front().plan;
            return QFVM_OK;
        }
    }
    qfvm_plan* p = nullptr;
    QSV_TRY(make_plan(n, arith, ops, n_ops, matpool, matpool_len, 0, 0, &p));
    CachedPlan c;
    c.n = n;
    c.arith = arith;
    c.key = std::move(key);
    c.plan = p;
    g_plan_cache.insert(g_plan_cache.begin(), std::move(c));
    if (g_plan_cache.size() > PLAN_CACHE_SIZE) {
        free_plan(g_plan_cache.back().plan);
        g_plan_cache.pop_back();
    }
    *out = p;
    return QFVM_OK;
}

int log2_len(uint64_t len, int* n) {
    if (len < 2 || (len & (len - 1)) != 0) return fail(QFVM_ERR_INVALID, "state length must be a power of two >= 2");
    int k = 0;
    while ((1ULL << k) < len) ++k;
    if (k > QFVM_MAX_QUBITS) return fail(QFVM_ERR_INVALID, "state too large");
    *n = k;
    return QFVM_OK;
}

}  // namespace

extern "C" {

const char* qfvm_last_error(void) { return g_err.c_str(); }
int32_t qfvm_abi_version(void) { return QFVM_ABI_VERSION; }
uint64_t qfvm_launch_count(void) { return g_launches.load(); }

int qfvm_set_c128_arithmetic(int32_t arith) {
    if (arith != QFVM_C128 && arith != QFVM_C128_DS)
        return fail(QFVM_ERR_INVALID, "complex128 arithmetic must be QFVM_C128 or QFVM_C128_DS");
    g_c128_arith.store(arith);
    return QFVM_OK;
}
int32_t qfvm_get_c128_arithmetic(void) { return c128_arith(); }

int qfvm_test_fault(int32_t kind, int64_t countdown) {
    if (kind < FAULT_NONE || kind > QFVM_FAULT_WAIT) return fail(QFVM_ERR_INVALID, "fault kind must be 0 .. 3");
    if (kind != FAULT_NONE && countdown < 1) return fail(QFVM_ERR_INVALID, "fault countdown must be >= 1");
    if (kind == QFVM_FAULT_WAIT) {
        if (countdown > 10000) return fail(QFVM_ERR_INVALID, "wait limit above 10 s");
        jit_set_wait_test(16, static_cast<uint64_t>(countdown) * 1000000ull);
        return QFVM_OK;
    }
    if (kind == FAULT_NONE) jit_set_wait_test(0, 0);
    g_fault_kind.store(FAULT_NONE);
    g_fault_count.store(countdown);
    g_fault_kind.store(kind);
    return QFVM_OK;
}

int qfvm_sv_create(int32_t num_qubits, int32_t precision, qfvm_sv** out) {
    if (!out) return fail(QFVM_ERR_INVALID, "null output");
    return sv_create(num_qubits, precision, out);
}
int qfvm_sv_destroy(qfvm_sv* sv) {
    sv_free(sv);
    return QFVM_OK;
}
int qfvm_sv_set_zero(qfvm_sv* sv) {
    if (!sv) return fail(QFVM_ERR_INVALID, "null state");
    QSV_TRY(sv_set_zero(sv));
    QSV_CUDA(cudaStreamSynchronize(sv->stream), "set_zero sync");
    return QFVM_OK;
}
int qfvm_sv_upload(qfvm_sv* sv, const double* host, uint64_t n_amps) {
    if (!sv) return fail(QFVM_ERR_INVALID, "null state");
    return sv_upload(sv, host, n_amps);
}
int qfvm_sv_download(qfvm_sv* sv, double* host, uint64_t n_amps) {
    if (!sv) return fail(QFVM_ERR_INVALID, "null state");
    return sv_download(sv, host, n_amps);
}
int qfvm_sv_apply(qfvm_sv* sv, const qfvm_op* ops, int64_t n_ops, const double* matpool, int64_t matpool_len) {
    if (!sv) return fail(QFVM_ERR_INVALID, "null state");
    qfvm_plan* p = nullptr;
    QSV_TRY(make_plan(sv->n, sv->arith, ops, n_ops, matpool, matpool_len, 0, 0, &p));
    int rc = run_plan(p, sv);
    cudaError_t e = cudaStreamSynchronize(sv->stream);
    free_plan(p);
    if (rc != QFVM_OK) return rc;
    QSV_CUDA(e, "apply sync");
    return check_status(sv->stream);
}
int qfvm_sv_expect(qfvm_sv* sv, const uint64_t* x_masks, const uint64_t* z_masks, const int32_t* y_counts,
                   int64_t n_terms, double* out) {
    if (!sv) return fail(QFVM_ERR_INVALID, "null state");
    return sv_expect(sv, x_masks, z_masks, y_counts, n_terms, out);
}
int qfvm_sv_sample(qfvm_sv* sv, const double* uniforms, int64_t shots, uint64_t* out_indices) {
    if (!sv) return fail(QFVM_ERR_INVALID, "null state");
    return sv_sample(sv, uniforms, shots, out_indices);
}
int qfvm_sv_sample_stats(qfvm_sv* sv, int64_t* sequential_blocks) {
    if (!sv || !sequential_blocks) return fail(QFVM_ERR_INVALID, "null argument");
    *sequential_blocks = sv->last_seq_blocks;
    return QFVM_OK;
}
int qfvm_sv_norm2(qfvm_sv* sv, double* out) {
    if (!sv || !out) return fail(QFVM_ERR_INVALID, "null argument");
    uint64_t x = 0, z = 0;
    int32_t y = 0;
    return sv_expect(sv, &x, &z, &y, 1, out);
}
int qfvm_sv_device_ptr(qfvm_sv* sv, void** dev_ptr, uint64_t* nbytes) {
    if (!sv) return fail(QFVM_ERR_INVALID, "null state");
    if (dev_ptr) *dev_ptr = sv->d;
    if (nbytes) *nbytes = sv->N * amp_bytes(sv->precision);
    return QFVM_OK;
}
int qfvm_sv_stream(qfvm_sv* sv, void** stream) {
    if (!sv || !stream) return fail(QFVM_ERR_INVALID, "null argument");
    *stream = sv->stream;
    return QFVM_OK;
}

int qfvm_plan_create(int32_t num_qubits, int32_t precision, const qfvm_op* ops, int64_t n_ops, const double* matpool,
                     int64_t matpool_len, int32_t tile_qubits, int32_t reg_qubits, qfvm_plan** out) {
    if (!out) return fail(QFVM_ERR_INVALID, "null output");
    QSV_TRY(check_device());
    return make_plan(num_qubits, precision, ops, n_ops, matpool, matpool_len, tile_qubits, reg_qubits, out);
}
int qfvm_plan_destroy(qfvm_plan* plan) {
    free_plan(plan);
    return QFVM_OK;
}
int qfvm_plan_stats(const qfvm_plan* plan, int64_t* passes, int64_t* rounds, int64_t* gates, double* pass_bytes,
                    double* gate_bytes) {
    if (!plan) return fail(QFVM_ERR_INVALID, "null plan");
    const PlanStats& s = plan->hp.stats;
    if (passes) *passes = s.passes;
    if (rounds) *rounds = s.rounds;
    if (gates) *gates = s.gates;
    if (pass_bytes) *pass_bytes = s.pass_bytes;
    if (gate_bytes) *gate_bytes = s.gate_bytes;
    return QFVM_OK;
}
int qfvm_plan_run(qfvm_plan* plan, qfvm_sv* sv) {
    if (!plan || !sv) return fail(QFVM_ERR_INVALID, "null argument");
    if (!plan->dbuf) return fail(QFVM_ERR_INVALID, "host-only plan cannot run");
    return run_plan(plan, sv);
}

int qfvm_plan_run_timed(qfvm_plan* plan, qfvm_sv* sv, float* pass_ms, int32_t* pass_type) {
    if (!plan || !sv) return fail(QFVM_ERR_INVALID, "null argument");
    if (!plan->dbuf) return fail(QFVM_ERR_INVALID, "host-only plan cannot run");
    QSV_TRY(run_plan(plan, sv, true));
    QSV_CUDA(cudaEventSynchronize(plan->events.back()), "timed run sync");
    QSV_TRY(check_status(sv->stream));
    for (size_t i = 0; i < plan->hp.passes.size(); ++i) {
        float ms = 0.f;
        QSV_CUDA(cudaEventElapsedTime(&ms, plan->events[i], plan->events[i + 1]), "elapsed");
        if (pass_ms) pass_ms[i] = ms;
        if (pass_type) pass_type[i] = plan->hp.passes[i].type;
    }
    return QFVM_OK;
}

int qfvm_plan_host_build(int32_t num_qubits, int32_t precision, const qfvm_op* ops, int64_t n_ops,
                         const double* matpool, int64_t matpool_len, int32_t tile_qubits, int32_t reg_qubits,
                         qfvm_plan** out) {
    if (!out) return fail(QFVM_ERR_INVALID, "null output");
    if (num_qubits < 1 || num_qubits > QFVM_MAX_QUBITS) return fail(QFVM_ERR_INVALID, "qubit count out of range");
    if (n_ops < 0 || (n_ops > 0 && ops == nullptr)) return fail(QFVM_ERR_INVALID, "bad op list");
    std::vector<GOp> gops;
    std::string err;
    if (!classify(num_qubits, ops, n_ops, matpool, matpool_len, &gops, &err)) return fail(QFVM_ERR_INVALID, err);
    fuse_single_qubit(&gops);
    unnormalize_hadamards(&gops);
    if (tile_qubits > 0 || reg_qubits > 0) {
        int dT, dR;
        default_shape(num_qubits, store_precision(precision), &dT, &dR);
        const int tt = tile_qubits > 0 ? tile_qubits : dT, rr = reg_qubits > 0 ? reg_qubits : dR;
        if (!pass_shape_supported(store_precision(precision), tt, rr))
            return fail(QFVM_ERR_INVALID, "tile shape not compiled in");
    } else {
        resolve_shape(precision, 0, num_qubits, &tile_qubits, &reg_qubits);
    }
    qfvm_plan* p = new qfvm_plan();
    if (!build_plan(num_qubits, store_precision(precision), gops, tile_qubits, reg_qubits, &p->hp, &err)) {
        delete p;
        return fail(QFVM_ERR_INVALID, err);
    }
    p->hp.arith = precision;
    merge_round_diagonals(&p->hp);
    *out = p;
    return QFVM_OK;
}

int qfvm_plan_host_build_adjoint(int32_t num_qubits, int32_t precision, const qfvm_op* ops, int64_t n_ops,
                                 const double* matpool, int64_t matpool_len, qfvm_plan** out) {
    if (!out) return fail(QFVM_ERR_INVALID, "null output");
    if (num_qubits < 1 || num_qubits > QFVM_MAX_QUBITS) return fail(QFVM_ERR_INVALID, "qubit count out of range");
    std::vector<GOp> gops, sweep;
    std::string err;
    if (!classify(num_qubits, ops, n_ops, matpool, matpool_len, &gops, &err)) return fail(QFVM_ERR_INVALID, err);
    if (!build_adjoint_sweep(gops, &sweep, &err)) return fail(QFVM_ERR_INVALID, err);
    int aT = 0, aR = 0;
    resolve_shape(precision, 1, num_qubits, &aT, &aR);
    qfvm_plan* p = new qfvm_plan();
    if (!build_plan(num_qubits, store_precision(precision), sweep, aT, aR, &p->hp, &err)) {
        delete p;
        return fail(QFVM_ERR_INVALID, err);
    }
    p->hp.arith = precision;
    *out = p;
    return QFVM_OK;
}

int qfvm_plan_host_build_batched(int32_t num_qubits, int32_t precision, const qfvm_op* ops, int64_t n_ops,
                                 const double* matpool, int64_t matpool_len, int32_t adjoint, qfvm_plan** out) {
    if (!out) return fail(QFVM_ERR_INVALID, "null output");
    if (num_qubits < 1 || num_qubits > QFVM_MAX_QUBITS) return fail(QFVM_ERR_INVALID, "qubit count out of range");
    std::vector<GOp> gops, sweep;
    std::string err;
    if (!classify(num_qubits, ops, n_ops, matpool, matpool_len, &gops, &err)) return fail(QFVM_ERR_INVALID, err);
    if (!unfix_bound(&gops, &err)) return fail(QFVM_ERR_UNSUPPORTED, err);
    int T = 0, R = 0;
    if (adjoint) {
        if (!build_adjoint_sweep(gops, &sweep, &err)) return fail(QFVM_ERR_INVALID, err);
        resolve_shape(precision, 1, num_qubits, &T, &R);
    }
    qfvm_plan* p = new qfvm_plan();
    if (!build_plan(num_qubits, store_precision(precision), adjoint ? sweep : gops, T, R, &p->hp, &err)) {
        delete p;
        return fail(QFVM_ERR_INVALID, err);
    }
    p->hp.arith = precision;
    *out = p;
    return QFVM_OK;
}

int qfvm_plan_host_binds(const qfvm_plan* plan, int64_t* count, int32_t* records) {
    if (!plan || !count) return fail(QFVM_ERR_INVALID, "null argument");
    *count = static_cast<int64_t>(plan->hp.binds.size());
    if (records) {
        for (size_t i = 0; i < plan->hp.binds.size(); ++i) {
            const Bind& b = plan->hp.binds[i];
            records[4 * i] = static_cast<int32_t>(b.off);
            records[4 * i + 1] = b.kind;
            records[4 * i + 2] = b.sign;
            records[4 * i + 3] = b.slot;
        }
    }
    return QFVM_OK;
}

int qfvm_plan_host_probe_slots(const qfvm_plan* plan, int32_t* slots) {
    if (!plan || !slots) return fail(QFVM_ERR_INVALID, "null argument");
    for (size_t i = 0; i < plan->hp.probe_slot.size(); ++i) slots[i] = plan->hp.probe_slot[i];
    return QFVM_OK;
}

int qfvm_plan_host_counts(const qfvm_plan* plan, int64_t counts[4], int32_t shape[3]) {
    if (!plan || !counts || !shape) return fail(QFVM_ERR_INVALID, "null argument");
    counts[0] = static_cast<int64_t>(plan->hp.passes.size());
    counts[1] = static_cast<int64_t>(plan->hp.steps.size());
    counts[2] = static_cast<int64_t>(plan->hp.ops.size());
    counts[3] = static_cast<int64_t>(plan->hp.coef.size());
    shape[0] = plan->hp.T;
    shape[1] = plan->hp.R;
    shape[2] = plan->hp.L;
    return QFVM_OK;
}

int qfvm_plan_host_copy(const qfvm_plan* plan, void* passes, void* steps, void* kops, double* coef) {
    if (!plan) return fail(QFVM_ERR_INVALID, "null plan");
    const HostPlan& hp = plan->hp;
    if (passes) std::memcpy(passes, hp.passes.data(), hp.passes.size() * sizeof(PassDesc));
    if (steps) std::memcpy(steps, hp.steps.data(), hp.steps.size() * sizeof(StepDesc));
    if (kops) std::memcpy(kops, hp.ops.data(), hp.ops.size() * sizeof(KOp));
    if (coef) std::memcpy(coef, hp.coef.data(), hp.coef.size() * sizeof(double));
    return QFVM_OK;
}

int qfvm_simulate_circuit(int32_t num_qubits, const qfvm_op* ops, int64_t n_ops, const double* matpool,
                          int64_t matpool_len, double* state, int32_t state_given, const double* uniforms,
                          int64_t shots, uint64_t* out_indices) {
    std::lock_guard<std::mutex> lk(g_boundary_mu);
    if (!state) return fail(QFVM_ERR_INVALID, "null state buffer");
    QSV_TRY(check_device());
    // QFVM_TRACE=1: wall time of every stage on stderr (stages synchronised)
    static const bool trace = [] {
        const char* e = std::getenv("QFVM_TRACE");
        return e && e[0] == '1';
    }();
    using clk = std::chrono::steady_clock;
    auto t0 = clk::now();
    double ms[6] = {0, 0, 0, 0, 0, 0};
    auto stage = [&](int k, qfvm_sv* s) {
        if (!trace) return;
        if (s) cudaStreamSynchronize(s->stream);
        const auto t1 = clk::now();
        ms[k] = std::chrono::duration<double, std::milli>(t1 - t0).count();
        t0 = t1;
    };
    qfvm_plan* p = nullptr;
    QSV_TRY(cached_plan(num_qubits, c128_arith(), ops, n_ops, matpool, matpool_len, &p));
    stage(0, nullptr);
    qfvm_sv* sv = nullptr;
    int rc = cached_state(num_qubits, QFVM_C128, &sv);
    stage(1, nullptr);
    if (rc == QFVM_OK) rc = state_given ? sv_upload(sv, state, sv->N) : sv_set_zero(sv);
    stage(2, sv);
    if (rc == QFVM_OK) rc = run_plan(p, sv);
    stage(3, sv);
    if (rc == QFVM_OK && shots > 0) rc = sv_sample(sv, uniforms, shots, out_indices);
    if (rc == QFVM_OK) rc = sv_download(sv, state, sv->N);
    stage(4, sv);
    stage(5, nullptr);
    if (trace)
        std::fprintf(stderr,
                     "qfvm trace simulate_circuit: plan %.1f ms, state %.1f ms, upload %.1f ms, run %.1f ms, "
                     "sample+download %.1f ms, release %.1f ms\n",
                     ms[0], ms[1], ms[2], ms[3], ms[4], ms[5]);
    return rc;
}

int qfvm_applyop_statevec(const qfvm_op* op, const double* matpool, int64_t matpool_len, double* state,
                          uint64_t state_len) {
    std::lock_guard<std::mutex> lk(g_boundary_mu);
    if (!op || !state) return fail(QFVM_ERR_INVALID, "null argument");
    int n = 0;
    QSV_TRY(log2_len(state_len, &n));
    QSV_TRY(check_device());
    qfvm_plan* p = nullptr;
    QSV_TRY(make_plan(n, c128_arith(), op, 1, matpool, matpool_len, 0, 0, &p));
    qfvm_sv* sv = nullptr;
    int rc = cached_state(n, QFVM_C128, &sv);
    if (rc == QFVM_OK) rc = sv_upload(sv, state, sv->N);
    if (rc == QFVM_OK) rc = run_plan(p, sv);
    if (rc == QFVM_OK) rc = sv_download(sv, state, sv->N);
    free_plan(p);
    return rc;
}

int qfvm_sampling_statevec(const double* state, uint64_t state_len, const double* uniforms, int64_t shots,
                           uint64_t* out_indices) {
    std::lock_guard<std::mutex> lk(g_boundary_mu);
    if (!state) return fail(QFVM_ERR_INVALID, "null state buffer");
    int n = 0;
    QSV_TRY(log2_len(state_len, &n));
    QSV_TRY(check_device());
    qfvm_sv* sv = nullptr;
    QSV_TRY(cached_state(n, QFVM_C128, &sv));
    QSV_TRY(sv_upload(sv, state, sv->N));
    return sv_sample(sv, uniforms, shots, out_indices);
}

int qfvm_adjoint(int32_t num_qubits, int32_t precision, const qfvm_op* ops, int64_t n_ops, const double* matpool,
                 int64_t matpool_len, const uint64_t* x_masks, const uint64_t* z_masks, const int32_t* y_counts,
                 const double* coeffs, int64_t n_terms, const double* psi_in, double* energy, double* grads,
                 int64_t n_slots) {
    NvtxRange range("qfvm adjoint gradient");
    std::lock_guard<std::mutex> lk(g_boundary_mu);
    const int n = num_qubits;
    if (n < 1 || n > QFVM_MAX_QUBITS) return fail(QFVM_ERR_INVALID, "qubit count out of range");
    if (n_terms < 1 || !x_masks || !z_masks || !y_counts || !coeffs)
        return fail(QFVM_ERR_INVALID, "the observable needs at least one Pauli term");
    if (n_slots < 0 || (n_slots > 0 && !grads)) return fail(QFVM_ERR_INVALID, "bad gradient buffer");
    if (precision != QFVM_C128 && precision != QFVM_C64 && precision != QFVM_C128_DS)
        return fail(QFVM_ERR_INVALID, "unknown precision");
    QSV_TRY(check_device());
    const uint64_t lim = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
    for (int64_t t = 0; t < n_terms; ++t)
        if ((x_masks[t] | z_masks[t]) & ~lim) return fail(QFVM_ERR_INVALID, "Pauli term acts outside the state");
    std::vector<GOp> gops;
    std::string err;
    if (!classify(n, ops, n_ops, matpool, matpool_len, &gops, &err)) return fail(QFVM_ERR_INVALID, err);
    for (const GOp& g : gops)
        if (g.slot >= n_slots) return fail(QFVM_ERR_INVALID, "parameter slot beyond n_slots");
    std::vector<GOp> sweep;
    if (!build_adjoint_sweep(gops, &sweep, &err)) return fail(QFVM_ERR_INVALID, err);
    for (const GOp& g : sweep)
        if (g.kind == K_PROBE && __builtin_popcountll(g.xmask) > 2)
            return fail(QFVM_ERR_UNSUPPORTED, "generators flipping more than two qubits are not supported");
    const int storage = store_precision(precision);
    const int arith = precision;

    // forward pass on psi
    qfvm_plan* fwd = nullptr;
    QSV_TRY(make_plan_gops(n, precision, gops, 0, 0, &fwd));
    int aT = 0, aR = 0;
    resolve_shape(arith, 1, n, &aT, &aR);
    qfvm_plan* rev = nullptr;
    int rc = make_plan_gops(n, precision, sweep, aT, aR, &rev);
    if (rc != QFVM_OK) {
        free_plan(fwd);
        return rc;
    }
    auto done = [&](int code) {
        free_plan(fwd);
        free_plan(rev);
        return code;
    };
#define ADJ_CUDA(call, what)                                                                          \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return done(fail(QFVM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_))); \
    } while (0)
    qfvm_sv* psi = nullptr;
    rc = cached_state(n, storage, &psi);
    if (rc != QFVM_OK) return done(rc);
    static qfvm_sv* lam_cache[2] = {nullptr, nullptr};
    const int ck = storage == QFVM_C64 ? 1 : 0;
    if (!lam_cache[ck] || lam_cache[ck]->n != n) {
        if (lam_cache[ck]) sv_free(lam_cache[ck]);
        lam_cache[ck] = nullptr;
        rc = sv_create(n, storage, &lam_cache[ck]);
        if (rc != QFVM_OK) return done(rc);
    }
    qfvm_sv* lam = lam_cache[ck];
    rc = psi_in ? sv_upload(psi, psi_in, psi->N) : sv_set_zero(psi);
    if (rc == QFVM_OK) rc = run_plan(fwd, psi);
    if (rc != QFVM_OK) return done(rc);

    // energy = sum_t c_t <P_t>
    std::vector<double> ev(static_cast<size_t>(n_terms));
    rc = sv_expect(psi, x_masks, z_masks, y_counts, n_terms, ev.data());
    if (rc != QFVM_OK) return done(rc);
    double e = 0.0;
    for (int64_t t = 0; t < n_terms; ++t) e += coeffs[t] * ev[t];
    if (energy) *energy = e;

    // lam = H psi (terms sorted by flip mask so the kernel reuses loads)
    std::vector<int64_t> ord(static_cast<size_t>(n_terms));
    for (int64_t t = 0; t < n_terms; ++t) ord[t] = t;
    std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return x_masks[a] < x_masks[b]; });
    const size_t nt = static_cast<size_t>(n_terms);
    std::vector<uint64_t> hx(nt), hz(nt);
    std::vector<int32_t> hy(nt);
    std::vector<double> hc(nt);
    for (size_t i = 0; i < nt; ++i) {
        hx[i] = x_masks[ord[i]];
        hz[i] = z_masks[ord[i]];
        hy[i] = y_counts[ord[i]];
        hc[i] = coeffs[ord[i]];
    }
    const size_t nprobe = rev->hp.probe_slot.size();
    const int gcap = pass2_grid_cap();
    const size_t b8 = align256(nt * 8), b4 = align256(nt * 4);
    const size_t bvals = align256(std::max<size_t>(nprobe, 1) * 8);
    const size_t bpart = align256(static_cast<size_t>(MAX_PASS_PROBES) * gcap * 8);
    rc = lam->masks.ensure(3 * b8 + b4 + bvals + bpart);
    if (rc != QFVM_OK) return done(rc);
    char* mb = static_cast<char*>(lam->masks.p);
    uint64_t* dx = reinterpret_cast<uint64_t*>(mb);
    uint64_t* dz = reinterpret_cast<uint64_t*>(mb + b8);
    double* dc = reinterpret_cast<double*>(mb + 2 * b8);
    int32_t* dy = reinterpret_cast<int32_t*>(mb + 3 * b8);
    double* dvals = reinterpret_cast<double*>(mb + 3 * b8 + b4);
    double* dpart = reinterpret_cast<double*>(mb + 3 * b8 + b4 + bvals);
    cudaStream_t st = psi->stream;
    ADJ_CUDA(cudaStreamSynchronize(lam->stream), "adjoint sync");
    ADJ_CUDA(cudaMemcpyAsync(dx, hx.data(), nt * 8, cudaMemcpyHostToDevice, st), "term upload");
    ADJ_CUDA(cudaMemcpyAsync(dz, hz.data(), nt * 8, cudaMemcpyHostToDevice, st), "term upload");
    ADJ_CUDA(cudaMemcpyAsync(dc, hc.data(), nt * 8, cudaMemcpyHostToDevice, st), "term upload");
    ADJ_CUDA(cudaMemcpyAsync(dy, hy.data(), nt * 4, cudaMemcpyHostToDevice, st), "term upload");
    ADJ_CUDA(launch_hamiltonian(storage, psi->d, lam->d, psi->N, dx, dz, dy, dc, static_cast<int>(nt), st),
             "hamiltonian");
    g_launches.fetch_add(1, std::memory_order_relaxed);

    // reverse sweep over both states
    const HostPlan& hp = rev->hp;
    for (size_t i = 0; i < hp.passes.size(); ++i) {
        const PassDesc& pd = hp.passes[i];
        cudaError_t ce = cudaSuccess;
        if (pd.type == PASS_TILE) {
            int grid = 0;
            bool done = false;
            ce = jit_launch_pass(rev, static_cast<int>(i), psi->d, lam->d, rev->dcoef, 1, 0, nullptr, 0, dpart, &grid,
                                 st, &done);
            if (ce == cudaSuccess && !done)
                ce = launch_pass2(arith, hp.T, hp.R, psi->d, lam->d, rev->dpass + i, rev->dsteps, rev->dops, rev->dcoef,
                                  n, pd.H, 1, 0, 0, dpart, &grid, st);
            g_launches.fetch_add(1, std::memory_order_relaxed);
            if (ce == cudaSuccess && pd.nprobe > 0) {
                ce = launch_probe_reduce(dpart, grid, pd.nprobe, dvals + pd.probe_base, st);
                g_launches.fetch_add(1, std::memory_order_relaxed);
            }
        } else if (pd.type == PASS_SMALL) {
            ce = launch_small2(arith, psi->d, lam->d, n, rev->dops + pd.op_begin, pd.op_count, rev->dcoef, 1, 0,
                               dvals, 0, st);
            g_launches.fetch_add(1, std::memory_order_relaxed);
        } else {
            ce = launch_globalop(arith, psi->d, n, rev->hp.ops[pd.op_begin].k, rev->dops + pd.op_begin, rev->dcoef, 1, 0, nullptr, st);
            if (ce == cudaSuccess) ce = launch_globalop(arith, lam->d, n, rev->hp.ops[pd.op_begin].k, rev->dops + pd.op_begin, rev->dcoef, 1, 0, nullptr, st);
            g_launches.fetch_add(2, std::memory_order_relaxed);
        }
        if (ce != cudaSuccess) return done(fail(QFVM_ERR_CUDA, std::string("adjoint pass: ") + cudaGetErrorString(ce)));
    }
    std::vector<double> vals(nprobe);
    if (nprobe) ADJ_CUDA(cudaMemcpyAsync(vals.data(), dvals, nprobe * 8, cudaMemcpyDeviceToHost, st), "probe download");
    ADJ_CUDA(cudaStreamSynchronize(st), "adjoint sync");
    if (const int src = check_status(st)) return done(src);
    for (int64_t k = 0; k < n_slots; ++k) grads[k] = 0.0;
    for (size_t p = 0; p < nprobe; ++p) grads[hp.probe_slot[p]] += vals[p];
    return done(QFVM_OK);
#undef ADJ_CUDA
}

int qfvm_expect_statevec(const double* state, uint64_t state_len, const uint64_t* x_masks, const uint64_t* z_masks,
                         const int32_t* y_counts, int64_t n_terms, double* out) {
    std::lock_guard<std::mutex> lk(g_boundary_mu);
    if (!state) return fail(QFVM_ERR_INVALID, "null state buffer");
    int n = 0;
    QSV_TRY(log2_len(state_len, &n));
    QSV_TRY(check_device());
    qfvm_sv* sv = nullptr;
    QSV_TRY(cached_state(n, QFVM_C128, &sv));
    QSV_TRY(sv_upload(sv, state, sv->N));
    return sv_expect(sv, x_masks, z_masks, y_counts, n_terms, out);
}

}  // extern "C"
