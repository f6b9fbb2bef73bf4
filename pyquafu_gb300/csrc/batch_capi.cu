// Batched runs behind the C ABI (qfvm_batch_* in include/qfvm_gb300.h).
//
// A batch session holds groups; a group is `items` circuits that share one
// gate structure (and one observable) and differ only in the values of their
// slotted rx/ry/rz/p/cp/rzz angles.  Each group keeps its items' states back
// to back (item i at offset i << n), so one fused pass over items << (n - T)
// tiles serves the whole group; per-item coefficient pools are rewritten on
// the device from the items' slot values.  A run uploads every group's values,
// computes per-item expectation values of the group's observables and, in
// gradient mode, the adjoint gradient of sum_o w[item, o] <O_o> for every
// slot; then it downloads the results.  Groups run on their own streams; each
// run mode is captured once into a CUDA graph and then replayed as one graph
// launch.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "jit.h"
#include "kernels.h"

using namespace qsv;
using namespace qsv_capi;

namespace {

struct BatchGroup {
    int n = 0, items = 0, nslots = 0, nterms = 0, nobs = 1, nprobe = 0;
    qfvm_plan* fwd = nullptr;
    qfvm_plan* rev = nullptr;
    uint64_t fstride = 0, rstride = 0;  // coefficient pool stride per item, in pool elements
    int nbf = 0, nbr = 0;               // bind records of the forward / reverse plan
    DevBuf fpool, rpool, binds, psi, lam, terms, scratch;
    uint64_t* dx = nullptr;
    uint64_t* dz = nullptr;
    double* dc = nullptr;
    int32_t* dy = nullptr;
    int32_t* doptr = nullptr;   // observable o = terms [doptr[o], doptr[o + 1])
    int32_t* dtobs = nullptr;   // observable of every term
    double* epart = nullptr;    // per-chunk expectation sums
    double* pvals = nullptr;    // items x nprobe probe values
    double* partial = nullptr;  // MAX_PASS_PROBES rows of per-tile probe sums
    int32_t* sptr = nullptr;    // slot -> probes (CSR)
    int32_t* sidx = nullptr;
    int64_t voff = 0, woff = 0, eoff = 0, goff = 0;  // offsets into the session's value, weight, result arrays
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
};

void free_group(BatchGroup* g) {
    if (!g) return;
    free_plan(g->fwd);
    free_plan(g->rev);
    g->fpool.release();
    g->rpool.release();
    g->binds.release();
    g->psi.release();
    g->lam.release();
    g->terms.release();
    g->scratch.release();
    if (g->done) cudaEventDestroy(g->done);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

size_t coef_elem_bytes(int arith) { return arith == QFVM_C64 ? 4 : 8; }

}  // namespace

struct qfvm_batch {
    int precision = QFVM_C64, flags = 0, T = 0, R = 0, aT = 0, aR = 0;
    std::vector<BatchGroup*> groups;
    int64_t nvals = 0, nweight = 0, nexp = 0, ngrad = 0;
    cudaStream_t main = nullptr;
    cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
    DevBuf dvals, dout;
    double* hvals = nullptr;  // pinned staging
    double* hout = nullptr;
    size_t hvals_cap = 0, hout_cap = 0;
    // per run mode (0 expectation values, 1 with gradients)
    cudaGraph_t graph[2] = {nullptr, nullptr};
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    int eager_runs[2] = {0, 0};
    uint64_t kernels_per_run[2] = {0, 0};
};

namespace {

void drop_graph(qfvm_batch* b) {
    for (int m = 0; m < 2; ++m) {
        if (b->exec[m]) cudaGraphExecDestroy(b->exec[m]);
        if (b->graph[m]) cudaGraphDestroy(b->graph[m]);
        b->exec[m] = nullptr;
        b->graph[m] = nullptr;
        b->eager_runs[m] = 0;
    }
}

// Per-item coefficient pool: the plan's uploaded pool is item 0's template,
// replicated to every item; a run then rewrites only the bound blocks.
int make_pool(const qfvm_plan* p, int arith, int items, DevBuf* pool, uint64_t* stride, cudaStream_t st) {
    const uint64_t len = p->hp.coef.size();
    const uint64_t s = (std::max<uint64_t>(len, 1) + 31) & ~31ULL;  // 128-byte aligned item pools
    const size_t eb = coef_elem_bytes(arith);
    QSV_TRY(pool->ensure(static_cast<size_t>(s) * items * eb));
    if (len) {
        QSV_CUDA(cudaMemcpyAsync(pool->p, p->dcoef, len * eb, cudaMemcpyDeviceToDevice, st), "pool init");
        QSV_CUDA(launch_replicate(arith, pool->p, s, len, items, st), "pool replicate");
    }
    *stride = s;
    return QFVM_OK;
}

}  // namespace

namespace {

int add_group(qfvm_batch* b, int n, const qfvm_op* ops, int64_t n_ops, const double* matpool, int64_t matpool_len,
              const uint64_t* x_masks, const uint64_t* z_masks, const int32_t* y_counts, const double* coeffs,
              const int32_t* obs_index, int64_t n_terms, int64_t n_obs, int64_t n_items, int64_t n_slots) {
    if (n < 1 || n > QFVM_MAX_QUBITS) return fail(QFVM_ERR_INVALID, "qubit count out of range");
    if (n_items < 1 || n_items > (1LL << 24)) return fail(QFVM_ERR_INVALID, "item count out of range");
    if (n_slots < 0 || n_slots > (1LL << 24)) return fail(QFVM_ERR_INVALID, "slot count out of range");
    if (n_ops < 0 || (n_ops > 0 && !ops)) return fail(QFVM_ERR_INVALID, "bad op list");
    if (n_terms < 1 || !x_masks || !z_masks || !y_counts || !coeffs)
        return fail(QFVM_ERR_INVALID, "the observable needs at least one Pauli term");
    if (n_obs < 1 || n_obs > 4096) return fail(QFVM_ERR_INVALID, "observable count out of range");
    const uint64_t lim = (1ULL << n) - 1;
    for (int64_t t = 0; t < n_terms; ++t) {
        if ((x_masks[t] | z_masks[t]) & ~lim) return fail(QFVM_ERR_INVALID, "Pauli term acts outside the state");
        if (obs_index && (obs_index[t] < 0 || obs_index[t] >= n_obs))
            return fail(QFVM_ERR_INVALID, "term observable index out of range");
    }
    if (!obs_index && n_obs != 1) return fail(QFVM_ERR_INVALID, "several observables need a term observable index");
    const bool grads = (b->flags & QFVM_BATCH_GRADS) != 0;
    const int arith = b->precision;
    const int storage = store_precision(arith);
    const uint64_t amps = static_cast<uint64_t>(n_items) << n;
    if (amps / static_cast<uint64_t>(n_items) != (1ULL << n) || n + 24 > 62)
        return fail(QFVM_ERR_INVALID, "batch too large");

    std::vector<GOp> gops;
    std::string err;
    if (!classify(n, ops, n_ops, matpool, matpool_len, &gops, &err)) return fail(QFVM_ERR_INVALID, err);
    for (const GOp& g : gops)
        if (g.slot >= n_slots) return fail(QFVM_ERR_INVALID, "parameter slot beyond n_slots");
    if (!unfix_bound(&gops, &err)) return fail(QFVM_ERR_UNSUPPORTED, err);
    std::vector<GOp> sweep;
    if (grads) {
        if (!build_adjoint_sweep(gops, &sweep, &err)) return fail(QFVM_ERR_INVALID, err);
        for (const GOp& g : sweep)
            if (g.kind == K_PROBE && __builtin_popcountll(g.xmask) > 2)
                return fail(QFVM_ERR_UNSUPPORTED, "generators flipping more than two qubits are not supported");
    }

    BatchGroup* g = new BatchGroup();
    auto bail = [&](int rc) {
        free_group(g);
        return rc;
    };
    g->n = n;
    g->items = static_cast<int>(n_items);
    g->nslots = static_cast<int>(n_slots);
    g->nterms = static_cast<int>(n_terms);
    g->nobs = static_cast<int>(n_obs);
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(QFVM_ERR_CUDA, "batch stream creation"));
    int rc = make_plan_gops(n, arith, gops, b->T, b->R, &g->fwd);
    if (rc != QFVM_OK) return bail(rc);
    if (grads) {
        int aT = b->aT, aR = b->aR;
        if (aT == 0) resolve_shape(arith, 1, n, &aT, &aR);
        rc = make_plan_gops(n, arith, sweep, aT, aR, &g->rev);
        if (rc != QFVM_OK) return bail(rc);
        g->nprobe = static_cast<int>(g->rev->hp.probe_slot.size());
    }
    {
        // specialised kernels now: graph captures must not compile
        std::string jerr;
        jit_prepare(g->fwd, 1, &jerr);
        if (grads) jit_prepare(g->rev, 2, &jerr);
    }
    cudaStream_t st = g->stream;
    rc = make_pool(g->fwd, arith, g->items, &g->fpool, &g->fstride, st);
    if (rc == QFVM_OK && grads) rc = make_pool(g->rev, arith, g->items, &g->rpool, &g->rstride, st);
    if (rc != QFVM_OK) return bail(rc);

    // bind records: forward, then reverse
    std::vector<Bind> bl(g->fwd->hp.binds);
    g->nbf = static_cast<int>(bl.size());
    if (grads) bl.insert(bl.end(), g->rev->hp.binds.begin(), g->rev->hp.binds.end());
    g->nbr = static_cast<int>(bl.size()) - g->nbf;
    if (!bl.empty()) {
        rc = g->binds.ensure(bl.size() * sizeof(Bind));
        if (rc != QFVM_OK) return bail(rc);
        if (cudaMemcpyAsync(g->binds.p, bl.data(), bl.size() * sizeof(Bind), cudaMemcpyHostToDevice, st) !=
            cudaSuccess)
            return bail(fail(QFVM_ERR_CUDA, "bind upload"));
    }

    // states
    const size_t sbytes = static_cast<size_t>(amps) * amp_bytes(storage);
    rc = g->psi.ensure(sbytes);
    if (rc == QFVM_OK) rc = g->lam.ensure(sbytes);
    if (rc != QFVM_OK) return bail(rc);

    // observables: terms grouped by observable, then sorted by flip mask
    // (stable), so the kernels reuse the load of psi[i ^ x]
    const size_t nt = static_cast<size_t>(n_terms);
    auto obs_of = [&](int64_t t) { return obs_index ? obs_index[t] : 0; };
    std::vector<int64_t> ord(nt);
    for (size_t t = 0; t < nt; ++t) ord[t] = static_cast<int64_t>(t);
    std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t c) {
        return obs_of(a) != obs_of(c) ? obs_of(a) < obs_of(c) : x_masks[a] < x_masks[c];
    });
    const size_t b8 = align256(nt * 8), b4 = align256(nt * 4), bo = align256((static_cast<size_t>(n_obs) + 1) * 4);
    std::vector<unsigned char> th(3 * b8 + 2 * b4 + bo, 0);
    std::vector<int32_t> optr(static_cast<size_t>(n_obs) + 1, 0);
    for (size_t i = 0; i < nt; ++i) {
        const int32_t o = obs_of(ord[i]);
        std::memcpy(th.data() + i * 8, &x_masks[ord[i]], 8);
        std::memcpy(th.data() + b8 + i * 8, &z_masks[ord[i]], 8);
        std::memcpy(th.data() + 2 * b8 + i * 8, &coeffs[ord[i]], 8);
        std::memcpy(th.data() + 3 * b8 + i * 4, &y_counts[ord[i]], 4);
        std::memcpy(th.data() + 3 * b8 + b4 + i * 4, &o, 4);
        optr[static_cast<size_t>(o) + 1]++;
    }
    for (size_t o = 0; o < static_cast<size_t>(n_obs); ++o) optr[o + 1] += optr[o];
    std::memcpy(th.data() + 3 * b8 + 2 * b4, optr.data(), optr.size() * 4);
    rc = g->terms.ensure(th.size());
    if (rc != QFVM_OK) return bail(rc);
    if (cudaMemcpyAsync(g->terms.p, th.data(), th.size(), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return bail(fail(QFVM_ERR_CUDA, "term upload"));
    char* tb = static_cast<char*>(g->terms.p);
    g->dx = reinterpret_cast<uint64_t*>(tb);
    g->dz = reinterpret_cast<uint64_t*>(tb + b8);
    g->dc = reinterpret_cast<double*>(tb + 2 * b8);
    g->dy = reinterpret_cast<int32_t*>(tb + 3 * b8);
    g->dtobs = reinterpret_cast<int32_t*>(tb + 3 * b8 + b4);
    g->doptr = reinterpret_cast<int32_t*>(tb + 3 * b8 + 2 * b4);

    // scratch: energy chunks, probe values, per-tile partials, slot CSR
    const uint64_t chunks = ((1ULL << n) / hamiltonian_chunk(n)) * static_cast<uint64_t>(n_items);
    size_t b_part = 0, b_pv = 0, b_csr = 0;
    std::vector<int32_t> csr;
    if (grads) {
        const int rT = g->rev->hp.T;
        const uint64_t tiles = n >= rT ? (static_cast<uint64_t>(n_items) << (n - rT)) : 0;
        b_part = align256(static_cast<size_t>(tiles) * MAX_PASS_PROBES * 8);
        b_pv = align256(static_cast<size_t>(n_items) * std::max(g->nprobe, 1) * 8);
        // CSR of slot -> probe ids, ascending probe id within a slot
        std::vector<int32_t> cnt(static_cast<size_t>(n_slots) + 1, 0);
        for (int ps : g->rev->hp.probe_slot) cnt[static_cast<size_t>(ps) + 1]++;
        for (size_t s = 0; s < static_cast<size_t>(n_slots); ++s) cnt[s + 1] += cnt[s];
        std::vector<int32_t> idx(g->rev->hp.probe_slot.size());
        std::vector<int32_t> pos(cnt.begin(), cnt.end() - 1);
        for (size_t p = 0; p < idx.size(); ++p) idx[pos[g->rev->hp.probe_slot[p]]++] = static_cast<int32_t>(p);
        csr = cnt;
        csr.insert(csr.end(), idx.begin(), idx.end());
        b_csr = align256(csr.size() * 4);
    }
    const size_t b_ep = align256(static_cast<size_t>(chunks) * n_obs * 8);
    rc = g->scratch.ensure(b_ep + b_pv + b_part + b_csr);
    if (rc != QFVM_OK) return bail(rc);
    char* sb = static_cast<char*>(g->scratch.p);
    g->epart = reinterpret_cast<double*>(sb);
    if (grads) {
        g->pvals = reinterpret_cast<double*>(sb + b_ep);
        g->partial = reinterpret_cast<double*>(sb + b_ep + b_pv);
        g->sptr = reinterpret_cast<int32_t*>(sb + b_ep + b_pv + b_part);
        g->sidx = g->sptr + (n_slots + 1);
        if (cudaMemcpyAsync(g->sptr, csr.data(), csr.size() * 4, cudaMemcpyHostToDevice, st) != cudaSuccess)
            return bail(fail(QFVM_ERR_CUDA, "slot map upload"));
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return bail(fail(QFVM_ERR_CUDA, "batch group setup"));

    g->voff = b->nvals;
    g->woff = b->nweight;
    g->eoff = b->nexp;
    g->goff = b->ngrad;
    b->nvals += n_items * n_slots;
    b->nweight += n_items * n_obs;
    b->nexp += n_items * n_obs;
    if (grads) b->ngrad += n_items * n_slots;
    b->groups.push_back(g);
    drop_graph(b);
    return QFVM_OK;
}

}  // namespace

namespace {

#define QSV_LAUNCH(call, what)                                                                          \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return fail(QFVM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
        ++*nk;                                                                                         \
    } while (0)
// a launch that may decline (launched == false: nothing issued, not counted)
#define QSV_LAUNCH_IF(call, launched, what)                                                             \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return fail(QFVM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
        if (launched) ++*nk;                                                                           \
    } while (0)

// One group's run on its own stream: bind, forward, expectation values; in
// gradient mode also lam = sum_o w_o O_o psi, the reverse sweep and the slot
// sums.
int enqueue_group(qfvm_batch* b, BatchGroup* g, int mode, uint64_t* nk) {
    const int arith = b->precision, storage = store_precision(arith);
    const int n = g->n, items = g->items;
    cudaStream_t st = g->stream;
    const double* vals = b->dvals.as<double>() + g->voff;
    const double* weights = b->dvals.as<double>() + b->nvals + g->woff;
    double* expv = b->dout.as<double>() + g->eoff;
    double* grads = b->dout.as<double>() + b->nexp + g->goff;
    const Bind* bf = static_cast<const Bind*>(g->binds.p);

    if (g->nbf) QSV_LAUNCH(launch_bind(arith, g->fpool.p, g->fstride, bf, g->nbf, vals, g->nslots, items, st), "bind");
    QSV_LAUNCH(launch_zero_items(storage, g->psi.p, n, items, st), "initial states");
    const HostPlan& fp = g->fwd->hp;
    for (size_t i = 0; i < fp.passes.size(); ++i) {
        const PassDesc& pd = fp.passes[i];
        if (pd.type == PASS_TILE) {
            bool done = false;
            QSV_LAUNCH_IF(jit_launch_pass(g->fwd, static_cast<int>(i), g->psi.p, nullptr, g->fpool.p, items,
                                          g->fstride, nullptr, 0, nullptr, nullptr, st, &done),
                          done, "batched pass");
            if (!done)
                QSV_LAUNCH(launch_tile_pass(arith, fp.T, fp.R, g->psi.p, g->fwd->dpass + i, g->fwd->dsteps,
                                            g->fwd->dops, g->fpool.p, n, pd.H, items, g->fstride, nullptr, st),
                           "batched pass");
        } else if (pd.type == PASS_SMALL)
            QSV_LAUNCH(launch_small(arith, g->psi.p, 1ULL << n, items, n, g->fwd->dops + pd.op_begin, pd.op_count,
                                    g->fpool.p, g->fstride, nullptr, st),
                       "batched small pass");
        else
            QSV_LAUNCH(launch_globalop(arith, g->psi.p, n, g->fwd->hp.ops[pd.op_begin].k, g->fwd->dops + pd.op_begin, g->fpool.p, items, g->fstride,
                                       nullptr, st),
                       "batched global op");
    }
    QSV_LAUNCH(launch_expect_seg(storage, g->psi.p, n, items, g->dx, g->dz, g->dy, g->dc, g->doptr, g->nobs, g->epart,
                                 expv, st),
               "batched expectation");
    ++*nk;  // the segmented sum
    if (mode == 0) return QFVM_OK;

    QSV_LAUNCH(launch_lambda_seg(storage, g->psi.p, g->lam.p, n, items, g->dx, g->dz, g->dy, g->dc, g->dtobs,
                                 g->nterms, g->nobs, weights, st),
               "batched lambda");
    if (g->nbr)
        QSV_LAUNCH(launch_bind(arith, g->rpool.p, g->rstride, bf + g->nbf, g->nbr, vals, g->nslots, items, st),
                   "bind");
    const HostPlan& rp = g->rev->hp;
    for (size_t i = 0; i < rp.passes.size(); ++i) {
        const PassDesc& pd = rp.passes[i];
        if (pd.type == PASS_TILE) {
            int grid = 0;
            bool done = false;
            QSV_LAUNCH_IF(jit_launch_pass(g->rev, static_cast<int>(i), g->psi.p, g->lam.p, g->rpool.p, items,
                                          g->rstride, nullptr, 1, g->partial, &grid, st, &done),
                          done, "batched adjoint pass");
            if (!done)
                QSV_LAUNCH(launch_pass2(arith, rp.T, rp.R, g->psi.p, g->lam.p, g->rev->dpass + i, g->rev->dsteps,
                                        g->rev->dops, g->rpool.p, n, pd.H, items, g->rstride, 1, g->partial, &grid, st),
                           "batched adjoint pass");
            if (pd.nprobe > 0) {
                const uint64_t tpi = 1ULL << (n - rp.T);
                QSV_LAUNCH(launch_probe_reduce_seg(g->partial, tpi * items, static_cast<int>(tpi), items, pd.nprobe,
                                                   g->pvals, g->nprobe, pd.probe_base, st),
                           "probe sums");
            }
        } else if (pd.type == PASS_SMALL) {
            QSV_LAUNCH(launch_small2(arith, g->psi.p, g->lam.p, n, g->rev->dops + pd.op_begin, pd.op_count, g->rpool.p,
                                     items, g->rstride, g->pvals, static_cast<uint64_t>(g->nprobe), st),
                       "batched adjoint small pass");
        } else {
            QSV_LAUNCH(launch_globalop(arith, g->psi.p, n, g->rev->hp.ops[pd.op_begin].k, g->rev->dops + pd.op_begin, g->rpool.p, items, g->rstride,
                                       nullptr, st),
                       "batched global op");
            QSV_LAUNCH(launch_globalop(arith, g->lam.p, n, g->rev->hp.ops[pd.op_begin].k, g->rev->dops + pd.op_begin, g->rpool.p, items, g->rstride,
                                       nullptr, st),
                       "batched global op");
        }
    }
    if (g->nslots)
        QSV_LAUNCH(launch_slot_gather(g->pvals, g->nprobe, items, g->sptr, g->sidx, g->nslots, grads, st),
                   "slot sums");
    return QFVM_OK;
}

// The whole run on b->main: values (and weights) up, fork to the group
// streams, join, results down.
int enqueue_run(qfvm_batch* b, int mode, uint64_t* nk) {
    cudaStream_t m = b->main;
    const int64_t up = b->nvals + (mode ? b->nweight : 0);
    const int64_t down = b->nexp + (mode ? b->ngrad : 0);
    if (up) QSV_CUDA(cudaMemcpyAsync(b->dvals.p, b->hvals, up * 8, cudaMemcpyHostToDevice, m), "value upload");
    QSV_CUDA(cudaEventRecord(b->fork, m), "fork");
    for (BatchGroup* g : b->groups) {
        QSV_CUDA(cudaStreamWaitEvent(g->stream, b->fork, 0), "fork");
        QSV_TRY(enqueue_group(b, g, mode, nk));
        QSV_CUDA(cudaEventRecord(g->done, g->stream), "join");
        QSV_CUDA(cudaStreamWaitEvent(m, g->done, 0), "join");
    }
    QSV_CUDA(cudaMemcpyAsync(b->hout, b->dout.p, down * 8, cudaMemcpyDeviceToHost, m), "result download");
    return QFVM_OK;
}

int ensure_host(double** p, size_t* cap, size_t count) {
    const size_t bytes = std::max<size_t>(count, 1) * 8;
    if (bytes <= *cap) return QFVM_OK;
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    *cap = 0;
    QSV_CUDA(cudaMallocHost(reinterpret_cast<void**>(p), bytes), "pinned staging");
    *cap = bytes;
    return QFVM_OK;
}

int batch_run(qfvm_batch* b, int mode, const double* values, const double* weights, double* expvals, double* grads,
              float* device_ms) {
    if (b->groups.empty()) return fail(QFVM_ERR_INVALID, "batch has no groups");
    if (mode != 0 && mode != 1) return fail(QFVM_ERR_INVALID, "unknown run mode");
    if (mode == 1 && !(b->flags & QFVM_BATCH_GRADS))
        return fail(QFVM_ERR_INVALID, "gradient runs need a batch created with QFVM_BATCH_GRADS");
    if (b->nvals && !values) return fail(QFVM_ERR_INVALID, "missing slot values");
    if (!expvals) return fail(QFVM_ERR_INVALID, "missing expectation-value buffer");
    if (mode == 1 && b->ngrad && !grads) return fail(QFVM_ERR_INVALID, "missing gradient buffer");
    const size_t nin = static_cast<size_t>(b->nvals + b->nweight), nout = static_cast<size_t>(b->nexp + b->ngrad);
    QSV_TRY(ensure_host(&b->hvals, &b->hvals_cap, nin));
    QSV_TRY(ensure_host(&b->hout, &b->hout_cap, nout));
    QSV_TRY(b->dvals.ensure(std::max<size_t>(nin, 1) * 8));
    QSV_TRY(b->dout.ensure(std::max<size_t>(nout, 1) * 8));
    if (b->nvals) std::memcpy(b->hvals, values, static_cast<size_t>(b->nvals) * 8);
    if (mode == 1) {
        double* w = b->hvals + b->nvals;
        if (weights) std::memcpy(w, weights, static_cast<size_t>(b->nweight) * 8);
        else
            for (int64_t i = 0; i < b->nweight; ++i) w[i] = 1.0;
    }

    const bool use_graph = !(b->flags & QFVM_BATCH_NO_GRAPH);
    // the first run of a mode is eager (it also settles every launcher's
    // one-time setup); the second captures the mode's graph, later runs replay it
    if (use_graph && !b->exec[mode] && b->eager_runs[mode] > 0) {
        uint64_t nk = 0;
        QSV_CUDA(cudaStreamBeginCapture(b->main, cudaStreamCaptureModeRelaxed), "graph capture");
        const int rc = enqueue_run(b, mode, &nk);
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(b->main, &graph);
        if (rc != QFVM_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (ce != cudaSuccess) return fail(QFVM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        b->graph[mode] = graph;
        QSV_CUDA(cudaGraphInstantiate(&b->exec[mode], graph, 0), "graph instantiate");
        b->kernels_per_run[mode] = nk;
    }
    if (device_ms) QSV_CUDA(cudaEventRecord(b->t0, b->main), "event");
    if (b->exec[mode]) {
        QSV_CUDA(cudaGraphLaunch(b->exec[mode], b->main), "graph launch");
        g_launches.fetch_add(b->kernels_per_run[mode], std::memory_order_relaxed);
    } else {
        uint64_t nk = 0;
        QSV_TRY(enqueue_run(b, mode, &nk));
        g_launches.fetch_add(nk, std::memory_order_relaxed);
        b->kernels_per_run[mode] = nk;
        ++b->eager_runs[mode];
    }
    if (device_ms) QSV_CUDA(cudaEventRecord(b->t1, b->main), "event");
    QSV_CUDA(cudaStreamSynchronize(b->main), "batch run");
    QSV_TRY(check_status(b->main));
    if (device_ms) QSV_CUDA(cudaEventElapsedTime(device_ms, b->t0, b->t1), "event");
    std::memcpy(expvals, b->hout, static_cast<size_t>(b->nexp) * 8);
    if (mode == 1 && b->ngrad) std::memcpy(grads, b->hout + b->nexp, static_cast<size_t>(b->ngrad) * 8);
    return QFVM_OK;
}

void free_batch(qfvm_batch* b) {
    if (!b) return;
    if (b->main) cudaStreamSynchronize(b->main);
    drop_graph(b);
    for (BatchGroup* g : b->groups) free_group(g);
    b->dvals.release();
    b->dout.release();
    if (b->hvals) cudaFreeHost(b->hvals);
    if (b->hout) cudaFreeHost(b->hout);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->t1) cudaEventDestroy(b->t1);
    if (b->main) cudaStreamDestroy(b->main);
    delete b;
}

}  // namespace

extern "C" {

int qfvm_batch_create(int32_t precision, int32_t flags, const int32_t* shapes, qfvm_batch** out) {
    if (!out) return fail(QFVM_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (precision != QFVM_C128 && precision != QFVM_C64 && precision != QFVM_C128_DS)
        return fail(QFVM_ERR_INVALID, "unknown precision");
    if (flags & ~(QFVM_BATCH_GRADS | QFVM_BATCH_NO_GRAPH)) return fail(QFVM_ERR_INVALID, "unknown batch flags");
    int sh[4] = {0, 0, 0, 0};
    if (shapes)
        for (int k = 0; k < 4; ++k) sh[k] = shapes[k];
    if (sh[0] > 0 || sh[1] > 0) {
        int dT = 0, dR = 0;
        default_shape(20, store_precision(precision), &dT, &dR);
        if (sh[0] <= 0) sh[0] = dT;
        if (sh[1] <= 0) sh[1] = dR;
        if (!pass_shape_supported(precision, sh[0], sh[1]))
            return fail(QFVM_ERR_INVALID, "forward tile shape not compiled in");
    }
    if (sh[2] > 0 || sh[3] > 0) {
        int dT = 0, dR = 0;
        adjoint_shape(precision, &dT, &dR);
        if (sh[2] <= 0) sh[2] = dT;
        if (sh[3] <= 0) sh[3] = dR;
        if (!pass2_shape_supported(precision, sh[2], sh[3]))
            return fail(QFVM_ERR_INVALID, "reverse-sweep tile shape not compiled in");
    }
    QSV_TRY(check_device());
    qfvm_batch* b = new qfvm_batch();
    b->precision = precision;
    b->flags = flags;
    b->T = sh[0];
    b->R = sh[1];
    b->aT = sh[2];
    b->aR = sh[3];
    if (cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->t0) != cudaSuccess || cudaEventCreate(&b->t1) != cudaSuccess) {
        free_batch(b);
        return fail(QFVM_ERR_CUDA, "batch stream creation");
    }
    *out = b;
    return QFVM_OK;
}

int qfvm_batch_add_group(qfvm_batch* batch, int32_t num_qubits, const qfvm_op* ops, int64_t n_ops,
                         const double* matpool, int64_t matpool_len, const uint64_t* x_masks, const uint64_t* z_masks,
                         const int32_t* y_counts, const double* coeffs, const int32_t* obs_index, int64_t n_terms,
                         int64_t n_obs, int64_t n_items, int64_t n_slots) {
    if (!batch) return fail(QFVM_ERR_INVALID, "null batch");
    return add_group(batch, num_qubits, ops, n_ops, matpool, matpool_len, x_masks, z_masks, y_counts, coeffs,
                     obs_index, n_terms, n_obs, n_items, n_slots);
}

int qfvm_batch_run(qfvm_batch* batch, int32_t mode, const double* values, const double* weights, double* expvals,
                   double* grads) {
    qsv_capi::NvtxRange range("qfvm batched run");
    if (!batch) return fail(QFVM_ERR_INVALID, "null batch");
    return batch_run(batch, mode, values, weights, expvals, grads, nullptr);
}

int qfvm_batch_run_timed(qfvm_batch* batch, int32_t mode, const double* values, const double* weights,
                         double* expvals, double* grads, float* device_ms) {
    qsv_capi::NvtxRange range("qfvm batched run");
    if (!batch || !device_ms) return fail(QFVM_ERR_INVALID, "null argument");
    return batch_run(batch, mode, values, weights, expvals, grads, device_ms);
}

int qfvm_batch_info(const qfvm_batch* batch, int64_t* n_groups, int64_t* n_values, int64_t* n_expvals,
                    int64_t* n_grads, int64_t kernels_per_run[2], int32_t graph_ready[2]) {
    if (!batch) return fail(QFVM_ERR_INVALID, "null batch");
    if (n_groups) *n_groups = static_cast<int64_t>(batch->groups.size());
    if (n_values) *n_values = batch->nvals;
    if (n_expvals) *n_expvals = batch->nexp;
    if (n_grads) *n_grads = batch->ngrad;
    for (int m = 0; m < 2; ++m) {
        if (kernels_per_run) kernels_per_run[m] = static_cast<int64_t>(batch->kernels_per_run[m]);
        if (graph_ready) graph_ready[m] = batch->exec[m] ? 1 : 0;
    }
    return QFVM_OK;
}

int qfvm_set_tuned_shape(int32_t precision, int32_t kind, int32_t num_qubits, int32_t tile_qubits,
                         int32_t reg_qubits) {
    if (precision != QFVM_C128 && precision != QFVM_C64 && precision != QFVM_C128_DS)
        return fail(QFVM_ERR_INVALID, "unknown precision");
    if (!set_tuned_shape(precision, kind, num_qubits, tile_qubits, reg_qubits))
        return fail(QFVM_ERR_INVALID, "shape not compiled in, or bad kind / qubit count");
    return QFVM_OK;
}

int qfvm_get_shape(int32_t precision, int32_t kind, int32_t num_qubits, int32_t* tile_qubits, int32_t* reg_qubits) {
    if (!tile_qubits || !reg_qubits) return fail(QFVM_ERR_INVALID, "null argument");
    int T = 0, R = 0;
    resolve_shape(precision, kind, num_qubits, &T, &R);
    *tile_qubits = T;
    *reg_qubits = R;
    return QFVM_OK;
}

int32_t qfvm_shape_supported(int32_t precision, int32_t kind, int32_t tile_qubits, int32_t reg_qubits) {
    if (precision != QFVM_C128 && precision != QFVM_C64 && precision != QFVM_C128_DS) return 0;
    if (kind == 0) return pass_shape_supported(precision, tile_qubits, reg_qubits) ? 1 : 0;
    if (kind == 1) return pass2_shape_supported(precision, tile_qubits, reg_qubits) ? 1 : 0;
    return 0;
}

int qfvm_batch_destroy(qfvm_batch* batch) {
    free_batch(batch);
    return QFVM_OK;
}

}  // extern "C"
