// Compilation, cache and launch of the circuit-specialised tile passes.
//
// The PTX of a pass (jit_ptx.cpp) depends on the circuit's structure only
// (kinds, targets, masks, coefficient offsets), not on its angles, so one
// compiled module serves every re-run and every rebinding of a plan.  Modules
// are cached process-wide by their PTX text and kept until exit (CUDA graphs
// may hold their kernels).  The driver API is reached through the runtime's
// entry-point query, so the library does not link libcuda itself.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "capi_internal.h"
#include "jit.h"

#ifdef QSV_PTXCOMPILER
#include <nvPTXCompiler.h>
#endif

namespace qsv {
namespace {

struct Driver {
    bool ok = false;
    std::string err;
    CUresult (*load)(CUmodule*, const void*, unsigned int, CUjit_option*, void**) = nullptr;
    CUresult (*get_function)(CUfunction*, CUmodule, const char*) = nullptr;
    CUresult (*set_attribute)(CUfunction, CUfunction_attribute, int) = nullptr;
    CUresult (*launch)(CUfunction, unsigned int, unsigned int, unsigned int, unsigned int, unsigned int, unsigned int,
                       unsigned int, CUstream, void**, void**) = nullptr;
    CUresult (*occupancy)(int*, CUfunction, int, size_t) = nullptr;
    CUresult (*error_string)(CUresult, const char**) = nullptr;
};

template <class F>
bool entry(const char* name, F* fn, std::string* err) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || p == nullptr) {
        *err = std::string("driver entry point not found: ") + name;
        return false;
    }
    *fn = reinterpret_cast<F>(p);
    return true;
}

// bounded waits of the specialised passes: 2 s of %globaltimer by default
constexpr uint64_t kDefaultWaitNs = 2000000000ull;
std::atomic<uint64_t> g_wait_ns{kDefaultWaitNs};
std::atomic<uint32_t> g_extra_tx{0};

// per-device status word (allocated on first use, zeroed)
std::mutex g_status_mu;
uint32_t* g_status[64] = {nullptr};

uint32_t* status_word_if_any() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_status_mu);
    return g_status[dev];
}

uint32_t* status_word() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_status_mu);
    if (g_status[dev] == nullptr) {
        void* p = nullptr;
        if (cudaMalloc(&p, 16) != cudaSuccess) return nullptr;
        if (cudaMemset(p, 0, 16) != cudaSuccess) {
            cudaFree(p);
            return nullptr;
        }
        g_status[dev] = static_cast<uint32_t*>(p);
    }
    return g_status[dev];
}

Driver& driver() {
    static Driver d = [] {
        Driver x;
        x.ok = entry("cuModuleLoadDataEx", &x.load, &x.err) && entry("cuModuleGetFunction", &x.get_function, &x.err) &&
               entry("cuFuncSetAttribute", &x.set_attribute, &x.err) && entry("cuLaunchKernel", &x.launch, &x.err) &&
               entry("cuOccupancyMaxActiveBlocksPerMultiprocessor", &x.occupancy, &x.err) &&
               entry("cuGetErrorString", &x.error_string, &x.err);
        return x;
    }();
    return d;
}

std::string cu_error(CUresult r) {
    const char* s = nullptr;
    if (driver().error_string) driver().error_string(r, &s);
    return s ? s : "unknown driver error";
}

struct Kernel {
    std::string entry;
    CUmodule mod = nullptr;
    CUfunction fn = nullptr;
    int threads = 0;
    size_t smem = 0;
    int grid_cap = 0;
    int T = 0;
};

std::mutex g_mu;
std::unordered_map<std::string, std::unique_ptr<Kernel>>& cache() {
    static std::unordered_map<std::string, std::unique_ptr<Kernel>> c;
    return c;
}

JitConfig initial_config() {
    JitConfig c;
    const char* e = std::getenv("QFVM_JIT");
    if (e && e[0] == '0') c.enabled = 0;
    return c;
}
JitConfig& config() {
    static JitConfig c = initial_config();
    return c;
}

// PTX -> cubin.  With the toolkit's PTX compiler library linked in this runs
// on any host thread without a CUDA context, so a plan's passes compile in
// parallel; otherwise the driver compiles the PTX when the module is loaded.
bool to_cubin(const std::string& ptx, std::string* image, std::string* err, std::string* info = nullptr) {
#ifdef QSV_PTXCOMPILER
    nvPTXCompilerHandle h = nullptr;
    if (nvPTXCompilerCreate(&h, ptx.size(), ptx.c_str()) != NVPTXCOMPILE_SUCCESS) {
        *err = "PTX compiler: create failed";
        return false;
    }
    const char* opts[] = {"--gpu-name=sm_103a", "-O3", "-v"};
    bool ok = nvPTXCompilerCompile(h, info ? 3 : 2, opts) == NVPTXCOMPILE_SUCCESS;
    if (info) {
        size_t n = 0;
        nvPTXCompilerGetInfoLogSize(h, &n);
        std::string log(n + 1, '\0');
        if (n) nvPTXCompilerGetInfoLog(h, &log[0]);
        *info = log.c_str();
    }
    if (!ok) {
        size_t n = 0;
        nvPTXCompilerGetErrorLogSize(h, &n);
        std::string log(n + 1, '\0');
        if (n) nvPTXCompilerGetErrorLog(h, &log[0]);
        *err = "PTX compiler: " + log;
    } else {
        size_t n = 0;
        ok = nvPTXCompilerGetCompiledProgramSize(h, &n) == NVPTXCOMPILE_SUCCESS;
        image->assign(n, '\0');
        ok = ok && nvPTXCompilerGetCompiledProgram(h, &(*image)[0]) == NVPTXCOMPILE_SUCCESS;
        if (!ok) *err = "PTX compiler: no program";
    }
    nvPTXCompilerDestroy(&h);
    return ok;
#else
    *image = ptx;  // loaded as PTX: the driver compiles it
    (void)err;
    if (info) *info = "driver compilation";
    return true;
#endif
}

// load a compiled image and set the kernel up (thread with the context current)
int load(int dev, const std::string& image, Kernel* k, std::string* err) {
    Driver& d = driver();
    char log[4096] = "";
    CUjit_option opt[2] = {CU_JIT_ERROR_LOG_BUFFER, CU_JIT_ERROR_LOG_BUFFER_SIZE_BYTES};
    void* val[2] = {log, reinterpret_cast<void*>(static_cast<uintptr_t>(sizeof log))};
    CUresult r = d.load(&k->mod, image.c_str(), 2, opt, val);
    if (r != CUDA_SUCCESS) {
        *err = "specialised pass load failed: " + cu_error(r) + ": " + log;
        return 1;
    }
    r = d.get_function(&k->fn, k->mod, k->entry.c_str());
    if (r == CUDA_SUCCESS && k->smem > 48 * 1024)
        r = d.set_attribute(k->fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, static_cast<int>(k->smem));
    int per_sm = 0;
    if (r == CUDA_SUCCESS) r = d.occupancy(&per_sm, k->fn, k->threads, k->smem);
    if (r != CUDA_SUCCESS) {
        *err = "specialised pass setup failed: " + cu_error(r);
        return 1;
    }
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    k->grid_cap = (nsm > 0 ? nsm : 1) * (per_sm > 0 ? per_sm : 1);
    return 0;
}

JitShape shape_for(const HostPlan& hp, int nstates) {
    JitConfig c;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        c = config();
    }
    JitShape sh;
    sh.nstates = nstates;
    sh.nb = nstates == 1 ? c.nb1 : c.nb2;
    int minb = nstates == 1 ? c.minb1 : c.minb2;
    if (minb <= 0) {
        // 128 registers per thread, or the full 255 when the round's
        // amplitudes alone need more than 64 (two states of FP64 or float-pair
        // amplitudes at R = 4: 128 registers; at 128 the sweep spilled and
        // wrote 5x its algorithmic bytes to DRAM)
        // Complex64 one-state passes: 80 (three CTAs of 256 threads per SM;
        // tile (13,5) at 26 qubits measured 10.1 ms against 10.6 ms at 128).
        const int nt = 1 << (hp.T - hp.R);
        const int per_amp = hp.arith == QFVM_C64 ? 2 : 4;
        int budget = nstates * (1 << hp.R) * per_amp > 64 ? 255 : 128;
        if (hp.arith == QFVM_C64 && nstates == 1) budget = 80;
        minb = 65536 / (nt * budget);
        if (minb < 1) minb = 1;
    }
    sh.minb = minb;
    return sh;
}

}  // namespace

std::string jit_entry_name(int arith, int nstates) {
    const char* a = arith == QFVM_C64 ? "c64" : (arith == QFVM_C128_DS ? "ds" : "c128");
    return std::string(nstates == 2 ? "qsv_tile_sweep_" : "qsv_tile_pass_") + a;
}

JitConfig jit_config() {
    std::lock_guard<std::mutex> lk(g_mu);
    return config();
}
void jit_set_config(const JitConfig& c) {
    std::lock_guard<std::mutex> lk(g_mu);
    config() = c;
}

// The shape a plan's passes are compiled with: the configured or automatic
// register budget (shape_for), coefficients in the kernel parameters when no
// bind rewrites the pool on the device, the bounds mode, the float-pair
// chain, and double buffering only where the register budget's resident
// CTAs (minb) still fit in the SM's shared memory with two tiles each
// (otherwise the second buffer costs a resident CTA: measured 1.5x slower
// for double-single (12,4)).  optin / per_sm: the device's shared memory per
// block (opt-in) and per SM.
JitShape plan_shape(const qfvm_plan* p, int nstates, size_t optin, size_t per_sm) {
    const HostPlan& hp = p->hp;
    JitShape sh = shape_for(hp, nstates);
    sh.pcoef = hp.binds.empty() ? 1 : 0;
    sh.bounds = bounds_check_env();
    sh.chain = p->chain_ok ? chain_for(hp, sh) : 0;
    JitShape two_sh = sh;
    two_sh.nb = 2;
    const size_t two = jit_smem_bytes(hp, two_sh, MAX_PASS_PROBES);
    if (sh.nb == 2 && (two > optin || static_cast<size_t>(sh.minb) * (two + 1024) > per_sm)) sh.nb = 1;
    return sh;
}

// plan_shape with the current device's shared memory, or sm_103a's (227 KiB
// per block, 228 KiB per SM) on a machine without a device: the shape the
// host-side PTX queries report is the one the device path compiles
JitShape host_query_shape(const qfvm_plan* p, int nstates) {
    int dev = 0, optin = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess) {
        cudaGetLastError();
        optin = 227 * 1024;
        per_sm = 228 * 1024;
    }
    return plan_shape(p, nstates, static_cast<size_t>(optin), static_cast<size_t>(per_sm));
}

namespace {
int prepare_impl(qfvm_plan* p, int nstates, std::string* err);
}

// A pass that cannot be compiled runs on the interpreting kernel: the
// failure is reported once on stderr and the plan continues without
// specialised passes for that state count.
int jit_prepare(qfvm_plan* p, int nstates, std::string* err) {
    const int si = nstates == 2 ? 1 : 0;
    if (p->jit_ready[si]) return 0;
    if (prepare_impl(p, nstates, err) == 0) return 0;
    static std::atomic<bool> warned{false};
    if (!warned.exchange(true)) {
        std::fprintf(stderr, "qfvm: specialised passes unavailable, interpreting kernels used: %s\n", err->c_str());
    }
    p->jit[si].assign(p->hp.passes.size(), nullptr);
    p->jit_ready[si] = true;
    return 0;
}

namespace {
int prepare_impl(qfvm_plan* p, int nstates, std::string* err) {
    const int si = nstates == 2 ? 1 : 0;
    const HostPlan& hp = p->hp;
    std::vector<const void*> ks(hp.passes.size(), nullptr);
    JitShape sh;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!config().enabled || (hp.arith != QFVM_C64 && hp.arith != QFVM_C128 && hp.arith != QFVM_C128_DS)) {
            p->jit[si] = ks;
            p->jit_ready[si] = true;
            return 0;
        }
    }
    bool any_tile = false;
    for (const PassDesc& pd : hp.passes) any_tile |= pd.type == PASS_TILE;
    if (!any_tile) {
        p->jit[si] = ks;
        p->jit_ready[si] = true;
        return 0;
    }
    if (!driver().ok) {
        *err = driver().err;
        return 1;
    }
    if (status_word() == nullptr) {
        *err = "device status word: allocation failed";
        return 1;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    {
        int optin = 0, per_sm = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        sh = plan_shape(p, nstates, static_cast<size_t>(optin), static_cast<size_t>(per_sm));
    }
    // look the passes up by structure; generate and compile the missing ones
    std::vector<std::string> keys(hp.passes.size());
    std::vector<int> todo;  // first pass of each missing structure
    {
        std::lock_guard<std::mutex> lk(g_mu);
        for (size_t i = 0; i < hp.passes.size(); ++i) {
            std::string why;
            if (!jit_pass_key(hp, static_cast<int>(i), sh, &keys[i], &why)) {
                keys[i].clear();
                continue;
            }
            keys[i] += "@" + std::to_string(dev);
            auto it = cache().find(keys[i]);
            if (it != cache().end()) {
                ks[i] = it->second.get();
                continue;
            }
            bool dup = false;
            for (int j : todo) dup |= keys[j] == keys[i];
            if (!dup) todo.push_back(static_cast<int>(i));
        }
    }
    std::vector<std::string> images(todo.size()), errs(todo.size());
    std::vector<char> oks(todo.size(), 0);
    const unsigned hw = std::thread::hardware_concurrency();
    const size_t nthreads = std::min<size_t>(todo.size(), hw ? hw : 4);
    std::vector<std::thread> pool;
    std::mutex qmu;
    size_t next = 0;
    for (size_t t = 0; t < nthreads; ++t) {
        pool.emplace_back([&] {
            for (;;) {
                size_t w;
                {
                    std::lock_guard<std::mutex> lk(qmu);
                    if (next >= todo.size()) return;
                    w = next++;
                }
                std::string ptx, why;
                if (!jit_pass_ptx(hp, todo[w], sh, jit_entry_name(hp.arith, nstates), &ptx, &why)) {
                    errs[w] = "specialised pass: " + why;
                    continue;
                }
                oks[w] = to_cubin(ptx, &images[w], &errs[w]);
            }
        });
    }
    for (auto& t : pool) t.join();
    for (size_t w = 0; w < todo.size(); ++w)
        if (!oks[w]) {
            *err = errs[w];
            return 1;
        }
    std::lock_guard<std::mutex> lk(g_mu);
    for (size_t w = 0; w < todo.size(); ++w) {
        const int i = todo[w];
        if (cache().count(keys[i])) continue;
        auto k = std::make_unique<Kernel>();
        const int nt = 1 << (hp.T - hp.R);
        const int np = nstates == 2 ? hp.passes[i].nprobe : 0;
        k->threads = nt;
        k->T = hp.T;
        k->entry = jit_entry_name(hp.arith, nstates);
        k->smem = jit_smem_bytes(hp, sh, np);
        if (load(dev, images[w], k.get(), err)) return 1;
        cache().emplace(keys[i], std::move(k));
    }
    for (size_t i = 0; i < hp.passes.size(); ++i) {
        if (ks[i] || keys[i].empty()) continue;
        auto it = cache().find(keys[i]);
        if (it != cache().end()) ks[i] = it->second.get();
    }
    // the coefficient parameter blocks of the compiled passes
    p->jit_cblob[si].assign(hp.passes.size(), {});
    for (size_t i = 0; i < hp.passes.size(); ++i) {
        uint32_t lo = 0, hi = 0;
        if (!ks[i] || !jit_pass_coef_block(hp, static_cast<int>(i), sh, &lo, &hi)) continue;
        std::vector<unsigned char>& blob = p->jit_cblob[si][i];
        const size_t eb = hp.arith == QFVM_C64 ? 4 : 8;
        blob.assign(((hi - lo) * eb + 15) / 16 * 16, 0);
        for (uint32_t c = lo; c < hi; ++c) {
            const double v = hp.coef[c];
            unsigned char* d = blob.data() + (c - lo) * eb;
            if (hp.arith == QFVM_C64) {
                const float f = static_cast<float>(v);
                std::memcpy(d, &f, 4);
            } else if (hp.arith == QFVM_C128_DS) {
                const float h = static_cast<float>(v);
                const float l = static_cast<float>(v - static_cast<double>(h));
                std::memcpy(d, &h, 4);
                std::memcpy(d + 4, &l, 4);
            } else {
                std::memcpy(d, &v, 8);
            }
        }
    }
    p->jit[si] = ks;
    p->jit_chain[si] = sh.chain != 0;
    p->jit_ready[si] = true;
    return 0;
}
}  // namespace

int chain_for(const HostPlan& hp, const JitShape& sh) {
    // float pairs between the passes of a double-single plan whose passes
    // are all specialised tile passes (an interpreted pass reads FP64); the
    // kernels between the passes of a reverse sweep read only probe partials
    if (hp.arith != QFVM_C128_DS || hp.passes.size() < 2) return 0;
    JitShape s0 = sh;
    s0.chain = 0;
    for (size_t i = 0; i < hp.passes.size(); ++i) {
        std::string k, why;
        if (hp.passes[i].type != PASS_TILE || !jit_pass_key(hp, static_cast<int>(i), s0, &k, &why)) return 0;
    }
    return 1;
}

int bounds_check_env() {
    const char* e = std::getenv("QFVM_BOUNDS_CHECK");
    return (e && e[0] == '1') ? 1 : 0;
}

int jit_status_take(cudaStream_t st) {
    uint32_t* d = status_word_if_any();
    if (d == nullptr) return 0;
    uint32_t v = 0;
    if (cudaMemcpyAsync(&v, d, sizeof v, cudaMemcpyDeviceToHost, st) != cudaSuccess) return QFVM_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return QFVM_ERR_CUDA;
    if (v == 0) return 0;
    cudaMemsetAsync(d, 0, sizeof v, st);
    cudaStreamSynchronize(st);
    return v == static_cast<uint32_t>(QFVM_ERR_BOUNDS) ? QFVM_ERR_BOUNDS : QFVM_ERR_TIMEOUT;
}

void jit_set_wait_test(uint32_t extra, uint64_t wait_ns) {
    g_extra_tx.store(extra);
    g_wait_ns.store(wait_ns ? wait_ns : kDefaultWaitNs);
}

void jit_release(qfvm_plan* p) {
    for (int s = 0; s < 2; ++s) {
        p->jit[s].clear();
        p->jit_cblob[s].clear();
        p->jit_chain[s] = false;
        p->jit_ready[s] = false;
    }
}

int jit_compiled_passes(const qfvm_plan* p, int nstates) {
    const int si = nstates == 2 ? 1 : 0;
    int c = 0;
    for (const void* k : p->jit[si]) c += k != nullptr;
    return c;
}

cudaError_t jit_launch_pass(qfvm_plan* p, int pi, void* psi, void* lam, const void* dcoef, int items,
                            uint64_t cstride, const uint8_t* active, int per_tile, double* partial, int* grid_out,
                            cudaStream_t st, bool* launched) {
    *launched = false;
    const int nstates = lam ? 2 : 1;
    const int si = nstates - 1;
    if (!p->jit_ready[si]) {
        // never compile inside a stream capture: run interpreted instead
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return cudaSuccess;
        std::string err;
        jit_prepare(p, nstates, &err);
    }
    if (pi < 0 || pi >= static_cast<int>(p->jit[si].size()) || !p->jit[si][pi]) return cudaSuccess;
    // the kernels record a failed wait or bound in this device's status word;
    // without one (its allocation failed on this device) the pass is not
    // launched: the interpreting kernel runs it, or, inside a float-pair
    // chain, the run reports the failure
    void* a_status = status_word();
    if (a_status == nullptr) {
        *launched = p->jit_chain[si];
        return p->jit_chain[si] ? cudaErrorMemoryAllocation : cudaSuccess;
    }
    const Kernel* k = static_cast<const Kernel*>(p->jit[si][pi]);
    const HostPlan& hp = p->hp;
    uint64_t ntiles = static_cast<uint64_t>(items) << (hp.n - hp.T);
    const unsigned grid = static_cast<unsigned>(ntiles < static_cast<uint64_t>(k->grid_cap) ? ntiles : k->grid_cap);
    void* a_psi = psi;
    void* a_lam = lam;
    const void* a_coef = dcoef;
    uint64_t a_cs = cstride;
    uint32_t a_ish = static_cast<uint32_t>(hp.n - hp.T);
    const void* a_act = active;
    int32_t a_pt = per_tile;
    void* a_part = partial;
    uint64_t a_wait = g_wait_ns.load();
    uint32_t a_extra = g_extra_tx.load();
    // the coefficient block (when the kernel takes one) is its last parameter
    const std::vector<std::vector<unsigned char>>& blobs = p->jit_cblob[si];
    void* a_blob = (pi < static_cast<int>(blobs.size()) && !blobs[pi].empty())
                       ? const_cast<unsigned char*>(blobs[pi].data())
                       : nullptr;
    void* args[] = {&a_psi, &a_lam, &ntiles, &a_coef, &a_cs, &a_ish, &a_act, &a_pt, &a_part, &a_status, &a_wait, &a_extra,
                    a_blob};
    CUresult r = driver().launch(k->fn, grid, 1, 1, k->threads, 1, 1, static_cast<unsigned>(k->smem),
                                 reinterpret_cast<CUstream>(st), args, nullptr);
    if (grid_out) *grid_out = static_cast<int>(grid);
    if (r == CUDA_SUCCESS) {
        *launched = true;
        return cudaSuccess;
    }
    if (!p->jit_chain[si] &&
        (r == CUDA_ERROR_INVALID_VALUE || r == CUDA_ERROR_LAUNCH_OUT_OF_RESOURCES || r == CUDA_ERROR_INVALID_HANDLE)) {
        // a launch-configuration error leaves the context usable: the caller
        // runs the interpreting kernel for this pass instead
        static std::atomic<int> reported{0};
        if (reported.fetch_add(1) == 0)
            std::fprintf(stderr, "qfvm: specialised pass launch refused (%s); running the interpreting kernel\n",
                         cu_error(r).c_str());
        return cudaSuccess;
    }
    // anything else is reported with the driver's own code (the runtime and
    // driver APIs share the numbering of these errors); so is a refused
    // launch inside a float-pair chain, whose neighbours expect float pairs
    *launched = true;
    return static_cast<cudaError_t>(r);
}

}  // namespace qsv

using qsv_capi::fail;

extern "C" {

int qfvm_jit_configure(int32_t enabled, int32_t nb_one, int32_t minb_one, int32_t nb_two, int32_t minb_two) {
    if ((nb_one != 1 && nb_one != 2) || (nb_two != 1 && nb_two != 2) || minb_one < 0 || minb_two < 0 ||
        minb_one > 16 || minb_two > 16)
        return fail(QFVM_ERR_INVALID, "tile buffers must be 1 or 2 and minimum CTAs 0..16");
    qsv::JitConfig c;
    c.enabled = enabled ? 1 : 0;
    c.nb1 = nb_one;
    c.minb1 = minb_one;
    c.nb2 = nb_two;
    c.minb2 = minb_two;
    qsv::jit_set_config(c);
    return QFVM_OK;
}

int qfvm_jit_get_config(int32_t config[5]) {
    if (!config) return fail(QFVM_ERR_INVALID, "null argument");
    const qsv::JitConfig c = qsv::jit_config();
    config[0] = c.enabled;
    config[1] = c.nb1;
    config[2] = c.minb1;
    config[3] = c.nb2;
    config[4] = c.minb2;
    return QFVM_OK;
}

int qfvm_jit_pass_ptx(const qfvm_plan* plan, int32_t pass, int32_t nstates, char* text, int64_t capacity,
                      int64_t* len) {
    if (!plan || !len || (nstates != 1 && nstates != 2)) return fail(QFVM_ERR_INVALID, "bad argument");
    const qsv::JitShape sh = qsv::host_query_shape(plan, nstates);
    std::string ptx, why;
    if (!qsv::jit_pass_ptx(plan->hp, pass, sh, qsv::jit_entry_name(plan->hp.arith, nstates), &ptx, &why))
        return fail(QFVM_ERR_UNSUPPORTED, "pass runs interpreted: " + why);
    *len = static_cast<int64_t>(ptx.size());
    if (text) {
        if (capacity < *len + 1) return fail(QFVM_ERR_INVALID, "text buffer too small");
        std::memcpy(text, ptx.c_str(), ptx.size() + 1);
    }
    return QFVM_OK;
}

int qfvm_jit_pass_compile(const qfvm_plan* plan, int32_t pass, int32_t nstates, char* info, int64_t capacity) {
    if (!plan || (nstates != 1 && nstates != 2)) return fail(QFVM_ERR_INVALID, "bad argument");
    const qsv::JitShape sh = qsv::host_query_shape(plan, nstates);
    std::string ptx, why, image, err, log;
    if (!qsv::jit_pass_ptx(plan->hp, pass, sh, qsv::jit_entry_name(plan->hp.arith, nstates), &ptx, &why))
        return fail(QFVM_ERR_UNSUPPORTED, "pass runs interpreted: " + why);
    const bool ok = qsv::to_cubin(ptx, &image, &err, &log);
    if (info && capacity > 0) {
        const std::string& m = ok ? log : err;
        const size_t n = std::min<size_t>(m.size(), static_cast<size_t>(capacity - 1));
        std::memcpy(info, m.data(), n);
        info[n] = 0;
    }
    return ok ? QFVM_OK : fail(QFVM_ERR_INVALID, err);
}

int qfvm_jit_plan_passes(const qfvm_plan* plan, int32_t nstates, int64_t* count) {
    if (!plan || !count) return fail(QFVM_ERR_INVALID, "null argument");
    *count = qsv::jit_compiled_passes(plan, nstates);
    return QFVM_OK;
}

}  // extern "C"
