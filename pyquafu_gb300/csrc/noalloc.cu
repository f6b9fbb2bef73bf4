// Allocation-free Pauli expectation on a caller-owned device state.
//
// Some callers cannot allocate GPU memory once they are running: serving
// processes that reserve the whole HBM budget for their own pool at start-up,
// or latency-critical loops where cudaMalloc / cudaFree would synchronise the
// device and stall every other stream.  For them this file provides one entry
// point that computes <P_k> without any allocation: its scratch (per-block
// partial sums, the uploaded term masks and the results) lives in a
// file-scope __device__ array of fixed size, loaded with the library and held
// by every GPU that loads it until the process exits.
//
// Limits and sharing:
//   * at most QFVM_NOALLOC_MAX_TERMS Pauli terms per call;
//   * the scratch array is shared by every call on a device and keeps the last
//     call's contents; each call rewrites all the entries it reads, so
//     nothing has to start at zero, but calls that overlap on the GPU (from
//     several host threads or streams) race on it and must be serialised by
//     the caller;
//   * the first call on each device looks the array's device address up with
//     cudaGetSymbolAddress (with that device current) and caches it;
//   * a call waits for its own results (cudaStreamSynchronize) and copies
//     through pageable host memory, so it cannot be recorded into a stream
//     capture: on a capturing stream it returns QFVM_ERR_UNSUPPORTED before
//     touching the stream;
//   * the state must be device (or managed) memory of the current device;
//     anything else (a host pointer, another GPU's memory) is refused with
//     QFVM_ERR_INVALID before any launch.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "kernels.h"
#include "qfvm_gb300.h"
#include "reduce.cuh"

namespace {

constexpr int MAXT = QFVM_NOALLOC_MAX_TERMS;
constexpr size_t PARTIAL_BYTES = sizeof(double) * qsv::REDUCE_BLOCKS * qsv::EXPECT_BATCH;
constexpr size_t ZM_OFF = PARTIAL_BYTES;
constexpr size_t NY_OFF = ZM_OFF + sizeof(uint64_t) * MAXT;
constexpr size_t OUT_OFF = NY_OFF + sizeof(int32_t) * MAXT;
constexpr size_t SCRATCH_BYTES = OUT_OFF + sizeof(double) * MAXT;
static_assert(SCRATCH_BYTES <= 64 * 1024, "allocation-free scratch stays below 64 KiB");

// The scratch itself.  In host code this name is only a stand-in for the
// symbol; kernels receive the device address obtained from
// cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
void* g_scratch_ptr[MAX_DEVICES] = {nullptr};

// last error message of the calling thread (fixed buffer: no allocation)
thread_local char g_noalloc_err[256] = "";

int nfail(int code, const char* what, const char* detail = "") {
    std::snprintf(g_noalloc_err, sizeof(g_noalloc_err), "%s%s%s", what, detail[0] ? ": " : "", detail);
    return code;
}

// Once per device, with that device current: the scratch array's address.
int scratch_for_current_device(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return nfail(QFVM_ERR_NODEVICE, "cudaGetDevice", cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES) return nfail(QFVM_ERR_UNSUPPORTED, "device index beyond the scratch table");
    void* p = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        p = g_scratch_ptr[dev];
    }
    if (!p) {
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) return nfail(QFVM_ERR_CUDA, "cudaGetSymbolAddress", cudaGetErrorString(e));
        std::lock_guard<std::mutex> lk(g_mu);
        g_scratch_ptr[dev] = p;
    }
    *out = static_cast<unsigned char*>(p);
    return QFVM_OK;
}

#define NA_CUDA(call, what)                                                                       \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return nfail(QFVM_ERR_CUDA, what, cudaGetErrorString(e_));       \
    } while (0)

}  // namespace

extern "C" const char* qfvm_noalloc_last_error(void) { return g_noalloc_err; }

extern "C" int qfvm_expect_device_noalloc(const void* dev_state, uint64_t state_len, int32_t precision,
                                          const uint64_t* x_masks, const uint64_t* z_masks,
                                          const int32_t* y_counts, int64_t n_terms, double* out, void* stream) {
    using namespace qsv;
    if (!dev_state || !x_masks || !z_masks || !y_counts || !out)
        return nfail(QFVM_ERR_INVALID, "null argument");
    if (precision != QFVM_C128 && precision != QFVM_C64)
        return nfail(QFVM_ERR_INVALID, "precision must be QFVM_C128 or QFVM_C64");
    if (state_len < 2 || (state_len & (state_len - 1)) != 0 || state_len > (1ULL << QFVM_MAX_QUBITS))
        return nfail(QFVM_ERR_INVALID, "state length must be a power of two between 2 and 2^34");
    if (n_terms < 0 || n_terms > MAXT)
        return nfail(QFVM_ERR_INVALID, "n_terms must be between 0 and QFVM_NOALLOC_MAX_TERMS (1024)");
    if (n_terms == 0) return QFVM_OK;
    const uint64_t lim = state_len - 1;
    for (int64_t t = 0; t < n_terms; ++t)
        if ((x_masks[t] | z_masks[t]) & ~lim) return nfail(QFVM_ERR_INVALID, "Pauli term acts outside the state");

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    NA_CUDA(cudaStreamIsCapturing(st, &cs), "cudaStreamIsCapturing");
    if (cs != cudaStreamCaptureStatusNone)
        return nfail(QFVM_ERR_UNSUPPORTED, "the allocation-free expectation cannot run inside a stream capture");
    int dev = 0;
    NA_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    cudaPointerAttributes attr;
    std::memset(&attr, 0, sizeof(attr));
    if (cudaPointerGetAttributes(&attr, dev_state) != cudaSuccess) {
        cudaGetLastError();  // the lookup's error is not sticky: clear it for the caller
        return nfail(QFVM_ERR_INVALID, "dev_state is not a pointer the CUDA runtime knows");
    }
    if ((attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged) || attr.device != dev)
        return nfail(QFVM_ERR_INVALID, "dev_state is not device memory of the current device");
    const size_t elem = precision == QFVM_C64 ? 8 : 16;
    if (reinterpret_cast<uintptr_t>(dev_state) % elem != 0)
        return nfail(QFVM_ERR_INVALID, "dev_state is not aligned to one amplitude");

    unsigned char* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != QFVM_OK) return rc;
    double* d_partial = reinterpret_cast<double*>(scratch);
    uint64_t* d_zm = reinterpret_cast<uint64_t*>(scratch + ZM_OFF);
    int32_t* d_ny = reinterpret_cast<int32_t*>(scratch + NY_OFF);
    double* d_out = reinterpret_cast<double*>(scratch + OUT_OFF);

    // group the terms by flip mask (fixed-size stack arrays: no allocation)
    int32_t order[MAXT];
    uint64_t hz[MAXT];
    int32_t hy[MAXT];
    double hres[MAXT];
    bool taken[MAXT];
    int64_t m = 0;
    for (int64_t t = 0; t < n_terms; ++t) taken[t] = false;
    for (int64_t t = 0; t < n_terms; ++t) {
        if (taken[t]) continue;
        for (int64_t u = t; u < n_terms; ++u) {
            if (!taken[u] && x_masks[u] == x_masks[t]) {
                taken[u] = true;
                order[m] = static_cast<int32_t>(u);
                hz[m] = z_masks[u];
                hy[m] = y_counts[u];
                ++m;
            }
        }
    }
    NA_CUDA(cudaMemcpyAsync(d_zm, hz, sizeof(uint64_t) * n_terms, cudaMemcpyHostToDevice, st), "term upload");
    NA_CUDA(cudaMemcpyAsync(d_ny, hy, sizeof(int32_t) * n_terms, cudaMemcpyHostToDevice, st), "term upload");
    const int nblocks = static_cast<int>(state_len / 2048 < static_cast<uint64_t>(REDUCE_BLOCKS)
                                             ? (state_len / 2048 > 0 ? state_len / 2048 : 1)
                                             : REDUCE_BLOCKS);
    for (int64_t i = 0; i < m;) {
        const uint64_t x = x_masks[order[i]];
        int64_t cnt = 0;
        while (i + cnt < m && cnt < EXPECT_BATCH && x_masks[order[i + cnt]] == x) ++cnt;
        if (x == 0) {
            if (precision == QFVM_C64)
                k_expect_z<P32><<<nblocks, 256, 0, st>>>(static_cast<const float2*>(dev_state), state_len, d_zm + i,
                                                         static_cast<int>(cnt), d_partial);
            else
                k_expect_z<P64><<<nblocks, 256, 0, st>>>(static_cast<const double2*>(dev_state), state_len, d_zm + i,
                                                         static_cast<int>(cnt), d_partial);
        } else {
            const int flip_q = 63 - __builtin_clzll(x);
            if (precision == QFVM_C64)
                k_expect_x<P32><<<nblocks, 256, 0, st>>>(static_cast<const float2*>(dev_state), state_len, x, flip_q,
                                                         d_zm + i, d_ny + i, static_cast<int>(cnt), d_partial);
            else
                k_expect_x<P64><<<nblocks, 256, 0, st>>>(static_cast<const double2*>(dev_state), state_len, x, flip_q,
                                                         d_zm + i, d_ny + i, static_cast<int>(cnt), d_partial);
        }
        NA_CUDA(cudaGetLastError(), "expectation kernel");
        k_reduce_partials<<<1, 256, 0, st>>>(d_partial, nblocks, static_cast<int>(cnt), d_out + i);
        NA_CUDA(cudaGetLastError(), "reduction kernel");
        i += cnt;
    }
    NA_CUDA(cudaMemcpyAsync(hres, d_out, sizeof(double) * n_terms, cudaMemcpyDeviceToHost, st), "result download");
    NA_CUDA(cudaStreamSynchronize(st), "stream synchronize");
    for (int64_t i = 0; i < m; ++i) out[order[i]] = hres[i];
    return QFVM_OK;
}
