// sp_fold_noalloc: the GSW fold for callers that cannot allocate device
// memory.
//
// Some callers are not allowed to call cudaMalloc when they need an answer:
// a host process whose device memory is handed out by another allocator (a
// framework's caching allocator that already holds the GPU's free memory),
// or a service that reserves all of its memory once at start-up and forbids
// allocation afterwards.  sp_fold allocates its device buffers per call; this
// variant takes its device storage from one fixed array that the library
// declares at file scope, so a call allocates nothing.
//
// The array is FOLD_SCRATCH_BYTES (8 MiB + 4 KiB).  It exists on every GPU on
// which the library is loaded, for as long as the process runs.  It holds the
// ciphertexts being folded (in place), the GSW ciphertexts as uploaded and in
// Montgomery form, the launch descriptor and, in checked mode, a guard region
// with the guard check's region list and result word.  Every region is fully
// written by a call before the kernels read it, so nothing needs clearing and
// the contents left by the previous call are never read.
#include <mutex>

#include <nvtx3/nvToolsExt.h>

#include "answer.cuh"
#include "ctx_view.h"

namespace {

constexpr uint64_t FOLD_SCRATCH_BYTES = (8ull << 20) + 4096;
// Kept free after the data in every call: in checked mode a guard region of
// GUARD_BYTES (filled with GUARD_FILL before the fold, verified after it),
// then the check's region list (16 bytes) and result word.
constexpr uint64_t GUARD_BYTES = 1024;
constexpr uint64_t TAIL_BYTES = GUARD_BYTES + 256;
constexpr uint8_t GUARD_FILL = 0xA5;
constexpr int MAX_DEVICES = 256;

static __device__ __align__(256) uint8_t g_fold_scratch[FOLD_SCRATCH_BYTES];

// Device address of g_fold_scratch per device, resolved with that device
// current on the first call for a context on it.  In host code the symbol's
// name is only a host-side handle, never a device address; the kernels get
// this pointer.
std::mutex g_scratch_mu;
uint8_t *g_scratch_addr[MAX_DEVICES] = {};

// Makes `device` current for the scope of a call and restores the caller's
// current device afterwards (the context's stream and twiddles live there,
// and so must the array copy the kernels use).
struct DeviceScope {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceScope(int device) {
        int cur = 0;
        err = cudaGetDevice(&cur);
        if (err == cudaSuccess && cur != device) {
            err = cudaSetDevice(device);
            if (err == cudaSuccess) prev = cur;
        }
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

struct TraceRange {
    TraceRange() { nvtxRangePushA("sp_fold_noalloc"); }
    ~TraceRange() { nvtxRangePop(); }
};

// The array's device address on `device`, which must be current.
int scratch_of_device(int device, uint8_t **out) {
    if (device < 0 || device >= MAX_DEVICES) return sp::set_last_error(SP_ERR_UNSUPPORTED, "device index too large");
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_fold_scratch);
        if (e != cudaSuccess || !p)
            return sp::set_last_error(SP_ERR_CUDA, "cudaGetSymbolAddress of the fold scratch failed");
        g_scratch_addr[device] = static_cast<uint8_t *>(p);
    }
    *out = g_scratch_addr[device];
    return SP_OK;
}

uint64_t round256(uint64_t x) { return (x + 255) & ~255ull; }

}  // namespace

extern "C" int sp_fold_noalloc(sp_ctx *ctx, const uint64_t *cts, const uint64_t *gsw, int32_t T, int32_t nu2,
                               uint64_t *out) {
    using namespace sp;
    if (!ctx || !cts || !gsw || !out) return set_last_error(SP_ERR_INVALID, "NULL argument");
    CtxView v;
    int rc = ctx_view(ctx, &v);
    if (rc) return rc;
    if (T < 1 || T > v.params.T || nu2 < 1 || nu2 > 14)
        return set_last_error(SP_ERR_INVALID, "T or nu2 out of range");
    TraceRange trace;
    const uint64_t raw_bytes = (((uint64_t)T * 2 * D) << nu2) * 8;
    const uint64_t gwords = (uint64_t)nu2 * 2 * 2 * v.params.t_gsw * 2 * D;
    const uint64_t data = round256(raw_bytes) + round256(gwords * 8) + round256(gwords * 4) + round256(sizeof(QDesc));
    if (data + TAIL_BYTES > FOLD_SCRATCH_BYTES)
        return set_last_error(SP_ERR_INVALID,
                              "sp_fold_noalloc: inputs need more than its fixed 8 MiB device scratch "
                              "(T * 2^nu2 * 32 KiB of ciphertexts plus nu2 * t_gsw * 192 KiB for the GSW "
                              "ciphertexts); use sp_fold");
    // One lock for the whole process: every call shares the same array, so
    // calls must not overlap on the GPU; each call waits for its work below.
    std::lock_guard<std::mutex> lk_scratch(g_scratch_mu);
    std::lock_guard<std::mutex> lk_ctx(*v.mu);
    DeviceScope dev(v.device);
    if (dev.err != cudaSuccess) return set_last_error(SP_ERR_CUDA, cudaGetErrorString(dev.err));
    uint8_t *base = nullptr;
    rc = scratch_of_device(v.device, &base);
    if (rc) return rc;
    uint64_t *d_raw = reinterpret_cast<uint64_t *>(base);
    uint64_t *d_g64 = reinterpret_cast<uint64_t *>(base + round256(raw_bytes));
    uint32_t *d_g32 = reinterpret_cast<uint32_t *>(base + round256(raw_bytes) + round256(gwords * 8));
    QDesc *d_qd = reinterpret_cast<QDesc *>(base + round256(raw_bytes) + round256(gwords * 8) + round256(gwords * 4));
    uint8_t *guard = base + data;
    uint64_t *d_list = reinterpret_cast<uint64_t *>(guard + GUARD_BYTES);
    uint32_t *d_bad = reinterpret_cast<uint32_t *>(guard + GUARD_BYTES + 16);
    QDesc d{};
    d.raw = d_raw;
    d.gsw = d_g32;
    d.nu2 = nu2;
    d.active = 1;
    StageParams sp = v.params;
    sp.T = T;
    const uint64_t list[2] = {(uint64_t)(uintptr_t)guard, GUARD_BYTES};
    uint32_t bad = 0xffffffffu;
    cudaError_t e = cudaSuccess;
    if (v.checked) e = cudaMemsetAsync(guard, GUARD_FILL, GUARD_BYTES, v.st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_raw, cts, raw_bytes, cudaMemcpyHostToDevice, v.st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_g64, gsw, gwords * 8, cudaMemcpyHostToDevice, v.st);
    if (e == cudaSuccess) e = launch_narrow(d_g64, d_g32, gwords / D, true, v.st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_qd, &d, sizeof(QDesc), cudaMemcpyHostToDevice, v.st);
    for (int lvl = 0; lvl < nu2 && e == cudaSuccess; lvl++)
        e = launch_fold_level(d_qd, 1, lvl, T << (nu2 - 1 - lvl), sp, v.tw, nullptr, v.st);
    for (int t = 0; t < T && e == cudaSuccess; t++)
        e = cudaMemcpyAsync(out + (uint64_t)t * 2 * D, d_raw + ((uint64_t)t << nu2) * 2 * D, 2ull * D * 8,
                            cudaMemcpyDeviceToHost, v.st);
    if (v.checked) {
        // the guard after the data must still hold its fill
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_list, list, sizeof(list), cudaMemcpyHostToDevice, v.st);
        if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0xff, sizeof(uint32_t), v.st);
        if (e == cudaSuccess) e = launch_check_guards(d_list, 1, GUARD_FILL, d_bad, v.st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(uint32_t), cudaMemcpyDeviceToHost, v.st);
    }
    const cudaError_t s = cudaStreamSynchronize(v.st);
    if (e == cudaSuccess) e = s;
    if (e != cudaSuccess) return set_last_error(SP_ERR_CUDA, cudaGetErrorString(e));
    if (bad != 0xffffffffu)
        return set_last_error(SP_ERR_DEVICE, "device buffer overrun: the guard after the sp_fold_noalloc data "
                                             "in its fixed array was overwritten");
    return SP_OK;
}
