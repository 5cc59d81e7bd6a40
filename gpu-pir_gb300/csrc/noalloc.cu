// sp_fold_noalloc: the GSW fold for callers that cannot allocate device
// memory.
//
// Some callers are not allowed to call cudaMalloc when they need an answer:
// code running inside a CUDA stream capture or a stream-ordered section, a
// host process whose device memory is handed out by another allocator, or a
// service that reserves all of its memory once at start-up and forbids
// allocation afterwards.  sp_fold allocates its device buffers per call; this
// variant takes its device storage from one fixed array that the library
// declares at file scope, so a call allocates nothing.
//
// The array is FOLD_SCRATCH_BYTES (8 MiB + 4 KiB).  It exists on every GPU on
// which the library is loaded, for as long as the process runs.  It holds the
// ciphertexts being folded (in place), the GSW ciphertexts as uploaded and in
// Montgomery form, and the launch descriptor; every region is fully written
// by a call before the kernels read it, so nothing needs clearing and the
// contents left by the previous call are never read.
#include <mutex>

#include "answer.cuh"
#include "ctx_view.h"

namespace {

constexpr uint64_t FOLD_SCRATCH_BYTES = (8ull << 20) + 4096;
constexpr int MAX_DEVICES = 256;

static __device__ __align__(256) uint8_t g_fold_scratch[FOLD_SCRATCH_BYTES];

// Device address of g_fold_scratch per device, resolved on the first call
// made with that device current.  In host code the symbol's name is only a
// host-side handle, never a device address; the kernels get this pointer.
std::mutex g_scratch_mu;
uint8_t *g_scratch_addr[MAX_DEVICES] = {};

int scratch_of_current_device(uint8_t **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return sp::set_last_error(SP_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES) return sp::set_last_error(SP_ERR_UNSUPPORTED, "device index too large");
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_fold_scratch);
        if (e != cudaSuccess || !p)
            return sp::set_last_error(SP_ERR_CUDA, "cudaGetSymbolAddress of the fold scratch failed");
        g_scratch_addr[dev] = static_cast<uint8_t *>(p);
    }
    *out = g_scratch_addr[dev];
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
    const uint64_t raw_bytes = (((uint64_t)T * 2 * D) << nu2) * 8;
    const uint64_t gwords = (uint64_t)nu2 * 2 * 2 * v.params.t_gsw * 2 * D;
    const uint64_t need = round256(raw_bytes) + round256(gwords * 8) + round256(gwords * 4) + round256(sizeof(QDesc));
    if (need > FOLD_SCRATCH_BYTES)
        return set_last_error(SP_ERR_INVALID,
                              "sp_fold_noalloc: inputs need more than its fixed 8 MiB device scratch "
                              "(T * 2^nu2 * 32 KiB of ciphertexts plus the GSW ciphertexts); use sp_fold");
    // One lock for the whole process: every call shares the same array, so
    // calls must not overlap on the GPU; each call waits for its work below.
    std::lock_guard<std::mutex> lk_scratch(g_scratch_mu);
    std::lock_guard<std::mutex> lk_ctx(*v.mu);
    uint8_t *base = nullptr;
    rc = scratch_of_current_device(&base);
    if (rc) return rc;
    uint64_t *d_raw = reinterpret_cast<uint64_t *>(base);
    uint64_t *d_g64 = reinterpret_cast<uint64_t *>(base + round256(raw_bytes));
    uint32_t *d_g32 = reinterpret_cast<uint32_t *>(base + round256(raw_bytes) + round256(gwords * 8));
    QDesc *d_qd = reinterpret_cast<QDesc *>(base + round256(raw_bytes) + round256(gwords * 8) + round256(gwords * 4));
    QDesc d{};
    d.raw = d_raw;
    d.gsw = d_g32;
    d.nu2 = nu2;
    d.active = 1;
    StageParams sp = v.params;
    sp.T = T;
    cudaError_t e = cudaMemcpyAsync(d_raw, cts, raw_bytes, cudaMemcpyHostToDevice, v.st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_g64, gsw, gwords * 8, cudaMemcpyHostToDevice, v.st);
    if (e == cudaSuccess) e = launch_narrow(d_g64, d_g32, gwords / D, true, v.st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_qd, &d, sizeof(QDesc), cudaMemcpyHostToDevice, v.st);
    for (int lvl = 0; lvl < nu2 && e == cudaSuccess; lvl++)
        e = launch_fold_level(d_qd, 1, lvl, T << (nu2 - 1 - lvl), sp, v.tw, nullptr, v.st);
    for (int t = 0; t < T && e == cudaSuccess; t++)
        e = cudaMemcpyAsync(out + (uint64_t)t * 2 * D, d_raw + ((uint64_t)t << nu2) * 2 * D, 2ull * D * 8,
                            cudaMemcpyDeviceToHost, v.st);
    cudaError_t s = cudaStreamSynchronize(v.st);
    if (e == cudaSuccess) e = s;
    if (e != cudaSuccess) return set_last_error(SP_ERR_CUDA, cudaGetErrorString(e));
    return SP_OK;
}
