// Internal read-only view of a context, for entry points that live outside
// api.cu.  Not part of the C ABI.
#pragma once
#include <mutex>

#include "../../include/spiralpir.h"
#include "kernels.cuh"

namespace sp {

struct CtxView {
    cudaStream_t st;
    const TwiddleSet *tw;
    StageParams params;
    std::mutex *mu;
    int device;      // the GPU the context (its stream, memory) lives on
    bool checked;    // checked mode (guard regions verified after calls)
};

// Fills `out` for a live context; returns SP_OK or an error code.
int ctx_view(sp_ctx *c, CtxView *out);
// Records `msg` as the calling thread's last error and returns `code`.
int set_last_error(int code, const char *msg);

}  // namespace sp
