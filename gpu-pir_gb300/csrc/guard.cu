// Guard-region check of the checked mode: every region (address, length)
// must still hold the fill byte it was initialised with.  The lowest index
// of a region that differs is written to *bad (left unchanged when all hold).
#include "kernels.cuh"

namespace sp {

__global__ void k_check_guards(const uint64_t *__restrict__ regions, int n, uint8_t fill, uint32_t *bad) {
    for (int r = blockIdx.x; r < n; r += gridDim.x) {
        const uint8_t *p = reinterpret_cast<const uint8_t *>(regions[2 * r]);
        const uint64_t len = regions[2 * r + 1];
        bool ok = true;
        for (uint64_t i = threadIdx.x; i < len; i += blockDim.x) ok &= p[i] == fill;
        if (!ok) atomicMin(bad, (uint32_t)r);
    }
}

cudaError_t launch_check_guards(const uint64_t *regions, int n, uint8_t fill, uint32_t *bad, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_check_guards<<<n < 1024 ? n : 1024, 256, 0, st>>>(regions, n, fill, bad);
    return cudaGetLastError();
}

}  // namespace sp
