// Batched NTT / inverse NTT / automorphism kernels (R1, R2, R3, R7).
#include "kernels.cuh"

namespace sp {

namespace {

uint32_t brev11(uint32_t x) {
    uint32_t r = 0;
    for (int i = 0; i < LOGD; i++) { r = (r << 1) | (x & 1); x >>= 1; }
    return r;
}

// Restride entries of the last three stages for layout C (entry m + k*128 + t
// holds twiddle m + c*t + k, c = m/128); other entries stay in place.
void restride(const uint32_t *plain, uint32_t *out) {
    for (int i = 0; i < 256; i++) out[i] = plain[i];
    for (int L = 8; L < 11; L++) {
        const int m = 1 << L, c = m / GROUP;
        for (int t = 0; t < GROUP; t++)
            for (int k = 0; k < c; k++) out[m + k * GROUP + t] = plain[m + c * t + k];
    }
}

}  // namespace

void build_twiddles_host(TwiddleSet *h) {
    const uint32_t psi[2] = {66687u, 158221u};
    for (int k = 0; k < 2; k++) {
        const Prime c = prime_of(k);
        const uint64_t p = c.p;
        uint32_t f[D], fq[D], rf[D], rfq[D];
        for (uint32_t i = 0; i < (uint32_t)D; i++) {
            f[i] = (uint32_t)powmod_c(psi[k], brev11(i), p);
            fq[i] = (uint32_t)(((uint64_t)f[i] << 32) / p);      // Shoup companions
        }
        restride(f, rf);
        restride(fq, rfq);
        for (int i = 0; i < D; i++) h->t[k][i] = make_uint2(rf[i], rfq[i]);
    }
}

// Shared memory of the NTT kernels: 2 twiddle tables + 2 groups x 2 buffers.
constexpr int NTT_SMEM_WORDS = TW_WORDS + 2 * 2 * D;

__global__ void __launch_bounds__(256) k_to_ntt(const uint64_t *__restrict__ raw, uint32_t *__restrict__ out,
                                                int count, const TwiddleSet *__restrict__ tws) {
    extern __shared__ __align__(16) uint32_t smem[];
    load_twiddles(smem, tws);
    __syncthreads();
    const int g = threadIdx.x >> 7, t = threadIdx.x & (GROUP - 1);
    const Prime c = prime_of(g);
    uint32_t *buf = smem + TW_WORDS + g * 2 * D;
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        uint32_t v[VPT];
        const uint64_t *src = raw + (size_t)i * D;
#pragma unroll
        for (int j = 0; j < VPT; j++) v[j] = mod_u64(src[t + GROUP * j], c);
        ntt_fwd(v, tw_of(smem, g), buf, c, t, 1 + g);
#pragma unroll
        for (int j = 0; j < VPT; j++) v[j] = canon4(v[j], c.p);
        st16(out + ((size_t)i * 2 + g) * D + VPT * t, v);
    }
}

__global__ void __launch_bounds__(256) k_from_ntt(const uint32_t *__restrict__ in, uint64_t *__restrict__ raw,
                                                  int count, const TwiddleSet *__restrict__ tws) {
    extern __shared__ __align__(16) uint32_t smem[];
    load_twiddles(smem, tws);
    __syncthreads();
    const int g = threadIdx.x >> 7, t = threadIdx.x & (GROUP - 1);
    const Prime c = prime_of(g);
    uint32_t *buf = smem + TW_WORDS + g * 2 * D;
    // exchange area: reuse of the twiddle-free region is not possible (tables
    // are live), so it follows the group buffers.
    uint32_t *xch = smem + NTT_SMEM_WORDS;
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        uint32_t v[VPT];
        ld16(v, in + ((size_t)i * 2 + g) * D + VPT * t);
#pragma unroll
        for (int j = 0; j < VPT; j++) v[j] = reduce2(v[j], 2 * c.p) ;
        ntt_inv(v, tw_of(smem, g), buf, c, t, 1 + g);
#pragma unroll
        for (int j = 0; j < VPT; j++) xch[g * D + t + GROUP * j] = v[j];
        __syncthreads();
        uint64_t *dst = raw + (size_t)i * D;
#pragma unroll
        for (int k = 0; k < D / 256; k++) {
            const int e = threadIdx.x + 256 * k;
            dst[e] = icrt(xch[e], xch[D + e]);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_ntt_planes(uint32_t *__restrict__ a, int count, int inverse,
                                                    const TwiddleSet *__restrict__ tws) {
    extern __shared__ __align__(16) uint32_t smem[];
    load_twiddles(smem, tws);
    __syncthreads();
    const int g = threadIdx.x >> 7, t = threadIdx.x & (GROUP - 1);
    const Prime c = prime_of(g);
    uint32_t *buf = smem + TW_WORDS + g * 2 * D;
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        uint32_t *pl = a + ((size_t)i * 2 + g) * D;
        uint32_t v[VPT];
        if (!inverse) {
#pragma unroll
            for (int j = 0; j < VPT; j++) v[j] = pl[t + GROUP * j];
            ntt_fwd(v, tw_of(smem, g), buf, c, t, 1 + g);
#pragma unroll
            for (int j = 0; j < VPT; j++) v[j] = canon4(v[j], c.p);
            group_sync(1 + g);  // all reads of this plane done before writes
            st16(pl + VPT * t, v);
        } else {
            ld16(v, pl + VPT * t);
            ntt_inv(v, tw_of(smem, g), buf, c, t, 1 + g);
#pragma unroll
            for (int j = 0; j < VPT; j++) {
                uint32_t x = mont_mul(v[j], c.ninv_m, c.p, c.pinv);
                v[j] = min(x, x - c.p);
            }
            group_sync(1 + g);
#pragma unroll
            for (int j = 0; j < VPT; j++) pl[t + GROUP * j] = v[j];
        }
    }
}

__global__ void k_automorph(const uint64_t *__restrict__ in, uint64_t *__restrict__ out, int count,
                            uint32_t tau) {
    const size_t total = (size_t)count * D;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const size_t poly = idx / D;
        const uint32_t i = (uint32_t)(idx % D);
        const uint64_t it = (uint64_t)i * tau;
        const uint64_t v = in[idx];
        out[poly * D + (it % D)] = ((it / D) & 1) ? (v ? QQ - v : 0) : v;
    }
}

static int grid_for(int count) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int g = sms * 3;
    return count < g ? (count > 0 ? count : 1) : g;
}

template <typename K>
static cudaError_t set_smem(K kernel, int bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t launch_to_ntt(const uint64_t *raw, uint32_t *out, int count, const TwiddleSet *tw,
                          cudaStream_t st) {
    const int smem = NTT_SMEM_WORDS * 4;
    cudaError_t e = set_smem(k_to_ntt, smem);
    if (e != cudaSuccess) return e;
    k_to_ntt<<<grid_for(count), 256, smem, st>>>(raw, out, count, tw);
    return cudaGetLastError();
}

cudaError_t launch_from_ntt(const uint32_t *in, uint64_t *raw, int count, const TwiddleSet *tw,
                            cudaStream_t st) {
    const int smem = (NTT_SMEM_WORDS + 2 * D) * 4;
    cudaError_t e = set_smem(k_from_ntt, smem);
    if (e != cudaSuccess) return e;
    k_from_ntt<<<grid_for(count), 256, smem, st>>>(in, raw, count, tw);
    return cudaGetLastError();
}

cudaError_t launch_ntt_planes(uint32_t *a, int count, bool inverse, const TwiddleSet *tw,
                              cudaStream_t st) {
    const int smem = NTT_SMEM_WORDS * 4;
    cudaError_t e = set_smem(k_ntt_planes, smem);
    if (e != cudaSuccess) return e;
    k_ntt_planes<<<grid_for(count), 256, smem, st>>>(a, count, inverse ? 1 : 0, tw);
    return cudaGetLastError();
}

cudaError_t launch_automorph(const uint64_t *in, uint64_t *out, int count, uint32_t t,
                             cudaStream_t st) {
    const size_t total = (size_t)count * D;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    k_automorph<<<blocks, 256, 0, st>>>(in, out, count, t);
    return cudaGetLastError();
}

}  // namespace sp
