// Seed expansion of public parameters on the device (the plan of
// gpu-pir/optplan.md:88-92): a client may send a 32-byte seed in place of
// the uniform row 0 of every key matrix, and the library regenerates those
// rows here, straight into the key buffer in Montgomery form.
//
// Stream: the ChaCha20 block function of RFC 8439 (20 rounds) with
// key = seed, counter = block b, nonce = (poly index P, prime index k,
// SEED_DOMAIN); block b gives residues 8b .. 8b+7 of the polynomial's plane
// mod q_k, residue z from block words 2(z mod 8) (low) and 2(z mod 8)+1
// (high), reduced mod q_k.  The host restatement is spiralpir/prg.py.
#include "seeded.cuh"

namespace sp {

namespace {

constexpr uint32_t SEED_DOMAIN = 0x3153504Bu;

__device__ __forceinline__ uint32_t rotl(uint32_t x, int n) { return __funnelshift_l(x, x, n); }

__device__ __forceinline__ void quarter(uint32_t &a, uint32_t &b, uint32_t &c, uint32_t &d) {
    a += b; d ^= a; d = rotl(d, 16);
    c += d; b ^= c; b = rotl(b, 12);
    a += b; d ^= a; d = rotl(d, 8);
    c += d; b ^= c; b = rotl(b, 7);
}

// One thread per (row-0 polynomial P, prime k, block b): 8 residues.
__global__ void k_seed_rows(SeedKey key, SeedRowMap map, uint32_t *__restrict__ keys) {
    const uint64_t total = (uint64_t)map.polys * 2 * (D / 8);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = (uint32_t)(i % (D / 8));
        const uint32_t k = (uint32_t)((i / (D / 8)) % 2);
        const uint32_t P = (uint32_t)(i / (2 * (D / 8)));
        const uint32_t in[16] = {0x61707865u, 0x3320646Eu, 0x79622D32u, 0x6B206574u,
                                 key.w[0], key.w[1], key.w[2], key.w[3], key.w[4], key.w[5], key.w[6], key.w[7],
                                 b, P, k, SEED_DOMAIN};
        uint32_t x[16];
#pragma unroll
        for (int j = 0; j < 16; j++) x[j] = in[j];
#pragma unroll 1
        for (int r = 0; r < 10; r++) {
            quarter(x[0], x[4], x[8], x[12]);
            quarter(x[1], x[5], x[9], x[13]);
            quarter(x[2], x[6], x[10], x[14]);
            quarter(x[3], x[7], x[11], x[15]);
            quarter(x[0], x[5], x[10], x[15]);
            quarter(x[1], x[6], x[11], x[12]);
            quarter(x[2], x[7], x[8], x[13]);
            quarter(x[3], x[4], x[9], x[14]);
        }
        const Prime c = prime_of((int)k);
        uint32_t *dst = keys + map.offset(P) + (uint64_t)k * D + 8 * b;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const uint32_t lo = x[2 * j] + in[2 * j], hi = x[2 * j + 1] + in[2 * j + 1];
            const uint32_t r = mod_u64(((uint64_t)(hi % c.p) << 32) | lo, c);    // canonical
            const uint32_t m = mont_mul(r, c.r2, c.p, c.pinv);                   // Montgomery form
            dst[j] = min(m, m - c.p);
        }
    }
}

}  // namespace

// Word offset (in the client key buffer) of row-0 polynomial P.
__host__ __device__ uint64_t SeedRowMap::offset(uint32_t P) const {
    const uint64_t poly = 2ull * D;
    if (P < (uint32_t)(n_left * t_left)) {
        const uint32_t r = P / t_left, j = P % t_left;
        return ((uint64_t)r * 2 * t_left + j) * poly;                         // left [r][row 0][j]
    }
    P -= n_left * t_left;
    const uint64_t base_r = (uint64_t)n_left * 2 * t_left * poly;
    if (P < (uint32_t)(n_right * t_right)) {
        const uint32_t r = P / t_right, j = P % t_right;
        return base_r + ((uint64_t)r * 2 * t_right + j) * poly;               // right [r][row 0][j]
    }
    P -= n_right * t_right;
    const uint64_t base_c = base_r + (uint64_t)n_right * 2 * t_right * poly;
    if (P < (uint32_t)(2 * t_conv)) return base_c + (uint64_t)P * poly;     // conv [row 0][j]
    P -= 2 * t_conv;
    const uint64_t base_p = base_c + 2ull * 2 * t_conv * poly;
    const uint32_t r = P / t_conv, j = P % t_conv;
    return base_p + ((uint64_t)r * (n + 1) * t_conv + j) * poly;              // pack [r][row 0][j]
}

cudaError_t launch_seed_rows(const SeedKey &key, const SeedRowMap &map, uint32_t *keys, cudaStream_t st) {
    const uint64_t total = (uint64_t)map.polys * 2 * (D / 8);
    if (!total) return cudaSuccess;
    const int blocks = (int)std::min<uint64_t>((total + 255) / 256, 8192);
    k_seed_rows<<<blocks, 256, 0, st>>>(key, map, keys);
    return cudaGetLastError();
}

}  // namespace sp
