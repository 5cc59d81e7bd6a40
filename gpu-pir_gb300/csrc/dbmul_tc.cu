// Tensor-core first-dimension multiply for batches of queries (R11, batched).
//
// For one slot z and one prime the multiply of B queries is a plain matrix
// product:  out[m][n] = sum_row DB[m][row] * SEL[row][n]  (mod p), with m one
// of the 128 combos of an image unit, n = 2*query + ciphertext row, and
// row < 2^nu1.  Residues are < 2^28, so the product is made exact on the
// fp16 tensor cores by splitting both operands into four signed digits:
//   x (centred to (-p/2, p/2]) = a0 + a1*2^7 + a2*2^14 + a3*2^21,
//   a0..a2 in [-64, 63], a3 in [-64, 64]   (all exactly representable in fp16)
// and accumulating the 16 digit products by weight class d = i + j in seven
// fp32 accumulators C_d.  Every product is at most 2^12 in magnitude and a
// class holds at most 4 digit pairs, so |C_d| <= 4 * 512 * 2^12 = 2^23 for up
// to 512 rows: every partial sum is an integer below 2^24, which fp32 holds
// exactly.  The epilogue returns sum_d C_d * (2^(7d) mod p) reduced mod p,
// bit-identical to the integer-pipe multiplies.
//
// Layout of the work (tcgen05, cta_group::1, kind::f16, M = 128, N = 2B
// rounded up to 16 (<= 64), K = 16 per instruction):
//  * A = database digits, 128 combos x 32 rows per stage, K-major canonical
//    (no swizzle: 8x8 core matrices of 128 B, SBO = 128 B between 8-combo
//    groups, LBO = 2 KiB between 8-row groups), written to shared memory by
//    the converter warps from the u32 image;
//  * B = selector digits, prepared once per batch by k_tc_limbs in the same
//    canonical form (SBO = 128 B, LBO = N*16 B) and fetched per stage with one
//    1-D bulk TMA copy;
//  * D = seven accumulators of N fp32 columns each in tensor memory (7*64 =
//    448 of the 512 columns).
// Warp roles of the persistent CTA (one per SM; 168 KiB of shared memory
// keeps it alone on its SM, so its 512-column TMEM allocation never waits):
//   warp 0      TMA producer of the selector stages
//   warp 1      TMEM allocation, MMA issue (one thread), TMEM release
//   warps 2..5  converters: image residues -> digit tiles
//   warps 6..9  epilogue: TMEM -> registers -> mod p -> accumulator planes
// Every barrier wait is bounded in time; a wait that runs out sets an error
// flag, the other roles stop at their next wait, in-flight copies and MMAs
// are drained (bounded), the TMEM is released and the kernel returns.
#include <cuda_fp16.h>

#include "async.cuh"
#include "kernels.cuh"

namespace sp {
namespace {

constexpr int TC_M = 128;
constexpr int TC_KC = 32;                     // rows per stage
constexpr int TC_NA = 3;                      // digit-tile (A) stages
constexpr int TC_NS = 4;                      // selector (B) stages
constexpr int TC_MAX_N = 2 * TC_MAX_Q;        // 64
constexpr uint32_t A_LIMB_BYTES = TC_M * TC_KC * 2;          // 8 KiB
constexpr uint32_t A_STAGE_BYTES = 4 * A_LIMB_BYTES;         // 32 KiB
constexpr uint32_t S_STAGE_MAX = 4 * TC_KC * TC_MAX_N * 2;   // 16 KiB
constexpr uint32_t A_RING = 0;
constexpr uint32_t S_RING = A_RING + TC_NA * A_STAGE_BYTES;  // 96 KiB
constexpr uint32_t GUARD = 8192;
constexpr uint32_t CTRL = S_RING + TC_NS * S_STAGE_MAX + GUARD;  // 168 KiB
constexpr uint32_t TC_SMEM = CTRL + 1024;
constexpr int TC_THREADS = 320;
constexpr uint32_t TMEM_COLS = 512;
constexpr int32_t DIGIT_BIAS = 64 * (1 + 128 + 128 * 128);   // 1056832

struct Ctrl {
    uint64_t s_full[TC_NS], s_empty[TC_NS];
    uint64_t a_full[TC_NA], a_empty[TC_NA];
    uint64_t acc_full, acc_empty, drain;
    uint32_t tmem_base;
    int abort;
    uint32_t *acc[TC_MAX_Q];
};
static_assert(sizeof(Ctrl) <= 1024, "control block");

// Digits of a canonical residue x < p, offset by +64 (u in [0, 128]).
__device__ __forceinline__ void digits4(uint32_t x, uint32_t p, uint32_t (&u)[4]) {
    const int32_t xc = (int32_t)x - (x > (p >> 1) ? (int32_t)p : 0);
    const int32_t y = xc + DIGIT_BIAS;
    u[0] = (uint32_t)y & 127u;
    u[1] = ((uint32_t)y >> 7) & 127u;
    u[2] = ((uint32_t)y >> 14) & 127u;
    u[3] = (uint32_t)((y >> 21) + 64);
}

// Two offset digits -> packed fp16 pair of the signed digits (lo, hi).
// 0x6400 | u is the fp16 value 1024 + u (u < 1024); subtracting 1088 is exact.
__device__ __forceinline__ uint32_t digit_pair(uint32_t ulo, uint32_t uhi) {
    uint32_t w = (ulo | (uhi << 16)) | 0x64006400u;
    __half2 h = *reinterpret_cast<__half2 *>(&w);
    h = __hsub2(h, __halves2half2(__ushort_as_half(0x6440), __ushort_as_half(0x6440)));   // 1088
    return *reinterpret_cast<uint32_t *>(&h);
}

__device__ __forceinline__ void sts128(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d)
                 : "memory");
}

// tcgen05 shared-memory matrix descriptor, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor: kind::f16, D fp32, A = B = fp16, both K-major.
__device__ __forceinline__ uint32_t instr_desc(int n) {
    return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

}  // namespace

// ------------------------------------------------------ selector digits
// Thread (n, z, row group of 8): n = 2*query + ciphertext row.  Writes, for
// both primes, the four digit planes of 8 consecutive rows as 16-byte rows of
// the canonical K-major B tiles:
//   limbs[prime][z][stage][digit][8-row group][N/8][8 n][8 rows]  (fp16)
__global__ void __launch_bounds__(256) k_tc_limbs(const QDesc *__restrict__ qd, int nq, int rows, int N,
                                                  uint8_t *__restrict__ limbs) {
    const uint64_t total = (uint64_t)N * D * (rows / 8);
    for (uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        const int n = (int)(idx % N);
        const uint64_t rest = idx / N;
        const int z = (int)(rest % D);
        const int rg = (int)(rest / D);
        const int b = n >> 1, k = n & 1;
        uint32_t x[2][8];
        if (b < nq) {
            const uint32_t *sel = qd[b].sel;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const uint2 v = __ldg(reinterpret_cast<const uint2 *>(sel + ((uint64_t)(rg * 8 + j) * D + z) * 4 + k * 2));
                x[0][j] = v.x;
                x[1][j] = v.y;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 8; j++) x[0][j] = x[1][j] = 0;
        }
        const int s = rg / 4, kg = rg % 4;
#pragma unroll
        for (int prime = 0; prime < 2; prime++) {
            const uint32_t p = prime ? QP1 : QP0;
            uint32_t u[8][4];
#pragma unroll
            for (int j = 0; j < 8; j++) digits4(x[prime][j], p, u[j]);
            uint8_t *base = limbs + ((uint64_t)prime * D + z) * rows * N * 8;
#pragma unroll
            for (int l = 0; l < 4; l++) {
                uint4 w;
                w.x = digit_pair(u[0][l], u[1][l]);
                w.y = digit_pair(u[2][l], u[3][l]);
                w.z = digit_pair(u[4][l], u[5][l]);
                w.w = digit_pair(u[6][l], u[7][l]);
                const uint64_t off = ((uint64_t)(s * 4 + l) * 4 + kg) * (N / 8) * 128 + (n / 8) * 128 + (n % 8) * 16;
                *reinterpret_cast<uint4 *>(base + off) = w;
            }
        }
    }
}

// ------------------------------------------------------------ multiply
__global__ void __launch_bounds__(TC_THREADS, 1) k_db_mul_tc(const uint32_t *__restrict__ db, DbLayout L,
                                                             const QDesc *__restrict__ qd, int nq, int N,
                                                             const uint8_t *__restrict__ limbs, int *err) {
    extern __shared__ __align__(1024) uint8_t smem_tc[];
    Ctrl &C = *reinterpret_cast<Ctrl *>(smem_tc + CTRL);
    volatile int *abort = &C.abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t sbase = smem_addr(smem_tc);
    const int rows = L.rows;
    const int S = rows / TC_KC;                        // stages per unit
    const uint32_t s_bytes = 4u * TC_KC * N * 2;       // selector stage bytes
    const uint64_t units = L.units();

    if (threadIdx.x == 0) {
        for (int i = 0; i < TC_NS; i++) {
            mbar_init(&C.s_full[i], 1);
            mbar_init(&C.s_empty[i], 1);
        }
        for (int i = 0; i < TC_NA; i++) {
            mbar_init(&C.a_full[i], 128);
            mbar_init(&C.a_empty[i], 1);
        }
        mbar_init(&C.acc_full, 1);
        mbar_init(&C.acc_empty, 128);
        mbar_init(&C.drain, 1);
        C.abort = 0;
        fence_mbar_init();
    }
    if (threadIdx.x < TC_MAX_Q) C.acc[threadIdx.x] = threadIdx.x < nq ? qd[threadIdx.x].acc : nullptr;
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(&C.tmem_base)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = C.tmem_base;

    if (warp == 0) {
        // ---------------------------------------------------- producer
        if (lane == 0) {
            uint32_t G = 0;
            bool stop = false;
            for (uint64_t u = blockIdx.x; u < units && !stop; u += gridDim.x) {
                const uint64_t pz = u / L.ncb;        // prime*D + z
                const uint8_t *src = limbs + pz * (uint64_t)rows * N * 8;
                for (int s = 0; s < S; s++, G++) {
                    const int slot = G % TC_NS;
                    if (G >= (uint32_t)TC_NS &&
                        !mbar_wait_bounded(&C.s_empty[slot], ((G / TC_NS) + 1) & 1, abort)) {
                        stop = true;
                        break;
                    }
                    mbar_expect_tx(&C.s_full[slot], s_bytes);
                    tma_bulk_g2s(smem_tc + S_RING + slot * S_STAGE_MAX, src + (uint64_t)s * s_bytes, s_bytes,
                                 &C.s_full[slot]);
                }
            }
            if (stop) {
                // let the copies already issued land before the CTA can exit
                for (uint32_t k = (G > (uint32_t)TC_NS ? G - TC_NS : 0); k < G; k++)
                    mbar_wait_timed(&C.s_full[k % TC_NS], (k / TC_NS) & 1);
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA
        if (lane == 0) {
            const uint32_t idesc = instr_desc(N);
            uint32_t G = 0, ui = 0;
            bool stop = false;
            for (uint64_t u = blockIdx.x; u < units && !stop; u += gridDim.x, ui++) {
                if (ui > 0 && !mbar_wait_bounded(&C.acc_empty, (ui - 1) & 1, abort)) break;
                tc_fence_after();
                uint32_t inited = 0;
                for (int s = 0; s < S; s++, G++) {
                    const int as = G % TC_NA, ss = G % TC_NS;
                    if (!mbar_wait_bounded(&C.a_full[as], (G / TC_NA) & 1, abort) ||
                        !mbar_wait_bounded(&C.s_full[ss], (G / TC_NS) & 1, abort)) {
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a0 = sbase + A_RING + as * A_STAGE_BYTES;
                    const uint32_t b0 = sbase + S_RING + ss * S_STAGE_MAX;
#pragma unroll
                    for (int ks = 0; ks < TC_KC / 16; ks++) {
#pragma unroll
                        for (int i = 0; i < 4; i++) {
                            const uint64_t ad = smem_desc(a0 + i * A_LIMB_BYTES + ks * 2 * 2048, 2048, 128);
#pragma unroll
                            for (int j = 0; j < 4; j++) {
                                const int d = i + j;
                                const uint64_t bd =
                                    smem_desc(b0 + j * (N * 64) + ks * 2 * (N * 16), (uint32_t)N * 16, 128);
                                mma_f16(tmem + d * N, ad, bd, idesc, (inited >> d) & 1);
                                inited |= 1u << d;
                            }
                        }
                    }
                    mma_commit(&C.a_empty[as]);
                    mma_commit(&C.s_empty[ss]);
                }
                if (!stop) mma_commit(&C.acc_full);
            }
            // all MMAs issued by this thread have completed once `drain` flips
            mma_commit(&C.drain);
            mbar_wait_timed(&C.drain, 0);
        }
    } else if (warp < 6) {
        // --------------------------------------------------- converters
        const int m = threadIdx.x - 64;      // combo within the unit
        const uint32_t sts_off = (m >> 3) * 128 + (m & 7) * 16;
        uint32_t G = 0;
        bool stop = false;
        for (uint64_t u = blockIdx.x; u < units && !stop; u += gridDim.x) {
            const uint32_t p = (u / ((uint64_t)L.ncb * D)) ? QP1 : QP0;
            const uint32_t *src = db + u * L.unit_words32() + m;
            uint32_t xr[TC_KC];
#pragma unroll
            for (int j = 0; j < TC_KC; j++) xr[j] = __ldg(src + j * TC_M);
            for (int s = 0; s < S; s++, G++) {
                uint32_t xn[TC_KC];
                if (s + 1 < S) {
#pragma unroll
                    for (int j = 0; j < TC_KC; j++) xn[j] = __ldg(src + ((s + 1) * TC_KC + j) * TC_M);
                }
                const int as = G % TC_NA;
                if (G >= (uint32_t)TC_NA && !mbar_wait_bounded(&C.a_empty[as], ((G / TC_NA) + 1) & 1, abort)) {
                    stop = true;
                    break;
                }
                const uint32_t a0 = sbase + A_RING + as * A_STAGE_BYTES + sts_off;
#pragma unroll
                for (int kg = 0; kg < TC_KC / 8; kg++) {
                    uint32_t uu[8][4];
#pragma unroll
                    for (int j = 0; j < 8; j++) digits4(xr[kg * 8 + j], p, uu[j]);
#pragma unroll
                    for (int l = 0; l < 4; l++)
                        sts128(a0 + l * A_LIMB_BYTES + kg * 2048, digit_pair(uu[0][l], uu[1][l]),
                               digit_pair(uu[2][l], uu[3][l]), digit_pair(uu[4][l], uu[5][l]),
                               digit_pair(uu[6][l], uu[7][l]));
                }
                // make the generic-proxy stores visible to the tensor cores
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(&C.a_full[as]);
#pragma unroll
                for (int j = 0; j < TC_KC; j++) xr[j] = xn[j];
            }
        }
    } else {
        // ----------------------------------------------------- epilogue
        const int q4 = warp & 3;             // TMEM lane quarter of this warp
        const int m = q4 * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(q4 * 32) << 16);
        uint32_t ui = 0;
        for (uint64_t u = blockIdx.x; u < units; u += gridDim.x, ui++) {
            // tcgen05.ld is warp-collective: the warp leaves together
            const bool ok = mbar_wait_bounded(&C.acc_full, ui & 1, abort);
            if (!__all_sync(0xffffffffu, ok)) break;
            tc_fence_after();
            const int cbi = (int)(u % L.ncb);
            const int z = (int)((u / L.ncb) % D);
            const int prime = (int)(u / ((uint64_t)L.ncb * D));
            const uint32_t p = prime ? QP1 : QP0;
            const uint64_t mu = ~0ull / p;
            const uint64_t off = ((1ull << 54) / p + 1) * p;
            uint32_t w[7];
            w[0] = 1;
#pragma unroll
            for (int d = 1; d < 7; d++) w[d] = (uint32_t)(((uint64_t)w[d - 1] << 7) % p);
            const uint64_t mg = (uint64_t)cbi * TC_M + m;
            for (int n0 = 0; n0 < N; n0 += 16) {
                uint32_t v[7][16];
#pragma unroll
                for (int d = 0; d < 7; d++) tmem_ld16(lane_addr + d * N + n0, v[d]);
                tmem_wait_ld();
#pragma unroll
                for (int c = 0; c < 16; c++) {
                    const int n = n0 + c, b = n >> 1, k = n & 1;
                    int64_t s = 0;
#pragma unroll
                    for (int d = 0; d < 7; d++) s += (int64_t)__float2int_rn(__uint_as_float(v[d][c])) * w[d];
                    if (b < nq)
                        C.acc[b][((mg * 2 + k) * 2 + prime) * D + z] =
                            mod_u64_barrett((uint64_t)(s + (int64_t)off), p, mu);
                }
            }
            tc_fence_before();
            mbar_arrive(&C.acc_empty);
        }
    }

    __syncthreads();
    if (C.abort && threadIdx.x == 0) atomicExch(err, 1);
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                     : "memory");
    }
}

bool db_mul_tc_supported(const DbLayout &L) {
    return L.cb == TC_M && L.rows % TC_KC == 0 && L.rows >= TC_KC && L.rows <= 512;
}

uint64_t tc_limb_bytes(const DbLayout &L) { return 2ull * D * L.rows * TC_MAX_N * 8; }

cudaError_t launch_db_mul_tc(const uint32_t *db, const DbLayout &L, const QDesc *qd, int nq, uint8_t *limbs,
                             int *err, cudaStream_t st) {
    if (!db_mul_tc_supported(L) || nq < 1 || nq > TC_MAX_Q) return cudaErrorInvalidValue;
    const int N = ((2 * nq + 15) / 16) * 16;
    const uint64_t total = (uint64_t)N * D * (L.rows / 8);
    const int sms = sm_count();
    uint64_t blocks = (total + 255) / 256;
    if (blocks > (uint64_t)sms * 16) blocks = (uint64_t)sms * 16;
    k_tc_limbs<<<(unsigned)blocks, 256, 0, st>>>(qd, nq, L.rows, N, limbs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_db_mul_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    if (e != cudaSuccess) return e;
    const uint64_t units = L.units();
    const int grid = (int)(units < (uint64_t)sms ? units : (uint64_t)sms);
    k_db_mul_tc<<<grid, TC_THREADS, TC_SMEM, st>>>(db, L, qd, nq, N, limbs, err);
    return cudaGetLastError();
}

}  // namespace sp
