// Tensor-core first-dimension multiply for batches of queries (R11, batched).
//
// For one slot z and one prime the multiply of B queries is a plain matrix
// product:  out[m][n] = sum_row DB[m][row] * SEL[row][n]  (mod p), with m one
// of the 128 combos of an image unit, n = 2*query + ciphertext row, and
// row < 2^nu1.  Residues are < 2^28, so the product is made exact on the
// fp16 tensor cores by splitting both operands into four 7-bit digits: the
// database residue x (as stored, in [0, 2^28)) into unsigned digits
//   x = u0 + u1*2^7 + u2*2^14 + u3*2^21,   u_i in [0, 127],
// the selector s (centred to (-p/2, p/2]) into signed digits
//   s = a0 + a1*2^7 + a2*2^14 + a3*2^21,   a0..a2 in [-64, 63], a3 in [-64, 64]
// (all exactly representable in fp16), and accumulating the 16 digit
// products by weight class d = i + j in seven fp32 accumulators C_d.  Every
// product is at most 127 * 64 in magnitude and a class holds at most 4 digit
// pairs, so |C_d| <= 4 * 512 * 127 * 64 < 2^24 for up to 512 rows: every
// partial sum is an integer that fp32 holds exactly.  The epilogue returns
// sum_d C_d * (2^(7d) mod p) reduced mod p, bit-identical to the
// integer-pipe multiplies.
//
// Layout of the work (tcgen05, cta_group::1, kind::f16, M = 128, K = 16 per
// instruction; N = 2B rounded up to 16, at most 64, selector columns):
//  * A = database digits, 128 combos x 16 rows per K-step, in tensor memory:
//    lane = combo, 8 columns of fp16 pairs (rows 2c, 2c+1) per digit.  The
//    converter warps write them with tcgen05.st from the packed image rows
//    (the digits are the residue's bit fields) that
//    the producer stages in shared memory; two K-step buffers of 32 columns;
//  * B = the four selector digits side by side, 4N columns (digit j in
//    columns jN .. jN+N-1), prepared once per batch by k_tc_limbs in the
//    K-major canonical shared-memory form (no swizzle: 8x8 core matrices of
//    128 B, SBO = 128 B between 8-column groups, LBO = 4N*16 B between 8-row
//    groups) and fetched per stage with one 1-D bulk TMA copy;
//  * D = seven accumulators C_0..C_6 of N fp32 columns each, adjacent (7*64 =
//    448 columns); with the A buffers (64 columns) that fills the 512
//    columns of tensor memory.
// One instruction per A digit i and K-step: A_i x [B_0 B_1 B_2 B_3] (N' = 4N,
// 256 at N = 64) into columns iN .. iN+4N-1, i.e. A_i B_j lands in C_(i+j):
// the weight classes are summed by the tensor core itself.  The columns of
// consecutive instructions overlap, so every instruction accumulates and the
// accumulators are zeroed as they are read.
// Tensor memory holds one accumulator set, so the MMAs of the next unit wait
// until the current one is drained; all sixteen converter and epilogue warps
// drain it (each lane quarter by four warps, each a quarter of the columns).
// Warp roles of the persistent CTA (one per SM; the shared-memory footprint
// keeps it alone on its SM, so its 512-column TMEM allocation never waits):
//   warp 0       TMA producer of the selector stages and of the image rows
//   warp 1       TMEM allocation, MMA issue (one thread), TMEM release
//   warps 2..9   converters: image rows -> digit pairs -> tensor memory
//                (warps 2..5 even K-steps, 6..9 odd; lane = combo)
//                then their share of the drain
//   warps 10..17 drain: TMEM -> registers -> mod p -> chunk output
// Queries beyond 32 run as further passes over the image.
// Every barrier wait is bounded in time; a wait that runs out sets an error
// flag, the other roles stop at their next wait, in-flight copies and MMAs
// are drained (bounded), the TMEM is released and the kernel returns.
#include <cuda_fp16.h>

#include "async.cuh"
#include "kernels.cuh"

namespace sp {
namespace {

constexpr int TC_M = 128;
constexpr int TC_KC = 32;                     // rows per stage (two K-steps)
constexpr int TC_NS = 6;                      // selector (B) stages
constexpr int TC_ND = 6;                      // image stages (packed rows)
constexpr int TC_MAX_N = 2 * TC_MAX_Q;        // 64
constexpr uint32_t S_STAGE_MAX = 4 * TC_KC * TC_MAX_N * 2;   // 16 KiB
constexpr uint32_t D_STAGE_BYTES = TC_KC * TC_M * 4;         // 16 KiB slot
constexpr int TC_RW = TC_M / 8 * 7;                          // words per packed row (112)
constexpr uint32_t D_COPY_BYTES = TC_KC * TC_RW * 4;         // 14 KiB of packed rows per stage
constexpr uint32_t S_RING = 0;
constexpr uint32_t D_RING = S_RING + TC_NS * S_STAGE_MAX;    // 96 KiB
constexpr uint32_t CTRL = D_RING + TC_ND * D_STAGE_BYTES;    // 192 KiB
constexpr uint32_t TC_SMEM = CTRL + 1024;
constexpr int TC_THREADS = 576;
constexpr int TC_CONV = 128;                  // converter threads per K-step parity
constexpr int TC_DRAIN = 512;                 // converter + epilogue threads
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t TMEM_A = 448;              // first column of the A buffers
constexpr int32_t DIGIT_BIAS = 64 * (1 + 128 + 128 * 128);   // 1056832

struct Ctrl {
    uint64_t s_full[TC_NS], s_empty[TC_NS];
    uint64_t a_full[2], a_empty[2];
    uint64_t d_full[TC_ND], d_empty[TC_ND];
    uint64_t acc_full, acc_empty, drain;
    uint32_t tmem_base;
    int abort;
    // drain constants per prime, computed once: weights 2^(7d) * 2^32 mod p
    // and a multiple of p above the largest |weighted sum|
    int32_t wts[2][7];
    int64_t off[2];
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


__device__ __forceinline__ uint32_t hsub1024(uint32_t w) {
    __half2 h = *reinterpret_cast<__half2 *>(&w);
    h = __hsub2(h, __halves2half2(__ushort_as_half(0x6400), __ushort_as_half(0x6400)));
    return *reinterpret_cast<uint32_t *>(&h);
}

// The four fp16 digit pairs (digit l of xa, digit l of xb), l = 0..3, of two
// residues < 2^28 (unsigned 7-bit digits), with byte permutes instead of
// per-digit shifts.  0x6400 | u is the fp16 value 1024 + u; subtracting 1024
// is exact.
__device__ __forceinline__ void digit_pairs(uint32_t xa, uint32_t xb, uint32_t (&w)[4]) {
    const uint32_t t0 = __byte_perm(xa, xb, 0x5410);   // bits 0-15 of each
    const uint32_t t1 = __byte_perm(xa, xb, 0x6521);   // bits 8-23
    const uint32_t t2 = __byte_perm(xa, xb, 0x7632);   // bits 16-31
    w[0] = hsub1024((t0 & 0x007F007Fu) | 0x64006400u);
    w[1] = hsub1024(((t0 >> 7) & 0x007F007Fu) | 0x64006400u);
    w[2] = hsub1024(((t1 >> 6) & 0x007F007Fu) | 0x64006400u);
    w[3] = hsub1024(((t2 >> 5) & 0x007F007Fu) | 0x64006400u);
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

// D (tmem) (+)= A (tmem) * B (shared memory descriptor)
__device__ __forceinline__ void mma_f16_ts(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc,
                                           uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(tmem_d),
        "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&v)[8]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
                 "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
}

__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

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

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&v)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                 : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

}  // namespace

// Exact fp32 integer -> int32 for |x| <= 2^22 with one add: the sum with
// 1.5 * 2^23 holds x in its low mantissa bits (also at the +-2^22 ends).
__device__ __forceinline__ int32_t f2i_small(uint32_t bits) {
    return __float_as_int(__fadd_rn(__uint_as_float(bits), 12582912.0f)) - 0x4B400000;
}

// Drain one lane quarter of the accumulators for columns c0, c0 + 32, ...
// (chunks of 8): read C_0..C_6, zero them, and write
//   sum_d C_d 2^(7d) mod p
// into the chunk output [prime][z - z0][n][combo].  |C_d| <= (pairs of
// class d) * 512 * 127 * 64, so classes 0 and 6 (one digit pair, below 2^22)
// convert with f2i_small and classes 1 to 5 with cvt.
__device__ __forceinline__ void drain_quarter(uint32_t lane_addr, int N, int c0, const DbLayout &L, int z0,
                                              int zc, uint64_t u, int m, uint32_t *out, const int32_t (&wts)[2][7],
                                              const int64_t (&offs)[2]) {
    // unit -> (prime, slot, block) in 32-bit arithmetic (units < 2^31)
    const uint32_t uu = (uint32_t)u, ncb = (uint32_t)L.ncb;
    const int cbi = (int)(uu % ncb);
    const int zl = (int)((uu / ncb) % D) - z0;
    const int prime = (int)(uu / (ncb * D));
    const uint32_t p = prime ? QP1 : QP0;
    const uint32_t npinv = 0u - (prime ? P1_PINV : P0_PINV);
    // weights 2^(7d) * 2^32 mod p: one Montgomery reduction of the weighted
    // sum returns sum_d C_d 2^(7d) mod p
    int32_t w[7];
#pragma unroll
    for (int d = 0; d < 7; d++) w[d] = wts[prime][d];
    const int64_t off = offs[prime];
    const uint32_t mg = (uint32_t)cbi * TC_M + m;
    uint32_t *o = out + ((uint64_t)prime * zc + zl) * N * L.combos + mg;
    const uint32_t zero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int n0 = c0; n0 < N; n0 += 32) {
        uint32_t v8[7][8];
#pragma unroll
        for (int d = 0; d < 7; d++) tmem_ld8(lane_addr + d * N + n0, v8[d]);
        tmem_wait_ld();
#pragma unroll
        for (int d = 0; d < 7; d++) tmem_st8(lane_addr + d * N + n0, zero8);
#pragma unroll
        for (int c = 0; c < 8; c++) {
            int64_t sum = off;
            sum += (int64_t)f2i_small(v8[0][c]) * w[0];
            sum += (int64_t)__float2int_rn(__uint_as_float(v8[1][c])) * w[1];
            sum += (int64_t)__float2int_rn(__uint_as_float(v8[2][c])) * w[2];
            sum += (int64_t)__float2int_rn(__uint_as_float(v8[3][c])) * w[3];
            sum += (int64_t)__float2int_rn(__uint_as_float(v8[4][c])) * w[4];
            sum += (int64_t)__float2int_rn(__uint_as_float(v8[5][c])) * w[5];
            sum += (int64_t)f2i_small(v8[6][c]) * w[6];
            const uint64_t x = (uint64_t)sum;
            const uint64_t t = x + (uint64_t)((uint32_t)x * npinv) * p;
            uint32_t r = (uint32_t)(t >> 32);
            r = r >= p ? r - p : r;
            o[(uint64_t)(n0 + c) * L.combos] = r;     // a warp writes 128 contiguous bytes
        }
    }
    tmem_wait_st();
}

// ------------------------------------------------------ selector digits
// Thread (n, z, row group of 8): n = 2*query + ciphertext row.  Writes, for
// both primes, the four digits of 8 consecutive rows as 16-byte rows of the
// canonical K-major B tiles (column = digit*N + n):
//   limbs[prime][z][stage][8-row group][digit][N/8][8 n][8 rows]  (fp16)
__global__ void __launch_bounds__(256) k_tc_limbs(const QDesc *__restrict__ qd, int nq, int rows, int N,
                                                  uint8_t *__restrict__ limbs) {
    // index space N * D * rows / 8 < 2^32: 32-bit index arithmetic
    const uint32_t total = (uint32_t)N * D * (uint32_t)(rows / 8);
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int n = (int)(idx % (uint32_t)N);
        const uint32_t rest = idx / (uint32_t)N;
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
                const uint64_t off = ((uint64_t)(s * 4 + kg) * 4 + l) * (N / 8) * 128 + (n / 8) * 128 + (n % 8) * 16;
                *reinterpret_cast<uint4 *>(base + off) = w;
            }
        }
    }
}

// ------------------------------------------------------------ multiply
// Units of one launch: both primes, slots [z0, z0 + zc), every combo block;
// chunk-local index v -> image unit.
__device__ __forceinline__ uint64_t chunk_unit(const DbLayout &L, int z0, int zc, uint64_t v) {
    const uint32_t per_prime = (uint32_t)zc * (uint32_t)L.ncb, vv = (uint32_t)v;
    const uint32_t prime = vv / per_prime, r = vv % per_prime;
    return ((uint64_t)prime * D + z0 + r / (uint32_t)L.ncb) * L.ncb + r % (uint32_t)L.ncb;
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_db_mul_tc(const uint32_t *__restrict__ db, DbLayout L, int nq,
                                                             int N, int z0, int zc,
                                                             const uint8_t *__restrict__ limbs,
                                                             uint32_t *__restrict__ out, int *err) {
    extern __shared__ __align__(1024) uint8_t smem_tc[];
    Ctrl &C = *reinterpret_cast<Ctrl *>(smem_tc + CTRL);
    volatile int *abort = &C.abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t sbase = smem_addr(smem_tc);
    const int rows = L.rows;
    const int S = rows / TC_KC;                        // stages per unit
    const uint32_t s_bytes = 4u * TC_KC * N * 2;       // selector stage bytes
    const uint64_t units = 2ull * zc * L.ncb;      // units of this launch

    if (threadIdx.x == 0) {
        for (int i = 0; i < TC_NS; i++) {
            mbar_init(&C.s_full[i], 1);
            mbar_init(&C.s_empty[i], 1);
        }
        for (int i = 0; i < 2; i++) {
            mbar_init(&C.a_full[i], TC_CONV);
            mbar_init(&C.a_empty[i], 1);
        }
        for (int i = 0; i < TC_ND; i++) {
            mbar_init(&C.d_full[i], 1);
            mbar_init(&C.d_empty[i], 2 * TC_CONV);
        }
        mbar_init(&C.acc_full, 1);
        mbar_init(&C.acc_empty, TC_DRAIN);
        mbar_init(&C.drain, 1);
        C.abort = 0;
        for (int pr = 0; pr < 2; pr++) {
            const uint32_t p = pr ? QP1 : QP0;
            uint64_t wd = (1ull << 32) % p;
            for (int d = 0; d < 7; d++) {
                C.wts[pr][d] = (int32_t)wd;
                wd = (wd << 7) % p;
            }
            // a multiple of p above the largest |sum| (< 7 * 2^24 * 2^28)
            C.off[pr] = (int64_t)(((1ull << 55) / p + 1) * p);
        }
        fence_mbar_init();
    }
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
        // per stage: the selector digit tile (for the MMA) and the image
        // rows (for the converters), each into its own ring
        if (lane == 0) {
            uint32_t G = 0;
            bool stop = false;
            for (uint64_t v = blockIdx.x; v < units && !stop; v += gridDim.x) {
                const uint64_t u = chunk_unit(L, z0, zc, v);
                const uint64_t pz = u / L.ncb;        // prime*D + z
                const uint8_t *sel_src = limbs + pz * (uint64_t)rows * N * 8;
                const uint32_t *db_src = db + u * L.unit_words32();
                for (int s = 0; s < S; s++, G++) {
                    const int ss = G % TC_NS, ds = G % TC_ND;
                    if (G >= (uint32_t)TC_NS &&
                        !mbar_wait_bounded(&C.s_empty[ss], ((G / TC_NS) + 1) & 1, abort)) {
                        stop = true;
                        break;
                    }
                    mbar_expect_tx(&C.s_full[ss], s_bytes);
                    tma_bulk_g2s(smem_tc + S_RING + ss * S_STAGE_MAX, sel_src + (uint64_t)s * s_bytes, s_bytes,
                                 &C.s_full[ss]);
                    if (G >= (uint32_t)TC_ND &&
                        !mbar_wait_bounded(&C.d_empty[ds], ((G / TC_ND) + 1) & 1, abort)) {
                        // the selector copy of this stage is in flight: count it
                        G++;
                        stop = true;
                        break;
                    }
                    mbar_expect_tx(&C.d_full[ds], D_COPY_BYTES);
                    tma_bulk_g2s(smem_tc + D_RING + ds * D_STAGE_BYTES, db_src + (uint64_t)s * TC_KC * TC_RW,
                                 D_COPY_BYTES, &C.d_full[ds]);
                }
            }
            if (stop) {
                // let the copies already issued land before the CTA can exit
                for (uint32_t k = (G > (uint32_t)TC_NS ? G - TC_NS : 0); k < G; k++) {
                    mbar_wait_timed(&C.s_full[k % TC_NS], (k / TC_NS) & 1);
                    mbar_wait_timed(&C.d_full[k % TC_ND], (k / TC_ND) & 1);
                }
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA
        if (lane == 0) {
            const uint32_t idesc = instr_desc(4 * N);
            uint32_t G = 0, ui = 0;
            bool stop = false;
            for (uint64_t v = blockIdx.x; v < units && !stop; v += gridDim.x, ui++) {
                // phase 0 of acc_empty: accumulators cleared at start;
                // phase ui: unit ui - 1 drained
                const uint32_t dacc = tmem;
                if (!mbar_wait_bounded(&C.acc_empty, ui & 1, abort)) break;
                tc_fence_after();
                for (int s = 0; s < S; s++, G++) {
                    const int ss = G % TC_NS;
                    if (!mbar_wait_bounded(&C.s_full[ss], (G / TC_NS) & 1, abort)) {
                        stop = true;
                        break;
                    }
                    const uint32_t b0 = sbase + S_RING + ss * S_STAGE_MAX;
#pragma unroll
                    for (int ks = 0; ks < TC_KC / 16; ks++) {
                        if (!mbar_wait_bounded(&C.a_full[ks], G & 1, abort)) {
                            stop = true;
                            break;
                        }
                        tc_fence_after();
                        const uint64_t bd = smem_desc(b0 + ks * 2 * (N * 64), (uint32_t)N * 64, 128);
#pragma unroll
                        for (int i = 0; i < 4; i++)
                            mma_f16_ts(dacc + i * N, tmem + TMEM_A + 32 * ks + 8 * i, bd, idesc, 1);
                        mma_commit(&C.a_empty[ks]);
                    }
                    if (stop) break;
                    mma_commit(&C.s_empty[ss]);
                }
                if (!stop) mma_commit(&C.acc_full);
            }
            // all MMAs issued by this thread have completed once `drain` flips
            mma_commit(&C.drain);
            mbar_wait_timed(&C.drain, 0);
        }
    } else if (warp < 10) {
        // --------------------------------------------------- converters
        // warp quarter q4 owns TMEM lanes (= combos) 32*q4 .. 32*q4+31;
        // h = 0 converts rows 0..15 of each stage (K-step 0), h = 1 rows 16..31
        const int q4 = warp & 3, h = (warp - 2) >> 2;
        const int m = q4 * 32 + lane;
        const uint32_t lds_off = h * 16 * TC_RW * 4;   // this parity's first packed row
        // this combo's word and bit in a packed row; the pair of words read for
        // the last combo of a row reaches into the next row or the unused tail
        // of the stage slot (the stray bits are masked off)
        const int cw = (28 * m) >> 5, csh = (28 * m) & 31;
        const uint32_t ta0 = tmem + ((uint32_t)(q4 * 32) << 16) + TMEM_A + 32 * h;
        const uint32_t lane_addr = tmem + ((uint32_t)(q4 * 32) << 16);
        const int c0 = h * 8;                 // drain chunks h, h + 4, ...
        {
            // tensor memory is undefined after allocation: clear this warp's
            // accumulator chunks before the first unit
            const uint32_t zero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (int n0 = c0; n0 < N; n0 += 32)
#pragma unroll
                for (int d = 0; d < 7; d++) tmem_st8(lane_addr + d * N + n0, zero8);
            tmem_wait_st();
            tc_fence_before();
            mbar_arrive(&C.acc_empty);
        }
        // The converters drain their share of unit ui - 1 after converting
        // the first stage of unit ui: the digit buffers are free as soon as
        // the accumulators are full, so the next unit's first MMAs do not
        // wait for the conversion after the drain.
        uint64_t prev_u = 0;
        auto drain_unit = [&](uint32_t unit_idx, uint64_t uu) -> bool {
            const bool ok = mbar_wait_bounded(&C.acc_full, unit_idx & 1, abort);
            if (!__all_sync(0xffffffffu, ok)) return false;
            tc_fence_after();
            drain_quarter(lane_addr, N, c0, L, z0, zc, uu, m, out, C.wts, C.off);
            tc_fence_before();
            mbar_arrive(&C.acc_empty);
            return true;
        };
        uint32_t G = 0, ui = 0;
        bool stop = false;
        for (uint64_t v = blockIdx.x; v < units && !stop; v += gridDim.x, ui++) {
            const uint64_t u = chunk_unit(L, z0, zc, v);
            for (int s = 0; s < S; s++, G++) {
                const int ds = G % TC_ND;
                bool ok = mbar_wait_bounded(&C.d_full[ds], (G / TC_ND) & 1, abort);
                if (!__all_sync(0xffffffffu, ok)) {
                    stop = true;
                    break;
                }
                const uint32_t *xs = reinterpret_cast<const uint32_t *>(smem_tc + D_RING + ds * D_STAGE_BYTES + lds_off);
                uint32_t xr[16];
#pragma unroll
                for (int j = 0; j < 16; j++)
                    xr[j] = __funnelshift_r(xs[j * TC_RW + cw], xs[j * TC_RW + cw + 1], csh) & RES_MASK;
                mbar_arrive(&C.d_empty[ds]);
                uint32_t w[4][8];     // [digit][row pair]
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    uint32_t d4[4];
                    digit_pairs(xr[2 * j], xr[2 * j + 1], d4);
#pragma unroll
                    for (int l = 0; l < 4; l++) w[l][j] = d4[l];
                }
                // buffer h held this parity's K-step of the previous stage
                ok = G == 0 || mbar_wait_bounded(&C.a_empty[h], (G - 1) & 1, abort);
                if (!__all_sync(0xffffffffu, ok)) {
                    stop = true;
                    break;
                }
                tc_fence_after();
#pragma unroll
                for (int l = 0; l < 4; l++) tmem_st8(ta0 + 8 * l, w[l]);
                tmem_wait_st();
                tc_fence_before();
                mbar_arrive(&C.a_full[h]);
                if (s == 0 && ui > 0 && !drain_unit(ui - 1, prev_u)) {
                    stop = true;
                    break;
                }
            }
            prev_u = u;
        }
        if (!stop && ui > 0) drain_unit(ui - 1, prev_u);
    } else {
        // -------------------------------------------------------- drain
        const int q4 = warp & 3;             // TMEM lane quarter of this warp
        const int c0 = (2 + ((warp - 10) >> 2)) * 8;   // drain chunks 2, 6, ... or 3, 7, ...
        const int m = q4 * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(q4 * 32) << 16);
        {
            const uint32_t zero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (int n0 = c0; n0 < N; n0 += 32)
#pragma unroll
                for (int d = 0; d < 7; d++) tmem_st8(lane_addr + d * N + n0, zero8);
            tmem_wait_st();
            tc_fence_before();
            mbar_arrive(&C.acc_empty);
        }
        uint32_t ui = 0;
        for (uint64_t v = blockIdx.x; v < units; v += gridDim.x, ui++) {
            // tcgen05.ld is warp-collective: the warp leaves together
            const bool ok = mbar_wait_bounded(&C.acc_full, ui & 1, abort);
            if (!__all_sync(0xffffffffu, ok)) break;
            tc_fence_after();
            drain_quarter(lane_addr, N, c0, L, z0, zc, chunk_unit(L, z0, zc, v), m, out, C.wts, C.off);
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

// ------------------------------------------------------------ transpose
// Chunk output [prime][z - z0][n][combo] -> each query's accumulator planes
// [combo][ct row][prime][z].  Tile: 8 n x 32 slots x 32 combos through
// shared memory; 128-byte reads and writes.
__global__ void __launch_bounds__(256) k_tc_transpose(const uint32_t *__restrict__ in, const QDesc *__restrict__ qd,
                                                      int nq, int N, int combos, int z0, int zc) {
    __shared__ uint32_t tile[8][32][33];
    const int mb = blockIdx.x * 32;
    const int zb = blockIdx.y * 32;
    const int prime = blockIdx.z / (N / 8), nb = (blockIdx.z % (N / 8)) * 8;
    for (int i = threadIdx.x; i < 8 * 32 * 32; i += 256) {
        const int m = i & 31, z = (i >> 5) & 31, n = i >> 10;
        tile[n][z][m] = in[(((uint64_t)prime * zc + zb + z) * N + nb + n) * combos + mb + m];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 8 * 32 * 32; i += 256) {
        const int z = i & 31, m = (i >> 5) & 31, n = i >> 10;
        const int b = (nb + n) >> 1, k = (nb + n) & 1;
        if (b < nq) qd[b].acc[(((uint64_t)(mb + m) * 2 + k) * 2 + prime) * D + z0 + zb + z] = tile[n][z][m];
    }
}

bool db_mul_tc_supported(const DbLayout &L) {
    return L.cb == TC_M && L.rows % TC_KC == 0 && L.rows >= TC_KC && L.rows <= 512;
}

uint64_t tc_limb_bytes(const DbLayout &L) { return 2ull * D * L.rows * TC_MAX_N * 8; }

// Slots per launch: the chunk output (2 * zc * combos * 64 * 4 bytes) stays
// within 512 MiB.
static int tc_chunk(const DbLayout &L) {
    int zc = D;
    while (zc > 32 && 2ull * zc * L.combos * TC_MAX_N * 4 > (512ull << 20)) zc >>= 1;
    return zc;
}

uint64_t tc_out_bytes(const DbLayout &L) { return 2ull * tc_chunk(L) * L.combos * TC_MAX_N * 4; }

int tc_launches(const DbLayout &L) { return 1 + 2 * (D / tc_chunk(L)); }

cudaError_t launch_db_mul_tc(const uint32_t *db, const DbLayout &L, const QDesc *qd, int nq, uint8_t *limbs,
                             uint32_t *out, int *err, cudaStream_t st) {
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
    const int zc = tc_chunk(L);
    for (int z0 = 0; z0 < D; z0 += zc) {
        const uint64_t units = 2ull * zc * L.ncb;
        const int grid = (int)(units < (uint64_t)sms ? units : (uint64_t)sms);
        k_db_mul_tc<<<grid, TC_THREADS, TC_SMEM, st>>>(db, L, nq, N, z0, zc, limbs, out, err);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        dim3 tg(L.combos / 32, zc / 32, 2 * (N / 8));
        k_tc_transpose<<<tg, 256, 0, st>>>(out, qd, nq, N, L.combos, z0, zc);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace sp
