// Database image (R5) and first-dimension multiply (R11).
//
// The multiply is HBM-bound for one query (every database word is read once
// and used for 4 multiply-adds).  Each CTA owns one (z tile, column group)
// stream of the tiled image, a contiguous region of rows * T*cg*64 words, and
// pulls it through shared memory with 1-D bulk TMA copies
// (cp.async.bulk ... mbarrier::complete_tx) into a ring of stages, together
// with the 64-slot selector slice of each row.  Products of canonical
// residues (< 2^56) accumulate in 64-bit registers and are reduced every 128
// rows, which keeps the sum below 2^64.
#include "kernels.cuh"

namespace sp {

DbLayout make_db_layout(int T, int nu1, int nu2) {
    DbLayout L{};
    L.T = T;
    L.nu1 = nu1;
    L.nu2 = nu2;
    L.rows = 1 << nu1;
    L.cols = 1 << nu2;
    L.zt = 64;
    L.nzt = D / L.zt;
    // T*cg words per (row, z) of a tile: 16 when possible (4 accumulator sets
    // per thread), at least one column.
    int cg = 16 / T;
    if (cg < 1) cg = 1;
    if (cg > L.cols) cg = L.cols;
    L.cg = cg;
    L.ncg = L.cols / cg;
    L.words = (uint64_t)L.rows * L.cols * T * D;
    return L;
}

// ----------------------------------------------------------------- encode
// One CTA per (record, t) polynomial: group g transforms residues mod q_g of
// the recentred plaintext and writes its 32-bit half of the packed words.
constexpr int ENC_SMEM_WORDS = 4 * D + 2 * 2 * D;

__global__ void __launch_bounds__(256) k_db_encode(const uint8_t *__restrict__ rec, uint64_t rec_begin,
                                                   uint64_t rec_count, int pt_bits, DbLayout L,
                                                   uint64_t *__restrict__ db,
                                                   const TwiddleSet *__restrict__ tws) {
    extern __shared__ __align__(16) uint32_t smem[];
    load_twiddles(smem, tws);
    __syncthreads();
    const int g = threadIdx.x >> 7, t = threadIdx.x & (GROUP - 1);
    const Prime c = prime_of(g);
    uint32_t *buf = smem + 4 * D + g * 2 * D;
    const uint32_t pm = 1u << pt_bits;
    const uint64_t polys = rec_count * L.T;
    uint32_t *db32 = reinterpret_cast<uint32_t *>(db);
    for (uint64_t i = blockIdx.x; i < polys; i += gridDim.x) {
        const uint64_t r_local = i / L.T;
        const int tt = (int)(i % L.T);
        const uint64_t r = rec_begin + r_local;
        const int row = (int)(r / L.cols), col = (int)(r % L.cols);
        const uint8_t *src = rec + i * D;
        uint32_t v[VPT];
#pragma unroll
        for (int j = 0; j < VPT; j++) {
            uint32_t x = src[t + GROUP * j];
            v[j] = (x > pm / 2) ? c.p - (pm - x) : x;   // recentre to (-p/2, p/2]
        }
        ntt_fwd(v, smem + g * D, buf, c, t, 1 + g);
#pragma unroll
        for (int j = 0; j < VPT; j++) {
            const int z = VPT * t + j;
            db32[2 * L.offset(tt, row, col, z) + g] = canon4(v[j], c.p);
        }
    }
}

cudaError_t launch_db_encode(const uint8_t *records, uint64_t rec_begin, uint64_t rec_count,
                             int pt_bits, const DbLayout &L, uint64_t *db, const TwiddleSet *tw,
                             cudaStream_t st) {
    const int smem = ENC_SMEM_WORDS * 4;
    cudaError_t e = cudaFuncSetAttribute(k_db_encode, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t polys = rec_count * L.T;
    int grid = (int)(polys < (uint64_t)sms * 3 ? polys : (uint64_t)sms * 3);
    if (grid < 1) grid = 1;
    k_db_encode<<<grid, 256, smem, st>>>(records, rec_begin, rec_count, pt_bits, L, db, tw);
    return cudaGetLastError();
}

__global__ void k_db_import(const uint32_t *__restrict__ planes, DbLayout L, uint64_t *__restrict__ db) {
    const uint64_t total = (uint64_t)L.T * L.cols * L.rows * D;
    for (uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        const int z = (int)(idx % D);
        uint64_t r = idx / D;
        const int row = (int)(r % L.rows); r /= L.rows;
        const int col = (int)(r % L.cols); r /= L.cols;
        const int t = (int)r;
        const uint32_t *src = planes + (((uint64_t)t * L.cols + col) * L.rows + row) * 2 * D;
        db[L.offset(t, row, col, z)] = (uint64_t)src[z] | ((uint64_t)src[D + z] << 32);
    }
}

cudaError_t launch_db_import(const uint32_t *planes, const DbLayout &L, uint64_t *db, cudaStream_t st) {
    k_db_import<<<4096, 256, 0, st>>>(planes, L, db);
    return cudaGetLastError();
}

// --------------------------------------------------------------- multiply
namespace {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Bounded wait on phase `parity` of an mbarrier; false after ~2^24 polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = smem_addr(bar);
    for (int i = 0; i < (1 << 24); i++) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ uint32_t mod_u64_barrett(uint64_t x, uint32_t p, uint64_t mu) {
    // mu = floor(2^64 / p); quotient estimate is at most 2 below the truth
    uint64_t q = __umul64hi(x, mu);
    uint64_t r = x - q * p;
    r = r >= p ? r - p : r;
    r = r >= p ? r - p : r;
    return (uint32_t)r;
}

constexpr int MUL_THREADS = 256;
constexpr int MUL_ZT = 64;
constexpr int MUL_R = 2;         // rows per stage
constexpr int MUL_STAGES = 4;
constexpr int MUL_REDUCE = 128;  // rows between reductions

}  // namespace

// TPT: (t, c) pairs per thread; the tile holds T*cg = 4*TPT pairs.
template <int TPT>
__global__ void __launch_bounds__(MUL_THREADS) k_db_mul(const uint64_t *__restrict__ db, DbLayout L,
                                                        const QDesc *__restrict__ qd, int *err) {
    constexpr int TCG = 4 * TPT;
    constexpr uint32_t DB_CHUNK = TCG * MUL_ZT * 8;     // bytes per row
    constexpr uint32_t SEL_CHUNK = MUL_ZT * 16;
    constexpr uint32_t STAGE = MUL_R * (DB_CHUNK + SEL_CHUNK);
    extern __shared__ __align__(128) uint8_t smem_mul[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem_mul);
    uint8_t *stages = smem_mul + 128;

    const uint32_t *__restrict__ sel = qd[blockIdx.y].sel;
    uint32_t *__restrict__ out = qd[blockIdx.y].acc;
    const int zti = blockIdx.x % L.nzt, grp = blockIdx.x / L.nzt;
    const int rows = L.rows;
    const uint64_t *src_db = db + (uint64_t)(zti * L.ncg + grp) * rows * TCG * MUL_ZT;
    const uint32_t *src_sel = sel + (uint64_t)zti * MUL_ZT * 4;
    const int n_iter = rows / MUL_R;

    if (threadIdx.x == 0) {
        for (int s = 0; s < MUL_STAGES; s++) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();

    auto issue = [&](int it, int s) {
        uint8_t *st = stages + s * STAGE;
        mbar_expect_tx(&bars[s], STAGE);
        tma_bulk_g2s(st, src_db + (uint64_t)it * MUL_R * TCG * MUL_ZT, MUL_R * DB_CHUNK, &bars[s]);
        for (int r = 0; r < MUL_R; r++)
            tma_bulk_g2s(st + MUL_R * DB_CHUNK + r * SEL_CHUNK,
                         src_sel + (uint64_t)(it * MUL_R + r) * D * 4, SEL_CHUNK, &bars[s]);
    };
    if (threadIdx.x == 0)
        for (int s = 0; s < MUL_STAGES && s < n_iter; s++) issue(s, s);

    const int zi = threadIdx.x % MUL_ZT, tg = threadIdx.x / MUL_ZT;
    uint64_t acc[TPT][4];
#pragma unroll
    for (int u = 0; u < TPT; u++)
#pragma unroll
        for (int k = 0; k < 4; k++) acc[u][k] = 0;
    const uint64_t mu0 = ~0ull / QP0, mu1 = ~0ull / QP1;

    bool ok = true;
    int it = 0;
    for (; it < n_iter; it++) {
        const int s = it % MUL_STAGES;
        // A thread whose wait runs out still computes (on stale data) so that
        // the whole CTA reaches the barrier below and leaves together.
        const bool arrived = mbar_wait(&bars[s], (uint32_t)((it / MUL_STAGES) & 1));
        const uint8_t *st = stages + s * STAGE;
#pragma unroll
        for (int r = 0; r < MUL_R; r++) {
            const uint64_t *dbs = reinterpret_cast<const uint64_t *>(st + r * DB_CHUNK);
            const uint4 sv = reinterpret_cast<const uint4 *>(st + MUL_R * DB_CHUNK + r * SEL_CHUNK)[zi];
#pragma unroll
            for (int u = 0; u < TPT; u++) {
                const uint64_t d = dbs[(tg * TPT + u) * MUL_ZT + zi];
                const uint32_t d0 = (uint32_t)d, d1 = (uint32_t)(d >> 32);
                acc[u][0] += (uint64_t)sv.x * d0;
                acc[u][1] += (uint64_t)sv.y * d1;
                acc[u][2] += (uint64_t)sv.z * d0;
                acc[u][3] += (uint64_t)sv.w * d1;
            }
        }
        if (((it + 1) * MUL_R) % MUL_REDUCE == 0) {
#pragma unroll
            for (int u = 0; u < TPT; u++) {
                acc[u][0] = mod_u64_barrett(acc[u][0], QP0, mu0);
                acc[u][1] = mod_u64_barrett(acc[u][1], QP1, mu1);
                acc[u][2] = mod_u64_barrett(acc[u][2], QP0, mu0);
                acc[u][3] = mod_u64_barrett(acc[u][3], QP1, mu1);
            }
        }
        // every thread is done with stage s; any timed-out wait ends the loop
        if (__syncthreads_or(!arrived)) { ok = false; break; }
        if (threadIdx.x == 0 && it + MUL_STAGES < n_iter) issue(it + MUL_STAGES, s);
    }
    if (!ok) {
        // A copy never completed: report it, drain what is still in flight
        // (bounded), and leave without writing results.
        if (threadIdx.x == 0) {
            atomicExch(err, 1);
            for (int k = it; k < n_iter && k < it + MUL_STAGES; k++)
                mbar_wait(&bars[k % MUL_STAGES], (uint32_t)((k / MUL_STAGES) & 1));
        }
        __syncthreads();
        return;
    }
    const int z = zti * MUL_ZT + zi;
#pragma unroll
    for (int u = 0; u < TPT; u++) {
        const int tc = tg * TPT + u;
        const int t = tc / L.cg, col = grp * L.cg + tc % L.cg;
        uint32_t *o = out + (((uint64_t)t * L.cols + col) * 4) * D + z;
        o[0 * D] = mod_u64_barrett(acc[u][0], QP0, mu0);
        o[1 * D] = mod_u64_barrett(acc[u][1], QP1, mu1);
        o[2 * D] = mod_u64_barrett(acc[u][2], QP0, mu0);
        o[3 * D] = mod_u64_barrett(acc[u][3], QP1, mu1);
    }
}

int db_mul_ctas(const DbLayout &L) { return L.nzt * L.ncg; }

template <int TPT>
static cudaError_t launch_mul_t(const uint64_t *db, const DbLayout &L, const QDesc *qd, int nq, int *err,
                                cudaStream_t st) {
    constexpr int TCG = 4 * TPT;
    const int smem = 128 + MUL_STAGES * MUL_R * (TCG * MUL_ZT * 8 + MUL_ZT * 16);
    cudaError_t e = cudaFuncSetAttribute(k_db_mul<TPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    dim3 grid(L.nzt * L.ncg, nq);
    k_db_mul<TPT><<<grid, MUL_THREADS, smem, st>>>(db, L, qd, err);
    return cudaGetLastError();
}

cudaError_t launch_db_mul(const uint64_t *db, const DbLayout &L, const QDesc *qd, int nq, int *err,
                          cudaStream_t st) {
    const int tcg = L.T * L.cg;
    if (L.rows % MUL_REDUCE != 0 && L.rows > MUL_REDUCE) return cudaErrorInvalidValue;
    if (L.rows % MUL_R != 0) return cudaErrorInvalidValue;
    switch (tcg) {
        case 4: return launch_mul_t<1>(db, L, qd, nq, err, st);
        case 8: return launch_mul_t<2>(db, L, qd, nq, err, st);
        case 16: return launch_mul_t<4>(db, L, qd, nq, err, st);
        default: return cudaErrorInvalidValue;
    }
}

// ------------------------------------------------------- batched multiply
// Several queries against one database: compute-bound once more than ~3
// queries share a database word (4 multiply-adds per word per query on the
// integer pipe), so the database is streamed from global memory directly
// into registers and each word is reused for BQ queries; CTAs that read the
// same database stream for different query groups are adjacent in the grid
// (query group is the fastest grid index) so the stream is fetched from HBM
// about once and served from L2 to the others.
//
// CTA: 256 threads = 32 slots (half of a 64-slot z tile) x 8 pairs of tile
// words; each thread accumulates 2 words x BQ queries x 4 (row0/row1 x
// prime) in 64-bit registers, reduced every 128 rows.  Selectors of BQ
// queries for BR rows are staged in shared memory, double buffered.
constexpr int BQ = 4;     // queries per CTA
constexpr int BR = 8;     // rows per selector stage

__global__ void __launch_bounds__(256, 2) k_db_mul_batch(const uint64_t *__restrict__ db, DbLayout L,
                                                        const QDesc *__restrict__ qd, int nq) {
    __shared__ __align__(16) uint4 ssel[2][BR][BQ][32];
    const int qg = blockIdx.x;                  // query group
    const int tile = blockIdx.y;                // (z tile, z half, column group)
    const int zh = tile & 1;
    const int zti = (tile >> 1) % L.nzt, grp = (tile >> 1) / L.nzt;
    const int zi = threadIdx.x & 31, pair = threadIdx.x >> 5;     // pair of tile words 2*pair, 2*pair+1
    const int rows = L.rows;
    const uint64_t *src = db + (uint64_t)(zti * L.ncg + grp) * rows * 16 * 64 + zh * 32 + zi;
    const int q0 = qg * BQ;
    const uint32_t *sp[BQ];
#pragma unroll
    for (int k = 0; k < BQ; k++) sp[k] = (q0 + k < nq) ? qd[q0 + k].sel : qd[q0].sel;
    const uint64_t mu0 = ~0ull / QP0, mu1 = ~0ull / QP1;

    // cooperative selector load for rows [r0, r0+BR): BR*BQ*32 uint4 = 1024 -> 4 per thread
    auto stage = [&](int buf, int r0) {
#pragma unroll
        for (int k = 0; k < (BR * BQ * 32) / 256; k++) {
            const int idx = threadIdx.x + 256 * k;
            const int zz = idx & 31, qq = (idx >> 5) % BQ, rr = (idx >> 5) / BQ;
            const uint4 *s = reinterpret_cast<const uint4 *>(sp[qq]) +
                             ((uint64_t)(r0 + rr) * D + zti * 64 + zh * 32 + zz);
            ssel[buf][rr][qq][zz] = __ldg(s);
        }
    };

    uint64_t acc[2][BQ][4];
#pragma unroll
    for (int w = 0; w < 2; w++)
#pragma unroll
        for (int q = 0; q < BQ; q++)
#pragma unroll
            for (int k = 0; k < 4; k++) acc[w][q][k] = 0;

    stage(0, 0);
    __syncthreads();
    for (int r0 = 0, it = 0; r0 < rows; r0 += BR, it++) {
        const int buf = it & 1;
        if (r0 + BR < rows) stage(buf ^ 1, r0 + BR);
        uint64_t dv[BR][2];
#pragma unroll
        for (int r = 0; r < BR; r++)
#pragma unroll
            for (int w = 0; w < 2; w++) dv[r][w] = __ldg(src + ((uint64_t)(r0 + r) * 16 + 2 * pair + w) * 64);
#pragma unroll
        for (int r = 0; r < BR; r++) {
#pragma unroll
            for (int q = 0; q < BQ; q++) {
                const uint4 sv = ssel[buf][r][q][zi];
#pragma unroll
                for (int w = 0; w < 2; w++) {
                    const uint32_t d0 = (uint32_t)dv[r][w], d1 = (uint32_t)(dv[r][w] >> 32);
                    acc[w][q][0] += (uint64_t)sv.x * d0;
                    acc[w][q][1] += (uint64_t)sv.y * d1;
                    acc[w][q][2] += (uint64_t)sv.z * d0;
                    acc[w][q][3] += (uint64_t)sv.w * d1;
                }
            }
        }
        if ((r0 + BR) % MUL_REDUCE == 0) {
#pragma unroll
            for (int w = 0; w < 2; w++)
#pragma unroll
                for (int q = 0; q < BQ; q++) {
                    acc[w][q][0] = mod_u64_barrett(acc[w][q][0], QP0, mu0);
                    acc[w][q][1] = mod_u64_barrett(acc[w][q][1], QP1, mu1);
                    acc[w][q][2] = mod_u64_barrett(acc[w][q][2], QP0, mu0);
                    acc[w][q][3] = mod_u64_barrett(acc[w][q][3], QP1, mu1);
                }
        }
        __syncthreads();
    }
    const int z = zti * 64 + zh * 32 + zi;
#pragma unroll
    for (int q = 0; q < BQ; q++) {
        if (q0 + q >= nq) break;
        uint32_t *out = qd[q0 + q].acc;
#pragma unroll
        for (int w = 0; w < 2; w++) {
            const int tc = 2 * pair + w;
            const int t = tc / L.cg, col = grp * L.cg + tc % L.cg;
            uint32_t *o = out + (((uint64_t)t * L.cols + col) * 4) * D + z;
            o[0 * D] = mod_u64_barrett(acc[w][q][0], QP0, mu0);
            o[1 * D] = mod_u64_barrett(acc[w][q][1], QP1, mu1);
            o[2 * D] = mod_u64_barrett(acc[w][q][2], QP0, mu0);
            o[3 * D] = mod_u64_barrett(acc[w][q][3], QP1, mu1);
        }
    }
}

bool db_mul_batch_supported(const DbLayout &L) { return L.T * L.cg == 16 && (L.rows % BR) == 0; }

cudaError_t launch_db_mul_batch(const uint64_t *db, const DbLayout &L, const QDesc *qd, int nq, cudaStream_t st) {
    if (!db_mul_batch_supported(L)) return cudaErrorInvalidValue;
    if (L.rows > MUL_REDUCE && L.rows % MUL_REDUCE) return cudaErrorInvalidValue;
    dim3 grid((nq + BQ - 1) / BQ, L.nzt * 2 * L.ncg);
    if (grid.y > 65535) return cudaErrorInvalidValue;
    k_db_mul_batch<<<grid, 256, 0, st>>>(db, L, qd, nq);
    return cudaGetLastError();
}

}  // namespace sp
