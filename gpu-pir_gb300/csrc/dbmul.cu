// Database image (R5) and the integer-pipe first-dimension multiplies (R11).
//
// For one query the multiply is HBM-bound: every residue of the image is read
// once and used for 2 multiply-adds.  Each CTA owns one unit of the image
// (one prime, one slot z, one block of up to 128 combos: a contiguous stream
// of rows*cb residues) and pulls it through shared memory with 1-D bulk TMA
// copies (cp.async.bulk ... mbarrier::complete_tx) into a ring of stages.
// Products of canonical residues (< 2^56) accumulate in 64-bit registers and
// are reduced at least every 128 rows, which keeps the sums below 2^64.
#include <type_traits>

#include "async.cuh"
#include "kernels.cuh"

namespace sp {

DbLayout make_db_layout(int T, int nu1, int nu2) {
    DbLayout L{};
    L.T = T;
    L.nu1 = nu1;
    L.nu2 = nu2;
    L.rows = 1 << nu1;
    L.cols = 1 << nu2;
    L.combos = T * L.cols;
    L.cb = L.combos < 128 ? L.combos : 128;
    L.ncb = L.combos / L.cb;
    L.words = (uint64_t)L.rows * L.combos * D;
    return L;
}

// ----------------------------------------------------------------- encode
// One CTA per (record, t) polynomial: group g transforms residues mod q_g of
// the recentred plaintext and writes its 32-bit half of the packed words.
constexpr int ENC_SMEM_WORDS = TW_WORDS + 2 * 2 * D;

__global__ void __launch_bounds__(256) k_db_encode(const uint8_t *__restrict__ rec, uint64_t rec_begin,
                                                   uint64_t rec_count, int pt_bits, DbLayout L,
                                                   uint32_t *__restrict__ db,
                                                   const TwiddleSet *__restrict__ tws) {
    extern __shared__ __align__(16) uint32_t smem[];
    load_twiddles(smem, tws);
    __syncthreads();
    const int g = threadIdx.x >> 7, t = threadIdx.x & (GROUP - 1);
    const Prime c = prime_of(g);
    uint32_t *buf = smem + TW_WORDS + g * 2 * D;
    const uint32_t pm = 1u << pt_bits;
    const uint64_t polys = rec_count * L.T;
    for (uint64_t i = blockIdx.x; i < polys; i += gridDim.x) {
        const uint64_t r_local = i / L.T;
        const int tt = (int)(i % L.T);
        const uint64_t r = rec_begin + r_local;
        const int row = (int)(r / L.cols), m = tt * L.cols + (int)(r % L.cols);
        const uint8_t *src = rec + i * D;
        uint32_t v[VPT];
#pragma unroll
        for (int j = 0; j < VPT; j++) {
            uint32_t x = src[t + GROUP * j];
            v[j] = (x > pm / 2) ? c.p - (pm - x) : x;   // recentre to (-p/2, p/2]
        }
        ntt_fwd(v, tw_of(smem, g), buf, c, t, 1 + g);
#pragma unroll
        for (int j = 0; j < VPT; j++) {
            const int z = VPT * t + j;
            db[L.offset32(g, m, row, z)] = canon4(v[j], c.p);
        }
    }
}

cudaError_t launch_db_encode(const uint8_t *records, uint64_t rec_begin, uint64_t rec_count,
                             int pt_bits, const DbLayout &L, uint32_t *db, const TwiddleSet *tw,
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

__global__ void k_db_import(const uint32_t *__restrict__ planes, DbLayout L, uint32_t *__restrict__ db) {
    const uint64_t total = (uint64_t)L.T * L.cols * L.rows * D;
    for (uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        const int z = (int)(idx % D);
        uint64_t r = idx / D;
        const int row = (int)(r % L.rows); r /= L.rows;
        const int col = (int)(r % L.cols); r /= L.cols;
        const int t = (int)r;
        const uint32_t *src = planes + (((uint64_t)t * L.cols + col) * L.rows + row) * 2 * D;
        const int m = t * L.cols + col;
        db[L.offset32(0, m, row, z)] = src[z];
        db[L.offset32(1, m, row, z)] = src[D + z];
    }
}

cudaError_t launch_db_import(const uint32_t *planes, const DbLayout &L, uint32_t *db, cudaStream_t st) {
    k_db_import<<<4096, 256, 0, st>>>(planes, L, db);
    return cudaGetLastError();
}

// --------------------------------------------------------------- multiply
namespace {

constexpr int MUL_THREADS = 256;
constexpr uint32_t MUL_STAGE_BYTES = 16384;
constexpr int MUL_STAGES = 2;
constexpr int MUL_REDUCE = 128;  // own rows between reductions (sums < 2^64)

__host__ __device__ inline int mul_stage_rows(const DbLayout &L) {
    const int r = (int)(MUL_STAGE_BYTES / (L.cb * 4));
    return L.rows < r ? L.rows : r;
}

__host__ __device__ inline int mul_sel_bytes(const DbLayout &L) { return ((L.rows * 8 + 127) / 128) * 128; }

}  // namespace

// Units per CTA: whole (prime, z) groups of ncb units, about 1 MiB of image
// or more, so that pipeline start-up is paid rarely; at most 8 groups, which
// leaves at least 2*D/8 = 512 CTAs per query.
__host__ __device__ inline int mul_units_per_cta(const DbLayout &L) {
    const uint64_t group = (uint64_t)L.ncb * L.unit_words32() * 4;
    int k = 1;
    while (group * k < (1u << 20) && k < 8) k <<= 1;
    return L.ncb * k;
}

// One CTA per (run of units, query).  The run is one contiguous stream of
// the image.  Thread (row phase rp, combo group mg) accumulates, for CPT
// consecutive combos, rows r = rp (mod RS) for both ciphertext rows: one
// 4*CPT-byte image load and one selector load feed 2*CPT independent
// multiply-adds.  At the end of each unit the row phases are summed through
// shared memory and the unit's outputs written.
template <int CPT>
__global__ void __launch_bounds__(MUL_THREADS) k_db_mul(const uint32_t *__restrict__ db, DbLayout L,
                                                        const QDesc *__restrict__ qd, int *err) {
    using Vec = typename std::conditional<CPT == 4, uint4, uint32_t>::type;
    extern __shared__ __align__(128) uint8_t smem_mul[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem_mul);
    uint2 *ssel = reinterpret_cast<uint2 *>(smem_mul + 128);          // [rows] (ct row 0, ct row 1)
    uint2 *red = reinterpret_cast<uint2 *>(smem_mul + 128 + mul_sel_bytes(L));   // [RS][cb]
    uint8_t *stages = smem_mul + 128 + mul_sel_bytes(L) + MUL_THREADS * CPT * 8;

    const QDesc &Q = qd[blockIdx.y];
    const uint32_t *__restrict__ sel = Q.sel;
    const int U = mul_units_per_cta(L);
    const uint64_t u0 = (uint64_t)blockIdx.x * U;
    const int rows = L.rows, cb = L.cb;
    const int SR = mul_stage_rows(L);
    const int SPU = rows / SR;                 // stages per unit
    const uint32_t stage_bytes = (uint32_t)SR * cb * 4;
    const int n_iter = U * SPU;
    const uint32_t *src = db + u0 * L.unit_words32();

    if (threadIdx.x == 0) {
        for (int s = 0; s < MUL_STAGES; s++) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](int it, int s) {
        mbar_expect_tx(&bars[s], stage_bytes);
        tma_bulk_g2s(stages + s * MUL_STAGE_BYTES, src + (uint64_t)it * SR * cb, stage_bytes, &bars[s]);
    };
    if (threadIdx.x == 0)
        for (int s = 0; s < MUL_STAGES && s < n_iter; s++) issue(s, s);

    const int groups = cb / CPT;               // threads per row
    const int mg = threadIdx.x % groups, rp = threadIdx.x / groups, RS = MUL_THREADS / groups;
    int prime = 0, z = 0;
    uint32_t p = QP0;
    uint64_t mu = ~0ull / QP0;
    uint64_t a0[CPT], a1[CPT];
#pragma unroll
    for (int c = 0; c < CPT; c++) a0[c] = a1[c] = 0;
    int since = 0;
    bool ok = true;
    int it = 0;
    for (; it < n_iter; it++) {
        const int s = it % MUL_STAGES;
        const int local = it % SPU, ui = it / SPU;
        const uint64_t u = u0 + ui;
        if (local == 0 && (ui == 0 || u % L.ncb == 0)) {
            // new (prime, z): gather its selectors (L2-resident) for every row
            z = (int)((u / L.ncb) % D);
            prime = (int)(u / ((uint64_t)L.ncb * D));
            p = prime ? QP1 : QP0;
            mu = ~0ull / p;
            for (int r = threadIdx.x; r < rows; r += MUL_THREADS) {
                const uint32_t *sr = sel + ((uint64_t)r * D + z) * 4;
                ssel[r] = make_uint2(__ldg(sr + prime), __ldg(sr + 2 + prime));
            }
            __syncthreads();
        }
        // A thread whose wait runs out still computes (on stale data) so that
        // the whole CTA reaches the barrier below and leaves together.
        const bool arrived = mbar_wait_timed(&bars[s], (uint32_t)((it / MUL_STAGES) & 1));
        const Vec *st = reinterpret_cast<const Vec *>(stages + s * MUL_STAGE_BYTES);
        const uint2 *sv = ssel + local * SR;
#pragma unroll 4
        for (int r = rp; r < SR; r += RS) {
            const Vec d = st[r * groups + mg];
            const uint2 v = sv[r];
            if constexpr (CPT == 4) {
                a0[0] += (uint64_t)v.x * d.x;
                a1[0] += (uint64_t)v.y * d.x;
                a0[1] += (uint64_t)v.x * d.y;
                a1[1] += (uint64_t)v.y * d.y;
                a0[2] += (uint64_t)v.x * d.z;
                a1[2] += (uint64_t)v.y * d.z;
                a0[3] += (uint64_t)v.x * d.w;
                a1[3] += (uint64_t)v.y * d.w;
            } else {
                a0[0] += (uint64_t)v.x * d;
                a1[0] += (uint64_t)v.y * d;
            }
        }
        since += (SR + RS - 1) / RS;
        if (since >= MUL_REDUCE) {
#pragma unroll
            for (int c = 0; c < CPT; c++) {
                a0[c] = mod_u64_barrett(a0[c], p, mu);
                a1[c] = mod_u64_barrett(a1[c], p, mu);
            }
            since = 0;
        }
        const bool last = local == SPU - 1;
        if (last) {
#pragma unroll
            for (int c = 0; c < CPT; c++) {
                red[rp * cb + mg * CPT + c] = make_uint2(mod_u64_barrett(a0[c], p, mu), mod_u64_barrett(a1[c], p, mu));
                a0[c] = a1[c] = 0;
            }
            since = 0;
        }
        // every thread is done with stage s; any timed-out wait ends the loop
        if (__syncthreads_or(!arrived)) {
            ok = false;
            break;
        }
        if (threadIdx.x == 0 && it + MUL_STAGES < n_iter) issue(it + MUL_STAGES, s);
        if (last) {
            if (threadIdx.x < 2 * cb) {
                const int mm = threadIdx.x >> 1, k = threadIdx.x & 1;
                uint64_t sum = 0;
                for (int q = 0; q < RS; q++) {
                    const uint2 v = red[q * cb + mm];
                    sum += k ? v.y : v.x;
                }
                const uint64_t mgl = (u % L.ncb) * cb + mm;
                Q.acc[((mgl * 2 + k) * 2 + prime) * D + z] = (uint32_t)(sum % p);
            }
            // `red` is rewritten at the end of the next unit
            __syncthreads();
        }
    }
    if (!ok) {
        // A copy never completed: report it, drain what is still in flight
        // (bounded), and leave without writing further results.
        if (threadIdx.x == 0) {
            atomicExch(err, 1);
            for (int k = it; k < n_iter && k < it + MUL_STAGES; k++)
                mbar_wait_timed(&bars[k % MUL_STAGES], (uint32_t)((k / MUL_STAGES) & 1));
        }
        __syncthreads();
    }
}

template <int CPT>
static cudaError_t launch_mul_cpt(const uint32_t *db, const DbLayout &L, const QDesc *qd, int nq, int *err,
                                  cudaStream_t st) {
    const uint64_t ctas = L.units() / mul_units_per_cta(L);
    if (ctas * mul_units_per_cta(L) != L.units() || ctas > 0x7fffffffull) return cudaErrorInvalidValue;
    const int smem = 128 + mul_sel_bytes(L) + MUL_THREADS * CPT * 8 + MUL_STAGES * MUL_STAGE_BYTES;
    cudaError_t e = cudaFuncSetAttribute(k_db_mul<CPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)ctas, nq);
    k_db_mul<CPT><<<grid, MUL_THREADS, smem, st>>>(db, L, qd, err);
    return cudaGetLastError();
}

cudaError_t launch_db_mul(const uint32_t *db, const DbLayout &L, const QDesc *qd, int nq, int *err,
                          cudaStream_t st) {
    if (L.rows % mul_stage_rows(L) != 0 || MUL_THREADS % L.cb != 0) return cudaErrorInvalidValue;
    if (L.cb >= 4) return launch_mul_cpt<4>(db, L, qd, nq, err, st);
    return launch_mul_cpt<1>(db, L, qd, nq, err, st);
}

// ------------------------------------------------------- batched multiply
// Several queries against one database on the integer pipe: each residue is
// loaded once per group of BQ queries (straight from global memory into
// registers; the CTAs of the query groups of one unit are adjacent in the
// grid, so the unit comes from HBM about once and from L2 for the others)
// and used for 2*BQ multiply-adds.  Selectors of the BQ queries are staged in
// shared memory per chunk of rows.
constexpr int BQ = 8;
constexpr int BCH = 32;   // rows per selector chunk

__global__ void __launch_bounds__(256) k_db_mul_batch(const uint32_t *__restrict__ db, DbLayout L,
                                                     const QDesc *__restrict__ qd, int nq) {
    __shared__ uint2 ssel[BCH][BQ];
    __shared__ uint2 red[256][BQ];
    // query groups of one unit are adjacent in the grid
    const int groups = (nq + BQ - 1) / BQ;
    const uint64_t unit = blockIdx.x / groups;
    const int cbi = (int)(unit % L.ncb);
    const int z = (int)((unit / L.ncb) % D);
    const int prime = (int)(unit / ((uint64_t)L.ncb * D));
    const int q0 = (int)(blockIdx.x % groups) * BQ;
    const int rows = L.rows, cb = L.cb;
    const int m = threadIdx.x % cb, rp = threadIdx.x / cb, RS = 256 / cb;
    const int CH = rows < BCH ? rows : BCH;
    const uint32_t *src = db + unit * L.unit_words32() + m;
    const uint32_t p = prime ? QP1 : QP0;
    const uint64_t mu = ~0ull / p;

    uint64_t acc[BQ][2];
#pragma unroll
    for (int q = 0; q < BQ; q++) acc[q][0] = acc[q][1] = 0;
    int since = 0;
    for (int c0 = 0; c0 < rows; c0 += CH) {
        for (int i = threadIdx.x; i < CH * BQ; i += 256) {
            const int r = i / BQ, q = i % BQ;
            uint2 v = make_uint2(0, 0);
            if (q0 + q < nq) {
                const uint32_t *sr = qd[q0 + q].sel + ((uint64_t)(c0 + r) * D + z) * 4;
                v = make_uint2(__ldg(sr + prime), __ldg(sr + 2 + prime));
            }
            ssel[r][q] = v;
        }
        __syncthreads();
        for (int r = rp; r < CH; r += RS) {
            const uint32_t d = __ldg(src + (uint64_t)(c0 + r) * cb);
#pragma unroll
            for (int q = 0; q < BQ; q++) {
                const uint2 v = ssel[r][q];
                acc[q][0] += (uint64_t)v.x * d;
                acc[q][1] += (uint64_t)v.y * d;
            }
        }
        since += (CH + RS - 1) / RS;
        if (since >= MUL_REDUCE) {
#pragma unroll
            for (int q = 0; q < BQ; q++) {
                acc[q][0] = mod_u64_barrett(acc[q][0], p, mu);
                acc[q][1] = mod_u64_barrett(acc[q][1], p, mu);
            }
            since = 0;
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < BQ; q++)
        red[threadIdx.x][q] = make_uint2(mod_u64_barrett(acc[q][0], p, mu), mod_u64_barrett(acc[q][1], p, mu));
    __syncthreads();
    for (int i = threadIdx.x; i < cb * BQ * 2; i += 256) {
        const int k = i & 1, mm = (i >> 1) % cb, q = (i >> 1) / cb;
        if (q0 + q >= nq) continue;
        uint64_t s = 0;
        for (int ph = 0; ph < RS; ph++) {
            const uint2 v = red[ph * cb + mm][q];
            s += k ? v.y : v.x;
        }
        const int mg = cbi * cb + mm;
        qd[q0 + q].acc[(((uint64_t)mg * 2 + k) * 2 + prime) * D + z] = (uint32_t)(s % p);
    }
}

bool db_mul_batch_supported(const DbLayout &L) { return 256 % L.cb == 0; }

cudaError_t launch_db_mul_batch(const uint32_t *db, const DbLayout &L, const QDesc *qd, int nq, cudaStream_t st) {
    if (!db_mul_batch_supported(L)) return cudaErrorInvalidValue;
    const uint64_t groups = (uint64_t)(nq + BQ - 1) / BQ;
    if (L.units() * groups > 0x7fffffffull) return cudaErrorInvalidValue;
    k_db_mul_batch<<<(unsigned)(L.units() * groups), 256, 0, st>>>(db, L, qd, nq);
    return cudaGetLastError();
}

}  // namespace sp
