// Database image (R5) and the integer-pipe first-dimension multiplies (R11).
//
// For one query the multiply is HBM-bound: every residue of the image is read
// once and used for 2 multiply-adds; residues are packed 28 bits each (8 in 7
// words), so a query reads 7/8 of the bytes of u32 residues.  Each CTA owns
// runs of units of the image (one prime, one slot z, one block of up to 128
// combos: a contiguous stream of `rows` packed rows) and pulls them through
// shared memory with 1-D bulk TMA copies (cp.async.bulk ...
// mbarrier::complete_tx) into a ring of stages.  Products of canonical
// residues (< 2^56) accumulate in 64-bit registers and are reduced at least
// every 128 rows, which keeps the sums below 2^64.
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
    L.cbp = (L.cb + 7) / 8 * 8;
    L.rw = L.cbp / 8 * 7;
    L.words = (uint64_t)L.rows * L.combos * D;
    return L;
}

// ----------------------------------------------------------------- encode
// One CTA per (record, t) polynomial of the chunk: group g transforms residues
// mod q_g of the recentred plaintext into tmp [record][t][prime][z]; then
// k_db_pack packs the chunk's groups of 8 combos into the image.
constexpr int ENC_SMEM_WORDS = TW_WORDS + 2 * 2 * D;

__global__ void __launch_bounds__(256) k_db_encode(const uint8_t *__restrict__ rec, uint64_t rec_count, int pt_bits,
                                                   DbLayout L, uint32_t *__restrict__ tmp,
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
        const uint8_t *src = rec + i * D;
        uint32_t v[VPT];
#pragma unroll
        for (int j = 0; j < VPT; j++) {
            uint32_t x = src[t + GROUP * j];
            v[j] = (x > pm / 2) ? c.p - (pm - x) : x;   // recentre to (-p/2, p/2]
        }
        ntt_fwd(v, tw_of(smem, g), buf, c, t, 1 + g);
#pragma unroll
        for (int j = 0; j < VPT; j++) v[j] = canon4(v[j], c.p);
        st16(tmp + (i * 2 + g) * D + VPT * t, v);
    }
}

// One thread per (row, group of 8 combos, prime, z) of the rows the chunk of
// records [rec_begin, rec_begin + rec_count) touches; groups outside the
// chunk (aligned chunks hold every group whole) are left to other chunks.
__global__ void k_db_pack(const uint32_t *__restrict__ tmp, uint64_t rec_begin, uint64_t rec_count, DbLayout L,
                          uint32_t *__restrict__ db) {
    const uint64_t row0 = rec_begin / L.cols, row1 = (rec_begin + rec_count - 1) / L.cols + 1;
    const int gpr = L.ncb * L.cbp / 8;   // groups per row
    const uint64_t total = (row1 - row0) * gpr * 2 * D;
    for (uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        const int z = (int)(idx % D);
        uint64_t r = idx / D;
        const int prime = (int)(r & 1);
        r >>= 1;
        const int k = (int)(r % gpr);
        const uint64_t row = row0 + r / gpr;
        const uint64_t first = row * L.cols + (uint64_t)((8 * k) % L.cols);   // the group's first record
        if (first < rec_begin || first >= rec_begin + rec_count) continue;
        uint32_t v[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int m = 8 * k + j;
            v[j] = 0;
            if (m < L.combos) {
                const uint64_t rec = row * L.cols + (uint64_t)(m % L.cols);
                v[j] = tmp[(((rec - rec_begin) * L.T + m / L.cols) * 2 + prime) * D + z];
            }
        }
        uint32_t w[7];
        pack8(v, w);
        uint32_t *dst = db + L.row_offset32(prime, z, 8 * k / L.cbp, (int)row) + (8 * k % L.cbp) / 8 * 7;
#pragma unroll
        for (int i = 0; i < 7; i++) dst[i] = w[i];
    }
}

cudaError_t launch_db_encode(const uint8_t *records, uint64_t rec_begin, uint64_t rec_count,
                             int pt_bits, const DbLayout &L, uint32_t *tmp, uint32_t *db, const TwiddleSet *tw,
                             cudaStream_t st) {
    const uint64_t n_rec = (uint64_t)L.rows * L.cols;
    if (rec_count == 0 || rec_begin % 8 != 0 || (rec_count % 8 != 0 && rec_begin + rec_count != n_rec))
        return cudaErrorInvalidValue;
    const int smem = ENC_SMEM_WORDS * 4;
    cudaError_t e = cudaFuncSetAttribute(k_db_encode, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t polys = rec_count * L.T;
    int grid = (int)(polys < (uint64_t)sms * 3 ? polys : (uint64_t)sms * 3);
    if (grid < 1) grid = 1;
    k_db_encode<<<grid, 256, smem, st>>>(records, rec_count, pt_bits, L, tmp, tw);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_db_pack<<<4096, 256, 0, st>>>(tmp, rec_begin, rec_count, L, db);
    return cudaGetLastError();
}

// One thread per (row, group of 8 combos, prime, z); residues are reduced
// mod the prime (the planes are meant to be canonical) so that each fits
// its 28 bits.
__global__ void k_db_import(const uint32_t *__restrict__ planes, DbLayout L, uint32_t *__restrict__ db) {
    const int gpr = L.ncb * L.cbp / 8;
    const uint64_t total = (uint64_t)L.rows * gpr * 2 * D;
    for (uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        const int z = (int)(idx % D);
        uint64_t r = idx / D;
        const int prime = (int)(r & 1);
        r >>= 1;
        const int k = (int)(r % gpr);
        const int row = (int)(r / gpr);
        const uint32_t p = prime ? QP1 : QP0;
        uint32_t v[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int m = 8 * k + j;
            v[j] = 0;
            if (m < L.combos) {
                const int t = m / L.cols, col = m % L.cols;
                const uint32_t x = planes[((((uint64_t)t * L.cols + col) * L.rows + row) * 2 + prime) * D + z];
                v[j] = x < p ? x : x % p;
            }
        }
        uint32_t w[7];
        pack8(v, w);
        uint32_t *dst = db + L.row_offset32(prime, z, 8 * k / L.cbp, row) + (8 * k % L.cbp) / 8 * 7;
#pragma unroll
        for (int i = 0; i < 7; i++) dst[i] = w[i];
    }
}

cudaError_t launch_db_import(const uint32_t *planes, const DbLayout &L, uint32_t *db, cudaStream_t st) {
    k_db_import<<<4096, 256, 0, st>>>(planes, L, db);
    return cudaGetLastError();
}

// --------------------------------------------------------------- multiply
namespace {

constexpr int MUL_THREADS = 256;              // consumer threads (plus one producer warp)
constexpr uint32_t MUL_STAGE_BYTES = 32768;   // largest stage (a stage holds whole packed rows)
constexpr int MUL_STAGES = 3;                 // 2 CTAs per SM: 6 stages of 28 KiB per SM
constexpr int MUL_REDUCE = 128;  // own rows between reductions (sums < 2^64)
constexpr int MUL_WARPS = MUL_THREADS / 32;

// Packed rows per stage: a power of two that fills at most one stage slot
// (rows is a power of two, so stages tile a unit).
__host__ __device__ inline int mul_stage_rows(const DbLayout &L) {
    int r = 1;
    while (2 * r <= L.rows && (uint32_t)(2 * r) * L.rw * 4 <= MUL_STAGE_BYTES) r *= 2;
    return r;
}

__host__ __device__ inline int mul_sel_bytes(const DbLayout &L) { return ((L.rows * 8 + 127) / 128) * 128; }

// bytes of one stage slot: the stage's packed rows, 128-byte aligned
__host__ __device__ inline int mul_stage_slot(const DbLayout &L) {
    return (mul_stage_rows(L) * L.rw * 4 + 127) / 128 * 128;
}

// shared memory: barriers and abort flag, selectors, per-warp row sums
// [8][cbp], stage ring
__host__ __device__ inline int mul_smem_bytes(const DbLayout &L) {
    return 128 + mul_sel_bytes(L) + MUL_WARPS * L.cbp * 8 + MUL_STAGES * mul_stage_slot(L);
}

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
// the image.  Warp 8 issues the stage copies; consumer thread (row phase rp,
// group mg) accumulates, for the 8 combos of packed group mg, rows
// r = rp (mod RS) for both ciphertext rows.  Consumers release a stage with
// an arrival on its `empty` barrier, so only the producer waits for the
// slowest warp.  At the end of each unit the row phases are summed (warp
// shuffles, then through shared memory) and the unit's outputs written.
// As a dependent launch (after the expansion) the producer starts streaming
// the image at once, since the image does not depend on earlier kernels;
// the consumers wait for the previous kernel before reading the descriptor
// and the selectors.
__global__ void __launch_bounds__(MUL_THREADS + 32, 2) k_db_mul(const uint32_t *__restrict__ db, DbLayout L,
                                                        const QDesc *__restrict__ qd, int *err) {
    extern __shared__ __align__(128) uint8_t smem_mul[];
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_mul);              // [MUL_STAGES]
    uint64_t *empty = full + MUL_STAGES;                                   // [MUL_STAGES]
    volatile int *abort = reinterpret_cast<volatile int *>(smem_mul + 120);
    uint2 *ssel = reinterpret_cast<uint2 *>(smem_mul + 128);          // [rows] (ct row 0, ct row 1)
    uint2 *red = reinterpret_cast<uint2 *>(smem_mul + 128 + mul_sel_bytes(L));   // [warp][cbp]
    uint8_t *stages = smem_mul + 128 + mul_sel_bytes(L) + MUL_WARPS * L.cbp * 8;

    pdl_launch_dependents();
    const int U = mul_units_per_cta(L);
    const uint64_t u0 = (uint64_t)blockIdx.x * U;
    const int rows = L.rows, cb = L.cb, cbp = L.cbp, rw = L.rw;
    const int SR = mul_stage_rows(L);
    const int SPU = rows / SR;                 // stages per unit
    const uint32_t stage_bytes = (uint32_t)SR * rw * 4;
    const int slot = mul_stage_slot(L);
    const int n_iter = U * SPU;
    const uint32_t *src = db + u0 * L.unit_words32();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    if (threadIdx.x == 0) {
        for (int s = 0; s < MUL_STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], MUL_THREADS);
        }
        *abort = 0;
        fence_mbar_init();
    }
    __syncthreads();
    if (warp == MUL_WARPS) {
        // ------------------------------------------------------- producer
        if (lane == 0) {
            int it = 0;
            for (; it < n_iter; it++) {
                const int s = it % MUL_STAGES;
                if (it >= MUL_STAGES && !mbar_wait_bounded(&empty[s], ((it / MUL_STAGES) - 1) & 1, abort)) break;
                mbar_expect_tx(&full[s], stage_bytes);
                tma_bulk_g2s(stages + s * slot, src + (uint64_t)it * SR * rw, stage_bytes, &full[s]);
            }
            // the copies still in flight land before the CTA may exit
            for (int k = it > MUL_STAGES ? it - MUL_STAGES : 0; k < it; k++)
                mbar_wait_timed(&full[k % MUL_STAGES], (uint32_t)((k / MUL_STAGES) & 1));
        }
        return;
    }
    // ---------------------------------------------------------- consumers
    pdl_wait();   // the selectors come from the previous kernel
    const QDesc &Q = qd[blockIdx.y];
    const uint32_t *__restrict__ sel = Q.sel;
    auto consumers_sync = []() { asm volatile("bar.sync 1, %0;" ::"n"(MUL_THREADS) : "memory"); };
    const int groups = cbp / 8;                // threads per row
    const int mg = threadIdx.x % groups, rp = threadIdx.x / groups, RS = MUL_THREADS / groups;
    int prime = 0, z = 0;
    uint32_t p = QP0;
    uint64_t mu = ~0ull / QP0;
    uint64_t a0[8], a1[8];
#pragma unroll
    for (int c = 0; c < 8; c++) a0[c] = a1[c] = 0;
    int since = 0;
    for (int it = 0; it < n_iter; it++) {
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
            consumers_sync();
        }
        // a wait that runs out sets the abort flag; the thread still computes
        // (on stale data) and leaves with the others at the end of the unit
        mbar_wait_bounded(&full[s], (uint32_t)((it / MUL_STAGES) & 1), abort);
        const uint32_t *st = reinterpret_cast<const uint32_t *>(stages + s * slot) + 7 * mg;
        const uint2 *sv = ssel + local * SR;
#pragma unroll 4
        for (int r = rp; r < SR; r += RS) {
            uint32_t w[7], d[8];
#pragma unroll
            for (int i = 0; i < 7; i++) w[i] = st[r * rw + i];
            unpack8(w, d);
            const uint2 v = sv[r];
#pragma unroll
            for (int c = 0; c < 8; c++) {
                a0[c] += (uint64_t)v.x * d[c];
                a1[c] += (uint64_t)v.y * d[c];
            }
        }
        mbar_arrive(&empty[s]);   // this thread is done with stage s
        since += (SR + RS - 1) / RS;
        if (since >= MUL_REDUCE) {
#pragma unroll
            for (int c = 0; c < 8; c++) {
                a0[c] = mod_u64_barrett(a0[c], p, mu);
                a1[c] = mod_u64_barrett(a1[c], p, mu);
            }
            since = 0;
        }
        if (local == SPU - 1) {
            // sum the warp's row phases (lanes groups apart), then one slot
            // per warp and combo
#pragma unroll
            for (int c = 0; c < 8; c++) {
                uint32_t x0 = mod_u64_barrett(a0[c], p, mu), x1 = mod_u64_barrett(a1[c], p, mu);
                for (int off = 16; off >= groups; off >>= 1) {
                    x0 += __shfl_xor_sync(0xffffffffu, x0, off);
                    x1 += __shfl_xor_sync(0xffffffffu, x1, off);
                    x0 = x0 >= p ? x0 - p : x0;
                    x1 = x1 >= p ? x1 - p : x1;
                }
                if (lane < groups) red[warp * cbp + mg * 8 + c] = make_uint2(x0, x1);
                a0[c] = a1[c] = 0;
            }
            since = 0;
            consumers_sync();
            const bool stop = *abort != 0;   // the same for every consumer after the barrier
            if (!stop && threadIdx.x < 2 * cb) {
                const int mm = threadIdx.x >> 1, k = threadIdx.x & 1;
                uint32_t sum = 0;   // < 8p < 2^31
#pragma unroll
                for (int q = 0; q < MUL_WARPS; q++) {
                    const uint2 v = red[q * cbp + mm];
                    sum += k ? v.y : v.x;
                }
                const uint64_t mgl = (u % L.ncb) * cb + mm;
                Q.acc[((mgl * 2 + k) * 2 + prime) * D + z] = sum % p;
            }
            // `red` is rewritten at the end of the next unit
            consumers_sync();
            if (stop) {
                if (threadIdx.x == 0) atomicExch(err, 1);
                break;
            }
        }
    }
}

cudaError_t launch_db_mul(const uint32_t *db, const DbLayout &L, const QDesc *qd, int nq, int *err,
                          cudaStream_t st, bool pdl) {
    const int SR = mul_stage_rows(L);
    if (L.rows % SR != 0 || ((uint64_t)SR * L.rw * 4) % 16 != 0 || MUL_THREADS % (L.cbp / 8) != 0)
        return cudaErrorInvalidValue;
    const uint64_t ctas = L.units() / mul_units_per_cta(L);
    if (ctas * mul_units_per_cta(L) != L.units() || ctas > 0x7fffffffull) return cudaErrorInvalidValue;
    const int smem = mul_smem_bytes(L);
    cudaError_t e = cudaFuncSetAttribute(k_db_mul, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    e = launch_ex(k_db_mul, dim3((unsigned)ctas, nq), dim3(MUL_THREADS + 32), (size_t)smem, st, pdl, db, L, qd, err);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
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
    const uint32_t *src = db + unit * L.unit_words32();
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
            const uint32_t d = unpack1(src + (uint64_t)(c0 + r) * L.rw, m);
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

// ----------------------------------------------------- bounded-wait probe
// The failure path of the multiply kernels' barrier waits, run on purpose
// without a GPU fault: every thread waits on an mbarrier whose one expected
// arrival never comes, with the same bounded wait as the multiply (limit
// `limit_ns`).  The first thread to give up sets the shared abort flag, the
// others stop at their next check, and thread 0 sets the error flag the host
// reads (code 1, as a multiply timeout) before the kernel returns.
__global__ void k_wait_probe(int *err, uint64_t limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ int abort;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        abort = 0;
        fence_mbar_init();
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&bar, 0, &abort, limit_ns);
    __syncthreads();
    if (threadIdx.x == 0 && !ok) atomicExch(err, 1);
}

cudaError_t launch_wait_probe(int *err, uint64_t limit_ns, cudaStream_t st) {
    k_wait_probe<<<1, 64, 0, st>>>(err, limit_ns);
    return cudaGetLastError();
}

}  // namespace sp
